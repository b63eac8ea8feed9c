// sort.cu -- device-side particle ordering by grid cell for the batched path.
//
// The scatter kernels pre-reduce a warp's contributions per stencil base
// (batched.cu): that only pays when the 32 particles of a warp share few
// bases, i.e. when particles that are close in space are close in memory.
// Objects arrive in sampling order (random positions), and particles drift
// as the simulation runs, so the batch re-orders its particles on the device:
// every env's particles are ranked by the 4^3 grid block of their stencil
// base cell, then by the cell within the block (the block layout of the
// grids), then by their previous index (a deterministic order).  Particles
// never leave their env's range, so tiles, envs and offsets are unchanged.
//
// Counting sort, one launch per phase for all envs:
//   count  -- per particle: its key cell; the cell's count (warp-aggregated
//             atomic) gives the particle a rank within its cell; the key's
//             block joins a list of occupied blocks;
//   cells  -- per occupied block (one warp): exclusive scan of its 64 cell
//             counts, block total;
//   scan   -- exclusive scan of the block totals over all blocks of the
//             batch in block order (two launches: chunk sums, then chunk
//             scans) -- env e's blocks follow env e-1's, so block bases are
//             global particle indices;
//   place  -- perm[base(block) + start(cell) + rank] = old index;
//   fix    -- per occupied block (a warp; a CTA for large blocks): each
//             cell's segment of perm put in increasing old index (the ranks
//             came from atomics in arbitrary order); then the counts, totals,
//             flags and list are zeroed for the next sort;
//   permute -- the 24 state planes gathered into the new order.
// The caller permutes whatever else is per particle (material, targets) with
// dexmpm_permute and the same perm.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_math.cuh"
#include "../../include/dexmpm.h"

using namespace dexmpm;

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kScanThreads = 1024;
constexpr int kScanChunk = DEXMPM_SORT_CHUNK;  // block totals per scan CTA (4 per thread)
static_assert(kScanChunk == 4 * kScanThreads, "scan chunk");

// Key cell of a particle at x: its stencil base cell (floor(x inv_dx - 0.5)
// per axis, the P2G stencil's base up to rounding at cell faces; product and
// difference each rounded to FP32, no fused multiply-add), clamped into the
// env's grid, as a global cell index of the block layout.
__device__ __forceinline__ int key_cell(const DexEnv &E, float x, float y, float z) {
  const float xs[3] = {__fmul_rn(x, E.inv_dx), __fmul_rn(y, E.inv_dx), __fmul_rn(z, E.inv_dx)};
  const int g[3] = {E.gx, E.gy, E.gz};
  int c[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float f = floorf(__fsub_rn(xs[d], 0.5f));
    // NaN and out-of-range positions land on the nearest boundary cell
    c[d] = f >= 0.f ? (f < (float)(g[d] - 1) ? (int)f : g[d] - 1) : 0;
  }
  const int nby = E.gy >> 2, nbz = E.gz >> 2;
  const int blk = E.blk_off + ((c[0] >> 2) * nby + (c[1] >> 2)) * nbz + (c[2] >> 2);
  return (blk << 6) + ((c[0] & 3) << 4) + ((c[1] & 3) << 2) + (c[2] & 3);
}

__global__ void __launch_bounds__(256) k_sort_count(DexBatch B, DexSortWork W, const float *__restrict__ S) {
  const int tile = blockIdx.x;
  const DexEnv E = B.envs[B.tiles[2 * tile]];
  const int loc = B.tiles[2 * tile + 1] + threadIdx.x;
  const bool in = loc < E.n;
  const int N = B.n_particles;
  const int p = E.p_off + (in ? loc : 0);
  const int lane = threadIdx.x & 31;
  const int ci = in ? key_cell(E, __ldg(S + p), __ldg(S + N + p), __ldg(S + 2 * N + p)) : -1;
  // lanes of one cell take consecutive ranks with one atomic
  const unsigned same = __match_any_sync(kFull, ci);
  const int leader = __ffs(same) - 1;
  int first = 0;
  if (in && lane == leader) first = atomicAdd(W.cell_count + ci, __popc(same));
  first = __shfl_sync(kFull, first, leader);
  if (!in) return;
  W.rank[p] = first + __popc(same & ((1u << lane) - 1u));
  W.key[p] = ci;
  const int blk = ci >> 6;
  if (lane == leader && *reinterpret_cast<volatile uint32_t *>(W.block_flag + blk) == 0u &&
      atomicExch(W.block_flag + blk, 1u) == 0u)
    W.block_list[atomicAdd(W.counters, 1)] = blk;
}

// Warp-wide exclusive scan of one value per lane; *total receives the sum.
__device__ __forceinline__ int warp_exclusive(int v, int lane, int *total) {
  int incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int t = __shfl_up_sync(kFull, incl, d);
    if (lane >= d) incl += t;
  }
  *total = __shfl_sync(kFull, incl, 31);
  return incl - v;
}

// One warp per occupied block: cell_start = exclusive scan of its 64 cell
// counts (lane l: cells 2l, 2l + 1), block_total = their sum.
__global__ void __launch_bounds__(256) k_sort_cells(DexSortWork W) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  const int cnt = *reinterpret_cast<volatile int32_t *>(W.counters);
  for (int item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); item < cnt; item += warps) {
    const int blk = W.block_list[item];
    const int2 c = reinterpret_cast<const int2 *>(W.cell_count + (blk << 6))[lane];
    int total;
    const int ex = warp_exclusive(c.x + c.y, lane, &total);
    reinterpret_cast<int2 *>(W.cell_start + (blk << 6))[lane] = make_int2(ex, ex + c.x);
    if (lane == 0) W.block_total[blk] = total;
  }
}

// Sum of the block totals of each chunk of kScanChunk blocks.
__device__ __forceinline__ int4 load4(const int32_t *a, int i, int n) {
  if (i + 3 < n) return *reinterpret_cast<const int4 *>(a + i);
  return make_int4(i < n ? a[i] : 0, i + 1 < n ? a[i + 1] : 0, i + 2 < n ? a[i + 2] : 0, 0);
}

__device__ __forceinline__ int block_reduce(int v, int *smem) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
  if (lane == 0) smem[w] = v;
  __syncthreads();
  int t = 0;
  if (w == 0) {
    t = lane < (blockDim.x >> 5) ? smem[lane] : 0;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(kFull, t, d);
  }
  return t;  // valid in warp 0
}

__global__ void __launch_bounds__(kScanThreads) k_scan_chunks(DexSortWork W, int n_blocks) {
  __shared__ int smem[32];
  const int i = blockIdx.x * kScanChunk + 4 * threadIdx.x;
  const int4 v = load4(W.block_total, i, n_blocks);
  const int t = block_reduce(v.x + v.y + v.z + v.w, smem);
  if (threadIdx.x == 0) W.partial[blockIdx.x] = t;
}

// block_base = exclusive scan of block_total: the chunk's offset is the sum
// of the partials before it, then a CTA-wide scan of the chunk.
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(DexSortWork W, int n_blocks) {
  __shared__ int smem[32];
  __shared__ int offset;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int pre = 0;
  for (int c = threadIdx.x; c < blockIdx.x; c += blockDim.x) pre += W.partial[c];
  const int off = block_reduce(pre, smem);
  if (threadIdx.x == 0) offset = off;
  __syncthreads();
  const int i = blockIdx.x * kScanChunk + 4 * threadIdx.x;
  const int4 v = load4(W.block_total, i, n_blocks);
  const int s = v.x + v.y + v.z + v.w;
  int wt;
  const int ex = warp_exclusive(s, lane, &wt);
  if (lane == 0) smem[w] = wt;
  __syncthreads();
  if (w == 0) {
    int tot;
    const int e = warp_exclusive(lane < (blockDim.x >> 5) ? smem[lane] : 0, lane, &tot);
    smem[lane] = e;
  }
  __syncthreads();
  const int base = offset + smem[w] + ex;
  if (i < n_blocks) W.block_base[i] = base;
  if (i + 1 < n_blocks) W.block_base[i + 1] = base + v.x;
  if (i + 2 < n_blocks) W.block_base[i + 2] = base + v.x + v.y;
  if (i + 3 < n_blocks) W.block_base[i + 3] = base + v.x + v.y + v.z;
}

__global__ void __launch_bounds__(256) k_sort_place(DexBatch B, DexSortWork W, int32_t *__restrict__ perm) {
  const int tile = blockIdx.x;
  const DexEnv E = B.envs[B.tiles[2 * tile]];
  const int loc = B.tiles[2 * tile + 1] + threadIdx.x;
  if (loc >= E.n) return;
  const int p = E.p_off + loc;
  const int ci = W.key[p];
  perm[W.block_base[ci >> 6] + W.cell_start[ci] + W.rank[p]] = p;
}

// Per occupied block: each of its cells' segments of perm put in increasing
// old index, then the cell counts, block total and flag cleared.  The ranks
// within a cell came from atomics in arbitrary order.  The block's entries
// (contiguous in perm, cell after cell) are staged in shared memory in one
// coalesced pass; a cell whose staged entries are already in order (the
// usual case after an env step of drift) is left alone, the entries of any
// other cell are placed at their rank -- the number of smaller entries (old
// indices are distinct) -- each lane counting for every 32nd entry.
//   k_sort_fix      one warp per block of at most kFixRow entries, staged in
//                   the warp's row of shared memory; larger blocks are left;
//   k_sort_fix_big  one CTA per block of more than kFixRow entries, staged in
//                   the CTA's whole shared memory (kFixWarps * kFixRow
//                   entries), its warps taking every kFixWarps-th cell; a
//                   block larger still is done cell by cell (a cell of more
//                   than kFixRow entries insertion-sorted in place by one
//                   lane).  The last CTA to finish resets the list count and
//                   its own ticket.
constexpr int kFixRow = 1024;
constexpr int kFixWarps = 8;  // 256-thread CTAs
constexpr int kFixAll = kFixRow * kFixWarps;

// Ranks of the n entries row[0 .. n) written to seg[rank] (warp-wide).
__device__ __forceinline__ void place_by_rank(const int32_t *row, int32_t *seg, int n, int lane) {
  for (int i = lane; i < n; i += 32) {
    const int32_t v = row[i];
    int r = 0;
    for (int j = 0; j < n; ++j) r += row[j] < v;
    seg[r] = v;
  }
}

// The cell (n entries staged at row[0 .. n), perm segment seg) put in order
// by the calling warp, unless its entries already are.
__device__ __forceinline__ void fix_cell(const int32_t *row, int32_t *seg, int n, int lane) {
  bool ordered = true;
  for (int i = lane; i + 1 < n; i += 32) ordered = ordered && row[i] < row[i + 1];
  if (!__all_sync(kFull, ordered)) place_by_rank(row, seg, n, lane);
}

// Cell counts, block total and flag of a finished block back to zero.
__device__ __forceinline__ void clear_block(DexSortWork &W, int blk, int lane) {
  W.cell_count[(blk << 6) + lane] = 0;
  W.cell_count[(blk << 6) + 32 + lane] = 0;
  if (lane == 0) {
    W.block_total[blk] = 0;
    W.block_flag[blk] = 0u;
  }
}

__global__ void __launch_bounds__(256) k_sort_fix(DexSortWork W, int32_t *__restrict__ perm) {
  __shared__ int32_t rows[kFixWarps][kFixRow];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int32_t *row = rows[wid];
  const int warps = gridDim.x * kFixWarps;
  const int cnt = *reinterpret_cast<volatile int32_t *>(W.counters);
  for (int item = blockIdx.x * kFixWarps + wid; item < cnt; item += warps) {
    const int blk = W.block_list[item];
    const int total = W.block_total[blk];
    if (total > kFixRow) continue;  // k_sort_fix_big
    const int base = W.block_base[blk];
    // lane l owns cells l and l + 32 of the block
    const int n0 = W.cell_count[(blk << 6) + lane], n1 = W.cell_count[(blk << 6) + 32 + lane];
    const int st0 = W.cell_start[(blk << 6) + lane], st1 = W.cell_start[(blk << 6) + 32 + lane];
#pragma unroll 4
    for (int i = lane; i < total; i += 32) row[i] = perm[base + i];
    __syncwarp();
    bool ok0 = true, ok1 = true;
    for (int a = 1; a < n0; ++a) ok0 = ok0 && row[st0 + a - 1] < row[st0 + a];
    for (int a = 1; a < n1; ++a) ok1 = ok1 && row[st1 + a - 1] < row[st1 + a];
    const unsigned bad[2] = {__ballot_sync(kFull, !ok0), __ballot_sync(kFull, !ok1)};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      for (unsigned rest = bad[h]; rest; rest &= rest - 1u) {
        const int owner = __ffs(rest) - 1;
        const int n = __shfl_sync(kFull, h ? n1 : n0, owner);
        const int st = __shfl_sync(kFull, h ? st1 : st0, owner);
        place_by_rank(row + st, perm + base + st, n, lane);
      }
    }
    __syncwarp();
    clear_block(W, blk, lane);
  }
}

__global__ void __launch_bounds__(256) k_sort_fix_big(DexSortWork W, int32_t *__restrict__ perm) {
  __shared__ int32_t all[kFixAll];
  __shared__ int32_t big[256];               // this window's large blocks
  __shared__ int32_t cnt_c[64], start_c[64];  // the block's cell counts and starts
  __shared__ int n_big;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int cnt = *reinterpret_cast<volatile int32_t *>(W.counters);
  // windows of blockDim.x list entries, one per thread, the CTAs taking
  // every gridDim.x-th entry (so that the large blocks spread over all of
  // them): the window's large blocks (k_sort_fix cleared the others' totals)
  // are collected, then done one after the other by the whole CTA
  const int stride = gridDim.x * blockDim.x;
  for (int first = blockIdx.x; first < cnt; first += stride) {
    if (threadIdx.x == 0) n_big = 0;
    __syncthreads();
    const int item = first + gridDim.x * threadIdx.x;
    if (item < cnt) {
      const int blk = W.block_list[item];
      if (W.block_total[blk] > kFixRow) big[atomicAdd(&n_big, 1)] = blk;
    }
    __syncthreads();
    const int nb = n_big;
    for (int k = 0; k < nb; ++k) {
      const int blk = big[k];
      const int total = W.block_total[blk];  // the same for every thread of the CTA
      const int base = W.block_base[blk];
      if (threadIdx.x < 64) {
        cnt_c[threadIdx.x] = W.cell_count[(blk << 6) + threadIdx.x];
        start_c[threadIdx.x] = W.cell_start[(blk << 6) + threadIdx.x];
      }
      if (total <= kFixAll) {
#pragma unroll 4
        for (int i = threadIdx.x; i < total; i += blockDim.x) all[i] = perm[base + i];
      }
      __syncthreads();
      if (total <= kFixAll) {
        for (int c = wid; c < 64; c += kFixWarps) {
          const int n = cnt_c[c];
          if (n > 1) fix_cell(all + start_c[c], perm + base + start_c[c], n, lane);
        }
      } else {
        int32_t *row = all + wid * kFixRow;
        for (int c = wid; c < 64; c += kFixWarps) {
          const int n = cnt_c[c];
          if (n < 2) continue;
          int32_t *seg = perm + base + start_c[c];
          if (n > kFixRow) {
            if (lane == 0) {
              for (int a = 1; a < n; ++a) {
                const int32_t v = seg[a];
                int b = a - 1;
                while (b >= 0 && seg[b] > v) {
                  seg[b + 1] = seg[b];
                  --b;
                }
                seg[b + 1] = v;
              }
            }
            __syncwarp();
            continue;
          }
          for (int i = lane; i < n; i += 32) row[i] = seg[i];
          __syncwarp();
          fix_cell(row, seg, n, lane);
          __syncwarp();
        }
      }
      __syncthreads();  // the block's cells are done before the staging is reused
      if (wid == 0) clear_block(W, blk, lane);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const int ticket = atomicAdd(W.counters + 1, 1);
    if (ticket == (int)gridDim.x - 1) {
      W.counters[0] = 0;
      W.counters[1] = 0;
      __threadfence();
    }
  }
}

// dst[q][i] = src[q][perm[i]] (gather) or dst[q][perm[i]] = src[q][i]
// (scatter, the inverse) for planes q of n 32-bit words.
template <bool kScatter>
__global__ void __launch_bounds__(256) k_permute(const int32_t *__restrict__ perm, const uint32_t *__restrict__ src,
                                                 uint32_t *__restrict__ dst, int n, int planes) {
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int j = __ldg(perm + i);
    for (int q = 0; q < planes; ++q) {
      const size_t o = (size_t)q * n;
      if (kScatter)
        dst[o + j] = __ldg(src + o + i);
      else
        dst[o + i] = __ldg(src + o + j);
    }
  }
}

// Segmented plane copy: blockIdx.y = segment, x-threads over its (plane,
// column) elements, one independent load and store each.  The segment table
// travels in the launch parameters (12 KB of the 32 KB they may hold).
struct SegmentTable {
  DexSegment s[DEXMPM_SEGMENTS_PER_LAUNCH];
};
__global__ void __launch_bounds__(256) k_copy_segments(const __grid_constant__ SegmentTable tab, int planes,
                                                       float *__restrict__ buf, int buf_stride, int mode) {
  const DexSegment s = tab.s[blockIdx.y];
  const long long total = (long long)planes * s.count;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(e / s.count), i = (int)(e - (long long)q * s.count);
    float *o = s.other + (size_t)q * s.other_stride + i;
    float *b = buf + (size_t)q * buf_stride + s.offset + i;
    if (mode == DEXMPM_SEGMENTS_GATHER)
      *b = *o;
    else if (mode == DEXMPM_SEGMENTS_SCATTER)
      *o = *b;
    else
      *o += *b;
  }
}

int check_launch() { return cudaGetLastError() == cudaSuccess ? DEXMPM_OK : DEXMPM_ERR_LAUNCH; }

int device_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                 cudaSuccess || sms < 1)
    return 1;
  return sms;
}

// cell_count and cell_start are read and written as int2, block_total as int4
bool work_ok(const DexSortWork *w) {
  return w && w->cell_count && w->cell_start && w->block_total && w->block_base && w->block_flag && w->block_list &&
         w->rank && w->key && w->partial && w->counters && (reinterpret_cast<uintptr_t>(w->cell_count) & 7u) == 0 &&
         (reinterpret_cast<uintptr_t>(w->cell_start) & 7u) == 0 && (reinterpret_cast<uintptr_t>(w->block_total) & 15u) == 0;
}

bool batch_ok(const DexBatch *b) {
  return b && b->envs && b->tiles && b->n_tiles >= 0 && b->n_blocks > 0 && b->n_particles > 0 &&
         (b->tile_size == 64 || b->tile_size == 128 || b->tile_size == 256);
}

}  // namespace

extern "C" {

int dexmpm_sort(const DexBatch *b, const DexSortWork *w, const float *s, float *sorted_s, int32_t *perm,
                dexmpm_stream_t stream) {
  if (!batch_ok(b) || !work_ok(w) || !s || !sorted_s || !perm || s == sorted_s) return DEXMPM_ERR_ARG;
  const int chunks = (b->n_blocks + kScanChunk - 1) / kScanChunk;
  if (chunks > kScanThreads) return DEXMPM_ERR_ARG;  // more than 4M blocks
  cudaStream_t st = (cudaStream_t)stream;
  const int persistent = 4 * device_sms();
  if (b->n_tiles > 0) {
    k_sort_count<<<b->n_tiles, b->tile_size, 0, st>>>(*b, *w, s);
    if (int rc = check_launch()) return rc;
  }
  k_sort_cells<<<persistent, 256, 0, st>>>(*w);
  if (int rc = check_launch()) return rc;
  k_scan_chunks<<<chunks, kScanThreads, 0, st>>>(*w, b->n_blocks);
  if (int rc = check_launch()) return rc;
  k_scan_apply<<<chunks, kScanThreads, 0, st>>>(*w, b->n_blocks);
  if (int rc = check_launch()) return rc;
  if (b->n_tiles > 0) {
    k_sort_place<<<b->n_tiles, b->tile_size, 0, st>>>(*b, *w, perm);
    if (int rc = check_launch()) return rc;
  }
  k_sort_fix<<<persistent, 256, 0, st>>>(*w, perm);
  if (int rc = check_launch()) return rc;
  k_sort_fix_big<<<persistent, 256, 0, st>>>(*w, perm);
  if (int rc = check_launch()) return rc;
  return dexmpm_permute(perm, s, sorted_s, b->n_particles, DEXMPM_STATE_PLANES, 0, stream);
}

int dexmpm_copy_segments(const DexSegment *seg, int n, int planes, float *buf, int buf_stride, int mode,
                         int max_count, dexmpm_stream_t stream) {
  if (n < 0 || planes < 0 || max_count < 0 || buf_stride < 0 || mode < DEXMPM_SEGMENTS_GATHER ||
      mode > DEXMPM_SEGMENTS_SCATTER_ADD)
    return DEXMPM_ERR_ARG;
  if (n == 0 || planes == 0 || max_count == 0) return DEXMPM_OK;
  if (!seg || !buf) return DEXMPM_ERR_ARG;
  const long long elems = (long long)planes * max_count;
  const int per_seg = (int)((elems + 255) / 256 < 512 ? (elems + 255) / 256 : 512);
  for (int first = 0; first < n; first += DEXMPM_SEGMENTS_PER_LAUNCH) {
    const int m = n - first < DEXMPM_SEGMENTS_PER_LAUNCH ? n - first : DEXMPM_SEGMENTS_PER_LAUNCH;
    SegmentTable tab;
    for (int i = 0; i < m; ++i) tab.s[i] = seg[first + i];
    const dim3 grid(per_seg, m);
    k_copy_segments<<<grid, 256, 0, (cudaStream_t)stream>>>(tab, planes, buf, buf_stride, mode);
    if (int rc = check_launch()) return rc;
  }
  return DEXMPM_OK;
}

int dexmpm_permute(const int32_t *perm, const void *src, void *dst, int n, int planes, int inverse,
                   dexmpm_stream_t stream) {
  if (!perm || !src || !dst || src == dst || n < 0 || planes < 0) return DEXMPM_ERR_ARG;
  if (n == 0 || planes == 0) return DEXMPM_OK;
  const int per_sm = 8;
  long long want = ((long long)n + 255) / 256;
  const long long cap = (long long)per_sm * device_sms();
  const int grid = (int)(want < cap ? want : cap);
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t *in = static_cast<const uint32_t *>(src);
  uint32_t *out = static_cast<uint32_t *>(dst);
  if (inverse)
    k_permute<true><<<grid, 256, 0, st>>>(perm, in, out, n, planes);
  else
    k_permute<false><<<grid, 256, 0, st>>>(perm, in, out, n, planes);
  return check_launch();
}

}  // extern "C"
