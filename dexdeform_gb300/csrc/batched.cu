// batched.cu -- the batched MLS-MPM substep and its adjoint for sm_103a.
//
// Work decomposition (one launch per phase for all environments):
//   * particle phases (P2G, G2P, their adjoints, and G2P fused with the next
//     substep's P2G): one CTA per tile of `tile_size` particles of one env
//     (tiles never straddle envs);
//   * grid phases (grid update and its adjoint): a persistent grid of at most
//     the resident number of CTAs walking the active-block list, 64 threads
//     per block.
// Scatters (P2G and the G2P adjoint) pre-reduce in the warp: the warp groups
// its lanes by stencil base cell (one match instruction and a prefix sum of
// the group sizes), equal bases form segments, and each segment's 27 node
// sums are formed through a transposed shared-memory buffer and added with
// one 8-byte vector atomic per node and component pair.  Grid storage is an array of slots (mass/momentum grid,
// post-update velocities, active-block list per slot): forward substeps
// alternate two slots and each grid update clears the slot the previous
// substep used; the adjoint of an env step reads the slots its recomputed
// substeps left behind (and the tape of their SVDs and stresses) and clears
// each one after use, so nothing is recomputed inside the adjoint and nothing
// is memset per substep.
//
// Arithmetic follows mpm/csrc/integrator.cu (kernels cited per function); the
// SVD and stress use the cancellation-free forms of mpm_math.cuh.
#include <cuda_runtime.h>
#include <stdint.h>
#include <atomic>
#include <climits>

#include "mpm_math.cuh"
#include "../../include/dexmpm.h"

using namespace dexmpm;

// Compile-time tuning knobs.  Defaults were picked by timing every kernel on
// GB300 over the 64-env batch: minimum resident CTAs per SM (register caps:
// P2G and fused G2P/P2G 85, G2P adjoint 85, P2G adjoint 128, the fused adjoint
// 96 -- five 128-thread CTAs per SM --, grid update and its adjoint 64 -- four
// 256-thread CTAs per SM, so that the persistent grid kernels cover the
// active blocks in fewer rounds) and the unrolling of the outer loop over the
// 27 stencil nodes in the adjoints (full unrolling keeps the weight arrays out
// of local memory).
#ifndef DEX_P2G_MINB
#define DEX_P2G_MINB 3
#endif
#ifndef DEX_P2G_GRAD_MINB
#define DEX_P2G_GRAD_MINB 4
#endif
#ifndef DEX_P2G2G_GRAD_MINB
#define DEX_P2G2G_GRAD_MINB 5
#endif
#ifndef DEX_GRID_OP_MINB
#define DEX_GRID_OP_MINB 4
#endif
#ifndef DEX_GRID_OP_GRAD_MINB
#define DEX_GRID_OP_GRAD_MINB 4
#endif
#ifndef DEX_G2P2G_MINB
#define DEX_G2P2G_MINB 3
#endif
#ifndef DEX_G2P_GRAD_UNROLL
#define DEX_G2P_GRAD_UNROLL 3
#endif
#ifndef DEX_G2P_GRAD_MINB
#define DEX_G2P_GRAD_MINB 3
#endif
// Scatter: warps with more than DEX_DIRECT_SEGS segments of equal stencil
// base use per-lane atomics instead of the transposed reduction.
#ifndef DEX_DIRECT_SEGS
#define DEX_DIRECT_SEGS 12
#endif
// Scatter: unrolling of the walk over a segment's positions (the sum keeps
// its order, so the unrolling changes no result).
#ifndef DEX_WALK_UNROLL
#define DEX_WALK_UNROLL 4
#endif
constexpr int kG2pGradUnroll = DEX_G2P_GRAD_UNROLL;
constexpr int kWalkUnroll = DEX_WALK_UNROLL;

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int PX = 0, PV = 3, PF = 6, PC = 15;  // state plane offsets
constexpr float kBlockReach = 2.6f;  // >= 1.5 sqrt(3): block centre to its farthest cell, in cells

__device__ __forceinline__ f3 ldf3(const float *__restrict__ S, int N, int plane, int p) {
  return mk3(__ldg(S + (size_t)plane * N + p), __ldg(S + (size_t)(plane + 1) * N + p),
             __ldg(S + (size_t)(plane + 2) * N + p));
}
__device__ __forceinline__ void stf3(float *S, int N, int plane, int p, f3 v) {
  S[(size_t)plane * N + p] = v.x;
  S[(size_t)(plane + 1) * N + p] = v.y;
  S[(size_t)(plane + 2) * N + p] = v.z;
}
__device__ __forceinline__ m33 ldm33(const float *__restrict__ S, int N, int plane, int p) {
  m33 m;
#pragma unroll
  for (int i = 0; i < 9; ++i) m.a[i / 3][i % 3] = __ldg(S + (size_t)(plane + i) * N + p);
  return m;
}
// A load that is not merged with an earlier one of the same address: the
// caller reads the value again instead of keeping it in a register between.
__device__ __forceinline__ float ld_again(const float *a) {
  float v;
  asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(a));
  return v;
}
__device__ __forceinline__ m33 ldm33_again(const float *S, int N, int plane, int p) {
  m33 m;
#pragma unroll
  for (int i = 0; i < 9; ++i) m.a[i / 3][i % 3] = ld_again(S + (size_t)(plane + i) * N + p);
  return m;
}
__device__ __forceinline__ void stm33(float *S, int N, int plane, int p, const m33 &m) {
#pragma unroll
  for (int i = 0; i < 9; ++i) S[(size_t)(plane + i) * N + p] = m.a[i / 3][i % 3];
}

// L2 prefetch of the cache lines holding particles p0 .. p1 of one plane.
__device__ __forceinline__ void prefetch_plane(const float *plane, int p0, int p1) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(plane + p0));
  asm volatile("prefetch.global.L2 [%0];" ::"l"(plane + p1));
}

// SVD tape: the recomputed forward P2G stores each particle's SVD of F_tmp
// and its stress in kTapePlanes planes (U 0-8, V 9-17, sigma 18-20,
// sigma - 1 21-23, P 24-32, before the -dt vol 4 inv_dx^2 scale) so that the
// P2G adjoint reads them instead of repeating the SVD and return mapping.
constexpr int kTapePlanes = 33;
static_assert(kTapePlanes == DEXMPM_TAPE_PLANES, "tape layout");
// The tape is written with streaming stores and read once with evict-first
// loads: it is consumed by the adjoint long after it is written, so it should
// not displace the grid slots and states the next substeps reuse from L2.
__device__ __forceinline__ void tape_put(float *T, int N, int plane, int p, float v) {
  __stcs(T + (size_t)plane * N + p, v);
}
__device__ __forceinline__ float tape_get(const float *T, int N, int plane, int p) {
  return __ldcs(T + (size_t)plane * N + p);
}
__device__ __forceinline__ void store_tape(float *T, int N, int p, const SVD3 &sv, const m33 &P) {
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    tape_put(T, N, i, p, sv.U.a[i / 3][i % 3]);
    tape_put(T, N, 9 + i, p, sv.V.a[i / 3][i % 3]);
    tape_put(T, N, 24 + i, p, P.a[i / 3][i % 3]);
  }
  tape_put(T, N, 18, p, sv.s.x); tape_put(T, N, 19, p, sv.s.y); tape_put(T, N, 20, p, sv.s.z);
  tape_put(T, N, 21, p, sv.d.x); tape_put(T, N, 22, p, sv.d.y); tape_put(T, N, 23, p, sv.d.z);
}
__device__ __forceinline__ m33 tape_m33(const float *T, int N, int plane, int p) {
  m33 m;
#pragma unroll
  for (int i = 0; i < 9; ++i) m.a[i / 3][i % 3] = tape_get(T, N, plane + i, p);
  return m;
}
__device__ __forceinline__ SVD3 load_svd(const float *__restrict__ T, int N, int p) {
  SVD3 sv;
  sv.U = tape_m33(T, N, 0, p);
  sv.V = tape_m33(T, N, 9, p);
  sv.s = mk3(tape_get(T, N, 18, p), tape_get(T, N, 19, p), tape_get(T, N, 20, p));
  sv.d = mk3(tape_get(T, N, 21, p), tape_get(T, N, 22, p), tape_get(T, N, 23, p));
  return sv;
}

// Stencil-node arithmetic: affine terms M dpos are built from M's columns,
// M ((i, j, k) - fx) h = m0 + i h M0 + j h M1 + k h M2 with m0 = -h M fx, one
// step per axis (folded to nothing / an add when the offset is a constant).
__device__ __forceinline__ f3 step3(f3 a, f3 c, int i) { return i == 0 ? a : (i == 1 ? a + c : a + c * 2.f); }
__device__ __forceinline__ f3 mcol(const m33 &M, int c) { return mk3(M.a[0][c], M.a[1][c], M.a[2][c]); }

__device__ __forceinline__ float *slot_grid(const DexBatch &B, int k) {
  return B.grid + (size_t)k * B.n_blocks * 256;  // 64 cells x float4 per block
}
__device__ __forceinline__ float *slot_vout(const DexBatch &B, int k) {
  return B.vout + (size_t)k * B.n_blocks * 256;
}
__device__ __forceinline__ uint32_t *slot_flags(const DexBatch &B, int k) {
  return B.block_flag + (size_t)k * B.n_blocks;
}
__device__ __forceinline__ int32_t *slot_list(const DexBatch &B, int k) {
  return B.block_list + (size_t)k * B.n_blocks;
}


// Grid cells are stored in 4^3 blocks of 64 float4 cells: cell (x, y, z) of an
// env is entry ((blk_off + (x/4 * nby + y/4) * nbz + z/4) * 64 + (x%4) * 16 +
// (y%4) * 4 + z%4), nby = gy/4, nbz = gz/4.  The 27 stencil nodes of base
// (b0, b1, b2) are then x[i] + y[j] + z[k] with per-axis terms.
struct NodeCells {
  int x[3], y[3], z[3];
  __device__ __forceinline__ int at(int i, int j, int k) const { return x[i] + y[j] + z[k]; }
};
__device__ __forceinline__ NodeCells node_cells(const DexEnv &E, const int base[3]) {
  const int nbz = E.gz >> 2, nyz = (E.gy >> 2) * nbz;
  NodeCells c;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int x = base[0] + d, y = base[1] + d, z = base[2] + d;
    c.x[d] = ((E.blk_off + (x >> 2) * nyz) << 6) + ((x & 3) << 4);
    c.y[d] = (((y >> 2) * nbz) << 6) + ((y & 3) << 2);
    c.z[d] = ((z >> 2) << 6) + (z & 3);
  }
  return c;
}

__device__ __forceinline__ bool stencil_in_grid(const DexEnv &E, const Stencil &st) {
  return st.base[0] >= 0 && st.base[1] >= 0 && st.base[2] >= 0 && st.base[0] + 2 < E.gx &&
         st.base[1] + 2 < E.gy && st.base[2] + 2 < E.gz;
}

// G2P gather of the grid velocities g_n of the 27 stencil nodes with weights
// w_n = wx_i wy_j wz_k: s0 = sum w g and the offset moments si = sum i w g,
// sj = sum j w g, sk = sum k w g, summed one axis at a time (z within a row,
// then y, then x) so that no node needs its own weight product.  Lanes with
// ok false read nothing and get zeros.
struct Moments {
  f3 s0, si, sj, sk;
};
__device__ __forceinline__ f3 xyz(float4 g) { return mk3(g.x, g.y, g.z); }
__device__ __forceinline__ Moments gather_moments(const float4 *__restrict__ grid, const NodeCells &nc,
                                                  const Stencil &st, bool ok) {
  Moments o;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    f3 q, qj, qk;  // sums over the x-row i: w_y w_z g, j w_y w_z g, k w_y w_z g
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const f3 g0 = xyz(ok ? __ldg(grid + nc.at(i, j, 0)) : z4);
      const f3 g1 = xyz(ok ? __ldg(grid + nc.at(i, j, 1)) : z4);
      const f3 g2 = xyz(ok ? __ldg(grid + nc.at(i, j, 2)) : z4);
      const f3 t1 = g1 * st.w[2][1];
      const f3 pz = g0 * st.w[2][0] + t1 + g2 * st.w[2][2];  // sum_k w_z g
      const f3 kz = t1 + g2 * (2.f * st.w[2][2]);           // sum_k k w_z g
      const float wy = st.w[1][j];
      if (j == 0) {
        q = pz * wy;
        qk = kz * wy;
      } else {
        q += pz * wy;
        qk += kz * wy;
        qj = j == 1 ? pz * wy : qj + pz * (2.f * wy);
      }
    }
    const float wx = st.w[0][i];
    if (i == 0) {
      o.s0 = q * wx;
      o.sj = qj * wx;
      o.sk = qk * wx;
    } else {
      o.s0 += q * wx;
      o.sj += qj * wx;
      o.sk += qk * wx;
      o.si = i == 1 ? q * wx : o.si + q * (2.f * wx);
    }
  }
  return o;
}

__device__ __forceinline__ void red_add4(float *dst, float a, float b, float c, float d) {
  atomicAdd(reinterpret_cast<float4 *>(dst), make_float4(a, b, c, d));
}


// ------------------------------------------------ transposed warp scatter
// The scatter kernels add 27 node contributions per particle to the grid.
// Every lane keeps its own particle; the warp gives its lanes positions such
// that equal stencil bases (the same 27 target cells) form contiguous segments
// (lanes of equal key found with a match instruction, segments placed by a
// warp prefix sum of their sizes).  Per group of up to 16 nodes every lane
// stores its float4 per node at its position's column of a per-warp shared
// buffer; then lane l owns component pair (l & 1) of node (l >> 1), sums it
// over each segment with plain loads, and the segment's total goes to the
// grid in one 8-byte vector atomic.  Rows are padded to 132 floats so that the
// loads (8 B per lane, one row per lane pair) are free of bank conflicts.
// The segment's target cells come from a per-warp table of its head lane's
// per-axis cell terms (NodeCells), written once per warp.  Warps with more
// than DEX_DIRECT_SEGS segments (about one particle per cell) add their
// contributions with per-lane float4 atomics instead.
constexpr int kRedRow = 132;  // floats per node row (32 lanes x 4 + 4 pad)
constexpr int kDirectSegs = DEX_DIRECT_SEGS;
constexpr int kSegTable = 16 * kRedRow;                      // after the 16 node rows
// + 9 cell terms per segment, rounded up to 4 floats: every warp's buffer
// must start on a 16-byte boundary for the float4 row stores and float2
// row loads (a stride of 2,166 floats, with 6 segments, misaligns odd warps)
constexpr int kRedWarpFloats = (kSegTable + 9 * kDirectSegs + 3) & ~3;
constexpr size_t kScatterSmemPerWarp = sizeof(float) * kRedWarpFloats;
static_assert(kRedWarpFloats % 4 == 0, "per-warp scatter buffers must stay 16-byte aligned");
static_assert(kDirectSegs >= 1 && kDirectSegs <= 32, "a warp has 1 to 32 segments");

__device__ __forceinline__ float *warp_red_buffer() {
  extern __shared__ float4 s_dyn[];
  return reinterpret_cast<float *>(s_dyn) + (threadIdx.x >> 5) * kRedWarpFloats;
}

// Per-lane values parked in a column of shared memory (entry k at base[32 k]:
// the 32 lanes of a warp hit 32 banks).
__device__ __forceinline__ void stash3(float *base, int k, f3 a) {
  base[32 * k] = a.x;
  base[32 * (k + 1)] = a.y;
  base[32 * (k + 2)] = a.z;
}
__device__ __forceinline__ f3 unstash3(const float *base, int k) {
  return mk3(base[32 * k], base[32 * (k + 1)], base[32 * (k + 2)]);
}
__device__ __forceinline__ void stash33(float *base, int k, const m33 &a) {
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) base[32 * (k + 3 * r + c)] = a.a[r][c];
}
__device__ __forceinline__ m33 unstash33(const float *base, int k) {
  m33 a;
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) a.a[r][c] = base[32 * (k + 3 * r + c)];
  return a;
}

// This lane's position in the warp's segment order and the segment
// structure of that order (key INT_MAX: no contribution, placed last).
struct Ranked {
  int r;           // position of this lane
  unsigned heads;  // bit q: position q starts a segment of live lanes
  int n_live;      // live lanes occupy positions [0, n_live)
  bool head;       // this lane starts its segment
};
__device__ __forceinline__ Ranked rank_lanes(int key, int lane) {
  // Lanes with equal keys found in one match; segments are ordered by their
  // lowest lane, positions within a segment by lane, dead lanes (INT_MAX)
  // after all live ones.
  const unsigned same = __match_any_sync(kFull, key);
  const unsigned below = (1u << lane) - 1u;
  const bool live = key != INT_MAX;
  const bool lead = (same & below) == 0u;
  const int size = (lead && live) ? __popc(same) : 0;
  int incl = size;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int t = __shfl_up_sync(kFull, incl, d);
    if (lane >= d) incl += t;
  }
  Ranked R;
  R.n_live = __shfl_sync(kFull, incl, 31);
  const int seg0 = __shfl_sync(kFull, incl - size, __ffs(same) - 1);
  const int within = __popc(same & below);
  R.r = (live ? seg0 : R.n_live) + within;
  R.head = lead && live;
  R.heads = __reduce_or_sync(kFull, R.head ? (1u << seg0) : 0u);
  return R;
}

// Head lanes of the first kDirectSegs segments store their cell terms in the
// warp's segment table (entry = segment ordinal); a __syncwarp must follow
// before red_walk reads it.
__device__ __forceinline__ void put_segment(float *red, const Ranked &R, const NodeCells &nc) {
  const int sidx = __popc(R.heads & ((1u << R.r) - 1u));
  if (R.head && sidx < kDirectSegs) {
    int *t = reinterpret_cast<int *>(red + kSegTable) + 9 * sidx;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      t[d] = nc.x[d];
      t[3 + d] = nc.y[d];
      t[6 + d] = nc.z[d];
    }
  }
}

__device__ __forceinline__ void red_put(float *red, int c, int pos, float a, float b, float d, float e) {
  *reinterpret_cast<float4 *>(red + c * kRedRow + 4 * pos) = make_float4(a, b, d, e);
}

// Sum the stored rows of nodes node0 .. node0 + n_nodes - 1 over every segment
// of positions and add them at the segment's stencil nodes (cell terms from
// the segment table).  Warp-uniform; at most kDirectSegs segments.
__device__ __forceinline__ void red_walk(const float *red, const Ranked &R, int node0, int n_nodes, float *grid,
                                         int lane) {
  const int c = lane >> 1, h = lane & 1;
  const bool act = c < n_nodes;
  const int n = act ? node0 + c : 0;
  const int ni = n / 9, nj = (n / 3) % 3, nk = n % 3;
  const float *col = red + c * kRedRow + 2 * h;
  const int *tab = reinterpret_cast<const int *>(red + kSegTable);
  unsigned rest = R.heads;
  for (int sidx = 0; rest; ++sidx) {
    const int start = __ffs(rest) - 1;
    rest &= rest - 1u;
    const int end = rest ? __ffs(rest) - 1 : R.n_live;
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll kWalkUnroll
    for (int q = start; q < end; ++q) {
      const float2 t = *reinterpret_cast<const float2 *>(col + 4 * q);
      acc.x += t.x;
      acc.y += t.y;
    }
    if (act) {
      const int *t = tab + 9 * sidx;
      const int ci = t[ni] + t[3 + nj] + t[6 + nk];
      atomicAdd(reinterpret_cast<float2 *>(grid + 4 * (size_t)ci + 2 * h), acc);
    }
  }
}

// Reduce-scatter of 16 values over the warp: on return lane l holds the
// warp sum of value ((l >> 4) & 1) * 8 + ((l >> 3) & 1) * 4 + ((l >> 2) & 1) * 2
// + ((l >> 1) & 1) (lanes l and l ^ 1 hold the same value).  16 shuffles in
// place of 16 x 5 for separate butterflies.
__device__ __forceinline__ float warp_reduce_scatter16(float v[16], int lane) {
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const bool up = lane & 16;
    const float r = __shfl_xor_sync(kFull, up ? v[i] : v[i + 8], 16);
    v[i] = (up ? v[i + 8] : v[i]) + r;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const bool up = lane & 8;
    const float r = __shfl_xor_sync(kFull, up ? v[i] : v[i + 4], 8);
    v[i] = (up ? v[i + 4] : v[i]) + r;
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const bool up = lane & 4;
    const float r = __shfl_xor_sync(kFull, up ? v[i] : v[i + 2], 4);
    v[i] = (up ? v[i + 2] : v[i]) + r;
  }
  {
    const bool up = lane & 2;
    const float r = __shfl_xor_sync(kFull, up ? v[0] : v[1], 2);
    v[0] = (up ? v[1] : v[0]) + r;
  }
  return v[0] + __shfl_xor_sync(kFull, v[0], 1);
}
__device__ __forceinline__ int reduce_scatter16_index(int lane) {
  return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
}

// Mark the 1 to 8 blocks (2 per axis at most) that a stencil with base b
// touches as active in slot X, appending newly marked ones to its list.  The
// flags of all of them are read first (independent loads), then the unmarked
// ones are claimed with an exchange.
__device__ __forceinline__ void mark_blocks(const DexBatch &B, const DexEnv &E, int X, const int b[3]) {
  const int nby = E.gy >> 2, nbz = E.gz >> 2;
  const int bx = b[0] >> 2, by = b[1] >> 2, bz = b[2] >> 2;
  const bool ex = ((b[0] + 2) >> 2) != bx, ey = ((b[1] + 2) >> 2) != by, ez = ((b[2] + 2) >> 2) != bz;
  const int blk0 = E.blk_off + (bx * nby + by) * nbz + bz;
  uint32_t *flags = slot_flags(B, X);
  uint32_t f[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const bool use = (!(c & 4) || ex) && (!(c & 2) || ey) && (!(c & 1) || ez);
    const int blk = blk0 + (((c >> 2) & 1) * nby + ((c >> 1) & 1)) * nbz + (c & 1);
    f[c] = use ? *reinterpret_cast<volatile uint32_t *>(flags + blk) : 1u;
  }
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int blk = blk0 + (((c >> 2) & 1) * nby + ((c >> 1) & 1)) * nbz + (c & 1);
    if (f[c] == 0u && atomicExch(flags + blk, 1u) == 0u) {
      const int at = atomicAdd(B.block_count + X, 1);
      slot_list(B, X)[at] = blk;
    }
  }
}

__device__ __forceinline__ void load_pose(const float *__restrict__ P, int b, BodyPose &o) {
  float4 a = __ldg(reinterpret_cast<const float4 *>(P) + 2 * b);
  float4 q = __ldg(reinterpret_cast<const float4 *>(P) + 2 * b + 1);
  o.p = mk3(a.x, a.y, a.z);
  o.q = mkq(q.x, q.y, q.z, q.w);
}
__device__ __forceinline__ void load_shape(const float *__restrict__ S, int b, BodyShape &o) {
  float4 a = __ldg(reinterpret_cast<const float4 *>(S) + 2 * b);
  float4 q = __ldg(reinterpret_cast<const float4 *>(S) + 2 * b + 1);
  o.tfsr = mkq(a.x, a.y, a.z, a.w);
  o.args = mkq(q.x, q.y, q.z, q.w);
}

// Bodies of env E that can touch some cell of the 4^3 block (bx, by, bz)
// (body_may_touch with the block centre and its half-diagonal 1.5 sqrt(3) dx):
// bit b for body b, the same in every lane of the warp (one lane per body).
// Skipping the other bodies leaves every node of the block as it was.
__device__ __forceinline__ uint32_t bodies_near_block(const DexBatch &B, const DexEnv &E, const float *__restrict__ pose,
                                                      int bx, int by, int bz, int nbod) {
  const int lane = threadIdx.x & 31;
  bool near = false;
  if (lane < nbod) {
    BodyPose cur;
    BodyShape sh;
    load_pose(pose, E.body_off + lane, cur);
    load_shape(B.body_shape, E.body_off + lane, sh);
    const f3 c = mk3((4 * bx + 1.5f) * E.dx, (4 * by + 1.5f) * E.dx, (4 * bz + 1.5f) * E.dx);
    near = body_may_touch(c, kBlockReach * E.dx, cur, sh);
  }
  return __ballot_sync(kFull, near);
}

// =================================================================== P2G
// integrator.cu:84-100 (compute_svd) fused with :312-394 (p2g) for the
// particle of this lane: SVD of F_tmp = (I + dt C) F, return mapping, the
// projected F (to Fout's F planes), the tape, and the APIC momentum + stress
// scatter into grid slot X, marking the blocks the stencil touches.  `live`
// lanes contribute; every lane of the warp calls it.
// Per-particle material: mass, volume, mu, lambda, yield stress.
struct Material {
  float m, vol, mu, lam, ys;
};
__device__ __forceinline__ Material load_material(const DexBatch &B, int p) {
  const int N = B.n_particles;
  return Material{__ldg(B.mass + p), __ldg(B.vol + p), __ldg(B.mu_lam_yield + p), __ldg(B.mu_lam_yield + N + p),
                  __ldg(B.mu_lam_yield + 2 * N + p)};
}

__device__ __forceinline__ void p2g_lane(const DexBatch &B, const DexEnv &E, int X, int p, bool live, f3 x, f3 v,
                                         const m33 &F, const m33 &C, const Material &mat, float *Fout, float *tape,
                                         int lane) {
  const int N = B.n_particles;
  Stencil st;
  make_stencil(x, E.inv_dx, st);
  int key = INT_MAX;
  if (live) {
    if (stencil_in_grid(E, st)) {
      key = (st.base[0] * E.gy + st.base[1]) * E.gz + st.base[2];
    } else {
      atomicOr(B.error, DEXMPM_ERR_OUT_OF_GRID);
      live = false;
    }
  }
  if (!live) st.base[0] = st.base[1] = st.base[2] = 0;
  float *red = warp_red_buffer();
  const Ranked R = rank_lanes(key, lane);

  const float m = live ? mat.m : 0.f;
  const float vol = mat.vol, mu = mat.mu, lam = mat.lam, ys = mat.ys;
  const m33 Et = deviation_tmp(F, C, E.dt);
  const SVD3 sv = svd3_from_deviation(Et);
  m33 Ft = Et;
  Ft.a[0][0] += 1.f; Ft.a[1][1] += 1.f; Ft.a[2][2] += 1.f;
  const Plastic pl = constitutive(sv, Ft, mu, lam, ys);
  if (Fout != nullptr && live) stm33(Fout, N, PF, p, pl.newF);
  if (tape != nullptr && live) store_tape(tape, N, p, sv, pl.P);

  const float scale = live ? -E.dt * vol * 4.f * E.inv_dx * E.inv_dx : 0.f;
  const m33 A = pl.P * scale + C * m;
  // node momentum mom + A dpos, dpos = ((i, j, k) - fx) dx, as b0 + i a0 +
  // j a1 + k a2 with the columns a of A dx: the node offsets are constants of
  // the unrolled loops, so the sums are shared between nodes
  const f3 a0 = mcol(A, 0) * E.dx, a1 = mcol(A, 1) * E.dx, a2 = mcol(A, 2) * E.dx;
  const f3 b0 = v * m - (a0 * st.fx[0] + a1 * st.fx[1] + a2 * st.fx[2]);
  float *grid = slot_grid(B, X);

  if (__popc(R.heads) > kDirectSegs) {
    // nearly one particle per cell: per-lane vector atomics
    const NodeCells nc = node_cells(E, st.base);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float w = st.w[0][i] * st.w[1][j] * st.w[2][k];
          const f3 c = step3(step3(step3(b0, a0, i), a1, j), a2, k) * w;
          if (live) {
            const int ci = nc.at(i, j, k);
            red_add4(grid + 4 * (size_t)ci, c.x, c.y, c.z, m * w);
          }
        }
  } else {
    if (R.head) put_segment(red, R, node_cells(E, st.base));
#pragma unroll
    for (int g = 0; g < 2; ++g) {
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int n = 16 * g + c;
        if (n < 27) {
          const int i = n / 9, j = (n / 3) % 3, k = n % 3;
          const float w = st.w[0][i] * st.w[1][j] * st.w[2][k];
          const f3 cv = step3(step3(step3(b0, a0, i), a1, j), a2, k) * w;
          red_put(red, c, R.r, cv.x, cv.y, cv.z, m * w);
        }
      }
      __syncwarp();
      red_walk(red, R, 16 * g, g == 0 ? 16 : 11, grid, lane);
      __syncwarp();
    }
  }

  if (live && R.head) mark_blocks(B, E, X, st.base);
}

// P2G of state S into slot X (projected F to Snext, nullable; tape nullable).
__global__ void __launch_bounds__(256, DEX_P2G_MINB) k_p2g(DexBatch B, int X, const float *__restrict__ S,
                                                           float *__restrict__ Snext, float *__restrict__ tape) {
  const int tile = blockIdx.x;
  const DexEnv E = B.envs[B.tiles[2 * tile]];
  const int first = B.tiles[2 * tile + 1];
  const int N = B.n_particles;
  const int lane = threadIdx.x & 31;
  const int loc = first + threadIdx.x;
  const bool in = loc < E.n;
  const int p = E.p_off + (in ? loc : 0);
  p2g_lane(B, E, X, p, in, ldf3(S, N, PX, p), ldf3(S, N, PV, p), ldm33(S, N, PF, p), ldm33(S, N, PC, p),
           load_material(B, p), Snext, tape, lane);
}

// G2P of substep t fused with P2G of substep t + 1 (integrator.cu:1059-1109
// then :84-100, :312-394).  From x_t in S and the velocities of grid slot Xg:
// x, v, C of state t + 1 to Snext; then, with F_{t+1} from Snext's F planes,
// the P2G of state t + 1 into slot Xs, its projected F to S2's F planes and
// its tape.  S2 may be S: only x is read from S and only F is written to S2.
__global__ void __launch_bounds__(256, DEX_G2P2G_MINB) k_g2p2g(DexBatch B, int Xg, int Xs, const float *S,
                                                             float *Snext, float *S2, float *__restrict__ tape) {
  const int tile = blockIdx.x;
  const DexEnv E = B.envs[B.tiles[2 * tile]];
  const int first = B.tiles[2 * tile + 1];
  const int N = B.n_particles;
  const int lane = threadIdx.x & 31;
  const int loc = first + threadIdx.x;
  const bool in = loc < E.n;
  const int p = E.p_off + (in ? loc : 0);
  const f3 x = ldf3(S, N, PX, p);
  // F of state t + 1 (written by the previous P2G), loaded before the gather
  const m33 F1 = ldm33(Snext, N, PF, p);
  Stencil st;
  make_stencil(x, E.inv_dx, st);
  const bool ok = in && stencil_in_grid(E, st);  // out-of-grid particles were reported by their P2G
  if (!ok) st.base[0] = st.base[1] = st.base[2] = 0;
  const NodeCells nc = node_cells(E, st.base);
  const float4 *__restrict__ vout = reinterpret_cast<const float4 *>(slot_vout(B, Xg));
  // v = sum w v_n;  C = 4 inv_dx sum w v_n ((i, j, k) - fx)^T
  //   = 4 inv_dx (sum w v_n (i, j, k)^T - v fx^T)
  const Moments mo = gather_moments(vout, nc, st, ok);
  const f3 nv = mo.s0;
  const float c4 = 4.f * E.inv_dx;
  const f3 col[3] = {mo.si - nv * st.fx[0], mo.sj - nv * st.fx[1], mo.sk - nv * st.fx[2]};
  m33 nC;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    nC.a[0][c] = col[c].x * c4;
    nC.a[1][c] = col[c].y * c4;
    nC.a[2][c] = col[c].z * c4;
  }
  f3 nx = x + nv * E.dt;
  const float lo = E.ground_height * E.dx;
  nx.x = fmaxf(fminf(nx.x, (E.gx - 3.f) * E.dx), lo);
  nx.y = fmaxf(fminf(nx.y, (E.gy - 3.f) * E.dx), lo);
  nx.z = fmaxf(fminf(nx.z, (E.gz - 3.f) * E.dx), lo);
  if (ok) {
    stf3(Snext, N, PX, p, nx);
    stf3(Snext, N, PV, p, nv);
    stm33(Snext, N, PC, p, nC);
  }
  p2g_lane(B, E, Xs, p, ok, nx, nv, F1, nC, load_material(B, p), S2, tape, lane);
}

// ============================================================ grid update
// integrator.cu:647-777 on the active blocks of slot X, then (Y >= 0) clearing
// of the blocks slot Y used.  The last CTA to finish resets the list count of
// Y (ticket on done_counter; no CTA waits on another).
__global__ void __launch_bounds__(256, DEX_GRID_OP_MINB) k_grid_op(DexBatch B, int X, int Y, const float *__restrict__ pose,
                                                 const float *__restrict__ next_pose) {
  const int sub = threadIdx.x >> 6, cell = threadIdx.x & 63;
  const int per_cta = blockDim.x >> 6;
  const int cnt = *reinterpret_cast<volatile int *>(B.block_count + X);
  const float4 *__restrict__ grid = reinterpret_cast<const float4 *>(slot_grid(B, X));
  float4 *vout = reinterpret_cast<float4 *>(slot_vout(B, X));
  const int32_t *list = slot_list(B, X);
  // node velocity of this cell of block (bx, by, bz) of env E
  auto update = [&](const DexEnv &E, int bx, int by, int bz, float4 g, uint32_t near) -> float4 {
    if (!(g.w > kMassEps)) return make_float4(0.f, 0.f, 0.f, 0.f);
    const int gxi = (bx << 2) + (cell >> 4), gyi = (by << 2) + ((cell >> 2) & 3), gzi = (bz << 2) + (cell & 3);
    const float inv_m = 1.f / g.w;
    f3 v = mk3(g.x * inv_m, g.y * inv_m, g.z * inv_m) + mk3(E.gravity[0], E.gravity[1], E.gravity[2]) * E.dt;
    const f3 gx = mk3(gxi * E.dx, gyi * E.dx, gzi * E.dx);
    uint32_t hit = 0u;  // bodies whose contact changed this node's velocity
    for (uint32_t rest = near; rest; rest &= rest - 1u) {
      const int b = __ffs(rest) - 1;
      BodyPose cur, nxt;
      BodyShape sh;
      load_pose(pose, E.body_off + b, cur);
      load_pose(next_pose, E.body_off + b, nxt);
      load_shape(B.body_shape, E.body_off + b, sh);
      if (contact_forward(gx, v, cur, nxt, sh, E.dt)) hit |= 1u << b;
    }
    v = boundary_forward(v, gxi, gyi, gzi, E.gx, E.gy, E.gz, E.ground_friction);
    return make_float4(v.x, v.y, v.z, __uint_as_float(hit));
  };
  // the block's coordinates in its env (a table lookup, not three integer
  // divisions per cell)
  auto coords = [&](int blk, int &bx, int &by, int &bz) {
    const int c = B.block_xyz[blk];
    bx = c >> 20;
    by = (c >> 10) & 1023;
    bz = c & 1023;
  };
  const int stride = gridDim.x * per_cta;
  // the list entries of the next two items and the env of the next one are
  // loaded while this item is processed (each load's address is known then)
  int item = blockIdx.x * per_cta + sub;
  int blk_a = item < cnt ? list[item] : 0;
  int blk_b = item + stride < cnt ? list[item + stride] : 0;
  int env_a = item < cnt ? B.block_env[blk_a] : 0;
  for (; item < cnt; item += stride) {
    const int blk = blk_a, env = env_a;
    env_a = item + stride < cnt ? B.block_env[blk_b] : 0;
    blk_a = blk_b;
    blk_b = item + 2 * stride < cnt ? list[item + 2 * stride] : 0;
    const DexEnv E = B.envs[env];
    int bx, by, bz;
    coords(blk, bx, by, bz);
    const int ci = (blk << 6) + cell;
    const float4 g = grid[ci];
    const uint32_t near = bodies_near_block(B, E, pose, bx, by, bz, E.n_bodies);
    vout[ci] = update(E, bx, by, bz, g, near);
  }
  if (Y < 0) return;
  // clear the blocks slot Y used
  const int cnt_y = *reinterpret_cast<volatile int *>(B.block_count + Y);
  float4 *gy = reinterpret_cast<float4 *>(slot_grid(B, Y));
  const int32_t *list_y = slot_list(B, Y);
  uint32_t *flags_y = slot_flags(B, Y);
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int item = blockIdx.x * per_cta + sub; item < cnt_y; item += gridDim.x * per_cta) {
    const int blk = list_y[item];
    gy[(blk << 6) + cell] = z4;
    if (cell == 0) flags_y[blk] = 0u;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned ticket = atomicAdd(B.done_counter, 1u);
    if (ticket == gridDim.x - 1) {
      B.block_count[Y] = 0;
      *B.done_counter = 0u;
      __threadfence();
    }
  }
}

// =================================================================== G2P
// integrator.cu:1059-1109.
__global__ void __launch_bounds__(256, 3) k_g2p(DexBatch B, int X, const float *__restrict__ S,
                                             float *__restrict__ Snext) {
  const int tile = blockIdx.x;
  const DexEnv E = B.envs[B.tiles[2 * tile]];
  const int first = B.tiles[2 * tile + 1];
  const int loc = first + threadIdx.x;
  if (loc >= E.n) return;
  const int N = B.n_particles;
  const int p = E.p_off + loc;
  const f3 x = ldf3(S, N, PX, p);
  Stencil st;
  make_stencil(x, E.inv_dx, st);
  if (!stencil_in_grid(E, st)) return;  // reported by P2G
  const NodeCells nc = node_cells(E, st.base);
  const float4 *__restrict__ vout = reinterpret_cast<const float4 *>(slot_vout(B, X));
  // v = sum w v_n;  C = 4 inv_dx sum w v_n ((i, j, k) - fx)^T
  const Moments mo = gather_moments(vout, nc, st, true);
  const f3 nv = mo.s0;
  const float c4 = 4.f * E.inv_dx;
  const f3 col[3] = {mo.si - nv * st.fx[0], mo.sj - nv * st.fx[1], mo.sk - nv * st.fx[2]};
  m33 nC;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    nC.a[0][c] = col[c].x * c4;
    nC.a[1][c] = col[c].y * c4;
    nC.a[2][c] = col[c].z * c4;
  }
  f3 nx = x + nv * E.dt;
  const float lo = E.ground_height * E.dx;
  nx.x = fmaxf(fminf(nx.x, (E.gx - 3.f) * E.dx), lo);
  nx.y = fmaxf(fminf(nx.y, (E.gy - 3.f) * E.dx), lo);
  nx.z = fmaxf(fminf(nx.z, (E.gz - 3.f) * E.dx), lo);
  stf3(Snext, N, PX, p, nx);
  stf3(Snext, N, PV, p, nv);
  stm33(Snext, N, PC, p, nC);
}

// ============================================================ G2P adjoint
// integrator.cu:1527-1614 for the particle of this lane: from its position x
// in state s, its velocity vnext in state s + 1 and the incoming gradients of
// state s + 1 (gx, gnv, gC), scatters dL/dv_out into the adjoint grid and
// writes (not adds) the x gradient of state s to G.  Every lane of the warp
// calls it; `in`: the lane has a particle.
__device__ __forceinline__ void g2p_grad_lane(const DexBatch &B, const DexEnv &E, int X, int p, bool in, f3 x,
                                              f3 vnext, f3 gx, f3 gnv, m33 gC, float *G, int lane) {
  const int N = B.n_particles;
  Stencil st;
  make_stencil(x, E.inv_dx, st);
  int key = INT_MAX;
  if (in) {
    if (stencil_in_grid(E, st))
      key = (st.base[0] * E.gy + st.base[1]) * E.gz + st.base[2];
    else
      atomicOr(B.error, DEXMPM_ERR_OUT_OF_GRID);
  }
  const bool live = key != INT_MAX;
  if (!live) st.base[0] = st.base[1] = st.base[2] = 0;
  float *red = warp_red_buffer();
  const Ranked R = rank_lanes(key, lane);
  if (!live) gC = mzero();
  const f3 nx = x + vnext * E.dt;
  const float lo = E.ground_height * E.dx;
  if (nx.x > (E.gx - 3.f) * E.dx || nx.x < lo) gx.x = 0.f;
  if (nx.y > (E.gy - 3.f) * E.dx || nx.y < lo) gx.y = 0.f;
  if (nx.z > (E.gz - 3.f) * E.dx || nx.z < lo) gx.z = 0.f;
  gnv += gx * E.dt;
  if (!live) gnv = mk3(0.f, 0.f, 0.f);
  float w1[3][3];
  make_dweights(st, E.inv_dx, w1);
  const NodeCells nc = node_cells(E, st.base);
  const float4 *__restrict__ vout = reinterpret_cast<const float4 *>(slot_vout(B, X));
  float *vg = B.vout_grad;
  const float c4 = 4.f * E.inv_dx;
  // per node: t = gnv + c4 gC dpos (dpos in cells) = t0 + i t1 + j t2 + k t3,
  // the node's dL/dv_out is w t and its weight-gradient factor v_out . t
  const f3 t1 = mcol(gC, 0) * c4, t2 = mcol(gC, 1) * c4, t3 = mcol(gC, 2) * c4;
  const f3 t0 = gnv - (t1 * st.fx[0] + t2 * st.fx[1] + t3 * st.fx[2]);
  f3 wgv = mk3(0.f, 0.f, 0.f);  // sum of w v_out over the nodes
  // one stencil node: gather-side gradient terms into gx; returns the node's
  // dL/dv_out contribution
  auto node = [&](int i, int j, int k, int ci) -> f3 {
    const float w = st.w[0][i] * st.w[1][j] * st.w[2][k];
    const f3 t = step3(step3(step3(t0, t1, i), t2, j), t3, k);
    const float4 g4 = live ? __ldg(vout + ci) : make_float4(0.f, 0.f, 0.f, 0.f);
    const f3 gv = mk3(g4.x, g4.y, g4.z);
    wgv += gv * w;
    const float gw = dot(gv, t);
    const f3 dw = mk3(w1[0][i] * st.w[1][j] * st.w[2][k], st.w[0][i] * w1[1][j] * st.w[2][k],
                      st.w[0][i] * st.w[1][j] * w1[2][k]);
    gx += dw * gw;
    return t * w;
  };
  if (__popc(R.heads) > kDirectSegs) {
#pragma unroll kG2pGradUnroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const int ci = nc.at(i, j, k);
          const f3 ggv = node(i, j, k, ci);
          if (live) red_add4(vg + 4 * (size_t)ci, ggv.x, ggv.y, ggv.z, 0.f);
        }
  } else {
    put_segment(red, R, nc);
#pragma unroll
    for (int g = 0; g < 2; ++g) {
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int n = 16 * g + c;
        if (n < 27) {
          const int i = n / 9, j = (n / 3) % 3, k = n % 3;
          const int ci = nc.at(i, j, k);
          const f3 ggv = node(i, j, k, ci);
          red_put(red, c, R.r, ggv.x, ggv.y, ggv.z, 0.f);
        }
      }
      __syncwarp();
      red_walk(red, R, 16 * g, g == 0 ? 16 : 11, vg, lane);
      __syncwarp();
    }
  }
  // the C-gradient term of every node: sum_n gC^T v_n (-inv_dx c4 w_n)
  gx += mtv(gC, wgv) * (-E.inv_dx * c4);
  if (live) stf3(G, N, PX, p, gx);
}

// G2P adjoint of substep s: x of state s from S, v of state s + 1 from Snext,
// the gradients of state s + 1 from Gnext; the x gradient of state s to G.
__global__ void __launch_bounds__(256, DEX_G2P_GRAD_MINB) k_g2p_grad(DexBatch B, int X, const float *__restrict__ S,
                                                  const float *__restrict__ Snext, const float *__restrict__ Gnext,
                                                  float *__restrict__ G) {
  const int tile = blockIdx.x;
  const DexEnv E = B.envs[B.tiles[2 * tile]];
  const int first = B.tiles[2 * tile + 1];
  const int N = B.n_particles;
  const int lane = threadIdx.x & 31;
  const int loc = first + threadIdx.x;
  const bool in = loc < E.n;
  const int p = E.p_off + (in ? loc : 0);
  g2p_grad_lane(B, E, X, p, in, ldf3(S, N, PX, p), ldf3(Snext, N, PV, p), ldf3(Gnext, N, PX, p),
                ldf3(Gnext, N, PV, p), ldm33(Gnext, N, PC, p), G, lane);
}

// ===================================================== grid update adjoint
// integrator.cu:779-1057 on the blocks of slot X.  The per-body velocities
// entering each contact are replayed here from (m, mv) instead of being stored
// by the forward; only the contacts the grid update applied (the bits it left
// in vout.w) are replayed.  Body-pose gradients are reduced in the warp before one
// atomic per warp and value.  Every cell of a listed block gets its
// dL/d(mv, m) written (zero where there is no mass), and dL/dv_out and the
// slot's grid are zeroed after they are read, so the next use finds them
// clean; the last CTA resets the slot's list.
__global__ void __launch_bounds__(256, DEX_GRID_OP_GRAD_MINB) k_grid_op_grad(DexBatch B, int X, const float *__restrict__ pose,
                                                      const float *__restrict__ next_pose, float *__restrict__ bgrad,
                                                      float *__restrict__ next_bgrad) {
  const int sub = threadIdx.x >> 6, cell = threadIdx.x & 63;
  const int per_cta = blockDim.x >> 6;
  const int lane = threadIdx.x & 31;
  const bool exact_capsule = (B.flags & DEXMPM_FLAG_EXACT_CAPSULE_GRAD) != 0;
  const int cnt = *reinterpret_cast<volatile int *>(B.block_count + X);
  float4 *grid = reinterpret_cast<float4 *>(slot_grid(B, X));
  const float4 *vo = reinterpret_cast<const float4 *>(slot_vout(B, X));
  float4 *vgrad = reinterpret_cast<float4 *>(B.vout_grad);
  float4 *igrad = reinterpret_cast<float4 *>(B.in_grad);
  const int32_t *list = slot_list(B, X);
  uint32_t *flags = slot_flags(B, X);
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  // uniform trip count per CTA so that whole warps run the body loop together
  const int stride = gridDim.x * per_cta;
  const int trips = (cnt + stride - 1) / stride;
  for (int t = 0; t < trips; ++t) {
    const int item = t * stride + blockIdx.x * per_cta + sub;
    const bool in_list = item < cnt;
    const int blk = in_list ? list[item] : 0;
    const DexEnv E = B.envs[B.block_env[blk]];
    const int c = B.block_xyz[blk];  // the block's coordinates in its env
    const int bx = c >> 20, by = (c >> 10) & 1023, bz = c & 1023;
    const int gxi = (bx << 2) + (cell >> 4), gyi = (by << 2) + ((cell >> 2) & 3), gzi = (bz << 2) + (cell & 3);
    const int ci = (blk << 6) + cell;
    const float4 g = in_list ? grid[ci] : z4;
    const bool active = in_list && g.w > kMassEps;
    const float inv_m = active ? 1.f / g.w : 0.f;
    const f3 gx = mk3(gxi * E.dx, gyi * E.dx, gzi * E.dx);
    // forward replay of the contacts the grid update applied to this node
    // (their bodies' bits in vout.w; the others leave the velocity as it is)
    f3 vin[DEXMPM_MAX_BODIES];
    uint32_t touched = 0u;
    f3 v = mk3(g.x * inv_m, g.y * inv_m, g.z * inv_m) + mk3(E.gravity[0], E.gravity[1], E.gravity[2]) * E.dt;
    const uint32_t applied = active ? __float_as_uint(vo[ci].w) : 0u;
    for (uint32_t rest = applied; rest; rest &= rest - 1u) {
      const int b = __ffs(rest) - 1;
      BodyPose cur, nxt;
      BodyShape sh;
      load_pose(pose, E.body_off + b, cur);
      load_pose(next_pose, E.body_off + b, nxt);
      load_shape(B.body_shape, E.body_off + b, sh);
      f3 before = v;
      if (contact_forward(gx, v, cur, nxt, sh, E.dt)) {
        vin[b] = before;
        touched |= 1u << b;
      }
    }
    const float4 gv4 = active ? vgrad[ci] : z4;
    f3 gv = boundary_backward(mk3(gv4.x, gv4.y, gv4.z), v, gxi, gyi, gzi, E.gx, E.gy, E.gz, E.ground_friction);
    // the warp's lanes share one block, hence one env and one body count;
    // bodies in reverse order of application, any lane's
    const uint32_t any = __reduce_or_sync(kFull, touched);
    for (uint32_t rest = any; rest; rest &= ~(1u << (31 - __clz(rest)))) {
      const int b = 31 - __clz(rest);
      const bool hit = (touched >> b) & 1u;
      float gc[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      float gn[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (hit) {
        BodyPose cur, nxt;
        BodyShape sh;
        load_pose(pose, E.body_off + b, cur);
        load_pose(next_pose, E.body_off + b, nxt);
        load_shape(B.body_shape, E.body_off + b, sh);
        contact_backward(gx, vin[b], gv, cur, nxt, sh, E.dt, gc, gn, exact_capsule);
      }
      // the 14 pose-gradient values (7 at each end of the substep) summed
      // over the warp, then added by 14 lanes in one atomic instruction
      float vals[16];
#pragma unroll
      for (int c = 0; c < 7; ++c) {
        vals[c] = gc[c];
        vals[7 + c] = gn[c];
      }
      vals[14] = vals[15] = 0.f;
      const float total = warp_reduce_scatter16(vals, lane);
      const int vi = reduce_scatter16_index(lane);
      if ((lane & 1) == 0 && vi < 14) {
        const int c = vi < 7 ? vi : vi - 7;
        const int o = 8 * (E.body_off + b) + (c < 3 ? c : c + 1);
        atomicAdd((vi < 7 ? bgrad : next_bgrad) + o, total);
      }
    }
    if (in_list) {
      const f3 mom = mk3(g.x, g.y, g.z);
      igrad[ci] = active ? make_float4(gv.x * inv_m, gv.y * inv_m, gv.z * inv_m, -inv_m * inv_m * dot(mom, gv)) : z4;
      vgrad[ci] = z4;
      grid[ci] = z4;
      if (cell == 0) flags[blk] = 0u;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned ticket = atomicAdd(B.done_counter, 1u);
    if (ticket == gridDim.x - 1) {
      B.block_count[X] = 0;
      *B.done_counter = 0u;
      __threadfence();
    }
  }
}

// ============================================================ P2G adjoint
// integrator.cu:396-627 (p2g_grad) fused with :110-186 (compute_svd_grad) for
// particle p at x (stencil st inside the grid): the gradients of its state s
// (x: the part from the G2P adjoint, read from G, plus this part; v, F, C) from the
// adjoint grid of slot X (dL/d(mv, m), in in_grad) and the incoming F
// gradient of state s + 1.  With kTape the SVD and stress of F_tmp come from
// the tape the recomputed forward wrote (same values, without the SVD's
// registers and arithmetic).  v: the particle's velocity in state s.
//
// With kStash (the fused kernel), the results the stress adjoint does not
// touch -- the x and v gradients, the direct C gradient m Gs and v -- wait
// across it in `stash` (this lane's column of the warp's shared scatter rows,
// unused until the G2P adjoint: entry k at stash[32 k]) instead of in
// registers; o_gx, o_gv and v are then not written (read them back with
// unstash3 at 0, 3 and 15).
template <bool kTape, bool kStash = false>
__device__ __forceinline__ void p2g_grad_particle(const DexBatch &B, const DexEnv &E, int p, const Stencil &st,
                                                  const float *__restrict__ S, const float *__restrict__ Gnext,
                                                  const float *G, const float *__restrict__ tape, f3 &v, f3 &o_gx,
                                                  f3 &o_gv, m33 &o_gF, m33 &o_gC, float *stash = nullptr) {
  const int N = B.n_particles;
  v = ldf3(S, N, PV, p);
  const m33 C = ldm33(S, N, PC, p);
  const float m = __ldg(B.mass + p), vol = __ldg(B.vol + p);
  const float gss = -E.dt * E.inv_dx * vol * 4.f * E.inv_dx;
  // forward quantities: from the tape, the stress now and the SVD and return
  // mapping after the gather (fewer values live across its loop); without,
  // recomputed here
  m33 F, P;
  SVD3 sv;
  Plastic pl;
  float mu, lam, ys;
  auto forward_state = [&]() {
    F = ldm33(S, N, PF, p);
    mu = __ldg(B.mu_lam_yield + p);
    lam = __ldg(B.mu_lam_yield + N + p);
    ys = __ldg(B.mu_lam_yield + 2 * N + p);
    const m33 Et = deviation_tmp(F, C, E.dt);
    sv = kTape ? load_svd(tape, N, p) : svd3_from_deviation(Et);
    m33 Ft = Et;
    Ft.a[0][0] += 1.f; Ft.a[1][1] += 1.f; Ft.a[2][2] += 1.f;
    pl = constitutive(sv, Ft, mu, lam, ys);
  };
  if constexpr (kTape) {
    P = tape_m33(tape, N, 24, p);
  } else {
    forward_state();
    P = pl.P;
  }
  const m33 A = P * gss + C * m;

  float w1[3][3];
  make_dweights(st, E.inv_dx, w1);
  const NodeCells nc = node_cells(E, st.base);
  const float4 *__restrict__ ig = reinterpret_cast<const float4 *>(B.in_grad);
  // per node n with weight N_n, offset dpos_n and incoming dL/d(mv), dL/dm
  // (gov_n, gm_n):  dL/dstress = gss Gs, dL/dC = m Gs with Gs = sum N gov dpos^T;
  // dL/dv = m sum N gov; dL/dx = sum dN (m gm + m v.gov + gov.(A dpos)) - A^T sum N gov.
  // A dpos = a0 + i A0 dx + j A1 dx + k A2 dx.
  const f3 a0c = mcol(A, 0) * E.dx, a1c = mcol(A, 1) * E.dx, a2c = mcol(A, 2) * E.dx;
  const f3 a0 = -(a0c * st.fx[0] + a1c * st.fx[1] + a2c * st.fx[2]);
  const f3 u = v * m;
  // Gs = sum N gov ((i, j, k) - fx)^T dx = (sum N gov (i, j, k)^T - gw fx^T) dx.
  // With s_n = m gm + (u + A dpos).gov = m gm + (b + i A0 dx + j A1 dx + k A2 dx).gov,
  // dL/dx = (sum dNx s, sum dNy s, sum dNz s) - A^T gw.  Every sum over the
  // nodes is taken one axis at a time (z within a row, then y, then x), the
  // weight and its derivative factors applied per axis.
  const f3 b = u + a0;
  f3 gw, si, sj, sk;
  float gxx, gxy, gxz;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const f3 bi = step3(b, a0c, i);
    f3 q0, qj, qk;        // over the x-row i: sum w_y w_z gov, sum j w_y w_z gov, sum k w_y w_z gov
    float t00, t10, t01;  // sum w_y w_z s, sum w1_y w_z s, sum w_y w1_z s
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const f3 bij = step3(bi, a1c, j);
      const float4 h0 = __ldg(ig + nc.at(i, j, 0)), h1 = __ldg(ig + nc.at(i, j, 1)), h2 = __ldg(ig + nc.at(i, j, 2));
      const f3 g0 = xyz(h0), g1 = xyz(h1), g2 = xyz(h2);
      const float s0 = h0.w * m + dot(bij, g0);
      const float s1 = h1.w * m + dot(bij + a2c, g1);
      const float s2 = h2.w * m + dot(bij + a2c * 2.f, g2);
      const f3 t1 = g1 * st.w[2][1];
      const f3 p0 = g0 * st.w[2][0] + t1 + g2 * st.w[2][2];  // sum_k w_z gov
      const f3 p1 = t1 + g2 * (2.f * st.w[2][2]);           // sum_k k w_z gov
      const float S0 = s0 * st.w[2][0] + s1 * st.w[2][1] + s2 * st.w[2][2];
      const float S1 = s0 * w1[2][0] + s1 * w1[2][1] + s2 * w1[2][2];
      const float wy = st.w[1][j], dwy = w1[1][j];
      if (j == 0) {
        q0 = p0 * wy;
        qk = p1 * wy;
        t00 = S0 * wy;
        t10 = S0 * dwy;
        t01 = S1 * wy;
      } else {
        q0 += p0 * wy;
        qk += p1 * wy;
        qj = j == 1 ? p0 * wy : qj + p0 * (2.f * wy);
        t00 += S0 * wy;
        t10 += S0 * dwy;
        t01 += S1 * wy;
      }
    }
    const float wx = st.w[0][i], dwx = w1[0][i];
    if (i == 0) {
      gw = q0 * wx;
      sj = qj * wx;
      sk = qk * wx;
      gxx = t00 * dwx;
      gxy = t10 * wx;
      gxz = t01 * wx;
    } else {
      gw += q0 * wx;
      sj += qj * wx;
      sk += qk * wx;
      si = i == 1 ? q0 * wx : si + q0 * (2.f * wx);
      gxx += t00 * dwx;
      gxy += t10 * wx;
      gxz += t01 * wx;
    }
  }
  const f3 g_x = mk3(gxx, gxy, gxz) - mtv(A, gw);
  m33 Gs;
  {
    const f3 c0 = (si - gw * st.fx[0]) * E.dx, c1 = (sj - gw * st.fx[1]) * E.dx, c2 = (sk - gw * st.fx[2]) * E.dx;
    Gs.a[0][0] = c0.x; Gs.a[1][0] = c0.y; Gs.a[2][0] = c0.z;
    Gs.a[0][1] = c1.x; Gs.a[1][1] = c1.y; Gs.a[2][1] = c1.z;
    Gs.a[0][2] = c2.x; Gs.a[1][2] = c2.y; Gs.a[2][2] = c2.z;
  }
  const m33 g_stress = Gs * gss;
  m33 g_C = Gs * m;
  const f3 g_v = gw * m;
  if constexpr (kStash) {
    stash3(stash, 0, ldf3(G, N, PX, p) + g_x);
    stash3(stash, 3, g_v);
    stash33(stash, 6, g_C);
    stash3(stash, 15, v);
  }
  if constexpr (kTape) forward_state();

  // stress and projection -> F_tmp gradient (integrator.cu:541-625)
  const m33 Gt = kStash ? plastic_stress_backward_at(sv, pl, g_stress, [&]() { return ldm33_again(Gnext, N, PF, p); },
                                                    mu, lam, ys)
                        : plastic_stress_backward(sv, pl, g_stress, ldm33(Gnext, N, PF, p), mu, lam, ys);
  // F_tmp = (I + dt C) F
  if constexpr (kStash) {
    // F and C read again rather than held across the stress adjoint
    g_C = unstash33(stash, 6);
    F = ldm33_again(S, N, PF, p);
  }
  const m33 gC_total = g_C + mm(Gt, mT(F)) * E.dt;
  m33 IdtC = (kStash ? ldm33_again(S, N, PC, p) : C) * E.dt;
  IdtC.a[0][0] += 1.f; IdtC.a[1][1] += 1.f; IdtC.a[2][2] += 1.f;
  const m33 gF = mm(mT(IdtC), Gt);
  if constexpr (!kStash) {
    o_gx = ldf3(G, N, PX, p) + g_x;
    o_gv = g_v;
  }
  o_gF = gF;
  o_gC = gC_total;
}

// P2G adjoint of substep s: adds to the x gradient written by k_g2p_grad and
// writes the v, F, C gradients of state s (G); 128-thread CTAs, `split` per tile.
template <bool kTape>
__global__ void __launch_bounds__(128, DEX_P2G_GRAD_MINB) k_p2g_grad(DexBatch B, int X, const float *__restrict__ S,
                                                  const float *__restrict__ Gnext, float *__restrict__ G,
                                                  int split, const float *__restrict__ tape) {
  const int tile = blockIdx.x / split, part = blockIdx.x % split;
  const DexEnv E = B.envs[B.tiles[2 * tile]];
  const int first = B.tiles[2 * tile + 1];
  const int loc = first + part * blockDim.x + threadIdx.x;
  const int N = B.n_particles;
  if constexpr (kTape) {
    // the 48 planes read after the gather (F, material, SVD, incoming F and x
    // gradients) for this warp's particles, one plane per lane, into L2
    const int w0 = first + part * blockDim.x + (threadIdx.x & ~31);
    if (w0 < E.n) {
      const int p0 = E.p_off + w0, p1 = E.p_off + min(w0 + 31, E.n - 1);
      const int lane = threadIdx.x & 31;
#pragma unroll
      for (int q = lane; q < 48; q += 32) {
        const float *pl = q < 9    ? S + (size_t)(PF + q) * N
                          : q < 12 ? B.mu_lam_yield + (size_t)(q - 9) * N
                          : q < 36 ? tape + (size_t)(q - 12) * N
                          : q < 45 ? Gnext + (size_t)(PF + q - 36) * N
                                   : G + (size_t)(q - 45) * N;
        prefetch_plane(pl, p0, p1);
      }
    }
  }
  if (loc >= E.n) return;
  const int p = E.p_off + loc;
  const f3 x = ldf3(S, N, PX, p);
  Stencil st;
  make_stencil(x, E.inv_dx, st);
  if (!stencil_in_grid(E, st)) return;
  f3 v, gx, gv;
  m33 gF, gC;
  p2g_grad_particle<kTape>(B, E, p, st, S, Gnext, G, tape, v, gx, gv, gF, gC);
  stf3(G, N, PX, p, gx);
  stf3(G, N, PV, p, gv);
  stm33(G, N, PF, p, gF);
  stm33(G, N, PC, p, gC);
}

// P2G adjoint of substep s fused with the G2P adjoint of substep s - 1 for
// the same particle (the adjoint counterpart of k_g2p2g).  The gradients of
// state s stay in registers between the two: only its F gradient goes to G
// (read by the P2G adjoint of substep s - 1); the G2P adjoint of substep s - 1
// scatters into the adjoint grid and writes the x gradient of state s - 1 to
// Gprev.  S: state s, Sprev: state s - 1, Gnext: gradients of state s + 1 (F
// read), G: gradients of state s (x read: the part from the G2P adjoint of
// substep s; F written).  Gprev may be Gnext (different planes).
template <bool kTape>
__global__ void __launch_bounds__(128, DEX_P2G2G_GRAD_MINB) k_p2g2g_grad(DexBatch B, int X, int Xprev, const float *S,
                                                    const float *Sprev, const float *Gnext, float *G, float *Gprev,
                                                    int split, const float *__restrict__ tape) {
  const int tile = blockIdx.x / split, part = blockIdx.x % split;
  const DexEnv E = B.envs[B.tiles[2 * tile]];
  const int first = B.tiles[2 * tile + 1];
  const int loc = first + part * blockDim.x + threadIdx.x;
  const int N = B.n_particles;
  const int lane = threadIdx.x & 31;
  if constexpr (kTape) {
    // as in k_p2g_grad: the planes read after the gather, into L2
    const int w0 = first + part * blockDim.x + (threadIdx.x & ~31);
    if (w0 < E.n) {
      const int p0 = E.p_off + w0, p1 = E.p_off + min(w0 + 31, E.n - 1);
#pragma unroll
      for (int q = lane; q < 48; q += 32) {
        const float *pl = q < 9    ? S + (size_t)(PF + q) * N
                          : q < 12 ? B.mu_lam_yield + (size_t)(q - 9) * N
                          : q < 36 ? tape + (size_t)(q - 12) * N
                          : q < 45 ? Gnext + (size_t)(PF + q - 36) * N
                                   : G + (size_t)(q - 45) * N;
        prefetch_plane(pl, p0, p1);
      }
    }
  }
  const bool in = loc < E.n;
  const int p = E.p_off + (in ? loc : 0);
  const f3 x = ldf3(S, N, PX, p);
  // the G2P adjoint's position, loaded ahead and parked in shared memory
  // with the P2G adjoint's results (this lane's column of the warp's scatter
  // rows, entries 0-17 by p2g_grad_particle, 18-20 here)
  float *stash = warp_red_buffer() + lane;
  stash3(stash, 18, ldf3(Sprev, N, PX, p));
  Stencil st;
  make_stencil(x, E.inv_dx, st);
  const bool ok = in && stencil_in_grid(E, st);  // out-of-grid particles were reported by the G2P adjoint
  if (!ok) st.base[0] = st.base[1] = st.base[2] = 0;
  f3 v, gx, gv;
  m33 gF, gC;
  p2g_grad_particle<kTape, true>(B, E, p, st, S, Gnext, G, tape, v, gx, gv, gF, gC, stash);
  gx = unstash3(stash, 0);
  gv = unstash3(stash, 3);
  v = unstash3(stash, 15);
  const f3 xprev = unstash3(stash, 18);
  __syncwarp();  // every lane has its values back before the scatter rows are written
  if (ok) {
    stm33(G, N, PF, p, gF);
  } else {
    gx = gv = mk3(0.f, 0.f, 0.f);
    gC = mzero();
  }
  g2p_grad_lane(B, E, Xprev, p, in, xprev, v, gx, gv, gC, Gprev, lane);
}

// Zero the grid cells and flags of the listed blocks of slots [first, last)
// and, by the last CTA to finish (ticket on done_counter), their list counts:
// a kept slot whose adjoint will not run is made clean for reuse.
__global__ void __launch_bounds__(256) k_clear_slots(DexBatch B, int first, int last) {
  const int sub = threadIdx.x >> 6, cell = threadIdx.x & 63;
  const int per_cta = blockDim.x >> 6;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int X = first; X < last; ++X) {
    const int cnt = *reinterpret_cast<volatile int *>(B.block_count + X);
    float4 *grid = reinterpret_cast<float4 *>(slot_grid(B, X));
    const int32_t *list = slot_list(B, X);
    uint32_t *flags = slot_flags(B, X);
    for (int item = blockIdx.x * per_cta + sub; item < cnt; item += gridDim.x * per_cta) {
      const int blk = list[item];
      grid[(blk << 6) + cell] = z4;
      if (cell == 0) flags[blk] = 0u;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned ticket = atomicAdd(B.done_counter, 1u);
    if (ticket == gridDim.x - 1) {
      for (int X = first; X < last; ++X) B.block_count[X] = 0;
      *B.done_counter = 0u;
      __threadfence();
    }
  }
}

__global__ void k_reset_counts(DexBatch B) {
  for (int k = threadIdx.x; k < B.n_slots; k += blockDim.x) B.block_count[k] = 0;
  if (threadIdx.x == 0) {
    *B.done_counter = 0u;
    *B.error = 0;
  }
}

int check_launch() { return cudaGetLastError() == cudaSuccess ? DEXMPM_OK : DEXMPM_ERR_LAUNCH; }

// The kernels read and write the grid slots, their velocities and adjoints,
// the body shapes and the poses as float4: those must start on 16-byte
// boundaries (an offset pointer would fault the kernel, so it is refused).
bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

bool valid(const DexBatch *b) {
  return b && b->envs && b->tiles && b->block_env && b->block_xyz && b->mass && b->vol && b->mu_lam_yield && b->grid &&
         b->vout &&
         b->block_flag && b->block_list && b->block_count && b->done_counter && b->error && b->n_tiles >= 0 &&
         b->n_blocks > 0 && b->n_slots > 0 && (b->tile_size == 64 || b->tile_size == 128 || b->tile_size == 256) &&
         b->grid_ctas > 0 && aligned16(b->grid) && aligned16(b->vout) && aligned16(b->body_shape);
}
bool slot_ok(const DexBatch *b, int k) { return k >= 0 && k < b->n_slots; }

// CTAs of a 256-thread grid kernel resident on the whole device at once
// (occupancy x SM count, cached per device): the persistent grid kernels
// launch at most that many, so that they run in one wave.
enum { kGridOp = 0, kGridOpGrad = 1, kClearSlots = 2, kGridKernels = 3 };
int resident_ctas(const void *kernel, int id) {
  static std::atomic<int> cache[64][kGridKernels];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  int c = cache[dev][id].load(std::memory_order_relaxed);
  if (c == 0) {
    int per_sm = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    c = per_sm * sms;
    cache[dev][id].store(c, std::memory_order_relaxed);
  }
  return c;
}
int grid_ctas(const DexBatch *b, const void *kernel, int id) {
  const int r = resident_ctas(kernel, id);
  return b->grid_ctas < r ? b->grid_ctas : r;
}

// Dynamic shared memory of the scatter kernels for CTAs of `threads`.
size_t scatter_smem(int threads) { return (size_t)(threads / 32) * kScatterSmemPerWarp; }

// Opt the scatter kernels in to the dynamic shared memory of 256-thread CTAs
// (above the 48 KB default), once per device.
int scatter_attr_ready() {
  static std::atomic<int> ready[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DEXMPM_ERR_LAUNCH;
  if (ready[dev].load(std::memory_order_acquire)) return DEXMPM_OK;
  const int bytes = (int)scatter_smem(256);
  if (cudaFuncSetAttribute(k_p2g, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess ||
      cudaFuncSetAttribute(k_g2p2g, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess ||
      cudaFuncSetAttribute(k_g2p_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
    return DEXMPM_ERR_LAUNCH;
  ready[dev].store(1, std::memory_order_release);
  return DEXMPM_OK;
}
bool grad_ok(const DexBatch *b) {
  return valid(b) && b->vout_grad && b->in_grad && aligned16(b->vout_grad) && aligned16(b->in_grad);
}

// Kernel launch on the caller's stream; returns the launch status.
template <typename... P, typename... A>
int launch(void (*kernel)(P...), int grid, int block, size_t smem, dexmpm_stream_t stream, A... args) {
  kernel<<<grid, block, smem, (cudaStream_t)stream>>>(args...);
  return check_launch();
}

}  // namespace

extern "C" {

const char *dexmpm_version(void) { return "dexmpm 0.2 sm_103a"; }

int dexmpm_reset(const DexBatch *b, dexmpm_stream_t stream) {
  if (!valid(b)) return DEXMPM_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t cells = (size_t)b->n_blocks * 64 * sizeof(float4);
  if (cudaMemsetAsync(b->grid, 0, cells * b->n_slots, s) != cudaSuccess) return DEXMPM_ERR_LAUNCH;
  if (cudaMemsetAsync(b->vout, 0, cells * b->n_slots, s) != cudaSuccess) return DEXMPM_ERR_LAUNCH;
  if (b->vout_grad && cudaMemsetAsync(b->vout_grad, 0, cells, s) != cudaSuccess) return DEXMPM_ERR_LAUNCH;
  if (b->in_grad && cudaMemsetAsync(b->in_grad, 0, cells, s) != cudaSuccess) return DEXMPM_ERR_LAUNCH;
  if (cudaMemsetAsync(b->block_flag, 0, (size_t)b->n_blocks * b->n_slots * sizeof(uint32_t), s) != cudaSuccess)
    return DEXMPM_ERR_LAUNCH;
  k_reset_counts<<<1, 256, 0, s>>>(*b);
  if (int rc = check_launch()) return rc;
  return scatter_attr_ready();
}

int dexmpm_p2g(const DexBatch *b, int slot, const float *S, float *Snext, float *tape, dexmpm_stream_t stream) {
  if (!valid(b) || !S || !slot_ok(b, slot)) return DEXMPM_ERR_ARG;
  if (b->n_tiles == 0) return DEXMPM_OK;
  if (int rc = scatter_attr_ready()) return rc;
  return launch(k_p2g, b->n_tiles, b->tile_size, scatter_smem(b->tile_size), stream, *b, slot, S, Snext, tape);
}

int dexmpm_grid_op(const DexBatch *b, int slot, int clear_slot, const float *pose, const float *next_pose,
                   dexmpm_stream_t stream) {
  if (!valid(b) || !slot_ok(b, slot) || (clear_slot >= 0 && (!slot_ok(b, clear_slot) || clear_slot == slot)))
    return DEXMPM_ERR_ARG;
  if (b->n_bodies > 0 && (!pose || !next_pose || !b->body_shape || !aligned16(pose) || !aligned16(next_pose)))
    return DEXMPM_ERR_ARG;
  return launch(k_grid_op, grid_ctas(b, (const void *)k_grid_op, kGridOp), 256, 0, stream, *b, slot,
                clear_slot < 0 ? -1 : clear_slot, pose, next_pose);
}

int dexmpm_g2p(const DexBatch *b, int slot, const float *S, float *Snext, dexmpm_stream_t stream) {
  if (!valid(b) || !S || !Snext || !slot_ok(b, slot)) return DEXMPM_ERR_ARG;
  if (b->n_tiles == 0) return DEXMPM_OK;
  return launch(k_g2p, b->n_tiles, b->tile_size, 0, stream, *b, slot, S, Snext);
}

int dexmpm_g2p2g(const DexBatch *b, int slot_g, int slot_s, const float *S, float *Snext, float *S2, float *tape,
                 dexmpm_stream_t stream) {
  if (!valid(b) || !S || !Snext || !S2 || Snext == S || Snext == S2 || !slot_ok(b, slot_g) || !slot_ok(b, slot_s) ||
      slot_g == slot_s)
    return DEXMPM_ERR_ARG;
  if (b->n_tiles == 0) return DEXMPM_OK;
  if (int rc = scatter_attr_ready()) return rc;
  return launch(k_g2p2g, b->n_tiles, b->tile_size, scatter_smem(b->tile_size), stream, *b, slot_g, slot_s, S, Snext,
                S2, tape);
}

int dexmpm_substep(const DexBatch *b, int slot, int clear_slot, const float *S, float *Snext, const float *pose,
                   const float *next_pose, float *tape, dexmpm_stream_t stream) {
  int rc = dexmpm_p2g(b, slot, S, Snext, tape, stream);
  if (rc) return rc;
  rc = dexmpm_grid_op(b, slot, clear_slot, pose, next_pose, stream);
  if (rc) return rc;
  return dexmpm_g2p(b, slot, S, Snext, stream);
}

int dexmpm_g2p_grad(const DexBatch *b, int slot, const float *S, const float *Snext, const float *Gnext, float *G,
                    dexmpm_stream_t stream) {
  if (!grad_ok(b) || !S || !Snext || !Gnext || !G || !slot_ok(b, slot)) return DEXMPM_ERR_ARG;
  if (b->n_tiles == 0) return DEXMPM_OK;
  if (int rc = scatter_attr_ready()) return rc;
  return launch(k_g2p_grad, b->n_tiles, b->tile_size, scatter_smem(b->tile_size), stream, *b, slot, S, Snext, Gnext,
                G);
}

int dexmpm_grid_op_grad(const DexBatch *b, int slot, const float *pose, const float *next_pose, float *bgrad,
                        float *next_bgrad, dexmpm_stream_t stream) {
  if (!grad_ok(b) || !slot_ok(b, slot)) return DEXMPM_ERR_ARG;
  if (b->n_bodies > 0 && (!pose || !next_pose || !bgrad || !next_bgrad || !b->body_shape || !aligned16(pose) ||
                          !aligned16(next_pose)))
    return DEXMPM_ERR_ARG;
  return launch(k_grid_op_grad, grid_ctas(b, (const void *)k_grid_op_grad, kGridOpGrad), 256, 0, stream, *b, slot,
                pose, next_pose, bgrad, next_bgrad);
}

int dexmpm_p2g_grad(const DexBatch *b, int slot, const float *S, const float *Gnext, float *G, const float *tape,
                    dexmpm_stream_t stream) {
  if (!grad_ok(b) || !S || !Gnext || !G || !slot_ok(b, slot)) return DEXMPM_ERR_ARG;
  if (b->n_tiles == 0) return DEXMPM_OK;
  // the adjoint is register-heavy: 128-thread CTAs, tile_size/128 of them per tile
  const int cta = b->tile_size < 128 ? b->tile_size : 128;
  const int split = b->tile_size / cta;
  if (tape) return launch(k_p2g_grad<true>, b->n_tiles * split, cta, 0, stream, *b, slot, S, Gnext, G, split, tape);
  return launch(k_p2g_grad<false>, b->n_tiles * split, cta, 0, stream, *b, slot, S, Gnext, G, split,
                (const float *)nullptr);
}

int dexmpm_p2g_g2p_grad(const DexBatch *b, int slot, int prev_slot, const float *S, const float *Sprev,
                        const float *Gnext, float *G, float *Gprev, const float *tape, dexmpm_stream_t stream) {
  if (!grad_ok(b) || !S || !Sprev || !Gnext || !G || !Gprev || G == Gnext || G == Gprev || !slot_ok(b, slot) ||
      !slot_ok(b, prev_slot) || slot == prev_slot)
    return DEXMPM_ERR_ARG;
  if (b->n_tiles == 0) return DEXMPM_OK;
  const int cta = b->tile_size < 128 ? b->tile_size : 128;
  const int split = b->tile_size / cta;
  if (tape)
    return launch(k_p2g2g_grad<true>, b->n_tiles * split, cta, scatter_smem(cta), stream, *b, slot, prev_slot, S,
                  Sprev, Gnext, G, Gprev, split, tape);
  return launch(k_p2g2g_grad<false>, b->n_tiles * split, cta, scatter_smem(cta), stream, *b, slot, prev_slot, S, Sprev,
                Gnext, G, Gprev, split, (const float *)nullptr);
}

int dexmpm_substep_grad(const DexBatch *b, int slot, const float *S, const float *Snext, const float *Gnext,
                        float *G, const float *pose, const float *next_pose, float *bgrad, float *next_bgrad,
                        const float *tape, dexmpm_stream_t stream) {
  int rc = dexmpm_g2p_grad(b, slot, S, Snext, Gnext, G, stream);
  if (rc) return rc;
  rc = dexmpm_grid_op_grad(b, slot, pose, next_pose, bgrad, next_bgrad, stream);
  if (rc) return rc;
  return dexmpm_p2g_grad(b, slot, S, Gnext, G, tape, stream);
}

int dexmpm_clear_slots(const DexBatch *b, int first, int last, dexmpm_stream_t stream) {
  if (!valid(b) || first < 0 || last > b->n_slots || first > last) return DEXMPM_ERR_ARG;
  if (first == last) return DEXMPM_OK;
  return launch(k_clear_slots, grid_ctas(b, (const void *)k_clear_slots, kClearSlots), 256, 0, stream, *b, first,
                last);
}

int dexmpm_get_error(const DexBatch *b, int32_t *out, dexmpm_stream_t stream) {
  if (!b || !b->error || !out) return DEXMPM_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(out, b->error, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return DEXMPM_ERR_LAUNCH;
  if (cudaStreamSynchronize(s) != cudaSuccess) return DEXMPM_ERR_LAUNCH;
  if (cudaMemsetAsync(b->error, 0, sizeof(int32_t), s) != cudaSuccess) return DEXMPM_ERR_LAUNCH;
  return DEXMPM_OK;
}

}  // extern "C"
