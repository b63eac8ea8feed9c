// noalloc.cu -- one forward substep of one environment without any device
// allocation by this library or by the caller.
//
// Some callers cannot call cudaMalloc.  A host application may own nearly all
// device memory through its own pool allocator and forbid allocations from
// plugins (runtimes that reserve most of the GPU up front do this), and a
// real-time control loop may not be allowed to block on, or fail in, an
// allocation in the middle of an episode.  Such callers pass only their
// inputs and outputs; the grids, active-block lists and counters the substep
// needs live in one file-scope device array of fixed size, below.
//
// Limits of that array: grids up to 262,144 cells (64^3, the reference's
// default domain) and up to 1,048,576 particles, 32 bodies.  It takes 8.5 MB
// on every GPU that loads this part of the library, held until the process
// exits (with CUDA's default lazy module loading that happens on the first
// call on a device).
//
// Every call shares the array and leaves its contents behind; each call
// clears what must start at zero before it runs.  Calls whose work overlaps on
// the GPU (different streams or threads, no ordering between them) race on the
// array and give wrong results: order them on one stream.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/dexmpm.h"

namespace {

constexpr int kMaxCells = 64 * 64 * 64;
constexpr int kMaxBlocks = kMaxCells / 64;
constexpr int kMaxParticles = 1 << 20;
constexpr int kTile = 128;
constexpr int kMaxTiles = kMaxParticles / kTile;

// byte offsets inside the array (each region 256-byte aligned)
constexpr size_t kGrid0 = 0;
constexpr size_t kVout = kGrid0 + (size_t)kMaxCells * 16;
constexpr size_t kFlag0 = kVout + (size_t)kMaxCells * 16;
constexpr size_t kList0 = kFlag0 + (size_t)kMaxBlocks * 4;
constexpr size_t kBlockEnv = kList0 + (size_t)kMaxBlocks * 4;
constexpr size_t kBlockXyz = kBlockEnv + (size_t)kMaxBlocks * 4;
constexpr size_t kTiles = kBlockXyz + (size_t)kMaxBlocks * 4;
constexpr size_t kEnv = kTiles + (size_t)kMaxTiles * 8;
constexpr size_t kCounts = kEnv + 256;  // block_count, done_counter, error
constexpr size_t kBytes = kCounts + 256;

__device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

// Device address of the array for the current device (host code only has a
// stand-in symbol; the address must come from the runtime).  Looked up on
// every call, so that it stays valid across a cudaDeviceReset, which unloads
// and reloads the module.
int scratch_address(void **out) {
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return DEXMPM_ERR_LAUNCH;
  *out = p;
  return DEXMPM_OK;
}

// Streaming multiprocessors of the current device (persistent grid kernels
// launch up to four CTAs per SM).
int device_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                 cudaSuccess || sms < 1)
    return 1;
  return sms;
}

bool positive_finite(float v) { return v > 0.f && v <= 3.0e38f; }

// Writes the env descriptor, the tiles and the block tables (owner,
// coordinates), and zeroes the flags, list counts and ticket used by this
// call.
__global__ void k_noalloc_setup(DexEnv env, int n_tiles, int n_blocks) {
  unsigned char *base = g_noalloc_scratch;
  int32_t *tiles = reinterpret_cast<int32_t *>(base + kTiles);
  int32_t *block_env = reinterpret_cast<int32_t *>(base + kBlockEnv);
  int32_t *block_xyz = reinterpret_cast<int32_t *>(base + kBlockXyz);
  const int nby = env.gy >> 2, nbz = env.gz >> 2;
  uint32_t *flag0 = reinterpret_cast<uint32_t *>(base + kFlag0);
  int stride = gridDim.x * blockDim.x;
  int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  for (int t = t0; t < n_tiles; t += stride) {
    tiles[2 * t] = 0;
    tiles[2 * t + 1] = t * kTile;
  }
  for (int b = t0; b < n_blocks; b += stride) {
    block_env[b] = 0;
    block_xyz[b] = ((b / (nby * nbz)) << 20) | (((b / nbz) % nby) << 10) | (b % nbz);
    flag0[b] = 0u;
  }
  if (t0 == 0) {
    *reinterpret_cast<DexEnv *>(base + kEnv) = env;
    int32_t *counts = reinterpret_cast<int32_t *>(base + kCounts);
    counts[0] = 0;  // block count of the single slot
    counts[2] = 0;  // done_counter
  }
}

}  // namespace

extern "C" int dexmpm_substep_noalloc(const DexEnv *env, const float *s, float *next_s, const float *mass,
                                      const float *vol, const float *mu_lam_yield, const float *body_shape,
                                      const float *pose, const float *next_pose, int32_t *error,
                                      dexmpm_stream_t stream) {
  // the error word is required: without it an out-of-grid particle would be
  // skipped with no sign to the caller
  if (!env || !s || !next_s || !mass || !vol || !mu_lam_yield || !error) return DEXMPM_ERR_ARG;
  const DexEnv e = *env;
  if (!positive_finite(e.dx) || !positive_finite(e.inv_dx) || !positive_finite(e.dt)) return DEXMPM_ERR_ARG;
  if (fabsf(e.dx * e.inv_dx - 1.f) > 1e-4f) return DEXMPM_ERR_ARG;
  if (e.p_off != 0 || e.blk_off != 0 || e.body_off != 0 || e.n < 0 || e.n > kMaxParticles) return DEXMPM_ERR_ARG;
  if (e.gx < 8 || e.gy < 8 || e.gz < 8 || (e.gx & 3) || (e.gy & 3) || (e.gz & 3)) return DEXMPM_ERR_ARG;
  if ((long long)e.gx * e.gy * e.gz > kMaxCells) return DEXMPM_ERR_ARG;
  if (e.n_bodies < 0 || e.n_bodies > DEXMPM_MAX_BODIES) return DEXMPM_ERR_ARG;
  // body shapes and poses are read as float4: 16-byte boundaries
  auto a16 = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
  if (e.n_bodies > 0 && (!body_shape || !pose || !next_pose || !a16(body_shape) || !a16(pose) || !a16(next_pose)))
    return DEXMPM_ERR_ARG;
  void *addr = nullptr;
  int rc = scratch_address(&addr);
  if (rc) return rc;
  unsigned char *base = static_cast<unsigned char *>(addr);
  cudaStream_t st = (cudaStream_t)stream;
  const int n_blocks = (e.gx / 4) * (e.gy / 4) * (e.gz / 4);
  const int n_tiles = (e.n + kTile - 1) / kTile;
  // the P2G target grid of this call must start at zero
  if (cudaMemsetAsync(base + kGrid0, 0, (size_t)n_blocks * 64 * 16, st) != cudaSuccess) return DEXMPM_ERR_LAUNCH;
  const int threads = 256, work = n_blocks > n_tiles ? n_blocks : n_tiles;
  const int blocks = (work + threads - 1) / threads > 0 ? (work + threads - 1) / threads : 1;
  k_noalloc_setup<<<blocks, threads, 0, st>>>(e, n_tiles, n_blocks);
  if (cudaGetLastError() != cudaSuccess) return DEXMPM_ERR_LAUNCH;

  DexBatch b;
  b.n_envs = 1;
  b.n_particles = e.n > 0 ? e.n : 1;
  b.n_tiles = n_tiles;
  b.n_blocks = n_blocks;
  b.n_bodies = e.n_bodies;
  b.tile_size = kTile;
  b.grid_ctas = 4 * device_sms();
  b.flags = 0;
  b.n_slots = 1;
  b.pad0 = b.pad1 = b.pad2 = 0;
  b.envs = reinterpret_cast<const DexEnv *>(base + kEnv);
  b.tiles = reinterpret_cast<const int32_t *>(base + kTiles);
  b.block_env = reinterpret_cast<const int32_t *>(base + kBlockEnv);
  b.block_xyz = reinterpret_cast<const int32_t *>(base + kBlockXyz);
  b.mass = mass;
  b.vol = vol;
  b.mu_lam_yield = mu_lam_yield;
  b.grid = reinterpret_cast<float *>(base + kGrid0);
  b.vout = reinterpret_cast<float *>(base + kVout);
  b.vout_grad = nullptr;
  b.in_grad = nullptr;
  b.block_flag = reinterpret_cast<uint32_t *>(base + kFlag0);
  b.block_list = reinterpret_cast<int32_t *>(base + kList0);
  b.block_count = reinterpret_cast<int32_t *>(base + kCounts);
  b.done_counter = reinterpret_cast<uint32_t *>(base + kCounts + 8);
  b.body_shape = body_shape;
  b.error = error;
  // one grid slot, nothing to clear afterwards (the next call re-zeroes it)
  return dexmpm_substep(&b, 0, -1, s, next_s, pose, next_pose, nullptr, stream);
}
