// ref_host.cpp -- TEST INFRASTRUCTURE ONLY (the parity checker, never the product).
//
// Compiles DexDeform's own mpm/csrc/integrator.cu, unmodified and read from where
// it lies in the reference tree, as plain host C++ with g++, so that the
// reference's kernel bodies run serially on the CPU.  The reference's extern "C"
// launchers (compute_svd, p2g, grid_op_v2, g2p and the *_grad twins,
// integrator.cu:1616-1985) are exported unchanged and take HOST pointers:
//   * __global__/__device__/__host__ expand to nothing,
//   * threadIdx/blockIdx/blockDim are ordinary globals set by a serial loop,
//   * launch_kernel (common.h:20-25) is redefined as that loop,
//   * atomicAdd/atomicMin become plain read-modify-writes (one thread at a time),
//   * curand is served by the renderer's counter-based generator
//     (shim/curand_kernel.h), and the render launcher's cudaMalloc/cudaFree of
//     its generator states by malloc/free.
// The include path of integrator.cu is passed in by the build recipe
// (oracle/build_ref_host.sh) through REF_CSRC.
#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __STORAGE__ extern
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <algorithm>
extern "C" {
uint3 threadIdx;
uint3 blockIdx;
dim3 blockDim;
dim3 gridDim;
int warpSize = 32;
}
static inline float atomicAdd(float *a, float b) { float o = *a; *a += b; return o; }
static inline int atomicMin(int *a, int b) { int o = *a; if (b < o) *a = b; return o; }
static inline int atomicMax(int *a, int b) { int o = *a; if (b > o) *a = b; return o; }
static inline long long atomicMin(long long *a, long long b) { long long o = *a; if (b < o) *a = b; return o; }
using std::max;
using std::min;
// CUDA's headers put float overloads of abs/log/exp in the global namespace
// (vec3.h:111-119 calls ::abs, ::log, ::exp on floats); the host C library
// only has int abs(int) and double log/exp there, and ::abs(float) would
// truncate to an integer.  Give them the meaning they have under nvcc.
static inline float abs(float a) { return fabsf(a); }
static inline float log(float a) { return logf(a); }
static inline float exp(float a) { return expf(a); }
// CUDA's device headers overload min/max on mixed float/double arguments; the
// host library does not, so give the mixed forms the device meaning.
static inline double min(float a, double b) { return a < b ? (double)a : b; }
static inline double max(float a, double b) { return a > b ? (double)a : b; }
static inline double max(double a, float b) { return a > b ? a : (double)b; }

#define STR2(x) #x
#define STR(x) STR2(x)
#include STR(REF_CSRC/common.h)
#undef launch_kernel
#define launch_kernel(kernel, dim, stream, args)                                  \
  {                                                                               \
    (void)(stream);                                                               \
    blockDim.x = 256; blockDim.y = blockDim.z = 1;                                \
    gridDim.x = ((dim) + 255) / 256; gridDim.y = gridDim.z = 1;                   \
    for (unsigned b_ = 0; b_ < gridDim.x; ++b_)                                   \
      for (unsigned t_ = 0; t_ < 256; ++t_) {                                     \
        blockIdx.x = b_; threadIdx.x = t_;                                        \
        kernel args;                                                              \
      }                                                                           \
  }
#include <cstdlib>
#include <type_traits>
#define cudaMalloc(ptr, size) \
  (*(ptr) = (std::remove_reference<decltype(*(ptr))>::type)std::malloc(size), cudaSuccess)
#define cudaFree(ptr) (std::free(ptr), cudaSuccess)
#include STR(REF_CSRC/integrator.cu)
