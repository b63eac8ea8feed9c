// render.cu -- particle volume bake and SDF path tracer for sm_103a, behind
// the reference's launchers particle_sdf and render (mpm/csrc/integrator.cu:
// 1862-1933; Python side mpm/renderer.py:88-169).
//
// Volume bake (particle_sdf):
//   * splat: every particle writes, into the (2 bake)^3 voxels around its
//     voxel, the packed value (quantised distance << 24) | rgb with a 64-bit
//     atomicMin, so each voxel keeps its nearest particle (ties: smaller
//     color) whatever the order of the atomics;
//   * unpack: distance / 255 and rgb / 255;
//   * two 3^3 box filters of the distance (border voxels 1).
//   The file is compiled without multiply-add contraction, and the few double
//   operations of the reference are kept, so the volume is bit-identical to
//   the reference's and the image matches its code run on the host up to the
//   rounding of cos and sin.
// Path tracer (render): one thread per pixel, 16 x 16 pixel tiles per CTA,
// the scene's bodies staged in shared memory.  Each sample jitters the pixel,
// then up to max_ray_depth bounces: the nearest of the ground plane, the
// bodies (sphere tracing) and the baked volume (ray marching with bisection),
// a cosine-weighted diffuse bounce and a shadow ray towards a jittered
// directional light.  Random numbers come from a counter-based generator
// (SplitMix64 of (seed, pixel, draw index); Steele, Lea & Flood, "Fast
// splittable pseudorandom number generators", OOPSLA 2014) drawn in the
// order the reference's code consumes them, instead of per-pixel curand
// states allocated on every call.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_math.cuh"
#include "../../include/dexmpm.h"

using namespace dexmpm;

namespace {

constexpr int kMaxRenderBodies = 64;
constexpr float kDistLimit = 100.f;

// ------------------------------------------------------------------ RNG
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
struct Rng {
  uint64_t key, ctr;
  __device__ Rng(int seed, int pixel)
      : key(splitmix64(((uint64_t)(uint32_t)seed << 32) ^ (uint64_t)(uint32_t)pixel)), ctr(0) {}
  // uniform in (0, 1], 24 bits
  __device__ __forceinline__ float uniform() {
    ++ctr;
    const uint64_t h = splitmix64(key + ctr * 0x9E3779B97F4A7C15ull);
    return (float)((h >> 40) + 1ull) * (1.f / 16777216.f);
  }
};

// shape.h:7-15 normalisation by division (the renderer's images are compared
// with the reference's code pixel by pixel; the simulation kernels use a
// reciprocal multiply)
__device__ __forceinline__ f3 normalized(f3 a) {
  const float l = sqrtf(dot(a, a) + kLenEps);
  return mk3(a.x / l, a.y / l, a.z / l);
}
// shape.h:63-102 with that normalisation
__device__ f3 body_normal_local(qf tfsr, qf args, f3 g) {
  const int type = shape_type(tfsr);
  f3 grad = mk3(0.f, 0.f, 0.f);
  if (type == 0) {
    const f3 q = fabs3(g) - mk3(args.w, args.x, args.y);
    const float inside = fmaxf(fmaxf(q.x, q.y), q.z);
    if (inside <= 0.f) {
      if (q.x == inside) grad.x += 1.f;
      if (q.y == inside) grad.y += 1.f;
      if (q.z == inside) grad.z += 1.f;
    } else {
      grad = normalized(fmax3(q, 0.f));
    }
    if (g.x < 0.f) grad.x = -grad.x;
    if (g.y < 0.f) grad.y = -grad.y;
    if (g.z < 0.f) grad.z = -grad.z;
  } else if (type == 1) {
    const float h = args.x;
    f3 p2 = g;
    p2.y += h / 2;
    p2.y -= fminf(fmaxf(p2.y, 0.f), h);
    return normalized(p2);
  }
  return grad;
}

// --------------------------------------------------------------- volume
struct Volume {
  const float *sdf;
  const float *color;  // [n][3]
  f3 lower, upper;
  int dx, dy, dz;
  float thr;
};

// Trilinear interpolation of a voxel array (mpm/csrc/array.h:7-50): false
// outside [lower, upper).  C = 1 (distance) or 3 (color) floats per voxel.
template <int C>
__device__ bool volume_query(const Volume &V, const float *values, f3 point, float out[C]) {
  const f3 ratio = mk3((point.x - V.lower.x) / (V.upper.x - V.lower.x), (point.y - V.lower.y) / (V.upper.y - V.lower.y),
                       (point.z - V.lower.z) / (V.upper.z - V.lower.z));
  if (!(ratio.x >= 0.f && ratio.y >= 0.f && ratio.z >= 0.f && ratio.x < 1.f && ratio.y < 1.f && ratio.z < 1.f))
    return false;
  const f3 g = mk3(ratio.x * (float)V.dx, ratio.y * (float)V.dy, ratio.z * (float)V.dz);
  const int x0 = min(max((int)floorf(g.x), 0), V.dx - 1);
  const int y0 = min(max((int)floorf(g.y), 0), V.dy - 1);
  const int z0 = min(max((int)floorf(g.z), 0), V.dz - 1);
  const float fx = g.x - (float)x0, fy = g.y - (float)y0, fz = g.z - (float)z0;
  const int i000 = (x0 * V.dy + y0) * V.dz + z0;
  const int sz = z0 + 1 < V.dz, sy = (y0 + 1 < V.dy) * V.dz, sx = (x0 + 1 < V.dx) * V.dy * V.dz;
  const int idx[8] = {i000, i000 + sz, i000 + sy, i000 + sy + sz, i000 + sx, i000 + sx + sz, i000 + sx + sy,
                      i000 + sx + sy + sz};
  const float wx[8] = {1 - fx, 1 - fx, 1 - fx, 1 - fx, fx, fx, fx, fx};
  const float wy[8] = {1 - fy, 1 - fy, fy, fy, 1 - fy, 1 - fy, fy, fy};
  const float wz[8] = {1 - fz, fz, 1 - fz, fz, 1 - fz, fz, 1 - fz, fz};
  // value * wx * wy * wz, summed corner by corner (the reference's order)
#pragma unroll
  for (int c = 0; c < C; ++c) {
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q)
      acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(__fmul_rn(__ldg(values + (size_t)C * idx[q] + c), wx[q]), wy[q]),
                                     wz[q]));
    out[c] = acc;
  }
  return true;
}

// array.h:52-60: distance minus threshold inside the box, 0 outside
__device__ float sample_sdf(const Volume &V, f3 p, float thr) {
  float v[1] = {0.f};
  if (volume_query<1>(V, V.sdf, p, v)) v[0] -= thr;
  return v[0];
}

// array.h:63-72: central differences, eps 1e-3
__device__ f3 sample_normal(const Volume &V, f3 p) {
  const float e = 1e-3f;
  const float x0 = sample_sdf(V, p + mk3(-e, 0.f, 0.f), 0.f), x1 = sample_sdf(V, p + mk3(e, 0.f, 0.f), 0.f);
  const float y0 = sample_sdf(V, p + mk3(0.f, -e, 0.f), 0.f), y1 = sample_sdf(V, p + mk3(0.f, e, 0.f), 0.f);
  const float z0 = sample_sdf(V, p + mk3(0.f, 0.f, -e), 0.f), z1 = sample_sdf(V, p + mk3(0.f, 0.f, e), 0.f);
  return mk3(x1 - x0, y1 - y0, z1 - z0) * (float)(0.5 / (double)e);
}

// integrator.cu:1111-1140
__device__ bool ray_box(f3 lo, f3 hi, f3 o, f3 d, float &tn, float &tf) {
  const float dd[3] = {d.x, d.y, d.z}, oo[3] = {o.x, o.y, o.z}, l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
  tn = -1e9f;
  tf = 1e9f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (dd[i] == 0.f) {
      if (oo[i] < l[i] || oo[i] > h[i]) return false;
    } else {
      const float a = (l[i] - oo[i]) / dd[i], b = (h[i] - oo[i]) / dd[i];
      tf = fminf(fmaxf(a, b), tf);
      tn = fmaxf(fminf(a, b), tn);
    }
  }
  return !(tn > tf);
}

struct Scene {
  Volume V;
  const BodyPose *pose;    // shared memory
  const BodyShape *shape;  // shared memory
  int nb;
  bool volume_on;
  float ground;
};

struct Hit {
  f3 normal, color;
};

// Nearest hit along o + t d (integrator.cu:1142-1285): ground plane (checker
// inside the unit square), bodies by sphere tracing, the volume by marching
// with bisection refinement.  Returns the distance (1e9 when nothing is hit);
// on a hit sets the normal and color.
__device__ float next_hit(const Scene &S, f3 o, f3 d, Hit &h) {
  float closest = 1e9f;
  if (d.y < 0.f) {
    const float gd = (o.y - S.ground) / (-d.y);
    if (gd < kDistLimit && gd < closest) {
      closest = gd;
      h.normal = mk3(0.f, 1.f, 0.f);
      f3 c = mk3(0.3f, 0.5f, 0.7f);
      const f3 p = o + d * closest;
      if (p.x <= 1.f && p.x >= 0.f && p.z <= 1.f && p.z >= 0.f)
        c = c * (float)((double)((((int)(p.x / 0.25f) + (int)(p.z / 0.25f)) % 2)) * 0.2 + 0.35);
      else
        c = c * 0.4f;
      h.color = c;
    }
  }
  if (S.nb > 0) {
    int j = 0, id = 0;
    float dist = 0.f, sv = 1e9f;
    f3 pp = o;
    while (j < 200 && dist < kDistLimit && sv > 1e-8f) {
      pp = o + d * dist;
      sv = 1e9f;
      for (int b = 0; b < S.nb; ++b) {
        const float t = shape_sdf(S.shape[b].tfsr, S.shape[b].args, xform_inv(S.pose[b].p, S.pose[b].q, pp));
        if (t < sv) {
          sv = t;
          id = b;
        }
      }
      dist += sv;
      ++j;
    }
    if (dist < closest && dist < kDistLimit) {
      closest = dist;
      const f3 gb = xform_inv(S.pose[id].p, S.pose[id].q, pp);
      h.normal = qrot(S.pose[id].q, normalized(body_normal_local(S.shape[id].tfsr, S.shape[id].args, gb)));
      h.color = mk3(0.5f, 0.5f, 0.5f);
    }
  }
  float tn = 0.f, tf = 0.f;
  if (S.volume_on && ray_box(S.V.lower, S.V.upper, o, d, tn, tf)) {
    tn = fmaxf(tn, 0.f);
    f3 pos = o + d * (float)((double)tn + 1e-4);
    f3 step = mk3(0.f, 0.f, 0.f);
    for (int j = 0; j < 500; ++j) {
      const float s = sample_sdf(S.V, pos, S.V.thr);
      if (s < 0.f) {
        f3 back = step;
        for (int k = 0; k < 20; ++k) {
          back = back * 0.5f;
          if (sample_sdf(S.V, pos - back, S.V.thr) < 0.f) pos = pos - back;
        }
        const f3 od = o - pos;
        const float dist = sqrtf(dot(od, od));
        if (dist < closest) {
          closest = dist;
          h.normal = normalized(sample_normal(S.V, pos));
          float c[3] = {0.f, 0.f, 0.f};
          volume_query<3>(S.V, S.V.color, pos, c);
          h.color = mk3(c[0], c[1], c[2]);
        }
        break;
      }
      step = d * (float)fmax((double)s * 0.05, 0.01);
      pos = pos + step;
    }
  }
  return closest;
}

struct Camera {
  float rot[9], intr[9];
  f3 pos, light;
};

__device__ __forceinline__ f3 mat_vec(const float m[9], f3 v) {
  return mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
             m[6] * v.x + m[7] * v.y + m[8] * v.z);
}

// integrator.cu:1287-1436
__global__ void __launch_bounds__(256) k_render(Volume V, const float *__restrict__ body_pos,
                                                const float *__restrict__ body_rot,
                                                const float *__restrict__ body_tfsr,
                                                const float *__restrict__ body_args, int nb, bool volume_on,
                                                Camera cam, int H, int W, int max_depth, int spp, float ground, int seed,
                                                float *__restrict__ color_buf, float *__restrict__ depth_buf) {
  __shared__ BodyPose s_pose[kMaxRenderBodies];
  __shared__ BodyShape s_shape[kMaxRenderBodies];
  for (int b = threadIdx.y * blockDim.x + threadIdx.x; b < nb; b += blockDim.x * blockDim.y) {
    s_pose[b].p = mk3(body_pos[3 * b], body_pos[3 * b + 1], body_pos[3 * b + 2]);
    s_pose[b].q = mkq(body_rot[4 * b], body_rot[4 * b + 1], body_rot[4 * b + 2], body_rot[4 * b + 3]);
    s_shape[b].tfsr = mkq(body_tfsr[4 * b], body_tfsr[4 * b + 1], body_tfsr[4 * b + 2], body_tfsr[4 * b + 3]);
    s_shape[b].args = mkq(body_args[4 * b], body_args[4 * b + 1], body_args[4 * b + 2], body_args[4 * b + 3]);
  }
  __syncthreads();
  const int u = blockIdx.x * blockDim.x + threadIdx.x;  // column, < W
  const int v = blockIdx.y * blockDim.y + threadIdx.y;  // row, < H
  if (u >= W || v >= H) return;
  const int p = v * W + u;
  Scene S{V, s_pose, s_shape, nb, volume_on, ground};
  Rng rng(seed, p);
  f3 acc = mk3(0.f, 0.f, 0.f);
  float depth = 0.f;
  for (int sample = 0; sample < spp; ++sample) {
    // the reference's host build draws the second jitter first
    const float jy = rng.uniform();
    const float jx = rng.uniform();
    f3 dir = mat_vec(cam.intr, mk3((float)u + jx, (float)v + jy, 1.f));
    f3 d = mat_vec(cam.rot, normalized(dir));
    f3 pos = cam.pos;
    f3 contrib = mk3(0.f, 0.f, 0.f), through = mk3(1.f, 1.f, 1.f);
    float first = 0.f;
    for (int bounce = 0; bounce < max_depth; ++bounce) {
      Hit h;
      h.normal = mk3(0.f, 0.f, 0.f);
      h.color = mk3(0.f, 0.f, 0.f);
      const float closest = next_hit(S, pos, d, h);
      if (bounce == 0) first = closest;
      const f3 hit = pos + d * closest;
      if (!(dot(h.normal, h.normal) > 1e-10f)) break;
      f3 t1 = mk3(1.f, 0.f, 0.f);
      if ((double)fabsf(h.normal.y) < 1 - 1e-3) t1 = normalized(cross(h.normal, mk3(0.f, 1.f, 0.f)));
      const f3 t2 = cross(h.normal, t1);
      const float phi = (float)(2.0 * 3.14159265358979323846 * (double)rng.uniform());
      const float r = rng.uniform();
      const float ay = sqrtf(r), ax = sqrtf(1.f - r);
      // cos and sin in double, rounded to float, as the reference's host build
      const float cph = (float)cos((double)phi), sph = (float)sin((double)phi);
      const f3 out = (t1 * cph + t2 * sph) * ax + h.normal * ay;
      d = normalized(out);
      pos = hit + d * 1e-4f;
      through = hadamard(through, h.color);
      const float nz = rng.uniform() - 0.5f, ny = rng.uniform() - 0.5f, nx = rng.uniform() - 0.5f;
      const f3 direct = normalized(cam.light + mk3(nx, ny, nz) * 0.1f);
      const float cosl = dot(direct, h.normal);
      if (cosl > 0.f) {
        Hit hs;
        if (next_hit(S, pos, direct, hs) > kDistLimit) contrib = contrib + (through * cosl) * 0.8f;
      }
    }
    // every path ends with the sky term (integrator.cu:1393-1398)
    contrib = contrib + through * 0.8f;
    const float fs = (float)spp;
    acc = acc + mk3(contrib.x / fs, contrib.y / fs, contrib.z / fs);
    depth += first / fs;
  }
  const float uu = (float)(1.0 * u / W), vv = (float)(1.0 * v / H);
  const float r2 = (uu - 0.5f) * (uu - 0.5f) + (vv - 0.5f) * (vv - 0.5f);
  const float darken = (float)(1.0 - (double)0.9f * fmax(sqrt((double)r2), 0.0));
  const f3 c = acc * darken * 1.5f;
  color_buf[3 * (size_t)p] = sqrtf(c.x);
  color_buf[3 * (size_t)p + 1] = sqrtf(c.y);
  color_buf[3 * (size_t)p + 2] = sqrtf(c.z);
  depth_buf[p] = depth;
}

// ------------------------------------------------------------ bake
// integrator.cu:1480-1523.  Work item w = ((particle * width + i) * width + j) * width + k.
__global__ void k_bake(long long *__restrict__ volume, const float *__restrict__ x, const int *__restrict__ color,
                       const float *__restrict__ bmin, int bake, int gx, int gy, int gz, float inv_dx, long long total) {
  const int width = 2 * bake;
  const f3 lo = mk3(__ldg(bmin), __ldg(bmin + 1), __ldg(bmin + 2));
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < total;
       w += (long long)gridDim.x * blockDim.x) {
    long long q = w;
    const int k = (int)(q % width) - bake;
    q /= width;
    const int j = (int)(q % width) - bake;
    q /= width;
    const int i = (int)(q % width) - bake;
    const int p = (int)(q / width);
    const float px = __fmul_rn(__fsub_rn(__ldg(x + 3 * p), lo.x), inv_dx);
    const float py = __fmul_rn(__fsub_rn(__ldg(x + 3 * p + 1), lo.y), inv_dx);
    const float pz = __fmul_rn(__fsub_rn(__ldg(x + 3 * p + 2), lo.z), inv_dx);
    const int ix = (int)floorf(px) + i, iy = (int)floorf(py) + j, iz = (int)floorf(pz) + k;
    if (ix < 0 || iy < 0 || iz < 0 || ix >= gx || iy >= gy || iz >= gz) continue;
    const float ex = __fsub_rn((float)ix, px), ey = __fsub_rn((float)iy, py), ez = __fsub_rn((float)iz, pz);
    const float dd = __fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez));
    float dist = sqrtf(__fadd_rn(dd, 0.f));
    dist = fminf(fmaxf(0.f, __fmul_rn(255.0f * 0.2f, dist)), 255.f);
    const long long packed = ((long long)dist << 24) + (long long)__ldg(color + p);
    atomicMin(volume + ((size_t)ix * gy + iy) * gz + iz, packed);
  }
}

// integrator.cu:1463-1478
__global__ void k_unpack(const long long *__restrict__ volume, float *__restrict__ sdf, float *__restrict__ color,
                         int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    long long c = volume[t];
    const float z = (float)((double)(c & 255) / 255.);
    c >>= 8;
    const float y = (float)((double)(c & 255) / 255.);
    c >>= 8;
    const float xx = (float)((double)(c & 255) / 255.);
    c >>= 8;
    color[3 * (size_t)t] = xx;
    color[3 * (size_t)t + 1] = y;
    color[3 * (size_t)t + 2] = z;
    sdf[t] = (float)((double)(c & 255) / 255.);
  }
}

// integrator.cu:1438-1461: 3^3 box filter, border voxels 1
__global__ void k_smooth(const float *__restrict__ in, float *__restrict__ out, int gx, int gy, int gz) {
  const int n = gx * gy * gz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int x = t / gz / gy, y = (t / gz) % gy, z = t % gz;
    if (x >= 1 && y >= 1 && z >= 1 && x < gx - 1 && y < gy - 1 && z < gz - 1) {
      float sum = 0.f;
      for (int i = -1; i < 2; ++i)
        for (int j = -1; j < 2; ++j)
          for (int k = -1; k < 2; ++k) sum = __fadd_rn(sum, __ldg(in + ((x + i) * gy + (y + j)) * gz + (z + k)));
      out[t] = (float)((double)sum / 27.);
    } else {
      out[t] = 1.f;
    }
  }
}

int launched() { return cudaGetLastError() == cudaSuccess ? DEXMPM_OK : DEXMPM_ERR_LAUNCH; }

// Grid of a grid-stride launch over n items: at most 16 CTAs per SM of the
// current device.
int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                 cudaSuccess || sms < 1)
    sms = 1;
  const long long cap = 16LL * sms;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

extern "C" {

int particle_sdf(long long *volume, float *particle_x, int *particle_color, float *bbox_min, float *bbox_max,
                 int bake_size, const int *grid_dim, float inv_dx, float *sdf, float *color, float *sdf_tmp,
                 int n_particles, dexmpm_stream_t stream) {
  (void)bbox_max;
  if (!grid_dim || grid_dim[0] <= 0 || grid_dim[1] <= 0 || grid_dim[2] <= 0 || n_particles < 0 || bake_size < 0)
    return DEXMPM_ERR_ARG;
  if (!volume || !sdf || !color || !sdf_tmp || !bbox_min || (n_particles > 0 && (!particle_x || !particle_color)))
    return DEXMPM_ERR_ARG;
  const int gx = grid_dim[0], gy = grid_dim[1], gz = grid_dim[2];
  if ((long long)gx * gy * gz > (1LL << 31) - 1) return DEXMPM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const long long width = 2LL * bake_size;
  const long long total = (long long)n_particles * width * width * width;
  if (total > 0) {
    k_bake<<<grid_for(total, 256), 256, 0, st>>>(volume, particle_x, particle_color, bbox_min, bake_size, gx, gy, gz,
                                                 inv_dx, total);
    if (int rc = launched()) return rc;
  }
  const int n = gx * gy * gz;
  k_unpack<<<grid_for(n, 256), 256, 0, st>>>(volume, sdf, color, n);
  if (int rc = launched()) return rc;
  k_smooth<<<grid_for(n, 256), 256, 0, st>>>(sdf, sdf_tmp, gx, gy, gz);
  if (int rc = launched()) return rc;
  k_smooth<<<grid_for(n, 256), 256, 0, st>>>(sdf_tmp, sdf, gx, gy, gz);
  return launched();
}

int render(float *sdf_volume, float *box_min, float *box_max, float *color_volume, float *body_pos, float *body_rot,
           float *body_type_friction_softness_round, float *body_args, float *camera_rot, float *camera_pos,
           float *camera_intrinsic, float *color_buffer, float *depth_buffer, float sdf_threshold, const int *grid_dim,
           int n_bodies, bool visualize_shape, const int *image_dim, int max_ray_depth, int spp, float ground_height,
           int seed, float *light_direction, dexmpm_stream_t stream) {
  if (!grid_dim || !image_dim || !camera_rot || !camera_pos || !camera_intrinsic || !color_buffer || !depth_buffer ||
      !light_direction || !box_min || !box_max)
    return DEXMPM_ERR_ARG;
  if (n_bodies < 0 || n_bodies > kMaxRenderBodies || spp < 1 || max_ray_depth < 0) return DEXMPM_ERR_ARG;
  if (n_bodies > 0 && (!body_pos || !body_rot || !body_type_friction_softness_round || !body_args))
    return DEXMPM_ERR_ARG;
  if (visualize_shape && (!sdf_volume || !color_volume || grid_dim[0] <= 0 || grid_dim[1] <= 0 || grid_dim[2] <= 0))
    return DEXMPM_ERR_ARG;
  const int H = image_dim[0], W = image_dim[1];
  if (H <= 0 || W <= 0) return DEXMPM_ERR_ARG;
  // the small inputs (camera, box, light) are device pointers, as in the
  // reference; read them once into the launch parameters
  cudaStream_t st = (cudaStream_t)stream;
  float host[9 + 9 + 3 + 3 + 3 + 3];
  const struct {
    const float *src;
    int n;
  } parts[] = {{camera_rot, 9}, {camera_intrinsic, 9}, {camera_pos, 3}, {light_direction, 3}, {box_min, 3},
               {box_max, 3}};
  int off = 0;
  for (const auto &pt : parts) {
    if (cudaMemcpyAsync(host + off, pt.src, sizeof(float) * pt.n, cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return DEXMPM_ERR_LAUNCH;
    off += pt.n;
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return DEXMPM_ERR_LAUNCH;
  Camera cam;
  for (int i = 0; i < 9; ++i) cam.rot[i] = host[i], cam.intr[i] = host[9 + i];
  cam.pos = mk3(host[18], host[19], host[20]);
  cam.light = mk3(host[21], host[22], host[23]);
  Volume V;
  V.sdf = sdf_volume;
  V.color = color_volume;
  V.lower = mk3(host[24], host[25], host[26]);
  V.upper = mk3(host[27], host[28], host[29]);
  V.dx = grid_dim[0];
  V.dy = grid_dim[1];
  V.dz = grid_dim[2];
  V.thr = sdf_threshold;
  const dim3 block(16, 16), grid((W + 15) / 16, (H + 15) / 16);
  k_render<<<grid, block, 0, st>>>(V, body_pos, body_rot, body_type_friction_softness_round, body_args, n_bodies,
                                   visualize_shape, cam, H, W, max_ray_depth, spp, ground_height, seed, color_buffer,
                                   depth_buffer);
  return launched();
}

}  // extern "C"
