// ref_abi.cu -- drop-in replacements for the reference's extern "C" kernel
// launchers (mpm/csrc/integrator.cu:1616-1985): same names, arguments, AoS
// layouts and dense x-major grids, so mpm/types.py can bind this library in
// place of libmaniskill_mpm.so for the substep path.
//
// Each kernel restates the cited reference kernel in FP32 (the reference's own
// precision); compute_svd uses the SVD of mpm_math.cuh (same conventions).
// Scatter kernels reduce per-warp before atomics where lanes share an address
// (body-pose gradients); particle scatters use one atomic per value as the
// reference layout (12-byte vec3 cells) admits no vector atomics.
// Departures from the reference, all on invalid input only: particles whose
// stencil leaves the grid are skipped and flagged instead of corrupting memory,
// and every launcher returns a status.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_math.cuh"
#include "../../include/dexmpm.h"

using namespace dexmpm;

namespace {

constexpr unsigned kFull = 0xffffffffu;
__device__ int32_t g_abi_error = 0;

__device__ __forceinline__ f3 ld3(const float *p, long i) { return mk3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void st3(float *p, long i, f3 v) { p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }
__device__ __forceinline__ void add3(float *p, long i, f3 v) { p[3 * i] += v.x; p[3 * i + 1] += v.y; p[3 * i + 2] += v.z; }
__device__ __forceinline__ void atomic3(float *p, long i, f3 v) {
  atomicAdd(p + 3 * i, v.x); atomicAdd(p + 3 * i + 1, v.y); atomicAdd(p + 3 * i + 2, v.z);
}
__device__ __forceinline__ m33 ld9(const float *p, long i) {
  m33 m;
#pragma unroll
  for (int k = 0; k < 9; ++k) m.a[k / 3][k % 3] = p[9 * i + k];
  return m;
}
__device__ __forceinline__ void st9(float *p, long i, const m33 &m) {
#pragma unroll
  for (int k = 0; k < 9; ++k) p[9 * i + k] = m.a[k / 3][k % 3];
}
__device__ __forceinline__ void add9(float *p, long i, const m33 &m) {
#pragma unroll
  for (int k = 0; k < 9; ++k) p[9 * i + k] += m.a[k / 3][k % 3];
}
__device__ __forceinline__ qf ldq(const float *p, long i) { return mkq(p[4 * i], p[4 * i + 1], p[4 * i + 2], p[4 * i + 3]); }

struct Grid {
  int x, y, z;
};
__device__ __forceinline__ long gidx(const Grid &g, int x, int y, int z) { return ((long)x * g.y + y) * g.z + z; }

__device__ __forceinline__ f3 lower_offset(const int *grid_lower, float dx) {
  if (!grid_lower) return mk3(0.f, 0.f, 0.f);
  return mk3(grid_lower[0] * dx, grid_lower[1] * dx, grid_lower[2] * dx);
}

__device__ __forceinline__ bool in_grid(const Grid &g, const Stencil &st) {
  bool ok = st.base[0] >= 0 && st.base[1] >= 0 && st.base[2] >= 0 && st.base[0] + 2 < g.x && st.base[1] + 2 < g.y &&
            st.base[2] + 2 < g.z;
  if (!ok) atomicOr(&g_abi_error, DEXMPM_ERR_OUT_OF_GRID);
  return ok;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
  return v;
}

// integrator.cu:84-100
__global__ void k_compute_svd(const float *F, const float *C, float *newF, float *U, float *V, float *sig, float dt,
                              int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  m33 E = deviation_tmp(ld9(F, p), ld9(C, p), dt);
  SVD3 s = svd3_from_deviation(E);
  E.a[0][0] += 1.f; E.a[1][1] += 1.f; E.a[2][2] += 1.f;
  st9(newF, p, E);
  st9(U, p, s.U);
  st9(V, p, s.V);
  st3(sig, p, s.s);
}

// integrator.cu:110-186
__global__ void k_compute_svd_grad(const float *F, const float *C, const float *U, const float *V, const float *sig,
                                   float *newF_grad, const float *U_grad, const float *V_grad, const float *sig_grad,
                                   float *F_grad, float *C_grad, float dt, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  SVD3 sv;
  sv.U = ld9(U, p);
  sv.V = ld9(V, p);
  sv.s = ld3(sig, p);
  sv.d = mk3(sv.s.x - 1.f, sv.s.y - 1.f, sv.s.z - 1.f);
  m33 g = svd_backward(sv, ld9(U_grad, p), ld3(sig_grad, p), ld9(V_grad, p), ld9(newF_grad, p));
  st9(newF_grad, p, g);
  m33 Fp = ld9(F, p), Cp = ld9(C, p);
  add9(C_grad, p, mm(g, mT(Fp)) * dt);
  m33 I = Cp * dt;
  I.a[0][0] += 1.f; I.a[1][1] += 1.f; I.a[2][2] += 1.f;
  add9(F_grad, p, mm(mT(I), g));
}

// von Mises as written in integrator.cu:42-67 on given (F_tmp, U, sigma, V)
__device__ __forceinline__ float von_mises_ref(const m33 &F, const m33 &U, f3 s, const m33 &V, float ys, float mu,
                                               m33 &outF) {
  f3 sn = fmax3(s, kSigClip);
  f3 e = mk3(logf(sn.x), logf(sn.y), logf(sn.z));
  float mean = (e.x + e.y + e.z) / 3.f;
  f3 eh = mk3(e.x - mean, e.y - mean, e.z - mean);
  float ehn = sqrtf(dot(eh, eh) + kNormEps);
  float dg = ehn - ys / (2.f * mu);
  if (dg > 0.f) {
    e = e - eh * (dg / ehn);
    f3 ee = mk3(expf(e.x), expf(e.y), expf(e.z));
    outF = usv(U, ee, V);
    return ee.x * ee.y * ee.z;
  }
  outF = F;
  return s.x * s.y * s.z;
}

// integrator.cu:312-394
__global__ void k_p2g(const float *x, const float *v, const float *m, const float *vol, const float *F,
                      const float *U, const float *sig, const float *V, const float *C, const float *mly,
                      const int *grid_lower, Grid g, float dx, float inv_dx, float dt, float *outF, float *grid_mv,
                      float *grid_m, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  f3 xp = ld3(x, p) - lower_offset(grid_lower, dx);
  Stencil st;
  make_stencil(xp, inv_dx, st);
  if (!in_grid(g, st)) return;
  m33 Um = ld9(U, p), Vm = ld9(V, p), nF;
  f3 mlyp = ld3(mly, p);
  float J = von_mises_ref(ld9(F, p), Um, ld3(sig, p), Vm, mlyp.z, mlyp.x, nF);
  st9(outF, p, nF);
  m33 r = mm(Um, mT(Vm));
  m33 stress = mm(nF - r, mT(nF)) * (2.f * mlyp.x);
  float iso = mlyp.y * J * (J - 1.f);
  stress.a[0][0] += iso; stress.a[1][1] += iso; stress.a[2][2] += iso;
  stress = stress * (-dt * vol[p] * 4.f * inv_dx * inv_dx);
  float mp = m[p];
  m33 affine = stress + ld9(C, p) * mp;
  f3 mom = ld3(v, p) * mp;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        float w = st.w[0][i] * st.w[1][j] * st.w[2][k];
        f3 dpos = mk3(((float)i - st.fx[0]) * dx, ((float)j - st.fx[1]) * dx, ((float)k - st.fx[2]) * dx);
        long id = gidx(g, st.base[0] + i, st.base[1] + j, st.base[2] + k);
        atomicAdd(grid_m + id, mp * w);
        atomic3(grid_mv, id, (mom + mv(affine, dpos)) * w);
      }
}

// integrator.cu:396-627
__global__ void k_p2g_grad(const float *x, const float *v, const float *m, const float *vol, const float *F,
                           const float *U, const float *sig, const float *V, const float *C, const float *mly,
                           const int *grid_lower, Grid g, float dx, float inv_dx, float dt, float *x_grad,
                           float *v_grad, float *F_grad, float *C_grad, float *U_grad, float *sig_grad, float *V_grad,
                           const float *outF_grad, const float *grid_v_grad, const float *grid_m_grad, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  f3 xp = ld3(x, p) - lower_offset(grid_lower, dx);
  Stencil st;
  make_stencil(xp, inv_dx, st);
  if (!in_grid(g, st)) return;
  m33 Um = ld9(U, p), Vm = ld9(V, p);
  f3 s = ld3(sig, p), mlyp = ld3(mly, p);
  float mu = mlyp.x, lam = mlyp.y, ys = mlyp.z;
  f3 sn = fmax3(s, kSigClip);
  f3 e = mk3(logf(sn.x), logf(sn.y), logf(sn.z));
  float mean = (e.x + e.y + e.z) / 3.f;
  f3 eh = mk3(e.x - mean, e.y - mean, e.z - mean);
  float ehn = sqrtf(dot(eh, eh) + kNormEps);
  float dg = ehn - ys / (2.f * mu);
  m33 nF;
  float J;
  f3 ee = mk3(0.f, 0.f, 0.f);
  if (dg > 0.f) {
    f3 ep = e - eh * (dg / ehn);
    ee = mk3(expf(ep.x), expf(ep.y), expf(ep.z));
    nF = usv(Um, ee, Vm);
    J = ee.x * ee.y * ee.z;
  } else {
    nF = ld9(F, p);
    J = s.x * s.y * s.z;
  }
  m33 r = mm(Um, mT(Vm));
  float gss = -dt * inv_dx * vol[p] * 4.f * inv_dx;
  m33 stress = mm(nF - r, mT(nF)) * (2.f * mu);
  float iso = lam * J * (J - 1.f);
  stress.a[0][0] += iso; stress.a[1][1] += iso; stress.a[2][2] += iso;
  float mp = m[p];
  m33 affine = stress * gss + ld9(C, p) * mp;
  f3 vp = ld3(v, p);
  float w1[3][3];
  make_dweights(st, inv_dx, w1);
  m33 g_stress = mzero(), g_C = mzero();
  f3 g_x = mk3(0.f, 0.f, 0.f), g_v = mk3(0.f, 0.f, 0.f);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        long id = gidx(g, st.base[0] + i, st.base[1] + j, st.base[2] + k);
        float N = st.w[0][i] * st.w[1][j] * st.w[2][k];
        f3 dpos = mk3(((float)i - st.fx[0]) * dx, ((float)j - st.fx[1]) * dx, ((float)k - st.fx[2]) * dx);
        f3 gov = ld3(grid_v_grad, id);
        f3 gN = mk3(w1[0][i] * st.w[1][j] * st.w[2][k], st.w[0][i] * w1[1][j] * st.w[2][k],
                    st.w[0][i] * st.w[1][j] * w1[2][k]);
        m33 tmp = outer(gov, dpos);
        g_stress += tmp * (N * gss);
        g_C += tmp * (N * mp);
        float gm = grid_m_grad[id];
        g_v += gov * (N * mp);
        g_x += gN * (gm * mp);
        g_x += gN * (dot(vp, gov) * mp);
        g_x += mtv(affine, gov) * (-N) + gN * dot(mv(affine, dpos), gov);
      }
  add3(x_grad, p, g_x);
  add3(v_grad, p, g_v);
  add9(C_grad, p, g_C);
  m33 g_r = mm(g_stress, nF) * (-2.f * mu);
  m33 gU = mm(g_r, Vm);
  m33 gV = mm(mT(g_r), Um);
  m33 g_nF = ld9(outF_grad, p) + (mm(mT(g_stress), nF - r) + mm(g_stress, nF)) * (2.f * mu);
  float g_J = ((2.f * J - 1.f) * lam) * trace(g_stress);
  f3 g_s = mk3(0.f, 0.f, 0.f);
  m33 g_F = mzero();
  if (dg > 0.f) {
    m33 ed = mdiag(ee);
    gU += mm(mm(g_nF, Vm), ed);
    gV += mm(mm(mT(g_nF), Um), ed);
    m33 t = mm(mm(mT(Um), g_nF), Vm);
    f3 Fpart = mk3(t.a[0][0], t.a[1][1], t.a[2][2]);
    f3 Jpart = mk3(g_J * ee.y * ee.z, g_J * ee.x * ee.z, g_J * ee.x * ee.y);
    f3 g_e = hadamard(ee, Jpart + Fpart);
    f3 g_eh = g_e * (-dg / ehn);
    float g_ehn = -dot(eh * (1.f / ehn), g_e) * (ys / (2.f * mu)) / ehn;
    g_eh += eh * (g_ehn / ehn);
    float sm = (g_eh.x + g_eh.y + g_eh.z) / 3.f;
    g_e += mk3(g_eh.x - sm, g_eh.y - sm, g_eh.z - sm);
    if (s.x >= kSigClip) g_s.x += g_e.x / s.x;
    if (s.y >= kSigClip) g_s.y += g_e.y / s.y;
    if (s.z >= kSigClip) g_s.z += g_e.z / s.z;
  } else {
    g_s = mk3(g_J * s.y * s.z, g_J * s.x * s.z, g_J * s.x * s.y);
    g_F = g_nF;
  }
  add9(U_grad, p, gU);
  add9(V_grad, p, gV);
  add3(sig_grad, p, g_s);
  add9(F_grad, p, g_F);
}

// integrator.cu:647-777
__global__ void k_grid_op(const float *grid_m, const float *grid_v_in, float *grid_body_v_in, const int *grid_lower,
                          const float *gravity, const float *bpos, const float *brot, const float *nbpos,
                          const float *nbrot, const float *tfsr, const float *bargs, float dx, float dt, float gf,
                          float *out_v, Grid g, int nb, long dim) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= dim || !(grid_m[t] > kMassEps)) return;
  int gxi = (int)(t / g.z / g.y), gyi = (int)((t / g.z) % g.y), gzi = (int)(t % g.z);
  float m = grid_m[t];
  f3 v = ld3(grid_v_in, t) * (1.f / m) + ld3(gravity, 0) * dt;
  f3 gx = lower_offset(grid_lower, dx) + mk3(gxi * dx, gyi * dx, gzi * dx);
  for (int b = 0; b < nb; ++b) {
    st3(grid_body_v_in, t * (nb + 1) + b, v);
    BodyPose cur, nxt;
    BodyShape sh;
    cur.p = ld3(bpos, b); cur.q = ldq(brot, b);
    nxt.p = ld3(nbpos, b); nxt.q = ldq(nbrot, b);
    sh.tfsr = ldq(tfsr, b); sh.args = ldq(bargs, b);
    contact_forward(gx, v, cur, nxt, sh, dt);
  }
  st3(grid_body_v_in, t * (nb + 1) + nb, v);
  st3(out_v, t, boundary_forward(v, gxi, gyi, gzi, g.x, g.y, g.z, gf));
}

// integrator.cu:779-1057; body-pose gradients reduced per warp before atomics
__global__ void k_grid_op_grad(const float *grid_m, const float *grid_v_in, const float *grid_body_v_in,
                               const int *grid_lower, const float *bpos, const float *brot, const float *nbpos,
                               const float *nbrot, const float *tfsr, const float *bargs, float *grid_m_grad,
                               float *grid_v_in_grad, float *bpos_grad, float *brot_grad, float *nbpos_grad,
                               float *nbrot_grad, float dx, float dt, float gf, const float *out_v_grad, Grid g, int nb,
                               long dim) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  bool active = t < dim && grid_m[t] > kMassEps;
  long tt = active ? t : 0;
  int gxi = (int)(tt / g.z / g.y), gyi = (int)((tt / g.z) % g.y), gzi = (int)(tt % g.z);
  f3 gv = mk3(0.f, 0.f, 0.f);
  if (active)
    gv = boundary_backward(ld3(out_v_grad, t), ld3(grid_body_v_in, t * (nb + 1) + nb), gxi, gyi, gzi, g.x, g.y, g.z, gf);
  f3 gx = lower_offset(grid_lower, dx) + mk3(gxi * dx, gyi * dx, gzi * dx);
  for (int b = nb - 1; b >= 0; --b) {
    float gc[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, gn[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    BodyPose cur, nxt;
    BodyShape sh;
    cur.p = ld3(bpos, b); cur.q = ldq(brot, b);
    nxt.p = ld3(nbpos, b); nxt.q = ldq(nbrot, b);
    sh.tfsr = ldq(tfsr, b); sh.args = ldq(bargs, b);
    if (active) contact_backward(gx, ld3(grid_body_v_in, t * (nb + 1) + b), gv, cur, nxt, sh, dt, gc, gn);
    bool any = false;
#pragma unroll
    for (int c = 0; c < 7; ++c) any |= (gc[c] != 0.f) | (gn[c] != 0.f);
    if (!__any_sync(kFull, any)) continue;
#pragma unroll
    for (int c = 0; c < 7; ++c) {
      float a = warp_sum(gc[c]), n = warp_sum(gn[c]);
      if (lane == 0) {
        if (c < 3) {
          atomicAdd(bpos_grad + 3 * b + c, a);
          atomicAdd(nbpos_grad + 3 * b + c, n);
        } else {
          atomicAdd(brot_grad + 4 * b + c - 3, a);
          atomicAdd(nbrot_grad + 4 * b + c - 3, n);
        }
      }
    }
  }
  if (active) {
    float m = grid_m[t];
    add3(grid_v_in_grad, t, gv * (1.f / m));
    grid_m_grad[t] += (-1.f / m / m) * dot(ld3(grid_v_in, t), gv);
  }
}

// integrator.cu:1059-1109
__global__ void k_g2p(const float *x, const float *grid_v, const int *grid_lower, float dx, float inv_dx, float dt,
                      Grid g, float *out_v, float gh, float *out_C, float *out_x, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  f3 low = lower_offset(grid_lower, dx);
  f3 xp = ld3(x, p) - low;
  Stencil st;
  make_stencil(xp, inv_dx, st);
  if (!in_grid(g, st)) return;
  f3 nv = mk3(0.f, 0.f, 0.f);
  m33 nC = mzero();
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        float w = st.w[0][i] * st.w[1][j] * st.w[2][k];
        f3 dpos = mk3((float)i - st.fx[0], (float)j - st.fx[1], (float)k - st.fx[2]);
        f3 gv = ld3(grid_v, gidx(g, st.base[0] + i, st.base[1] + j, st.base[2] + k));
        nv += gv * w;
        nC += outer(gv, dpos) * (w * inv_dx * 4.f);
      }
  f3 nx = xp + nv * dt;
  nx.x = fmaxf(fminf(nx.x, (g.x - 3.f) * dx), gh * dx);
  nx.y = fmaxf(fminf(nx.y, (g.y - 3.f) * dx), gh * dx);
  nx.z = fmaxf(fminf(nx.z, (g.z - 3.f) * dx), gh * dx);
  st3(out_x, p, nx + low);
  st3(out_v, p, nv);
  st9(out_C, p, nC);
}

// integrator.cu:1527-1614
__global__ void k_g2p_grad(const float *x, const float *grid_v, const int *grid_lower, float dx, float inv_dx,
                           float dt, Grid g, const float *out_v, float gh, float *x_grad, float *grid_v_grad,
                           const float *out_v_grad, const float *out_C_grad, const float *out_x_grad, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  f3 xp = ld3(x, p) - lower_offset(grid_lower, dx);
  Stencil st;
  make_stencil(xp, inv_dx, st);
  if (!in_grid(g, st)) return;
  f3 gx = ld3(out_x_grad, p), gnv = ld3(out_v_grad, p);
  m33 gC = ld9(out_C_grad, p);
  f3 nx = xp + ld3(out_v, p) * dt;
  float lo = gh * dx;
  if (nx.x > (g.x - 3.f) * dx || nx.x < lo) gx.x = 0.f;
  if (nx.y > (g.y - 3.f) * dx || nx.y < lo) gx.y = 0.f;
  if (nx.z > (g.z - 3.f) * dx || nx.z < lo) gx.z = 0.f;
  gnv += gx * dt;
  float w1[3][3];
  make_dweights(st, inv_dx, w1);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        float w = st.w[0][i] * st.w[1][j] * st.w[2][k];
        f3 dpos = mk3((float)i - st.fx[0], (float)j - st.fx[1], (float)k - st.fx[2]);
        long id = gidx(g, st.base[0] + i, st.base[1] + j, st.base[2] + k);
        f3 gv = ld3(grid_v, id);
        float xx = w * inv_dx * 4.f;
        atomic3(grid_v_grad, id, gnv * w + mv(gC, dpos) * xx);
        gx += mtv(gC, gv) * (-inv_dx * xx);
        float gw = dot(gnv, gv) + inv_dx * 4.f * dot(gv, mv(gC, dpos));
        gx += mk3(w1[0][i] * st.w[1][j] * st.w[2][k], st.w[0][i] * w1[1][j] * st.w[2][k],
                  st.w[0][i] * st.w[1][j] * w1[2][k]) * gw;
      }
  add3(x_grad, p, gx);
}

// integrator.cu:188-237
__global__ void k_compute_dist(const float *x, const float *bpos, const float *brot, const float *tfsr,
                               const float *bargs, float *dist, int nb, float *x_grad, float *bpos_grad,
                               float *brot_grad, const float *dist_grad, int compute_grad, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  bool act = p < n;
  int pp = act ? p : 0;
  f3 xp = ld3(x, pp);
  f3 gxp = mk3(0.f, 0.f, 0.f);
  for (int b = 0; b < nb; ++b) {
    f3 bx = ld3(bpos, b);
    qf bq = ldq(brot, b), tf = ldq(tfsr, b), ar = ldq(bargs, b);
    f3 gxb = xform_inv(bx, bq, xp);
    if (!compute_grad) {
      if (act) dist[(long)p * nb + b] = shape_sdf(tf, ar, gxb);
      continue;
    }
    float gd = act ? dist_grad[(long)p * nb + b] : 0.f;
    f3 g_gxb = shape_grad(tf, ar, gxb) * gd;
    f3 g_bx = mk3(0.f, 0.f, 0.f);
    qf g_bq = mkq(0.f, 0.f, 0.f, 0.f);
    xform_inv_backward(bx, bq, xp, g_gxb, g_bx, g_bq, gxp);
    float vals[7] = {g_bx.x, g_bx.y, g_bx.z, g_bq.w, g_bq.x, g_bq.y, g_bq.z};
#pragma unroll
    for (int c = 0; c < 7; ++c) {
      float s = warp_sum(vals[c]);
      if (lane == 0) atomicAdd(c < 3 ? bpos_grad + 3 * b + c : brot_grad + 4 * b + c - 3, s);
    }
  }
  if (compute_grad && act) add3(x_grad, p, gxp);
}

// integrator.cu:239-310
__global__ void k_particle2mass(const float *x, const float *mass, const int *grid_lower, Grid g, float dx,
                                float inv_dx, float *grid_m, const float *grid_m_grad, float *x_grad, const int *ids,
                                int id, int compute_grad, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (id != -1 && ids[p] != id) return;
  f3 xp = ld3(x, p) - lower_offset(grid_lower, dx);
  Stencil st;
  make_stencil(xp, inv_dx, st);
  if (!in_grid(g, st)) return;
  float w1[3][3];
  make_dweights(st, inv_dx, w1);
  f3 gx = mk3(0.f, 0.f, 0.f);
  float mp = mass[p];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        long gi = gidx(g, st.base[0] + i, st.base[1] + j, st.base[2] + k);
        if (compute_grad) {
          gx += mk3(w1[0][i] * st.w[1][j] * st.w[2][k], st.w[0][i] * w1[1][j] * st.w[2][k],
                    st.w[0][i] * st.w[1][j] * w1[2][k]) * (grid_m_grad[gi] * mp);
        } else {
          atomicAdd(grid_m + gi, mp * st.w[0][i] * st.w[1][j] * st.w[2][k]);
        }
      }
  if (compute_grad) add3(x_grad, p, gx);
}

constexpr int kThreads = 256;
inline int blocks_for(long n) { return (int)((n + kThreads - 1) / kThreads); }
inline int launched() { return cudaGetLastError() == cudaSuccess ? DEXMPM_OK : DEXMPM_ERR_LAUNCH; }
inline bool grid_ok(const int *gd) { return gd && gd[0] > 0 && gd[1] > 0 && gd[2] > 0; }

}  // namespace

extern "C" {

int compute_svd(float *F, float *C, float *newF, float *U, float *V, float *sig, float dt, int dim,
                dexmpm_stream_t stream) {
  if (dim < 0 || (dim > 0 && (!F || !C || !newF || !U || !V || !sig))) return DEXMPM_ERR_ARG;
  if (dim == 0) return DEXMPM_OK;
  k_compute_svd<<<blocks_for(dim), kThreads, 0, (cudaStream_t)stream>>>(F, C, newF, U, V, sig, dt, dim);
  return launched();
}

int compute_svd_grad(float *F, float *C, float *U, float *V, float *sig, float *newF_grad, float *U_grad,
                     float *V_grad, float *sig_grad, float *F_grad, float *C_grad, float dt, int dim,
                     dexmpm_stream_t stream) {
  if (dim < 0) return DEXMPM_ERR_ARG;
  if (dim == 0) return DEXMPM_OK;
  k_compute_svd_grad<<<blocks_for(dim), kThreads, 0, (cudaStream_t)stream>>>(F, C, U, V, sig, newF_grad, U_grad, V_grad,
                                                                              sig_grad, F_grad, C_grad, dt, dim);
  return launched();
}

int p2g(float *particle_x, float *particle_v, float *particle_m, float *particle_vol, float *particle_F,
        float *particle_U, float *particle_sig, float *particle_V, float *particle_C,
        float *particle_mu_lam_yield, int *grid_lower, const int *grid_dim, float dx, float inv_dx, float dt,
        float *out_particle_F, float *out_grid_mv, float *out_grid_m, int dim, dexmpm_stream_t stream) {
  if (dim < 0 || !grid_ok(grid_dim)) return DEXMPM_ERR_ARG;
  if (dim == 0) return DEXMPM_OK;
  Grid g{grid_dim[0], grid_dim[1], grid_dim[2]};
  k_p2g<<<blocks_for(dim), kThreads, 0, (cudaStream_t)stream>>>(
      particle_x, particle_v, particle_m, particle_vol, particle_F, particle_U, particle_sig, particle_V, particle_C,
      particle_mu_lam_yield, grid_lower, g, dx, inv_dx, dt, out_particle_F, out_grid_mv, out_grid_m, dim);
  return launched();
}

int p2g_grad(float *particle_x, float *particle_v, float *particle_m, float *particle_vol, float *particle_F,
             float *particle_U, float *particle_sig, float *particle_V, float *particle_C,
             float *particle_mu_lam_yield, int *grid_lower, const int *grid_dim, float dx, float inv_dx,
             float dt, float *out_particle_F, float *out_grid_mv, float *out_grid_m, float *particle_x_grad,
             float *particle_v_grad, float *particle_F_grad, float *particle_C_grad, float *particle_U_grad,
             float *particle_sig_grad, float *particle_V_grad, float *out_particle_F_grad,
             float *out_grid_v_grad, float *out_grid_m_grad, int dim, dexmpm_stream_t stream) {
  (void)out_particle_F; (void)out_grid_mv; (void)out_grid_m;
  if (dim < 0 || !grid_ok(grid_dim)) return DEXMPM_ERR_ARG;
  if (dim == 0) return DEXMPM_OK;
  Grid g{grid_dim[0], grid_dim[1], grid_dim[2]};
  k_p2g_grad<<<blocks_for(dim), kThreads, 0, (cudaStream_t)stream>>>(
      particle_x, particle_v, particle_m, particle_vol, particle_F, particle_U, particle_sig, particle_V, particle_C,
      particle_mu_lam_yield, grid_lower, g, dx, inv_dx, dt, particle_x_grad, particle_v_grad, particle_F_grad,
      particle_C_grad, particle_U_grad, particle_sig_grad, particle_V_grad, out_particle_F_grad, out_grid_v_grad,
      out_grid_m_grad, dim);
  return launched();
}

int grid_op_v2(float *grid_m, float *grid_v_in, float *grid_body_v_in, int *grid_lower, float *gravity,
               float *body_pos, float *body_rot, float *next_body_pos, float *next_body_rot,
               float *body_type_friction_softness_round, float *body_args, float dx, float inv_dx, float dt,
               float ground_friction, float *out_grid_v, const int *grid_dim, int n_bodies,
               dexmpm_stream_t stream) {
  (void)inv_dx;
  if (!grid_ok(grid_dim) || n_bodies < 0) return DEXMPM_ERR_ARG;
  Grid g{grid_dim[0], grid_dim[1], grid_dim[2]};
  long dim = (long)g.x * g.y * g.z;
  k_grid_op<<<blocks_for(dim), kThreads, 0, (cudaStream_t)stream>>>(
      grid_m, grid_v_in, grid_body_v_in, grid_lower, gravity, body_pos, body_rot, next_body_pos, next_body_rot,
      body_type_friction_softness_round, body_args, dx, dt, ground_friction, out_grid_v, g, n_bodies, dim);
  return launched();
}

int grid_op_v2_grad(float *grid_m, float *grid_v_in, float *grid_body_v_in, int *grid_lower, float *gravity,
                    float *body_pos, float *body_rot, float *next_body_pos, float *next_body_rot,
                    float *body_type_friction_softness_round, float *body_args, float *grid_m_grad,
                    float *grid_v_in_grad, float *body_pos_grad, float *body_rot_grad, float *next_body_pos_grad,
                    float *next_body_rot_grad, float dx, float inv_dx, float dt, float ground_friction,
                    float *out_grid_v, float *out_grid_v_grad, const int *grid_dim, int n_bodies,
                    dexmpm_stream_t stream) {
  (void)inv_dx; (void)gravity; (void)out_grid_v;
  if (!grid_ok(grid_dim) || n_bodies < 0) return DEXMPM_ERR_ARG;
  Grid g{grid_dim[0], grid_dim[1], grid_dim[2]};
  long dim = (long)g.x * g.y * g.z;
  k_grid_op_grad<<<blocks_for(dim), kThreads, 0, (cudaStream_t)stream>>>(
      grid_m, grid_v_in, grid_body_v_in, grid_lower, body_pos, body_rot, next_body_pos, next_body_rot,
      body_type_friction_softness_round, body_args, grid_m_grad, grid_v_in_grad, body_pos_grad, body_rot_grad,
      next_body_pos_grad, next_body_rot_grad, dx, dt, ground_friction, out_grid_v_grad, g, n_bodies, dim);
  return launched();
}

int g2p(float *particle_x, float *grid_v, int *grid_lower, float dx, float inv_dx, float dt, const int *grid_dim,
        float *out_particle_v, float ground_height, float *out_particle_C, float *out_particle_x, int dim,
        dexmpm_stream_t stream) {
  if (dim < 0 || !grid_ok(grid_dim)) return DEXMPM_ERR_ARG;
  if (dim == 0) return DEXMPM_OK;
  Grid g{grid_dim[0], grid_dim[1], grid_dim[2]};
  k_g2p<<<blocks_for(dim), kThreads, 0, (cudaStream_t)stream>>>(particle_x, grid_v, grid_lower, dx, inv_dx, dt, g,
                                                                 out_particle_v, ground_height, out_particle_C,
                                                                 out_particle_x, dim);
  return launched();
}

int g2p_grad(float *particle_x, float *grid_v, int *grid_lower, float dx, float inv_dx, float dt,
             const int *grid_dim, float *out_particle_v, float ground_height, float *out_particle_C,
             float *out_particle_x, int dim, float *particle_x_grad, float *grid_v_grad,
             float *out_particle_v_grad, float *out_particle_C_grad, float *out_particle_x_grad,
             dexmpm_stream_t stream) {
  (void)out_particle_C; (void)out_particle_x;
  if (dim < 0 || !grid_ok(grid_dim)) return DEXMPM_ERR_ARG;
  if (dim == 0) return DEXMPM_OK;
  Grid g{grid_dim[0], grid_dim[1], grid_dim[2]};
  k_g2p_grad<<<blocks_for(dim), kThreads, 0, (cudaStream_t)stream>>>(
      particle_x, grid_v, grid_lower, dx, inv_dx, dt, g, out_particle_v, ground_height, particle_x_grad, grid_v_grad,
      out_particle_v_grad, out_particle_C_grad, out_particle_x_grad, dim);
  return launched();
}

int compute_dist(float *particle_x, float *body_pos, float *body_rot, float *body_type_friction_softness_round,
                 float *body_args, float *dist, int n_bodies, float *particle_x_grad, float *body_pos_grad,
                 float *body_rot_grad, float *dist_grad, int compute_grad, int dim, dexmpm_stream_t stream) {
  if (dim < 0 || n_bodies < 0) return DEXMPM_ERR_ARG;
  if (dim == 0 || n_bodies == 0) return DEXMPM_OK;
  k_compute_dist<<<blocks_for(dim), kThreads, 0, (cudaStream_t)stream>>>(
      particle_x, body_pos, body_rot, body_type_friction_softness_round, body_args, dist, n_bodies, particle_x_grad,
      body_pos_grad, body_rot_grad, dist_grad, compute_grad, dim);
  return launched();
}

int particle2mass(float *particle_x, float *particle_m, int *grid_lower, const int *grid_dim, float dx,
                  float inv_dx, float *out_grid_m, float *out_grid_m_grad, float *particle_x_grad,
                  int *particle_ids, int id, int compute_grad, int dim, dexmpm_stream_t stream) {
  if (dim < 0 || !grid_ok(grid_dim)) return DEXMPM_ERR_ARG;
  if (dim == 0) return DEXMPM_OK;
  Grid g{grid_dim[0], grid_dim[1], grid_dim[2]};
  k_particle2mass<<<blocks_for(dim), kThreads, 0, (cudaStream_t)stream>>>(
      particle_x, particle_m, grid_lower, g, dx, inv_dx, out_grid_m, out_grid_m_grad, particle_x_grad, particle_ids,
      id, compute_grad, dim);
  return launched();
}

int dexmpm_abi_get_error(int32_t *out) {
  if (!out) return DEXMPM_ERR_ARG;
  int32_t zero = 0;
  if (cudaMemcpyFromSymbol(out, g_abi_error, sizeof(int32_t)) != cudaSuccess) return DEXMPM_ERR_LAUNCH;
  if (cudaMemcpyToSymbol(g_abi_error, &zero, sizeof(int32_t)) != cudaSuccess) return DEXMPM_ERR_LAUNCH;
  return DEXMPM_OK;
}

}  // extern "C"
