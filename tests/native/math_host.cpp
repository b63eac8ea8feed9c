// Host build of the product's FP32 arithmetic (dexdeform_gb300/csrc/mpm_math.cuh)
// so the CPU test suite can check it against the FP64 oracle without a GPU.
#include "../../dexdeform_gb300/csrc/mpm_math.cuh"
using namespace dexmpm;

static m33 load9(const float *p) { m33 m; for (int i = 0; i < 9; ++i) m.a[i / 3][i % 3] = p[i]; return m; }
static void store9(float *p, const m33 &m) { for (int i = 0; i < 9; ++i) p[i] = m.a[i / 3][i % 3]; }

extern "C" {
// F_tmp = (I + dt C) F ; SVD of F_tmp ; outputs U, sig, d = sig - 1, V and F_tmp.
void host_svd(int n, const float *F, const float *C, float dt, float *U, float *sig, float *d, float *V, float *Ftmp) {
  for (int p = 0; p < n; ++p) {
    m33 Fm = load9(F + 9 * p), Cm = load9(C + 9 * p);
    m33 E = deviation_tmp(Fm, Cm, dt);
    SVD3 s = svd3_from_deviation(E);
    store9(U + 9 * p, s.U);
    store9(V + 9 * p, s.V);
    sig[3 * p] = s.s.x; sig[3 * p + 1] = s.s.y; sig[3 * p + 2] = s.s.z;
    d[3 * p] = s.d.x; d[3 * p + 1] = s.d.y; d[3 * p + 2] = s.d.z;
    m33 Ft = E; Ft.a[0][0] += 1.f; Ft.a[1][1] += 1.f; Ft.a[2][2] += 1.f;
    store9(Ftmp + 9 * p, Ft);
  }
}
// projected F and stress P (before the -dt vol 4 inv_dx^2 scale)
void host_constitutive(int n, const float *F, const float *C, float dt, const float *mly, float *newF, float *P, float *J) {
  for (int p = 0; p < n; ++p) {
    m33 E = deviation_tmp(load9(F + 9 * p), load9(C + 9 * p), dt);
    SVD3 s = svd3_from_deviation(E);
    m33 Ft = E; Ft.a[0][0] += 1.f; Ft.a[1][1] += 1.f; Ft.a[2][2] += 1.f;
    Plastic o = constitutive(s, Ft, mly[3 * p], mly[3 * p + 1], mly[3 * p + 2]);
    store9(newF + 9 * p, o.newF);
    store9(P + 9 * p, o.P);
    J[p] = o.J;
  }
}
// dL/dF_tmp of the return mapping and stress from dL/dP (gP) and dL/dnewF (gF),
// with the product's SVD and constitutive intermediates of F_tmp = (I + dt C) F;
// also returns F_tmp and the yield flag
void host_stress_backward(int n, const float *F, const float *C, float dt, const float *mly, const float *gP,
                          const float *gF, float *out, float *Ftmp, int *yielded) {
  for (int p = 0; p < n; ++p) {
    m33 E = deviation_tmp(load9(F + 9 * p), load9(C + 9 * p), dt);
    SVD3 s = svd3_from_deviation(E);
    m33 Ft = E; Ft.a[0][0] += 1.f; Ft.a[1][1] += 1.f; Ft.a[2][2] += 1.f;
    Plastic o = constitutive(s, Ft, mly[3 * p], mly[3 * p + 1], mly[3 * p + 2]);
    store9(out + 9 * p, plastic_stress_backward(s, o, load9(gP + 9 * p), load9(gF + 9 * p), mly[3 * p],
                                                mly[3 * p + 1], mly[3 * p + 2]));
    store9(Ftmp + 9 * p, Ft);
    yielded[p] = o.yielded ? 1 : 0;
  }
}
// the return mapping's logarithm-free elastic test for sigma - 1 = d
void host_surely_elastic(int n, const float *d, float mu, const float *ys, int *out) {
  for (int p = 0; p < n; ++p)
    out[p] = surely_elastic(mk3(d[3 * p], d[3 * p + 1], d[3 * p + 2]), mu, ys[p]) ? 1 : 0;
}
// gradient of F_tmp from gradients of (U, sigma, V) for given SVDs (U, sig, d, V)
void host_svd_backward(int n, const float *U, const float *sig, const float *d, const float *V, const float *gU,
                       const float *gs, const float *gV, const float *gdirect, float *out) {
  for (int p = 0; p < n; ++p) {
    SVD3 sv;
    sv.U = load9(U + 9 * p);
    sv.V = load9(V + 9 * p);
    sv.s = mk3(sig[3 * p], sig[3 * p + 1], sig[3 * p + 2]);
    sv.d = mk3(d[3 * p], d[3 * p + 1], d[3 * p + 2]);
    store9(out + 9 * p, svd_backward(sv, load9(gU + 9 * p), mk3(gs[3 * p], gs[3 * p + 1], gs[3 * p + 2]),
                                     load9(gV + 9 * p), load9(gdirect + 9 * p)));
  }
}
}

// Serial host emulation of one forward substep with the product's FP32
// arithmetic on a dense x-major grid (the schedule of mpm/simulator.py:561-571),
// for CPU-side numerical checks against the FP64 oracle.  Body arrays:
// pose [nb][8] (p xyz 0 q wxyz), shapes [nb][8] (tfsr, args).
#include <vector>
extern "C" void host_substep(int n, const float *x, const float *v, const float *F, const float *C, const float *mass,
                             const float *vol, const float *mly, int gx, int gy, int gz, float dx, float dt,
                             const float *gravity, float gf, int nb, const float *pose, const float *npose,
                             const float *shapes, float *ox, float *ov, float *oF, float *oC) {
  const float inv_dx = 1.f / dx;
  std::vector<float> gm((size_t)gx * gy * gz, 0.f), gmv((size_t)gx * gy * gz * 3, 0.f), gv((size_t)gx * gy * gz * 3, 0.f);
  auto idx = [&](int a, int b, int c) { return ((size_t)a * gy + b) * gz + c; };
  for (int p = 0; p < n; ++p) {
    m33 Fm = load9(F + 9 * p), Cm = load9(C + 9 * p);
    m33 E = deviation_tmp(Fm, Cm, dt);
    SVD3 s = svd3_from_deviation(E);
    m33 Ft = E; Ft.a[0][0] += 1.f; Ft.a[1][1] += 1.f; Ft.a[2][2] += 1.f;
    Plastic pl = constitutive(s, Ft, mly[3 * p], mly[3 * p + 1], mly[3 * p + 2]);
    store9(oF + 9 * p, pl.newF);
    m33 A = pl.P * (-dt * vol[p] * 4.f * inv_dx * inv_dx) + Cm * mass[p];
    f3 mom = mk3(v[3 * p], v[3 * p + 1], v[3 * p + 2]) * mass[p];
    Stencil st;
    make_stencil(mk3(x[3 * p], x[3 * p + 1], x[3 * p + 2]), inv_dx, st);
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) for (int k = 0; k < 3; ++k) {
      float w = st.w[0][i] * st.w[1][j] * st.w[2][k];
      f3 dpos = mk3((i - st.fx[0]) * dx, (j - st.fx[1]) * dx, (k - st.fx[2]) * dx);
      size_t id = idx(st.base[0] + i, st.base[1] + j, st.base[2] + k);
      f3 c = (mom + mv(A, dpos)) * w;
      gm[id] += mass[p] * w; gmv[3 * id] += c.x; gmv[3 * id + 1] += c.y; gmv[3 * id + 2] += c.z;
    }
  }
  for (int a = 0; a < gx; ++a) for (int b = 0; b < gy; ++b) for (int c = 0; c < gz; ++c) {
    size_t id = idx(a, b, c);
    if (!(gm[id] > kMassEps)) continue;
    float im = 1.f / gm[id];
    f3 vv = mk3(gmv[3 * id] * im, gmv[3 * id + 1] * im, gmv[3 * id + 2] * im) + mk3(gravity[0], gravity[1], gravity[2]) * dt;
    f3 gxw = mk3(a * dx, b * dx, c * dx);
    for (int bb = 0; bb < nb; ++bb) {
      BodyPose cur, nxt; BodyShape sh;
      cur.p = mk3(pose[8 * bb], pose[8 * bb + 1], pose[8 * bb + 2]); cur.q = mkq(pose[8 * bb + 4], pose[8 * bb + 5], pose[8 * bb + 6], pose[8 * bb + 7]);
      nxt.p = mk3(npose[8 * bb], npose[8 * bb + 1], npose[8 * bb + 2]); nxt.q = mkq(npose[8 * bb + 4], npose[8 * bb + 5], npose[8 * bb + 6], npose[8 * bb + 7]);
      sh.tfsr = mkq(shapes[8 * bb], shapes[8 * bb + 1], shapes[8 * bb + 2], shapes[8 * bb + 3]);
      sh.args = mkq(shapes[8 * bb + 4], shapes[8 * bb + 5], shapes[8 * bb + 6], shapes[8 * bb + 7]);
      contact_forward(gxw, vv, cur, nxt, sh, dt);
    }
    vv = boundary_forward(vv, a, b, c, gx, gy, gz, gf);
    gv[3 * id] = vv.x; gv[3 * id + 1] = vv.y; gv[3 * id + 2] = vv.z;
  }
  for (int p = 0; p < n; ++p) {
    Stencil st;
    f3 xp = mk3(x[3 * p], x[3 * p + 1], x[3 * p + 2]);
    make_stencil(xp, inv_dx, st);
    f3 nv = mk3(0.f, 0.f, 0.f); m33 nC = mzero();
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) for (int k = 0; k < 3; ++k) {
      float w = st.w[0][i] * st.w[1][j] * st.w[2][k];
      size_t id = idx(st.base[0] + i, st.base[1] + j, st.base[2] + k);
      f3 g = mk3(gv[3 * id], gv[3 * id + 1], gv[3 * id + 2]);
      nv += g * w;
      nC += outer(g, mk3(i - st.fx[0], j - st.fx[1], k - st.fx[2])) * (w * 4.f * inv_dx);
    }
    f3 nx = xp + nv * dt;
    nx.x = fmaxf(fminf(nx.x, (gx - 3.f) * dx), 3.f * dx);
    nx.y = fmaxf(fminf(nx.y, (gy - 3.f) * dx), 3.f * dx);
    nx.z = fmaxf(fminf(nx.z, (gz - 3.f) * dx), 3.f * dx);
    ox[3 * p] = nx.x; ox[3 * p + 1] = nx.y; ox[3 * p + 2] = nx.z;
    ov[3 * p] = nv.x; ov[3 * p + 1] = nv.y; ov[3 * p + 2] = nv.z;
    store9(oC + 9 * p, nC);
  }
}

// Block culling check: for case c, a body (pose [8], shape [8]) and a 4^3
// block with origin cell blk[3c..3c+2].  may[c] = the block test's answer;
// touched[c] = 1 if contact_forward's activation holds at any of the 64 cells.
extern "C" void host_block_cull(int n, const float *pose, const float *shapes, const int *blk, float dx, int *may,
                                int *touched) {
  for (int c = 0; c < n; ++c) {
    BodyPose cur;
    cur.p = mk3(pose[8 * c], pose[8 * c + 1], pose[8 * c + 2]);
    cur.q = mkq(pose[8 * c + 4], pose[8 * c + 5], pose[8 * c + 6], pose[8 * c + 7]);
    BodyShape sh;
    sh.tfsr = mkq(shapes[8 * c], shapes[8 * c + 1], shapes[8 * c + 2], shapes[8 * c + 3]);
    sh.args = mkq(shapes[8 * c + 4], shapes[8 * c + 5], shapes[8 * c + 6], shapes[8 * c + 7]);
    const int bx = blk[3 * c], by = blk[3 * c + 1], bz = blk[3 * c + 2];
    f3 centre = mk3((bx + 1.5f) * dx, (by + 1.5f) * dx, (bz + 1.5f) * dx);
    may[c] = body_may_touch(centre, 2.6f * dx, cur, sh) ? 1 : 0;
    int t = 0;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 4; ++k) {
          f3 g = mk3((bx + i) * dx, (by + j) * dx, (bz + k) * dx);
          float dist = shape_sdf(sh.tfsr, sh.args, xform_inv(cur.p, cur.q, g));
          float infl = fminf(expf(-dist * sh.tfsr.y), 1.f);
          if ((sh.tfsr.y > 0.f && infl > 0.1f) || dist <= 0.f) t = 1;
        }
    touched[c] = t;
  }
}
