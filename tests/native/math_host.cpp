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
}
