// mpm_math.cuh -- FP32 per-particle / per-node arithmetic of the MLS-MPM substep.
//
// Header-only; compiles as CUDA device code (the product) and as plain host C++
// (the CPU unit tests of the arithmetic).  Conventions follow the DexDeform
// reference (mpm/csrc): mat3 row-major, quaternions (w,x,y,z), quadratic
// B-spline stencil with base = floor(x/dx - 0.5).
//
// Numerics.  The reference stores F, U, V in FP32 and forms the deviatoric
// stress as 2*mu*(F - U V^T) F^T (integrator.cu:364-369).  Near a rest state
// F - U V^T is a difference of nearly equal FP32 numbers; it carries ~1e-7
// absolute noise, which after one substep from rest shows up as a 1e-4
// relative velocity error even in the reference itself.  Here the SVD works on
// E = F - I (formed exactly from the stored F), its eigen-analysis runs on
// S = F^T F - I = E + E^T + E^T E, and sigma - 1 is taken from the eigenvalues
// of S, so
//     (F - U V^T) F^T = U diag(sigma (sigma - 1)) U^T,
//     J - 1 = prod(1 + d_i) - 1,   log(sigma) = log1p(sigma - 1)
// keep full relative precision in the strain.  These are algebraic identities
// of the reference's formulas, not a different model.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define DX_HD __host__ __device__ __forceinline__
#else
#define DX_HD inline
#endif

namespace dexmpm {

constexpr float kNormEps = 1e-8f;     // integrator.cu:11
constexpr float kSigClip = 0.05f;     // integrator.cu:12
constexpr float kLenEps = 1e-30f;     // shape.h:4
constexpr float kMassEps = 1e-12f;    // integrator.cu:671
constexpr int kBound = 3;             // integrator.cu:735

// ------------------------------------------------------------------ vec3
struct f3 {
  float x, y, z;
};
DX_HD f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
DX_HD f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
DX_HD f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
DX_HD f3 operator-(f3 a) { return mk3(-a.x, -a.y, -a.z); }
DX_HD f3 operator*(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
DX_HD f3 operator*(float s, f3 a) { return mk3(a.x * s, a.y * s, a.z * s); }
DX_HD f3 hadamard(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
DX_HD f3 &operator+=(f3 &a, f3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
DX_HD f3 &operator-=(f3 &a, f3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
DX_HD float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DX_HD f3 cross(f3 a, f3 b) { return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
DX_HD float comp(f3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// ------------------------------------------------------------------ mat3
struct m33 {
  float a[3][3];
};
DX_HD m33 mzero() { m33 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.a[i][j] = 0.f; return r; }
DX_HD m33 meye() { m33 r = mzero(); r.a[0][0] = r.a[1][1] = r.a[2][2] = 1.f; return r; }
DX_HD m33 mdiag(f3 d) { m33 r = mzero(); r.a[0][0] = d.x; r.a[1][1] = d.y; r.a[2][2] = d.z; return r; }
DX_HD m33 mT(const m33 &m) { m33 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.a[i][j] = m.a[j][i]; return r; }
DX_HD m33 operator+(const m33 &x, const m33 &y) { m33 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][j] + y.a[i][j]; return r; }
DX_HD m33 operator-(const m33 &x, const m33 &y) { m33 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][j] - y.a[i][j]; return r; }
DX_HD m33 operator*(const m33 &x, float s) { m33 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][j] * s; return r; }
DX_HD m33 operator*(float s, const m33 &x) { return x * s; }
DX_HD m33 &operator+=(m33 &x, const m33 &y) { for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) x.a[i][j] += y.a[i][j]; return x; }
DX_HD m33 hadamard(const m33 &x, const m33 &y) { m33 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][j] * y.a[i][j]; return r; }
DX_HD m33 mm(const m33 &x, const m33 &y) {
  m33 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][0] * y.a[0][j] + x.a[i][1] * y.a[1][j] + x.a[i][2] * y.a[2][j];
  return r;
}
DX_HD f3 mv(const m33 &m, f3 b) {
  return mk3(m.a[0][0] * b.x + m.a[0][1] * b.y + m.a[0][2] * b.z, m.a[1][0] * b.x + m.a[1][1] * b.y + m.a[1][2] * b.z,
             m.a[2][0] * b.x + m.a[2][1] * b.y + m.a[2][2] * b.z);
}
// m^T b
DX_HD f3 mtv(const m33 &m, f3 b) {
  return mk3(m.a[0][0] * b.x + m.a[1][0] * b.y + m.a[2][0] * b.z, m.a[0][1] * b.x + m.a[1][1] * b.y + m.a[2][1] * b.z,
             m.a[0][2] * b.x + m.a[1][2] * b.y + m.a[2][2] * b.z);
}
DX_HD m33 outer(f3 a, f3 b) {
  m33 r;
  r.a[0][0] = a.x * b.x; r.a[0][1] = a.x * b.y; r.a[0][2] = a.x * b.z;
  r.a[1][0] = a.y * b.x; r.a[1][1] = a.y * b.y; r.a[1][2] = a.y * b.z;
  r.a[2][0] = a.z * b.x; r.a[2][1] = a.z * b.y; r.a[2][2] = a.z * b.z;
  return r;
}
DX_HD float msum(const m33 &m) { float s = 0.f; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) s += m.a[i][j]; return s; }
DX_HD float trace(const m33 &m) { return m.a[0][0] + m.a[1][1] + m.a[2][2]; }
// U diag(d) U^T
DX_HD m33 sym_from_eig(const m33 &U, f3 d) {
  m33 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = U.a[i][0] * d.x * U.a[j][0] + U.a[i][1] * d.y * U.a[j][1] + U.a[i][2] * d.z * U.a[j][2];
  return r;
}
// U diag(d) V^T
DX_HD m33 usv(const m33 &U, f3 d, const m33 &V) {
  m33 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = U.a[i][0] * d.x * V.a[j][0] + U.a[i][1] * d.y * V.a[j][1] + U.a[i][2] * d.z * V.a[j][2];
  return r;
}

// ------------------------------------------------------------------ quat
struct qf {
  float w, x, y, z;
};
DX_HD qf mkq(float w, float x, float y, float z) { qf q; q.w = w; q.x = x; q.y = y; q.z = z; return q; }
DX_HD qf qinv(qf q) { return mkq(q.w, -q.x, -q.y, -q.z); }
// q * v (quat.h:14-19)
DX_HD f3 qrot(qf q, f3 v) {
  f3 qv = mk3(q.x, q.y, q.z);
  f3 uv = cross(qv, v), uuv = cross(qv, uv);
  return v + 2.f * (q.w * uv + uuv);
}
// q*v - v: the rotation increment, without forming v + (small) and
// subtracting v again
DX_HD f3 qrot_delta(qf q, f3 v) {
  f3 qv = mk3(q.x, q.y, q.z);
  f3 uv = cross(qv, v), uuv = cross(qv, uv);
  return 2.f * (q.w * uv + uuv);
}
DX_HD f3 xform(f3 p, qf q, f3 pt) { return p + qrot(q, pt); }            // quat.h:89-92
DX_HD f3 xform_inv(f3 p, qf q, f3 pt) { return qrot(qinv(q), pt - p); }  // quat.h:94-97
// adjoint of q*v (quat.h:25-49)
DX_HD void qrot_backward(qf q, f3 v, f3 gout, qf &gq, f3 &gv) {
  f3 qv = mk3(q.x, q.y, q.z);
  f3 uv = cross(qv, v);
  gq.w += dot(uv, gout) * 2.f;
  f3 g_uv = (2.f * q.w) * gout;
  f3 g_uuv = 2.f * gout;
  f3 g_qv = cross(uv, g_uuv);
  g_uv += cross(g_uuv, qv);
  g_qv += cross(v, g_uv);
  gv += gout + cross(g_uv, qv);
  gq.x += g_qv.x; gq.y += g_qv.y; gq.z += g_qv.z;
}
// quat.h:52-63
DX_HD void xform_backward(qf q, f3 pt, f3 gout, f3 &gp, qf &gq, f3 &gpt) {
  gp += gout;
  qrot_backward(q, pt, gout, gq, gpt);
}
// quat.h:65-80
DX_HD void xform_inv_backward(f3 p, qf q, f3 pt, f3 gout, f3 &gp, qf &gq, f3 &gpt) {
  qf tq = mkq(0.f, 0.f, 0.f, 0.f);
  f3 tp = mk3(0.f, 0.f, 0.f);
  qrot_backward(qinv(q), pt - p, gout, tq, tp);
  gq.w += tq.w; gq.x -= tq.x; gq.y -= tq.y; gq.z -= tq.z;
  gp -= tp;
  gpt += tp;
}

// ------------------------------------------------------------- shapes
DX_HD float vlength(f3 a) { return sqrtf(dot(a, a) + kLenEps); }      // shape.h:7-9
DX_HD f3 vnormalized(f3 a) { return a * (1.f / vlength(a)); }       // shape.h:13-15
DX_HD f3 vnormalized_backward(f3 a, f3 g) {                         // shape.h:17-25
  float d = dot(a, a) + kLenEps;
  return (g - a * dot(a * (1.f / d), g)) * (1.f / sqrtf(d));
}
DX_HD int shape_type(qf tfsr) { return (int)floorf(tfsr.w + 0.1f); }  // shape.h:33-35
DX_HD f3 fabs3(f3 a) { return mk3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
DX_HD f3 fmax3(f3 a, float b) { return mk3(fmaxf(a.x, b), fmaxf(a.y, b), fmaxf(a.z, b)); }
DX_HD void abs_backward(f3 g, f3 &gr) {                              // shape.h:27-31
  if (g.x < 0) gr.x = -gr.x;
  if (g.y < 0) gr.y = -gr.y;
  if (g.z < 0) gr.z = -gr.z;
}

// Box (type 0, half extents args.w,x,y) or capsule (type 1, radius args.w, full
// length args.x along y) minus the rounding radius tfsr.z (shape.h:37-61).  Other
// type codes give distance 0 - round (the reference prints an error there).
DX_HD float shape_sdf(qf tfsr, qf args, f3 g) {
  int type = shape_type(tfsr);
  float sdf = 0.f;
  if (type == 0) {
    f3 q = fabs3(g) - mk3(args.w, args.x, args.y);
    sdf = vlength(fmax3(q, 0.f)) + fminf(fmaxf(fmaxf(q.x, q.y), q.z), 0.f);
  } else if (type == 1) {
    float h = args.x;
    f3 p2 = g;
    p2.y += h * 0.5f;
    p2.y -= fminf(fmaxf(p2.y, 0.f), h);
    sdf = vlength(p2) - args.w;
  }
  return sdf - tfsr.z;
}
// shape.h:65-102 (unnormalised outward direction)
DX_HD f3 shape_grad(qf tfsr, qf args, f3 g) {
  int type = shape_type(tfsr);
  f3 grad = mk3(0.f, 0.f, 0.f);
  if (type == 0) {
    f3 q = fabs3(g) - mk3(args.w, args.x, args.y);
    float inside = fmaxf(fmaxf(q.x, q.y), q.z);
    if (inside <= 0) {
      if (q.x == inside) grad.x += 1.f;
      if (q.y == inside) grad.y += 1.f;
      if (q.z == inside) grad.z += 1.f;
    } else {
      grad = vnormalized(fmax3(q, 0.f));
    }
    abs_backward(g, grad);
  } else if (type == 1) {
    float h = args.x;
    f3 p2 = g;
    p2.y += h * 0.5f;
    p2.y -= fminf(fmaxf(p2.y, 0.f), h);
    return vnormalized(p2);
  }
  return grad;
}
// shape.h:104-152.  The reference's capsule branch back-propagates its own
// zero-initialised accumulator instead of grad_out, so it always returns 0
// (the capsule-normal term of the pose gradient is dropped); that behaviour is
// the default, for gradient parity.  exact_capsule = true gives the true
// derivative of normalized(p2(g)) instead, where p2.y does not depend on g.y
// inside the segment span.
DX_HD f3 shape_grad_backward(qf tfsr, qf args, f3 g, f3 gout, bool exact_capsule = false) {
  int type = shape_type(tfsr);
  f3 gin = mk3(0.f, 0.f, 0.f);
  if (type == 0) {
    f3 q = fabs3(g) - mk3(args.w, args.x, args.y);
    float inside = fmaxf(fmaxf(q.x, q.y), q.z);
    gin = gout;
    abs_backward(g, gin);
    if (inside <= 0) {
      gin = mk3(0.f, 0.f, 0.f);
    } else {
      gin = vnormalized_backward(fmax3(q, 0.f), gin);
      if (q.x < 0) gin.x = 0.f;
      if (q.y < 0) gin.y = 0.f;
      if (q.z < 0) gin.z = 0.f;
      abs_backward(g, gin);
    }
  } else if (type == 1 && exact_capsule) {
    float h = args.x;
    f3 p2 = g;
    p2.y += h * 0.5f;
    bool inside = p2.y >= 0.f && p2.y <= h;
    p2.y -= fminf(fmaxf(p2.y, 0.f), h);
    gin = vnormalized_backward(p2, gout);
    if (inside) gin.y = 0.f;
  }
  return gin;
}

// ------------------------------------------------------------- stencil
// Quadratic B-spline weights and their x-derivatives (integrator.cu:348-352,
// 492-493); w[axis][node], dpos in cell units = node - fx.
struct Stencil {
  int base[3];
  float fx[3];
  float w[3][3];
};
DX_HD void make_stencil(f3 x, float inv_dx, Stencil &s) {
  float xs[3] = {x.x * inv_dx, x.y * inv_dx, x.z * inv_dx};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int b = (int)floorf(xs[d] - 0.5f);
    float f = xs[d] - (float)b;
    s.base[d] = b;
    s.fx[d] = f;
    s.w[d][0] = 0.5f * (1.5f - f) * (1.5f - f);
    s.w[d][1] = 0.75f - (f - 1.f) * (f - 1.f);
    s.w[d][2] = 0.5f * (f - 0.5f) * (f - 0.5f);
  }
}
DX_HD void make_dweights(const Stencil &s, float inv_dx, float w1[3][3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float f = s.fx[d];
    w1[d][0] = -inv_dx * (1.5f - f);
    w1[d][1] = inv_dx * (-2.f * f + 2.f);
    w1[d][2] = -inv_dx * (-f + 0.5f);
  }
}

// ------------------------------------------------------------------ SVD
// A = U diag(sig) V^T for A = I + E, with U, V proper rotations, |sig| sorted
// descending and the sign of det(A) carried by sig.z (the conventions of the
// reference's svd3, mpm/csrc/svd.h).  d = sig - 1 computed without
// cancellation.  Algorithm: cyclic Jacobi with exact rotation angles on the
// symmetric S = A^T A - I (Golub & Van Loan, "Matrix Computations", sec. 8.5),
// column sort with sign-preserving swaps, then Givens QR of B = A V.
struct SVD3 {
  m33 U, V;
  f3 s, d;
};

// Reciprocal square root and division for rotation parameters, where a few
// ulp of error only perturb an angle: the hardware approximations on the GPU
// (callers keep the arguments finite and away from denormals), exact on the host.
DX_HD float rot_rsqrt(float x) {
#ifdef __CUDA_ARCH__
  return rsqrtf(x);
#else
  return 1.f / sqrtf(x);
#endif
}
DX_HD float rot_div(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}

// One Jacobi rotation zeroing S[p][q].  Skipped when the pivot is below FP32
// resolution of the diagonal pair (a rotation could change the eigenvalues by
// at most that, relative) or below 1e-30 in absolute terms.  The tangent is
// t = sgn(theta) / (|theta| + sqrt(theta^2 + 1)), theta = (S_qq - S_pp) / (2 S_pq),
// with |theta| capped at 1e18 (t below 5e-19 is no rotation at FP32).
DX_HD void jacobi_rotate(float S[3][3], m33 &V, int p, int q, int r) {
  float apq = S[p][q];
  const float app = S[p][p], aqq = S[q][q];
  if (!(fabsf(apq) > fmaxf(5.9604645e-8f * fmaxf(fabsf(app), fabsf(aqq)), 1e-30f))) return;
  float theta = rot_div(aqq - app, 2.f * apq);
  const float at = fminf(fabsf(theta), 1e18f);
  const float sq = at * at + 1.f;
  float t = rot_div(1.f, at + sq * rot_rsqrt(sq));
  t = theta < 0.f ? -t : t;
  float c = rot_rsqrt(t * t + 1.f), s = t * c;
  S[p][p] -= t * apq;
  S[q][q] += t * apq;
  S[p][q] = S[q][p] = 0.f;
  float arp = S[r][p], arq = S[r][q];
  S[r][p] = S[p][r] = c * arp - s * arq;
  S[r][q] = S[q][r] = s * arp + c * arq;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float vp = V.a[k][p], vq = V.a[k][q];
    V.a[k][p] = c * vp - s * vq;
    V.a[k][q] = s * vp + c * vq;
  }
}

// Whether every pivot of S is below jacobi_rotate's skip threshold: then a
// sweep leaves S and V as they are, and so do all later sweeps.
DX_HD bool jacobi_settled(const float S[3][3]) {
  auto below = [&](int p, int q) {
    return !(fabsf(S[p][q]) > fmaxf(5.9604645e-8f * fmaxf(fabsf(S[p][p]), fabsf(S[q][q])), 1e-30f));
  };
  return below(0, 1) && below(0, 2) && below(1, 2);
}

DX_HD void swap_neg_cols(m33 &M, int i, int j) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float t = M.a[k][i];
    M.a[k][i] = M.a[k][j];
    M.a[k][j] = -t;
  }
}

// Givens rotation on rows (i, j) zeroing B[j][col]; U accumulates G^T.
DX_HD void qr_rotate(m33 &B, m33 &U, int i, int j, int col) {
  float a = B.a[i][col], b = B.a[j][col];
  const float r2 = a * a + b * b;
  if (!(r2 > 1e-36f)) return;
  const float ir = rot_rsqrt(r2);
  float c = a * ir, s = b * ir;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float bi = B.a[i][k], bj = B.a[j][k];
    B.a[i][k] = c * bi + s * bj;
    B.a[j][k] = -s * bi + c * bj;
    float ui = U.a[k][i], uj = U.a[k][j];
    U.a[k][i] = c * ui + s * uj;
    U.a[k][j] = -s * ui + c * uj;
  }
}

DX_HD float sig_minus_one(float lam) {
  float l = fmaxf(lam, -1.f);
  return rot_div(l, 1.f + sqrtf(1.f + l));
}

DX_HD SVD3 svd3_from_deviation(const m33 &E) {
  SVD3 o;
  // S = E + E^T + E^T E
  float S[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      float v = E.a[i][j] + E.a[j][i] + E.a[0][i] * E.a[0][j] + E.a[1][i] * E.a[1][j] + E.a[2][i] * E.a[2][j];
      S[i][j] = v;
      S[j][i] = v;
    }
  o.V = meye();
#ifndef DEX_JACOBI_SWEEPS
#define DEX_JACOBI_SWEEPS 4
#endif
  // a lane leaves the sweeps once they would no longer change anything (the
  // result is that of all DEX_JACOBI_SWEEPS); a warp runs them while any of
  // its lanes needs them
#pragma unroll 1
  for (int sweep = 0; sweep < DEX_JACOBI_SWEEPS; ++sweep) {
    if (jacobi_settled(S)) break;
    jacobi_rotate(S, o.V, 0, 1, 2);
    jacobi_rotate(S, o.V, 0, 2, 1);
    jacobi_rotate(S, o.V, 1, 2, 0);
  }
  float lam[3] = {S[0][0], S[1][1], S[2][2]};
  // descending order of sigma^2 - 1, swaps as in svd.h:212-246
  if (lam[0] < lam[1]) { float t = lam[0]; lam[0] = lam[1]; lam[1] = t; swap_neg_cols(o.V, 0, 1); }
  if (lam[0] < lam[2]) { float t = lam[0]; lam[0] = lam[2]; lam[2] = t; swap_neg_cols(o.V, 0, 2); }
  if (lam[1] < lam[2]) { float t = lam[1]; lam[1] = lam[2]; lam[2] = t; swap_neg_cols(o.V, 1, 2); }
  m33 A = E;
  A.a[0][0] += 1.f; A.a[1][1] += 1.f; A.a[2][2] += 1.f;
  m33 B = mm(A, o.V);
  o.U = meye();
  qr_rotate(B, o.U, 0, 1, 0);
  qr_rotate(B, o.U, 0, 2, 0);
  qr_rotate(B, o.U, 1, 2, 1);
  // Near sigma = 1 the eigenvalue of S gives sigma - 1 to full relative
  // precision; far from 1 (large stretch or compression) the QR diagonal is
  // the accurate one (eigenvalues of A^T A lose precision for small sigma).
  float dd[3], ss[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float r = B.a[i][i];
    if (r >= 0.f && fabsf(lam[i]) < 0.25f) {
      dd[i] = sig_minus_one(lam[i]);
      ss[i] = 1.f + dd[i];
    } else {
      ss[i] = r;
      dd[i] = r - 1.f;
    }
  }
  o.s = mk3(ss[0], ss[1], ss[2]);
  o.d = mk3(dd[0], dd[1], dd[2]);
  return o;
}

// SVD of F_tmp = (I + dt C) F, with E_tmp = (F - I) + dt C F kept exact.
DX_HD m33 deviation_tmp(const m33 &F, const m33 &C, float dt) {
  m33 CF = mm(C, F);
  m33 E;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) E.a[i][j] = (F.a[i][j] - (i == j ? 1.f : 0.f)) + dt * CF.a[i][j];
  return E;
}

// ---------------------------------------------------------- constitutive
// Von Mises return mapping (integrator.cu:42-67) plus the fixed-corotated
// stress of p2g (:364-371) before the -dt*vol*4*inv_dx^2 scale.
struct Plastic {
  m33 newF;     // projected deformation gradient
  m33 P;        // 2 mu (newF - R) newF^T + lam J (J-1) I
  float J;
  bool yielded;
  f3 eps_hat;   // deviatoric log strain and its norm (for the adjoint)
  float eps_hat_norm, delta_gamma;
  f3 expe;      // singular values of newF
  f3 dm1;       // expe - 1 without cancellation
};

// Whether the return mapping certainly leaves sigma inside the yield surface,
// decided without logarithms.  For |d| <= 1/2, log1p(d) = d - d^2/2 + t with
// |t| <= |d|^3 / (3 (1 - |d|)) <= (2/3) |d|^3, so the deviatoric log strain
// satisfies |eps_hat| <= |dev(d - d^2/2)| + (2/3) sqrt(sum d^6); true when that
// bound (with the norm's epsilon) is below the yield radius yield / (2 mu) by 0.1%.
DX_HD bool surely_elastic(f3 d, float mu, float yield) {
  if (!(fabsf(d.x) <= 0.5f && fabsf(d.y) <= 0.5f && fabsf(d.z) <= 0.5f)) return false;
  const f3 d2 = hadamard(d, d);
  const f3 q = d - d2 * 0.5f;
  const float m = (q.x + q.y + q.z) * (1.f / 3.f);
  const f3 qh = mk3(q.x - m, q.y - m, q.z - m);
  const f3 d3 = hadamard(d2, mk3(fabsf(d.x), fabsf(d.y), fabsf(d.z)));
  const float ub = sqrtf(dot(qh, qh)) + (2.f / 3.f) * sqrtf(dot(d3, d3));
  const float r = yield / (2.f * mu);
  return ub * ub + kNormEps < 0.999f * r * r;
}

DX_HD Plastic constitutive(const SVD3 &sv, const m33 &Ftmp, float mu, float lam, float yield) {
  Plastic o;
  // log strain e, its deviatoric part and norm; left at zero (not used) when
  // the state is surely elastic
  float e[3] = {0.f, 0.f, 0.f}, dg = -1.f, ehn = 1.f;
  f3 eh = mk3(0.f, 0.f, 0.f);
  if (!surely_elastic(sv.d, mu, yield)) {
    const float dv[3] = {sv.d.x, sv.d.y, sv.d.z}, sv_[3] = {sv.s.x, sv.s.y, sv.s.z};
#pragma unroll
    for (int i = 0; i < 3; ++i) e[i] = sv_[i] >= kSigClip ? log1pf(dv[i]) : logf(kSigClip);
    const float mean = (e[0] + e[1] + e[2]) * (1.f / 3.f);
    eh = mk3(e[0] - mean, e[1] - mean, e[2] - mean);
    ehn = sqrtf(dot(eh, eh) + kNormEps);
    dg = ehn - yield / (2.f * mu);
  }
  o.eps_hat = eh;
  o.eps_hat_norm = ehn;
  o.delta_gamma = dg;
  if (dg > 0.f) {
    float k = dg / ehn;
    float ep[3] = {e[0] - k * eh.x, e[1] - k * eh.y, e[2] - k * eh.z};
    f3 em1 = mk3(expm1f(ep[0]), expm1f(ep[1]), expm1f(ep[2]));
    f3 ee = mk3(1.f + em1.x, 1.f + em1.y, 1.f + em1.z);  // exp(ep), one rounding from expm1
    o.expe = ee;
    o.dm1 = em1;
    o.newF = usv(sv.U, ee, sv.V);
    o.J = ee.x * ee.y * ee.z;
    float Jm1 = expm1f(ep[0] + ep[1] + ep[2]);
    o.P = sym_from_eig(sv.U, hadamard(em1, ee)) * (2.f * mu);
    float iso = lam * o.J * Jm1;
    o.P.a[0][0] += iso; o.P.a[1][1] += iso; o.P.a[2][2] += iso;
    o.yielded = true;
  } else {
    o.expe = sv.s;
    o.dm1 = sv.d;
    o.newF = Ftmp;
    o.J = sv.s.x * sv.s.y * sv.s.z;
    f3 d = sv.d;
    float Jm1 = d.x + d.y + d.z + d.x * d.y + d.x * d.z + d.y * d.z + d.x * d.y * d.z;
    o.P = sym_from_eig(sv.U, hadamard(sv.s, d)) * (2.f * mu);
    float iso = lam * o.J * Jm1;
    o.P.a[0][0] += iso; o.P.a[1][1] += iso; o.P.a[2][2] += iso;
    o.yielded = false;
  }
  return o;
}

// ----------------------------------------------------------- grid node
struct BodyPose {
  f3 p;
  qf q;
};
struct BodyShape {
  qf tfsr;  // type, friction, softness, round
  qf args;
};

// Velocity of the body-frame point gxb = T_cur^-1(gx) carried by the body from
// pose cur to pose nxt: (T_nxt(gxb) - gx) / dt (integrator.cu:716).  Written as
//   (p1 - p0) + [Q1(u) - u] + [u - r],   r = gx - p0,  u = Q0^-1(r) = gxb,
// which is the same quantity without subtracting two positions of size ~1
// that differ by |v| dt (FP32 leaves ~3e-4 m/s of noise there at dt = 1e-4).
DX_HD f3 body_velocity(f3 gx, f3 gxb, const BodyPose &cur, const BodyPose &nxt, float dt) {
  f3 r = gx - cur.p;
  f3 disp = (nxt.p - cur.p) + qrot_delta(nxt.q, gxb) + qrot_delta(qinv(cur.q), r);
  return disp * (1.f / dt);
}

// One body contact on a grid node (integrator.cu:694-730).  Returns true when
// the body touched the node.
DX_HD bool contact_forward(f3 gx, f3 &v, const BodyPose &cur, const BodyPose &nxt, const BodyShape &sh, float dt) {
  float friction = sh.tfsr.x, softness = sh.tfsr.y;
  f3 gxb = xform_inv(cur.p, cur.q, gx);
  float dist = shape_sdf(sh.tfsr, sh.args, gxb);
  float infl = fminf(expf(-dist * softness), 1.f);
  if (!((softness > 0.f && infl > 0.1f) || dist <= 0.f)) return false;
  f3 nrm = qrot(cur.q, vnormalized(shape_grad(sh.tfsr, sh.args, gxb)));
  f3 bv = body_velocity(gx, gxb, cur, nxt, dt);
  f3 rel = v - bv;
  float nc = dot(rel, nrm);
  f3 vt = rel - nrm * fminf(nc, 0.f);
  if (nc < 0.f && dot(vt, vt) > 1e-30f) {
    float vtn = vlength(vt);
    vt = vt * ((1.f / vtn) * fmaxf(0.f, vtn + nc * friction));
  }
  v = bv + rel * (1.f - infl) + vt * infl;
  return true;
}

// Whether a body can touch any grid node within distance `reach` of `centre`.
// A contact changes a node's velocity only where its signed distance d
// satisfies d <= 0 or exp(-softness d) > 0.1, i.e. d < ln(10) / softness
// (integrator.cu:700-712).  The body-frame map x -> q^-1 (x - p) has operator
// norm at most |1 - |q|^2| + |q|^2 (1 for a unit quaternion) and the box and
// capsule distances are 1-Lipschitz, so a node whose distance exceeds the
// cutoff at the centre by more than norm x reach is untouched.  A margin of
// 0.1% + 1e-5 covers FP32 rounding; a NaN distance keeps the body.
DX_HD bool body_may_touch(f3 centre, float reach, const BodyPose &cur, const BodyShape &sh) {
  const float d = shape_sdf(sh.tfsr, sh.args, xform_inv(cur.p, cur.q, centre));
  const float qn = cur.q.w * cur.q.w + cur.q.x * cur.q.x + cur.q.y * cur.q.y + cur.q.z * cur.q.z;
  const float lip = fabsf(1.f - qn) + qn;
  const float soft = sh.tfsr.y;
  const float cutoff = soft > 0.f ? 2.30258509f / soft : 0.f;
  return !(d - lip * reach > cutoff * 1.001f + 1e-5f);
}

// Walls and ground after the contacts (integrator.cu:734-774).
DX_HD f3 boundary_forward(f3 v, int gx, int gy, int gz, int Gx, int Gy, int Gz, float ground_friction) {
  if (gx < kBound && v.x < 0.f) v.x = 0.f;
  if (gx > Gx - kBound && v.x > 0.f) v.x = 0.f;
  if (gy < kBound && v.y < 0.f) {
    if (ground_friction > 0.f) {
      if (ground_friction < 99.f) {
        float lin = v.y;
        f3 vit = mk3(v.x, 0.f, v.z);
        float lit = sqrtf(dot(vit, vit) + kNormEps);
        v = vit * fmaxf(1.f + ground_friction * lin / lit, 0.f);
      } else {
        v = mk3(0.f, 0.f, 0.f);
      }
    }
    v.y = 0.f;
  }
  if (gy > Gy - kBound && v.y > 0.f) v.y = 0.f;
  if (gz < kBound && v.z < 0.f) v.z = 0.f;
  if (gz > Gz - kBound && v.z > 0.f) v.z = 0.f;
  return v;
}

// Adjoint of boundary_forward given the post-contact velocity vv
// (integrator.cu:824-893).
DX_HD f3 boundary_backward(f3 gv, f3 vv, int gx, int gy, int gz, int Gx, int Gy, int Gz, float ground_friction) {
  f3 vin = vv;
  if (gx > Gx - kBound && vv.x > 0.f) vin.x = 0.f;
  if (gx < kBound && vv.x < 0.f) vin.x = 0.f;
  float lin = 0.f, lit = 1.f;
  f3 vit = mk3(0.f, 0.f, 0.f);
  bool hit = gy < kBound && vin.y < 0.f;
  if (hit) {
    lin = vin.y;
    vit = mk3(vin.x, 0.f, vin.z);
    lit = sqrtf(dot(vit, vit) + kNormEps);
    vin = vit * fmaxf(1.f + ground_friction * lin / lit, 0.f);
  }
  if (gz > Gz - kBound && vin.z > 0.f) gv.z = 0.f;
  if (gz < kBound && vin.z < 0.f) gv.z = 0.f;
  if (gy > Gy - kBound && vin.y > 0.f) gv.y = 0.f;
  if (hit) {
    gv.y = 0.f;
    float flag = 1.f + ground_friction * lin / lit;
    if (flag >= 0.f) {
      f3 gvit = gv * flag;
      float g_dot = dot(vit, gv);
      float glin = ground_friction / lit * g_dot;
      float glit = -ground_friction * lin / lit / lit * g_dot;
      gvit += vit * (glit / lit);
      gv = mk3(gvit.x, glin, gvit.z);
    } else {
      gv = mk3(0.f, 0.f, 0.f);
    }
  }
  if (gx > Gx - kBound && vv.x > 0.f) gv.x = 0.f;
  if (gx < kBound && vv.x < 0.f) gv.x = 0.f;
  return gv;
}

// Adjoint of contact_forward for one body (integrator.cu:902-1051).  vo is the
// velocity entering this body's contact; gv is the gradient of the velocity
// leaving it and is replaced by the gradient of vo.  Pose gradients are added
// to g_cur (pos 3 + quat 4) and g_nxt.
DX_HD void contact_backward(f3 gx, f3 vo, f3 &gv, const BodyPose &cur, const BodyPose &nxt, const BodyShape &sh,
                            float dt, float g_cur[7], float g_nxt[7], bool exact_capsule = false) {
  float friction = sh.tfsr.x, softness = sh.tfsr.y;
  f3 gxb = xform_inv(cur.p, cur.q, gx);
  float dist = shape_sdf(sh.tfsr, sh.args, gxb);
  float infl = fminf(expf(-dist * softness), 1.f);
  if (!((softness > 0.f && infl > 0.1f) || dist <= 0.f)) return;
  f3 g_gxb = mk3(0.f, 0.f, 0.f), g_bx = mk3(0.f, 0.f, 0.f);
  qf g_bq = mkq(0.f, 0.f, 0.f, 0.f);
  f3 un = shape_grad(sh.tfsr, sh.args, gxb);
  f3 rn = vnormalized(un);
  f3 nrm = qrot(cur.q, rn);
  f3 bv = body_velocity(gx, gxb, cur, nxt, dt);
  f3 rel = vo - bv;
  float nc = dot(rel, nrm);
  f3 vtin = rel - nrm * fminf(nc, 0.f);
  bool fr = nc < 0.f && dot(vtin, vtin) > 1e-30f;
  f3 vt = vtin;
  float vtn = vlength(vtin);
  if (fr) vt = vtin * ((1.f / vtn) * fmaxf(vtn + nc * friction, 0.f));
  float g_nc = 0.f;
  f3 g_bv = gv, g_rel = gv * (1.f - infl), g_vt = gv * infl;
  float g_infl = dot(vt - rel, gv);
  if (fr) {
    float bf = vtn + nc * friction;
    if (bf > 0.f) {
      g_nc += dot(vtin, g_vt) * friction / vtn;
      float g_vtn = -nc * g_nc / vtn;
      g_vt = g_vt * ((1.f / vtn) * bf) + vtin * (g_vtn / vtn);
    } else {
      g_vt = mk3(0.f, 0.f, 0.f);
    }
  }
  f3 g_n = mk3(0.f, 0.f, 0.f);
  g_rel += g_vt;
  if (nc < 0.f) {
    g_nc += -dot(nrm, g_vt);
    g_n += g_vt * (-nc);
  }
  g_rel += nrm * g_nc;
  g_n += rel * g_nc;
  gv = g_rel;
  g_bv = g_bv - g_rel;
  f3 g_np = mk3(0.f, 0.f, 0.f);
  qf g_nq = mkq(0.f, 0.f, 0.f, 0.f);
  xform_backward(nxt.q, gxb, g_bv * (1.f / dt), g_np, g_nq, g_gxb);
  g_nxt[0] += g_np.x; g_nxt[1] += g_np.y; g_nxt[2] += g_np.z;
  g_nxt[3] += g_nq.w; g_nxt[4] += g_nq.x; g_nxt[5] += g_nq.y; g_nxt[6] += g_nq.z;
  f3 g_rn = mk3(0.f, 0.f, 0.f);
  qrot_backward(cur.q, rn, g_n, g_bq, g_rn);
  g_gxb += shape_grad_backward(sh.tfsr, sh.args, gxb, vnormalized_backward(un, g_rn), exact_capsule);
  float ed = expf(-dist * softness);
  if (ed <= 1.f) g_gxb += un * (-softness * ed * g_infl);
  f3 g_tmp = mk3(0.f, 0.f, 0.f);
  xform_inv_backward(cur.p, cur.q, gx, g_gxb, g_bx, g_bq, g_tmp);
  g_cur[0] += g_bx.x; g_cur[1] += g_bx.y; g_cur[2] += g_bx.z;
  g_cur[3] += g_bq.w; g_cur[4] += g_bq.x; g_cur[5] += g_bq.y; g_cur[6] += g_bq.z;
}

// --------------------------------------------------------- SVD adjoint
// integrator.cu:102-108
DX_HD float clamp_gap(float a) { return a >= 0.f ? fmaxf(a, 1e-6f) : fminf(a, -1e-6f); }

// Gradient of F_tmp from gradients of (U, sigma, V) (integrator.cu:131-159):
//   gF = gF_direct + U [ (F o (U^T gU - gU^T U)) S + S (F o (V^T gV - gV^T V)) + diag(gs) ] V^T
// with F_ij = 1 / clamp_gap(sigma_j^2 - sigma_i^2) off the diagonal, S = diag(sigma).
// sigma_j^2 - sigma_i^2 is formed as (d_j - d_i)(sigma_j + sigma_i), which is
// exactly antisymmetric in (i, j), so F_ji = -F_ij except at a zero gap, where
// clamp_gap gives +1e-6 for both orders; U^T gU - gU^T U is antisymmetric.  One
// reciprocal and two 3-term differences per pair, then U M V^T.
DX_HD m33 svd_backward(const SVD3 &sv, const m33 &gU, f3 gs, const m33 &gV, const m33 &gFtmp_direct) {
  const float d[3] = {sv.d.x, sv.d.y, sv.d.z}, s[3] = {sv.s.x, sv.s.y, sv.s.z};
  m33 M = mzero();
  M.a[0][0] = gs.x;
  M.a[1][1] = gs.y;
  M.a[2][2] = gs.z;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i + 1; j < 3; ++j) {
      const float gap = (d[j] - d[i]) * (s[j] + s[i]);
      const float fij = 1.f / clamp_gap(gap);
      const float fji = gap == 0.f ? fij : -fij;
      float wu = 0.f, wv = 0.f;  // (U^T gU - gU^T U)_ij, (V^T gV - gV^T V)_ij
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        wu += sv.U.a[k][i] * gU.a[k][j] - gU.a[k][i] * sv.U.a[k][j];
        wv += sv.V.a[k][i] * gV.a[k][j] - gV.a[k][i] * sv.V.a[k][j];
      }
      // entries (i, j) and (j, i) of u_in S + S v_in (u_in = F o (..), v_in likewise)
      M.a[i][j] = fij * wu * s[j] + s[i] * fij * wv;
      M.a[j][i] = -fji * wu * s[i] - s[j] * fji * wv;
    }
  return gFtmp_direct + mm(mm(sv.U, M), mT(sv.V));
}

// The same adjoint for callers that hold the rotated gradients: ku_p and kv_p
// are entry (i, j) of U^T gU - gU^T U and V^T gV - gV^T V for the pairs
// p = (0,1), (0,2), (1,2); returns U (M + madd) V^T (without a direct term).
// With opposite (kv = -ku, `opposite`) the pair entries F_ij ku (s_j - s_i)
// are formed from d_j - d_i, without the cancellation of the two products.
DX_HD m33 svd_backward_rot(const SVD3 &sv, const float ku[3], const float kv[3], f3 gs, const m33 &madd,
                           bool opposite) {
  const float d[3] = {sv.d.x, sv.d.y, sv.d.z}, s[3] = {sv.s.x, sv.s.y, sv.s.z};
  m33 M = madd;
  M.a[0][0] += gs.x;
  M.a[1][1] += gs.y;
  M.a[2][2] += gs.z;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int i = q == 2 ? 1 : 0, j = q == 0 ? 1 : 2;
    const float gap = (d[j] - d[i]) * (s[j] + s[i]);
    const float fij = 1.f / clamp_gap(gap);
    const float fji = gap == 0.f ? fij : -fij;
    if (opposite) {
      const float k = ku[q] * (d[j] - d[i]);
      M.a[i][j] += fij * k;
      M.a[j][i] += fji * k;
    } else {
      M.a[i][j] += fij * ku[q] * s[j] + s[i] * fij * kv[q];
      M.a[j][i] -= fji * ku[q] * s[i] + s[j] * fji * kv[q];
    }
  }
  return mm(mm(sv.U, M), mT(sv.V));
}

// Adjoint of the return mapping and stress (integrator.cu:541-625): dL/dF_tmp
// from dL/dP (g_stress, P = 2 mu (newF - R) newF^T + lam J (J - 1) I as
// `constitutive` returns it) and the incoming dL/dnewF (GF), given the SVD of
// F_tmp and the constitutive intermediates.  Worked in the frame of the SVD:
// with newF = U D V^T (D the projected singular values, sigma when not
// yielded), R = U V^T and X = U^T g_stress U,
//   U^T dL/dR V = -2 mu X D =: W,
//   U^T dL/dnewF V = U^T GF V + 2 mu (X^T (D - 1) + X D) = U^T GF V + Q,
// and the SVD adjoint needs only the antisymmetric parts of U^T dL/dU and
// V^T dL/dV: W - W^T and W^T - W, plus T E - (T E)^T and T^T E - (T^T E)^T
// after a yield (T = U^T dL/dnewF V, E = diag(D)).  Not yielded, newF is F_tmp
// itself and dL/dnewF passes to dL/dF_tmp directly.
// load_gf() returns dL/dnewF; it is called where the value is first needed
// (so that a caller that reads it from memory need not hold it before).
template <class LoadGF>
DX_HD m33 plastic_stress_backward_at(const SVD3 &sv, const Plastic &pl, const m33 &g_stress, LoadGF load_gf,
                                     float mu, float lam, float ys) {
  const m33 X = mm(mT(sv.U), mm(g_stress, sv.U));
  const f3 D3 = pl.expe, Dm3 = pl.dm1;
  const float Dv[3] = {D3.x, D3.y, D3.z}, Dm[3] = {Dm3.x, Dm3.y, Dm3.z};
  m33 Q;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Q.a[i][j] = (X.a[j][i] * Dm[j] + X.a[i][j] * Dv[j]) * (2.f * mu);
  const float g_J = ((2.f * pl.J - 1.f) * lam) * trace(g_stress);
  float ku[3], kv[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int i = q == 2 ? 1 : 0, j = q == 0 ? 1 : 2;
    const float w = (-2.f * mu) * (X.a[i][j] * Dv[j] - X.a[j][i] * Dv[i]);  // W_ij - W_ji
    ku[q] = w;
    kv[q] = -w;
  }
  f3 g_s;
  if (pl.yielded) {
    const m33 T = mm(mT(sv.U), mm(load_gf(), sv.V)) + Q;
    const f3 ee = pl.expe;
    const float ev[3] = {ee.x, ee.y, ee.z};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int i = q == 2 ? 1 : 0, j = q == 0 ? 1 : 2;
      ku[q] += T.a[i][j] * ev[j] - T.a[j][i] * ev[i];
      kv[q] += T.a[j][i] * ev[j] - T.a[i][j] * ev[i];
    }
    const f3 Fpart = mk3(T.a[0][0], T.a[1][1], T.a[2][2]);
    const f3 Jpart = mk3(g_J * ee.y * ee.z, g_J * ee.x * ee.z, g_J * ee.x * ee.y);
    f3 g_e = hadamard(ee, Jpart + Fpart);
    const f3 eh = pl.eps_hat;
    const float ehn = pl.eps_hat_norm;
    f3 g_eh = g_e * (-pl.delta_gamma / ehn);
    const float g_ehn = -dot(eh * (1.f / ehn), g_e) * (ys / (2.f * mu)) / ehn;
    g_eh += eh * (g_ehn / ehn);
    const float sm = (g_eh.x + g_eh.y + g_eh.z) * (1.f / 3.f);
    g_e += mk3(g_eh.x - sm, g_eh.y - sm, g_eh.z - sm);
    g_s = mk3(0.f, 0.f, 0.f);
    if (sv.s.x >= kSigClip) g_s.x += g_e.x / sv.s.x;
    if (sv.s.y >= kSigClip) g_s.y += g_e.y / sv.s.y;
    if (sv.s.z >= kSigClip) g_s.z += g_e.z / sv.s.z;
    return svd_backward_rot(sv, ku, kv, g_s, mzero(), false);
  } else {
    // dL/dF_tmp receives dL/dnewF directly: GF + U Q V^T
    g_s = mk3(g_J * sv.s.y * sv.s.z, g_J * sv.s.x * sv.s.z, g_J * sv.s.x * sv.s.y);
    const m33 r = svd_backward_rot(sv, ku, kv, g_s, Q, true);
    return load_gf() + r;
  }
}

DX_HD m33 plastic_stress_backward(const SVD3 &sv, const Plastic &pl, const m33 &g_stress, const m33 &GF, float mu,
                                  float lam, float ys) {
  return plastic_stress_backward_at(sv, pl, g_stress, [&]() { return GF; }, mu, lam, ys);
}

}  // namespace dexmpm
