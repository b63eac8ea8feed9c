/*
 * mpm_oracle.c -- FP64 CPU restatement of DexDeform's MLS-MPM substep and its
 * hand-written adjoint.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke
 * check and the CPU-baseline leg of bench.py call it as the checker.  Nothing
 * in the product library links or calls this file.
 *
 * Every function restates one reference routine, cited as path:line within
 * the DexDeform project (mpm/csrc/...).  Semantics follow the reference
 * exactly (same branches, thresholds, clamps and array layouts: AoS vec3 =
 * 3 values, mat3 = 9 values row-major, quat = (w,x,y,z), dense x-major grid
 * index (x*Gy + y)*Gz + z); only the arithmetic is widened to double.
 * grid_lower is identically zero in the reference (mpm/simulator.py:16,386),
 * so the oracle omits it.
 *
 * Parallel loops use OpenMP; scatters use `omp atomic` on doubles.
 */
#include <math.h>
#include <string.h>
#include <stdlib.h>

#define NORM_EPS 1e-8        /* integrator.cu:11 */
#define SIG_CLIP_EPS 0.05    /* integrator.cu:12 */
#define NORM_EPS2 1e-30      /* shape.h:4 */

/* ---------------------------------------------------------------- vec/mat */
typedef struct { double x, y, z; } v3;
typedef struct { double m[3][3]; } m3;
typedef struct { double w, x, y, z; } qt;

static inline v3 V3(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, double s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline v3 vhad(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double vget(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline v3 vload(const double *p) { return V3(p[0], p[1], p[2]); }
static inline void vstore(double *p, v3 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; }
static inline void vacc(double *p, v3 a) { p[0] += a.x; p[1] += a.y; p[2] += a.z; }

static inline m3 mzero(void) { m3 r; memset(&r, 0, sizeof(r)); return r; }
static inline m3 mdiag(v3 d) { m3 r = mzero(); r.m[0][0] = d.x; r.m[1][1] = d.y; r.m[2][2] = d.z; return r; }
static inline m3 meye(double s) { return mdiag(V3(s, s, s)); }
static inline m3 mload(const double *p) { m3 r; memcpy(r.m, p, 9 * sizeof(double)); return r; }
static inline void mstore(double *p, m3 a) { memcpy(p, a.m, 9 * sizeof(double)); }
static inline void macc(double *p, m3 a) { for (int i = 0; i < 9; ++i) p[i] += (&a.m[0][0])[i]; }
static inline m3 mT(m3 a) { m3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i]; return r; }
static inline m3 mmul(m3 a, m3 b) {
  m3 r = mzero();
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) for (int k = 0; k < 3; ++k) r.m[i][j] += a.m[i][k] * b.m[k][j];
  return r;
}
static inline v3 mvec(m3 a, v3 b) {
  return V3(a.m[0][0] * b.x + a.m[0][1] * b.y + a.m[0][2] * b.z,
            a.m[1][0] * b.x + a.m[1][1] * b.y + a.m[1][2] * b.z,
            a.m[2][0] * b.x + a.m[2][1] * b.y + a.m[2][2] * b.z);
}
static inline m3 madd(m3 a, m3 b) { m3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j]; return r; }
static inline m3 msub(m3 a, m3 b) { m3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] - b.m[i][j]; return r; }
static inline m3 mscale(m3 a, double s) { m3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] * s; return r; }
static inline m3 mhad(m3 a, m3 b) { m3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] * b.m[i][j]; return r; }
static inline double msum(m3 a) { double s = 0; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) s += a.m[i][j]; return s; }
/* outer(a,b)[i][j] = a_i b_j  (mat3.h:170-172) */
static inline m3 mouter(v3 a, v3 b) {
  m3 r; double av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = av[i] * bv[j];
  return r;
}
static inline double clampd(double a, double lo, double hi) { return a < lo ? lo : (a > hi ? hi : a); }

/* ------------------------------------------------------------ quaternions */
/* q * v  (quat.h:14-19) */
static inline v3 qrot(qt q, v3 v) {
  v3 qv = V3(q.x, q.y, q.z);
  v3 uv = vcross(qv, v), uuv = vcross(qv, uv);
  return vadd(v, vmul(vadd(vmul(uv, q.w), uuv), 2.0));
}
static inline qt qinv(qt q) { qt r = {q.w, -q.x, -q.y, -q.z}; return r; }
static inline qt qload(const double *p) { qt r = {p[0], p[1], p[2], p[3]}; return r; }
static inline v3 xform(v3 p, qt q, v3 pt) { return vadd(p, qrot(q, pt)); }            /* quat.h:89-92 */
static inline v3 xform_inv(v3 p, qt q, v3 pt) { return qrot(qinv(q), vsub(pt, p)); } /* quat.h:94-97 */

/* quat.h:25-49 */
static void qmul_backward(qt q, v3 v, v3 gout, qt *gq, v3 *gv) {
  v3 qv = V3(q.x, q.y, q.z);
  v3 uv = vcross(qv, v);
  gq->w += vdot(uv, gout) * 2.0;
  v3 g_uv = vmul(gout, 2.0 * q.w);
  v3 g_uuv = vmul(gout, 2.0);
  v3 g_qv = vcross(uv, g_uuv);
  g_uv = vadd(g_uv, vcross(g_uuv, qv));
  g_qv = vadd(g_qv, vcross(v, g_uv));
  *gv = vadd(*gv, vadd(gout, vcross(g_uv, qv)));
  gq->x += g_qv.x; gq->y += g_qv.y; gq->z += g_qv.z;
}
/* quat.h:52-63 */
static void xform_backward(v3 p, qt q, v3 pt, v3 gout, v3 *gp, qt *gq, v3 *gpt) {
  (void)p;
  *gp = vadd(*gp, gout);
  qmul_backward(q, pt, gout, gq, gpt);
}
/* quat.h:65-80 */
static void xform_inv_backward(v3 p, qt q, v3 pt, v3 gout, v3 *gp, qt *gq, v3 *gpt) {
  qt tq = {0, 0, 0, 0};
  v3 tp = V3(0, 0, 0);
  qmul_backward(qinv(q), vsub(pt, p), gout, &tq, &tp);
  gq->w += tq.w; gq->x -= tq.x; gq->y -= tq.y; gq->z -= tq.z;
  *gp = vsub(*gp, tp);
  *gpt = vadd(*gpt, tp);
}

/* ------------------------------------------------------------------ SDFs */
static inline double vlength(v3 a) { return sqrt(vdot(a, a) + NORM_EPS2); }       /* shape.h:7-9 */
static inline v3 vnormalized(v3 a) { return vmul(a, 1.0 / vlength(a)); }         /* shape.h:13-15 */
static inline v3 vnormalized_backward(v3 a, v3 g) {                             /* shape.h:17-25 */
  double d = vdot(a, a) + NORM_EPS2;
  return vmul(vsub(g, vmul(a, vdot(vmul(a, 1.0 / d), g))), 1.0 / sqrt(d));
}
static inline int shape_type(qt tfsr) { return (int)floor(tfsr.w + 0.1); }        /* shape.h:33-35 */

/* shape.h:37-61: box (type 0, half extents args.w,x,y) or capsule (type 1, radius args.w,
   full length args.x along y), minus the rounding radius tfsr.z */
static double shape_sdf(qt tfsr, qt args, v3 g) {
  int type = shape_type(tfsr);
  double sdf = 0.0;
  if (type == 0) {
    v3 q = vsub(V3(fabs(g.x), fabs(g.y), fabs(g.z)), V3(args.w, args.x, args.y));
    v3 qp = V3(fmax(q.x, 0.0), fmax(q.y, 0.0), fmax(q.z, 0.0));
    sdf = vlength(qp) + fmin(fmax(fmax(q.x, q.y), q.z), 0.0);
  } else if (type == 1) {
    double r = args.w, h = args.x;
    v3 p2 = g;
    p2.y += h / 2;
    p2.y -= fmin(fmax(p2.y, 0.0), h);
    sdf = vlength(p2) - r;
  }
  return sdf - tfsr.z;
}

static inline void abs_backward(v3 g, v3 *gr) {                                  /* shape.h:27-31 */
  if (g.x < 0) gr->x *= -1;
  if (g.y < 0) gr->y *= -1;
  if (g.z < 0) gr->z *= -1;
}

/* shape.h:65-102 */
static v3 shape_grad(qt tfsr, qt args, v3 g) {
  int type = shape_type(tfsr);
  v3 grad = V3(0, 0, 0);
  if (type == 0) {
    v3 q = vsub(V3(fabs(g.x), fabs(g.y), fabs(g.z)), V3(args.w, args.x, args.y));
    double inside = fmax(fmax(q.x, q.y), q.z);
    if (inside <= 0) {
      if (q.x == inside) grad.x += 1;
      if (q.y == inside) grad.y += 1;
      if (q.z == inside) grad.z += 1;
    } else {
      grad = vnormalized(V3(fmax(q.x, 0.0), fmax(q.y, 0.0), fmax(q.z, 0.0)));
    }
    abs_backward(g, &grad);
  } else if (type == 1) {
    double h = args.x;
    v3 p2 = g;
    p2.y += h / 2;
    p2.y -= fmin(fmax(p2.y, 0.0), h);
    return vnormalized(p2);
  }
  return grad;
}

/* Capsule-normal derivative: 0 restates the reference (below), 1 gives the
   true derivative (not part of the reference; used to test the product's
   optional exact mode). */
static int g_capsule_exact = 0;
void orc_set_capsule_grad(int exact) { g_capsule_exact = exact; }

/* shape.h:104-152.  The capsule branch back-propagates a zero vector (it reads
   grad_in, which is still zero, instead of grad_out), so it always returns 0. */
static v3 shape_grad_backward(qt tfsr, qt args, v3 g, v3 gout) {
  int type = shape_type(tfsr);
  v3 gin = V3(0, 0, 0);
  if (type == 0) {
    v3 q = vsub(V3(fabs(g.x), fabs(g.y), fabs(g.z)), V3(args.w, args.x, args.y));
    double inside = fmax(fmax(q.x, q.y), q.z);
    gin = gout;
    abs_backward(g, &gin);
    if (inside <= 0) {
      gin = V3(0, 0, 0);
    } else {
      v3 q2 = V3(fmax(q.x, 0.0), fmax(q.y, 0.0), fmax(q.z, 0.0));
      gin = vnormalized_backward(q2, gin);
      if (q.x < 0) gin.x = 0;
      if (q.y < 0) gin.y = 0;
      if (q.z < 0) gin.z = 0;
      abs_backward(g, &gin);
    }
  } else if (type == 1) {
    double h = args.x;
    v3 p2 = g;
    p2.y += h / 2;
    double zero_y = (p2.y >= 0.0 && p2.y <= h) ? 1.0 : 0.0;
    p2.y -= fmin(fmax(p2.y, 0.0), h);
    if (g_capsule_exact) {
      gin = vnormalized_backward(p2, gout);
      if (zero_y != 0.0) gin.y = 0.0;
      return gin;
    }
    gin = vnormalized_backward(p2, gin);
    gin.y *= zero_y;
    return gin;
  }
  return gin;
}

/* ------------------------------------------------------------------- SVD */
/* McAdams, Selle, Tamstorf, Teran, Sifakis (2011), "Computing the singular
   value decomposition of 3x3 matrices with minimal branching and elementary
   floating point operations", as vendored at mpm/csrc/svd.h:1-413 (computed
   in double there too).  Jacobi eigen-analysis of A^T A with approximate
   Givens quaternions (8 sweeps of the (1,2),(2,3),(1,3) rotations), column
   sort with sign-preserving swaps, Givens QR.  The reference's constants are
   float literals promoted to double (svd.h:19-21), reproduced as such. */
static const double SVD_GAMMA = (double)5.82842712474619f;
static const double SVD_CSTAR = (double)0.9238795325112867f;
static const double SVD_SSTAR = (double)0.3826834323650897f;
static const double SVD_EPS = 1e-6;

/* svd.h:121-135 */
static void approx_givens(double a11, double a12, double a22, double *ch, double *sh) {
  double c = 2.0 * (a11 - a22), s = a12;
  int ok = SVD_GAMMA * s * s < c * c;
  double w = 1.0 / sqrt(c * c + s * s);
  *ch = ok ? w * c : SVD_CSTAR;
  *sh = ok ? w * s : SVD_SSTAR;
}

/* svd.h:137-192: one conjugation on the (s11,s21,s22) pivot, quaternion update
   at component slots (x,y,z), then the cyclic relabelling of S. */
static void jacobi_conj(int x, int y, int z, double *S /* s11,s21,s22,s31,s32,s33 */, double *qV) {
  double ch, sh;
  approx_givens(S[0], S[1], S[2], &ch, &sh);
  double scale = ch * ch + sh * sh;
  double a = (ch * ch - sh * sh) / scale, b = (2.0 * sh * ch) / scale;
  double s11 = S[0], s21 = S[1], s22 = S[2], s31 = S[3], s32 = S[4], s33 = S[5];
  double n11 = a * (a * s11 + b * s21) + b * (a * s21 + b * s22);
  double n21 = a * (-b * s11 + a * s21) + b * (-b * s21 + a * s22);
  double n22 = -b * (-b * s11 + a * s21) + a * (-b * s21 + a * s22);
  double n31 = a * s31 + b * s32;
  double n32 = -b * s31 + a * s32;
  double n33 = s33;
  double t[3] = {qV[0] * sh, qV[1] * sh, qV[2] * sh};
  sh *= qV[3];
  qV[0] *= ch; qV[1] *= ch; qV[2] *= ch; qV[3] *= ch;
  qV[z] += sh;
  qV[3] -= t[z];
  qV[x] += t[y];
  qV[y] -= t[x];
  /* relabel: (s11,s21,s22,s31,s32,s33) <- (s22,s32,s33,s21,s31,s11) */
  S[0] = n22; S[1] = n32; S[2] = n33; S[3] = n21; S[4] = n31; S[5] = n11;
}

/* svd.h:253-262 */
static void qr_givens(double a1, double a2, double *ch, double *sh) {
  double r2 = a1 * a1 + a2 * a2;
  double rho = r2 / sqrt(r2);          /* accurateSqrt, svd.h:23 */
  double s = rho > SVD_EPS ? a2 : 0.0;
  double c = fabs(a1) + fmax(rho, SVD_EPS);
  if (a1 < 0) { double t = s; s = c; c = t; }
  double w = 1.0 / sqrt(c * c + s * s);
  *ch = c * w;
  *sh = s * w;
}

/* SVD mode.  0 (default): the reference's svd3 restated exactly, including
   the drift of its approximate Givens quaternions (the float-literal constants
   make c*^2 + s*^2 != 1, so V is a rotation scaled by up to ~1e-7; sigma - 1
   then carries ~1e-7 absolute error).  1: converged FP64 cyclic Jacobi with
   exact angles (Golub & Van Loan sec. 8.5) on A^T A, same sort / sign / QR
   conventions -- the reference's algorithm in exact arithmetic, used to
   separate that artifact from the rest of the substep. */
static int g_svd_mode = 0;
void orc_set_svd_mode(int mode) { g_svd_mode = mode; }

static void jacobi_exact(double S[3][3], m3 *V, int p, int q, int r) {
  double apq = S[p][q];
  if (apq == 0.0) return;
  double theta = (S[q][q] - S[p][p]) / (2.0 * apq);
  double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
  if (theta < 0) t = -t;
  double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
  S[p][p] -= t * apq; S[q][q] += t * apq; S[p][q] = S[q][p] = 0.0;
  double arp = S[r][p], arq = S[r][q];
  S[r][p] = S[p][r] = c * arp - s * arq;
  S[r][q] = S[q][r] = s * arp + c * arq;
  for (int k = 0; k < 3; ++k) {
    double vp = V->m[k][p], vq = V->m[k][q];
    V->m[k][p] = c * vp - s * vq; V->m[k][q] = s * vp + c * vq;
  }
}

static m3 eigvec_exact(m3 ATA) {
  double S[3][3];
  memcpy(S, ATA.m, sizeof(S));
  m3 V = meye(1.0);
  for (int it = 0; it < 12; ++it) {
    jacobi_exact(S, &V, 0, 1, 2);
    jacobi_exact(S, &V, 0, 2, 1);
    jacobi_exact(S, &V, 1, 2, 0);
  }
  return V;
}

/* A = U diag(sig) V^T, U and V proper rotations, |sig| sorted descending, the
   sign of det(A) carried by sig[2]  (svd.h:347-413) */
void orc_svd3(const double *A9, double *U9, double *sig3, double *V9) {
  m3 A = mload(A9);
  m3 ATA = mmul(mT(A), A);
  if (g_svd_mode == 1) {
    m3 V = eigvec_exact(ATA);
    m3 B = mmul(A, V);
    double rho[3];
    for (int c = 0; c < 3; ++c) rho[c] = B.m[0][c] * B.m[0][c] + B.m[1][c] * B.m[1][c] + B.m[2][c] * B.m[2][c];
    const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int pi = 0; pi < 3; ++pi) {
      int i = pr[pi][0], j = pr[pi][1];
      if (rho[i] < rho[j]) {
        for (int r = 0; r < 3; ++r) {
          double t = B.m[r][i]; B.m[r][i] = B.m[r][j]; B.m[r][j] = -t;
          t = V.m[r][i]; V.m[r][i] = V.m[r][j]; V.m[r][j] = -t;
        }
        double t = rho[i]; rho[i] = rho[j]; rho[j] = t;
      }
    }
    /* Givens QR with r >= 0 on the two pivots */
    m3 Q = meye(1.0);
    const int rows[3][3] = {{0, 1, 0}, {0, 2, 0}, {1, 2, 1}};
    for (int g = 0; g < 3; ++g) {
      int i = rows[g][0], j = rows[g][1], col = rows[g][2];
      double a = B.m[i][col], b = B.m[j][col], r = sqrt(a * a + b * b);
      if (!(r > 0.0)) continue;
      double c = a / r, s = b / r;
      for (int k = 0; k < 3; ++k) {
        double bi = B.m[i][k], bj = B.m[j][k];
        B.m[i][k] = c * bi + s * bj; B.m[j][k] = -s * bi + c * bj;
        double qi = Q.m[k][i], qj = Q.m[k][j];
        Q.m[k][i] = c * qi + s * qj; Q.m[k][j] = -s * qi + c * qj;
      }
    }
    mstore(U9, Q);
    sig3[0] = B.m[0][0]; sig3[1] = B.m[1][1]; sig3[2] = B.m[2][2];
    mstore(V9, V);
    return;
  }
  double S[6] = {ATA.m[0][0], ATA.m[1][0], ATA.m[1][1], ATA.m[2][0], ATA.m[2][1], ATA.m[2][2]};
  double qV[4] = {0, 0, 0, 1};  /* (x,y,z,w) */
  for (int it = 0; it < 8; ++it) {
    jacobi_conj(0, 1, 2, S, qV);
    jacobi_conj(1, 2, 0, S, qV);
    jacobi_conj(2, 0, 1, S, qV);
  }
  /* quaternion -> matrix (svd.h:94-119) */
  double w = qV[3], x = qV[0], y = qV[1], z = qV[2];
  m3 V;
  V.m[0][0] = 1 - 2 * (y * y + z * z); V.m[0][1] = 2 * (x * y - w * z); V.m[0][2] = 2 * (x * z + w * y);
  V.m[1][0] = 2 * (x * y + w * z); V.m[1][1] = 1 - 2 * (x * x + z * z); V.m[1][2] = 2 * (y * z - w * x);
  V.m[2][0] = 2 * (x * z - w * y); V.m[2][1] = 2 * (y * z + w * x); V.m[2][2] = 1 - 2 * (x * x + y * y);
  m3 B = mmul(A, V);
  /* sort columns by squared norm, swapping with a sign flip (svd.h:212-246) */
  double rho[3];
  for (int c = 0; c < 3; ++c) rho[c] = B.m[0][c] * B.m[0][c] + B.m[1][c] * B.m[1][c] + B.m[2][c] * B.m[2][c];
  const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int pi = 0; pi < 3; ++pi) {
    int i = pairs[pi][0], j = pairs[pi][1];
    if (rho[i] < rho[j]) {
      for (int r = 0; r < 3; ++r) {
        double t = B.m[r][i]; B.m[r][i] = B.m[r][j]; B.m[r][j] = -t;
        t = V.m[r][i]; V.m[r][i] = V.m[r][j]; V.m[r][j] = -t;
      }
      if (pi < 2) { double t = rho[i]; rho[i] = rho[j]; rho[j] = t; }
    }
  }
  /* Givens QR: rows (0,1) on column 0, rows (0,2) on column 0, rows (1,2) on
     column 1 (svd.h:264-344).  Each rotation G with a = cos, b = sin applies
     B <- G^T B; U accumulates G1 G2 G3. */
  double ch, sh, a, b;
  m3 R = B, Q = meye(1.0), G;
  qr_givens(R.m[0][0], R.m[1][0], &ch, &sh);
  a = 1 - 2 * sh * sh; b = 2 * ch * sh;
  G = meye(1.0); G.m[0][0] = a; G.m[0][1] = -b; G.m[1][0] = b; G.m[1][1] = a;
  R = mmul(mT(G), R); Q = mmul(Q, G);
  qr_givens(R.m[0][0], R.m[2][0], &ch, &sh);
  a = 1 - 2 * sh * sh; b = 2 * ch * sh;
  G = meye(1.0); G.m[0][0] = a; G.m[0][2] = -b; G.m[2][0] = b; G.m[2][2] = a;
  R = mmul(mT(G), R); Q = mmul(Q, G);
  qr_givens(R.m[1][1], R.m[2][1], &ch, &sh);
  a = 1 - 2 * sh * sh; b = 2 * ch * sh;
  G = meye(1.0); G.m[1][1] = a; G.m[1][2] = -b; G.m[2][1] = b; G.m[2][2] = a;
  R = mmul(mT(G), R); Q = mmul(Q, G);
  mstore(U9, Q);
  sig3[0] = R.m[0][0]; sig3[1] = R.m[1][1]; sig3[2] = R.m[2][2];
  mstore(V9, V);
}

/* ------------------------------------------------------------ von Mises */
/* integrator.cu:42-67 */
static double von_mises(m3 F, m3 U, v3 s, m3 V, double yield, double mu, m3 *outF) {
  v3 sn = V3(fmax(s.x, SIG_CLIP_EPS), fmax(s.y, SIG_CLIP_EPS), fmax(s.z, SIG_CLIP_EPS));
  v3 e = V3(log(sn.x), log(sn.y), log(sn.z));
  double mean = (e.x + e.y + e.z) / 3.0;
  v3 eh = V3(e.x - mean, e.y - mean, e.z - mean);
  double ehn = sqrt(vdot(eh, eh) + NORM_EPS);
  double dg = ehn - yield / (2 * mu);
  if (dg > 0.0) {
    e = vsub(e, vmul(eh, dg / ehn));
    v3 ee = V3(exp(e.x), exp(e.y), exp(e.z));
    *outF = mmul(mmul(U, mdiag(ee)), mT(V));
    return ee.x * ee.y * ee.z;
  }
  *outF = F;
  return s.x * s.y * s.z;
}

/* ------------------------------------------------- quadratic B-spline */
typedef struct { int base[3]; double fx[3]; double w[3][3]; double w1[3][3]; } stencil;

/* integrator.cu:348-352, 492-493: w[axis][i], w1 = d w / d x */
static inline void make_stencil(v3 x, double inv_dx, stencil *s) {
  double xs[3] = {x.x * inv_dx, x.y * inv_dx, x.z * inv_dx};
  for (int d = 0; d < 3; ++d) {
    s->base[d] = (int)floor(xs[d] - 0.5);
    double f = xs[d] - (double)s->base[d];
    s->fx[d] = f;
    s->w[d][0] = 0.5 * (1.5 - f) * (1.5 - f);
    s->w[d][1] = 0.75 - (f - 1.0) * (f - 1.0);
    s->w[d][2] = 0.5 * (f - 0.5) * (f - 0.5);
    s->w1[d][0] = -inv_dx * (1.5 - f);
    s->w1[d][1] = inv_dx * (-2.0 * f + 2.0);
    s->w1[d][2] = -inv_dx * (-f + 0.5);
  }
}
static inline long gidx(const int *g, int x, int y, int z) { return ((long)x * g[1] + y) * g[2] + z; }

/* integrator.cu:33-40 */
static inline v3 dweight(const stencil *s, int i, int j, int k) {
  return V3(s->w1[0][i] * s->w[1][j] * s->w[2][k], s->w[0][i] * s->w1[1][j] * s->w[2][k],
            s->w[0][i] * s->w[1][j] * s->w1[2][k]);
}

/* =================================================================== API */

/* integrator.cu:84-100 */
void orc_compute_svd(int n, const double *F, const double *C, double dt,
                     double *newF, double *U, double *V, double *sig) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < n; ++p) {
    m3 Ft = mmul(madd(meye(1.0), mscale(mload(C + 9 * p), dt)), mload(F + 9 * p));
    mstore(newF + 9 * p, Ft);
    orc_svd3(&Ft.m[0][0], U + 9 * p, sig + 3 * p, V + 9 * p);
  }
}

/* integrator.cu:312-394 */
void orc_p2g(int n, const double *x, const double *v, const double *mass, const double *vol,
             const double *Ftmp, const double *U, const double *sig, const double *V,
             const double *C, const double *mly, const int *gdim, double dx, double inv_dx,
             double dt, double *outF, double *grid_mv, double *grid_m) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < n; ++p) {
    stencil st;
    make_stencil(vload(x + 3 * p), inv_dx, &st);
    m3 Um = mload(U + 9 * p), Vm = mload(V + 9 * p), Fm = mload(Ftmp + 9 * p), nF;
    double mu = mly[3 * p], lam = mly[3 * p + 1], ys = mly[3 * p + 2];
    double J = von_mises(Fm, Um, vload(sig + 3 * p), Vm, ys, mu, &nF);
    mstore(outF + 9 * p, nF);
    m3 r = mmul(Um, mT(Vm));
    m3 stress = madd(mscale(mmul(msub(nF, r), mT(nF)), 2.0 * mu), meye(lam * J * (J - 1)));
    stress = mscale(stress, -dt * vol[p] * 4.0 * inv_dx * inv_dx);
    m3 affine = madd(stress, mscale(mload(C + 9 * p), mass[p]));
    v3 mv = vmul(vload(v + 3 * p), mass[p]);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          double w = st.w[0][i] * st.w[1][j] * st.w[2][k];
          v3 dpos = vmul(V3(i - st.fx[0], j - st.fx[1], k - st.fx[2]), dx);
          long id = gidx(gdim, st.base[0] + i, st.base[1] + j, st.base[2] + k);
          v3 c = vmul(vadd(mv, mvec(affine, dpos)), w);
#pragma omp atomic
          grid_m[id] += mass[p] * w;
#pragma omp atomic
          grid_mv[3 * id] += c.x;
#pragma omp atomic
          grid_mv[3 * id + 1] += c.y;
#pragma omp atomic
          grid_mv[3 * id + 2] += c.z;
        }
  }
}

/* one body-contact step of grid_op_v2 (integrator.cu:694-730); returns 1 when
   the body touched the node */
static int contact_fwd(v3 gx, v3 *vo, v3 bx, qt bq, v3 nbx, qt nbq, qt tfsr, qt args, double dt) {
  double friction = tfsr.x, softness = tfsr.y;
  v3 gxb = xform_inv(bx, bq, gx);
  double dist = shape_sdf(tfsr, args, gxb);
  double infl = fmin(exp(-dist * softness), 1.0);
  if ((softness > 0 && infl > 0.1) || dist <= 0) {
    v3 nrm = qrot(bq, vnormalized(shape_grad(tfsr, args, gxb)));
    v3 bv = vmul(vsub(xform(nbx, nbq, gxb), gx), 1.0 / dt);
    v3 rel = vsub(*vo, bv);
    double nc = vdot(rel, nrm);
    v3 vt = vsub(rel, vmul(nrm, fmin(nc, 0.0)));
    if (nc < 0.0 && vdot(vt, vt) > 1e-30) {
      double vtn = vlength(vt);
      vt = vmul(vt, (1.0 / vtn) * fmax(0.0, vtn + nc * friction));
    }
    *vo = vadd(vadd(bv, vmul(rel, 1 - infl)), vmul(vt, infl));
    return 1;
  }
  return 0;
}

/* integrator.cu:647-777.  grid_body_v_in may be NULL (it is only read by the
   adjoint). */
void orc_grid_op(const int *gdim, const double *grid_m, const double *grid_mv,
                 double *grid_body_v_in, const double *gravity, int nb, const double *bpos,
                 const double *brot, const double *nbpos, const double *nbrot,
                 const double *tfsr, const double *bargs, double dx, double inv_dx, double dt,
                 double ground_friction, double *grid_v_out) {
  (void)inv_dx;
  long dim = (long)gdim[0] * gdim[1] * gdim[2];
#pragma omp parallel for schedule(static)
  for (long t = 0; t < dim; ++t) {
    if (!(grid_m[t] > 1e-12)) continue;
    int gxi = (int)(t / gdim[2] / gdim[1]), gyi = (int)((t / gdim[2]) % gdim[1]), gzi = (int)(t % gdim[2]);
    double m = grid_m[t];
    v3 vo = vadd(vmul(vload(grid_mv + 3 * t), 1.0 / m), vmul(vload(gravity), dt));
    v3 gx = V3(gxi * dx, gyi * dx, gzi * dx);
    for (int b = 0; b < nb; ++b) {
      if (grid_body_v_in) vstore(grid_body_v_in + 3 * (t * (nb + 1) + b), vo);
      contact_fwd(gx, &vo, vload(bpos + 3 * b), qload(brot + 4 * b), vload(nbpos + 3 * b),
                  qload(nbrot + 4 * b), qload(tfsr + 4 * b), qload(bargs + 4 * b), dt);
    }
    if (grid_body_v_in) vstore(grid_body_v_in + 3 * (t * (nb + 1) + nb), vo);
    const int bound = 3;
    if (gxi < bound && vo.x < 0) vo.x = 0;
    if (gxi > gdim[0] - bound && vo.x > 0) vo.x = 0;
    if (gyi < bound && vo.y < 0) {
      if (ground_friction > 0.0) {
        if (ground_friction < 99.0) {
          double lin = vo.y;
          v3 vit = V3(vo.x, 0.0, vo.z);
          double lit = sqrt(vdot(vit, vit) + NORM_EPS);
          vo = vmul(vit, fmax(1.0 + ground_friction * lin / lit, 0.0));
        } else {
          vo = V3(0, 0, 0);
        }
      }
      vo.y = 0;
    }
    if (gyi > gdim[1] - bound && vo.y > 0) vo.y = 0;
    if (gzi < bound && vo.z < 0) vo.z = 0;
    if (gzi > gdim[2] - bound && vo.z > 0) vo.z = 0;
    vstore(grid_v_out + 3 * t, vo);
  }
}

/* integrator.cu:1059-1109 (ground_height is 3 cells: mpm/simulator.py:493-494) */
void orc_g2p(int n, const double *x, const double *grid_v, const int *gdim, double dx,
             double inv_dx, double dt, double ground_height, double *out_v, double *out_C,
             double *out_x) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < n; ++p) {
    stencil st;
    v3 xp = vload(x + 3 * p);
    make_stencil(xp, inv_dx, &st);
    v3 nv = V3(0, 0, 0);
    m3 nC = mzero();
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          double w = st.w[0][i] * st.w[1][j] * st.w[2][k];
          v3 dpos = V3(i - st.fx[0], j - st.fx[1], k - st.fx[2]);
          v3 gv = vload(grid_v + 3 * gidx(gdim, st.base[0] + i, st.base[1] + j, st.base[2] + k));
          nv = vadd(nv, vmul(gv, w));
          nC = madd(nC, mscale(mouter(gv, dpos), w * inv_dx * 4.0));
        }
    v3 nx = vadd(xp, vmul(nv, dt));
    nx.x = fmax(fmin(nx.x, (gdim[0] - 3.0) * dx), ground_height * dx);
    nx.y = fmax(fmin(nx.y, (gdim[1] - 3.0) * dx), ground_height * dx);
    nx.z = fmax(fmin(nx.z, (gdim[2] - 3.0) * dx), ground_height * dx);
    vstore(out_x + 3 * p, nx);
    vstore(out_v + 3 * p, nv);
    mstore(out_C + 9 * p, nC);
  }
}

/* --------------------------------------------------------------- adjoint */

/* integrator.cu:1527-1614 */
void orc_g2p_grad(int n, const double *x, const double *grid_v, const int *gdim, double dx,
                  double inv_dx, double dt, const double *out_v, double ground_height,
                  double *x_grad, double *grid_v_grad, const double *out_v_grad,
                  const double *out_C_grad, const double *out_x_grad) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < n; ++p) {
    v3 xp = vload(x + 3 * p);
    v3 gx = vload(out_x_grad + 3 * p), gnv = vload(out_v_grad + 3 * p);
    m3 gC = mload(out_C_grad + 9 * p);
    v3 nx = vadd(xp, vmul(vload(out_v + 3 * p), dt));
    double lo = ground_height * dx;
    if (nx.x > (gdim[0] - 3.0) * dx || nx.x < lo) gx.x = 0;
    if (nx.y > (gdim[1] - 3.0) * dx || nx.y < lo) gx.y = 0;
    if (nx.z > (gdim[2] - 3.0) * dx || nx.z < lo) gx.z = 0;
    gnv = vadd(gnv, vmul(gx, dt));
    stencil st;
    make_stencil(xp, inv_dx, &st);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          double w = st.w[0][i] * st.w[1][j] * st.w[2][k];
          v3 dpos = V3(i - st.fx[0], j - st.fx[1], k - st.fx[2]);
          long id = gidx(gdim, st.base[0] + i, st.base[1] + j, st.base[2] + k);
          v3 gv = vload(grid_v + 3 * id);
          double xx = w * inv_dx * 4.0;
          v3 ggv = vadd(vmul(gnv, w), vmul(mvec(gC, dpos), xx));
#pragma omp atomic
          grid_v_grad[3 * id] += ggv.x;
#pragma omp atomic
          grid_v_grad[3 * id + 1] += ggv.y;
#pragma omp atomic
          grid_v_grad[3 * id + 2] += ggv.z;
          gx = vadd(gx, vmul(mvec(mT(gC), gv), -inv_dx * xx));
          double gw = vdot(gnv, gv) + inv_dx * 4.0 * msum(mhad(mouter(gv, dpos), gC));
          gx = vadd(gx, vmul(dweight(&st, i, j, k), gw));
        }
    vacc(x_grad + 3 * p, gx);
  }
}

/* integrator.cu:779-1057.  Body-pose gradients are accumulated per thread and
   reduced at the end so the result does not depend on scheduling. */
void orc_grid_op_grad(const int *gdim, const double *grid_m, const double *grid_mv,
                      const double *grid_body_v_in, const double *gravity, int nb,
                      const double *bpos, const double *brot, const double *nbpos,
                      const double *nbrot, const double *tfsr, const double *bargs,
                      double *grid_m_grad, double *grid_v_in_grad, double *bpos_grad,
                      double *brot_grad, double *nbpos_grad, double *nbrot_grad, double dx,
                      double inv_dx, double dt, double ground_friction,
                      const double *grid_v_out_grad) {
  (void)gravity; (void)inv_dx;
  long dim = (long)gdim[0] * gdim[1] * gdim[2];
#pragma omp parallel
  {
    double *acc = (double *)calloc((size_t)nb * 14, sizeof(double)); /* pos3 rot4 npos3 nrot4 */
#pragma omp for schedule(static)
    for (long t = 0; t < dim; ++t) {
      if (!(grid_m[t] > 1e-12)) continue;
      int gxi = (int)(t / gdim[2] / gdim[1]), gyi = (int)((t / gdim[2]) % gdim[1]), gzi = (int)(t % gdim[2]);
      v3 gv = vload(grid_v_out_grad + 3 * t);
      double m = grid_m[t];
      v3 mv = vload(grid_mv + 3 * t);
      v3 vv = vload(grid_body_v_in + 3 * (t * (nb + 1) + nb));
      v3 vin = vv;
      const int bound = 3;
      if (gxi > gdim[0] - bound && vv.x > 0) vin.x = 0;
      if (gxi < bound && vv.x < 0) vin.x = 0;
      double lin = 0, lit = 1;
      v3 vit = V3(0, 0, 0);
      int hit = gyi < bound && vin.y < 0;
      if (hit) {
        lin = vin.y;
        vit = V3(vin.x, 0.0, vin.z);
        lit = sqrt(vdot(vit, vit) + NORM_EPS);
        double flag = 1.0 + ground_friction * lin / lit;
        vin = vmul(vit, fmax(flag, 0.0));
      }
      if (gzi > gdim[2] - bound && vin.z > 0) gv.z = 0;
      if (gzi < bound && vin.z < 0) gv.z = 0;
      if (gyi > gdim[1] - bound && vin.y > 0) gv.y = 0;
      if (hit) {
        gv.y = 0;
        double flag = 1.0 + ground_friction * lin / lit;
        if (flag >= 0.0) {
          v3 gvit = vmul(gv, flag);
          double glin = ground_friction / lit * vdot(vit, gv);
          double glit = -ground_friction * lin / lit / lit * vdot(vit, gv);
          gvit = vadd(gvit, vmul(vit, glit / lit));
          gv = V3(gvit.x, glin, gvit.z);
        } else {
          gv = V3(0, 0, 0);
        }
      }
      if (gxi > gdim[0] - bound && vv.x > 0) gv.x = 0;
      if (gxi < bound && vv.x < 0) gv.x = 0;

      v3 gx = V3(gxi * dx, gyi * dx, gzi * dx);
      for (int b = nb - 1; b >= 0; --b) {
        v3 vo = vload(grid_body_v_in + 3 * (t * (nb + 1) + b));
        v3 bx = vload(bpos + 3 * b), nbx = vload(nbpos + 3 * b);
        qt bq = qload(brot + 4 * b), nbq = qload(nbrot + 4 * b);
        qt tf = qload(tfsr + 4 * b), ar = qload(bargs + 4 * b);
        double friction = tf.x, softness = tf.y;
        v3 gxb = xform_inv(bx, bq, gx);
        double dist = shape_sdf(tf, ar, gxb);
        double infl = fmin(exp(-dist * softness), 1.0);
        if (!((softness > 0 && infl > 0.1) || dist <= 0)) continue;
        v3 g_gxb = V3(0, 0, 0), g_bx = V3(0, 0, 0);
        qt g_bq = {0, 0, 0, 0};
        double g_infl = 0.0;
        v3 un = shape_grad(tf, ar, gxb);
        v3 rn = vnormalized(un);
        v3 nrm = qrot(bq, rn);
        v3 bv = vmul(vsub(xform(nbx, nbq, gxb), gx), 1.0 / dt);
        v3 rel = vsub(vo, bv);
        double nc = vdot(rel, nrm);
        v3 vtin = vsub(rel, vmul(nrm, fmin(nc, 0.0)));
        int fr = nc < 0 && vdot(vtin, vtin) > 1e-30;
        v3 vt = vtin;
        double vtn = vlength(vtin);
        if (fr) vt = vmul(vtin, (1.0 / vtn) * fmax(vtn + nc * friction, 0.0));
        double g_nc = 0.0;
        v3 g_bv = gv, g_rel = vmul(gv, 1 - infl), g_vt = vmul(gv, infl);
        g_infl += vdot(vsub(vt, rel), gv);
        if (fr) {
          double bf = vtn + nc * friction;
          if (bf > 0.0) {
            g_nc += vdot(vtin, g_vt) * friction / vtn;
            double g_vtn = -nc * g_nc / vtn;
            g_vt = vadd(vmul(g_vt, (1.0 / vtn) * bf), vmul(vtin, g_vtn / vtn));
          } else {
            g_vt = V3(0, 0, 0);
          }
        }
        v3 g_n = V3(0, 0, 0);
        g_rel = vadd(g_rel, g_vt);
        if (nc < 0.0) {
          g_nc += -vdot(nrm, g_vt);
          g_n = vadd(g_n, vmul(g_vt, -nc));
        }
        g_rel = vadd(g_rel, vmul(nrm, g_nc));
        g_n = vadd(g_n, vmul(rel, g_nc));
        gv = g_rel;
        g_bv = vsub(g_bv, g_rel);
        v3 g_np = V3(0, 0, 0);
        qt g_nq = {0, 0, 0, 0};
        xform_backward(nbx, nbq, gxb, vmul(g_bv, 1.0 / dt), &g_np, &g_nq, &g_gxb);
        double *A = acc + 14 * b;
        A[7] += g_np.x; A[8] += g_np.y; A[9] += g_np.z;
        A[10] += g_nq.w; A[11] += g_nq.x; A[12] += g_nq.y; A[13] += g_nq.z;
        v3 g_rn = V3(0, 0, 0);
        qmul_backward(bq, rn, g_n, &g_bq, &g_rn);
        g_gxb = vadd(g_gxb, shape_grad_backward(tf, ar, gxb, vnormalized_backward(un, g_rn)));
        double ed = exp(-dist * softness);
        if (ed <= 1) g_gxb = vadd(g_gxb, vmul(un, -softness * ed * g_infl));
        v3 g_tmp = V3(0, 0, 0);
        xform_inv_backward(bx, bq, gx, g_gxb, &g_bx, &g_bq, &g_tmp);
        A[0] += g_bx.x; A[1] += g_bx.y; A[2] += g_bx.z;
        A[3] += g_bq.w; A[4] += g_bq.x; A[5] += g_bq.y; A[6] += g_bq.z;
      }
      vacc(grid_v_in_grad + 3 * t, vmul(gv, 1.0 / m));
      grid_m_grad[t] += (-1.0 / m / m) * vdot(mv, gv);
    }
#pragma omp critical
    for (int b = 0; b < nb; ++b) {
      for (int c = 0; c < 3; ++c) bpos_grad[3 * b + c] += acc[14 * b + c];
      for (int c = 0; c < 4; ++c) brot_grad[4 * b + c] += acc[14 * b + 3 + c];
      for (int c = 0; c < 3; ++c) nbpos_grad[3 * b + c] += acc[14 * b + 7 + c];
      for (int c = 0; c < 4; ++c) nbrot_grad[4 * b + c] += acc[14 * b + 10 + c];
    }
    free(acc);
  }
}

/* integrator.cu:396-627.  Ftmp is the SVD input F_tmp (temp.F in the
   reference), Ftmp_grad its gradient (temp.F_grad). */
void orc_p2g_grad(int n, const double *x, const double *v, const double *mass,
                  const double *vol, const double *Ftmp, const double *U, const double *sig,
                  const double *V, const double *C, const double *mly, const int *gdim,
                  double dx, double inv_dx, double dt, double *x_grad, double *v_grad,
                  double *Ftmp_grad, double *C_grad, double *U_grad, double *sig_grad,
                  double *V_grad, const double *outF_grad, const double *grid_mv_grad,
                  const double *grid_m_grad) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < n; ++p) {
    m3 Um = mload(U + 9 * p), Vm = mload(V + 9 * p);
    v3 s = vload(sig + 3 * p);
    double mu = mly[3 * p], lam = mly[3 * p + 1], ys = mly[3 * p + 2];
    double J;
    m3 nF;
    v3 sn = V3(fmax(s.x, SIG_CLIP_EPS), fmax(s.y, SIG_CLIP_EPS), fmax(s.z, SIG_CLIP_EPS));
    v3 e = V3(log(sn.x), log(sn.y), log(sn.z));
    double mean = (e.x + e.y + e.z) / 3.0;
    v3 eh = V3(e.x - mean, e.y - mean, e.z - mean);
    double ehn = sqrt(vdot(eh, eh) + NORM_EPS);
    double dg = ehn - ys / (2 * mu);
    v3 ee = V3(0, 0, 0);
    if (dg > 0.0) {
      v3 ep = vsub(e, vmul(eh, dg / ehn));
      ee = V3(exp(ep.x), exp(ep.y), exp(ep.z));
      nF = mmul(mmul(Um, mdiag(ee)), mT(Vm));
      J = ee.x * ee.y * ee.z;
    } else {
      nF = mload(Ftmp + 9 * p);
      J = s.x * s.y * s.z;
    }
    m3 r = mmul(Um, mT(Vm));
    double gss = -dt * inv_dx * vol[p] * 4.0 * inv_dx;
    m3 stress = madd(mscale(mmul(msub(nF, r), mT(nF)), 2.0 * mu), meye(lam * J * (J - 1)));
    m3 affine = madd(mscale(stress, gss), mscale(mload(C + 9 * p), mass[p]));
    double mp = mass[p];
    v3 vp = vload(v + 3 * p);
    stencil st;
    make_stencil(vload(x + 3 * p), inv_dx, &st);
    m3 g_stress = mzero(), g_C = mzero();
    v3 g_x = V3(0, 0, 0), g_v = V3(0, 0, 0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          long id = gidx(gdim, st.base[0] + i, st.base[1] + j, st.base[2] + k);
          double N = st.w[0][i] * st.w[1][j] * st.w[2][k];
          v3 dpos = vmul(V3(i - st.fx[0], j - st.fx[1], k - st.fx[2]), dx);
          v3 gov = vload(grid_mv_grad + 3 * id);
          v3 gN = dweight(&st, i, j, k);
          m3 tmp = mouter(gov, dpos);
          g_stress = madd(g_stress, mscale(tmp, N * gss));
          g_C = madd(g_C, mscale(tmp, N * mp));
          double gm = grid_m_grad[id];
          g_v = vadd(g_v, vmul(gov, N * mp));
          g_x = vadd(g_x, vmul(gN, gm * mp));
          g_x = vadd(g_x, vmul(gN, vdot(vp, gov) * mp));
          g_x = vadd(g_x, vadd(vmul(mvec(mT(affine), gov), -1.0 * N), vmul(gN, vdot(mvec(affine, dpos), gov))));
        }
    vacc(x_grad + 3 * p, g_x);
    vacc(v_grad + 3 * p, g_v);
    macc(C_grad + 9 * p, g_C);
    m3 g_r = mscale(mmul(g_stress, nF), -2.0 * mu);
    m3 g_U = mmul(g_r, Vm);
    m3 g_V = mmul(mT(g_r), Um);
    m3 g_nF = madd(mload(outF_grad + 9 * p),
                   mscale(madd(mmul(mT(g_stress), msub(nF, r)), mmul(g_stress, nF)), 2.0 * mu));
    double g_J = ((2 * J - 1) * lam) * (g_stress.m[0][0] + g_stress.m[1][1] + g_stress.m[2][2]);
    v3 g_s = V3(0, 0, 0);
    m3 g_F = mzero();
    if (dg > 0.0) {
      m3 ed = mdiag(ee);
      g_U = madd(g_U, mmul(mmul(g_nF, Vm), ed));
      g_V = madd(g_V, mmul(mmul(mT(g_nF), Um), ed));
      m3 t = mmul(mmul(mT(Um), g_nF), Vm);
      v3 Fpart = V3(t.m[0][0], t.m[1][1], t.m[2][2]);
      v3 Jpart = V3(g_J * ee.y * ee.z, g_J * ee.x * ee.z, g_J * ee.x * ee.y);
      v3 g_e = vhad(ee, vadd(Jpart, Fpart));
      v3 g_eh = vmul(g_e, -dg / ehn);
      double g_ehn = -vdot(vmul(eh, 1.0 / ehn), g_e) * (ys / (2 * mu)) / ehn;
      g_eh = vadd(g_eh, vmul(eh, g_ehn / ehn));
      double sm = (g_eh.x + g_eh.y + g_eh.z) / 3.0;
      g_e = vadd(g_e, V3(g_eh.x - sm, g_eh.y - sm, g_eh.z - sm));
      if (s.x >= SIG_CLIP_EPS) g_s.x += g_e.x / s.x;
      if (s.y >= SIG_CLIP_EPS) g_s.y += g_e.y / s.y;
      if (s.z >= SIG_CLIP_EPS) g_s.z += g_e.z / s.z;
    } else {
      g_s = vadd(g_s, V3(g_J * s.y * s.z, g_J * s.x * s.z, g_J * s.x * s.y));
      g_F = madd(g_F, g_nF);
    }
    macc(U_grad + 9 * p, g_U);
    macc(V_grad + 9 * p, g_V);
    vacc(sig_grad + 3 * p, g_s);
    macc(Ftmp_grad + 9 * p, g_F);
  }
}

/* integrator.cu:102-108 */
static inline double clamp_gap(double a) {
  const double eps = 1e-6;
  return a >= 0.0 ? fmax(a, eps) : fmin(a, -eps);
}

/* integrator.cu:110-186.  Ftmp_grad (temp.F_grad) is overwritten with the full
   F_tmp gradient, as the reference does. */
void orc_compute_svd_grad(int n, const double *F, const double *C, const double *U,
                          const double *V, const double *sig, double *Ftmp_grad,
                          const double *U_grad, const double *V_grad, const double *sig_grad,
                          double *F_grad, double *C_grad, double dt) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < n; ++p) {
    m3 u = mload(U + 9 * p), v = mload(V + 9 * p), gu = mload(U_grad + 9 * p), gv = mload(V_grad + 9 * p);
    v3 s = vload(sig + 3 * p);
    m3 S = mdiag(s), gS = mdiag(vload(sig_grad + 3 * p));
    m3 vt = mT(v), ut = mT(u);
    m3 sig_term = mmul(mmul(u, gS), vt);
    double s2[3] = {s.x * s.x, s.y * s.y, s.z * s.z};
    m3 FF = mzero();
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        if (i != j) FF.m[i][j] = 1.0 / clamp_gap(s2[j] - s2[i]);
    m3 u_term = mmul(mmul(u, mmul(mhad(FF, msub(mmul(ut, gu), mmul(mT(gu), u))), S)), vt);
    m3 v_term = mmul(u, mmul(S, mmul(mhad(FF, msub(mmul(vt, gv), mmul(mT(gv), v))), vt)));
    m3 g = madd(madd(madd(mload(Ftmp_grad + 9 * p), u_term), sig_term), v_term);
    mstore(Ftmp_grad + 9 * p, g);
    m3 Fp = mload(F + 9 * p), Cp = mload(C + 9 * p);
    macc(C_grad + 9 * p, mscale(mmul(g, mT(Fp)), dt));
    macc(F_grad + 9 * p, mmul(mT(madd(meye(1.0), mscale(Cp, dt))), g));
  }
}

/* -------------------------------------------------------- loss hooks */

/* integrator.cu:188-237: signed distance of every particle to every body
   (compute_grad == 0), or its adjoint into particle x and body pose grads. */
void orc_compute_dist(int n, const double *x, int nb, const double *bpos, const double *brot,
                      const double *tfsr, const double *bargs, double *dist, int compute_grad,
                      const double *dist_grad, double *x_grad, double *bpos_grad,
                      double *brot_grad) {
  for (int p = 0; p < n; ++p) {
    for (int b = 0; b < nb; ++b) {
      v3 bx = vload(bpos + 3 * b);
      qt bq = qload(brot + 4 * b), tf = qload(tfsr + 4 * b), ar = qload(bargs + 4 * b);
      v3 gxb = xform_inv(bx, bq, vload(x + 3 * p));
      if (!compute_grad) {
        dist[(long)p * nb + b] = shape_sdf(tf, ar, gxb);
      } else {
        double gd = dist_grad[(long)p * nb + b];
        v3 g_gxb = vmul(shape_grad(tf, ar, gxb), gd);
        v3 g_bx = V3(0, 0, 0), g_x = V3(0, 0, 0);
        qt g_bq = {0, 0, 0, 0};
        xform_inv_backward(bx, bq, vload(x + 3 * p), g_gxb, &g_bx, &g_bq, &g_x);
        vacc(x_grad + 3 * p, g_x);
        vacc(bpos_grad + 3 * b, g_bx);
        brot_grad[4 * b] += g_bq.w; brot_grad[4 * b + 1] += g_bq.x;
        brot_grad[4 * b + 2] += g_bq.y; brot_grad[4 * b + 3] += g_bq.z;
      }
    }
  }
}

/* integrator.cu:239-310: per-object grid mass (compute_grad == 0) or its
   adjoint into particle x. */
void orc_particle2mass(int n, const double *x, const double *mass, const int *gdim, double dx,
                       double inv_dx, double *grid_m, const double *grid_m_grad, double *x_grad,
                       const int *ids, int id, int compute_grad) {
  (void)dx;
  for (int p = 0; p < n; ++p) {
    if (id != -1 && ids[p] != id) continue;
    stencil st;
    make_stencil(vload(x + 3 * p), inv_dx, &st);
    v3 gx = V3(0, 0, 0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          long gi = gidx(gdim, st.base[0] + i, st.base[1] + j, st.base[2] + k);
          if (compute_grad) {
            gx = vadd(gx, vmul(dweight(&st, i, j, k), grid_m_grad[gi] * mass[p]));
          } else {
            grid_m[gi] += mass[p] * st.w[0][i] * st.w[1][j] * st.w[2][k];
          }
        }
    if (compute_grad) vacc(x_grad + 3 * p, gx);
  }
}
