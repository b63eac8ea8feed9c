/* render_oracle.c -- TEST INFRASTRUCTURE ONLY: a CPU restatement of the
 * reference renderer (mpm/csrc/integrator.cu:1111-1525, mpm/csrc/array.h:7-76,
 * mpm/csrc/shape.h:33-102, quat.h) used to check the product's CUDA renderer.
 * FP32 with the reference's operation order and its few double operations;
 * compiled without multiply-add contraction.  Random numbers: the same
 * counter-based generator as the product and as the reference host build's
 * curand shim (SplitMix64 of (seed, pixel), then of key + draw * golden),
 * consumed in the order the reference host build draws them.
 * Host pointers; vec3 = float[3], quat = float[4] (w, x, y, z), mat3 = float[9]
 * row-major. */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct {
  float x, y, z;
} v3;
typedef struct {
  float w, x, y, z;
} q4;

static v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 scl(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static v3 hmul(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 cross3(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static float len3(v3 a) { return (float)sqrt((double)dot3(a, a) + 1e-30); } /* shape.h:7-9 */
static v3 nrm3(v3 a) { float l = len3(a); return mk(a.x / l, a.y / l, a.z / l); }
/* quat.h:14-19 */
static v3 qrot(q4 q, v3 v) {
  v3 qv = mk(q.x, q.y, q.z), uv = cross3(qv, v), uuv = cross3(qv, uv);
  return add(v, scl(add(scl(uv, q.w), uuv), 2.f));
}
static v3 xinv(v3 p, q4 q, v3 pt) { q4 qi = {q.w, -q.x, -q.y, -q.z}; return qrot(qi, sub(pt, p)); }

/* shape.h:33-102 */
static int shape_type(q4 t) { return (int)floorf(t.w + 0.1f); }
static float shape_sdf(q4 t, q4 a, v3 g) {
  int type = shape_type(t);
  float sdf = 0.f;
  if (type == 0) {
    v3 q = sub(mk(fabsf(g.x), fabsf(g.y), fabsf(g.z)), mk(a.w, a.x, a.y));
    sdf = len3(mk(q.x > 0.f ? q.x : 0.f, q.y > 0.f ? q.y : 0.f, q.z > 0.f ? q.z : 0.f)) +
          fminf(fmaxf(fmaxf(q.x, q.y), q.z), 0.f);
  } else if (type == 1) {
    v3 p2 = g;
    float r = a.w, h = a.x;
    p2.y += h / 2;
    p2.y -= fminf(fmaxf(p2.y, 0.f), h);
    sdf = len3(p2) - r;
  }
  return sdf - t.z;
}
static v3 shape_grad(q4 t, q4 a, v3 g) {
  int type = shape_type(t);
  v3 grad = mk(0.f, 0.f, 0.f);
  if (type == 0) {
    v3 q = sub(mk(fabsf(g.x), fabsf(g.y), fabsf(g.z)), mk(a.w, a.x, a.y));
    float inside = fmaxf(fmaxf(q.x, q.y), q.z);
    if (inside <= 0) {
      if (q.x == inside) grad.x += 1;
      if (q.y == inside) grad.y += 1;
      if (q.z == inside) grad.z += 1;
    } else {
      grad = nrm3(mk(q.x > 0.f ? q.x : 0.f, q.y > 0.f ? q.y : 0.f, q.z > 0.f ? q.z : 0.f));
    }
    if (g.x < 0) grad.x *= -1;
    if (g.y < 0) grad.y *= -1;
    if (g.z < 0) grad.z *= -1;
  } else if (type == 1) {
    v3 p2 = g;
    float h = a.x;
    p2.y += h / 2;
    p2.y -= fminf(fmaxf(p2.y, 0.f), h);
    return nrm3(p2);
  }
  return grad;
}

/* ------------------------------------------------------------------ RNG */
static uint64_t smx(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
typedef struct {
  uint64_t key, ctr;
} rng_t;
static float uni(rng_t *r) {
  ++r->ctr;
  return (float)((smx(r->key + r->ctr * 0x9E3779B97F4A7C15ull) >> 40) + 1ull) * (1.f / 16777216.f);
}

/* --------------------------------------------------------------- volume */
typedef struct {
  const float *sdf, *color;
  v3 lo, hi;
  int d[3];
  float thr;
} vol_t;

/* array.h:7-50 */
static int vquery(const vol_t *V, const float *values, int C, v3 point, float *out) {
  v3 ratio = mk((point.x - V->lo.x) / (V->hi.x - V->lo.x), (point.y - V->lo.y) / (V->hi.y - V->lo.y),
                (point.z - V->lo.z) / (V->hi.z - V->lo.z));
  if (!(ratio.x >= 0 && ratio.y >= 0 && ratio.z >= 0 && ratio.x < 1. && ratio.y < 1. && ratio.z < 1.)) return 0;
  v3 g = mk(ratio.x * (float)V->d[0], ratio.y * (float)V->d[1], ratio.z * (float)V->d[2]);
  int x0 = (int)floor(g.x), y0 = (int)floor(g.y), z0 = (int)floor(g.z);
  x0 = x0 < 0 ? 0 : (x0 > V->d[0] - 1 ? V->d[0] - 1 : x0);
  y0 = y0 < 0 ? 0 : (y0 > V->d[1] - 1 ? V->d[1] - 1 : y0);
  z0 = z0 < 0 ? 0 : (z0 > V->d[2] - 1 ? V->d[2] - 1 : z0);
  float dx = g.x - (float)x0, dy = g.y - (float)y0, dz = g.z - (float)z0;
  int i000 = (x0 * V->d[1] + y0) * V->d[2] + z0;
  int fz = z0 + 1 < V->d[2], fy = y0 + 1 < V->d[1], fx = x0 + 1 < V->d[0];
  int i001 = i000 + fz, i010 = i000 + V->d[2] * fy, i011 = i010 + fz;
  int i100 = i000 + V->d[1] * V->d[2] * fx, i101 = i100 + fz, i110 = i100 + V->d[2] * fy, i111 = i110 + fz;
  for (int c = 0; c < C; ++c) {
    float v000 = values[C * i000 + c] * (1 - dx) * (1 - dy) * (1 - dz);
    float v001 = values[C * i001 + c] * (1 - dx) * (1 - dy) * dz;
    float v010 = values[C * i010 + c] * (1 - dx) * dy * (1 - dz);
    float v011 = values[C * i011 + c] * (1 - dx) * dy * dz;
    float v100 = values[C * i100 + c] * dx * (1 - dy) * (1 - dz);
    float v101 = values[C * i101 + c] * dx * (1 - dy) * dz;
    float v110 = values[C * i110 + c] * dx * dy * (1 - dz);
    float v111 = values[C * i111 + c] * dx * dy * dz;
    out[c] = v000 + v001 + v010 + v011 + v100 + v101 + v110 + v111;
  }
  return 1;
}
static float ssdf(const vol_t *V, v3 p, float thr) {
  float o = 0.f;
  if (vquery(V, V->sdf, 1, p, &o)) o -= thr;
  return o;
}
static v3 snormal(const vol_t *V, v3 p) {
  float e = 1e-3f;
  float x0 = ssdf(V, add(p, mk(-e, 0.f, 0.f)), 0.f), x1 = ssdf(V, add(p, mk(e, 0.f, 0.f)), 0.f);
  float y0 = ssdf(V, add(p, mk(0.f, -e, 0.f)), 0.f), y1 = ssdf(V, add(p, mk(0.f, e, 0.f)), 0.f);
  float z0 = ssdf(V, add(p, mk(0.f, 0.f, -e)), 0.f), z1 = ssdf(V, add(p, mk(0.f, 0.f, e)), 0.f);
  return scl(mk(x1 - x0, y1 - y0, z1 - z0), (float)(0.5 / (double)e));
}

/* integrator.cu:1111-1140 */
static int ray_box(v3 lo, v3 hi, v3 o, v3 d, float *tn, float *tf) {
  float dd[3] = {d.x, d.y, d.z}, oo[3] = {o.x, o.y, o.z}, l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
  *tn = -1e9f;
  *tf = 1e9f;
  for (int i = 0; i < 3; ++i) {
    if (dd[i] == 0) {
      if (oo[i] < l[i] || oo[i] > h[i]) return 0;
    } else {
      float a = (l[i] - oo[i]) / dd[i], b = (h[i] - oo[i]) / dd[i];
      float nf = a < b ? b : a, nn = b < a ? b : a;
      *tf = nf < *tf ? nf : *tf;
      *tn = *tn < nn ? nn : *tn;
    }
  }
  return !(*tn > *tf);
}

typedef struct {
  vol_t V;
  const float *pos, *rot, *tfsr, *args;
  int nb, vis;
  float ground;
} scene_t;

static q4 ldq(const float *a, int i) { q4 q = {a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3]}; return q; }
static v3 ldv(const float *a, int i) { return mk(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }

/* integrator.cu:1142-1285 */
static float next_hit(const scene_t *S, v3 o, v3 d, v3 *color, v3 *normal) {
  float closest = 1e9f;
  if (d.y < 0) {
    float gd = (o.y - S->ground) / (-d.y);
    if (gd < 100.f && gd < closest) {
      closest = gd;
      *normal = mk(0.f, 1.f, 0.f);
      v3 c = mk(0.3f, 0.5f, 0.7f);
      v3 p = add(o, scl(d, closest));
      if (p.x <= 1 && p.x >= 0 && p.z <= 1 && p.z >= 0)
        c = scl(c, (float)((double)((((int)(p.x / 0.25) + (int)(p.z / 0.25)) % 2)) * 0.2 + 0.35));
      else
        c = scl(c, 0.4f);
      *color = c;
    }
  }
  if (S->nb > 0) {
    int j = 0, id = 0;
    float dist = 0.f, sv = 1e9f;
    v3 pp = o;
    while (j < 200 && dist < 100.f && sv > 1e-8) {
      pp = add(o, scl(d, dist));
      sv = 1e9f;
      for (int i = 0; i < S->nb; ++i) {
        float t = shape_sdf(ldq(S->tfsr, i), ldq(S->args, i), xinv(ldv(S->pos, i), ldq(S->rot, i), pp));
        if (t < sv) {
          sv = t;
          id = i;
        }
      }
      dist += sv;
      j += 1;
    }
    if (dist < closest && dist < 100.f) {
      closest = dist;
      v3 gb = xinv(ldv(S->pos, id), ldq(S->rot, id), pp);
      *normal = qrot(ldq(S->rot, id), nrm3(shape_grad(ldq(S->tfsr, id), ldq(S->args, id), gb)));
      *color = mk(0.5f, 0.5f, 0.5f);
    }
  }
  float tn = 0.f, tf = 0.f;
  if (S->vis && ray_box(S->V.lo, S->V.hi, o, d, &tn, &tf)) {
    tn = (double)tn > 0. ? tn : 0.f;
    v3 pos = add(o, scl(d, (float)((double)tn + 1e-4)));
    v3 step = mk(0.f, 0.f, 0.f);
    for (int j = 0; j < 500; ++j) {
      float s = ssdf(&S->V, pos, S->V.thr);
      if (s < 0) {
        v3 back = step;
        for (int k = 0; k < 20; ++k) {
          back = scl(back, 0.5f);
          if (ssdf(&S->V, sub(pos, back), S->V.thr) < 0) pos = sub(pos, back);
        }
        v3 od = sub(o, pos);
        float dist = (float)sqrt((double)dot3(od, od));
        if (dist < closest) {
          closest = dist;
          *normal = nrm3(snormal(&S->V, pos));
          float c[3] = {0.f, 0.f, 0.f};
          vquery(&S->V, S->V.color, 3, pos, c);
          *color = mk(c[0], c[1], c[2]);
        }
        break;
      } else {
        double m = (double)s * 0.05;
        step = scl(d, (float)(m > 0.01 ? m : 0.01));
        pos = add(pos, step);
      }
    }
  }
  return closest;
}

static v3 mat_vec(const float *m, v3 v) {
  /* mat3.h:95-98: col(0) b.x + col(1) b.y + col(2) b.z */
  v3 c0 = mk(m[0], m[3], m[6]), c1 = mk(m[1], m[4], m[7]), c2 = mk(m[2], m[5], m[8]);
  return add(add(scl(c0, v.x), scl(c1, v.y)), scl(c2, v.z));
}

/* integrator.cu:1287-1436 (use_directional_light = 1, light noise 0.1) */
void orc_render(const float *sdf, const float *box_min, const float *box_max, const float *color_vol,
                const float *body_pos, const float *body_rot, const float *body_tfsr, const float *body_args,
                const float *cam_rot, const float *cam_pos, const float *cam_intr, float *color_buf, float *depth_buf,
                float thr, const int *gdim, int nb, int vis, const int *image_dim, int max_depth, int spp,
                float ground, int seed, const float *light) {
  scene_t S;
  S.V.sdf = sdf;
  S.V.color = color_vol;
  S.V.lo = ldv(box_min, 0);
  S.V.hi = ldv(box_max, 0);
  S.V.d[0] = gdim[0];
  S.V.d[1] = gdim[1];
  S.V.d[2] = gdim[2];
  S.V.thr = thr;
  S.pos = body_pos;
  S.rot = body_rot;
  S.tfsr = body_tfsr;
  S.args = body_args;
  S.nb = nb;
  S.vis = vis;
  S.ground = ground;
  const int H = image_dim[0], W = image_dim[1], dim = H * W;
  const v3 cpos = ldv(cam_pos, 0), ldir = ldv(light, 0);
#pragma omp parallel for schedule(dynamic, 64)
  for (int p = 0; p < dim; ++p) {
    rng_t r = {smx(((uint64_t)(uint32_t)seed << 32) ^ (uint64_t)(uint32_t)p), 0};
    int u = p % W, v = p / W;
    v3 cb = mk(0.f, 0.f, 0.f);
    float db = 0.f;
    for (int sample = 0; sample < spp; ++sample) {
      float jy = uni(&r);
      float jx = uni(&r);
      v3 dir = mat_vec(cam_intr, mk(u + jx, v + jy, 1.f));
      v3 d = mat_vec(cam_rot, nrm3(dir));
      v3 contrib = mk(0.f, 0.f, 0.f), through = mk(1.f, 1.f, 1.f);
      int depth = 0;
      float first = 0.f;
      v3 pos = cpos;
      while (depth < max_depth) {
        v3 normal = mk(0.f, 0.f, 0.f), color = mk(0.f, 0.f, 0.f);
        float closest = next_hit(&S, pos, d, &color, &normal);
        if (depth == 0) first = closest;
        v3 hit = add(pos, scl(d, closest));
        depth += 1;
        if (dot3(normal, normal) > 1e-10) {
          v3 t1 = mk(1.f, 0.f, 0.f);
          if (fabsf(normal.y) < 1 - 1e-3) t1 = nrm3(cross3(normal, mk(0.f, 1.f, 0.f)));
          v3 t2 = cross3(normal, t1);
          float phi = (float)(2 * M_PI * (double)uni(&r));
          float rr = uni(&r);
          float ay = (float)sqrt((double)rr), ax = (float)sqrt((double)(1 - rr));
          float cph = (float)cos((double)phi), sph = (float)sin((double)phi);
          v3 out = add(scl(add(scl(t1, cph), scl(t2, sph)), ax), scl(normal, ay));
          d = nrm3(out);
          pos = add(hit, scl(d, 1e-4f));
          through = hmul(through, color);
          float nz = (float)((double)uni(&r) - 0.5), ny = (float)((double)uni(&r) - 0.5),
                nx = (float)((double)uni(&r) - 0.5);
          v3 direct = nrm3(add(ldir, scl(mk(nx, ny, nz), 0.1f)));
          float cosl = dot3(direct, normal);
          if (cosl > 0) {
            v3 c2, n2;
            if (next_hit(&S, pos, direct, &c2, &n2) > 100.f) contrib = add(contrib, hmul(scl(through, cosl), mk(0.8f, 0.8f, 0.8f)));
          }
        } else {
          break;
        }
      }
      contrib = add(contrib, hmul(through, mk(0.8f, 0.8f, 0.8f)));
      cb = add(cb, mk(contrib.x / spp, contrib.y / spp, contrib.z / spp));
      db += first / spp;
    }
    float uu = (float)(1.0 * u / W), vv = (float)(1.0 * v / H);
    float r2 = (uu - 0.5f) * (uu - 0.5f) + (vv - 0.5f) * (vv - 0.5f);
    double rad = sqrt((double)r2) - 0.0;
    float darken = (float)(1.0 - (double)0.9f * (rad > 0. ? rad : 0.));
    v3 c = scl(scl(cb, darken), 1.5f);
    color_buf[3 * p] = (float)sqrt((double)c.x);
    color_buf[3 * p + 1] = (float)sqrt((double)c.y);
    color_buf[3 * p + 2] = (float)sqrt((double)c.z);
    depth_buf[p] = db;
  }
}

/* integrator.cu:1911-1933 with :1438-1523 (bake, copy, two smooth passes) */
void orc_particle_sdf(long long *volume, const float *x, const int *color, const float *bbox_min, int bake,
                      const int *gdim, float inv_dx, float *sdf, float *colv, float *sdf_tmp, int n) {
  const int gx = gdim[0], gy = gdim[1], gz = gdim[2], width = 2 * bake;
  const v3 lo = ldv(bbox_min, 0);
  for (int p = 0; p < n; ++p) {
    v3 xp = scl(sub(ldv(x, p), lo), inv_dx);
    int cx = (int)floor(xp.x), cy = (int)floor(xp.y), cz = (int)floor(xp.z);
    for (int i = 0; i < width; ++i)
      for (int j = 0; j < width; ++j)
        for (int k = 0; k < width; ++k) {
          int ix = cx + i - bake, iy = cy + j - bake, iz = cz + k - bake;
          if (ix < 0 || iy < 0 || iz < 0 || ix >= gx || iy >= gy || iz >= gz) continue;
          v3 e = sub(mk((float)ix, (float)iy, (float)iz), xp);
          float dist = sqrtf(dot3(e, e) + 0.f);
          float q = 255.0f * 0.2f * dist;
          q = q > 0.f ? q : 0.f;
          q = q < 255.f ? q : 255.f;
          long long out = ((long long)q << 24) + (long long)color[p];
          long long *cell = volume + ((long long)ix * gy + iy) * gz + iz;
          if (out < *cell) *cell = out;
        }
  }
  const int nv = gx * gy * gz;
  for (int t = 0; t < nv; ++t) {
    long long c = volume[t];
    float z = (float)((double)(c & 255) / 255.);
    c >>= 8;
    float y = (float)((double)(c & 255) / 255.);
    c >>= 8;
    float xx = (float)((double)(c & 255) / 255.);
    c >>= 8;
    colv[3 * t] = xx;
    colv[3 * t + 1] = y;
    colv[3 * t + 2] = z;
    sdf[t] = (float)((double)(c & 255) / 255.);
  }
  for (int pass = 0; pass < 2; ++pass) {
    const float *in = pass == 0 ? sdf : sdf_tmp;
    float *out = pass == 0 ? sdf_tmp : sdf;
    for (int t = 0; t < nv; ++t) {
      int x0 = t / gz / gy, y0 = (t / gz) % gy, z0 = t % gz;
      if (x0 >= 1 && y0 >= 1 && z0 >= 1 && x0 < gx - 1 && y0 < gy - 1 && z0 < gz - 1) {
        float sum = 0.f;
        for (int i = -1; i < 2; ++i)
          for (int j = -1; j < 2; ++j)
            for (int k = -1; k < 2; ++k) sum += in[((x0 + i) * gy + (y0 + j)) * gz + (z0 + k)];
        out[t] = (float)((double)sum / 27.);
      } else {
        out[t] = 1.f;
      }
    }
  }
}
