/*
 * vh_oracle.c -- CPU restatement of the voxelhashmt depth-fusion path.
 *
 * TEST INFRASTRUCTURE ONLY (parity oracle and CPU timing baseline); the CUDA
 * product never links it.  Every function cites the reference lines it follows.
 * Paths are relative to the reference project root.  Build with
 * -ffp-contract=off and without fast-math (oracle/build.py).
 *
 * Arithmetic type.  Built as is, `real` is float: every operation is rounded as the reference's float code
 * rounds it, and the results are bit-identical to the reference (the pinned restatement).  Built with
 * -DVO_FP64, `real` is double and the math functions are the double ones: the same equations in FP64
 * arithmetic (the FP64 transcription).  Its inputs and stored data stay the reference's float data: depth,
 * intrinsics, pose and its float inverse, the float constants, the filtered depth image and the voxel
 * records, which are rounded to float when stored, as the reference stores them.  The exponential is libm's
 * double exp in that build.
 */
#define _GNU_SOURCE
#include "vh_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifdef VO_FP64
typedef double real;
#define VO_FLOOR floor
#define VO_FABS fabs
#define VO_SQRT sqrt
#define VO_LROUND lround
#define VO_FMIN fmin
#define VO_FMAX fmax
#else
typedef float real;
#define VO_FLOOR floorf
#define VO_FABS fabsf
#define VO_SQRT sqrtf
#define VO_LROUND lroundf
#define VO_FMIN fminf
#define VO_FMAX fmaxf
#endif

#define GPU VO_FLAVOR_REF_GPU
#define CPU VO_FLAVOR_REF_CPU
#define BLOCK 8
#define BLOCK_VOLUME 512
#define DIRS 6
#define LAYERS 3

/* ------------------------------------------------------------------ vectors */
/* math_types.h:44-101, cuda_tsdf_integrator.cu:181-217 */
typedef struct {
  real x, y, z;
} v3;

static inline v3 mk(real x, real y, real z) {
  v3 r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
static inline v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vmul(v3 v, real s) { return mk(v.x * s, v.y * s, v.z * s); }
static inline v3 vdivs(v3 v, real s) { return mk(v.x / s, v.y / s, v.z / s); }
static inline real vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline real vnorm(v3 v) { return VO_SQRT(vdot(v, v)); }

/* GPU: cuda_tsdf_integrator.cu:201-209 and cuda_block_allocator.cu:127-135 (<=1e-6, multiply by 1/len);
 * CPU: math_types.h:95-101 (<=1e-8, divide by len). */
static inline v3 vnormalize(int fl, v3 v) {
  const real len = vnorm(v);
  if (fl == GPU) {
    if (len <= 1e-6f) return mk(0.0f, 0.0f, 0.0f);
    const real inv = 1.0f / len;
    return mk(v.x * inv, v.y * inv, v.z * inv);
  }
  if (len <= 1e-8f) return mk(0.0f, 0.0f, 0.0f);
  return vdivs(v, len);
}

/* CPU std::max/std::min (a<b?b:a) vs GPU fmaxf/fminf: equal for the finite non-NaN values used here. */
static inline real fmax_f(real a, real b) { return (a < b) ? b : a; }
static inline real fmin_f(real a, real b) { return (b < a) ? b : a; }
static inline real clamp_f(real v, real lo, real hi) { return fmax_f(lo, fmin_f(hi, v)); }

/* math_types.h:180-198 / cuda_tsdf_integrator.cu:452-466 */
static inline v3 pose_point(const vo_pose* P, v3 p) {
  return mk(P->R[0] * p.x + P->R[1] * p.y + P->R[2] * p.z + P->t[0],
            P->R[3] * p.x + P->R[4] * p.y + P->R[5] * p.z + P->t[1],
            P->R[6] * p.x + P->R[7] * p.y + P->R[8] * p.z + P->t[2]);
}
static inline v3 pose_vector(const vo_pose* P, v3 p) {
  return mk(P->R[0] * p.x + P->R[1] * p.y + P->R[2] * p.z, P->R[3] * p.x + P->R[4] * p.y + P->R[5] * p.z,
            P->R[6] * p.x + P->R[7] * p.y + P->R[8] * p.z);
}
/* Pose::inverse, math_types.h:192-197: R' = R^T, t' = R' * (t * -1) */
static void pose_inverse(const vo_pose* P, vo_pose* out) {
  const float* R = P->R;
  const real Rt[9] = {R[0], R[3], R[6], R[1], R[4], R[7], R[2], R[5], R[8]};
  const real nt[3] = {P->t[0] * -1.0f, P->t[1] * -1.0f, P->t[2] * -1.0f};
  for (int i = 0; i < 9; ++i) out->R[i] = (float)Rt[i];
  out->t[0] = Rt[0] * nt[0] + Rt[1] * nt[1] + Rt[2] * nt[2];
  out->t[1] = Rt[3] * nt[0] + Rt[4] * nt[1] + Rt[5] * nt[2];
  out->t[2] = Rt[6] * nt[0] + Rt[7] * nt[1] + Rt[8] * nt[2];
}

/* math_types.h:228-232, cuda_block_allocator.cu:145-151 */
static inline v3 back_project(int u, int v, real d, const vo_intrinsics* K) {
  return mk(((real)u - K->cx) * d / K->fx, ((real)v - K->cy) * d / K->fy, d);
}
/* voxel_hash_tsdf.h:586-593, cuda_tsdf_integrator.cu:570-579 */
static inline v3 back_project_cont(real u, real v, real d, const vo_intrinsics* K) {
  return mk((u - K->cx) * d / K->fx, (v - K->cy) * d / K->fy, d);
}
/* math_types.h:234-244, cuda_tsdf_integrator.cu:468-477 */
static inline int project_point(v3 pc, const vo_intrinsics* K, real* u, real* v) {
  if (pc.z <= 1e-6f) return 0;
  *u = K->fx * pc.x / pc.z + K->cx;
  *v = K->fy * pc.y / pc.z + K->cy;
  return *u >= 0.0f && *u <= (real)(K->width - 1) && *v >= 0.0f && *v <= (real)(K->height - 1);
}

/* ---------------------------------------------------------------------- exp */
/* The C library's single-precision exp, restated.  The reference's Gaussian weights call expf
 * (cuda_tsdf_integrator.cu:173-175, voxel_hash_tsdf.h:552-554); compiled for a host, that resolves to the GNU C
 * library's expf, which since glibc 2.28 is the table-driven algorithm published in ARM's optimized-routines
 * (N = 32): z = x * N/ln2 and k = z rounded to the nearest integer in double, r = fma(N/ln2, x, -k),
 * y = 2^(k/N) * (1 + C2 r + C1 r^2 + C0 r^3) in double with 2^(j/N) from a table, result (float) y.
 * Pinned against glibc 2.39 (x86_64, the host the reference was compiled on): equal for every float argument
 * (vo_expf_compare_libm, tests/test_oracle_cpu.py).  The CUDA product evaluates the same function on the
 * device (vh_expf), so the product is compared bit-for-bit with both VO_EXP_OWN and VO_EXP_LIBM. */
static const uint64_t k_exp2_tab[32] = {
    /* bits of the double nearest 2^(j/32) minus (j << 47): adding k << 47 scales by 2^floor(k/32) */
    0x3ff0000000000000ULL, 0x3fefd9b0d3158574ULL, 0x3fefb5586cf9890fULL, 0x3fef9301d0125b51ULL,
    0x3fef72b83c7d517bULL, 0x3fef54873168b9aaULL, 0x3fef387a6e756238ULL, 0x3fef1e9df51fdee1ULL,
    0x3fef06fe0a31b715ULL, 0x3feef1a7373aa9cbULL, 0x3feedea64c123422ULL, 0x3feece086061892dULL,
    0x3feebfdad5362a27ULL, 0x3feeb42b569d4f82ULL, 0x3feeab07dd485429ULL, 0x3feea47eb03a5585ULL,
    0x3feea09e667f3bcdULL, 0x3fee9f75e8ec5f74ULL, 0x3feea11473eb0187ULL, 0x3feea589994cce13ULL,
    0x3feeace5422aa0dbULL, 0x3feeb737b0cdc5e5ULL, 0x3feec49182a3f090ULL, 0x3feed503b23e255dULL,
    0x3feee89f995ad3adULL, 0x3feeff76f2fb5e47ULL, 0x3fef199bdd85529cULL, 0x3fef3720dcef9069ULL,
    0x3fef5818dcfba487ULL, 0x3fef7c97337b9b5fULL, 0x3fefa4afa2a490daULL, 0x3fefd0765b6e4540ULL};

float vo_expf_own(float x) {
  static const double inv_ln2_n = 0x1.71547652b82fep+0 * 32.0, shift = 0x1.8p+52;
  static const double c0 = 0x1.c6af84b912394p-20, c1 = 0x1.ebfce50fac4f3p-13, c2 = 0x1.62e42ff0c52d6p-6;
  if (x != x) return x + x;
  if (x < -0x1.9fe368p6f) return 0.0f;        /* below log(2^-150) */
  if (x > 0x1.62e42ep6f) return INFINITY;     /* above log(2^128) */
  union {
    double d;
    uint64_t u;
  } kd, s;
  const double xd = (double)x;
  const double z = inv_ln2_n * xd;
  kd.d = z + shift;
  const uint64_t ki = kd.u;
  const double k = kd.d - shift;
  const double r = fma(inv_ln2_n, xd, -k);
  s.u = k_exp2_tab[ki % 32] + (ki << 47);
  const double p = fma(c0, r, c1);
  const double r2 = r * r;
  double y = fma(c2, r, 1.0);
  y = fma(p, r2, y);
  y = y * s.d;
  return (float)y;
}

/* Element-wise vo_expf_own (test helper). */
void vo_expf_array(const float* x, float* y, size_t n) {
  for (size_t i = 0; i < n; ++i) y[i] = vo_expf_own(x[i]);
}

/* Compares vo_expf_own with the C library's expf on every float whose bit pattern lies in [first, first + count),
 * NaNs excluded, on `threads` threads: the number of differing results and the smallest differing pattern
 * (0xffffffff if none). */
typedef struct {
  uint64_t first, count, stride, offset, bad;
  uint32_t first_bad;
} cmp_slice;
static void* cmp_worker(void* arg) {
  cmp_slice* S = (cmp_slice*)arg;
  S->bad = 0;
  S->first_bad = 0xffffffffU;
  for (uint64_t i = S->offset; i < S->count; i += S->stride) {
    union {
      uint32_t u;
      float f;
    } x, a, b;
    x.u = (uint32_t)(S->first + i);
    if (x.f != x.f) continue;
    a.f = vo_expf_own(x.f);
    b.f = expf(x.f);
    if (a.u != b.u) {
      ++S->bad;
      if (x.u < S->first_bad) S->first_bad = x.u;
    }
  }
  return NULL;
}
void vo_expf_compare_libm(uint32_t first, uint64_t count, int threads, uint64_t* mismatches, uint32_t* first_mismatch) {
  cmp_slice S[256];
  pthread_t tid[256];
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  int started = 0;
  for (int t = 0; t < threads; ++t) {
    S[t].first = first;
    S[t].count = count;
    S[t].stride = (uint64_t)threads;
    S[t].offset = (uint64_t)t;
  }
  for (int t = 0; t < threads; ++t) {
    if (pthread_create(&tid[t], NULL, cmp_worker, &S[t]) != 0) break;
    ++started;
  }
  /* slices whose thread did not start run here */
  for (int t = started; t < threads; ++t) cmp_worker(&S[t]);
  for (int t = 0; t < started; ++t) pthread_join(tid[t], NULL);
  *mismatches = 0;
  *first_mismatch = 0xffffffffU;
  for (int t = 0; t < threads; ++t) {
    *mismatches += S[t].bad;
    if (S[t].first_bad < *first_mismatch) *first_mismatch = S[t].first_bad;
  }
}

static inline real vo_exp(const vo_config* c, real x) {
#ifdef VO_FP64
  (void)c;
  return exp(x);
#else
  return c->exp_impl == VO_EXP_OWN ? vo_expf_own(x) : expf(x);
#endif
}
/* voxel_hash_tsdf.h:552-554, cuda_tsdf_integrator.cu:173-175 */
static inline real gaussian(const vo_config* c, real sq, real inv_two_sigma_sq) {
  return vo_exp(c, -sq * inv_two_sigma_sq);
}
static inline real inv_two_sigma_sq(real s) { return 1.0f / (2.0f * s * s); }

/* ------------------------------------------------------------------- config */
void vo_config_default(vo_config* c, int32_t flavor) {
  memset(c, 0, sizeof(*c));
  c->flavor = flavor;
  c->exp_impl = VO_EXP_LIBM;
  c->filter_radius = 2;                /* cuda_tsdf_integrator.cu:31, reconstruction_backend.cpp:26 */
  c->filter_sigma_spatial = 1.5f;      /* :32 / :27 */
  c->filter_sigma_range = 0.0012f;     /* :33 / :28 */
  c->filter_sigma_angular = 0.35f;     /* :34 / :29 */
  c->normal_radius = 1;                /* cuda_tsdf_integrator.cu:23, voxel_hash_tsdf.h:196 */
  c->normal_sigma_spatial = 1.0f;      /* :24 / :197 */
  c->normal_sigma_range = 0.0012f;     /* :25 / :198 */
  c->normal_sigma_angular = 0.35f;     /* :26 / :199 */
  c->layer_merge_scale = 0.25f;        /* :29 / :202 */
  c->layer_extract_scale = 0.55f;      /* cuda_mesh_extractor.cu:20, voxel_hash_tsdf.h:203 */
  c->max_weight = 100.0f;              /* cuda_tsdf_integrator.cu:18, voxel_hash_tsdf.h:194 */
  c->depth_sigma = 1.5f;               /* :19 / :565 */
  c->huber_delta = 0.35f;              /* :20 / :571 */
  c->min_obs_weight = 0.05f;           /* :21 / :580 */
  c->min_view_weight = 0.15f;          /* :22 / :195 */
  c->threads = 1;
  if (flavor == GPU) {
    c->disc_base = 0.012f;             /* cuda_tsdf_integrator.cu:27 */
    c->disc_rel = 0.025f;              /* :28 */
    c->filter_min_cos = 0.9f;          /* :35 */
    c->layer_normal_cos = 0.9f;        /* :30 */
  } else {
    c->disc_base = 0.0012f;            /* reconstruction_backend.cpp:30, voxel_hash_tsdf.h:200 */
    c->disc_rel = 0.0025f;             /* :31 / :201 */
    c->filter_min_cos = 0.6f;          /* reconstruction_backend.cpp:32 */
    c->layer_normal_cos = 0.75f;       /* voxel_hash_tsdf.h:204 */
  }
}

/* -------------------------------------------------------------- parallel for */
typedef void (*pf_fn)(void* ctx, int64_t i);
typedef struct {
  pf_fn fn;
  void* ctx;
  int64_t n;
  int64_t next;
} pf_state;

static void* pf_worker(void* arg) {
  pf_state* s = (pf_state*)arg;
  for (;;) {
    const int64_t i = __atomic_fetch_add(&s->next, 1, __ATOMIC_RELAXED);
    if (i >= s->n) break;
    s->fn(s->ctx, i);
  }
  return NULL;
}

static void parallel_for(int threads, int64_t n, pf_fn fn, void* ctx) {
  if (threads <= 1 || n <= 1) {
    for (int64_t i = 0; i < n; ++i) fn(ctx, i);
    return;
  }
  if (threads > 256) threads = 256;
  if ((int64_t)threads > n) threads = (int)n;
  pf_state s = {fn, ctx, n, 0};
  pthread_t tid[256];
  int started = 0;
  for (int t = 1; t < threads; ++t) {
    if (pthread_create(&tid[started], NULL, pf_worker, &s) == 0) ++started;
  }
  pf_worker(&s);
  for (int t = 0; t < started; ++t) pthread_join(tid[t], NULL);
}

/* ----------------------------------------------------------- depth helpers */
/* cuda_tsdf_integrator.cu:177-179, voxel_hash_tsdf.h:226-228, reconstruction_backend.cpp:38-40 */
static inline real disc_threshold(const vo_config* c, real ref) {
  return fmax_f(c->disc_base, c->disc_rel * fmax_f(ref, 0.0f));
}

/* cuda_tsdf_integrator.cu:219-226, voxel_hash_tsdf.h:230-237 */
static inline v3 orient_toward_camera(int fl, v3 n, v3 pc) {
  if (vnorm(n) <= 1e-6f || vnorm(pc) <= 1e-6f) return n;
  const v3 view = vnormalize(fl, pc);
  return vdot(n, view) > 0.0f ? vmul(n, -1.0f) : n;
}

/* cuda_tsdf_integrator.cu:581-627, reconstruction_backend.cpp:57-94 */
static int pixel_normal(const vo_config* c, const float* depth, const vo_intrinsics* K, int u, int v, v3* normal) {
  const int W = K->width, H = K->height;
  if (u <= 0 || v <= 0 || u + 1 >= W || v + 1 >= H) return 0;
  const real dc = depth[(size_t)v * W + u];
  const real dl = depth[(size_t)v * W + u - 1];
  const real dr = depth[(size_t)v * W + u + 1];
  const real du = depth[(size_t)(v - 1) * W + u];
  const real dd = depth[(size_t)(v + 1) * W + u];
  if (!(dc > 0.0f) || !(dl > 0.0f) || !(dr > 0.0f) || !(du > 0.0f) || !(dd > 0.0f)) return 0;
  const real thr = disc_threshold(c, dc);
  if (VO_FABS(dl - dc) > thr || VO_FABS(dr - dc) > thr || VO_FABS(du - dc) > thr || VO_FABS(dd - dc) > thr) return 0;
  const v3 pl = back_project_cont((real)(u - 1), (real)v, dl, K);
  const v3 pr = back_project_cont((real)(u + 1), (real)v, dr, K);
  const v3 pu = back_project_cont((real)u, (real)(v - 1), du, K);
  const v3 pd = back_project_cont((real)u, (real)(v + 1), dd, K);
  const v3 dx = vsub(pr, pl);
  const v3 dy = vsub(pd, pu);
  v3 n = vnormalize(c->flavor, vcross(dy, dx));
  if (vnorm(n) <= 1e-6f) return 0;
  const v3 cp = back_project_cont((real)u, (real)v, dc, K);
  n = orient_toward_camera(c->flavor, n, cp);
  *normal = n;
  return vnorm(n) > 1e-6f;
}

typedef struct {
  const vo_config* c;
  const float* depth;
  const vo_intrinsics* K;
  float* normals;
  uint8_t* valid;
  float* out;
} filter_ctx;

static void normals_row(void* p, int64_t v) {
  filter_ctx* f = (filter_ctx*)p;
  const int W = f->K->width;
  for (int u = 0; u < W; ++u) {
    const size_t idx = (size_t)v * W + u;
    v3 n = mk(0.0f, 0.0f, 0.0f);
    if (pixel_normal(f->c, f->depth, f->K, u, (int)v, &n)) {
      f->normals[3 * idx + 0] = n.x;
      f->normals[3 * idx + 1] = n.y;
      f->normals[3 * idx + 2] = n.z;
      f->valid[idx] = 1;
    } else {
      f->normals[3 * idx + 0] = 0.0f;
      f->normals[3 * idx + 1] = 0.0f;
      f->normals[3 * idx + 2] = 0.0f;
      f->valid[idx] = 0;
    }
  }
}

/* cuda_tsdf_integrator.cu:650-725, reconstruction_backend.cpp:125-186 */
static void bilateral_row(void* p, int64_t vv) {
  filter_ctx* f = (filter_ctx*)p;
  const vo_config* c = f->c;
  const int W = f->K->width, H = f->K->height, v = (int)vv, R = c->filter_radius;
  const real ks = inv_two_sigma_sq(c->filter_sigma_spatial);
  const real kr = inv_two_sigma_sq(c->filter_sigma_range);
  const real ka = inv_two_sigma_sq(c->filter_sigma_angular);
  for (int u = 0; u < W; ++u) {
    const size_t ci = (size_t)v * W + u;
    const real center = f->depth[ci];
    if (center <= 0.0f) {
      f->out[ci] = 0.0f;
      continue;
    }
    const int has_cn = f->valid[ci] != 0;
    const v3 cn = has_cn ? mk(f->normals[3 * ci], f->normals[3 * ci + 1], f->normals[3 * ci + 2]) : mk(0.0f, 0.0f, 0.0f);
    const real thr = disc_threshold(c, center);
    real wds = 0.0f, ws = 0.0f;
    for (int dv = -R; dv <= R; ++dv) {
      const int sv = v + dv;
      if (sv < 0 || sv >= H) continue;
      for (int du = -R; du <= R; ++du) {
        const int su = u + du;
        if (su < 0 || su >= W) continue;
        const size_t si = (size_t)sv * W + su;
        const real sd = f->depth[si];
        if (sd <= 0.0f || VO_FABS(sd - center) > thr) continue;
        const real spatial = (real)(du * du + dv * dv);
        const real delta = sd - center;
        const real range = delta * delta;
        real w = gaussian(c, spatial, ks) * gaussian(c, range, kr);
        if (has_cn) {
          if (f->valid[si] == 0) continue;
          const v3 sn = mk(f->normals[3 * si], f->normals[3 * si + 1], f->normals[3 * si + 2]);
          const real cosine = clamp_f(vdot(cn, sn), -1.0f, 1.0f);
          if (cosine < c->filter_min_cos) continue;
          const real ad = 1.0f - cosine;
          w *= gaussian(c, ad * ad, ka);
        }
        wds += w * sd;
        ws += w;
      }
    }
    f->out[ci] = ws > 1e-6f ? (wds / ws) : center;
  }
}

void vo_depth_normals(const vo_config* c, const float* depth, const vo_intrinsics* K, float* normals,
                      uint8_t* valid) {
  filter_ctx f = {c, depth, K, normals, valid, NULL};
  parallel_for(c->threads, K->height, normals_row, &f);
}

void vo_filter_depth(const vo_config* c, const float* depth, const vo_intrinsics* K, float* out) {
  const size_t n = (size_t)K->width * (size_t)K->height;
  if (K->width <= 0 || K->height <= 0) return;
  float* normals = (float*)malloc(3 * n * sizeof(float));
  uint8_t* valid = (uint8_t*)malloc(n);
  filter_ctx f = {c, depth, K, normals, valid, out};
  parallel_for(c->threads, K->height, normals_row, &f);
  parallel_for(c->threads, K->height, bilateral_row, &f);
  free(normals);
  free(valid);
}

/* ---------------------------------------------------------------- sampling */
/* cuda_tsdf_integrator.cu:479-489 (floorf(x+0.5)), voxel_hash_tsdf.h:673-682 (lround) */
static inline int sample_nearest(int fl, const float* depth, const vo_intrinsics* K, real u, real v, real* d) {
  int ui, vi;
  if (fl == GPU) {
    ui = (int)VO_FLOOR(u + 0.5f);
    vi = (int)VO_FLOOR(v + 0.5f);
  } else {
    ui = (int)VO_LROUND(u);
    vi = (int)VO_LROUND(v);
  }
  if (ui < 0 || ui >= K->width || vi < 0 || vi >= K->height) return 0;
  *d = depth[(size_t)vi * K->width + ui];
  return *d > 0.0f;
}

/* cuda_tsdf_integrator.cu:504-568, voxel_hash_tsdf.h:684-748 */
static int sample_bilinear(const vo_config* c, const float* depth, const vo_intrinsics* K, real u, real v,
                           real* out) {
  const int W = K->width, H = K->height;
  if (W <= 0 || H <= 0) return 0;
  if (u < 0.0f || v < 0.0f || u > (real)(W - 1) || v > (real)(H - 1)) return 0;
  const int x0 = (int)VO_FLOOR(u);
  const int y0 = (int)VO_FLOOR(v);
  const int x1 = x0 + 1 < W - 1 ? x0 + 1 : W - 1;
  const int y1 = y0 + 1 < H - 1 ? y0 + 1 : H - 1;
  const real tx = u - (real)x0;
  const real ty = v - (real)y0;
  const real d00 = depth[(size_t)y0 * W + x0];
  const real d10 = depth[(size_t)y0 * W + x1];
  const real d01 = depth[(size_t)y1 * W + x0];
  const real d11 = depth[(size_t)y1 * W + x1];
  if (d00 > 0.0f && d10 > 0.0f && d01 > 0.0f && d11 > 0.0f) {
    real ref = 0.0f;
    if (!sample_nearest(c->flavor, depth, K, u, v, &ref)) ref = d00;
    const real thr = disc_threshold(c, ref);
    const real mn = fmin_f(fmin_f(d00, d10), fmin_f(d01, d11));
    const real mx = fmax_f(fmax_f(d00, d10), fmax_f(d01, d11));
    const real top = d00 + (d10 - d00) * tx;
    const real bottom = d01 + (d11 - d01) * tx;
    if (mx - mn <= thr) {
      *out = top + (bottom - top) * ty;
      return 1;
    }
    const real bw[4] = {(1.0f - tx) * (1.0f - ty), tx * (1.0f - ty), (1.0f - tx) * ty, tx * ty};
    const real nd[4] = {d00, d10, d01, d11};
    real wds = 0.0f, ws = 0.0f;
    for (int i = 0; i < 4; ++i) {
      if (VO_FABS(nd[i] - ref) > thr) continue;
      wds += bw[i] * nd[i];
      ws += bw[i];
    }
    if (ws > 1e-6f) {
      *out = wds / ws;
      return 1;
    }
  }
  return sample_nearest(c->flavor, depth, K, u, v, out);
}

/* cuda_tsdf_integrator.cu:727-752, voxel_hash_tsdf.h:750-771 */
static int base_normal(const vo_config* c, const float* depth, const vo_intrinsics* K, real u, real v, v3* n) {
  real dl = 0.0f, dr = 0.0f, du = 0.0f, dd = 0.0f;
  if (!sample_bilinear(c, depth, K, u - 1.0f, v, &dl) || !sample_bilinear(c, depth, K, u + 1.0f, v, &dr) ||
      !sample_bilinear(c, depth, K, u, v - 1.0f, &du) || !sample_bilinear(c, depth, K, u, v + 1.0f, &dd)) {
    return 0;
  }
  const v3 pl = back_project_cont(u - 1.0f, v, dl, K);
  const v3 pr = back_project_cont(u + 1.0f, v, dr, K);
  const v3 pu = back_project_cont(u, v - 1.0f, du, K);
  const v3 pd = back_project_cont(u, v + 1.0f, dd, K);
  const v3 dx = vsub(pr, pl);
  const v3 dy = vsub(pd, pu);
  *n = vnormalize(c->flavor, vcross(dy, dx));
  return vnorm(*n) > 1e-6f;
}

/* cuda_tsdf_integrator.cu:754-832, voxel_hash_tsdf.h:773-840 */
static int surface_normal(const vo_config* c, const float* depth, const vo_intrinsics* K, real u, real v,
                          v3* normal) {
  const int fl = c->flavor;
  v3 cn = mk(0.0f, 0.0f, 0.0f);
  if (!base_normal(c, depth, K, u, v, &cn)) return 0;
  real cd = 0.0f;
  if (!sample_bilinear(c, depth, K, u, v, &cd)) return 0;
  const v3 cp = back_project_cont(u, v, cd, K);
  cn = orient_toward_camera(fl, cn, cp);
  const real ks = inv_two_sigma_sq(c->normal_sigma_spatial);
  const real kr = inv_two_sigma_sq(c->normal_sigma_range);
  const real ka = inv_two_sigma_sq(c->normal_sigma_angular);
  v3 wsum = mk(0.0f, 0.0f, 0.0f);
  real ws = 0.0f;
  const int R = c->normal_radius;
  for (int dv = -R; dv <= R; ++dv) {
    for (int du = -R; du <= R; ++du) {
      const real su = u + (real)du;
      const real sv = v + (real)dv;
      v3 sn = mk(0.0f, 0.0f, 0.0f);
      if (!base_normal(c, depth, K, su, sv, &sn)) continue;
      real sd = 0.0f;
      if (!sample_bilinear(c, depth, K, su, sv, &sd)) continue;
      const v3 sp = back_project_cont(su, sv, sd, K);
      sn = orient_toward_camera(fl, sn, sp);
      const real spatial = (real)(du * du + dv * dv);
      const real delta = sd - cd;
      const real range = delta * delta;
      const real cosine = clamp_f(vdot(cn, sn), -1.0f, 1.0f);
      const real ad = 1.0f - cosine;
      const real as = ad * ad;
      const real w = gaussian(c, spatial, ks) * gaussian(c, range, kr) * gaussian(c, as, ka);
      wsum.x += sn.x * w;
      wsum.y += sn.y * w;
      wsum.z += sn.z * w;
      ws += w;
    }
  }
  if (ws <= 1e-6f) {
    *normal = cn;
    return 1;
  }
  const real inv = 1.0f / ws;
  v3 n = vnormalize(fl, mk(wsum.x * inv, wsum.y * inv, wsum.z * inv));
  n = orient_toward_camera(fl, n, cp);
  if (vnorm(n) <= 1e-6f) n = cn;
  *normal = n;
  return vnorm(n) > 1e-6f;
}

/* -------------------------------------------------------------- weighting */
/* cuda_tsdf_integrator.cu:429-450, voxel_hash_tsdf.h:556-584 */
float vo_observation_weight(const vo_config* c, float depth, float sd, float trunc, float view) {
  if (depth <= 0.0f || trunc <= 1e-6f) return 0.0f;
  const real dr = depth / c->depth_sigma;
  const real dw = 1.0f / (1.0f + dr * dr);
  const real nr = VO_FABS(sd) / trunc;
  real rw = 1.0f;
  if (nr > c->huber_delta) rw = c->huber_delta / nr;
  const real bw = 1.0f - 0.5f * clamp_f(nr, 0.0f, 1.0f);
  const real base = fmax_f(c->min_obs_weight, dw * rw * bw);
  const real aw = clamp_f(view, c->min_view_weight, 1.0f);
  return base * aw;
}

/* cuda_tsdf_integrator.cu:228-243, voxel_hash_tsdf.h:239-254 */
static inline int dominant_direction(v3 n) {
  const real nx = VO_FABS(n.x), ny = VO_FABS(n.y), nz = VO_FABS(n.z);
  if (nx <= 1e-6f && ny <= 1e-6f && nz <= 1e-6f) return -1;
  if (nx >= ny && nx >= nz) return n.x >= 0.0f ? 0 : 1;
  if (ny >= nx && ny >= nz) return n.y >= 0.0f ? 2 : 3;
  return n.z >= 0.0f ? 4 : 5;
}

/* GPU: cuda_tsdf_integrator.cu:296-313; CPU: voxel_hash_tsdf.h:311-330 (dot with the unit axis) */
static inline real coordinate_along(int fl, v3 p, int d) {
  if (fl == GPU) {
    switch (d) {
      case 0: return p.x;
      case 1: return -p.x;
      case 2: return p.y;
      case 3: return -p.y;
      case 4: return p.z;
      default: return -p.z;
    }
  }
  static const real axes[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  return vdot(p, mk(axes[d][0], axes[d][1], axes[d][2]));
}

static inline real sign_not_zero(real v) { return v >= 0.0f ? 1.0f : -1.0f; }

/* GPU: cuda_tsdf_integrator.cu:253-278 (floorf(x*65535+0.5)); CPU: voxel_hash_tsdf.h:268-289 (lround) */
static uint32_t pack_normal(int fl, v3 raw) {
  const v3 n = vnormalize(fl, raw);
  const real s = VO_FABS(n.x) + VO_FABS(n.y) + VO_FABS(n.z);
  if (s <= 1e-6f) return 0U;
  v3 p = vdivs(n, s);
  if (p.z < 0.0f) {
    const real px = (1.0f - VO_FABS(p.y)) * sign_not_zero(p.x);
    const real py = (1.0f - VO_FABS(p.x)) * sign_not_zero(p.y);
    p.x = px;
    p.y = py;
  }
  uint32_t q[2];
  const real comp[2] = {p.x, p.y};
  for (int i = 0; i < 2; ++i) {
    const real cl = clamp_f(comp[i] * 0.5f + 0.5f, 0.0f, 1.0f);
    if (fl == GPU) {
      q[i] = (uint32_t)VO_FLOOR(cl * 65535.0f + 0.5f);
    } else {
      q[i] = (uint32_t)VO_LROUND(cl * 65535.0f);
    }
  }
  return q[0] | (q[1] << 16U);
}

/* GPU integrator: cuda_tsdf_integrator.cu:258-294 (normalizeVec, zero on degenerate);
 * GPU mesh extractor: cuda_mesh_extractor.cu:233-257 ((0,0,1) on degenerate);
 * CPU: voxel_hash_tsdf.h:291-309 (normalized). */
static v3 unpack_normal(int fl, int mesh_variant, uint32_t packed) {
  v3 n = mk((real)(packed & 0xffffU) / 65535.0f * 2.0f - 1.0f,
            (real)((packed >> 16U) & 0xffffU) / 65535.0f * 2.0f - 1.0f, 0.0f);
  n.z = 1.0f - VO_FABS(n.x) - VO_FABS(n.y);
  if (n.z < 0.0f) {
    const real px = (1.0f - VO_FABS(n.y)) * sign_not_zero(n.x);
    const real py = (1.0f - VO_FABS(n.x)) * sign_not_zero(n.y);
    n.x = px;
    n.y = py;
  }
  if (fl == GPU && mesh_variant) {
    const real len = VO_SQRT(n.x * n.x + n.y * n.y + n.z * n.z);
    if (len <= 1e-6f) return mk(0.0f, 0.0f, 1.0f);
    const real inv = 1.0f / len;
    return mk(n.x * inv, n.y * inv, n.z * inv);
  }
  return vnormalize(fl, n);
}

uint32_t vo_pack_normal(int32_t flavor, const float n[3]) { return pack_normal(flavor, mk(n[0], n[1], n[2])); }
void vo_unpack_normal(int32_t flavor, int32_t mesh_variant, uint32_t packed, float out[3]) {
  const v3 n = unpack_normal(flavor, mesh_variant, packed);
  out[0] = n.x;
  out[1] = n.y;
  out[2] = n.z;
}

/* ---------------------------------------------------------- layer update */
/* cuda_tsdf_integrator.cu:319-336, voxel_hash_tsdf.h:341-355 */
static void sort_layers(vo_layer* L) {
  for (int pass = 0; pass < LAYERS - 1; ++pass) {
    for (int i = 0; i < LAYERS - pass - 1; ++i) {
      const int lv = L[i].weight > 0.0f;
      const int rv = L[i + 1].weight > 0.0f;
      const int swap = (!lv && rv) || (lv && rv && L[i].surface_coord > L[i + 1].surface_coord);
      if (swap) {
        const vo_layer t = L[i];
        L[i] = L[i + 1];
        L[i + 1] = t;
      }
    }
  }
}

/* cuda_tsdf_integrator.cu:338-372, voxel_hash_tsdf.h:357-392 */
static int find_layer_slot(int fl, const vo_layer* L, real sc, v3 n, real tol, real min_cos) {
  int empty = -1, best = -1;
  real best_delta = fl == GPU ? 1e30f : FLT_MAX;
  for (int i = 0; i < LAYERS; ++i) {
    if (!(L[i].weight > 0.0f)) {
      if (empty < 0) empty = i;
      continue;
    }
    const v3 ln = unpack_normal(fl, 0, L[i].packed_normal);
    if (vdot(ln, n) < min_cos) continue;
    const real delta = VO_FABS(L[i].surface_coord - sc);
    if (delta < best_delta) {
      best_delta = delta;
      best = i;
    }
  }
  if (best >= 0 && best_delta <= tol) return best;
  return empty;
}

/* cuda_tsdf_integrator.cu:374-427, voxel_hash_tsdf.h:479-529 */
static void integrate_sample(const vo_config* c, real vs, vo_voxel* voxel, int d, real sc, v3 sp, v3 nw,
                             real obs) {
  const int fl = c->flavor;
  if (d < 0 || d >= DIRS || obs <= 0.0f) return;
  const v3 n = vnormalize(fl, nw);
  if (vnorm(n) <= 1e-6f) return;
  const real plane_offset = vdot(n, sp);
  const real tol = fmax_f(1e-6f, vs * c->layer_merge_scale);
  vo_layer* L = voxel->layers[d];
  const int li = find_layer_slot(fl, L, sc, n, tol, c->layer_normal_cos);
  if (li < 0) return;
  vo_layer* layer = &L[li];
  const real pw = layer->weight;
  const real ew = fmin_f(obs, fmax_f(0.0f, c->max_weight - pw));
  if (ew <= 0.0f) return;
  const real nwt = pw + ew;
  v3 blended = n;
  layer->surface_coord = pw > 0.0f ? ((layer->surface_coord * pw + sc * ew) / nwt) : sc;
  layer->plane_offset = pw > 0.0f ? ((layer->plane_offset * pw + plane_offset * ew) / nwt) : plane_offset;
  if (pw > 0.0f) {
    const v3 pn = unpack_normal(fl, 0, layer->packed_normal);
    if (fl == GPU) {
      blended = vnormalize(fl, vmul(vadd(vmul(pn, pw), vmul(n, ew)), 1.0f / nwt));
    } else {
      blended = vnormalize(fl, vdivs(vadd(vmul(pn, pw), vmul(n, ew)), nwt));
    }
    if (vnorm(blended) <= 1e-6f) blended = n;
  }
  layer->weight = nwt;
  layer->packed_normal = pack_normal(fl, blended);
  sort_layers(L);
}

/* ------------------------------------------------------------ block keys */
/* cuda_block_allocator.cu:153-159 */
uint32_t vo_hash_block_key(int32_t x, int32_t y, int32_t z) {
  uint32_t seed = 0U;
  seed ^= (uint32_t)x * 73856093U + 0x9e3779b9U + (seed << 6U) + (seed >> 2U);
  seed ^= (uint32_t)y * 19349663U + 0x9e3779b9U + (seed << 6U) + (seed >> 2U);
  seed ^= (uint32_t)z * 83492791U + 0x9e3779b9U + (seed << 6U) + (seed >> 2U);
  return seed;
}

/* cuda_block_allocator.cu:161-174 (21 bits per axis, bias 2^20) */
int32_t vo_pack_block_key(int32_t x, int32_t y, int32_t z, uint64_t* packed) {
  const int32_t bias = 1 << 20;
  if (x < -bias || x > bias - 1 || y < -bias || y > bias - 1 || z < -bias || z > bias - 1) return 0;
  *packed = (uint64_t)(x + bias) | ((uint64_t)(y + bias) << 21) | ((uint64_t)(z + bias) << 42);
  return 1;
}

/* voxel_hash_tsdf.h:531-546 */
static inline int floor_div(int value, int divisor) {
  int q = value / divisor;
  const int r = value % divisor;
  if (r != 0 && ((r < 0) != (divisor < 0))) --q;
  return q;
}
static inline int positive_mod(int value, int divisor) {
  int r = value % divisor;
  if (r < 0) r += divisor;
  return r;
}

/* simple open-addressing key set/map used by the oracle (not the reference's structure) */
typedef struct {
  vo_key* keys;
  int64_t* vals;
  int64_t cap, count;
} keymap;

static uint64_t key_hash(vo_key k) {
  uint64_t h = (uint64_t)(uint32_t)k.x * 0x9E3779B97F4A7C15ULL;
  h ^= (uint64_t)(uint32_t)k.y * 0xC2B2AE3D27D4EB4FULL + (h << 6) + (h >> 2);
  h ^= (uint64_t)(uint32_t)k.z * 0x165667B19E3779F9ULL + (h << 6) + (h >> 2);
  h ^= h >> 29;
  return h;
}

static void keymap_init(keymap* m, int64_t cap) {
  int64_t c = 16;
  while (c < cap * 2) c <<= 1;
  m->cap = c;
  m->count = 0;
  m->keys = (vo_key*)malloc((size_t)c * sizeof(vo_key));
  m->vals = (int64_t*)malloc((size_t)c * sizeof(int64_t));
  for (int64_t i = 0; i < c; ++i) m->vals[i] = -1;
}
static void keymap_free(keymap* m) {
  free(m->keys);
  free(m->vals);
  memset(m, 0, sizeof(*m));
}
static int64_t keymap_find(const keymap* m, vo_key k) {
  if (m->cap == 0) return -1;
  int64_t s = (int64_t)(key_hash(k) & (uint64_t)(m->cap - 1));
  for (;;) {
    if (m->vals[s] < 0) return -1;
    if (m->keys[s].x == k.x && m->keys[s].y == k.y && m->keys[s].z == k.z) return m->vals[s];
    s = (s + 1) & (m->cap - 1);
  }
}
static void keymap_put(keymap* m, vo_key k, int64_t v);
static void keymap_grow(keymap* m) {
  keymap n;
  keymap_init(&n, m->cap);
  for (int64_t i = 0; i < m->cap; ++i)
    if (m->vals[i] >= 0) keymap_put(&n, m->keys[i], m->vals[i]);
  keymap_free(m);
  *m = n;
}
/* inserts if absent; returns 1 if inserted */
static int keymap_insert(keymap* m, vo_key k, int64_t v) {
  if ((m->count + 1) * 2 > m->cap) keymap_grow(m);
  int64_t s = (int64_t)(key_hash(k) & (uint64_t)(m->cap - 1));
  for (;;) {
    if (m->vals[s] < 0) {
      m->keys[s] = k;
      m->vals[s] = v;
      ++m->count;
      return 1;
    }
    if (m->keys[s].x == k.x && m->keys[s].y == k.y && m->keys[s].z == k.z) return 0;
    s = (s + 1) & (m->cap - 1);
  }
}
static void keymap_put(keymap* m, vo_key k, int64_t v) { (void)keymap_insert(m, k, v); }

static int key_cmp(const void* a, const void* b) {
  const vo_key* p = (const vo_key*)a;
  const vo_key* q = (const vo_key*)b;
  if (p->x != q->x) return p->x < q->x ? -1 : 1;
  if (p->y != q->y) return p->y < q->y ? -1 : 1;
  if (p->z != q->z) return p->z < q->z ? -1 : 1;
  return 0;
}

/* GPU: cuda_block_allocator.cu:198-272 (floorf(p / (8 vs)), 27 neighbours, range-checked packing);
 * CPU: voxel_hash_tsdf.h:595-671 (floorDiv(floor(p / vs), 8), 27 neighbours). */
static int insert_neighbourhood(int fl, v3 p, real vs, keymap* set) {
  int bx, by, bz;
  if (fl == GPU) {
    const real bws = vs * 8.0f;
    bx = (int)VO_FLOOR(p.x / bws);
    by = (int)VO_FLOOR(p.y / bws);
    bz = (int)VO_FLOOR(p.z / bws);
  } else {
    bx = floor_div((int)VO_FLOOR(p.x / vs), BLOCK);
    by = floor_div((int)VO_FLOOR(p.y / vs), BLOCK);
    bz = floor_div((int)VO_FLOOR(p.z / vs), BLOCK);
  }
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const vo_key k = {bx + dx, by + dy, bz + dz};
        if (fl == GPU) {
          uint64_t packed;
          if (!vo_pack_block_key(k.x, k.y, k.z, &packed)) return 0;
        }
        keymap_insert(set, k, 0);
      }
  return 1;
}

static int collect_into(const vo_config* c, const float* depth, const vo_intrinsics* K, const vo_pose* T, real vs,
                        real trunc, int32_t stride, keymap* set) {
  const int fl = c->flavor;
  const int s = stride > 1 ? stride : 1;
  const v3 cam = mk(T->t[0], T->t[1], T->t[2]);
  for (int v = 0; v < K->height; v += s) {
    for (int u = 0; u < K->width; u += s) {
      const real d = depth[(size_t)v * K->width + u];
      if (d <= 0.0f) continue;
      const v3 pc = back_project(u, v, d, K);
      const v3 pw = pose_point(T, pc);
      const v3 ray = vnormalize(fl, vsub(pw, cam));
      const v3 front = vsub(pw, vmul(ray, trunc));
      const v3 back = vadd(pw, vmul(ray, trunc));
      if (!insert_neighbourhood(fl, pw, vs, set)) return 0;
      if (!insert_neighbourhood(fl, front, vs, set)) return 0;
      if (!insert_neighbourhood(fl, back, vs, set)) return 0;
    }
  }
  return 1;
}

int64_t vo_collect_blocks(const vo_config* c, const float* depth, const vo_intrinsics* K, const vo_pose* T, float vs,
                          float trunc, int32_t stride, vo_key* out, int64_t max_out) {
  keymap set;
  keymap_init(&set, 1024);
  if (!collect_into(c, depth, K, T, vs, trunc, stride, &set)) {
    keymap_free(&set);
    return -1;
  }
  if (set.count > max_out) {
    const int64_t n = set.count;
    keymap_free(&set);
    return n > 0 ? -2 : 0;
  }
  int64_t n = 0;
  for (int64_t i = 0; i < set.cap; ++i)
    if (set.vals[i] >= 0) out[n++] = set.keys[i];
  qsort(out, (size_t)n, sizeof(vo_key), key_cmp);
  keymap_free(&set);
  return n;
}

/* The truncation-band allocation rule (the library's opt-in allocation mode 1; the reference has no such
 * rule): every block crossed by the segment [p - trunc*ray, p + trunc*ray] of each valid pixel, found by a
 * voxel walk (Amanatides & Woo, "A Fast Voxel Traversal Algorithm for Ray Tracing", 1987) over cells of
 * 8 vs with the start and end cells taken by floorf(x / (8 vs)).  The walk takes at most 64 steps, ends on
 * the end cell or when the next crossing lies past the segment (t > 1), and the end cell is always added.
 * Every visited key must pack into 21 bits per axis.  The point, ray and segment ends are computed as the
 * GPU flavour of the reference rule computes them (cuda_block_allocator.cu:231-258). */
static int insert_band(v3 a, v3 b, real bws, keymap* set) {
  int c[3] = {(int)VO_FLOOR(a.x / bws), (int)VO_FLOOR(a.y / bws), (int)VO_FLOOR(a.z / bws)};
  const int e[3] = {(int)VO_FLOOR(b.x / bws), (int)VO_FLOOR(b.y / bws), (int)VO_FLOOR(b.z / bws)};
  const real o[3] = {a.x, a.y, a.z};
  const real d[3] = {b.x - a.x, b.y - a.y, b.z - a.z};
  int st[3];
  real tmax[3], tdel[3];
  for (int k = 0; k < 3; ++k) {
    st[k] = d[k] > 0.0f ? 1 : (d[k] < 0.0f ? -1 : 0);
    if (st[k] != 0) {
      const real edge = (real)(c[k] + (st[k] > 0 ? 1 : 0)) * bws;
      tmax[k] = (edge - o[k]) / d[k];
      tdel[k] = bws / VO_FABS(d[k]);
    } else {
      tmax[k] = 3.0e38f;
      tdel[k] = 3.0e38f;
    }
  }
  uint64_t packed;
  for (int step = 0; step < 64; ++step) {
    if (!vo_pack_block_key(c[0], c[1], c[2], &packed)) return 0;
    keymap_insert(set, (vo_key){c[0], c[1], c[2]}, 0);
    if (c[0] == e[0] && c[1] == e[1] && c[2] == e[2]) break;
    /* the axis of the nearest crossing; ties go to the later axis */
    int k = 2;
    if (tmax[0] < tmax[1]) {
      if (tmax[0] < tmax[2]) k = 0;
    } else if (tmax[1] < tmax[2]) {
      k = 1;
    }
    if (tmax[k] > 1.0f) break;
    c[k] += st[k];
    tmax[k] += tdel[k];
  }
  if (!vo_pack_block_key(e[0], e[1], e[2], &packed)) return 0;
  keymap_insert(set, (vo_key){e[0], e[1], e[2]}, 0);
  return 1;
}

int64_t vo_collect_band_blocks(const float* depth, const vo_intrinsics* K, const vo_pose* T, float vs, float trunc,
                               int32_t stride, vo_key* out, int64_t max_out) {
  const int s = stride > 1 ? stride : 1;
  const v3 cam = mk(T->t[0], T->t[1], T->t[2]);
  const real bws = vs * 8.0f;
  keymap set;
  keymap_init(&set, 1024);
  for (int v = 0; v < K->height; v += s) {
    for (int u = 0; u < K->width; u += s) {
      const real d = depth[(size_t)v * K->width + u];
      if (!(d > 0.0f)) continue;
      const v3 pw = pose_point(T, back_project(u, v, d, K));
      const v3 ray = vnormalize(GPU, vsub(pw, cam));
      if (!insert_band(vsub(pw, vmul(ray, trunc)), vadd(pw, vmul(ray, trunc)), bws, &set)) {
        keymap_free(&set);
        return -1;
      }
    }
  }
  if (set.count > max_out) {
    const int64_t n = set.count;
    keymap_free(&set);
    return n > 0 ? -2 : 0;
  }
  int64_t n = 0;
  for (int64_t i = 0; i < set.cap; ++i)
    if (set.vals[i] >= 0) out[n++] = set.keys[i];
  qsort(out, (size_t)n, sizeof(vo_key), key_cmp);
  keymap_free(&set);
  return n;
}


/* ---------------------------------------------- the library's opt-in forms */
/* Restatements of the GPU library's opt-in switches as its exact compile evaluates them (no reference
 * counterpart; voxelhashmt_gb300/csrc/vh_common.cuh and vh_integrate.cu): the per-voxel interpolation of the
 * per-pixel normal map (map_normal) and the FP16 bin (decode_bin16, encode_bin16, integrate_bin16).  Explicit
 * float arithmetic, every operation rounded once, as the device's -fmad=false compile and its _rn intrinsics. */
typedef union {
  float f;
  uint32_t u;
} fbits;
static inline float u_as_f(uint32_t u) {
  fbits b;
  b.u = u;
  return b.f;
}
static inline uint32_t f_as_u(float f) {
  fbits b;
  b.f = f;
  return b.u;
}
/* binary16 -> float (exact) */
static float h2f(uint32_t h) {
  const uint32_t sign = (h & 0x8000U) << 16, e = (h >> 10) & 0x1fU, m = h & 0x3ffU;
  if (e == 0U) {
    const float f = (float)m * 0x1p-24f;
    return sign ? -f : f;
  }
  if (e == 31U) return u_as_f(sign | 0x7f800000U | (m << 13));
  return u_as_f(sign | ((e + 112U) << 23) | (m << 13));
}
/* float -> binary16, round to nearest even, with subnormals and overflow to infinity */
static uint32_t f2h(float f) {
  const uint32_t x = f_as_u(f);
  const uint32_t sign = (x >> 16) & 0x8000U, ax = x & 0x7fffffffU;
  if (ax >= 0x7f800000U) return sign | (ax > 0x7f800000U ? 0x7e00U : 0x7c00U);
  if (ax >= 0x477ff000U) return sign | 0x7c00U; /* >= 65520 rounds to infinity */
  if (ax <= 0x33000000U) return sign;          /* <= 2^-25 rounds to zero */
  const int e = (int)(ax >> 23) - 127;
  const uint32_t m = (ax & 0x7fffffU) | 0x800000U;
  if (e < -14) {
    const int shift = -1 - e;                  /* subnormal result: units of 2^-24 */
    uint32_t r = m >> shift;
    const uint32_t rem = m & ((1U << shift) - 1U), half = 1U << (shift - 1);
    if (rem > half || (rem == half && (r & 1U))) ++r;
    return sign | r;
  }
  uint32_t r = ((uint32_t)(e + 15) << 10) | ((m >> 13) & 0x3ffU);
  const uint32_t rem = m & 0x1fffU;
  if (rem > 0x1000U || (rem == 0x1000U && (r & 1U))) ++r;
  return sign | r;
}
/* 1/sqrt(x) correctly rounded (the device's __frsqrt_rn), for positive normal x: the double estimate, then the
 * nearest float decided exactly by the sign of m^2 x - 1 at the midpoints m to its neighbours (m^2 is exact in
 * double and the fused multiply-add rounds the product-minus-one once, so its sign is the exact sign). */
static float cr_rsqrtf(float x) {
  const double xd = (double)x;
  float r = (float)(1.0 / sqrt(xd));
  for (int it = 0; it < 4; ++it) {
    const float up = nextafterf(r, INFINITY);
    double m = ((double)r + (double)up) * 0.5;
    if (fma(m * m, xd, -1.0) < 0.0) {
      r = up;
      continue;
    }
    const float dn = nextafterf(r, 0.0f);
    m = ((double)dn + (double)r) * 0.5;
    if (fma(m * m, xd, -1.0) > 0.0) {
      r = dn;
      continue;
    }
    break;
  }
  return r;
}
float vo_rsqrtf_rn(float x) { return cr_rsqrtf(x); }

typedef struct {
  float x, y, z;
} f3o;
static inline f3o f3mk(float x, float y, float z) {
  f3o r = {x, y, z};
  return r;
}
static inline float f3dot(f3o a, f3o b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* vh_common.cuh: bin_normal (octahedral decode, normalised with the correctly rounded reciprocal root) */
static f3o bin_normal(uint32_t packed) {
  float x = (float)(packed & 0xffffU) / 65535.0f * 2.0f + -1.0f;
  float y = (float)(packed >> 16U) / 65535.0f * 2.0f + -1.0f;
  const float z = (1.0f + -fabsf(x)) + -fabsf(y);
  if (z < 0.0f) {
    const float fx = copysignf(1.0f + -fabsf(y), x >= 0.0f ? 1.0f : -1.0f);
    const float fy = copysignf(1.0f + -fabsf(x), y >= 0.0f ? 1.0f : -1.0f);
    x = fx;
    y = fy;
  }
  const float inv = cr_rsqrtf((x * x + y * y) + z * z);
  return f3mk(x * inv, y * inv, z * inv);
}
static inline float axis_coord(f3o p, int d) {
  const float a = (d >> 1) == 0 ? p.x : ((d >> 1) == 1 ? p.y : p.z);
  return (d & 1) ? -a : a;
}
static inline f3o voxel_centre_f(vo_key k, int li, float vs) {
  const int lx = li & 7, ly = (li >> 3) & 7, lz = li >> 6;
  return f3mk(((float)(k.x * BLOCK + lx) + 0.5f) * vs, ((float)(k.y * BLOCK + ly) + 0.5f) * vs,
              ((float)(k.z * BLOCK + lz) + 0.5f) * vs);
}
/* decode_layer16 / decode_bin16: the three layer records of a bin, w[8] = {A.x, A.y, A.z, A.w, B.x .. B.w} */
static void decode_bin16(const uint32_t* w, f3o c, int d, float vs, vo_layer* L) {
  const float cd = axis_coord(c, d);
  const uint32_t wt[3] = {w[0] & 0xffffU, w[1] >> 16, w[3] & 0xffffU};
  const uint32_t st[3] = {w[0] >> 16, w[2] & 0xffffU, w[3] >> 16};
  const uint32_t pt[3] = {w[1] & 0xffffU, w[2] >> 16, w[4] & 0xffffU};
  for (int l = 0; l < 3; ++l) {
    memset(&L[l], 0, sizeof(vo_layer));
    if (wt[l] == 0U) continue;
    const uint32_t packed = w[5 + l];
    const f3o n = bin_normal(packed);
    L[l].weight = h2f(wt[l]);
    L[l].surface_coord = cd + h2f(st[l]) * vs;
    L[l].plane_offset = f3dot(n, c) + h2f(pt[l]) * vs;
    L[l].packed_normal = packed;
  }
}
/* encode_bin16 (the store of decoded records: imports) */
static void encode_bin16(const vo_layer* L, f3o c, int d, float inv_vs, uint32_t* w) {
  const float cd = axis_coord(c, d);
  uint32_t ws[3] = {0U, 0U, 0U}, pp[3] = {0U, 0U, 0U}, nn[3] = {0U, 0U, 0U};
  for (int l = 0; l < 3; ++l) {
    if (!(L[l].weight > 0.0f)) continue;
    nn[l] = L[l].packed_normal;
    const f3o n = bin_normal(nn[l]);
    uint32_t wt = f2h(L[l].weight);
    if (wt == 0U) wt = 1U;
    ws[l] = wt | (f2h((L[l].surface_coord + -cd) * inv_vs) << 16);
    pp[l] = f2h((L[l].plane_offset + -f3dot(n, c)) * inv_vs);
  }
  w[0] = ws[0];
  w[1] = pp[0] | ((ws[1] & 0xffffU) << 16);
  w[2] = (ws[1] >> 16) | (pp[1] << 16);
  w[3] = ws[2];
  w[4] = pp[2];
  w[5] = nn[0];
  w[6] = nn[1];
  w[7] = nn[2];
}
/* integrate_bin16 (vh_integrate.cu): findLayerSlotForObservationGpu + integrateDirectionalSampleGpu
 * (cuda_tsdf_integrator.cu:338-427) on the binary16 triplets of one bin; returns 1 when a layer was updated */
static int integrate_bin16_o(const vo_config* cfg, float vs, float inv_vs, uint32_t* w, f3o c, int dir, float sc,
                             v3 sp, v3 nw, float obs) {
  if (obs <= 0.0f) return 0;
  const v3 n = vnormalize(GPU, nw);
  if (vnorm(n) <= 1e-6f) return 0;
  const float merge_tol = fmax_f(1e-6f, vs * cfg->layer_merge_scale);
  const float cd = axis_coord(c, dir);
  uint32_t w16[3] = {w[0] & 0xffffU, w[1] >> 16, w[3] & 0xffffU};
  uint32_t s16[3] = {w[0] >> 16, w[2] & 0xffffU, w[3] >> 16};
  uint32_t p16[3] = {w[1] & 0xffffU, w[2] >> 16, w[4] & 0xffffU};
  uint32_t nk[3] = {w[5], w[6], w[7]};
  float ls[3];
  f3o ln[3];
  int empty = -1, best = -1;
  float best_delta = 1e30f;
  for (int l = 0; l < 3; ++l) {
    ls[l] = cd + h2f(s16[l]) * vs;
    ln[l] = f3mk(0.0f, 0.0f, 1.0f);
    if (w16[l] == 0U) {
      if (empty < 0) empty = l;
      continue;
    }
    const float delta = fabsf(ls[l] - sc);
    if (!(delta <= merge_tol)) continue;
    ln[l] = bin_normal(nk[l]);
    if (ln[l].x * n.x + ln[l].y * n.y + ln[l].z * n.z < cfg->layer_normal_cos) continue;
    if (delta < best_delta) {
      best_delta = delta;
      best = l;
    }
  }
  const int li = (best >= 0 && best_delta <= merge_tol) ? best : empty;
  if (li < 0) return 0;
  const int had = w16[li] != 0U;
  const float pw = had ? h2f(w16[li]) : 0.0f;
  const float ew = fmin_f(obs, fmax_f(0.0f, cfg->max_weight - pw));
  if (ew <= 0.0f) return 0;
  const float nwt = pw + ew;
  const float plane_offset = vdot(n, sp);
  const v3 pn = mk(ln[li].x, ln[li].y, ln[li].z);
  float new_s = sc, new_p = plane_offset;
  v3 blended = n;
  if (had) {
    const float old_s = ls[li];
    const float old_p = f3dot(ln[li], c) + h2f(p16[li]) * vs;
    new_s = (old_s * pw + sc * ew) / nwt;
    new_p = (old_p * pw + plane_offset * ew) / nwt;
    blended = vnormalize(GPU, vmul(vadd(vmul(pn, pw), vmul(n, ew)), 1.0f / nwt));
    if (vnorm(blended) <= 1e-6f) blended = n;
  }
  const uint32_t packed = pack_normal(GPU, blended);
  uint32_t nwt16 = f2h(nwt);
  if (nwt16 == 0U) nwt16 = 1U;
  const uint32_t ns16 = f2h((new_s + -cd) * inv_vs);
  const uint32_t np16 = f2h((new_p + -f3dot(bin_normal(packed), c)) * inv_vs);
  w16[li] = nwt16;
  s16[li] = ns16;
  p16[li] = np16;
  nk[li] = packed;
  ls[li] = new_s;
  if (w16[1] != 0U || w16[2] != 0U) {
    static const int pairs[3][2] = {{0, 1}, {1, 2}, {0, 1}};
    for (int k = 0; k < 3; ++k) {
      const int a = pairs[k][0], b = pairs[k][1];
      const int av = w16[a] != 0U, bv = w16[b] != 0U;
      if ((!av && bv) || (av && bv && ls[a] > ls[b])) {
        uint32_t t = w16[a];
        w16[a] = w16[b];
        w16[b] = t;
        t = s16[a];
        s16[a] = s16[b];
        s16[b] = t;
        t = p16[a];
        p16[a] = p16[b];
        p16[b] = t;
        t = nk[a];
        nk[a] = nk[b];
        nk[b] = t;
        const float tf = ls[a];
        ls[a] = ls[b];
        ls[b] = tf;
      }
    }
  }
  w[0] = w16[0] | (s16[0] << 16);
  w[1] = p16[0] | (w16[1] << 16);
  w[2] = s16[1] | (p16[1] << 16);
  w[3] = w16[2] | (s16[2] << 16);
  w[4] = p16[2];
  w[5] = w16[0] ? nk[0] : 0U;
  w[6] = w16[1] ? nk[1] : 0U;
  w[7] = w16[2] ? nk[2] : 0U;
  return 1;
}
/* map_normal (vh_integrate.cu): the normal at (u, v), bilinear blend of the valid map taps, renormalised;
 * nmap: 4 floats per pixel (normal, valid 1/0) */
static int map_normal_o(const float* nmap, const vo_intrinsics* K, float u, float v, v3* n) {
  const int x0 = (int)floorf(u), y0 = (int)floorf(v);
  const int x1 = x0 + 1 < K->width - 1 ? x0 + 1 : K->width - 1;
  const int y1 = y0 + 1 < K->height - 1 ? y0 + 1 : K->height - 1;
  const float tx = u - (float)x0, ty = v - (float)y0;
  const float* a = nmap + 4 * ((size_t)y0 * K->width + x0);
  const float* b = nmap + 4 * ((size_t)y0 * K->width + x1);
  const float* c = nmap + 4 * ((size_t)y1 * K->width + x0);
  const float* d = nmap + 4 * ((size_t)y1 * K->width + x1);
  const float wa = (1.0f - tx) * (1.0f - ty) * a[3], wb = tx * (1.0f - ty) * b[3];
  const float wc = (1.0f - tx) * ty * c[3], wd = tx * ty * d[3];
  const v3 s = mk(wa * a[0] + wb * b[0] + wc * c[0] + wd * d[0], wa * a[1] + wb * b[1] + wc * c[1] + wd * d[1],
                  wa * a[2] + wb * b[2] + wc * c[2] + wd * d[2]);
  if (wa + wb + wc + wd <= 1e-6f || vnorm(s) <= 1e-6f) return 0;
  *n = vnormalize(GPU, s);
  return 1;
}

/* ------------------------------------------------------------------ volume */
struct vo_volume {
  vo_config cfg;
  real vs, trunc;
  keymap map;
  vo_key* keys;
  vo_voxel* voxels;
  uint32_t* bins16; /* layer_format 1: 8 words per (block, voxel, direction) */
  int64_t count, cap;
};
#define BIN16_WORDS (BLOCK_VOLUME * DIRS * 8)

vo_volume* vo_volume_new(const vo_config* c, float vs, float trunc) {
  vo_volume* v = (vo_volume*)calloc(1, sizeof(vo_volume));
  v->cfg = *c;
  v->vs = vs;
  v->trunc = trunc;
  keymap_init(&v->map, 1024);
  return v;
}

void vo_volume_free(vo_volume* v) {
  if (!v) return;
  keymap_free(&v->map);
  free(v->keys);
  free(v->voxels);
  free(v->bins16);
  free(v);
}

void vo_free(void* p) { free(p); }

static int64_t volume_ensure(vo_volume* v, vo_key k) {
  const int64_t f = keymap_find(&v->map, k);
  if (f >= 0) return f;
  if (v->count == v->cap) {
    const int64_t nc = v->cap ? v->cap * 2 : 64;
    v->keys = (vo_key*)realloc(v->keys, (size_t)nc * sizeof(vo_key));
    v->voxels = (vo_voxel*)realloc(v->voxels, (size_t)nc * BLOCK_VOLUME * sizeof(vo_voxel));
    if (v->cfg.layer_format == 1) v->bins16 = (uint32_t*)realloc(v->bins16, (size_t)nc * BIN16_WORDS * sizeof(uint32_t));
    v->cap = nc;
  }
  const int64_t idx = v->count++;
  v->keys[idx] = k;
  memset(&v->voxels[idx * BLOCK_VOLUME], 0, BLOCK_VOLUME * sizeof(vo_voxel));
  if (v->cfg.layer_format == 1) memset(&v->bins16[idx * BIN16_WORDS], 0, BIN16_WORDS * sizeof(uint32_t));
  keymap_insert(&v->map, k, idx);
  return idx;
}

int64_t vo_volume_block_count(const vo_volume* v) { return v->count; }

int64_t vo_volume_find_block(const vo_volume* v, int32_t x, int32_t y, int32_t z) {
  const vo_key k = {x, y, z};
  return keymap_find(&v->map, k);
}

void vo_volume_get_block(const vo_volume* v, int64_t i, vo_key* key, vo_voxel* voxels) {
  if (key) *key = v->keys[i];
  if (voxels) memcpy(voxels, &v->voxels[i * BLOCK_VOLUME], BLOCK_VOLUME * sizeof(vo_voxel));
}

/* layer_format 1: the voxel records of block idx decoded from its bins (the library's export) */
static void decode_block16(vo_volume* v, int64_t idx) {
  const float vs = (float)v->vs;
  for (int li = 0; li < BLOCK_VOLUME; ++li) {
    const f3o c = voxel_centre_f(v->keys[idx], li, vs);
    for (int d = 0; d < DIRS; ++d)
      decode_bin16(&v->bins16[idx * BIN16_WORDS + ((size_t)li * DIRS + d) * 8], c, d, vs,
                   v->voxels[idx * BLOCK_VOLUME + li].layers[d]);
  }
}

void vo_volume_set_block(vo_volume* v, vo_key key, const vo_voxel* voxels) {
  const int64_t idx = volume_ensure(v, key);
  memcpy(&v->voxels[idx * BLOCK_VOLUME], voxels, BLOCK_VOLUME * sizeof(vo_voxel));
  if (v->cfg.layer_format == 1) { /* the library encodes imported records into bins */
    const float vs = (float)v->vs, inv_vs = 1.0f / vs;
    for (int li = 0; li < BLOCK_VOLUME; ++li) {
      const f3o c = voxel_centre_f(key, li, vs);
      for (int d = 0; d < DIRS; ++d)
        encode_bin16(voxels[li].layers[d], c, d, inv_vs, &v->bins16[idx * BIN16_WORDS + ((size_t)li * DIRS + d) * 8]);
    }
    decode_block16(v, idx);
  }
}

/* VoxelHashTSDF::applyFlatBlocks (voxel_hash_tsdf.h:183-188): for each record in order, blocks_[key] (created
 * if absent) takes the record's 512 voxels; a key given twice keeps the later record. */
void vo_volume_apply_flat_blocks(vo_volume* v, const vo_key* keys, const vo_voxel* voxels, int64_t n) {
  for (int64_t i = 0; i < n; ++i) vo_volume_set_block(v, keys[i], voxels + i * BLOCK_VOLUME);
}

/* Removes the given keys (absent keys are ignored); the remaining blocks keep their relative order.  The state
 * of a volume after the library's eviction of those blocks (which has no reference counterpart). */
void vo_volume_remove_blocks(vo_volume* v, const vo_key* keys, int64_t n) {
  char* drop = (char*)calloc((size_t)(v->count > 0 ? v->count : 1), 1);
  for (int64_t i = 0; i < n; ++i) {
    const int64_t idx = keymap_find(&v->map, keys[i]);
    if (idx >= 0) drop[idx] = 1;
  }
  int64_t m = 0;
  for (int64_t i = 0; i < v->count; ++i) {
    if (drop[i]) continue;
    if (m != i) {
      v->keys[m] = v->keys[i];
      memmove(&v->voxels[m * BLOCK_VOLUME], &v->voxels[i * BLOCK_VOLUME], BLOCK_VOLUME * sizeof(vo_voxel));
      if (v->cfg.layer_format == 1)
        memmove(&v->bins16[m * BIN16_WORDS], &v->bins16[i * BIN16_WORDS], BIN16_WORDS * sizeof(uint32_t));
    }
    ++m;
  }
  v->count = m;
  keymap_free(&v->map);
  keymap_init(&v->map, 1024);
  for (int64_t i = 0; i < m; ++i) keymap_insert(&v->map, v->keys[i], i);
  free(drop);
}

/* voxel_hash_tsdf.h:113-123, cuda_tsdf_integrator.cu:905-930 */
int64_t vo_volume_observed_voxels(const vo_volume* v) {
  int64_t n = 0;
  for (int64_t i = 0; i < v->count * BLOCK_VOLUME; ++i) {
    const vo_voxel* vx = &v->voxels[i];
    int obs = 0;
    for (int d = 0; d < DIRS && !obs; ++d)
      for (int l = 0; l < LAYERS; ++l)
        if (vx->layers[d][l].weight > 0.0f) {
          obs = 1;
          break;
        }
    n += obs;
  }
  return n;
}

typedef struct {
  vo_volume* vol;
  const int64_t* idx;
  const float* depth;
  const float* nmap; /* normal_mode 1: the per-pixel normal map of depth */
  const vo_intrinsics* K;
  const vo_pose* T_wc;
  vo_pose T_cw;
} integ_ctx;

/* one block: cuda_tsdf_integrator.cu:834-903 (one thread per voxel), voxel_hash_tsdf.h:985-1060 */
static void integrate_block(void* p, int64_t i) {
  integ_ctx* g = (integ_ctx*)p;
  vo_volume* vol = g->vol;
  const vo_config* c = &vol->cfg;
  const int fl = c->flavor;
  const int64_t bi = g->idx[i];
  const vo_key key = vol->keys[bi];
  vo_voxel* vox = &vol->voxels[bi * BLOCK_VOLUME];
  const real vs = vol->vs, trunc = vol->trunc;
  for (int lz = 0; lz < BLOCK; ++lz)
    for (int ly = 0; ly < BLOCK; ++ly)
      for (int lx = 0; lx < BLOCK; ++lx) {
        const v3 pw = mk(((real)(key.x * BLOCK + lx) + 0.5f) * vs, ((real)(key.y * BLOCK + ly) + 0.5f) * vs,
                         ((real)(key.z * BLOCK + lz) + 0.5f) * vs);
        const v3 pc = pose_point(&g->T_cw, pw);
        if (pc.z <= 0.0f) continue;
        real u = 0.0f, v = 0.0f;
        if (!project_point(pc, g->K, &u, &v)) continue;
        real d = 0.0f;
        if (!sample_bilinear(c, g->depth, g->K, u, v, &d)) continue;
        const real sd = d - pc.z;
        if (sd <= -trunc) continue;
        const v3 view = vnormalize(fl, pc);
        real view_w = 1.0f;
        v3 nc = vmul(view, -1.0f);
        if (c->normal_mode == 1 ? map_normal_o(g->nmap, g->K, (float)u, (float)v, &nc)
                                : surface_normal(c, g->depth, g->K, u, v, &nc))
          view_w = VO_FABS(vdot(nc, view));
        const real obs = vo_observation_weight(c, d, sd, trunc, view_w);
        if (obs <= 0.0f) continue;
        const v3 spc = back_project_cont(u, v, d, g->K);
        const v3 spw = pose_point(g->T_wc, spc);
        const v3 nw = vnormalize(fl, pose_vector(g->T_wc, nc));
        const int dir = dominant_direction(nw);
        if (dir < 0 || dir >= DIRS) continue;
        const real sc = coordinate_along(fl, spw, dir);
        const int li = lx + BLOCK * (ly + BLOCK * lz);
        if (c->layer_format == 1) {
          integrate_bin16_o(c, (float)vs, 1.0f / (float)vs, &vol->bins16[bi * BIN16_WORDS + ((size_t)li * DIRS + dir) * 8],
                            voxel_centre_f(key, li, (float)vs), dir, (float)sc, spw, nw, (float)obs);
        } else {
          integrate_sample(c, vs, &vox[li], dir, sc, spw, nw, obs);
        }
      }
  if (c->layer_format == 1) decode_block16(vol, bi);
}

void vo_volume_integrate_blocks(vo_volume* vol, const vo_key* keys, int64_t n, const float* depth,
                                const vo_intrinsics* K, const vo_pose* T_wc) {
  int64_t* idx = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) idx[i] = volume_ensure(vol, keys[i]);
  integ_ctx g;
  g.vol = vol;
  g.idx = idx;
  g.depth = depth;
  g.nmap = NULL;
  float* nmap = NULL;
  if (vol->cfg.normal_mode == 1) { /* the map over the frame, as the library's map pass */
    const size_t np = (size_t)K->width * (size_t)K->height;
    nmap = (float*)calloc(np * 4, sizeof(float));
    for (int y = 0; y < K->height; ++y)
      for (int x = 0; x < K->width; ++x) {
        v3 n = mk(0.0f, 0.0f, 0.0f);
        if (surface_normal(&vol->cfg, depth, K, (real)x, (real)y, &n)) {
          float* o = nmap + 4 * ((size_t)y * K->width + x);
          o[0] = (float)n.x;
          o[1] = (float)n.y;
          o[2] = (float)n.z;
          o[3] = 1.0f;
        }
      }
    g.nmap = nmap;
  }
  g.K = K;
  g.T_wc = T_wc;
  pose_inverse(T_wc, &g.T_cw);
  parallel_for(vol->cfg.threads, n, integrate_block, &g);
  free(nmap);
  free(idx);
}

/* GPU: cuda_tsdf_integrator.cu:946-1010 (filter -> allocate on the filtered depth -> cache -> integrate);
 * CPU: reconstruction_backend.cpp:259-267 + voxel_hash_tsdf.h:70-73, 133-139. */
int64_t vo_volume_integrate_frame(vo_volume* vol, const float* depth, const vo_intrinsics* K, const vo_pose* T_wc,
                                  int32_t stride) {
  const size_t n = (size_t)K->width * (size_t)K->height;
  if (n == 0) return 0;
  float* filtered = (float*)malloc(n * sizeof(float));
  vo_filter_depth(&vol->cfg, depth, K, filtered);
  keymap set;
  keymap_init(&set, 1024);
  if (vol->cfg.alloc_mode == 1) { /* truncation band: the same walk as vo_collect_band_blocks */
    const int s = stride > 1 ? stride : 1;
    const v3 cam = mk(T_wc->t[0], T_wc->t[1], T_wc->t[2]);
    const real bws = vol->vs * 8.0f;
    for (int v = 0; v < K->height; v += s)
      for (int u = 0; u < K->width; u += s) {
        const real d = filtered[(size_t)v * K->width + u];
        if (!(d > 0.0f)) continue;
        const v3 pw = pose_point(T_wc, back_project(u, v, d, K));
        const v3 ray = vnormalize(GPU, vsub(pw, cam));
        if (!insert_band(vsub(pw, vmul(ray, vol->trunc)), vadd(pw, vmul(ray, vol->trunc)), bws, &set)) {
          keymap_free(&set);
          free(filtered);
          return -1;
        }
      }
  } else if (!collect_into(&vol->cfg, filtered, K, T_wc, vol->vs, vol->trunc, stride, &set)) {
    keymap_free(&set);
    free(filtered);
    return -1;
  }
  vo_key* keys = (vo_key*)malloc((size_t)(set.count > 0 ? set.count : 1) * sizeof(vo_key));
  int64_t m = 0;
  for (int64_t i = 0; i < set.cap; ++i)
    if (set.vals[i] >= 0) keys[m++] = set.keys[i];
  keymap_free(&set);
  qsort(keys, (size_t)m, sizeof(vo_key), key_cmp);
  if (m > 0) vo_volume_integrate_blocks(vol, keys, m, filtered, K, T_wc);
  free(keys);
  free(filtered);
  return m;
}

/* --------------------------------------------------------- marching cubes */
/* The marching-cubes tables (three.js, MIT; reference marching_cubes_tables.h) shared with the
 * product: vh_mc_tables.h, generated by oracle/gen_mc_tables.py. */
#include "vh_mc_tables.h"

static const int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
static const int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                 {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

/* cuda_mesh_extractor.cu:188-211, voxel_hash_tsdf.h:941-950 */
static const vo_voxel* find_voxel(const vo_volume* v, int vx, int vy, int vz) {
  const vo_key k = {floor_div(vx, BLOCK), floor_div(vy, BLOCK), floor_div(vz, BLOCK)};
  const int64_t bi = keymap_find(&v->map, k);
  if (bi < 0) return NULL;
  const int li = positive_mod(vx, BLOCK) + BLOCK * (positive_mod(vy, BLOCK) + BLOCK * positive_mod(vz, BLOCK));
  return &v->voxels[bi * BLOCK_VOLUME + li];
}

/* cuda_mesh_extractor.cu:259-262, voxel_hash_tsdf.h:336-339 */
static inline real plane_sd(int fl, const vo_layer* L, v3 p) {
  const v3 n = unpack_normal(fl, 1, L->packed_normal);
  return n.x * p.x + n.y * p.y + n.z * p.z - L->plane_offset;
}

/* cuda_mesh_extractor.cu:305-356, voxel_hash_tsdf.h:423-477 */
static int complete_cube(real values[8], int valid[8]) {
  int cnt = 0;
  real sum = 0.0f;
  for (int c = 0; c < 8; ++c) {
    if (!valid[c]) continue;
    ++cnt;
    sum += values[c];
  }
  if (cnt == 8) return 1;
  if (cnt < 6) return 0;
  const real global = cnt > 0 ? (sum / (real)cnt) : 0.0f;
  for (int c = 0; c < 8; ++c) {
    if (valid[c]) continue;
    real ns = 0.0f;
    int nc = 0;
    for (int e = 0; e < 12; ++e) {
      const int c0 = kEdge[e][0], c1 = kEdge[e][1];
      int nb = -1;
      if (c0 == c) {
        nb = c1;
      } else if (c1 == c) {
        nb = c0;
      }
      if (nb < 0 || !valid[nb]) continue;
      ns += values[nb];
      ++nc;
    }
    values[c] = nc > 0 ? (ns / (real)nc) : global;
    valid[c] = 1;
  }
  return 1;
}

/* marching_cubes.h:34-46, cuda_mesh_extractor.cu:358-374 */
static inline v3 interp_vertex(v3 p0, v3 p1, real v0, real v1, real iso) {
  const real delta = v1 - v0;
  if (VO_FABS(delta) < 1e-6f) return p0;
  const real t = clamp_f((iso - v0) / delta, 0.0f, 1.0f);
  return mk(p0.x + (p1.x - p0.x) * t, p0.y + (p1.y - p0.y) * t, p0.z + (p1.z - p0.z) * t);
}

typedef struct {
  vo_triangle* t;
  int64_t n, cap;
} tri_buf;

static void tri_push(tri_buf* b, v3 a, v3 c, v3 d) {
  if (b->n == b->cap) {
    b->cap = b->cap ? b->cap * 2 : 64;
    b->t = (vo_triangle*)realloc(b->t, (size_t)b->cap * sizeof(vo_triangle));
  }
  vo_triangle* t = &b->t[b->n++];
  t->v[0] = a.x;
  t->v[1] = a.y;
  t->v[2] = a.z;
  t->v[3] = c.x;
  t->v[4] = c.y;
  t->v[5] = c.z;
  t->v[6] = d.x;
  t->v[7] = d.y;
  t->v[8] = d.z;
}

/* marching_cubes.h:48-94, cuda_mesh_extractor.cu:376-437 */
static void polygonise(const v3 pos[8], const real val[8], real iso, tri_buf* out) {
  int ci = 0;
  for (int c = 0; c < 8; ++c)
    if (val[c] < iso) ci |= (1 << c);
  const int em = vh_mc_edge_table[ci];
  if (em == 0) return;
  v3 ev[12];
  memset(ev, 0, sizeof(ev));
  for (int e = 0; e < 12; ++e) {
    if ((em & (1 << e)) == 0) continue;
    const int c0 = kEdge[e][0], c1 = kEdge[e][1];
    ev[e] = interp_vertex(pos[c0], pos[c1], val[c0], val[c1], iso);
  }
  for (int i = 0; i < 16; i += 3) {
    const int e0 = vh_mc_tri_table[ci][i];
    if (e0 < 0) break;
    tri_push(out, ev[e0], ev[vh_mc_tri_table[ci][i + 1]], ev[vh_mc_tri_table[ci][i + 2]]);
  }
}

typedef struct {
  const vo_volume* vol;
  real iso;
  int dir;
  tri_buf* bufs;
} mesh_ctx;

/* GPU: cuda_mesh_extractor.cu:439-551 (+ kernels :553-632); CPU: voxel_hash_tsdf.h:842-939 */
static void mesh_block(void* p, int64_t bi) {
  mesh_ctx* m = (mesh_ctx*)p;
  const vo_volume* vol = m->vol;
  const vo_config* c = &vol->cfg;
  const int fl = c->flavor, d = m->dir;
  const real vs = vol->vs;
  const real tol = fmax_f(1e-6f, vs * c->layer_extract_scale);
  const vo_key key = vol->keys[bi];
  tri_buf* out = &m->bufs[bi];
  out->n = 0;
  for (int lz = 0; lz < BLOCK; ++lz)
    for (int ly = 0; ly < BLOCK; ++ly)
      for (int lx = 0; lx < BLOCK; ++lx) {
        const int bx = key.x * BLOCK + lx, by = key.y * BLOCK + ly, bz = key.z * BLOCK + lz;
        v3 cc;
        if (fl == GPU) {
          cc = mk(((real)bx + 1.0f) * vs, ((real)by + 1.0f) * vs, ((real)bz + 1.0f) * vs);
        } else {
          cc = mk(((real)bx + 0.5f) * vs + 0.5f * vs, ((real)by + 0.5f) * vs + 0.5f * vs,
                  ((real)bz + 0.5f) * vs + 0.5f * vs);
        }
        const vo_voxel* corners[8];
        v3 pos[8];
        real cand[24];
        int nc = 0;
        for (int k = 0; k < 8; ++k) {
          const int vx = bx + kCorner[k][0], vy = by + kCorner[k][1], vz = bz + kCorner[k][2];
          pos[k] = mk(((real)vx + 0.5f) * vs, ((real)vy + 0.5f) * vs, ((real)vz + 0.5f) * vs);
          corners[k] = find_voxel(vol, vx, vy, vz);
          if (!corners[k]) continue;
          for (int l = 0; l < LAYERS; ++l) {
            const vo_layer* L = &corners[k]->layers[d][l];
            if (!(L->weight > 0.0f)) continue;
            if (nc < 24) cand[nc++] = plane_sd(fl, L, cc);
          }
        }
        if (nc <= 0) continue;
        /* insertion sort (GPU, :264-274); std::sort (CPU) yields the same order */
        for (int i = 1; i < nc; ++i) {
          const real x = cand[i];
          int j = i - 1;
          while (j >= 0 && cand[j] > x) {
            cand[j + 1] = cand[j];
            --j;
          }
          cand[j + 1] = x;
        }
        real centers[24];
        int sizes[24];
        int ncl = 0;
        for (int i = 0; i < nc; ++i) {
          const real key_i = cand[i];
          if (ncl == 0 || VO_FABS(key_i - centers[ncl - 1]) > tol) {
            centers[ncl] = key_i;
            sizes[ncl] = 1;
            ++ncl;
            continue;
          }
          const int last = ncl - 1;
          const int cnt = sizes[last];
          centers[last] = (centers[last] * (real)cnt + key_i) / (real)(cnt + 1);
          sizes[last] = cnt + 1;
        }
        for (int ci = 0; ci < ncl; ++ci) {
          const real sk = centers[ci];
          real values[8] = {0, 0, 0, 0, 0, 0, 0, 0};
          int valid[8] = {0, 0, 0, 0, 0, 0, 0, 0};
          for (int k = 0; k < 8; ++k) {
            if (!corners[k]) continue;
            int best = -1;
            real best_delta = fl == GPU ? 1e30f : FLT_MAX;
            for (int l = 0; l < LAYERS; ++l) {
              const vo_layer* L = &corners[k]->layers[d][l];
              if (!(L->weight > 0.0f)) continue;
              const real delta = VO_FABS(plane_sd(fl, L, cc) - sk);
              if (delta <= tol && delta < best_delta) {
                best_delta = delta;
                best = l;
              }
            }
            if (best < 0) continue;
            values[k] = plane_sd(fl, &corners[k]->layers[d][best], pos[k]);
            valid[k] = 1;
          }
          if (!complete_cube(values, valid)) continue;
          polygonise(pos, values, m->iso, out);
        }
      }
}

int64_t vo_volume_extract_mesh(const vo_volume* vol, float iso, vo_triangle** out) {
  const int64_t nb = vol->count;
  tri_buf* bufs = (tri_buf*)calloc((size_t)(nb > 0 ? nb : 1), sizeof(tri_buf));
  tri_buf all = {NULL, 0, 0};
  for (int d = 0; d < DIRS; ++d) {
    mesh_ctx m = {vol, iso, d, bufs};
    parallel_for(vol->cfg.threads, nb, mesh_block, &m);
    for (int64_t b = 0; b < nb; ++b) {
      for (int64_t i = 0; i < bufs[b].n; ++i) {
        if (all.n == all.cap) {
          all.cap = all.cap ? all.cap * 2 : 256;
          all.t = (vo_triangle*)realloc(all.t, (size_t)all.cap * sizeof(vo_triangle));
        }
        all.t[all.n++] = bufs[b].t[i];
      }
    }
  }
  for (int64_t b = 0; b < nb; ++b) free(bufs[b].t);
  free(bufs);
  *out = all.t;
  return all.n;
}

/* estimateSurfaceNormalCamera (cuda_tsdf_integrator.cu:754-832) at one image position, for the per-pixel
 * normal map's parity test: returns 1 and the camera-frame normal, or 0 where the reference fails. */
int32_t vo_surface_normal(const vo_config* c, const float* depth, const vo_intrinsics* K, float u, float v,
                          float n[3]) {
  v3 r = mk(0.0f, 0.0f, 0.0f);
  const int ok = surface_normal(c, depth, K, u, v, &r);
  n[0] = r.x;
  n[1] = r.y;
  n[2] = r.z;
  return ok;
}

/* ------------------------------------------------------------- ray-cast */
/* Restatement of the product's depth ray-cast (voxelhashmt_gb300/csrc/vh_raycast.cu), which has no reference
 * counterpart; it uses the reference's marching-cubes surface (planeSignedDistanceGpu with the mesh unpack,
 * cuda_mesh_extractor.cu:237-262) on the GPU flavour's voxels. */
typedef struct {
  const vo_volume* v;
  const vo_intrinsics* K;
  const vo_pose* T;
  real min_depth, max_depth, step;
  float* out;
} raycast_ctx;

static int ray_plane_distance(const vo_volume* v, int gx, int gy, int gz, v3 x, v3 dw, real* sdf) {
  const vo_key k = {floor_div(gx, BLOCK), floor_div(gy, BLOCK), floor_div(gz, BLOCK)};
  const int64_t bi = keymap_find(&v->map, k);
  if (bi < 0) return 0;
  const int li = positive_mod(gx, BLOCK) + BLOCK * (positive_mod(gy, BLOCK) + BLOCK * positive_mod(gz, BLOCK));
  const vo_voxel* vox = &v->voxels[bi * BLOCK_VOLUME + li];
  int any = 0;
  real best = 0.0f, best_w = 0.0f;
  for (int d = 0; d < DIRS; ++d) {
    for (int l = 0; l < LAYERS; ++l) {
      const vo_layer* L = &vox->layers[d][l];
      if (!(L->weight > 0.0f)) continue;
      const v3 n = unpack_normal(GPU, 1, L->packed_normal);
      if (!(vdot(n, dw) < 0.0f)) continue;
      if (!any || L->weight > best_w) {
        any = 1;
        best = n.x * x.x + n.y * x.y + n.z * x.z - L->plane_offset;
        best_w = L->weight;
      }
    }
  }
  *sdf = best;
  return any;
}

static int ray_blended_distance(const vo_volume* v, v3 x, v3 dw, real* sdf) {
  const real vs = v->vs;
  const real fx = x.x / vs - 0.5f, fy = x.y / vs - 0.5f, fz = x.z / vs - 0.5f;
  const int x0 = (int)VO_FLOOR(fx), y0 = (int)VO_FLOOR(fy), z0 = (int)VO_FLOOR(fz);
  const real tx = fx - (real)x0, ty = fy - (real)y0, tz = fz - (real)z0;
  real ws = 0.0f, acc = 0.0f;
  for (int k = 0; k < 8; ++k) {
    const int ax = k & 1, ay = (k >> 1) & 1, az = k >> 2;
    const real w = (ax ? tx : 1.0f - tx) * (ay ? ty : 1.0f - ty) * (az ? tz : 1.0f - tz);
    real s = 0.0f;
    if (!ray_plane_distance(v, x0 + ax, y0 + ay, z0 + az, x, dw, &s)) continue;
    acc += w * s;
    ws += w;
  }
  if (!(ws >= 0.5f)) return 0;
  *sdf = acc / ws;
  return 1;
}

static void raycast_row(void* p, int64_t row) {
  const raycast_ctx* c = (const raycast_ctx*)p;
  const vo_volume* v = c->v;
  const vo_intrinsics* K = c->K;
  const real vs = v->vs;
  for (int u = 0; u < K->width; ++u) {
    const v3 dc = mk(((real)u - K->cx) / K->fx, ((real)row - K->cy) / K->fy, 1.0f);
    const v3 dw = pose_vector(c->T, dc);
    const v3 o = mk(c->T->t[0], c->T->t[1], c->T->t[2]);
    const real dz = c->step * vs / vnorm(dc);
    real z = c->min_depth, prev_sdf = 0.0f, prev_z = 0.0f, result = 0.0f;
    int prev_ok = 0;
    for (int it = 0; it < (1 << 16) && z <= c->max_depth; ++it) {
      const v3 x = mk(o.x + dw.x * z, o.y + dw.y * z, o.z + dw.z * z);
      const int gx = (int)VO_FLOOR(x.x / vs), gy = (int)VO_FLOOR(x.y / vs), gz = (int)VO_FLOOR(x.z / vs);
      const int bx = floor_div(gx, BLOCK), by = floor_div(gy, BLOCK), bz = floor_div(gz, BLOCK);
      const vo_key k = {bx, by, bz};
      const int64_t bi = keymap_find(&v->map, k);
      if (bi < 0) {
        prev_ok = 0;
        real zexit = 3.0e38f;
        const int bb[3] = {bx, by, bz};
        const real oo[3] = {o.x, o.y, o.z}, dd[3] = {dw.x, dw.y, dw.z};
        for (int a = 0; a < 3; ++a) {
          if (dd[a] > 0.0f) zexit = VO_FMIN(zexit, ((real)((bb[a] + 1) * BLOCK) * vs - oo[a]) / dd[a]);
          if (dd[a] < 0.0f) zexit = VO_FMIN(zexit, ((real)(bb[a] * BLOCK) * vs - oo[a]) / dd[a]);
        }
        z = VO_FMAX(z + dz, zexit + 0.25f * dz);
        continue;
      }
      real sdf = 0.0f;
      if (!ray_blended_distance(v, x, dw, &sdf)) {
        prev_ok = 0;
        z += dz;
        continue;
      }
      if (prev_ok && prev_sdf > 0.0f && sdf <= 0.0f && prev_sdf - sdf <= v->trunc) {
        result = prev_z + (z - prev_z) * (prev_sdf / (prev_sdf - sdf));
        break;
      }
      prev_ok = 1;
      prev_sdf = sdf;
      prev_z = z;
      z += dz;
    }
    c->out[(size_t)row * (size_t)K->width + (size_t)u] = result;
  }
}

void vo_raycast_depth(const vo_volume* v, const vo_intrinsics* K, const vo_pose* T_wc, float min_depth, float max_depth,
                      float step_voxels, float* out) {
  raycast_ctx c = {v, K, T_wc, min_depth, max_depth, step_voxels, out};
  parallel_for(v->cfg.threads, K->height, raycast_row, &c);
}

/* ------------------------------------------------------------- synthetic renderer */
/* Host restatement of the device renderer (voxelhashmt_gb300/csrc/vh_render.cu, vh_render_depth): the analytic
 * scenes ray-cast with FP32 geometry (IEEE add, multiply, divide, square root, no contraction), then Box-Muller
 * noise in FP64 from a counter-based hash, with the renderer's own logarithm and cosine series.  The same
 * operations in the same order, with explicit float and double types (independent of VO_FP64), so the frames are
 * bit-identical to the device's.  The reference renders its demo frames the same way in spirit
 * (src/main.cpp:189-335: ray-primitive hits, camera z, Gaussian noise, dropouts). */
typedef struct {
  float x, y, z;
} rf3;
static inline rf3 rmk(float x, float y, float z) {
  rf3 r = {x, y, z};
  return r;
}
static inline float rdot(rf3 a, rf3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline rf3 rsub(rf3 a, rf3 b) { return rmk(a.x - b.x, a.y - b.y, a.z - b.z); }

static uint32_t r_lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7FEB352DU;
  x ^= x >> 15;
  x *= 0x846CA68BU;
  x ^= x >> 16;
  return x;
}
static double r_uniform01(uint32_t seed, uint32_t frame, uint32_t idx, uint32_t stream) {
  const uint32_t key = seed * 0x9E3779B1U + frame * 0x85EBCA77U + stream * 0xC2B2AE3DU;
  const uint32_t h = r_lowbias32(idx ^ r_lowbias32(key));
  return ((double)h + 0.5) * 0x1p-32;
}
static const double r_atanh_c[11] = {0x1.0000000000000p+0, 0x1.5555555555555p-2, 0x1.999999999999ap-3,
                                     0x1.2492492492492p-3, 0x1.c71c71c71c71cp-4, 0x1.745d1745d1746p-4,
                                     0x1.3b13b13b13b14p-4, 0x1.1111111111111p-4, 0x1.e1e1e1e1e1e1ep-5,
                                     0x1.af286bca1af28p-5, 0x1.8618618618618p-5};
static const double r_cos_c[10] = {0x1.0000000000000p+0, 0x1.0000000000000p-1, 0x1.5555555555555p-5,
                                   0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-16, 0x1.27e4fb7789f5cp-22,
                                   0x1.1eed8eff8d898p-29, 0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-45,
                                   0x1.6827863b97d97p-53};
static const double r_sin_c[10] = {0x1.0000000000000p+0, 0x1.5555555555555p-3, 0x1.1111111111111p-7,
                                   0x1.a01a01a01a01ap-13, 0x1.71de3a556c734p-19, 0x1.ae64567f544e4p-26,
                                   0x1.6124613a86d09p-33, 0x1.ae7f3e733b81fp-41, 0x1.952c77030ad4ap-49,
                                   0x1.2f49b46814157p-57};
static double r_noise_log(double u) {
  int e = 0;
  double m = frexp(u, &e);
  if (m < 0x1.6a09e667f3bcdp-1) {
    m = m * 2.0;
    e -= 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double q = r_atanh_c[10];
  for (int k = 9; k >= 0; --k) q = q * s2 + r_atanh_c[k];
  return (double)e * 0x1.62e42fefa39efp-1 + 2.0 * (s * q);
}
static double r_noise_cos2pi(double w) {
  double a = fabs(w >= 0.5 ? w - 1.0 : w);
  double sign = 1.0;
  if (a > 0.25) {
    a = 0.5 - a;
    sign = -1.0;
  }
  double r;
  if (a <= 0.125) {
    const double x = 0x1.921fb54442d18p+2 * a, x2 = x * x;
    double q = r_cos_c[9];
    for (int k = 8; k >= 0; --k) q = q * -x2 + r_cos_c[k];
    r = q;
  } else {
    const double y = 0x1.921fb54442d18p+2 * (0.25 - a), y2 = y * y;
    double q = r_sin_c[9];
    for (int k = 8; k >= 0; --k) q = q * -y2 + r_sin_c[k];
    r = y * q;
  }
  return sign * r;
}
static float r_intersect(const float* pr, rf3 o, rf3 d) {
  const float kInf = 3.0e38f, kEps = 1e-4f;
  const int kind = (int)pr[0];
  const rf3 a = rmk(pr[1], pr[2], pr[3]);
  const rf3 b = rmk(pr[4], pr[5], pr[6]);
  const float r = pr[7], h = pr[8];
  if (kind == 0) {
    const float den = rdot(d, a);
    if (fabsf(den) < 1e-12f) return kInf;
    const float t = (r - rdot(o, a)) / den;
    return t > kEps ? t : kInf;
  }
  if (kind == 1) {
    const rf3 oc = rsub(o, a);
    const float bb = rdot(d, oc);
    const float c = rdot(oc, oc) - r * r;
    const float disc = bb * bb - c;
    if (disc < 0.0f) return kInf;
    const float sq = sqrtf(disc);
    const float t0 = -bb - sq, t1 = -bb + sq;
    const float t = t0 > kEps ? t0 : t1;
    return t > kEps ? t : kInf;
  }
  if (kind == 2 || kind == 4) {
    float tmin = -kInf, tmax = kInf;
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z}, lo[3] = {a.x, a.y, a.z}, hi[3] = {b.x, b.y, b.z};
    for (int k = 0; k < 3; ++k) {
      if (fabsf(dd[k]) < 1e-12f) {
        if (oo[k] < lo[k] || oo[k] > hi[k]) return kInf;
        continue;
      }
      const float inv = 1.0f / dd[k];
      float t0 = (lo[k] - oo[k]) * inv, t1 = (hi[k] - oo[k]) * inv;
      if (t0 > t1) {
        const float t = t0;
        t0 = t1;
        t1 = t;
      }
      tmin = fmaxf(tmin, t0);
      tmax = fminf(tmax, t1);
    }
    if (kind == 2) {
      if (tmax < tmin || tmax <= kEps) return kInf;
      return tmin > kEps ? tmin : tmax;
    }
    return tmax > kEps ? tmax : kInf;
  }
  if (kind == 3) {
    const float ox = o.x - a.x, oy = o.y - a.y;
    const float qa = d.x * d.x + d.y * d.y;
    const float qb = ox * d.x + oy * d.y;
    const float qc = ox * ox + oy * oy - r * r;
    float best = kInf;
    const float disc = qb * qb - qa * qc;
    if (qa > 1e-12f && disc >= 0.0f) {
      const float sq = sqrtf(disc);
      const float ts[2] = {(-qb - sq) / qa, (-qb + sq) / qa};
      for (int k = 0; k < 2; ++k) {
        const float z = o.z + ts[k] * d.z;
        if (ts[k] > kEps && z >= a.z && z <= a.z + h && ts[k] < best) best = ts[k];
      }
    }
    if (fabsf(d.z) > 1e-12f) {
      const float zc[2] = {a.z, a.z + h};
      for (int k = 0; k < 2; ++k) {
        const float t = (zc[k] - o.z) / d.z;
        const float px = ox + t * d.x, py = oy + t * d.y;
        if (t > kEps && px * px + py * py <= r * r && t < best) best = t;
      }
    }
    return best;
  }
  return kInf;
}
void vo_render_depth(const float* prims, int32_t n_prims, const vo_intrinsics* K, const vo_pose* T_wc, uint32_t seed,
                     uint32_t frame, float sigma_z2, float dropout, float max_depth, float* out) {
  const float kInf = 3.0e38f;
  const int n = K->width * K->height;
  const float* R = T_wc->R;
  const rf3 o = rmk(T_wc->t[0], T_wc->t[1], T_wc->t[2]);
  for (int i = 0; i < n; ++i) {
    const int u = i % K->width, v = i / K->width;
    rf3 dc = rmk(((float)u - K->cx) / K->fx, ((float)v - K->cy) / K->fy, 1.0f);
    const float inv = 1.0f / sqrtf(rdot(dc, dc));
    dc = rmk(dc.x * inv, dc.y * inv, dc.z * inv);
    const rf3 dw = rmk(R[0] * dc.x + R[1] * dc.y + R[2] * dc.z, R[3] * dc.x + R[4] * dc.y + R[5] * dc.z,
                       R[6] * dc.x + R[7] * dc.y + R[8] * dc.z);
    float t = kInf;
    for (int k = 0; k < n_prims; ++k) t = fminf(t, r_intersect(prims + 10 * k, o, dw));
    float z = t < kInf ? t * dc.z : 0.0f;
    if (z > 0.0f && sigma_z2 > 0.0f) {
      const double u1 = r_uniform01(seed, frame, (uint32_t)i, 0U);
      const double u2 = r_uniform01(seed, frame, (uint32_t)i, 1U);
      const double g = sqrt(-2.0 * r_noise_log(u1)) * r_noise_cos2pi(u2);
      const double zd = (double)z;
      z = (float)(zd + ((g * (double)sigma_z2) * zd) * zd);
    }
    if (r_uniform01(seed, frame, (uint32_t)i, 2U) < (double)dropout) z = 0.0f;
    if (z < 0.1f || z > max_depth) z = 0.0f;
    out[i] = z;
  }
}
