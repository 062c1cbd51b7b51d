// vh_render.cu -- synthetic depth renderer for the analytic benchmark scenes (one thread per pixel).
//
// The reference ray-casts its demo scene on the CPU (src/main.cpp:189-335: ray-sphere, ray-AABB, depth =
// camera-space z, Gaussian noise, random dropouts).  This kernel renders the scenes of
// voxelhashmt_gb300/scenes.py (plane, sphere, box, vertical cylinder, room interior) with the same counter-
// based noise (lowbias32 hash of (seed, frame, pixel), Box-Muller, sigma = k z^2, dropouts), so frames can be
// generated on the device at the rate the fusion path consumes them.
//
// Reproducible on a host: the ray geometry is FP32 with only IEEE-rounded additions, multiplications,
// divisions and square roots (the library is compiled without contraction), and the noise is FP64 with its
// own logarithm and cosine built from the same basic operations, so a host program that performs the same
// operations in the same order (the oracle's vo_render_depth) renders bit-identical frames.
#include "vh_common.cuh"
#include "vh_kernels.h"

namespace vh {
namespace {

constexpr int kPrimFields = 10;
constexpr float kEps = 1e-4f;
constexpr float kInf = 3.0e38f;

__device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7FEB352DU;
  x ^= x >> 15;
  x *= 0x846CA68BU;
  x ^= x >> 16;
  return x;
}

// (h + 0.5) / 2^32 for the hash h of (seed, frame, pixel, stream): exact in double, in (0, 1)
__device__ __forceinline__ double uniform01(uint32_t seed, uint32_t frame, uint32_t idx, uint32_t stream) {
  const uint32_t key = seed * 0x9E3779B1U + frame * 0x85EBCA77U + stream * 0xC2B2AE3DU;
  const uint32_t h = lowbias32(idx ^ lowbias32(key));
  return __dmul_rn(__dadd_rn(static_cast<double>(h), 0.5), 0x1p-32);
}

// 1 / (2k + 1), k = 0..10 (the atanh series) and 1 / (2k)!, 1 / (2k + 1)!, k = 0..9, correctly rounded
__constant__ double kAtanhC[11] = {0x1.0000000000000p+0, 0x1.5555555555555p-2, 0x1.999999999999ap-3,
                                   0x1.2492492492492p-3, 0x1.c71c71c71c71cp-4, 0x1.745d1745d1746p-4,
                                   0x1.3b13b13b13b14p-4, 0x1.1111111111111p-4, 0x1.e1e1e1e1e1e1ep-5,
                                   0x1.af286bca1af28p-5, 0x1.8618618618618p-5};
__constant__ double kCosC[10] = {0x1.0000000000000p+0, 0x1.0000000000000p-1, 0x1.5555555555555p-5,
                                 0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-16, 0x1.27e4fb7789f5cp-22,
                                 0x1.1eed8eff8d898p-29, 0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-45,
                                 0x1.6827863b97d97p-53};
__constant__ double kSinC[10] = {0x1.0000000000000p+0, 0x1.5555555555555p-3, 0x1.1111111111111p-7,
                                 0x1.a01a01a01a01ap-13, 0x1.71de3a556c734p-19, 0x1.ae64567f544e4p-26,
                                 0x1.6124613a86d09p-33, 0x1.ae7f3e733b81fp-41, 0x1.952c77030ad4ap-49,
                                 0x1.2f49b46814157p-57};
constexpr double kLn2 = 0x1.62e42fefa39efp-1;
constexpr double kTwoPi = 0x1.921fb54442d18p+2;

// ln u for u in (0, 1]: u = m 2^e with m in [sqrt(1/2), sqrt(2)), ln u = e ln 2 + 2 atanh(s) with
// s = (m - 1) / (m + 1), |s| <= 0.1716, the atanh series to s^21 in Horner form
__device__ double noise_log(double u) {
  int e = 0;
  double m = frexp(u, &e);  // m in [0.5, 1), exact
  if (m < 0x1.6a09e667f3bcdp-1) {
    m = __dmul_rn(m, 2.0);
    e -= 1;
  }
  const double s = __ddiv_rn(__dadd_rn(m, -1.0), __dadd_rn(m, 1.0));
  const double s2 = __dmul_rn(s, s);
  double q = kAtanhC[10];
  for (int k = 9; k >= 0; --k) q = __dadd_rn(__dmul_rn(q, s2), kAtanhC[k]);
  return __dadd_rn(__dmul_rn(static_cast<double>(e), kLn2), __dmul_rn(2.0, __dmul_rn(s, q)));
}

// cos(2 pi w) for w in [0, 1): folded exactly to a in [0, 1/4], then the cosine series of 2 pi a (a <= 1/8) or
// the sine series of 2 pi (1/4 - a), each to the 19th power
__device__ double noise_cos2pi(double w) {
  double a = fabs(w >= 0.5 ? __dadd_rn(w, -1.0) : w);
  double sign = 1.0;
  if (a > 0.25) {
    a = __dadd_rn(0.5, -a);
    sign = -1.0;
  }
  double r;
  if (a <= 0.125) {
    const double x = __dmul_rn(kTwoPi, a), x2 = __dmul_rn(x, x);
    double q = kCosC[9];
    for (int k = 8; k >= 0; --k) q = __dadd_rn(__dmul_rn(q, -x2), kCosC[k]);
    r = q;
  } else {
    const double y = __dmul_rn(kTwoPi, __dadd_rn(0.25, -a)), y2 = __dmul_rn(y, y);
    double q = kSinC[9];
    for (int k = 8; k >= 0; --k) q = __dadd_rn(__dmul_rn(q, -y2), kSinC[k]);
    r = __dmul_rn(y, q);
  }
  return __dmul_rn(sign, r);
}

__device__ float intersect(const float* pr, f3 o, f3 d) {
  const int kind = static_cast<int>(pr[0]);
  const f3 a = mk3(pr[1], pr[2], pr[3]);
  const f3 b = mk3(pr[4], pr[5], pr[6]);
  const float r = pr[7], h = pr[8];
  if (kind == 0) {  // plane n.p = r
    const float den = dot3(d, a);
    if (fabsf(den) < 1e-12f) return kInf;
    const float t = (r - dot3(o, a)) / den;
    return t > kEps ? t : kInf;
  }
  if (kind == 1) {  // sphere
    const f3 oc = sub3(o, a);
    const float bb = dot3(d, oc);
    const float c = dot3(oc, oc) - r * r;
    const float disc = bb * bb - c;
    if (disc < 0.0f) return kInf;
    const float sq = sqrtf(disc);
    const float t0 = -bb - sq, t1 = -bb + sq;
    const float t = t0 > kEps ? t0 : t1;
    return t > kEps ? t : kInf;
  }
  if (kind == 2 || kind == 4) {  // box / room interior
    float tmin = -kInf, tmax = kInf;
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z}, lo[3] = {a.x, a.y, a.z}, hi[3] = {b.x, b.y, b.z};
#pragma unroll
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
  if (kind == 3) {  // vertical cylinder: base centre a, radius r, height h, with caps
    const float ox = o.x - a.x, oy = o.y - a.y;
    const float qa = d.x * d.x + d.y * d.y;
    const float qb = ox * d.x + oy * d.y;
    const float qc = ox * ox + oy * oy - r * r;
    float best = kInf;
    const float disc = qb * qb - qa * qc;
    if (qa > 1e-12f && disc >= 0.0f) {
      const float sq = sqrtf(disc);
      const float ts[2] = {(-qb - sq) / qa, (-qb + sq) / qa};
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const float z = o.z + ts[k] * d.z;
        if (ts[k] > kEps && z >= a.z && z <= a.z + h && ts[k] < best) best = ts[k];
      }
    }
    if (fabsf(d.z) > 1e-12f) {
      const float zc[2] = {a.z, a.z + h};
#pragma unroll
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

__global__ void __launch_bounds__(256) render_kernel(const float* __restrict__ prims, int n_prims, const Params p,
                                                     uint32_t seed, uint32_t frame, float sigma_z2, float dropout,
                                                     float max_depth, float* __restrict__ out) {
  extern __shared__ float s_prims[];
  for (int i = threadIdx.x; i < n_prims * kPrimFields; i += blockDim.x) s_prims[i] = prims[i];
  __syncthreads();
  const int n = p.width * p.height;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int u = i % p.width, v = i / p.width;
    f3 dc = mk3((static_cast<float>(u) - p.cx) / p.fx, (static_cast<float>(v) - p.cy) / p.fy, 1.0f);
    const float inv = 1.0f / sqrtf(dot3(dc, dc));
    dc = mul3(dc, inv);
    const f3 dw = xform_vector(p.T_wc, dc);
    const f3 o = mk3(p.T_wc.t[0], p.T_wc.t[1], p.T_wc.t[2]);
    float t = kInf;
    for (int k = 0; k < n_prims; ++k) t = fminf(t, intersect(s_prims + k * kPrimFields, o, dw));
    float z = t < kInf ? t * dc.z : 0.0f;
    if (z > 0.0f && sigma_z2 > 0.0f) {
      const double u1 = uniform01(seed, frame, static_cast<uint32_t>(i), 0U);
      const double u2 = uniform01(seed, frame, static_cast<uint32_t>(i), 1U);
      const double g = __dmul_rn(__dsqrt_rn(__dmul_rn(-2.0, noise_log(u1))), noise_cos2pi(u2));
      const double zd = static_cast<double>(z);
      z = __double2float_rn(__dadd_rn(zd, __dmul_rn(__dmul_rn(__dmul_rn(g, static_cast<double>(sigma_z2)), zd), zd)));
    }
    if (uniform01(seed, frame, static_cast<uint32_t>(i), 2U) < static_cast<double>(dropout)) z = 0.0f;
    if (z < 0.1f || z > max_depth) z = 0.0f;
    out[i] = z;
  }
}

}  // namespace

cudaError_t launch_render(const float* prims, int n_prims, const Params& p, uint32_t seed, uint32_t frame,
                          float sigma_z2, float dropout, float max_depth, float* out, cudaStream_t s) {
  const int n = p.width * p.height;
  const int grid = (n + 255) / 256;
  render_kernel<<<grid, 256, n_prims * kPrimFields * sizeof(float), s>>>(prims, n_prims, p, seed, frame, sigma_z2,
                                                                          dropout, max_depth, out);
  return cudaGetLastError();
}

}  // namespace vh
