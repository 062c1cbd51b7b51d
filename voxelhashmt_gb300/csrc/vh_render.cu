// vh_render.cu -- synthetic depth renderer for the analytic benchmark scenes (one thread per pixel).
//
// The reference ray-casts its demo scene on the CPU (src/main.cpp:189-335: ray-sphere, ray-AABB, depth =
// camera-space z, Gaussian noise, random dropouts).  This kernel renders the scenes of
// voxelhashmt_gb300/scenes.py (plane, sphere, box, vertical cylinder, room interior) with the same counter-
// based noise (lowbias32 hash of (seed, frame, pixel), Box-Muller, sigma = k z^2, dropouts), so frames can be
// generated on the device at the rate the fusion path consumes them.
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

__device__ __forceinline__ float uniform01(uint32_t seed, uint32_t frame, uint32_t idx, uint32_t stream) {
  const uint32_t key = seed * 0x9E3779B1U + frame * 0x85EBCA77U + stream * 0xC2B2AE3DU;
  const uint32_t h = lowbias32(idx ^ lowbias32(key));
  return (static_cast<float>(h) + 0.5f) * 2.3283064365386963e-10f;
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
    const float inv = rsqrtf(dot3(dc, dc));
    dc = mul3(dc, inv);
    const f3 dw = xform_vector(p.T_wc, dc);
    const f3 o = mk3(p.T_wc.t[0], p.T_wc.t[1], p.T_wc.t[2]);
    float t = kInf;
    for (int k = 0; k < n_prims; ++k) t = fminf(t, intersect(s_prims + k * kPrimFields, o, dw));
    float z = t < kInf ? t * dc.z : 0.0f;
    if (z > 0.0f && sigma_z2 > 0.0f) {
      const float u1 = uniform01(seed, frame, static_cast<uint32_t>(i), 0U);
      const float u2 = uniform01(seed, frame, static_cast<uint32_t>(i), 1U);
      const float g = sqrtf(-2.0f * logf(u1)) * cosf(6.283185307179586f * u2);
      z = z + g * sigma_z2 * z * z;
    }
    if (uniform01(seed, frame, static_cast<uint32_t>(i), 2U) < dropout) z = 0.0f;
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
