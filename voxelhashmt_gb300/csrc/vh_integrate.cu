// vh_integrate.cu -- directional multi-layer TSDF update of the visible blocks.
//
// Reference: integrateActiveBlocksKernel (src/cuda_tsdf_integrator.cu:834-903) with its helpers
// (:319-568, :727-832), one CTA per active block and one thread per voxel.  Here the same per-voxel function
// runs as two persistent grid-stride passes whose launches need no host read-back: classify_kernel runs the
// cheap prefix (projection, bilinear depth, truncation test) over every voxel of the visible blocks and
// compacts the survivors into an active-voxel list; update_kernel runs the bilateral normal and the layer
// update over that list, one voxel per thread.  Layer storage is direction-major (vh_common.cuh), so a warp
// of neighbouring voxels with the same dominant direction reads and writes its 3 layers as 16-byte vector
// accesses over contiguous memory; a voxel's other 5 bins are never touched.  The observed-voxel bitmask
// keeps the observed-voxel count incremental.
//
// The per-voxel bilateral normal (estimateSurfaceNormalCamera, :754-832) evaluates 9 base normals, each from
// 4 bilinear depth samples, plus 10 more samples: 50 bilinear samples per voxel, all at (u + i, v + j) for
// integer i, j in [-2, 2].  Whenever the shifted coordinates are exact -- (u-1)+1 == u, (u+1)-1 == u and the
// same for v, which the kernel checks -- the reference evaluates every one of those samples at the same
// float coordinates, so the 21 distinct samples are computed once and reused; the result is bit-identical.
// Otherwise (u or v within 2 of a power of two, or below 1) the literal 50-sample sequence runs.
//
// The per-pixel normal-map form (Params::normal_mode 1) runs map_prepare_kernel (the normal map once per
// pixel, plus the visible list's {block key, pool index} entries) and fused_update_kernel (prefix, a
// shared-memory queue of the survivors and their update with the bilinearly interpolated map normal, from a
// device work queue of voxel-slot chunks).  filter_alloc_kernel filters a frame's depth and allocates its
// blocks tile by tile in one pass, and the batch_* kernels run the same device code as work-queue kernels
// over many volumes.
//
// The file is compiled twice: as vh::exact (the bit-reproducible FP32 form: -fmad=false, IEEE division and
// square root, vh_expf) and, with VH_FAST_MATH, as vh::fast (fused multiply-adds, approximate division, square
// root and exponential; selected per volume by vh_algorithm.fast_math).
#include "vh_alloc.cuh"
#include "vh_common.cuh"
#include "vh_filter.cuh"
#include "vh_kernels.h"

#ifdef VH_FAST_MATH
#define VH_INTEGRATE_NS fast
#else
#define VH_INTEGRATE_NS exact
#endif

namespace vh {
namespace VH_INTEGRATE_NS {
namespace {

constexpr int kThreads = 256;

// sampleDepthNearest (cuda_tsdf_integrator.cu:479-489)
__device__ __forceinline__ bool sample_nearest(const float* __restrict__ depth, const Params& p, float u, float v,
                                               float& d) {
  const int ui = static_cast<int>(floorf(u + 0.5f));
  const int vi = static_cast<int>(floorf(v + 0.5f));
  if (ui < 0 || ui >= p.width || vi < 0 || vi >= p.height) return false;
  d = __ldg(&depth[static_cast<size_t>(vi) * p.width + ui]);
  return d > 0.0f;
}

// sampleDepthBilinear (cuda_tsdf_integrator.cu:504-568)
__device__ __forceinline__ bool sample_bilinear(const float* __restrict__ depth, const Params& p, float u, float v,
                                                float& out) {
  if (u < 0.0f || v < 0.0f || u > static_cast<float>(p.width - 1) || v > static_cast<float>(p.height - 1)) {
    return false;
  }
  const int x0 = static_cast<int>(floorf(u));
  const int y0 = static_cast<int>(floorf(v));
  const int x1 = min(x0 + 1, p.width - 1);
  const int y1 = min(y0 + 1, p.height - 1);
  const float tx = u - static_cast<float>(x0);
  const float ty = v - static_cast<float>(y0);
  const float* r0 = depth + static_cast<size_t>(y0) * p.width;
  const float* r1 = depth + static_cast<size_t>(y1) * p.width;
  const float d00 = __ldg(r0 + x0), d10 = __ldg(r0 + x1), d01 = __ldg(r1 + x0), d11 = __ldg(r1 + x1);
  if (d00 > 0.0f && d10 > 0.0f && d01 > 0.0f && d11 > 0.0f) {
    // sampleDepthNearest always lands on one of the four taps here (u <= W-1 keeps floor(u+0.5) <= x0+1 and
    // x1 == x0 only when u == W-1), and all four are valid: select it instead of reloading.
    const int ui = static_cast<int>(floorf(u + 0.5f));
    const int vi = static_cast<int>(floorf(v + 0.5f));
    const float ref = (ui == x0) ? (vi == y0 ? d00 : d01) : (vi == y0 ? d10 : d11);
    const float thr = disc_threshold(p, ref);
    const float mn = fminf(fminf(d00, d10), fminf(d01, d11));
    const float mx = fmaxf(fmaxf(d00, d10), fmaxf(d01, d11));
    const float top = d00 + (d10 - d00) * tx;
    const float bottom = d01 + (d11 - d01) * tx;
    if (mx - mn <= thr) {
      out = top + (bottom - top) * ty;
      return true;
    }
    const float w00 = (1.0f - tx) * (1.0f - ty), w10 = tx * (1.0f - ty), w01 = (1.0f - tx) * ty, w11 = tx * ty;
    float wds = 0.0f, ws = 0.0f;
    if (!(fabsf(d00 - ref) > thr)) {
      wds += w00 * d00;
      ws += w00;
    }
    if (!(fabsf(d10 - ref) > thr)) {
      wds += w10 * d10;
      ws += w10;
    }
    if (!(fabsf(d01 - ref) > thr)) {
      wds += w01 * d01;
      ws += w01;
    }
    if (!(fabsf(d11 - ref) > thr)) {
      wds += w11 * d11;
      ws += w11;
    }
    if (ws > 1e-6f) {
      out = wds / ws;
      return true;
    }
  }
  return sample_nearest(depth, p, u, v, out);
}

// estimateSurfaceNormalBaseCamera (cuda_tsdf_integrator.cu:727-752)
__device__ __noinline__ bool base_normal_literal(const float* __restrict__ depth, const Params& p, float u, float v, f3& n) {
  float dl, dr, du, dd;
  if (!sample_bilinear(depth, p, u - 1.0f, v, dl) || !sample_bilinear(depth, p, u + 1.0f, v, dr) ||
      !sample_bilinear(depth, p, u, v - 1.0f, du) || !sample_bilinear(depth, p, u, v + 1.0f, dd)) {
    return false;
  }
  const f3 pl = backproject(u - 1.0f, v, dl, p);
  const f3 pr = backproject(u + 1.0f, v, dr, p);
  const f3 pu = backproject(u, v - 1.0f, du, p);
  const f3 pd = backproject(u, v + 1.0f, dd, p);
  n = normalize3(cross3(sub3(pd, pu), sub3(pr, pl)));
  return norm3(n) > 1e-6f;
}

// estimateSurfaceNormalCamera (cuda_tsdf_integrator.cu:754-832), literal evaluation order
__device__ __noinline__ bool surface_normal_literal(const float* __restrict__ depth, const Params& p, float u,
                                                    float v, const float gs[3], f3& normal) {
  f3 cn;
  if (!base_normal_literal(depth, p, u, v, cn)) return false;
  float cd;
  if (!sample_bilinear(depth, p, u, v, cd)) return false;
  const f3 cp = backproject(u, v, cd, p);
  cn = orient_toward_camera(cn, cp);
  f3 wsum = mk3(0.0f, 0.0f, 0.0f);
  float ws = 0.0f;
  for (int dv = -1; dv <= 1; ++dv) {
    for (int du = -1; du <= 1; ++du) {
      const float su = u + static_cast<float>(du);
      const float sv = v + static_cast<float>(dv);
      f3 sn;
      if (!base_normal_literal(depth, p, su, sv, sn)) continue;
      float sd;
      if (!sample_bilinear(depth, p, su, sv, sd)) continue;
      sn = orient_toward_camera(sn, backproject(su, sv, sd, p));
      const float delta = sd - cd;
      const float cosine = clampf(dot3(cn, sn), -1.0f, 1.0f);
      const float ad = 1.0f - cosine;
      const float w = gs[du * du + dv * dv] * gaussian(delta * delta, p.normal_k_range) *
                      gaussian(ad * ad, p.normal_k_angular);
      wsum.x += sn.x * w;
      wsum.y += sn.y * w;
      wsum.z += sn.z * w;
      ws += w;
    }
  }
  if (ws <= 1e-6f) {
    normal = cn;
    return true;
  }
  const float inv = 1.0f / ws;
  f3 n = normalize3(mk3(wsum.x * inv, wsum.y * inv, wsum.z * inv));
  n = orient_toward_camera(n, cp);
  if (norm3(n) <= 1e-6f) n = cn;
  normal = n;
  return norm3(n) > 1e-6f;
}

// The 21 distinct sample positions (i, j) of the fast path, i, j in [0, 4] (offsets i-2, j-2): row 0 and row 4
// hold columns 1..3, rows 1..3 all five columns.
__device__ __forceinline__ void sample_position(int s, int& i, int& j) {
  if (s < 3) {
    j = 0;
    i = s + 1;
  } else if (s < 18) {
    j = 1 + (s - 3) / 5;
    i = (s - 3) % 5;
  } else {
    j = 4;
    i = s - 17;
  }
}
__device__ __forceinline__ int sample_slot(int i, int j) {
  return j == 0 ? i - 1 : (j == 4 ? 17 + i : 3 + (j - 1) * 5 + i);
}
__device__ __forceinline__ float pick5(int k, float a0, float a1, float a2, float a3, float a4) {
  return k == 0 ? a0 : (k == 1 ? a1 : (k == 2 ? a2 : (k == 3 ? a3 : a4)));
}

constexpr int kSamples = 21;

// Per-thread scratch of the fast path: backprojected sample points, [component][sample][thread] so a warp's
// accesses hit 32 consecutive words.
template <int kT>
struct NormalScratch {
  float x[kSamples][kT];
  float y[kSamples][kT];
  float z[kSamples][kT];
};

// estimateSurfaceNormalCamera through the 21 distinct samples, valid when the shifted coordinates are exact
// (checked by the caller).  Rolled loops keep the code small; the samples live in shared memory.
template <int kT>
__device__ __forceinline__ bool surface_normal_fast(const float* __restrict__ depth, const Params& p, float u, float v,
                                                    const float gs[3], NormalScratch<kT>& S, int t, f3& normal) {
  const float um1 = u - 1.0f, up1 = u + 1.0f, vm1 = v - 1.0f, vp1 = v + 1.0f;
  const float U0 = um1 - 1.0f, U4 = up1 + 1.0f, V0 = vm1 - 1.0f, V4 = vp1 + 1.0f;
  uint32_t ok = 0U;
#pragma unroll 1
  for (int s = 0; s < kSamples; ++s) {
    int i, j;
    sample_position(s, i, j);
    const float su = pick5(i, U0, um1, u, up1, U4);
    const float sv = pick5(j, V0, vm1, v, vp1, V4);
    float d;
    if (sample_bilinear(depth, p, su, sv, d)) {
      ok |= 1U << s;
      const f3 q = backproject(su, sv, d, p);
      S.x[s][t] = q.x;
      S.y[s][t] = q.y;
      S.z[s][t] = q.z;
    }
  }
  auto point = [&](int i, int j) {
    const int s = sample_slot(i, j);
    return mk3(S.x[s][t], S.y[s][t], S.z[s][t]);
  };
  auto valid = [&](int i, int j) { return (ok >> sample_slot(i, j)) & 1U; };
  // base normal at (i, j): estimateSurfaceNormalBaseCamera on the cached samples
  auto base = [&](int i, int j, f3& n) -> bool {
    if (!(valid(i - 1, j) && valid(i + 1, j) && valid(i, j - 1) && valid(i, j + 1))) return false;
    n = normalize3(cross3(sub3(point(i, j + 1), point(i, j - 1)), sub3(point(i + 1, j), point(i - 1, j))));
    return norm3(n) > 1e-6f;
  };
  f3 cn;
  if (!base(2, 2, cn)) return false;
  if (!valid(2, 2)) return false;
  const f3 cp = point(2, 2);
  const float cd = cp.z;
  cn = orient_unit_toward_camera(cn, cp);
  f3 wsum = mk3(0.0f, 0.0f, 0.0f);
  float ws = 0.0f;
#pragma unroll 1
  for (int k = 0; k < 9; ++k) {
    const int i = 1 + k % 3, j = 1 + k / 3;
    f3 sn;
    if (!base(i, j, sn)) continue;
    if (!valid(i, j)) continue;
    const f3 sp = point(i, j);
    sn = orient_unit_toward_camera(sn, sp);
    const float delta = sp.z - cd;
    const float cosine = clampf(dot3(cn, sn), -1.0f, 1.0f);
    const float ad = 1.0f - cosine;
    const int r2 = (i - 2) * (i - 2) + (j - 2) * (j - 2);
    const float w = pick5(r2, gs[0], gs[1], gs[2], 0.0f, 0.0f) * gaussian(delta * delta, p.normal_k_range) *
                    gaussian(ad * ad, p.normal_k_angular);
    wsum.x += sn.x * w;
    wsum.y += sn.y * w;
    wsum.z += sn.z * w;
    ws += w;
  }
  if (ws <= 1e-6f) {
    normal = cn;
    return true;
  }
  const float inv = 1.0f / ws;
  f3 n = normalize3(mk3(wsum.x * inv, wsum.y * inv, wsum.z * inv));
  n = orient_toward_camera(n, cp);
  if (norm3(n) <= 1e-6f) n = cn;
  normal = n;
  return norm3(n) > 1e-6f;
}

template <int kT>
__device__ __forceinline__ bool surface_normal(const float* __restrict__ depth, const Params& p, float u, float v,
                                               const float gs[3], NormalScratch<kT>& S, int t, f3& normal) {
  const float um1 = u - 1.0f, up1 = u + 1.0f, vm1 = v - 1.0f, vp1 = v + 1.0f;
  if (!(um1 + 1.0f == u && up1 - 1.0f == u && vm1 + 1.0f == v && vp1 - 1.0f == v)) {
    return surface_normal_literal(depth, p, u, v, gs, normal);
  }
  return surface_normal_fast<kT>(depth, p, u, v, gs, S, t, normal);
}

// computeObservationWeightGpu (cuda_tsdf_integrator.cu:429-450)
__device__ __forceinline__ float observation_weight(const Params& p, float depth, float sd, float view) {
  if (depth <= 0.0f || p.truncation <= 1e-6f) return 0.0f;
  const float dr = depth / p.depth_sigma;
  const float dw = 1.0f / (1.0f + dr * dr);
  const float nr = fabsf(sd) / p.truncation;
  float rw = 1.0f;
  if (nr > p.huber_delta) rw = p.huber_delta / nr;
  const float bw = 1.0f - 0.5f * clampf(nr, 0.0f, 1.0f);
  const float base = fmaxf(p.min_obs_weight, dw * rw * bw);
  const float aw = clampf(view, p.min_view_weight, 1.0f);
  return base * aw;
}

// dominantDirectionIndexGpu (:228-243)
__device__ __forceinline__ int dominant_direction(f3 n) {
  const float nx = fabsf(n.x), ny = fabsf(n.y), nz = fabsf(n.z);
  if (nx <= 1e-6f && ny <= 1e-6f && nz <= 1e-6f) return -1;
  if (nx >= ny && nx >= nz) return n.x >= 0.0f ? 0 : 1;
  if (ny >= nx && ny >= nz) return n.y >= 0.0f ? 2 : 3;
  return n.z >= 0.0f ? 4 : 5;
}

// coordinateAlongDirectionGpu (:296-313)
__device__ __forceinline__ float coordinate_along(f3 p, int d) {
  switch (d) {
    case 0: return p.x;
    case 1: return -p.x;
    case 2: return p.y;
    case 3: return -p.y;
    case 4: return p.z;
    default: return -p.z;
  }
}

__device__ __forceinline__ float sign_not_zero(float v) { return v >= 0.0f ? 1.0f : -1.0f; }

// packNormalOctahedralGpu (:253-278)
__device__ __forceinline__ uint32_t pack_normal(f3 raw) {
  const f3 n = normalize3(raw);
  const float s = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
  if (s <= 1e-6f) return 0U;
  float px = n.x / s, py = n.y / s;
  const float pz = n.z / s;
  if (pz < 0.0f) {
    const float fx = (1.0f - fabsf(py)) * sign_not_zero(px);
    const float fy = (1.0f - fabsf(px)) * sign_not_zero(py);
    px = fx;
    py = fy;
  }
  const uint32_t qx = static_cast<uint32_t>(floorf(fminf(1.0f, fmaxf(0.0f, px * 0.5f + 0.5f)) * 65535.0f + 0.5f));
  const uint32_t qy = static_cast<uint32_t>(floorf(fminf(1.0f, fmaxf(0.0f, py * 0.5f + 0.5f)) * 65535.0f + 0.5f));
  return qx | (qy << 16U);
}

// unpackNormalOctahedralGpu (:258-294)
__device__ __forceinline__ f3 unpack_normal(uint32_t packed) {
  f3 n = mk3(div65535(static_cast<float>(packed & 0xffffU)) * 2.0f - 1.0f,
             div65535(static_cast<float>((packed >> 16U) & 0xffffU)) * 2.0f - 1.0f, 0.0f);
  n.z = 1.0f - fabsf(n.x) - fabsf(n.y);
  if (n.z < 0.0f) {
    const float fx = (1.0f - fabsf(n.y)) * sign_not_zero(n.x);
    const float fy = (1.0f - fabsf(n.x)) * sign_not_zero(n.y);
    n.x = fx;
    n.y = fy;
  }
  return normalize3(n);
}

__device__ __forceinline__ bool layer_valid(const float4& l) { return l.x > 0.0f; }

__device__ __forceinline__ void cswap(float4& a, float4& b, bool c) {
  const float4 t = a;
  a = c ? b : a;
  b = c ? t : b;
}

// sortDirectionalLayersGpu (:319-336): bubble sort, observed layers first, ascending surface_coord
__device__ __forceinline__ void sort_layers(float4& a, float4& b, float4& c) {
  auto should = [](const float4& l, const float4& r) {
    const bool lv = layer_valid(l), rv = layer_valid(r);
    return (!lv && rv) || (lv && rv && l.y > r.y);
  };
  cswap(a, b, should(a, b));
  cswap(b, c, should(b, c));
  cswap(a, b, should(a, b));
}

// findLayerSlotForObservationGpu + integrateDirectionalSampleGpu (:338-427) on the 3 layers of one bin.
// Returns true when a layer was updated.
__device__ __forceinline__ bool integrate_sample(const Params& p, float4& L0, float4& L1, float4& L2, float sc,
                                                 f3 sp, f3 nw, float obs) {
  if (obs <= 0.0f) return false;
  const f3 n = normalize3(nw);
  if (norm3(n) <= 1e-6f) return false;
  const float plane_offset = dot3(n, sp);
  int empty = -1, best = -1;
  float best_delta = 1e30f;
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    const float4& L = l == 0 ? L0 : (l == 1 ? L1 : L2);
    if (!layer_valid(L)) {
      if (empty < 0) empty = l;
      continue;
    }
    const f3 ln = unpack_normal(__float_as_uint(L.w));
    if (dot3(ln, n) < p.layer_normal_cos) continue;
    const float delta = fabsf(L.y - sc);
    if (delta < best_delta) {
      best_delta = delta;
      best = l;
    }
  }
  const int li = (best >= 0 && best_delta <= p.merge_tol) ? best : empty;
  if (li < 0) return false;
  float4 L = li == 0 ? L0 : (li == 1 ? L1 : L2);
  const float pw = L.x;
  const float ew = fminf(obs, fmaxf(0.0f, p.max_weight - pw));
  if (ew <= 0.0f) return false;
  const float nwt = pw + ew;
  f3 blended = n;
  L.y = pw > 0.0f ? ((L.y * pw + sc * ew) / nwt) : sc;
  L.z = pw > 0.0f ? ((L.z * pw + plane_offset * ew) / nwt) : plane_offset;
  if (pw > 0.0f) {
    const f3 pn = unpack_normal(__float_as_uint(L.w));
    blended = normalize3(mul3(add3(mul3(pn, pw), mul3(n, ew)), 1.0f / nwt));
    if (norm3(blended) <= 1e-6f) blended = n;
  }
  L.x = nwt;
  L.w = __uint_as_float(pack_normal(blended));
  if (li == 0) L0 = L;
  if (li == 1) L1 = L;
  if (li == 2) L2 = L;
  sort_layers(L0, L1, L2);
  return true;
}

// integrate_sample on an FP16 bin (A, B): each observed layer's normal is unpacked once (for the match and
// for its plane offset), only the updated layer is re-encoded, and the three layers are re-sorted as raw
// binary16 triplets.  Same decisions and blending formulas as integrate_sample on the decoded records.
// Returns true when a layer was updated (A, B then hold the new bin).
__device__ __forceinline__ uint32_t cswap_u32(uint32_t& a, uint32_t& b, bool c) {
  const uint32_t t = a;
  a = c ? b : a;
  b = c ? t : b;
  return 0U;
}

__device__ __forceinline__ bool integrate_bin16(const Params& p, const Volume& V, uint4& A, uint4& B, f3 c, int dir,
                                                float sc, f3 sp, f3 nw, float obs) {
  if (obs <= 0.0f) return false;
  const f3 n = normalize3(nw);
  if (norm3(n) <= 1e-6f) return false;
  const float vs = V.voxel_size, inv_vs = V.inv_voxel_size;
  const float cd = axis_coordinate(c, dir);
  uint32_t w16[3] = {A.x & 0xffffU, A.y >> 16, A.w & 0xffffU};
  uint32_t s16[3] = {A.x >> 16, A.z & 0xffffU, A.w >> 16};
  uint32_t p16[3] = {A.y & 0xffffU, A.z >> 16, B.x & 0xffffU};
  uint32_t nk[3] = {B.y, B.z, B.w};
  float ls[3];
  f3 ln[3];
  int empty = -1, best = -1;
  float best_delta = 1e30f;
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    ls[l] = __fadd_rn(cd, __fmul_rn(h2f(s16[l]), vs));
    ln[l] = mk3(0.0f, 0.0f, 1.0f);
    if (w16[l] == 0U) {
      if (empty < 0) empty = l;
      continue;
    }
    // a layer farther than merge_tol from the sample can never be the merged one (the best match is taken
    // only within merge_tol), so its normal is not decoded: the decision is the same as testing it
    const float delta = fabsf(ls[l] - sc);
    if (!(delta <= p.merge_tol)) continue;
    ln[l] = bin_normal(nk[l]);
    if (dot3(ln[l], n) < p.layer_normal_cos) continue;
    if (delta < best_delta) {
      best_delta = delta;
      best = l;
    }
  }
  const int li = (best >= 0 && best_delta <= p.merge_tol) ? best : empty;
  if (li < 0) return false;
  const uint32_t wli = li == 0 ? w16[0] : (li == 1 ? w16[1] : w16[2]);
  const uint32_t pli = li == 0 ? p16[0] : (li == 1 ? p16[1] : p16[2]);
  const bool had = wli != 0U;
  const float pw = had ? h2f(wli) : 0.0f;
  const float ew = fminf(obs, fmaxf(0.0f, p.max_weight - pw));
  if (ew <= 0.0f) return false;
  const float nwt = pw + ew;
  const float plane_offset = dot3(n, sp);
  const f3 pn = li == 0 ? ln[0] : (li == 1 ? ln[1] : ln[2]);
  float new_s = sc, new_p = plane_offset;
  f3 blended = n;
  if (had) {
    const float old_s = li == 0 ? ls[0] : (li == 1 ? ls[1] : ls[2]);
    const float old_p = __fadd_rn(dot_rn(pn, c), __fmul_rn(h2f(pli), vs));
    new_s = (old_s * pw + sc * ew) / nwt;
    new_p = (old_p * pw + plane_offset * ew) / nwt;
    blended = normalize3(mul3(add3(mul3(pn, pw), mul3(n, ew)), 1.0f / nwt));
    if (norm3(blended) <= 1e-6f) blended = n;
  }
  const uint32_t packed = pack_normal(blended);
  uint32_t nwt16 = f2h(nwt);
  if (nwt16 == 0U) nwt16 = 1U;
  const uint32_t ns16 = f2h(__fmul_rn(__fadd_rn(new_s, -cd), inv_vs));
  const uint32_t np16 = f2h(__fmul_rn(__fadd_rn(new_p, -dot_rn(bin_normal(packed), c)), inv_vs));
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    if (l == li) {
      w16[l] = nwt16;
      s16[l] = ns16;
      p16[l] = np16;
      nk[l] = packed;
      ls[l] = new_s;
    }
  }
  // sortDirectionalLayersGpu's bubble network: observed layers first, ascending surface coordinate
  auto step = [&](int a, int b) {
    const bool av = w16[a] != 0U, bv = w16[b] != 0U;
    const bool sw = (!av && bv) || (av && bv && ls[a] > ls[b]);
    cswap_u32(w16[a], w16[b], sw);
    cswap_u32(s16[a], s16[b], sw);
    cswap_u32(p16[a], p16[b], sw);
    cswap_u32(nk[a], nk[b], sw);
    const float t = ls[a];
    ls[a] = sw ? ls[b] : ls[a];
    ls[b] = sw ? t : ls[b];
  };
  if (w16[1] != 0U || w16[2] != 0U) {  // with at most layer 0 observed the network swaps nothing
    step(0, 1);
    step(1, 2);
    step(0, 1);
  }
  A = make_uint4(w16[0] | (s16[0] << 16), p16[0] | (w16[1] << 16), s16[1] | (p16[1] << 16), w16[2] | (s16[2] << 16));
  B = make_uint4(p16[2], w16[0] ? nk[0] : 0U, w16[1] ? nk[1] : 0U, w16[2] ? nk[2] : 0U);
  return true;
}

// First part of integrateActiveBlocksKernel for one voxel (:849-877): voxel centre, projection, bilinear
// depth, truncation test.  Returns false when the reference returns before touching the voxel.
__device__ __forceinline__ bool voxel_prefix(const float* __restrict__ depth, const Params& p, const int4& bk, int li,
                                             f3& pc, float& u, float& v, float& d) {
  const int lx = li & 7, ly = (li >> 3) & 7, lz = li >> 6;
  const f3 pw = mk3((static_cast<float>(bk.x * kBlockSide + lx) + 0.5f) * p.voxel_size,
                    (static_cast<float>(bk.y * kBlockSide + ly) + 0.5f) * p.voxel_size,
                    (static_cast<float>(bk.z * kBlockSide + lz) + 0.5f) * p.voxel_size);
  pc = xform_point(p.T_cw, pw);
  if (pc.z <= 0.0f) return false;
  if (pc.z <= 1e-6f) return false;
  u = p.fx * pc.x / pc.z + p.cx;
  v = p.fy * pc.y / pc.z + p.cy;
  if (!(u >= 0.0f && u <= static_cast<float>(p.width - 1) && v >= 0.0f && v <= static_cast<float>(p.height - 1))) {
    return false;
  }
  if (!sample_bilinear(depth, p, u, v, d)) return false;
  return !(d - pc.z <= -p.truncation);
}

// Rest of integrateActiveBlocksKernel (:879-899): bilateral normal, observation weight, surface point,
// direction bin.  Returns the direction bin, or -1 when the reference skips the voxel.
template <int kT>
__device__ __forceinline__ int voxel_observation(const float* __restrict__ depth, const Params& p, f3 pc, float u,
                                                 float v, float d, const float gs[3], NormalScratch<kT>& S, int t,
                                                 float& sc, f3& spw, f3& nw, float& obs) {
  const float sd = d - pc.z;
  const f3 view = normalize3(pc);
  float view_w = 1.0f;
  f3 nc = mul3(view, -1.0f);
  if (surface_normal<kT>(depth, p, u, v, gs, S, t, nc)) view_w = fabsf(dot3(nc, view));
  obs = observation_weight(p, d, sd, view_w);
  if (obs <= 0.0f) return -1;
  spw = xform_point(p.T_wc, backproject(u, v, d, p));
  nw = normalize3(xform_vector(p.T_wc, nc));
  const int dir = dominant_direction(nw);
  if (dir < 0 || dir >= kDirs) return -1;
  sc = coordinate_along(spw, dir);
  return dir;
}

// Pass 1: every voxel of every visible block; the ones that reach the layer update in the reference are
// appended to V.active (warp-aggregated: one atomic per warp).  Cheap and uniform per voxel.
__global__ void __launch_bounds__(kThreads) classify_kernel(const float* __restrict__ depth, const Volume V,
                                                            const Params p) {
  const uint32_t nvis = V.counters->visible_count;
  const unsigned long long total = static_cast<unsigned long long>(nvis) * kBlockVoxels;
  const int lane = threadIdx.x & 31;
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
  // every lane of a warp runs the same number of iterations (the total is a multiple of 512)
  for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += stride) {
    const uint32_t item = static_cast<uint32_t>(i >> 9);
    const int li = static_cast<int>(i & 511U);
    const uint32_t b = V.slot_block[V.visible[item]];
    bool pass = false;
    if (li == 0 && b != kInvalidBlock) V.block_stamp[b] = V.counters->frame;  // for incremental meshing
    if (b != kInvalidBlock) {
      const int4 bk = V.block_keys[b];
      f3 pc;
      float u, v, d;
      pass = voxel_prefix(depth, p, bk, li, pc, u, v, d);
    }
    const uint32_t ballot = __ballot_sync(0xffffffffU, pass);
    if (ballot) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(&V.counters->active_voxels, static_cast<uint32_t>(__popc(ballot)));
      base = __shfl_sync(0xffffffffU, base, 0);
      if (pass) V.active[base + __popc(ballot & ((1U << lane) - 1U))] = (b << 9) | static_cast<uint32_t>(li);
    }
  }
}

// Pass 2: the layer update of the active voxels, one voxel per thread, no CTA barriers: the expensive
// bilateral normal runs only where the reference runs it, and slow voxels no longer hold a whole block.
constexpr int kUpdateThreads = 128;

__global__ void __launch_bounds__(kUpdateThreads) update_kernel(const float* __restrict__ depth, const Volume V,
                                                                const Params p) {
  __shared__ NormalScratch<kUpdateThreads> S;
  const uint32_t n = V.counters->active_voxels;
  const uint32_t padded = (n + 31U) & ~31U;
  const int lane = threadIdx.x & 31;
  const float gs[3] = {gaussian(0.0f, p.normal_k_spatial), gaussian(1.0f, p.normal_k_spatial),
                       gaussian(2.0f, p.normal_k_spatial)};
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < padded; i += stride) {
    bool updated = false;
    uint32_t newly = 0U;
    if (i < n) {
      const uint32_t code = V.active[i];
      const uint32_t b = code >> 9;
      const int li = static_cast<int>(code & 511U);
      const int4 bk = V.block_keys[b];
      f3 pc;
      float u, v, d;
      voxel_prefix(depth, p, bk, li, pc, u, v, d);
      float sc = 0.0f, obs = 0.0f;
      f3 spw = mk3(0.0f, 0.0f, 0.0f), nw = spw;
      const int dir = voxel_observation<kUpdateThreads>(depth, p, pc, u, v, d, gs, S, threadIdx.x, sc, spw, nw, obs);
      if (dir >= 0) {
        float4 L0, L1, L2;
        load_bin(V, b, dir, li, bk, p.voxel_size, L0, L1, L2);
        updated = integrate_sample(p, L0, L1, L2, sc, spw, nw, obs);
        if (updated) {
          store_bin(V, b, dir, li, bk, p.voxel_size, L0, L1, L2);
          const size_t w = static_cast<size_t>(b) * (kBlockVoxels / 32) + (li >> 5);
          const uint32_t bit = 1U << (li & 31);
          if (!(V.obs_mask[w] & bit)) newly = (atomicOr(&V.obs_mask[w], bit) & bit) ? 0U : 1U;
          const uint32_t dbit = 1U << dir;
          if (!(V.dir_mask[b] & dbit)) atomicOr(&V.dir_mask[b], dbit);
        }
      }
    }
    const uint32_t upd = __ballot_sync(0xffffffffU, updated);
    const uint32_t nw_ = __ballot_sync(0xffffffffU, newly != 0U);
    if (lane == 0) {
      if (upd) atomicAdd(&V.counters->integrated_voxels, static_cast<uint32_t>(__popc(upd)));
      if (nw_) atomicAdd(&V.counters->observed_voxels, static_cast<unsigned long long>(__popc(nw_)));
    }
  }
}

// ---- per-pixel normal map (Params::normal_mode 1) ----
//
// At integer pixel coordinates sample_bilinear returns the pixel's own depth (weight 1 on d00, or the nearest
// tap), so estimateSurfaceNormalCamera evaluated at every pixel centre is a 5x5 stencil over the depth image:
// computed once per pixel here from a shared-memory tile, then bilinearly interpolated at each voxel's
// projection.  This replaces the reference's 50 subpixel samples per voxel by 4 map taps; the normal differs
// from the reference's at subpixel positions, which is why the mode is opt-in (results are evaluated by the
// Chamfer distance of the fused surface, not bit parity).
constexpr int kMapTX = 32, kMapTY = 8, kMapHalo = 2;
constexpr int kMapW = kMapTX + 2 * kMapHalo, kMapH = kMapTY + 2 * kMapHalo;

struct MapSmem {
  float px[kMapH][kMapW], py[kMapH][kMapW], pz[kMapH][kMapW];
  float nx[kMapH][kMapW], ny[kMapH][kMapW], nz[kMapH][kMapW];
  unsigned char pv[kMapH][kMapW], nv[kMapH][kMapW];
};

// the normal map of the 32x8 pixel tile at (x0, y0); every thread of the CTA calls it (it synchronises)
__device__ __forceinline__ void map_tile(const float* __restrict__ depth, const Params& p, float4* __restrict__ nmap,
                                         int x0t, int y0t, int tid, MapSmem& S) {
  const int x0 = x0t - kMapHalo, y0 = y0t - kMapHalo;
  // 1. backprojected points of the tile + halo (invalid outside the image or where depth <= 0)
  for (int k = tid; k < kMapW * kMapH; k += kMapTX * kMapTY) {
    const int ty = k / kMapW, tx = k - ty * kMapW;
    const int x = x0 + tx, y = y0 + ty;
    float d = 0.0f;
    if (x >= 0 && x < p.width && y >= 0 && y < p.height) d = __ldg(&depth[static_cast<size_t>(y) * p.width + x]);
    const bool ok = d > 0.0f;
    const f3 q = ok ? backproject(static_cast<float>(x), static_cast<float>(y), d, p) : mk3(0.0f, 0.0f, 0.0f);
    S.px[ty][tx] = q.x;
    S.py[ty][tx] = q.y;
    S.pz[ty][tx] = q.z;
    S.pv[ty][tx] = ok ? 1 : 0;
  }
  __syncthreads();
  // 2. base normals (estimateSurfaceNormalBaseCamera) of the tile + 1-pixel ring, oriented toward the camera
  for (int k = tid; k < kMapW * kMapH; k += kMapTX * kMapTY) {
    const int ty = k / kMapW, tx = k - ty * kMapW;
    bool ok = tx >= 1 && tx < kMapW - 1 && ty >= 1 && ty < kMapH - 1 && S.pv[ty][tx] && S.pv[ty][tx - 1] &&
              S.pv[ty][tx + 1] && S.pv[ty - 1][tx] && S.pv[ty + 1][tx];
    f3 n = mk3(0.0f, 0.0f, 0.0f);
    if (ok) {
      const f3 dv = mk3(S.px[ty + 1][tx] - S.px[ty - 1][tx], S.py[ty + 1][tx] - S.py[ty - 1][tx],
                        S.pz[ty + 1][tx] - S.pz[ty - 1][tx]);
      const f3 du = mk3(S.px[ty][tx + 1] - S.px[ty][tx - 1], S.py[ty][tx + 1] - S.py[ty][tx - 1],
                        S.pz[ty][tx + 1] - S.pz[ty][tx - 1]);
      n = normalize3(cross3(dv, du));
      ok = norm3(n) > 1e-6f;
      if (ok) n = orient_unit_toward_camera(n, mk3(S.px[ty][tx], S.py[ty][tx], S.pz[ty][tx]));
    }
    S.nx[ty][tx] = n.x;
    S.ny[ty][tx] = n.y;
    S.nz[ty][tx] = n.z;
    S.nv[ty][tx] = ok ? 1 : 0;
  }
  __syncthreads();
  // 3. the bilateral combination of the 3x3 base normals (estimateSurfaceNormalCamera)
  const int lx = tid % kMapTX, ly = tid / kMapTX;
  const int x = x0t + lx, y = y0t + ly;
  if (x >= p.width || y >= p.height) return;
  const int cx = lx + kMapHalo, cy = ly + kMapHalo;
  float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (S.nv[cy][cx]) {
    const f3 cn = mk3(S.nx[cy][cx], S.ny[cy][cx], S.nz[cy][cx]);
    const f3 cp = mk3(S.px[cy][cx], S.py[cy][cx], S.pz[cy][cx]);
    const float g1 = gaussian(1.0f, p.normal_k_spatial), g2 = gaussian(2.0f, p.normal_k_spatial);
    f3 wsum = mk3(0.0f, 0.0f, 0.0f);
    float ws = 0.0f;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const int dx = k % 3 - 1, dy = k / 3 - 1;
      if (!S.nv[cy + dy][cx + dx]) continue;
      const f3 sn = mk3(S.nx[cy + dy][cx + dx], S.ny[cy + dy][cx + dx], S.nz[cy + dy][cx + dx]);
      const float delta = S.pz[cy + dy][cx + dx] - cp.z;
      const float ad = 1.0f - clampf(dot3(cn, sn), -1.0f, 1.0f);
      const int r2 = dx * dx + dy * dy;
      const float w = (r2 == 0 ? 1.0f : (r2 == 1 ? g1 : g2)) * gaussian(delta * delta, p.normal_k_range) *
                      gaussian(ad * ad, p.normal_k_angular);
      wsum = add3(wsum, mul3(sn, w));
      ws += w;
    }
    f3 n = cn;
    if (ws > 1e-6f) {
      n = orient_toward_camera(normalize3(mul3(wsum, 1.0f / ws)), cp);
      if (norm3(n) <= 1e-6f) n = cn;
    }
    out = make_float4(n.x, n.y, n.z, 1.0f);
  }
  nmap[static_cast<size_t>(y) * p.width + x] = out;
}

__global__ void __launch_bounds__(kMapTX * kMapTY) pixel_normal_kernel(const float* __restrict__ depth, const Params p,
                                                                       float4* __restrict__ nmap) {
  __shared__ MapSmem S;
  map_tile(depth, p, nmap, blockIdx.x * kMapTX, blockIdx.y * kMapTY, threadIdx.y * kMapTX + threadIdx.x, S);
}

// The normal map of a frame (pixel_normal_kernel) plus, grid-stride over the frame's visible list (final: the
// allocation ran before), each entry's {block key, pool index} into V.visible_keys, so that the fused update
// reads one int4 per chunk instead of the dependent chain visible -> slot_block -> block_keys.
__global__ void __launch_bounds__(kMapTX * kMapTY) map_prepare_kernel(const float* __restrict__ depth, const Volume V,
                                                                      const Params p, float4* __restrict__ nmap) {
  __shared__ MapSmem S;
  const int tid = threadIdx.y * kMapTX + threadIdx.x;
  const uint32_t nvis = V.counters->visible_count;
  const uint32_t nthreads = gridDim.x * gridDim.y * kMapTX * kMapTY;
  for (uint32_t i = (blockIdx.y * gridDim.x + blockIdx.x) * (kMapTX * kMapTY) + tid; i < nvis; i += nthreads) {
    const uint32_t b = V.slot_block[V.visible[i]];
    int4 k = make_int4(0, 0, 0, static_cast<int>(kInvalidBlock));
    if (b != kInvalidBlock) {
      const int4 bk = V.block_keys[b];
      k = make_int4(bk.x, bk.y, bk.z, static_cast<int>(b));
    }
    V.visible_keys[i] = k;
  }
  map_tile(depth, p, nmap, blockIdx.x * kMapTX, blockIdx.y * kMapTY, tid, S);
}

// Normal at a voxel's projection (u, v): bilinear blend of the valid map taps around it, renormalised.
__device__ __forceinline__ bool map_normal(const float4* __restrict__ nmap, const Params& p, float u, float v, f3& n) {
  const int x0 = static_cast<int>(floorf(u)), y0 = static_cast<int>(floorf(v));
  const int x1 = min(x0 + 1, p.width - 1), y1 = min(y0 + 1, p.height - 1);
  const float tx = u - static_cast<float>(x0), ty = v - static_cast<float>(y0);
  const float4 a = __ldg(&nmap[static_cast<size_t>(y0) * p.width + x0]);
  const float4 b = __ldg(&nmap[static_cast<size_t>(y0) * p.width + x1]);
  const float4 c = __ldg(&nmap[static_cast<size_t>(y1) * p.width + x0]);
  const float4 d = __ldg(&nmap[static_cast<size_t>(y1) * p.width + x1]);
  const float wa = (1.0f - tx) * (1.0f - ty) * a.w, wb = tx * (1.0f - ty) * b.w;
  const float wc = (1.0f - tx) * ty * c.w, wd = tx * ty * d.w;
  const f3 s = mk3(wa * a.x + wb * b.x + wc * c.x + wd * d.x, wa * a.y + wb * b.y + wc * c.y + wd * d.y,
                   wa * a.z + wb * b.z + wc * c.z + wd * d.z);
  if (wa + wb + wc + wd <= 1e-6f || norm3(s) <= 1e-6f) return false;
  n = normalize3(s);
  return true;
}

// The layer update of one voxel that passed voxel_prefix, with the normal from the map.  Returns true when a
// layer was updated; newly = the voxel was observed for the first time.
__device__ __forceinline__ bool map_update_voxel(const float* __restrict__ depth, const float4* __restrict__ nmap,
                                                 const Volume& V, const Params& p, uint32_t b, int li, f3 pc, float u,
                                                 float v, float d, bool& newly) {
  newly = false;
  const int4 bk = V.block_keys[b];
  const float sd = d - pc.z;
  const f3 view = normalize3(pc);
  float view_w = 1.0f;
  f3 nc = mul3(view, -1.0f);
  if (map_normal(nmap, p, u, v, nc)) view_w = fabsf(dot3(nc, view));
  const float obs = observation_weight(p, d, sd, view_w);
  const f3 nw = normalize3(xform_vector(p.T_wc, nc));
  const int dir = obs > 0.0f ? dominant_direction(nw) : -1;
  if (dir < 0 || dir >= kDirs) return false;
  const f3 spw = xform_point(p.T_wc, backproject(u, v, d, p));
  const float sc = coordinate_along(spw, dir);
  bool updated;
  if (V.layers16 != nullptr) {
    uint4* q = V.layers16 + bin16_index(b, dir, li);
    uint4 A = q[0], B = q[1];
    updated = integrate_bin16(p, V, A, B, voxel_centre(bk, li, p.voxel_size), dir, sc, spw, nw, obs);
    if (updated) {
      q[0] = A;
      q[1] = B;
    }
  } else {
    float4 L0, L1, L2;
    load_bin(V, b, dir, li, bk, p.voxel_size, L0, L1, L2);
    updated = integrate_sample(p, L0, L1, L2, sc, spw, nw, obs);
    if (updated) store_bin(V, b, dir, li, bk, p.voxel_size, L0, L1, L2);
  }
  if (updated) {
    const size_t w = static_cast<size_t>(b) * (kBlockVoxels / 32) + (li >> 5);
    const uint32_t bit = 1U << (li & 31);
    if (!(V.obs_mask[w] & bit)) newly = !(atomicOr(&V.obs_mask[w], bit) & bit);
    const uint32_t dbit = 1U << dir;
    if (!(V.dir_mask[b] & dbit)) atomicOr(&V.dir_mask[b], dbit);
  }
  return updated;
}

// One pass over every voxel of the visible blocks with the normal from the map.  The voxel slots are cut in
// chunks of kT (a CTA's threads); each CTA takes the next chunk from a device work queue (a counter reset when
// the frame begins), runs voxel_prefix on one slot per thread, appends the survivors (warp-aggregated) to a
// shared-memory queue with their projection, and updates them one per thread in batches of kT (survivors
// carry over between chunks).  The expensive part runs on compacted threads, and the dynamic order keeps every
// CTA busy until the last chunk.
template <int kT, int kS = 1>
struct MapQueue {
  static constexpr int kQueue = kT * kS + kT;  // a pass's survivors plus fewer than kT carried over
  uint32_t code[kQueue];  // (pool block << 9) | voxel
  float u[kQueue], v[kQueue], d[kQueue], x[kQueue], y[kQueue], z[kQueue];
  uint32_t count;
};

template <class Queue>
__device__ __forceinline__ void map_update_entry(const float* __restrict__ depth, const float4* __restrict__ nmap,
                                                 const Volume& V, const Params& p, const Queue& Q, int e,
                                                 bool& updated, bool& newly) {
  const uint32_t code = Q.code[e];
  updated = map_update_voxel(depth, nmap, V, p, code >> 9, static_cast<int>(code & 511U), mk3(Q.x[e], Q.y[e], Q.z[e]),
                             Q.u[e], Q.v[e], Q.d[e], newly);
}

// per-CTA sums of the frame statistics, flushed to the volume's counters once per CTA (and scene): the
// counters share one L2 line, so per-warp atomics on them (hundreds of thousands a frame) would serialise there
struct CtaStats {
  uint32_t active, integrated;
  unsigned long long observed;
};

__device__ __forceinline__ void tally_updates(CtaStats& st, bool updated, bool newly, int lane) {
  const uint32_t upd = __ballot_sync(0xffffffffU, updated);
  const uint32_t nw_ = __ballot_sync(0xffffffffU, newly);
  if (lane == 0) {
    if (upd) atomicAdd(&st.integrated, static_cast<uint32_t>(__popc(upd)));
    if (nw_) atomicAdd(&st.observed, static_cast<unsigned long long>(__popc(nw_)));
  }
}

// kT threads per CTA, kS voxel slots per thread and pass (kT * kS divides 512, so a pass's chunk lies in one
// visible block), at least kMinBlocks resident CTAs per SM (which caps the registers).  A pass runs the prefix
// of its kS slots with independent loads, appends the survivors to the queue, then updates full batches of kT
// entries (the last kT entries, one per thread) while the queue holds kT or more; fewer than kT carry over to
// the next pass, and the rest is updated when the work queue is empty.  Each voxel is updated by exactly one
// thread and the updates of different voxels touch different bins, so the order does not change the result.
template <int kT, int kMinBlocks, int kS = 1>
__global__ void __launch_bounds__(kT, kMinBlocks) fused_update_kernel(const float* __restrict__ depth,
                                                                     const float4* __restrict__ nmap, const Volume V,
                                                                     const Params p) {
  static_assert(kBlockVoxels % (kT * kS) == 0, "a pass's chunk must divide the block's voxel count");
  constexpr int kChunk = kT * kS;
  __shared__ MapQueue<kT, kS> Q;
  __shared__ uint32_t s_item;
  __shared__ CtaStats s_stats;
  const uint32_t nvis = V.counters->visible_count;
  const uint32_t nchunks = nvis * static_cast<uint32_t>(kBlockVoxels / kChunk);
  const int tid = threadIdx.x, lane = tid & 31;
  if (tid == 0) {
    Q.count = 0U;
    s_stats.active = 0U;
    s_stats.integrated = 0U;
    s_stats.observed = 0ULL;
    s_item = atomicAdd(&V.counters->update_queue, 1U);
  }
  const uint32_t frame = V.counters->frame;
  // The loop exits through the break at its end, after the drained pass: the equivalent form with a
  // loop-carried flag as the loop condition lost one warp's survivors per chunk in the fast-math compile.
  for (;;) {
    __syncthreads();  // s_item and Q.count of this pass published
    const uint32_t item = s_item;
    const bool drained = item >= nchunks;
    // the following chunk is taken from the work queue now; its index is published at the end of the pass,
    // so the atomic's latency overlaps this chunk's work
    uint32_t next = 0U;
    if (tid == 0 && !drained) next = atomicAdd(&V.counters->update_queue, 1U);
    if (!drained) {
      // 1. prefix of kS slots per thread (one visible block per chunk), survivors appended to the queue
      const unsigned long long base_slot = static_cast<unsigned long long>(item) * kChunk;
      const int4 vk = V.visible_keys[static_cast<uint32_t>(base_slot >> 9)];
      const uint32_t b = static_cast<uint32_t>(vk.w);
      if ((base_slot & 511ULL) == 0ULL && tid == 0 && b != kInvalidBlock) V.block_stamp[b] = frame;
      bool pass[kS];
      f3 pc[kS];
      float u[kS], v[kS], d[kS];
#pragma unroll
      for (int j = 0; j < kS; ++j) {
        const int li = static_cast<int>((base_slot + static_cast<unsigned long long>(j * kT + tid)) & 511ULL);
        pass[j] = false;
        pc[j] = mk3(0.0f, 0.0f, 0.0f);
        u[j] = v[j] = d[j] = 0.0f;
        if (b != kInvalidBlock) pass[j] = voxel_prefix(depth, p, vk, li, pc[j], u[j], v[j], d[j]);
      }
#pragma unroll
      for (int j = 0; j < kS; ++j) {
        const uint32_t ballot = __ballot_sync(0xffffffffU, pass[j]);
        uint32_t base = 0U;
        if (lane == 0 && ballot) {
          base = atomicAdd(&Q.count, static_cast<uint32_t>(__popc(ballot)));
          atomicAdd(&s_stats.active, static_cast<uint32_t>(__popc(ballot)));
        }
        base = __shfl_sync(0xffffffffU, base, 0);
        if (pass[j]) {
          const int li = static_cast<int>((base_slot + static_cast<unsigned long long>(j * kT + tid)) & 511ULL);
          const uint32_t e = base + __popc(ballot & ((1U << lane) - 1U));
          Q.code[e] = (b << 9) | static_cast<uint32_t>(li);
          Q.u[e] = u[j];
          Q.v[e] = v[j];
          Q.d[e] = d[j];
          Q.x[e] = pc[j].x;
          Q.y[e] = pc[j].y;
          Q.z[e] = pc[j].z;
        }
      }
    }
    __syncthreads();
    // 2. batches of kT entries from the end of the queue, one per thread: while kT or more are queued, and the
    // rest once the work queue is empty.  One call site, so every voxel runs the same instructions (with
    // contraction on, two inlined copies of the update could round differently).
    uint32_t n = Q.count;
    while (n >= static_cast<uint32_t>(kT) || (drained && n > 0U)) {
      const uint32_t first = n >= static_cast<uint32_t>(kT) ? n - static_cast<uint32_t>(kT) : 0U;
      bool updated = false, newly = false;
      if (first + static_cast<uint32_t>(tid) < n) {
        map_update_entry(depth, nmap, V, p, Q, static_cast<int>(first) + tid, updated, newly);
      }
      tally_updates(s_stats, updated, newly, lane);
      n = first;
    }
    __syncthreads();  // the batches' entries and s_item are rewritten by the next chunk
    if (tid == 0) {
      Q.count = n;
      s_item = next;
    }
    if (drained) break;
  }
  __syncthreads();
  if (tid == 0) {
    if (s_stats.active) atomicAdd(&V.counters->active_voxels, s_stats.active);
    if (s_stats.integrated) atomicAdd(&V.counters->integrated_voxels, s_stats.integrated);
    if (s_stats.observed) atomicAdd(&V.counters->observed_voxels, s_stats.observed);
  }
}

// ---- multi-scene batch: three work-queue kernels over the items of every scene of the step ----
//
// 0. batch_begin_kernel: clears the work queues and starts every active scene's frame;
// 1. batch_filter_alloc_kernel: the filter + allocation tiles of all scenes;
// 2. batch_map_kernel: the normal-map tiles of all scenes, and each scene's visible-list keys;
// 3. batch_update_kernel: chunks of kThreads voxel slots of every scene's visible blocks (the per-scene
//    visible counts are final after kernel 1; every CTA derives the chunk prefix from them).
// Each CTA takes the next item from a global counter (a device work queue), so scenes of very different
// sizes share the GPU without idle tails; the scene of an item is found by binary search over the
// per-scene first items, and its descriptor is copied to shared memory when it changes.

// last scene whose first item <= item (firsts ascending; empty scenes share the next scene's first)
template <typename F>
__device__ __forceinline__ int find_scene(int n, uint32_t item, F first) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first(mid) <= item) {
      lo = mid;
    } else {
      hi = mid - 1;
    }
  }
  return lo;
}

__device__ __forceinline__ void copy_desc(SceneDesc& dst, const SceneDesc* __restrict__ src, int tid, int nthreads) {
  static_assert(sizeof(SceneDesc) % 4 == 0, "descriptor copied as words");
  const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
  uint32_t* d = reinterpret_cast<uint32_t*>(&dst);
  for (int i = tid; i < static_cast<int>(sizeof(SceneDesc) / 4); i += nthreads) d[i] = s[i];
}

// 0. the step's start: work-queue counters cleared, every active scene's frame started (before any
// allocation of the step touches a scene's counters)
__global__ void batch_begin_kernel(const SceneDesc* __restrict__ descs, const BatchHeader* __restrict__ hdr,
                                   uint32_t* __restrict__ queue) {
  if (threadIdx.x < 3) queue[threadIdx.x] = 0U;
  const int nsc = static_cast<int>(hdr->nscenes);
  for (int k = threadIdx.x; k < nsc; k += blockDim.x) {
    if (descs[k].active) filt::begin_frame(descs[k].V.counters);
  }
}

// 1. filter + allocation tiles of all scenes (filter_alloc_kernel per tile)
template <bool kBand>
union FilterAllocSmem {
  filt::Smem f;
  alloc::TileSets<kBand> a;
};

template <bool kBand>
__device__ __forceinline__ void batch_filter_alloc_body(const SceneDesc* __restrict__ descs,
                                                        const BatchHeader* __restrict__ hdr, uint32_t* __restrict__ queue,
                                                        FilterAllocSmem<kBand>& S, SceneDesc& D, uint32_t& s_item,
                                                        int& s_scene) {
  constexpr int kT = filt::kTX * filt::kTY;
  static_assert(filt::kTX == alloc::kTX && filt::kTY == alloc::kTY, "one tile for both passes");
  const int tid = threadIdx.x;
  const int nsc = static_cast<int>(hdr->nscenes);
  const uint32_t total = hdr->filter_total;
  int cur = -1;
  for (;;) {
    if (tid == 0) {
      const uint32_t it = atomicAdd(&queue[0], 1U);
      s_item = it;
      s_scene = it < total ? find_scene(nsc, it, [&](int k) { return descs[k].filter_first; }) : -1;
    }
    __syncthreads();
    const uint32_t item = s_item;
    const int sc = s_scene;
    if (item >= total) break;
    if (sc != cur) {
      copy_desc(D, descs + sc, tid, kT);
      cur = sc;
      __syncthreads();
    }
    const uint32_t local = item - D.filter_first;
    const uint32_t tiles_x = (static_cast<uint32_t>(D.p.width) + filt::kTX - 1) / filt::kTX;
    const int u0 = static_cast<int>(local % tiles_x) * filt::kTX, v0 = static_cast<int>(local / tiles_x) * filt::kTY;
    const float d = filt::filter_tile(D.depth_in, D.depth, D.p, u0, v0, tid, S.f);
    __syncthreads();  // the filter's staged tiles become the allocation's sets
    const int u = u0 + tid % filt::kTX, v = v0 + tid / filt::kTX;
    const int st = D.p.stride;
    const bool has = u < D.p.width && v < D.p.height && u % st == 0 && v % st == 0 && u / st < D.p.sample_width &&
                     v / st < D.p.sample_height;
    alloc::alloc_samples<kBand>(D.V, D.p, has, u, v, d, tid, S.a);
    __syncthreads();
  }
}

template <bool kBand>
__global__ void __launch_bounds__(filt::kTX * filt::kTY) batch_filter_alloc_kernel(const SceneDesc* __restrict__ descs,
                                                                                   const BatchHeader* __restrict__ hdr,
                                                                                   uint32_t* __restrict__ queue) {
  __shared__ FilterAllocSmem<kBand> S;
  __shared__ SceneDesc D;
  __shared__ uint32_t s_item;
  __shared__ int s_scene;
  batch_filter_alloc_body<kBand>(descs, hdr, queue, S, D, s_item, s_scene);
}

// 2. normal-map tiles of all scenes; the tiles of a scene also write its visible list's {key, pool index}
// entries (the list is final after kernel 1), tile L of M taking entries L * 256 + tid + j * M * 256
__device__ __forceinline__ void batch_map_body(const SceneDesc* __restrict__ descs, const BatchHeader* __restrict__ hdr,
                                               uint32_t* __restrict__ queue, MapSmem& M, SceneDesc& D, uint32_t& s_item,
                                               int& s_scene) {
  constexpr int kT = kMapTX * kMapTY;
  const int tid = threadIdx.x;
  const int nsc = static_cast<int>(hdr->nscenes);
  const uint32_t total = hdr->stage2_total;
  int cur = -1;
  for (;;) {
    if (tid == 0) {
      const uint32_t it = atomicAdd(&queue[1], 1U);
      s_item = it;
      s_scene = it < total ? find_scene(nsc, it, [&](int k) { return descs[k].map_first; }) : -1;
    }
    __syncthreads();
    const uint32_t item = s_item;
    const int sc = s_scene;
    if (item >= total) break;
    if (sc != cur) {
      copy_desc(D, descs + sc, tid, kT);
      cur = sc;
      __syncthreads();
    }
    const uint32_t local = item - D.map_first;
    const uint32_t nvis = D.V.counters->visible_count;
    for (uint32_t i = local * kT + tid; i < nvis; i += D.map_items * kT) {
      const uint32_t b = D.V.slot_block[D.V.visible[i]];
      int4 k = make_int4(0, 0, 0, static_cast<int>(kInvalidBlock));
      if (b != kInvalidBlock) {
        const int4 bk = D.V.block_keys[b];
        k = make_int4(bk.x, bk.y, bk.z, static_cast<int>(b));
      }
      D.V.visible_keys[i] = k;
    }
    const uint32_t tiles_x = (static_cast<uint32_t>(D.p.width) + kMapTX - 1) / kMapTX;
    map_tile(D.depth, D.p, D.nmap, static_cast<int>(local % tiles_x) * kMapTX, static_cast<int>(local / tiles_x) * kMapTY,
             tid, M);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kMapTX * kMapTY) batch_map_kernel(const SceneDesc* __restrict__ descs,
                                                                    const BatchHeader* __restrict__ hdr,
                                                                    uint32_t* __restrict__ queue) {
  __shared__ MapSmem M;
  __shared__ SceneDesc D;
  __shared__ uint32_t s_item;
  __shared__ int s_scene;
  batch_map_body(descs, hdr, queue, M, D, s_item, s_scene);
}

// Survivors carry over between the chunks of a scene as in fused_update_kernel; when the CTA's next chunk
// belongs to another scene, it first updates the scene's remaining survivors and flushes its statistics.
// kUT threads per CTA (the chunk of voxel slots), at least kUMinB resident CTAs per SM.  128 x 12 (40
// registers, a small spill) measured fastest, as the single-volume autotuner also finds for its kernel:
// 64-scene batch 3,614 Mpix/s, against 3,485 for 256 x 6 and 3,221 for 256 x 4 (64 registers).
template <int kUT>
struct BatchUpdateSmem {
  MapQueue<kUT> Q;
  uint32_t s_first[kMaxBatchScenes + 1];
  CtaStats s_stats;
};

template <int kUT>
__device__ __forceinline__ void batch_update_body(const SceneDesc* __restrict__ descs,
                                                  const BatchHeader* __restrict__ hdr, uint32_t* __restrict__ queue,
                                                  BatchUpdateSmem<kUT>& U, SceneDesc& D, uint32_t& s_item,
                                                  int& s_scene) {
  MapQueue<kUT>& Q = U.Q;
  uint32_t* s_first = U.s_first;
  CtaStats& s_stats = U.s_stats;
  const int tid = threadIdx.x, lane = tid & 31;
  const int nsc = static_cast<int>(hdr->nscenes);
  constexpr uint32_t kChunksPerBlock = kBlockVoxels / kUT;
  if (tid == 0) {
    uint32_t run = 0U;
    for (int k = 0; k < nsc; ++k) {
      s_first[k] = run;
      if (descs[k].active) run += descs[k].V.counters->visible_count * kChunksPerBlock;
    }
    s_first[nsc] = run;
    Q.count = 0U;
    s_stats.active = 0U;
    s_stats.integrated = 0U;
    s_stats.observed = 0ULL;
  }
  __syncthreads();
  const uint32_t total = s_first[nsc];
  int cur = -1;  // scene whose descriptor is in D and whose survivors are in the queue
  uint32_t item = 0U;
  int sc = -1;
  bool fetched = false;
  for (;;) {
    if (!fetched) {
      if (tid == 0) {
        const uint32_t it = atomicAdd(&queue[2], 1U);
        s_item = it;
        s_scene = it < total ? find_scene(nsc, it, [&](int k) { return s_first[k]; }) : -1;
      }
      __syncthreads();
      item = s_item;
      sc = s_scene;
      fetched = true;
    }
    // the current scene ends when the work queue is empty or the fetched chunk belongs to another scene: its
    // carried-over survivors are updated and its statistics flushed before the next scene starts
    const bool scene_end = cur >= 0 && (item >= total || sc != cur);
    if (!scene_end) {
      if (item >= total) break;
      if (sc != cur) {
        copy_desc(D, descs + sc, tid, kUT);
        cur = sc;
        __syncthreads();
      }
        // 1. prefix of one slot per thread, survivors appended to the queue
      const unsigned long long i = static_cast<unsigned long long>(item - s_first[sc]) * kUT + tid;
      const int4 vk = D.V.visible_keys[static_cast<uint32_t>(i >> 9)];
      const uint32_t b = static_cast<uint32_t>(vk.w);
      const int li = static_cast<int>(i & 511U);
      bool pass = false;
      if (li == 0 && b != kInvalidBlock) D.V.block_stamp[b] = D.V.counters->frame;  // for incremental meshing
      f3 pc = mk3(0.0f, 0.0f, 0.0f);
      float u = 0.0f, v = 0.0f, d = 0.0f;
      if (b != kInvalidBlock) pass = voxel_prefix(D.depth, D.p, vk, li, pc, u, v, d);
      const uint32_t ballot = __ballot_sync(0xffffffffU, pass);
      uint32_t base = 0U;
      if (lane == 0 && ballot) {
        base = atomicAdd(&Q.count, static_cast<uint32_t>(__popc(ballot)));
        atomicAdd(&s_stats.active, static_cast<uint32_t>(__popc(ballot)));
      }
      base = __shfl_sync(0xffffffffU, base, 0);
      if (pass) {
        const uint32_t e = base + __popc(ballot & ((1U << lane) - 1U));
        Q.code[e] = (b << 9) | static_cast<uint32_t>(li);
        Q.u[e] = u;
        Q.v[e] = v;
        Q.d[e] = d;
        Q.x[e] = pc.x;
        Q.y[e] = pc.y;
        Q.z[e] = pc.z;
      }
      fetched = false;
    }
    __syncthreads();
    // 2. entries [first, n) of the current scene, one per thread, from one call site (as in
    // fused_update_kernel): a full batch, nothing, or at the scene's end the carried-over rest
    const uint32_t n = Q.count;
    const uint32_t first =
        scene_end ? 0U : (n >= static_cast<uint32_t>(kUT) ? n - static_cast<uint32_t>(kUT) : n);
    bool updated = false, newly = false;
    if (first + static_cast<uint32_t>(tid) < n) {
      map_update_entry(D.depth, D.nmap, D.V, D.p, Q, static_cast<int>(first) + tid, updated, newly);
    }
    tally_updates(s_stats, updated, newly, lane);
    __syncthreads();
    if (tid == 0) {
      Q.count = first;
      if (scene_end) {
        if (s_stats.active) atomicAdd(&D.V.counters->active_voxels, s_stats.active);
        if (s_stats.integrated) atomicAdd(&D.V.counters->integrated_voxels, s_stats.integrated);
        if (s_stats.observed) atomicAdd(&D.V.counters->observed_voxels, s_stats.observed);
        s_stats.active = 0U;
        s_stats.integrated = 0U;
        s_stats.observed = 0ULL;
      }
    }
    if (scene_end) {
      __syncthreads();  // D, the statistics and the queue are rewritten by the next scene
      cur = -1;
    }
  }
}


template <int kUT, int kUMinB>
__global__ void __launch_bounds__(kUT, kUMinB) batch_update_kernel(const SceneDesc* __restrict__ descs,
                                                                const BatchHeader* __restrict__ hdr,
                                                                uint32_t* __restrict__ queue) {
  __shared__ BatchUpdateSmem<kUT> U;
  __shared__ SceneDesc D;
  __shared__ uint32_t s_item;
  __shared__ int s_scene;
  batch_update_body<kUT>(descs, hdr, queue, U, D, s_item, s_scene);
}

// ---- the batch step as one persistent launch ----
//
// batch_persistent_kernel runs the four phases of a step (start, filter + allocation, normal map, layer update)
// in one cooperative launch: every CTA is resident, and a grid-wide barrier separates the phases (each phase
// reads what the previous one wrote on other SMs).  Data written in a phase is first read in a later phase, so
// no SM holds a stale copy of it when the barrier's fences have run.  The waits are bounded: after about a
// second of %globaltimer time a CTA stops waiting, marks every scene of the step with the timeout bit (which
// vh_synchronize reports as VH_ERR_TIMEOUT) and returns.
// Six resident CTAs per SM (40 registers a thread, some spilled): the 64-scene batch step ran at 3,462 Mpix/s
// against 3,124 with four (64 registers, no spills).
constexpr int kPersistThreads = 256, kPersistMinB = 6;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// bar[0]: arrivals, bar[1]: generation.  Returns false when the wait gave up.
__device__ __forceinline__ bool grid_barrier(uint32_t* bar, uint32_t nctas, int& s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t* gen = bar + 1;
    const uint32_t g = *gen;
    __threadfence();
    bool ok = true;
    if (atomicAdd(&bar[0], 1U) == nctas - 1U) {
      bar[0] = 0U;  // reset before the release, so the next barrier counts from zero
      __threadfence();
      atomicAdd(&bar[1], 1U);
    } else {
      const unsigned long long t0 = global_ns();
      uint32_t polls = 0;
      while (*gen == g) {
        if ((++polls & 63U) == 0U && global_ns() - t0 > 1000000000ULL) {
          ok = false;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ void mark_step_timeout(const SceneDesc* __restrict__ descs, const BatchHeader* __restrict__ hdr) {
  if (threadIdx.x != 0) return;
  for (uint32_t k = 0; k < hdr->nscenes; ++k) {
    if (descs[k].active) atomicOr(&descs[k].V.counters->error, kErrTimeout);
  }
}

template <bool kBand>
__global__ void __launch_bounds__(kPersistThreads, kPersistMinB)
    batch_persistent_kernel(const SceneDesc* __restrict__ descs, const BatchHeader* __restrict__ hdr,
                            uint32_t* __restrict__ queue, uint32_t* __restrict__ bar) {
  static_assert(kPersistThreads == filt::kTX * filt::kTY && kPersistThreads == kMapTX * kMapTY,
                "one CTA shape for every phase");
  __shared__ union {
    FilterAllocSmem<kBand> fa;
    MapSmem m;
    BatchUpdateSmem<kPersistThreads> u;
  } S;
  __shared__ SceneDesc D;
  __shared__ uint32_t s_item;
  __shared__ int s_scene;
  __shared__ int s_ok;
  const uint32_t nctas = gridDim.x;
  // 0. the step's start: work-queue counters cleared, every active scene's frame started
  if (blockIdx.x == 0) {
    if (threadIdx.x < 3) queue[threadIdx.x] = 0U;
    const int nsc = static_cast<int>(hdr->nscenes);
    for (int k = threadIdx.x; k < nsc; k += blockDim.x) {
      if (descs[k].active) filt::begin_frame(descs[k].V.counters);
    }
  }
  if (!grid_barrier(bar, nctas, s_ok)) return mark_step_timeout(descs, hdr);
  batch_filter_alloc_body<kBand>(descs, hdr, queue, S.fa, D, s_item, s_scene);
  if (!grid_barrier(bar, nctas, s_ok)) return mark_step_timeout(descs, hdr);
  batch_map_body(descs, hdr, queue, S.m, D, s_item, s_scene);
  if (!grid_barrier(bar, nctas, s_ok)) return mark_step_timeout(descs, hdr);
  batch_update_body<kPersistThreads>(descs, hdr, queue, S.u, D, s_item, s_scene);
}

// the depth filter of one frame in this compile (the fast-math form's filter in the fast compile)
__global__ void __launch_bounds__(filt::kTX * filt::kTY) frame_filter_kernel(const float* __restrict__ in,
                                                                             float* __restrict__ out, const Params p,
                                                                             Counters* counters) {
  __shared__ filt::Smem S;
  const int tid = threadIdx.x;
  if (counters && blockIdx.x == 0 && blockIdx.y == 0 && tid == 0) filt::begin_frame(counters);
  filt::filter_tile(in, out, p, blockIdx.x * filt::kTX, blockIdx.y * filt::kTY, tid, S);
}

// Filter and allocation of one frame in one pass (the frame was started by a preceding launch): each CTA filters
// its 32x8 tile, then allocates the blocks of the tile's samples from the filtered depths it just computed.
// The allocation's dependent hash probes overlap the filter arithmetic of the other CTAs on the SM, and the
// filtered depth is not re-read.  kBand: the truncation-band rule (smaller tile sets, higher occupancy).
template <bool kBand>
__global__ void __launch_bounds__(filt::kTX * filt::kTY) filter_alloc_kernel(const float* __restrict__ in,
                                                                             float* __restrict__ out, const Volume V,
                                                                             const Params p) {
  static_assert(filt::kTX == alloc::kTX && filt::kTY == alloc::kTY, "one tile for both passes");
  __shared__ union Shared {
    filt::Smem f;
    alloc::TileSets<kBand> a;
  } S;
  const int tid = threadIdx.x;
  const int u0 = blockIdx.x * filt::kTX, v0 = blockIdx.y * filt::kTY;
  const float d = filt::filter_tile(in, out, p, u0, v0, tid, S.f);
  __syncthreads();  // the filter's staged tiles become the allocation's sets
  const int u = u0 + tid % filt::kTX, v = v0 + tid / filt::kTX;
  const bool has = u < p.width && v < p.height && u % p.stride == 0 && v % p.stride == 0 &&
                   u / p.stride < p.sample_width && v / p.stride < p.sample_height;
  alloc::alloc_samples<kBand>(V, p, has, u, v, d, tid, S.a);
}

}  // namespace

static int grid_for(const void* kernel, int threads) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
  return (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 1);
}

int integrate_grid_size() {
  static int grid = 0;
  if (grid == 0) grid = grid_for(reinterpret_cast<const void*>(update_kernel), kUpdateThreads);
  return grid;
}

cudaError_t launch_frame_filter(const float* in, float* out, const Params& p, Counters* begin_frame, cudaStream_t s) {
  if (p.filter_radius < 0 || p.filter_radius > filt::kR) return cudaErrorInvalidValue;
  const dim3 grid((p.width + filt::kTX - 1) / filt::kTX, (p.height + filt::kTY - 1) / filt::kTY);
  frame_filter_kernel<<<grid, filt::kTX * filt::kTY, 0, s>>>(in, out, p, begin_frame);
  return cudaGetLastError();
}

cudaError_t launch_filter_alloc(const float* in, float* out, const Volume& V, const Params& p, cudaStream_t s) {
  if (p.filter_radius < 0 || p.filter_radius > filt::kR || p.stride < 1) return cudaErrorInvalidValue;
  const cudaError_t e = launch_begin_frame(V.counters, s);
  if (e != cudaSuccess) return e;
  const dim3 grid((p.width + filt::kTX - 1) / filt::kTX, (p.height + filt::kTY - 1) / filt::kTY);
  if (p.alloc_mode == 1) {
    filter_alloc_kernel<true><<<grid, filt::kTX * filt::kTY, 0, s>>>(in, out, V, p);
  } else {
    filter_alloc_kernel<false><<<grid, filt::kTX * filt::kTY, 0, s>>>(in, out, V, p);
  }
  return cudaGetLastError();
}

cudaError_t launch_pixel_normals(const float* depth, const Params& p, float4* nmap, cudaStream_t s) {
  const dim3 mb(kMapTX, kMapTY), mg((p.width + kMapTX - 1) / kMapTX, (p.height + kMapTY - 1) / kMapTY);
  pixel_normal_kernel<<<mg, mb, 0, s>>>(depth, p, nmap);
  return cudaGetLastError();
}

// first kernel of the update: the active-voxel list (classify_kernel) or the per-pixel normal map with the
// visible-list keys (map_prepare_kernel)
cudaError_t launch_integrate_prepare(const float* depth, const Volume& V, const Params& p, float4* nmap,
                                     cudaStream_t s) {
  if (p.normal_mode == 1) {
    if (nmap == nullptr) return cudaErrorInvalidValue;
    const dim3 mb(kMapTX, kMapTY), mg((p.width + kMapTX - 1) / kMapTX, (p.height + kMapTY - 1) / kMapTY);
    map_prepare_kernel<<<mg, mb, 0, s>>>(depth, V, p, nmap);
    return cudaGetLastError();
  }
  static int classify_grid = 0;
  if (classify_grid == 0) classify_grid = grid_for(reinterpret_cast<const void*>(classify_kernel), kThreads);
  classify_kernel<<<classify_grid, kThreads, 0, s>>>(depth, V, p);
  return cudaGetLastError();
}

// second kernel: the layer update over the active list (update_kernel) or over every visible voxel with the
// map normal (fused_update_kernel)
// Launch shapes of fused_update_kernel the autotuner chooses from: (threads per CTA, minimum resident CTAs per
// SM).  The grid is always the number of CTAs that fit on the device at once.
struct FusedVariant {
  const void* fn;
  void (*launch)(int grid, cudaStream_t s, const float* depth, const float4* nmap, const Volume& V, const Params& p);
  int threads;
};

template <int kT, int kMinB, int kS>
void launch_fused_variant(int grid, cudaStream_t s, const float* depth, const float4* nmap, const Volume& V,
                          const Params& p) {
  fused_update_kernel<kT, kMinB, kS><<<grid, kT, 0, s>>>(depth, nmap, V, p);
}

// (threads per CTA, minimum resident CTAs per SM, voxel slots per thread and pass)
#define VH_FUSED_VARIANT(T, B, S) \
  FusedVariant { reinterpret_cast<const void*>(fused_update_kernel<T, B, S>), launch_fused_variant<T, B, S>, T }
static const FusedVariant kFusedVariants[] = {
    VH_FUSED_VARIANT(256, 4, 1), VH_FUSED_VARIANT(128, 8, 1),  VH_FUSED_VARIANT(256, 6, 1),
    VH_FUSED_VARIANT(128, 12, 1), VH_FUSED_VARIANT(512, 2, 1), VH_FUSED_VARIANT(64, 16, 1),
    VH_FUSED_VARIANT(128, 8, 4),  VH_FUSED_VARIANT(256, 4, 2), VH_FUSED_VARIANT(128, 12, 2),
    VH_FUSED_VARIANT(256, 6, 2),
};
#undef VH_FUSED_VARIANT
constexpr int kNumFusedVariants = static_cast<int>(sizeof(kFusedVariants) / sizeof(kFusedVariants[0]));

int fused_variant_count() { return kNumFusedVariants; }

void fused_variant_shape(int variant, int* threads, int* min_blocks) {
  static const int kMin[] = {4, 8, 6, 12, 2, 16, 8, 4, 12, 6};
  static_assert(sizeof(kMin) / sizeof(kMin[0]) == kNumFusedVariants, "one entry per variant");
  const int v = (variant >= 0 && variant < kNumFusedVariants) ? variant : 0;
  *threads = kFusedVariants[v].threads;
  *min_blocks = kMin[v];
}

cudaError_t launch_integrate_update(const float* depth, const Volume& V, const Params& p, int grid,
                                    const float4* nmap, cudaStream_t s, int variant) {
  if (p.normal_mode == 1) {
    if (nmap == nullptr) return cudaErrorInvalidValue;
    if (variant < 0 || variant >= kNumFusedVariants) variant = 0;
    static int fused_grid[kNumFusedVariants] = {};
    const FusedVariant& fv = kFusedVariants[variant];
    if (fused_grid[variant] == 0) fused_grid[variant] = grid_for(fv.fn, fv.threads);
    fv.launch(grid > 0 ? grid : fused_grid[variant], s, depth, nmap, V, p);
    return cudaGetLastError();
  }
  update_kernel<<<grid > 0 ? grid : integrate_grid_size(), kUpdateThreads, 0, s>>>(depth, V, p);
  return cudaGetLastError();
}

// launch shape of batch_update_kernel: threads per CTA (the chunk of voxel slots) and resident CTAs per SM
constexpr int kBatchUT = 128, kBatchUMinB = 12;

cudaError_t launch_batch(const SceneDesc* descs, const BatchHeader* hdr, uint32_t* queue, bool band, cudaStream_t s) {
  static int grids[4] = {0, 0, 0, 0};
  if (grids[0] == 0) {
    grids[0] = grid_for(reinterpret_cast<const void*>(batch_filter_alloc_kernel<false>), filt::kTX * filt::kTY);
    grids[1] = grid_for(reinterpret_cast<const void*>(batch_filter_alloc_kernel<true>), filt::kTX * filt::kTY);
    grids[2] = grid_for(reinterpret_cast<const void*>(batch_map_kernel), kMapTX * kMapTY);
    grids[3] = grid_for(reinterpret_cast<const void*>(batch_update_kernel<kBatchUT, kBatchUMinB>), kBatchUT);
  }
  batch_begin_kernel<<<1, 256, 0, s>>>(descs, hdr, queue);
  if (band) {
    batch_filter_alloc_kernel<true><<<grids[1], filt::kTX * filt::kTY, 0, s>>>(descs, hdr, queue);
  } else {
    batch_filter_alloc_kernel<false><<<grids[0], filt::kTX * filt::kTY, 0, s>>>(descs, hdr, queue);
  }
  batch_map_kernel<<<grids[2], kMapTX * kMapTY, 0, s>>>(descs, hdr, queue);
  batch_update_kernel<kBatchUT, kBatchUMinB><<<grids[3], kBatchUT, 0, s>>>(descs, hdr, queue);
  return cudaGetLastError();
}

// The step as one cooperative launch of batch_persistent_kernel (queue: 3 work-queue words; bar: 2 barrier words,
// zero before the first launch and left at zero arrivals by every completed launch).
cudaError_t launch_batch_persistent(const SceneDesc* descs, const BatchHeader* hdr, uint32_t* queue, uint32_t* bar,
                                    bool band, cudaStream_t s) {
  static int grids[2] = {0, 0};
  const void* fn = band ? reinterpret_cast<const void*>(batch_persistent_kernel<true>)
                        : reinterpret_cast<const void*>(batch_persistent_kernel<false>);
  int& grid = grids[band ? 1 : 0];
  if (grid == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kPersistThreads, 0);
    if (sms <= 0 || per_sm <= 0) return cudaErrorLaunchOutOfResources;
    grid = sms * per_sm;
  }
  void* args[] = {const_cast<SceneDesc**>(&descs), const_cast<BatchHeader**>(&hdr), &queue, &bar};
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kPersistThreads), args, 0, s);
}

cudaError_t launch_integrate(const float* depth, const Volume& V, const Params& p, int grid, float4* nmap,
                             cudaStream_t s) {
  const cudaError_t e = launch_integrate_prepare(depth, V, p, nmap, s);
  if (e != cudaSuccess) return e;
  return launch_integrate_update(depth, V, p, grid, nmap, s, 0);
}

}  // namespace VH_INTEGRATE_NS
}  // namespace vh
