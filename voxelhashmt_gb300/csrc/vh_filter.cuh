// vh_filter.cuh -- device code of the depth bilateral filter (reference: src/cuda_tsdf_integrator.cu:581-725),
// shared by the single-frame kernels (vh_filter.cu) and the multi-scene batch (vh_integrate.cu).
//
// One CTA of kTX x kTY threads stages a 32x8 output tile of depth plus a 3-pixel halo in shared memory,
// computes the normals of the tile plus a 2-pixel halo into shared memory, and runs the 5x5 joint bilateral
// from shared memory: HBM traffic is one read and one write of the depth image.
// Compiled with VH_FAST_MATH (the opt-in fast-math form), a tap's range and angular Gaussians are one hardware
// exponential of the summed exponents instead of two exact ones.
#pragma once

#include "vh_common.cuh"

namespace vh {
namespace filt {

constexpr int kTX = 32;
constexpr int kTY = 8;
constexpr int kR = 2;                    // largest filter radius the tile supports
constexpr int kDW = kTX + 2 * (kR + 1);  // depth tile incl. halo
constexpr int kDH = kTY + 2 * (kR + 1);
constexpr int kNW = kTX + 2 * kR;        // normal tile incl. halo
constexpr int kNH = kTY + 2 * kR;

// estimateSurfaceNormalAtPixel (cuda_tsdf_integrator.cu:581-627) on the staged tile; (sx, sy) = tile coords
// of pixel (u, v) in s_depth.
__device__ __forceinline__ float4 pixel_normal(const float (*s_depth)[kDW], int sx, int sy, int u, int v,
                                               const Params& p) {
  const float4 none = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (u <= 0 || v <= 0 || u + 1 >= p.width || v + 1 >= p.height) return none;
  const float dc = s_depth[sy][sx];
  const float dl = s_depth[sy][sx - 1];
  const float dr = s_depth[sy][sx + 1];
  const float du = s_depth[sy - 1][sx];
  const float dd = s_depth[sy + 1][sx];
  if (!(dc > 0.0f) || !(dl > 0.0f) || !(dr > 0.0f) || !(du > 0.0f) || !(dd > 0.0f)) return none;
  const float thr = disc_threshold(p, dc);
  if (fabsf(dl - dc) > thr || fabsf(dr - dc) > thr || fabsf(du - dc) > thr || fabsf(dd - dc) > thr) return none;
  const f3 pl = backproject(static_cast<float>(u - 1), static_cast<float>(v), dl, p);
  const f3 pr = backproject(static_cast<float>(u + 1), static_cast<float>(v), dr, p);
  const f3 pu = backproject(static_cast<float>(u), static_cast<float>(v - 1), du, p);
  const f3 pd = backproject(static_cast<float>(u), static_cast<float>(v + 1), dd, p);
  f3 n = normalize3(cross3(sub3(pd, pu), sub3(pr, pl)));
  if (norm3(n) <= 1e-6f) return none;
  n = orient_toward_camera(n, backproject(static_cast<float>(u), static_cast<float>(v), dc, p));
  if (!(norm3(n) > 1e-6f)) return none;
  return make_float4(n.x, n.y, n.z, 1.0f);
}

__device__ __forceinline__ void stage_tile(const float* __restrict__ in, float (*s_depth)[kDW],
                                           float4 (*s_normal)[kNW], int u0, int v0, const Params& p, int tid) {
  for (int i = tid; i < kDW * kDH; i += kTX * kTY) {
    const int dy = i / kDW, dx = i - dy * kDW;
    const int gu = u0 + dx - (kR + 1), gv = v0 + dy - (kR + 1);
    s_depth[dy][dx] = (gu >= 0 && gu < p.width && gv >= 0 && gv < p.height)
                          ? __ldg(&in[static_cast<size_t>(gv) * p.width + gu])
                          : 0.0f;
  }
  __syncthreads();
  for (int i = tid; i < kNW * kNH; i += kTX * kTY) {
    const int ny = i / kNW, nx = i - ny * kNW;
    s_normal[ny][nx] = pixel_normal(s_depth, nx + 1, ny + 1, u0 + nx - kR, v0 + ny - kR, p);
  }
  __syncthreads();
}

struct Smem {
  float depth[kDH][kDW];
  float4 normal[kNH][kNW];
  float spatial[(2 * kR + 1) * (2 * kR + 1)];
};

// The taps of radius R around staged pixel (tx, ty), in the reference's order (rows dv outer, columns du
// inner).  No image-bounds test per tap: the staged tile holds 0 outside the image, which the sd <= 0 test
// rejects exactly as the reference's bounds test does.
template <int R>
__device__ __forceinline__ void bilateral_taps(const Smem& S, int tx, int ty, float center, bool has_cn, f3 cn,
                                               float thr, const Params& p, float& wds, float& ws) {
#pragma unroll
  for (int dv = -R; dv <= R; ++dv) {
#pragma unroll
    for (int du = -R; du <= R; ++du) {
      const float sd = S.depth[ty + kR + 1 + dv][tx + kR + 1 + du];
      if (sd <= 0.0f || fabsf(sd - center) > thr) continue;
      const float delta = sd - center;
      const float range = delta * delta;
#ifdef VH_FAST_MATH
      // one hardware exponential of the summed exponents: exp(-a) exp(-b) = exp(-(a + b))
      float e = range * p.filter_k_range;
      if (has_cn) {
        const float4 sn = S.normal[ty + kR + dv][tx + kR + du];
        if (sn.w == 0.0f) continue;
        const float cosine = clampf(dot3(cn, mk3(sn.x, sn.y, sn.z)), -1.0f, 1.0f);
        if (cosine < p.filter_min_cos) continue;
        const float ad = 1.0f - cosine;
        e += ad * ad * p.filter_k_angular;
      }
      const float w = S.spatial[(dv + kR) * (2 * kR + 1) + (du + kR)] * __expf(-e);
#else
      float w = S.spatial[(dv + kR) * (2 * kR + 1) + (du + kR)] * gaussian(range, p.filter_k_range);
      if (has_cn) {
        const float4 sn = S.normal[ty + kR + dv][tx + kR + du];
        if (sn.w == 0.0f) continue;
        const float cosine = clampf(dot3(cn, mk3(sn.x, sn.y, sn.z)), -1.0f, 1.0f);
        if (cosine < p.filter_min_cos) continue;
        const float ad = 1.0f - cosine;
        w *= gaussian(ad * ad, p.filter_k_angular);
      }
#endif
      wds += w * sd;
      ws += w;
    }
  }
}

// bilateralFilterDepthKernel (cuda_tsdf_integrator.cu:650-725) for the output tile at (u0, v0); every thread of
// the CTA calls it (it synchronises); thread (tx, ty) = tid % kTX, tid / kTX writes pixel (u0 + tx, v0 + ty)
// and returns the value it wrote (0 for a pixel outside the image).
__device__ __forceinline__ float filter_tile(const float* __restrict__ in, float* __restrict__ out, const Params& p,
                                             int u0, int v0, int tid, Smem& S) {
  const int tx = tid % kTX, ty = tid / kTX;
  if (tid < (2 * kR + 1) * (2 * kR + 1)) {
    const int du = tid % (2 * kR + 1) - kR, dv = tid / (2 * kR + 1) - kR;
    // exp of the spatial term depends only on (du, dv): evaluated once per tile, same value as per tap
    S.spatial[tid] = gaussian(static_cast<float>(du * du + dv * dv), p.filter_k_spatial);
  }
  stage_tile(in, S.depth, S.normal, u0, v0, p, tid);

  const int u = u0 + tx, v = v0 + ty;
  if (u >= p.width || v >= p.height) return 0.0f;
  const size_t ci = static_cast<size_t>(v) * p.width + u;
  const float center = S.depth[ty + kR + 1][tx + kR + 1];
  if (center <= 0.0f) {
    out[ci] = 0.0f;
    return 0.0f;
  }
  const float4 cn4 = S.normal[ty + kR][tx + kR];
  const bool has_cn = cn4.w != 0.0f;
  const f3 cn = has_cn ? mk3(cn4.x, cn4.y, cn4.z) : mk3(0.0f, 0.0f, 0.0f);
  const float thr = disc_threshold(p, center);
  float wds = 0.0f, ws = 0.0f;
  if (p.filter_radius == 2) {
    bilateral_taps<2>(S, tx, ty, center, has_cn, cn, thr, p, wds, ws);
  } else if (p.filter_radius == 1) {
    bilateral_taps<1>(S, tx, ty, center, has_cn, cn, thr, p, wds, ws);
  } else {
    bilateral_taps<0>(S, tx, ty, center, has_cn, cn, thr, p, wds, ws);
  }
  const float result = ws > 1e-6f ? (wds / ws) : center;
  out[ci] = result;
  return result;
}

// the per-frame counter reset of a new frame (the frame stamp marks visible slots)
__device__ __forceinline__ void begin_frame(Counters* counters) {
  counters->frame += 1U;
  counters->visible_count = 0U;
  counters->new_blocks = 0U;
  counters->integrated_voxels = 0U;
  counters->active_voxels = 0U;
  counters->update_queue = 0U;
}

}  // namespace filt
}  // namespace vh
