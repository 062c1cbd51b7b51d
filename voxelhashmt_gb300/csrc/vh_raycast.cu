// vh_raycast.cu -- depth ray-cast of the fused volume (the TSDF ray-caster that produces depth maps of the
// fused surface, e.g. as training targets for a depth denoiser).  The reference has no ray-caster; the
// surface definition is the one its marching cubes uses: a voxel's observed layers are planes
// (planeSignedDistanceGpu, cuda_mesh_extractor.cu:259-262, normals unpacked as at :237-257).
//
// One thread per pixel.  The ray through the pixel centre is parameterised by camera depth z (camera-frame
// direction ((u - cx)/fx, (v - cy)/fy, 1)); it is sampled every `step` voxels of path length from min_depth
// to max_depth.  A voxel's distance at a point x is the plane distance n.x - offset of its heaviest observed
// layer, over all directions, whose normal faces the ray (n.d < 0; first such layer on ties): the
// best-supported surface of the voxel, so that the low-weight layers a few noisy observations leave in front
// of a surface do not stop the ray.  The distance at a sample x is the trilinear blend, with the weights of x
// among the 8 surrounding voxel centres, of those voxels' distances at x (over the voxels that have one,
// renormalised; none when they carry less than half of the weight).  The first step from a positive to a
// non-positive distance, with a drop of at most the truncation distance, is the hit; its depth is
// interpolated linearly.
// Unallocated blocks are skipped to the point where the ray leaves them.  Output: depth (camera z) per
// pixel, 0 where nothing is hit.
#include "vh_common.cuh"
#include "vh_kernels.h"

namespace vh {
namespace {

constexpr int kRTX = 16, kRTY = 8;
constexpr int kMaxRaySteps = 1 << 16;

// plane distance at world point x of the heaviest camera-facing layer of voxel (gx, gy, gz); false: no such layer
__device__ bool voxel_plane_distance(const Volume& V, const Params& p, int gx, int gy, int gz, f3 x, f3 dw,
                                     float& sdf) {
  const uint32_t b = lookup_block(V, gx >> 3, gy >> 3, gz >> 3);  // floor division by 8
  if (b == kInvalidBlock) return false;
  const int li = (gx & 7) + kBlockSide * ((gy & 7) + kBlockSide * (gz & 7));
  const uint32_t dirs = V.dir_mask[b];
  if (!dirs) return false;
  const int4 bk = V.block_keys[b];
  bool any = false;
  float best = 0.0f, best_w = 0.0f;
  for (int d = 0; d < kDirs; ++d) {
    if (!((dirs >> d) & 1U)) continue;
    float4 L[kLayers];
    load_bin(V, b, d, li, bk, p.voxel_size, L[0], L[1], L[2]);
#pragma unroll
    for (int l = 0; l < kLayers; ++l) {
      if (!(L[l].x > 0.0f)) continue;
      const f3 n = unpack_normal_mesh(__float_as_uint(L[l].w));
      if (!(dot3(n, dw) < 0.0f)) continue;
      if (!any || L[l].x > best_w) {
        any = true;
        best = n.x * x.x + n.y * x.y + n.z * x.z - L[l].z;
        best_w = L[l].x;
      }
    }
  }
  sdf = best;
  return any;
}

// trilinear blend at x of the plane distances of the 8 voxels whose centres surround x; false when less than
// half of the trilinear weight has a layer
__device__ bool blended_distance(const Volume& V, const Params& p, f3 x, f3 dw, float& sdf) {
  const float vs = p.voxel_size;
  const float fx = x.x / vs - 0.5f, fy = x.y / vs - 0.5f, fz = x.z / vs - 0.5f;
  const int x0 = static_cast<int>(floorf(fx)), y0 = static_cast<int>(floorf(fy)), z0 = static_cast<int>(floorf(fz));
  const float tx = fx - static_cast<float>(x0), ty = fy - static_cast<float>(y0), tz = fz - static_cast<float>(z0);
  float ws = 0.0f, acc = 0.0f;
  for (int k = 0; k < 8; ++k) {
    const int ax = k & 1, ay = (k >> 1) & 1, az = k >> 2;
    const float w = (ax ? tx : 1.0f - tx) * (ay ? ty : 1.0f - ty) * (az ? tz : 1.0f - tz);
    float s;
    if (!voxel_plane_distance(V, p, x0 + ax, y0 + ay, z0 + az, x, dw, s)) continue;
    acc += w * s;
    ws += w;
  }
  if (!(ws >= 0.5f)) return false;
  sdf = acc / ws;
  return true;
}

__global__ void __launch_bounds__(kRTX * kRTY) raycast_kernel(const Volume V, const Params p, float min_depth,
                                                              float max_depth, float step, float* __restrict__ out) {
  const int u = blockIdx.x * kRTX + threadIdx.x, v = blockIdx.y * kRTY + threadIdx.y;
  if (u >= p.width || v >= p.height) return;
  const f3 dc = mk3((static_cast<float>(u) - p.cx) / p.fx, (static_cast<float>(v) - p.cy) / p.fy, 1.0f);
  const f3 dw = xform_vector(p.T_wc, dc);
  const f3 o = mk3(p.T_wc.t[0], p.T_wc.t[1], p.T_wc.t[2]);
  const float dz = step * p.voxel_size / norm3(dc);
  const float vs = p.voxel_size;
  float z = min_depth;
  bool prev_ok = false;
  float prev_sdf = 0.0f, prev_z = 0.0f, result = 0.0f;
  for (int it = 0; it < kMaxRaySteps && z <= max_depth; ++it) {
    const f3 x = mk3(o.x + dw.x * z, o.y + dw.y * z, o.z + dw.z * z);
    const int gx = static_cast<int>(floorf(x.x / vs));
    const int gy = static_cast<int>(floorf(x.y / vs));
    const int gz = static_cast<int>(floorf(x.z / vs));
    const int bx = gx >> 3, by = gy >> 3, bz = gz >> 3;  // floor division by 8
    if (lookup_block(V, bx, by, bz) == kInvalidBlock) {
      // empty space: continue just past the point where the ray leaves this block
      prev_ok = false;
      float zexit = 3.0e38f;
      const int bb[3] = {bx, by, bz};
      const float oo[3] = {o.x, o.y, o.z}, dd[3] = {dw.x, dw.y, dw.z};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (dd[k] > 0.0f) zexit = fminf(zexit, (static_cast<float>((bb[k] + 1) * kBlockSide) * vs - oo[k]) / dd[k]);
        if (dd[k] < 0.0f) zexit = fminf(zexit, (static_cast<float>(bb[k] * kBlockSide) * vs - oo[k]) / dd[k]);
      }
      z = fmaxf(z + dz, zexit + 0.25f * dz);
      continue;
    }
    float sdf;
    if (!blended_distance(V, p, x, dw, sdf)) {
      prev_ok = false;
      z += dz;
      continue;
    }
    if (prev_ok && prev_sdf > 0.0f && sdf <= 0.0f && prev_sdf - sdf <= p.truncation) {
      result = prev_z + (z - prev_z) * (prev_sdf / (prev_sdf - sdf));
      break;
    }
    prev_ok = true;
    prev_sdf = sdf;
    prev_z = z;
    z += dz;
  }
  out[static_cast<size_t>(v) * p.width + u] = result;
}

}  // namespace

cudaError_t launch_raycast(const Volume& V, const Params& p, float min_depth, float max_depth, float step, float* out,
                           cudaStream_t s) {
  const dim3 block(kRTX, kRTY), grid((p.width + kRTX - 1) / kRTX, (p.height + kRTY - 1) / kRTY);
  raycast_kernel<<<grid, block, 0, s>>>(V, p, min_depth, max_depth, step, out);
  return cudaGetLastError();
}

}  // namespace vh
