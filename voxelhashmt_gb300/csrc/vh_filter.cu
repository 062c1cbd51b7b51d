// vh_filter.cu -- depth bilateral filter with normal gating, one kernel.
//
// Reference: src/cuda_tsdf_integrator.cu:581-648 (estimateSurfaceNormalAtPixel / estimateDepthNormalsKernel)
// and :650-725 (bilateralFilterDepthKernel), two kernels with a float3 + u8 normal map round trip through
// global memory.  Here one kernel (device code in vh_filter.cuh): HBM traffic is one read and one write of
// the depth image.
#include "vh_filter.cuh"
#include "vh_kernels.h"

namespace vh {
namespace {

using filt::kDH;
using filt::kDW;
using filt::kNH;
using filt::kNW;
using filt::kR;
using filt::kTX;
using filt::kTY;

template <bool kBeginFrame>
__global__ void __launch_bounds__(kTX* kTY) filter_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                          const Params p, Counters* counters) {
  __shared__ filt::Smem S;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  if (kBeginFrame && blockIdx.x == 0 && blockIdx.y == 0 && tid == 0) filt::begin_frame(counters);
  filt::filter_tile(in, out, p, blockIdx.x * kTX, blockIdx.y * kTY, tid, S);
}

__global__ void __launch_bounds__(kTX* kTY) normals_kernel(const float* __restrict__ in, float* __restrict__ normals,
                                                           unsigned char* __restrict__ valid, const Params p) {
  __shared__ float s_depth[kDH][kDW];
  __shared__ float4 s_normal[kNH][kNW];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTX + tx;
  const int u0 = blockIdx.x * kTX, v0 = blockIdx.y * kTY;
  filt::stage_tile(in, s_depth, s_normal, u0, v0, p, tid);
  const int u = u0 + tx, v = v0 + ty;
  if (u >= p.width || v >= p.height) return;
  const size_t ci = static_cast<size_t>(v) * p.width + u;
  const float4 n = s_normal[ty + kR][tx + kR];
  normals[3 * ci] = n.x;
  normals[3 * ci + 1] = n.y;
  normals[3 * ci + 2] = n.z;
  valid[ci] = n.w != 0.0f ? 1 : 0;
}

__global__ void begin_frame_kernel(Counters* counters) { filt::begin_frame(counters); }

}  // namespace

cudaError_t launch_filter(const float* in, float* out, const Params& p, Counters* begin_frame, cudaStream_t s) {
  if (p.filter_radius < 0 || p.filter_radius > kR) return cudaErrorInvalidValue;
  const dim3 block(kTX, kTY);
  const dim3 grid((p.width + kTX - 1) / kTX, (p.height + kTY - 1) / kTY);
  if (begin_frame) {
    filter_kernel<true><<<grid, block, 0, s>>>(in, out, p, begin_frame);
  } else {
    filter_kernel<false><<<grid, block, 0, s>>>(in, out, p, nullptr);
  }
  return cudaGetLastError();
}

cudaError_t launch_depth_normals(const float* in, float* normals, unsigned char* valid, const Params& p,
                                 cudaStream_t s) {
  const dim3 block(kTX, kTY);
  const dim3 grid((p.width + kTX - 1) / kTX, (p.height + kTY - 1) / kTY);
  normals_kernel<<<grid, block, 0, s>>>(in, normals, valid, p);
  return cudaGetLastError();
}

cudaError_t launch_begin_frame(Counters* c, cudaStream_t s) {
  begin_frame_kernel<<<1, 1, 0, s>>>(c);
  return cudaGetLastError();
}

}  // namespace vh
