// vh_alloc.cu -- block allocation kernels (reference: src/cuda_block_allocator.cu:198-300); the device code,
// with how it differs from the reference, is in vh_alloc.cuh.
#include "vh_alloc.cuh"
#include "vh_kernels.h"

namespace vh {
namespace {

using alloc::kThreads;
using alloc::kTX;
using alloc::kTY;

__global__ void __launch_bounds__(kThreads) alloc_kernel(const float* __restrict__ depth, const Volume V,
                                                         const Params p) {
  __shared__ alloc::Smem S;
  alloc::alloc_tile(depth, V, p, blockIdx.x * kTX, blockIdx.y * kTY, threadIdx.y * kTX + threadIdx.x, S);
}

__global__ void visible_keys_kernel(const Volume V, int* __restrict__ keys) {
  const uint32_t n = V.counters->visible_count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int x, y, z;
    unpack_block_key(V.slot_keys[V.visible[i]], x, y, z);
    keys[3 * i] = x;
    keys[3 * i + 1] = y;
    keys[3 * i + 2] = z;
  }
}

}  // namespace

cudaError_t launch_alloc(const float* depth, const Volume& V, const Params& p, cudaStream_t s) {
  if (p.sample_width <= 0 || p.sample_height <= 0) return cudaSuccess;
  const dim3 block(kTX, kTY);
  const dim3 grid((p.sample_width + kTX - 1) / kTX, (p.sample_height + kTY - 1) / kTY);
  alloc_kernel<<<grid, block, 0, s>>>(depth, V, p);
  return cudaGetLastError();
}

cudaError_t launch_visible_keys(const Volume& V, int* keys, cudaStream_t s) {
  visible_keys_kernel<<<152, 256, 0, s>>>(V, keys);
  return cudaGetLastError();
}

}  // namespace vh
