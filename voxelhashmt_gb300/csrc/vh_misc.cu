// vh_misc.cu -- pool-wide maintenance kernels: observed-voxel recount and export to the reference layout.
#include "vh_common.cuh"
#include "vh_kernels.h"

namespace vh {
namespace {

// countObservedVoxelsKernel (src/cuda_tsdf_integrator.cu:905-930) with a warp reduction and one atomic per
// warp; the integrate kernel maintains the same number incrementally, this pass re-derives it from the pool.
__global__ void __launch_bounds__(256) recount_kernel(const Volume V, unsigned long long* __restrict__ out) {
  const uint32_t nblocks = min(V.counters->num_blocks, V.max_blocks);
  const size_t nvox = static_cast<size_t>(nblocks) * kBlockVoxels;
  unsigned long long local = 0ULL;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < nvox;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const uint32_t b = static_cast<uint32_t>(i / kBlockVoxels);
    const int li = static_cast<int>(i % kBlockVoxels);
    bool obs = false;
    for (int d = 0; d < kDirs && !obs; ++d) {
      const float4* L = V.layers + layer_index(b, d, li, 0);
      obs = L[0].x > 0.0f || L[1].x > 0.0f || L[2].x > 0.0f;
    }
    local += obs ? 1ULL : 0ULL;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffU, local, o);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(out, local);
}

// pool (direction-major) -> reference Voxel layout: voxels[b][li][d][l]
__global__ void __launch_bounds__(256) export_kernel(const Volume V, uint32_t first, uint32_t count,
                                                     int* __restrict__ keys, float4* __restrict__ voxels) {
  const size_t total = static_cast<size_t>(count) * kBlockVoxels * kDirs * kLayers;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int l = static_cast<int>(i % kLayers);
    const int d = static_cast<int>((i / kLayers) % kDirs);
    const int li = static_cast<int>((i / (kLayers * kDirs)) % kBlockVoxels);
    const uint32_t bo = static_cast<uint32_t>(i / (static_cast<size_t>(kLayers) * kDirs * kBlockVoxels));
    voxels[i] = V.layers[layer_index(first + bo, d, li, l)];
    if (keys && d == 0 && l == 0 && li == 0) {
      const int4 k = V.block_keys[first + bo];
      keys[3 * bo] = k.x;
      keys[3 * bo + 1] = k.y;
      keys[3 * bo + 2] = k.z;
    }
  }
}

}  // namespace

cudaError_t launch_recount(const Volume& V, unsigned long long* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  recount_kernel<<<152 * 8, 256, 0, s>>>(V, out);
  return cudaGetLastError();
}

cudaError_t launch_export(const Volume& V, uint32_t first, uint32_t count, int* keys, float4* voxels,
                          cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  export_kernel<<<152 * 8, 256, 0, s>>>(V, first, count, keys, voxels);
  return cudaGetLastError();
}

}  // namespace vh
