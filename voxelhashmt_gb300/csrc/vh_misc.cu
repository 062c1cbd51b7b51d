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
    for (int d = 0; d < kDirs && !obs; ++d) obs = bin_observed(V, b, d, li);
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
    if (V.layers16 == nullptr) {
      voxels[i] = V.layers[layer_index(first + bo, d, li, l)];
    } else {
      float4 L[kLayers];
      load_bin(V, first + bo, d, li, V.block_keys[first + bo], V.voxel_size, L[0], L[1], L[2]);
      voxels[i] = L[l];
    }
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

namespace vh {
namespace {

// Insert (or find) each imported key; idx[i] receives its pool block (kInvalidBlock when the pool is full).
__global__ void import_keys_kernel(const Volume V, const int* __restrict__ keys, uint32_t n, uint32_t* __restrict__ idx) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int x = keys[3 * i], y = keys[3 * i + 1], z = keys[3 * i + 2];
    unsigned long long key;
    idx[i] = kInvalidBlock;
    if (!pack_block_key(x, y, z, key)) {
      atomicOr(&V.counters->error, kErrKeyRange);
      continue;
    }
    uint32_t slot = hash_block_key(x, y, z) & V.mask;
    bool done = false;
    for (uint32_t probe = 0; probe < V.capacity && !done; ++probe) {
      unsigned long long cur = atomicCAS(&V.slot_keys[slot], kEmptyKey, key);
      if (cur == kEmptyKey) {
        uint32_t b = atomicAdd(&V.counters->num_blocks, 1U);
        if (b >= V.max_blocks) {
          atomicOr(&V.counters->error, kErrPoolFull);
          b = kInvalidBlock;
        } else {
          V.block_keys[b] = make_int4(x, y, z, 0);
        }
        V.slot_block[slot] = b;
        idx[i] = b;
        done = true;
      } else if (cur == key) {
        idx[i] = V.slot_block[slot];
        done = true;
      } else {
        slot = (slot + 1U) & V.mask;
      }
    }
    if (!done) atomicOr(&V.counters->error, kErrHashFull);
  }
}

// reference Voxel layout [i][li][d][l] -> pool (direction-major); rebuilds the observed and direction masks
__global__ void __launch_bounds__(256) import_voxels_kernel(const Volume V, const float4* __restrict__ voxels,
                                                            uint32_t n, const uint32_t* __restrict__ idx) {
  for (size_t t = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; t < static_cast<size_t>(n) * kBlockVoxels;
       t += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const uint32_t i = static_cast<uint32_t>(t / kBlockVoxels);
    const int li = static_cast<int>(t % kBlockVoxels);
    const uint32_t b = idx[i];
    bool obs = false;
    uint32_t dirs = 0U;
    if (b != kInvalidBlock) {
      const float4* src = voxels + t * kDirs * kLayers;
      const int4 bk = V.block_keys[b];
      for (int d = 0; d < kDirs; ++d) {
        const float4 L0 = src[d * kLayers], L1 = src[d * kLayers + 1], L2 = src[d * kLayers + 2];
        store_bin(V, b, d, li, bk, V.voxel_size, L0, L1, L2);
        if (L0.x > 0.0f || L1.x > 0.0f || L2.x > 0.0f) {
          obs = true;
          dirs |= 1U << d;
        }
      }
    }
    const unsigned ballot = __ballot_sync(__activemask(), obs);
    if (b != kInvalidBlock) {
      if ((li & 31) == 0) V.obs_mask[static_cast<size_t>(b) * (kBlockVoxels / 32) + (li >> 5)] = ballot;
      if (dirs) atomicOr(&V.dir_mask[b], dirs);
    }
  }
}

}  // namespace

cudaError_t launch_import_keys(const Volume& V, const int* keys, uint32_t n, uint32_t* idx, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  import_keys_kernel<<<(n + 255) / 256, 256, 0, s>>>(V, keys, n, idx);
  return cudaGetLastError();
}

cudaError_t launch_import(const Volume& V, const int* keys, const float4* voxels, uint32_t n, uint32_t* idx,
                          cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  import_keys_kernel<<<(n + 255) / 256, 256, 0, s>>>(V, keys, n, idx);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  import_voxels_kernel<<<152 * 8, 256, 0, s>>>(V, voxels, n, idx);
  return cudaGetLastError();
}

}  // namespace vh
