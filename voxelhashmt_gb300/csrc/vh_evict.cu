// vh_evict.cu -- block eviction and lossless restore (vh_evict_blocks / vh_restore_blocks).
//
// The reference volume only grows: every block ever touched stays in host memory (voxel_hash_tsdf.h:133-139)
// and in the GPU cache (cuda_tsdf_integrator.cu:154-164).  A fixed device pool needs a way out for long
// trajectories: blocks whose layer update has not run for a while are copied out -- in the reference's Voxel
// layout (the export path, copyBlocksToFlat, voxel_hash_tsdf.h:147-163) or as the pool's own block image --
// and removed.  Removal keeps the pool dense, so every other kernel (marching cubes, export, recount) still
// walks [0, num_blocks):
//   1. victims: blocks with frame - block_stamp >= min_age_frames, and, down to a target count, the oldest further
//      ones (ties at the boundary age in pool order), listed in ascending pool order (two-level scan);
//   2. victims are copied out through a staging buffer;
//   3. the live blocks above the new count move down into the victims' slots below it (the two sets are
//      disjoint, so the moves run in parallel), with their keys, masks and stamps;
//   4. the freed tail is zeroed (new blocks start from zero layers) and the hash is rebuilt from the live keys
//      (no tombstones; the visible list of the last frame is cleared).
// Restore inserts blocks saved as block images back, bit for bit, for either layer format.
#include "vh_common.cuh"
#include "vh_kernels.h"

namespace vh {
namespace {

constexpr int kScanThreads = 1024;

__device__ __forceinline__ uint32_t block_age(const Volume& V, uint32_t b, uint32_t frame) {
  const uint32_t st = V.block_stamp[b];
  return st == 0U ? 0xffffffffU : frame - st;  // never updated: oldest
}

// histogram of block ages, bins [0, kAgeBins - 1], the last bin collecting older blocks
__global__ void __launch_bounds__(256) age_hist_kernel(const Volume V, uint32_t* __restrict__ hist) {
  const uint32_t n = min(V.counters->num_blocks, V.max_blocks);
  const uint32_t frame = V.counters->frame;
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
    atomicAdd(&hist[min(block_age(V, b, frame), static_cast<uint32_t>(kAgeBins - 1))], 1U);
  }
}

// predicate of the selection (EvictRule): 0 victims over [0, n); 1 survivors over [lo, n); 2 the blocks of the
// boundary bin that are not victims by age (the candidates of the pool-order tie break)
__device__ __forceinline__ bool selected(const Volume& V, uint32_t b, uint32_t frame, const EvictRule& r, int what,
                                         uint32_t lo) {
  const uint32_t age = block_age(V, b, frame);
  const uint32_t bin = min(age, static_cast<uint32_t>(kAgeBins - 1));
  if (what == 2) return bin == r.tie_bin && age < r.min_age;
  const bool victim = age >= r.min_age || bin > r.tie_bin || (bin == r.tie_bin && b < r.cut);
  return what == 0 ? victim : (b >= lo && !victim);
}

// per-CTA counts of the selected blocks of [cta * 1024, cta * 1024 + 1024)
__global__ void __launch_bounds__(kScanThreads) select_count_kernel(const Volume V, uint32_t n, const EvictRule rule,
                                                                    int what, uint32_t lo,
                                                                    uint32_t* __restrict__ cta_counts) {
  __shared__ uint32_t s_count;
  if (threadIdx.x == 0) s_count = 0U;
  __syncthreads();
  const uint32_t frame = V.counters->frame;
  const uint32_t b = blockIdx.x * kScanThreads + threadIdx.x;
  const bool sel = b < n && selected(V, b, frame, rule, what, lo);
  const uint32_t ballot = __ballot_sync(0xffffffffU, sel);
  if ((threadIdx.x & 31) == 0 && ballot) atomicAdd(&s_count, static_cast<uint32_t>(__popc(ballot)));
  __syncthreads();
  if (threadIdx.x == 0) cta_counts[blockIdx.x] = s_count;
}

// exclusive scan of the per-CTA counts in place (one CTA); total -> *total
__global__ void __launch_bounds__(kScanThreads) select_scan_kernel(uint32_t* __restrict__ cta_counts, uint32_t nctas,
                                                                   uint32_t* __restrict__ total) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_carry;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_carry = 0U;
  __syncthreads();
  for (uint32_t start = 0; start < nctas; start += kScanThreads) {
    const uint32_t i = start + tid;
    const uint32_t v = i < nctas ? cta_counts[i] : 0U;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffU, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const uint32_t w = s_warp[lane];
      uint32_t wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffU, wi, o);
        if (lane >= o) wi += t;
      }
      s_warp[lane] = wi - w;
    }
    __syncthreads();
    const uint32_t carry = s_carry;
    if (i < nctas) cta_counts[i] = carry + s_warp[warp] + incl - v;
    __syncthreads();
    if (tid == kScanThreads - 1) s_carry = carry + s_warp[warp] + incl;
    __syncthreads();
  }
  if (tid == 0) *total = s_carry;
}

// the selected blocks in ascending order: list[offset of the CTA + rank within the CTA] = b
__global__ void __launch_bounds__(kScanThreads) select_write_kernel(const Volume V, uint32_t n, const EvictRule rule,
                                                                    int what, uint32_t lo,
                                                                    const uint32_t* __restrict__ cta_offsets,
                                                                    uint32_t* __restrict__ list) {
  __shared__ uint32_t s_warp[32];
  const uint32_t frame = V.counters->frame;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t b = blockIdx.x * kScanThreads + tid;
  const bool sel = b < n && selected(V, b, frame, rule, what, lo);
  const uint32_t ballot = __ballot_sync(0xffffffffU, sel);
  if (lane == 0) s_warp[warp] = static_cast<uint32_t>(__popc(ballot));
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = s_warp[lane];
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffU, wi, o);
      if (lane >= o) wi += t;
    }
    s_warp[lane] = wi - w;
  }
  __syncthreads();
  if (sel) list[cta_offsets[blockIdx.x] + s_warp[warp] + __popc(ballot & ((1U << lane) - 1U))] = b;
}

__device__ __forceinline__ size_t block_words(const Volume& V) {  // uint4 words of one pool block
  return V.layers16 != nullptr ? static_cast<size_t>(kDirs) * kBlockVoxels * kBinWords16
                               : static_cast<size_t>(kDirs) * kBlockVoxels * kLayers;
}
__device__ __forceinline__ uint4* block_base(const Volume& V, uint32_t b) {
  return V.layers16 != nullptr ? V.layers16 + static_cast<size_t>(b) * block_words(V)
                               : reinterpret_cast<uint4*>(V.layers) + static_cast<size_t>(b) * block_words(V);
}

// listed blocks' images (the pool's own layout) and keys into a staging buffer: one CTA per block
__global__ void __launch_bounds__(256) copy_out_native_kernel(const Volume V, const uint32_t* __restrict__ list,
                                                              uint32_t n, int* __restrict__ keys,
                                                              uint4* __restrict__ out) {
  const size_t words = block_words(V);
  for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
    const uint32_t b = list[i];
    const uint4* src = block_base(V, b);
    uint4* dst = out + static_cast<size_t>(i) * words;
    for (size_t w = threadIdx.x; w < words; w += blockDim.x) dst[w] = src[w];
    if (threadIdx.x == 0) {
      const int4 k = V.block_keys[b];
      keys[3 * i] = k.x;
      keys[3 * i + 1] = k.y;
      keys[3 * i + 2] = k.z;
    }
  }
}

// listed blocks in the reference Voxel layout voxels[i][li][d][l] (decoded FP16 bins) and keys
__global__ void __launch_bounds__(256) copy_out_reference_kernel(const Volume V, const uint32_t* __restrict__ list,
                                                                 uint32_t n, int* __restrict__ keys,
                                                                 float4* __restrict__ out) {
  const size_t total = static_cast<size_t>(n) * kBlockVoxels * kDirs;
  for (size_t t = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int d = static_cast<int>(t % kDirs);
    const int li = static_cast<int>((t / kDirs) % kBlockVoxels);
    const uint32_t i = static_cast<uint32_t>(t / (static_cast<size_t>(kDirs) * kBlockVoxels));
    const uint32_t b = list[i];
    const int4 bk = V.block_keys[b];
    float4 L0, L1, L2;
    load_bin(V, b, d, li, bk, V.voxel_size, L0, L1, L2);
    float4* o = out + t * kLayers;
    o[0] = L0;
    o[1] = L1;
    o[2] = L2;
    if (d == 0 && li == 0) {
      keys[3 * i] = bk.x;
      keys[3 * i + 1] = bk.y;
      keys[3 * i + 2] = bk.z;
    }
  }
}

// block src[i] -> dst[i] with its key, masks and stamp: one CTA per move
// observed voxels of the victims (set bits of their observed-voxel masks; a bit is set exactly when the voxel
// has a layer of positive weight), subtracted from the volume's count once the victims are gone: the same
// number a recount of the surviving pool gives, without reading the pool
__global__ void __launch_bounds__(256) victim_observed_kernel(const Volume V, const uint32_t* __restrict__ list,
                                                              uint32_t n, unsigned long long* __restrict__ out) {
  constexpr uint32_t kWords = kBlockVoxels / 32;
  unsigned long long local = 0ULL;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n * kWords; i += gridDim.x * blockDim.x) {
    local += static_cast<unsigned long long>(__popc(V.obs_mask[static_cast<size_t>(list[i / kWords]) * kWords + i % kWords]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffU, local, o);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(out, local);
}

__global__ void subtract_observed_kernel(Counters* __restrict__ c, const unsigned long long* __restrict__ removed) {
  c->observed_voxels -= *removed;
}

__global__ void __launch_bounds__(256) move_blocks_kernel(const Volume V, const uint32_t* __restrict__ src,
                                                          const uint32_t* __restrict__ dst, uint32_t n) {
  const size_t words = block_words(V);
  for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
    const uint32_t s = src[i], d = dst[i];
    const uint4* from = block_base(V, s);
    uint4* to = block_base(V, d);
    for (size_t w = threadIdx.x; w < words; w += blockDim.x) to[w] = from[w];
    const int mw = kBlockVoxels / 32;
    if (threadIdx.x < mw) {
      V.obs_mask[static_cast<size_t>(d) * mw + threadIdx.x] = V.obs_mask[static_cast<size_t>(s) * mw + threadIdx.x];
    }
    if (threadIdx.x == 0) {
      V.block_keys[d] = V.block_keys[s];
      V.dir_mask[d] = V.dir_mask[s];
      V.block_stamp[d] = V.block_stamp[s];
    }
  }
}

// every live block's key into the emptied table (keys are unique: a plain claim of the first empty slot)
__global__ void __launch_bounds__(256) rehash_kernel(const Volume V, uint32_t live) {
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < live; b += gridDim.x * blockDim.x) {
    const int4 k = V.block_keys[b];
    unsigned long long key;
    if (!pack_block_key(k.x, k.y, k.z, key)) {
      atomicOr(&V.counters->error, kErrKeyRange);
      continue;
    }
    uint32_t slot = hash_block_key(k.x, k.y, k.z) & V.mask;
    bool done = false;
    for (uint32_t probe = 0; probe < V.capacity && !done; ++probe) {
      if (atomicCAS(&V.slot_keys[slot], kEmptyKey, key) == kEmptyKey) {
        V.slot_block[slot] = b;
        done = true;
      } else {
        slot = (slot + 1U) & V.mask;
      }
    }
    if (!done) atomicOr(&V.counters->error, kErrHashFull);
  }
}

// restore: block images into the pool blocks idx[i] (from import_keys), masks rebuilt, stamped with the frame
__global__ void __launch_bounds__(256) restore_native_kernel(const Volume V, const uint4* __restrict__ in, uint32_t n,
                                                             const uint32_t* __restrict__ idx) {
  const size_t words = block_words(V);
  const uint32_t frame = V.counters->frame;
  for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
    const uint32_t b = idx[i];
    if (b == kInvalidBlock) continue;
    uint4* to = block_base(V, b);
    const uint4* from = in + static_cast<size_t>(i) * words;
    for (size_t w = threadIdx.x; w < words; w += blockDim.x) to[w] = from[w];
    __syncthreads();
    // observed mask and direction mask from the copied bins
    for (int li = threadIdx.x; li < kBlockVoxels; li += blockDim.x) {
      uint32_t dirs = 0U;
      for (int d = 0; d < kDirs; ++d)
        if (bin_observed(V, b, d, li)) dirs |= 1U << d;
      const unsigned ballot = __ballot_sync(0xffffffffU, dirs != 0U);
      if ((li & 31) == 0) V.obs_mask[static_cast<size_t>(b) * (kBlockVoxels / 32) + (li >> 5)] = ballot;
      if (dirs) atomicOr(&V.dir_mask[b], dirs);
    }
    if (threadIdx.x == 0) V.block_stamp[b] = frame;
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_age_hist(const Volume& V, uint32_t* hist, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(hist, 0, kAgeBins * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  age_hist_kernel<<<152 * 8, 256, 0, s>>>(V, hist);
  return cudaGetLastError();
}

cudaError_t launch_select(const Volume& V, uint32_t n, const EvictRule& rule, int what, uint32_t lo,
                          uint32_t* cta_scratch, uint32_t* total, uint32_t* list, cudaStream_t s) {
  if (n == 0) return cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
  const uint32_t nctas = (n + kScanThreads - 1) / kScanThreads;
  select_count_kernel<<<nctas, kScanThreads, 0, s>>>(V, n, rule, what, lo, cta_scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  select_scan_kernel<<<1, kScanThreads, 0, s>>>(cta_scratch, nctas, total);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  select_write_kernel<<<nctas, kScanThreads, 0, s>>>(V, n, rule, what, lo, cta_scratch, list);
  return cudaGetLastError();
}

cudaError_t launch_copy_out(const Volume& V, const uint32_t* list, uint32_t n, int native, int* keys, void* out,
                            cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (native) {
    copy_out_native_kernel<<<152 * 4, 256, 0, s>>>(V, list, n, keys, static_cast<uint4*>(out));
  } else {
    copy_out_reference_kernel<<<152 * 8, 256, 0, s>>>(V, list, n, keys, static_cast<float4*>(out));
  }
  return cudaGetLastError();
}

cudaError_t launch_victim_observed(const Volume& V, const uint32_t* list, uint32_t n, unsigned long long* out,
                                   cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess || n == 0) return e;
  victim_observed_kernel<<<152 * 4, 256, 0, s>>>(V, list, n, out);
  return cudaGetLastError();
}

cudaError_t launch_subtract_observed(const Volume& V, const unsigned long long* removed, cudaStream_t s) {
  subtract_observed_kernel<<<1, 1, 0, s>>>(V.counters, removed);
  return cudaGetLastError();
}

cudaError_t launch_move_blocks(const Volume& V, const uint32_t* src, const uint32_t* dst, uint32_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  move_blocks_kernel<<<152 * 4, 256, 0, s>>>(V, src, dst, n);
  return cudaGetLastError();
}

cudaError_t launch_rehash(const Volume& V, uint32_t live, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(V.slot_keys, 0xFF, static_cast<size_t>(V.capacity) * sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(V.slot_stamp, 0, static_cast<size_t>(V.capacity) * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  if (live == 0) return cudaSuccess;
  rehash_kernel<<<(live + 255) / 256, 256, 0, s>>>(V, live);
  return cudaGetLastError();
}

cudaError_t launch_restore_native(const Volume& V, const void* in, uint32_t n, const uint32_t* idx, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  restore_native_kernel<<<152 * 4, 256, 0, s>>>(V, static_cast<const uint4*>(in), n, idx);
  return cudaGetLastError();
}

}  // namespace vh
