// vh_static_scratch.cu -- block allocation that allocates nothing: vh_allocate_static_scratch.
//
// Some callers cannot call cudaMalloc after start-up: real-time tracking loops whose latency budget forbids
// allocator calls, and applications that hand the whole device to their own memory pool, so that a library
// allocating behind their back would fail or fragment it.  For them this entry point runs the same
// allocation as vh_allocate on a keys-only table, but keeps its scratch (hash slots, slot stamps, visible
// list and counters) in the file-scope device array below.  The caller passes the depth and the output
// key buffer; nothing is allocated per call or at set-up.
//
// The array is part of the library image: every GPU that loads the library holds kScratchBytes of it until
// the process exits.  All calls share it and it keeps the last call's contents; each call clears the hash
// slots, stamps and counters it relies on.  Each GPU has its own copy; two calls that overlap on the same GPU
// (issued on different streams or from different host threads) race on it.
#include <cuda_runtime.h>

#include "../../include/voxelhash_gb300.h"
#include "vh_common.cuh"
#include "vh_kernels.h"

namespace {

// 2^20 slots: the reference sizes its table as nextPow2(2 * max(2048, 16 * samples))
// (cuda_block_allocator.cu:322-323), so frames of up to 32,768 sampled pixels fit.
constexpr uint32_t kStaticBuckets = 1U << 20;
constexpr size_t kKeysBytes = static_cast<size_t>(kStaticBuckets) * sizeof(unsigned long long);
constexpr size_t kSlotU32Bytes = static_cast<size_t>(kStaticBuckets) * sizeof(uint32_t);
constexpr size_t kCountersOffset = kKeysBytes + 3 * kSlotU32Bytes;
constexpr size_t kScratchBytes = kCountersOffset + 256;  // 20 MiB + 256 B

static __device__ __align__(256) unsigned char g_vh_static_scratch[kScratchBytes];

// The device address of the array in the current device's context.  The runtime resolves it on the host (no
// allocation, no stream operation).  It is looked up on every call rather than cached per device: a
// cudaDeviceReset destroys the context, and the next context may load the library's device code, and with it
// the array, at another address.
vh_status scratch_for_current_device(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return VH_ERR_NO_DEVICE;
  }
  void* ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, g_vh_static_scratch) != cudaSuccess || ptr == nullptr) {
    cudaGetLastError();
    return VH_ERR_CUDA;
  }
  *out = ptr;
  return VH_OK;
}

uint32_t next_pow2(uint64_t x) {
  uint64_t p = 1;
  while (p < x) p <<= 1;
  return p > 0xffffffffULL ? 0U : static_cast<uint32_t>(p);
}

}  // namespace

extern "C" vh_status vh_allocate_static_scratch(const float* depth, const vh_intrinsics* K, const vh_pose* T_wc,
                                                float voxel_size, float truncation_distance,
                                                int32_t allocation_stride, int32_t* keys_out, size_t max_keys,
                                                size_t* count, void* stream) {
  if (!depth || !K || K->width <= 0 || K->height <= 0 || K->fx == 0.0f || K->fy == 0.0f || !T_wc || !count ||
      !(voxel_size > 0.0f) || !(truncation_distance > 0.0f)) {
    return VH_ERR_INVALID_ARGUMENT;
  }
  *count = 0;  // every later return leaves a defined count
  const int stride = allocation_stride > 1 ? allocation_stride : 1;
  const uint64_t samples = static_cast<uint64_t>((K->width + stride - 1) / stride) *
                           static_cast<uint64_t>((K->height + stride - 1) / stride);
  const uint64_t estimated_blocks = 16ULL * samples > 2048ULL ? 16ULL * samples : 2048ULL;
  const uint32_t capacity = next_pow2(2ULL * estimated_blocks);
  if (capacity == 0U || capacity > kStaticBuckets) return VH_ERR_CAPACITY;  // frame larger than the scratch
  void* base = nullptr;
  vh_status st = scratch_for_current_device(&base);
  if (st != VH_OK) return st;
  unsigned char* b = static_cast<unsigned char*>(base);
  vh::Volume V{};
  V.slot_keys = reinterpret_cast<unsigned long long*>(b);
  V.slot_block = reinterpret_cast<uint32_t*>(b + kKeysBytes);
  V.slot_stamp = reinterpret_cast<uint32_t*>(b + kKeysBytes + kSlotU32Bytes);
  V.visible = reinterpret_cast<uint32_t*>(b + kKeysBytes + 2 * kSlotU32Bytes);
  V.counters = reinterpret_cast<vh::Counters*>(b + kCountersOffset);
  V.capacity = capacity;
  V.mask = capacity - 1U;
  V.max_blocks = 0U;  // keys only: no pool

  vh::Params p{};
  p.width = K->width;
  p.height = K->height;
  p.fx = K->fx;
  p.fy = K->fy;
  p.cx = K->cx;
  p.cy = K->cy;
  for (int i = 0; i < 9; ++i) p.T_wc.r[i] = T_wc->R[i];
  for (int i = 0; i < 3; ++i) p.T_wc.t[i] = T_wc->t[i];
  p.voxel_size = voxel_size;
  p.truncation = truncation_distance;
  p.block_world_size = voxel_size * 8.0f;
  p.stride = stride;
  p.sample_width = (K->width + stride - 1) / stride;
  p.sample_height = (K->height + stride - 1) / stride;

  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The previous call's keys, stamps and counters stay in the array: clear the part this call uses (empty
  // keys, zero stamps, zero counters, so the frame stamp starts again at 1 and matches no stale stamp).
  if (cudaMemsetAsync(V.slot_keys, 0xFF, static_cast<size_t>(capacity) * sizeof(unsigned long long), s) !=
          cudaSuccess ||
      cudaMemsetAsync(V.slot_stamp, 0, static_cast<size_t>(capacity) * sizeof(uint32_t), s) != cudaSuccess ||
      cudaMemsetAsync(V.counters, 0, sizeof(vh::Counters), s) != cudaSuccess ||
      vh::launch_begin_frame(V.counters, s) != cudaSuccess || vh::launch_alloc(depth, V, p, s) != cudaSuccess) {
    cudaGetLastError();
    return VH_ERR_CUDA;
  }
  vh::Counters c{};
  if (cudaMemcpyAsync(&c, V.counters, sizeof(c), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return VH_ERR_CUDA;
  }
  if (c.error & vh::kErrKeyRange) return VH_ERR_KEY_RANGE;
  if (c.error & vh::kErrHashFull) return VH_ERR_HASH_FULL;
  *count = c.visible_count;  // also on VH_ERR_BUFFER_TOO_SMALL: the size the caller needs
  if (c.visible_count == 0U) return VH_OK;
  if (!keys_out) return VH_OK;
  if (c.visible_count > max_keys) return VH_ERR_BUFFER_TOO_SMALL;
  if (vh::launch_visible_keys(V, keys_out, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    *count = 0;
    return VH_ERR_CUDA;
  }
  return VH_OK;
}
