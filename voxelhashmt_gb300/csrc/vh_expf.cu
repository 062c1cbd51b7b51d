// vh_expf.cu -- diagnostic entry points of the device exponential (vh_expf in vh_common.cuh).
//
// vh_expf is the C library's expf restated for the GPU: a float-float fast path that rounds the library's
// double-precision polynomial itself, and the library's double-precision sequence (expf_double) where the fast
// path cannot decide the rounding.  vh_expf_check runs both over a range of float bit patterns on the device and
// counts the arguments where they differ; over all 2^32 patterns that is the proof that the fast path never
// changes a result.  vh_expf_eval evaluates the product's exponential on a buffer, for comparison with the
// host restatement (oracle/) and with the C library itself.
#include <cuda_runtime.h>

#include "../../include/voxelhash_gb300.h"
#include "vh_common.cuh"

namespace vh {
namespace {

__global__ void __launch_bounds__(256) expf_eval_kernel(const float* __restrict__ x, float* __restrict__ y,
                                                         uint64_t n) {
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    y[i] = vh_expf(x[i]);
  }
}

// out[0]: arguments whose two results differ (bitwise), out[1]: smallest differing bit pattern (all ones if none)
__global__ void __launch_bounds__(256) expf_check_kernel(uint64_t first, uint64_t count,
                                                          unsigned long long* __restrict__ out) {
  unsigned long long bad = 0ULL;
  unsigned long long first_bad = ~0ULL;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint32_t bits = static_cast<uint32_t>(first + i);
    const float x = __uint_as_float(bits);
    const uint32_t a = __float_as_uint(vh_expf(x));
    const uint32_t b = __float_as_uint(expf_double(x));
    // NaN arguments return a NaN either way; compare everything else bit for bit
    if (a != b && !(x != x)) {
      ++bad;
      first_bad = min(first_bad, static_cast<unsigned long long>(bits));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    bad += __shfl_down_sync(0xffffffffU, bad, o);
    first_bad = min(first_bad, __shfl_down_sync(0xffffffffU, first_bad, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicAdd(&out[0], bad);
    if (first_bad != ~0ULL) atomicMin(&out[1], first_bad);
  }
}

}  // namespace
}  // namespace vh

extern "C" {

vh_status vh_expf_eval(const float* x, float* y, uint64_t n, void* stream) {
  if ((!x || !y) && n) return VH_ERR_INVALID_ARGUMENT;
  if (n == 0) return VH_OK;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  vh::expf_eval_kernel<<<152 * 8, 256, 0, s>>>(x, y, n);
  return cudaGetLastError() == cudaSuccess ? VH_OK : VH_ERR_CUDA;
}

vh_status vh_expf_check(uint32_t first_bits, uint64_t count, uint64_t* mismatches, uint32_t* first_mismatch,
                        void* stream) {
  if (!mismatches || !first_mismatch || count > (1ULL << 32) - first_bits) return VH_ERR_INVALID_ARGUMENT;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return VH_ERR_OUT_OF_MEMORY;
  const unsigned long long init[2] = {0ULL, ~0ULL};
  unsigned long long h[2] = {0ULL, ~0ULL};
  cudaError_t e = cudaMemcpyAsync(d, init, sizeof(init), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && count) {
    vh::expf_check_kernel<<<152 * 16, 256, 0, s>>>(first_bits, count, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d);
  if (e != cudaSuccess) return VH_ERR_CUDA;
  *mismatches = h[0];
  *first_mismatch = h[1] == ~0ULL ? 0xffffffffU : static_cast<uint32_t>(h[1]);
  return VH_OK;
}

}  // extern "C"
