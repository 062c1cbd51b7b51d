// vh_nn.h -- launchers of the learned depth denoiser's kernels (internal to the library).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace vh {
namespace nn {

enum { kForward = 0, kGrad = 1 };

// 32 -> 32 channel 3x3 convolution (NHWC BF16, zero padding) on the tensor cores; wpack from launch_pack_w32.
// kForward: out = relu?(conv(in) + bias); kGrad: out = conv(in) * (mask > 0).  error: set to 1 if the tensor
// core never signalled completion (bounded wait).
cudaError_t launch_conv32(const __nv_bfloat16* in, const __nv_bfloat16* wpack, const float* bias,
                          const __nv_bfloat16* mask, __nv_bfloat16* out, int batch, int width, int height, int mode,
                          int relu, unsigned int* error, cudaStream_t s);
// FP32 weights [co][ci][3][3] -> the B operand layout; transpose_flip gives the input-gradient weights
cudaError_t launch_pack_w32(const float* w, __nv_bfloat16* out, int transpose_flip, cudaStream_t s);
int conv32_smem_bytes();

}  // namespace nn
}  // namespace vh
