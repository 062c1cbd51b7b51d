// vh_nn.h -- launchers of the learned depth denoiser's kernels (internal to the library).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace vh {
namespace nn {

enum { kForward = 0, kGrad = 1 };

// 32 -> 32 channel 3x3 convolution (NHWC BF16, zero padding) on the tensor cores; wpack from launch_pack_w32.
// kForward: out = relu?(conv(in) + bias); kGrad: out = conv(in) * (mask > 0).  error: kErrTimeout (8) is or-ed
// in if a wait on the loads or the tensor cores gave up (about a second).  gate (device memory, may be null):
// the loads start once *gate is nonzero; a gate left at zero makes the waits give up (the timeout path's test).
cudaError_t launch_conv32(const __nv_bfloat16* in, const __nv_bfloat16* wpack, const float* bias,
                          const __nv_bfloat16* mask, __nv_bfloat16* out, int batch, int width, int height, int mode,
                          int relu, unsigned int* error, cudaStream_t s, const unsigned int* gate = nullptr);
// Weight gradient of a 32 -> 32 3x3 layer on the tensor cores: dw[co][ci][3][3] += sum_p g[p][co] x[p + off][ci],
// db[co] += sum_p g[p][co] (x: the layer input, g: the gradient at its output, NHWC BF16, 4-byte aligned).
// error: as launch_conv32.
cudaError_t launch_wgrad32(const __nv_bfloat16* x, const __nv_bfloat16* g, float* dw, float* db, int batch, int width,
                           int height, unsigned int* error, cudaStream_t s);
// FP32 weights [co][ci][3][3] -> the B operand layout; transpose_flip gives the input-gradient weights
cudaError_t launch_pack_w32(const float* w, __nv_bfloat16* out, int transpose_flip, cudaStream_t s);
int conv32_smem_bytes();

// The whole net.  params: FP32 [param_count()]; packed: 4 x 9,216 BF16 (w2, w3 forward, w2, w3 input-gradient);
// depth / out / target: batch x height x width FP32; ws: workspace_bytes(batch, width, height) of device memory
// holding the activations the backward pass reads (forward before backward on the same ws).
int param_count();
size_t workspace_bytes(int batch, int width, int height);
cudaError_t pack_weights(const float* params, __nv_bfloat16* packed, cudaStream_t s);
// fallback (may be null): per-pixel replacement where the correction exceeds the discontinuity threshold
cudaError_t forward(const float* params, const __nv_bfloat16* packed, const float* depth, const float* fallback,
                    float* out, int batch, int width, int height, unsigned char* ws, unsigned int* error,
                    cudaStream_t s);
// grads: FP32 [param_count()] (overwritten); loss: [sum of squared errors over masked pixels, their count]
cudaError_t backward(const float* params, const __nv_bfloat16* packed, const float* depth, const float* target,
                     const float* out, int batch, int width, int height, unsigned char* ws, float* grads, float* loss,
                     unsigned int* error, cudaStream_t s);
cudaError_t adam(float* params, const float* grads, float* m, float* v, float lr, float b1, float b2, float eps,
                 int step, cudaStream_t s);

}  // namespace nn
}  // namespace vh
