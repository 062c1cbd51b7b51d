// vh_nn.cu -- kernels of the learned depth denoiser: a 4-layer 3x3 convolutional net (input 4 channels -> 32
// -> 32 -> 32 -> 1, ReLU between layers, residual output), BF16 weights and activations, FP32 accumulation.
//
// The two 32 -> 32 layers carry ~95 % of the arithmetic and run on the 5th-generation tensor cores
// (tcgen05.mma, kind::f16 with BF16 operands, FP32 accumulator in tensor memory) as an implicit GEMM: one CTA
// computes 128 consecutive output pixels of one image row x 32 output channels, M = 128, N = 32,
// K = 9 taps x 32 input channels, issued as 18 MMAs of m128n32k16 into one TMEM accumulator (32 columns).
// The three input rows the tile needs (130 pixels each, 1-pixel halo) are staged in shared memory in the
// canonical no-swizzle K-major layout: [row][channel group of 8][pixel][8 channels], 16 bytes per pixel per
// group, so the A operand of tap (dy, dx) is the same layout starting dx pixels further -- a descriptor
// start address 16 bytes * dx higher; no im2col copy.  Weights are staged once per CTA as
// [tap][k-step][channel group][output channel][8 channels].  The epilogue reads the accumulator with
// tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = pixels 32w..32w+31), adds the bias and applies ReLU, or,
// for the input gradient, multiplies by the ReLU mask of the layer's input, and stores BF16.
//
// The input gradient of a 32 -> 32 layer is the same convolution with the weights flipped in space and
// transposed in channels, so the backward pass reuses the kernel.  The 4-channel input layer, the 1-channel
// output layer, the weight gradients (reductions over pixels) and Adam run on the CUDA cores in FP32.
//
// Safety: the shared-memory regions the tensor core reads are padded so that any byte the descriptors can
// address stays inside this CTA's allocation; the mbarrier wait gives up after a bounded number of polls,
// sets the error word and still waits (bounded) before freeing tensor memory.
#include <cuda_bf16.h>

#include <cstdint>

#include "vh_nn.h"

namespace vh {
namespace nn {
namespace {

constexpr int kTile = 128;                 // output pixels per CTA tile (MMA M)
constexpr int kC = 32;                     // channels of the hidden layers (MMA N, and K per tap)
constexpr int kRowPix = kTile + 2;         // staged pixels per input row
constexpr int kGroups = kC / 8;            // channel groups of 8 (16 bytes of BF16)
constexpr int kPlane = kRowPix * 16;       // bytes of one channel group of one staged row (the A operand's LBO)
constexpr int kRowBytes = kGroups * kPlane;
constexpr int kABytes = 3 * kRowBytes;     // 24,960
constexpr int kAPad = 65536;               // A region incl. padding (worst-case descriptor reach < 64 KB)
constexpr int kBBlock = 2 * kC * 16;       // one (tap, k-step) B operand: 2 groups x 32 rows x 16 B = 1,024
constexpr int kBBytes = 18 * kBBlock;      // 18,432
constexpr int kBPad = kBBytes + 8192;
constexpr int kThreads = 128;              // 4 warps: one per 32 TMEM lanes
constexpr int kSmem = kAPad + kBPad + 64;  // + mbarrier and TMEM address
constexpr uint32_t kMaxPolls = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor, no swizzle (canonical K-major core-matrix layout):
// start address, leading-dimension byte offset (between core matrices along K), stride-dimension byte offset
// (between core matrices along M/N), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1u) << 46;
  return d;
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, N = 32, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(kC >> 3) << 17) |
                            (static_cast<uint32_t>(kTile >> 4) << 24);

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  for (uint32_t i = 0; i < kMaxPolls; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase));
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// One 32 -> 32 3x3 convolution over a batch of images (NHWC BF16, zero padding), tcgen05 implicit GEMM.
// mode kForward: out = relu?(conv(in) + bias); mode kGrad: out = conv(in) * (mask > 0) (mask = the layer
// input's activations; the input gradient of the previous layer's ReLU).
__global__ void __launch_bounds__(kThreads) conv32_tc_kernel(const __nv_bfloat16* __restrict__ in,
                                                             const __nv_bfloat16* __restrict__ wpack,
                                                             const float* __restrict__ bias,
                                                             const __nv_bfloat16* __restrict__ mask,
                                                             __nv_bfloat16* __restrict__ out, int batch, int width,
                                                             int height, int mode, int relu,
                                                             unsigned int* __restrict__ error) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sA = smem;
  unsigned char* sB = smem + kAPad;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kAPad + kBPad);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kAPad + kBPad + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // weights: [tap][ks][g][co][8] BF16, 18,432 bytes, already packed in this order in global memory
  for (int i = tid; i < kBBytes / 16; i += kThreads) {
    reinterpret_cast<uint4*>(sB)[i] = reinterpret_cast<const uint4*>(wpack)[i];
  }
  for (int i = tid; i < (kAPad - kABytes) / 16; i += kThreads) reinterpret_cast<uint4*>(sA + kABytes)[i] = make_uint4(0, 0, 0, 0);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;\n" ::"r"(smem_u32(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  const uint32_t tmem = *tmem_slot;
  const uint32_t a_base = smem_u32(sA), b_base = smem_u32(sB), bar_addr = smem_u32(bar);

  const int tiles_x = (width + kTile - 1) / kTile;
  const long long ntiles = static_cast<long long>(batch) * height * tiles_x;
  uint32_t phase = 0;
  bool ok = true;
  for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const int tx = static_cast<int>(t % tiles_x);
    const long long rest = t / tiles_x;
    const int y = static_cast<int>(rest % height);
    const int img = static_cast<int>(rest / height);
    const int x0 = tx * kTile;
    // stage rows y-1, y, y+1, pixels x0-1 .. x0+128, as [row][g][pixel][8 channels]
    for (int i = tid; i < 3 * kRowPix * kGroups; i += kThreads) {
      const int g = i % kGroups;
      const int px = (i / kGroups) % kRowPix;
      const int r = i / (kGroups * kRowPix);
      const int sx = x0 - 1 + px, sy = y - 1 + r;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (sx >= 0 && sx < width && sy >= 0 && sy < height) {
        v = reinterpret_cast<const uint4*>(in + ((static_cast<size_t>(img) * height + sy) * width + sx) * kC)[g];
      }
      *reinterpret_cast<uint4*>(sA + r * kRowBytes + g * kPlane + px * 16) = v;
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n");
      int k = 0;
      for (int dy = 0; dy < 3; ++dy) {
        for (int dx = 0; dx < 3; ++dx) {
          for (int ks = 0; ks < 2; ++ks, ++k) {
            const uint64_t a = smem_desc(a_base + dy * kRowBytes + (2 * ks) * kPlane + dx * 16, kPlane, 128);
            const uint64_t b = smem_desc(b_base + k * kBBlock, kC * 16, 128);
            mma(tmem, a, b, k > 0 ? 1u : 0u);
          }
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar_addr)
                   : "memory");
    }
    // every thread polls the barrier; the CTA continues only if all saw the phase complete (uniform branch)
    ok = __syncthreads_and(mbar_wait(bar_addr, phase) ? 1 : 0) != 0;
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    if (!ok) break;
    // epilogue: warp w, lane l = output pixel 32w + l of the tile
    float acc[32];
    tmem_ld32(tmem + (static_cast<uint32_t>(warp * 32) << 16), acc);
    const int x = x0 + warp * 32 + lane;
    if (x < width) {
      const size_t o = ((static_cast<size_t>(img) * height + y) * width + x) * kC;
      __align__(16) __nv_bfloat16 res[32];
      if (mode == kForward) {
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          float v = acc[c] + (bias ? bias[c] : 0.0f);
          if (relu) v = fmaxf(v, 0.0f);
          res[c] = __float2bfloat16_rn(v);
        }
      } else {
        __align__(16) __nv_bfloat16 m[32];
#pragma unroll
        for (int q = 0; q < 4; ++q) reinterpret_cast<uint4*>(m)[q] = reinterpret_cast<const uint4*>(mask + o)[q];
#pragma unroll
        for (int c = 0; c < 32; ++c) res[c] = __float2bfloat16_rn(__bfloat162float(m[c]) > 0.0f ? acc[c] : 0.0f);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) reinterpret_cast<uint4*>(out + o)[q] = reinterpret_cast<const uint4*>(res)[q];
    }
    // the accumulator and the staged tile are reused by the next tile
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
  }
  if (!ok) {
    if (tid == 0) atomicOr(error, 1u);
    mbar_wait(bar_addr, phase ^ 1u);  // the MMAs in flight, bounded
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;\n" ::"r"(tmem));
}

}  // namespace

int conv32_smem_bytes() { return kSmem; }

cudaError_t launch_conv32(const __nv_bfloat16* in, const __nv_bfloat16* wpack, const float* bias,
                          const __nv_bfloat16* mask, __nv_bfloat16* out, int batch, int width, int height, int mode,
                          int relu, unsigned int* error, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(conv32_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long ntiles = static_cast<long long>(batch) * height * ((width + kTile - 1) / kTile);
  const int grid = static_cast<int>(ntiles < 2LL * sms ? ntiles : 2LL * sms);
  if (grid <= 0) return cudaSuccess;
  conv32_tc_kernel<<<grid, kThreads, kSmem, s>>>(in, wpack, bias, mask, out, batch, width, height, mode, relu, error);
  return cudaGetLastError();
}

// Packs 32 x 32 x 3 x 3 FP32 weights w[co][ci][ky][kx] (transpose_flip: the input-gradient form, w'[ci][co][2-ky][2-kx])
// into the B operand layout [tap = ky * 3 + kx][ks][g][co][8] in BF16.
__global__ void pack_w32_kernel(const float* __restrict__ w, __nv_bfloat16* __restrict__ out, int transpose_flip) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // one output element
  if (i >= 9 * kC * kC) return;
  const int c8 = i % 8;
  const int co = (i / 8) % kC;
  const int g = (i / (8 * kC)) % 2;
  const int ks = (i / (16 * kC)) % 2;
  const int tap = i / (32 * kC);
  const int ci = ks * 16 + g * 8 + c8;
  const int ky = tap / 3, kx = tap % 3;
  float v;
  if (!transpose_flip) {
    v = w[((co * kC + ci) * 3 + ky) * 3 + kx];
  } else {
    v = w[((ci * kC + co) * 3 + (2 - ky)) * 3 + (2 - kx)];
  }
  out[i] = __float2bfloat16_rn(v);
}

cudaError_t launch_pack_w32(const float* w, __nv_bfloat16* out, int transpose_flip, cudaStream_t s) {
  pack_w32_kernel<<<(9 * kC * kC + 255) / 256, 256, 0, s>>>(w, out, transpose_flip);
  return cudaGetLastError();
}

}  // namespace nn
}  // namespace vh
