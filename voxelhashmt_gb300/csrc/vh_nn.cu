// vh_nn.cu -- kernels of the learned depth denoiser: a 4-layer 3x3 convolutional net (input 4 channels -> 32
// -> 32 -> 32 -> 1, ReLU between layers, residual output), BF16 weights and activations, FP32 accumulation.
//
// The two 32 -> 32 layers carry ~95 % of the arithmetic and run on the 5th-generation tensor cores
// (tcgen05.mma, kind::f16 with BF16 operands, FP32 accumulator in tensor memory) as an implicit GEMM: each
// output row of a 128-pixel strip is M = 128 pixels x N = 32 output channels, K = 9 taps x 32 input channels,
// issued as 18 MMAs of m128n32k16 into a TMEM accumulator (32 columns; two accumulators).
// Input rows (130 pixels each, 1-pixel halo) are loaded by TMA (4 tensor-map boxes of {8 channels, 130
// pixels} per row, zero fill outside the image) into a ring of row slots in the canonical no-swizzle K-major
// layout: [channel group of 8][pixel][8 channels], 16 bytes per pixel per group (each group's plane padded to
// 2,176 bytes for the TMA's 128-byte destination alignment).  The A operand of tap (dy, dx) is the slot of
// input row y - 1 + dy starting dx pixels further -- a descriptor start address 16 bytes * dx higher; no
// im2col copy.  A CTA streams blocks of output rows of one strip, loading each input row once.  Weights are
// staged once per CTA as [tap][k-step][channel group][output channel][8 channels].  The epilogue reads the
// accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = pixels 32w..32w+31), adds the bias and
// applies ReLU, or, for the input gradient, multiplies by the ReLU mask of the layer's input, and stores BF16.
//
// The input gradient of a 32 -> 32 layer is the same convolution with the weights flipped in space and
// transposed in channels, so the backward pass reuses the kernel.  The weight gradient of a 32 -> 32 layer (a
// reduction over pixels) is a second tensor-core kernel, wgrad32_tc_kernel.  The 4-channel input layer, the
// 1-channel output layer, their weight gradients and Adam run on the CUDA cores in FP32.
//
// Safety: the descriptors address only staged bytes: an A operand reads at most 8,608 bytes into its 8,704-byte
// slot (pixels dx .. dx + 127 of each plane), the B operand exactly kBBytes, followed by a margin; the layout is
// checked bit-for-bit against a float64 convolution.  Every mbarrier wait gives up after about a second, sets
// the error word and the kernel still waits (bounded) for its loads and MMAs before freeing tensor memory.
#include <cuda.h>  // CUtensorMap and the tensor-map encoder's types (resolved at run time, no link dependency)
#include <cuda_bf16.h>

#include <cstdint>
#include <cstdlib>

#include "vh_nn.h"

namespace vh {
namespace nn {
namespace {

constexpr int kTile = 128;                 // output pixels per CTA tile (MMA M)
constexpr int kC = 32;                     // channels of the hidden layers (MMA N, and K per tap)
constexpr int kRowPix = kTile + 2;         // staged pixels per input row
constexpr int kGroups = kC / 8;            // channel groups of 8 (16 bytes of BF16)
constexpr int kPlaneData = kRowPix * 16;   // bytes of one channel group of one staged row: one TMA box
constexpr int kPlane = 2176;               // the plane padded to a multiple of 128 (TMA destination alignment);
                                           // the A operand's LBO
constexpr int kRowBytes = kGroups * kPlane;  // one ring slot: 8,704 bytes (8,320 written by a row's 4 boxes)
constexpr int kBBlock = 2 * kC * 16;       // one (tap, k-step) B operand: 2 groups x 32 rows x 16 B = 1,024
constexpr int kBBytes = 18 * kBBlock;      // 18,432
constexpr int kBPad = kBBytes + 1024;
// warps 0-3: epilogue (warp w owns TMEM lanes 32w..32w+31); warp 4: TMA producer; warp 5: TMEM owner, MMA issuer
constexpr int kEpilogueWarps = 4;
constexpr int kThreads = 32 * (kEpilogueWarps + 2);
constexpr int kAccs = 2;  // accumulators in tensor memory (32 columns each)
static_assert(kPlaneData <= kPlane && kPlane % 128 == 0, "TMA destinations 128-byte aligned");
// A wait gives up once kWaitNs of global time have passed since its first poll (kMaxPolls bounds the polls as
// well, should the timer not advance).  Legitimate waits in this kernel last microseconds.
constexpr uint64_t kWaitNs = 1000000000ull;
constexpr uint32_t kMaxPolls = 1u << 28;
constexpr unsigned int kErrorBit = 8u;  // the volume error word's timeout bit

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

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  uint64_t start = 0;
  for (uint32_t i = 0; i < kMaxPolls; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase));
    if (done) return true;
    if ((i & 255u) == 0u) {
      const uint64_t now = global_ns();
      if (i == 0u) {
        start = now;
      } else if (now - start > kWaitNs) {
        return false;
      }
    }
  }
  return false;
}

// The load gate of vh_nn_conv32_gated: true once *gate is nonzero, false if it stays zero for kWaitNs.
__device__ __forceinline__ bool gate_wait(const unsigned int* gate) {
  const uint64_t start = global_ns();
  for (uint32_t i = 0; i < kMaxPolls; ++i) {
    if (*reinterpret_cast<const volatile unsigned int*>(gate) != 0u) return true;
    if (global_ns() - start > kWaitNs) return false;
    __nanosleep(1000);
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

__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}

// A CTA owns blocks of kRows output rows of one 128-pixel strip and streams the block's kRows + 2 input rows
// once each through a ring of kSlots row slots, so an output row costs one new input row (4 TMA boxes) instead
// of three; the three taps' rows are three resident slots.

constexpr uint32_t kRowTxBytes = kGroups * kPlaneData;
static_assert(kRowBytes % 128 == 0, "ring slots keep the TMA destinations 128-byte aligned");

// loads input row y of image img (pixels x0-1 .. x0+128, 4 channel-group boxes, zero fill outside the image)
__device__ __forceinline__ void load_row(const CUtensorMap* map, uint32_t slot_base, uint32_t bar, int img, int y,
                                         int x0) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(kRowTxBytes) : "memory");
  const uint64_t m = reinterpret_cast<uint64_t>(map);
#pragma unroll
  for (int g = 0; g < kGroups; ++g) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(slot_base + g * kPlane),
        "l"(m), "r"(8 * g), "r"(x0 - 1), "r"(y), "r"(img), "r"(bar)
        : "memory");
  }
}

// the 18 MMAs of one output row: tap row dy reads the slot r0 / r1 / r2 (input rows y - 1, y, y + 1)
__device__ __forceinline__ void issue_row(uint32_t r0, uint32_t r1, uint32_t r2, uint32_t b_base, uint32_t tmem) {
  int k = 0;
  for (int dy = 0; dy < 3; ++dy) {
    const uint32_t rb = dy == 0 ? r0 : (dy == 1 ? r1 : r2);
    for (int dx = 0; dx < 3; ++dx) {
      for (int ks = 0; ks < 2; ++ks, ++k) {
        const uint64_t a = smem_desc(rb + (2 * ks) * kPlane + dx * 16, kPlane, 128);
        const uint64_t b = smem_desc(b_base + k * kBBlock, kC * 16, 128);
        mma(tmem, a, b, k > 0 ? 1u : 0u);
      }
    }
  }
}

// the epilogue's per-warp transpose buffer: 32 pixels x 64 bytes
constexpr int kEpiStage = 32 * kC * 2;

template <int kSlots>
constexpr int ring_smem_bytes() {
  return 128 + kSlots * kRowBytes + kBPad + kEpilogueWarps * kEpiStage + 8 * (2 * kSlots + 2 * kAccs) + 16;
}

// The epilogue moves a warp's 32 pixels x 64 bytes between registers (lane l: pixel l) and global memory
// through its shared-memory buffer, so that every global access instruction covers 512 contiguous bytes
// (lane l: 16-byte chunk u * 32 + l of the warp's 2 KB), not 32 half sectors.  Chunk q of pixel p sits at
// position 4p + (q ^ ((p >> 1) & 3)): the XOR spreads the lanes of each access phase over distinct banks.
__device__ __forceinline__ int epi_pos(int p, int q) { return 4 * p + (q ^ ((p >> 1) & 3)); }

// One 32 -> 32 3x3 convolution over a batch of images (NHWC BF16, zero padding), tcgen05 implicit GEMM.
// mode kForward: out = relu?(conv(in) + bias); mode kGrad: out = conv(in) * (mask > 0) (mask = the layer
// input's activations; the input gradient of the previous layer's ReLU).
//
// Warp-specialised, handing off through mbarriers only:
//   producer (warp 4, one lane): waits empty[s] (the MMAs that read the slot's previous row completed), then
//     TMA-loads input row q into slot s = q mod kSlots, completing full[s] by transaction bytes;
//   MMA issuer (warp 5, one lane): for each output row waits full[s] of the rows it adds and acc_empty[a] (the
//     epilogue has read accumulator a = row mod kAccs), issues the 18 MMAs and commits them to the top row's
//     empty[s] (that row is not read again) and to acc_full[a]; a block's last two rows are released after
//     its last output row;
//   epilogue (warps 0-3): waits acc_full[a], reads its 32 TMEM lanes, releases the accumulator (acc_empty[a],
//     one arrival per warp) and applies bias / ReLU or the gradient mask and stores BF16.
// Phase j of a barrier completes at its j-th use, so the waits use parity (q / kSlots) & 1 or (row / kAccs) & 1
// and the releases of an earlier use the parity before.  A ring of at least 3 slots cannot deadlock: the row
// an output row still needs to load was released by an earlier output row.  Every wait gives up after about
// a second: that role stops, the error word gets the timeout bit, and the roles waiting on it
// give up in turn; before tensor memory is freed, the loads and MMA groups still in flight are waited for
// (bounded).
template <int kSlots, int kRows>
__global__ void __launch_bounds__(kThreads, 1) conv32_tc_kernel(const __grid_constant__ CUtensorMap in_map,
                                                                  const __nv_bfloat16* __restrict__ wpack,
                                                                  const float* __restrict__ bias,
                                                                  const __nv_bfloat16* __restrict__ mask,
                                                                  __nv_bfloat16* __restrict__ out, int batch,
                                                                  int width, int height, int mode, int relu,
                                                                  const unsigned int* __restrict__ gate,
                                                                  unsigned int* __restrict__ error) {
  static_assert(kSlots >= 3, "an output row needs three resident input rows");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);  // TMA destinations: 128 B
  unsigned char* sB = smem + kSlots * kRowBytes;
  uint4* sEpi = reinterpret_cast<uint4*>(sB + kBPad);  // kEpilogueWarps x kEpiStage
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + kBPad + kEpilogueWarps * kEpiStage);  // full[S], empty[S],
                                                                                         // acc_full[A], acc_empty[A]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kSlots + 2 * kAccs);
  uint32_t* consumed = tmem_slot + 1;  // rows whose loads the MMA issuer has waited for (teardown)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  for (int i = tid; i < kBBytes / 16; i += kThreads) {
    reinterpret_cast<uint4*>(sB)[i] = reinterpret_cast<const uint4*>(wpack)[i];
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the weights, for the MMAs' async reads
  if (warp == kEpilogueWarps + 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(32 * kAccs));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    for (int i = 0; i < 2 * kSlots + kAccs; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bars[i])));
    }
    for (int i = 0; i < kAccs; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&bars[2 * kSlots + kAccs + i])),
                   "r"(kEpilogueWarps));
    }
    *consumed = 0u;
    asm volatile("fence.mbarrier_init.release.cluster;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  const uint32_t tmem = *tmem_slot;
  const uint32_t ring0 = smem_u32(smem), b_base = smem_u32(sB);
  const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[kSlots]);
  const uint32_t accf0 = smem_u32(&bars[2 * kSlots]), acce0 = smem_u32(&bars[2 * kSlots + kAccs]);
  auto slot_addr = [&](uint32_t q) { return ring0 + (q % kSlots) * static_cast<uint32_t>(kRowBytes); };

  // work item t = blockIdx.x + k gridDim.x: strip xt, row block rb, image img (32-bit: checked by the launcher)
  const uint32_t tiles_x = static_cast<uint32_t>((width + kTile - 1) / kTile);
  const uint32_t blocks_y = static_cast<uint32_t>((height + kRows - 1) / kRows);
  const uint32_t nitems = static_cast<uint32_t>(batch) * blocks_y * tiles_x;
  const uint32_t stride = gridDim.x;
  const int my_items = blockIdx.x < nitems ? static_cast<int>((nitems - 1u - blockIdx.x) / stride + 1u) : 0;
  auto item = [&](int k, int& img, int& y0, int& x0, int& rows) {
    const uint32_t t = blockIdx.x + static_cast<uint32_t>(k) * stride;
    const uint32_t rest = t / tiles_x;
    x0 = static_cast<int>(t - rest * tiles_x) * kTile;
    const uint32_t im = rest / blocks_y;
    y0 = static_cast<int>(rest - im * blocks_y) * kRows;
    img = static_cast<int>(im);
    rows = min(kRows, height - y0);
  };
  bool ok = true;
  uint32_t loaded = 0;  // producer: rows loaded
  uint32_t issued = 0;  // MMA issuer: output rows issued

  if (warp == kEpilogueWarps) {
    if (lane == 0) {  // producer
      if (gate != nullptr && my_items > 0 && !gate_wait(gate)) ok = false;  // nothing loaded, nothing in flight
      for (int k = 0; k < my_items && ok; ++k) {
        int img, y0, x0, rows;
        item(k, img, y0, x0, rows);
        for (int i = 0; i < rows + 2; ++i) {
          const uint32_t q = loaded;
          if (q >= kSlots && !mbar_wait(empty0 + 8 * (q % kSlots), (q / kSlots - 1) & 1u)) {
            ok = false;
            break;
          }
          load_row(&in_map, slot_addr(q), full0 + 8 * (q % kSlots), img, y0 - 1 + i, x0);
          loaded = q + 1;
        }
      }
    }
  } else if (warp == kEpilogueWarps + 1) {
    if (lane == 0) {  // MMA issuer
      uint32_t q = 0;  // first row of the current block
      for (int k = 0; k < my_items && ok; ++k) {
        int img, y0, x0, rows;
        item(k, img, y0, x0, rows);
        for (int r = 0; r < rows && ok; ++r) {
          for (uint32_t w = (r == 0 ? q : q + r + 2); w <= q + r + 2; ++w) {
            if (!mbar_wait(full0 + 8 * (w % kSlots), (w / kSlots) & 1u)) {
              ok = false;
              break;
            }
            *reinterpret_cast<volatile uint32_t*>(consumed) = w + 1;
          }
          if (!ok) break;
          const uint32_t a = issued % kAccs;
          if (issued >= kAccs && !mbar_wait(acce0 + 8 * a, (issued / kAccs - 1) & 1u)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;\n");
          issue_row(slot_addr(q + r), slot_addr(q + r + 1), slot_addr(q + r + 2), b_base, tmem + 32u * a);
          commit(empty0 + 8 * ((q + r) % kSlots));
          commit(accf0 + 8 * a);
          issued += 1;
        }
        if (!ok) break;
        commit(empty0 + 8 * ((q + rows) % kSlots));
        commit(empty0 + 8 * ((q + rows + 1) % kSlots));
        q += rows + 2;
      }
    }
  } else {  // epilogue: warp w, lane l = output pixel 32w + l of the row
    float bv[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) bv[c] = (mode == kForward && bias) ? __ldg(&bias[c]) : 0.0f;
    uint32_t j = 0;
    for (int k = 0; k < my_items && ok; ++k) {
      int img, y0, x0, rows;
      item(k, img, y0, x0, rows);
      for (int r = 0; r < rows; ++r, ++j) {
        const uint32_t a = j % kAccs;
        const bool got = mbar_wait(accf0 + 8 * a, (j / kAccs) & 1u);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        float acc[32];
        tmem_ld32(tmem + 32u * a + (static_cast<uint32_t>(warp * 32) << 16), acc);
        asm volatile("tcgen05.fence::before_thread_sync;\n");
        __syncwarp();
        if (lane == 0) arrive(acce0 + 8 * a);
        // the warp's 32 pixels start at pixel xw of row y0 + r; chunk u * 32 + lane belongs to pixel
        // xw + 8u + lane / 4, which must lie inside the image
        uint4* buf = sEpi + warp * (kEpiStage / 16);
        const int xw = x0 + warp * 32;
        const size_t row0 = ((static_cast<size_t>(img) * height + (y0 + r)) * width + xw) * kC;
        __align__(16) __nv_bfloat162 res[16];
        if (mode == kForward) {
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            float v0 = acc[2 * c] + bv[2 * c], v1 = acc[2 * c + 1] + bv[2 * c + 1];
            if (relu) {
              v0 = fmaxf(v0, 0.0f);
              v1 = fmaxf(v1, 0.0f);
            }
            res[c] = __floats2bfloat162_rn(v0, v1);
          }
        } else {
          // the gradient mask, read coalesced and transposed to lane = pixel through the buffer
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int p = 8 * u + (lane >> 2), q = lane & 3;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (xw + p < width) v = *reinterpret_cast<const uint4*>(mask + row0 + static_cast<size_t>(p) * kC + 8 * q);
            buf[epi_pos(p, q)] = v;
          }
          __syncwarp();
          __align__(16) __nv_bfloat162 m[16];
#pragma unroll
          for (int q = 0; q < 4; ++q) reinterpret_cast<uint4*>(m)[q] = buf[epi_pos(lane, q)];
          __syncwarp();
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const float2 mf = __bfloat1622float2(m[c]);
            res[c] = __floats2bfloat162_rn(mf.x > 0.0f ? acc[2 * c] : 0.0f, mf.y > 0.0f ? acc[2 * c + 1] : 0.0f);
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) buf[epi_pos(lane, q)] = reinterpret_cast<const uint4*>(res)[q];
        __syncwarp();
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int p = 8 * u + (lane >> 2), q = lane & 3;
          if (xw + p < width) {
            *reinterpret_cast<uint4*>(out + row0 + static_cast<size_t>(p) * kC + 8 * q) = buf[epi_pos(p, q)];
          }
        }
        __syncwarp();  // the buffer is rewritten for the next row
      }
    }
  }
  if (!ok && lane == 0) atomicOr(error, kErrorBit);
  __syncthreads();
  // in-flight work after a timeout (the waits return at once when nothing is pending)
  if (warp == kEpilogueWarps && lane == 0) {
    for (uint32_t w = *consumed; w < loaded; ++w) mbar_wait(full0 + 8 * (w % kSlots), (w / kSlots) & 1u);
  }
  if (warp == kEpilogueWarps + 1 && lane == 0 && issued > 0) {
    mbar_wait(accf0 + 8 * ((issued - 1) % kAccs), ((issued - 1) / kAccs) & 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  if (warp == kEpilogueWarps + 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(32 * kAccs));
  }
}

// cuTensorMapEncodeTiled, resolved through the runtime's driver entry point (no link dependency on libcuda)
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

cudaError_t encode_input_map(const __nv_bfloat16* in, int batch, int width, int height, CUtensorMap* map) {
  static EncodeTiledFn encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult qr = cudaDriverEntryPointSymbolNotFound;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr);
    if (e != cudaSuccess) return e;
    if (qr != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    encode = reinterpret_cast<EncodeTiledFn>(fn);
  }
  if (reinterpret_cast<uintptr_t>(in) % 16 != 0) return cudaErrorInvalidValue;
  // NHWC BF16: dims innermost first {channel, x, y, image}; byte strides of x, y, image
  const cuuint64_t dims[4] = {static_cast<cuuint64_t>(kC), static_cast<cuuint64_t>(width),
                              static_cast<cuuint64_t>(height), static_cast<cuuint64_t>(batch)};
  const cuuint64_t strides[3] = {static_cast<cuuint64_t>(kC) * 2, static_cast<cuuint64_t>(width) * kC * 2,
                                 static_cast<cuuint64_t>(height) * width * kC * 2};
  const cuuint32_t box[4] = {8, static_cast<cuuint32_t>(kRowPix), 1, 1};
  const cuuint32_t elem[4] = {1, 1, 1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(in), dims, strides,
                            box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Launch shapes of conv32_tc_kernel: ring slots, resident CTAs per SM, output rows per block.  Measured on
// 640x480 layers (CUDA events, batch 1 / batch 16): 6 slots x 2 CTAs x 8 rows 18.7 / 169 us; 8 x 2 x 8
// 18.7 / 178; 8 x 2 x 16 24.1 / 171; 6 x 3 x 8 18.7 / 219; 4 x 4 x 8 24.8 / 206; the earlier one-row-tile
// kernel (3 input rows loaded per output row) 22.8 / 277 us.
struct Conv32Variant {
  const void* fn;
  int slots, smem, ctas_per_sm, rows;
};
const Conv32Variant kConv32Variants[] = {
    {reinterpret_cast<const void*>(conv32_tc_kernel<6, 8>), 6, ring_smem_bytes<6>(), 2, 8},
    {reinterpret_cast<const void*>(conv32_tc_kernel<8, 8>), 8, ring_smem_bytes<8>(), 2, 8},
    {reinterpret_cast<const void*>(conv32_tc_kernel<8, 16>), 8, ring_smem_bytes<8>(), 2, 16},
};
constexpr int kConv32Default = 0;  // VH_CONV32_VARIANT selects another for launch-shape sweeps

const Conv32Variant& conv32_variant() {
  static int v = -1;
  if (v < 0) {
    v = kConv32Default;
    if (const char* env = std::getenv("VH_CONV32_VARIANT")) {
      const int x = std::atoi(env);
      if (x >= 0 && x < static_cast<int>(sizeof(kConv32Variants) / sizeof(kConv32Variants[0]))) v = x;
    }
  }
  return kConv32Variants[v];
}

}  // namespace

int conv32_smem_bytes() { return conv32_variant().smem; }

cudaError_t launch_conv32(const __nv_bfloat16* in, const __nv_bfloat16* wpack, const float* bias,
                          const __nv_bfloat16* mask, __nv_bfloat16* out, int batch, int width, int height, int mode,
                          int relu, unsigned int* error, cudaStream_t s, const unsigned int* gate) {
  const Conv32Variant& cv = conv32_variant();
  // persistent CTAs, cv.ctas_per_sm per SM: each CTA stages the weights and allocates tensor memory once
  static int ctas = 0;
  if (ctas == 0) {
    cudaError_t e = cudaFuncSetAttribute(cv.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, cv.smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    ctas = cv.ctas_per_sm * (sms > 0 ? sms : 152);
  }
  const long long ntiles = static_cast<long long>(batch) * height * ((width + kTile - 1) / kTile);
  if (ntiles > 0x7fffffffLL) return cudaErrorInvalidValue;  // the kernels' tile arithmetic is 32-bit
  const long long nitems =
      static_cast<long long>(batch) * ((height + cv.rows - 1) / cv.rows) * ((width + kTile - 1) / kTile);
  const int grid = static_cast<int>(nitems < ctas ? nitems : ctas);
  if (grid <= 0) return cudaSuccess;
  CUtensorMap map;
  const cudaError_t e = encode_input_map(in, batch, width, height, &map);
  if (e != cudaSuccess) return e;
  void* args[] = {&map,    const_cast<__nv_bfloat16**>(&wpack), const_cast<float**>(&bias),
                  const_cast<__nv_bfloat16**>(&mask), &out, &batch, &width, &height, &mode, &relu,
                  const_cast<unsigned int**>(&gate), &error};
  return cudaLaunchKernel(cv.fn, dim3(grid), dim3(kThreads), args, static_cast<size_t>(cv.smem), s);
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

// ---------------------------------------------------------------- weight gradient of a 32 -> 32 layer (tensor cores)
//
// dW[co][ci][ky][kx] += sum_p G[p][co] X[p + (ky - 1, kx - 1)][ci] and db[co] += sum_p G[p][co] over a batch of
// NHWC BF16 images (X: the layer's input activations, G: the gradient at its output, zero outside the image).
// As a GEMM per output row: M = (copy kx, input channel) = 3 x 32 rows plus a 32-row pad copy (M = 128), N = the
// 32 output channels, K = the row's pixels, one FP32 accumulator in tensor memory per tap row ky (3 x 32
// columns), summed over every output row the CTA takes and added to dW once at the end.
//
// A CTA takes items of kWgRows output rows of one kWgStrip-pixel strip.  Each input row is staged once, as three
// copies shifted by kx - 1 pixels, transposed into the canonical no-swizzle K-major layout
// [pixel group of 8 (K)][copy][channel][8 pixels]: the A operand of tap row ky of output row y is then the
// staged input row y - 1 + ky, its M rows (copy, channel) at a uniform 128-byte stride per 8 rows.  M rows
// 96..127 (the fourth "copy") read the next pixel group's first copy, or for the last group of the last ring
// slot the gradient ring that follows: staged values, finite, feeding only accumulator rows that are never
// read.  The gradient row is staged the same way as the B operand, [pixel group][output channel][8 pixels].  A
// thread loads a channel pair over 10 (8) pixels as 32-bit words and writes the transposed 16-byte rows with
// byte permutes; the loads of a row are issued before the wait for its ring slot, so they overlap the MMAs
// that still read the slot.  Rows live in rings (three input rows, two gradient rows); thread 0 issues an output
// row's 12 MMAs (3 tap rows x 4 k-steps of 16 pixels) and commits them to an mbarrier, and a ring slot is
// rewritten only after the MMAs that read it have completed.  Four CTAs per SM (their tensor memory fills the
// SM's 512 columns).  Waits are bounded as in conv32_tc_kernel; a timeout is agreed on by every thread
// (__syncthreads_and) before the CTA leaves its loop.
namespace {

constexpr int kWgStrip = 64;                         // pixels of an output row per item (K of a row)
constexpr int kWgGroups = kWgStrip / 8;              // pixel groups of 8 (16 bytes of BF16)
constexpr int kWgCopies = 3;                         // kx = 0, 1, 2
constexpr int kWgCore = kC * 16;                     // one copy of one pixel group: 32 channels x 16 bytes
constexpr int kWgXLbo = kWgCopies * kWgCore;         // A operand: bytes between pixel groups (K)
constexpr int kWgXRow = kWgGroups * kWgXLbo;         // one staged input row: 12,288 bytes
constexpr int kWgGRow = kWgGroups * kWgCore;         // one staged gradient row: 4,096 bytes
constexpr int kWgXSlots = 3;                         // an output row reads 3 input rows; the slot a new row
                                                     // takes was last read by the previous output row
constexpr int kWgGSlots = 2;
constexpr int kWgRows = 16;                          // output rows per item
constexpr int kWgThreads = 128;                      // thread t stages pixel group t / 16, channel pair t % 16
constexpr int kWgTmemCols = 128;                     // 3 accumulators x 32 columns, allocated as a power of 2
constexpr int kWgCtasPerSm = 4;
constexpr int kWgSmem = 128 + kWgXSlots * kWgXRow + kWgGSlots * kWgGRow + 2 * 8 + 16;
// the A operand reads up to 3,583 bytes from its start (a second pixel group at +LBO, 16 M groups of 128 bytes),
// at most 511 bytes past its ring slot, which the next slot or the gradient ring covers
static_assert(kWgGSlots * kWgGRow >= 4 * kWgCore, "the last slot's pad rows stay inside the gradient ring");
static_assert(kWgCtasPerSm * kWgTmemCols <= 512, "tensor memory of the resident CTAs");
static_assert(kWgThreads == kWgGroups * (kC / 2), "one (pixel group, channel pair) per thread");

__global__ void __launch_bounds__(kWgThreads, kWgCtasPerSm) wgrad32_tc_kernel(const __nv_bfloat16* __restrict__ X,
                                                                    const __nv_bfloat16* __restrict__ G,
                                                                    float* __restrict__ dW, float* __restrict__ db,
                                                                    int batch, int width, int height,
                                                                    unsigned int* __restrict__ error) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  unsigned char* sX = smem;
  unsigned char* sG = smem + kWgXSlots * kWgXRow;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sG + kWgGSlots * kWgGRow);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int pg = tid >> 4, cp = tid & 15;  // staging: pixel group, channel pair

  // the rings start zeroed, so that the pad rows read finite values before every slot has been staged
  for (int i = tid; i < (kWgXSlots * kWgXRow + kWgGSlots * kWgGRow) / 16; i += kWgThreads) {
    reinterpret_cast<uint4*>(sX)[i] = make_uint4(0u, 0u, 0u, 0u);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(kWgTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bars[i])));
    asm volatile("fence.mbarrier_init.release.cluster;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  const uint32_t tmem = *tmem_slot;
  const uint32_t xs0 = smem_u32(sX), gs0 = smem_u32(sG), bar0 = smem_u32(&bars[0]);

  const uint32_t strips = static_cast<uint32_t>((width + kWgStrip - 1) / kWgStrip);
  const uint32_t rblocks = static_cast<uint32_t>((height + kWgRows - 1) / kWgRows);
  const uint32_t nitems = static_cast<uint32_t>(batch) * rblocks * strips;

  bool ok = true;
  uint32_t xq = 0;      // input rows staged
  uint32_t oq = 0;      // output rows issued (MMA groups), group g commits to bars[g & 1]
  uint32_t waited = 0;  // groups whose completion has been waited for, in order
  int reader[kWgXSlots];  // the last group that reads each input-row slot
#pragma unroll
  for (int k = 0; k < kWgXSlots; ++k) reader[k] = -1;
  float bsum0 = 0.0f, bsum1 = 0.0f;

  // waits, in order, for the groups up to g: a group's barrier phase is waited for before the group two later
  // commits to the same barrier, so a parity never refers to a phase two completions old
  auto wait_through = [&](int g) {
    while (ok && static_cast<int>(waited) <= g) {
      if (!mbar_wait(bar0 + 8u * (waited & 1u), (waited >> 1) & 1u)) {
        ok = false;
        break;
      }
      ++waited;
    }
  };

  for (uint32_t it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
    const uint32_t rest = it / strips;
    const int xs = static_cast<int>(it - rest * strips) * kWgStrip;
    const uint32_t img = rest / rblocks;
    const int y0 = static_cast<int>(rest - img * rblocks) * kWgRows;
    const int rows = min(kWgRows, height - y0);
    const uint32_t xa = xq;  // ring index of input row y0 - 1
    const size_t img_base = static_cast<size_t>(img) * height;
    for (int i = -2; i < rows; ++i) {
      // stage input row y0 + i + 1 and, for i >= 0, gradient row y0 + i; then issue output row y0 + i.  The
      // global loads go first: they do not touch the rings, so they overlap the wait for the slots.
      const int y = y0 + i + 1;
      uint32_t wv[10];
      {
        const bool rok = y >= 0 && y < height;
        const unsigned int* rowp =
            reinterpret_cast<const unsigned int*>(X + (img_base + (rok ? y : 0)) * width * kC) + cp;
#pragma unroll
        for (int j = 0; j < 10; ++j) {
          const int px = xs - 1 + 8 * pg + j;
          wv[j] = (rok && px >= 0 && px < width) ? __ldg(rowp + static_cast<size_t>(px) * (kC / 2)) : 0u;
        }
      }
      uint32_t gv[8];
      if (i >= 0) {
        const unsigned int* growp =
            reinterpret_cast<const unsigned int*>(G + (img_base + (y0 + i)) * width * kC) + cp;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int px = xs + 8 * pg + j;
          gv[j] = px < width ? __ldg(growp + static_cast<size_t>(px) * (kC / 2)) : 0u;
        }
      }
      const uint32_t sx = xq % kWgXSlots;
      if (reader[sx] >= 0) wait_through(reader[sx]);
      if (i >= 0 && oq >= 2) wait_through(static_cast<int>(oq) - 2);
      if (ok) {
        unsigned char* dst = sX + sx * kWgXRow + pg * kWgXLbo + (2 * cp) * 16;
#pragma unroll
        for (int kx = 0; kx < 3; ++kx) {
          uint4 lo, hi;
          lo.x = __byte_perm(wv[kx + 0], wv[kx + 1], 0x5410);
          lo.y = __byte_perm(wv[kx + 2], wv[kx + 3], 0x5410);
          lo.z = __byte_perm(wv[kx + 4], wv[kx + 5], 0x5410);
          lo.w = __byte_perm(wv[kx + 6], wv[kx + 7], 0x5410);
          hi.x = __byte_perm(wv[kx + 0], wv[kx + 1], 0x7632);
          hi.y = __byte_perm(wv[kx + 2], wv[kx + 3], 0x7632);
          hi.z = __byte_perm(wv[kx + 4], wv[kx + 5], 0x7632);
          hi.w = __byte_perm(wv[kx + 6], wv[kx + 7], 0x7632);
          *reinterpret_cast<uint4*>(dst + kx * kWgCore) = lo;
          *reinterpret_cast<uint4*>(dst + kx * kWgCore + 16) = hi;
        }
        if (i >= 0) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            bsum0 += __uint_as_float(gv[j] << 16);
            bsum1 += __uint_as_float(gv[j] & 0xffff0000u);
          }
          unsigned char* gdst = sG + (oq % kWgGSlots) * kWgGRow + pg * kWgCore + (2 * cp) * 16;
          uint4 lo, hi;
          lo.x = __byte_perm(gv[0], gv[1], 0x5410);
          lo.y = __byte_perm(gv[2], gv[3], 0x5410);
          lo.z = __byte_perm(gv[4], gv[5], 0x5410);
          lo.w = __byte_perm(gv[6], gv[7], 0x5410);
          hi.x = __byte_perm(gv[0], gv[1], 0x7632);
          hi.y = __byte_perm(gv[2], gv[3], 0x7632);
          hi.z = __byte_perm(gv[4], gv[5], 0x7632);
          hi.w = __byte_perm(gv[6], gv[7], 0x7632);
          *reinterpret_cast<uint4*>(gdst) = lo;
          *reinterpret_cast<uint4*>(gdst + 16) = hi;
        }
      }
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the staged rows, for the MMAs' reads
      ok = __syncthreads_and(ok) != 0;
      ++xq;
      if (!ok) break;
      if (i < 0) continue;
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        const uint32_t b_row = gs0 + (oq % kWgGSlots) * kWgGRow;
        for (int ky = 0; ky < 3; ++ky) {
          const uint32_t a_row = xs0 + ((xa + static_cast<uint32_t>(i + ky)) % kWgXSlots) * kWgXRow;
          for (int ks = 0; ks < kWgStrip / 16; ++ks) {
            const uint64_t a = smem_desc(a_row + ks * 2 * kWgXLbo, kWgXLbo, 128);
            const uint64_t b = smem_desc(b_row + ks * 2 * kWgCore, kWgCore, 128);
            mma(tmem + 32u * ky, a, b, (oq == 0 && ks == 0) ? 0u : 1u);
          }
        }
        commit(bar0 + 8u * (oq & 1u));
      }
#pragma unroll
      for (int ky = 0; ky < 3; ++ky) reader[(xa + static_cast<uint32_t>(i + ky)) % kWgXSlots] = static_cast<int>(oq);
      ++oq;
    }
  }
  if (ok && oq > 0) wait_through(static_cast<int>(oq) - 1);
  ok = __syncthreads_and(ok) != 0;
  if (ok && oq > 0 && warp < 3) {  // warp kx reads TMEM lanes 32 kx .. 32 kx + 31 = input channel `lane`
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    for (int ky = 0; ky < 3; ++ky) {
      float acc[32];
      tmem_ld32(tmem + 32u * ky + (static_cast<uint32_t>(warp * 32) << 16), acc);
#pragma unroll
      for (int co = 0; co < kC; ++co) atomicAdd(&dW[(co * kC + lane) * 9 + ky * 3 + warp], acc[co]);
    }
  }
  if (ok) {
    // pixel groups pg and pg + 1 of a channel pair are lanes l and l ^ 16 of one warp
    bsum0 += __shfl_xor_sync(0xffffffffu, bsum0, 16);
    bsum1 += __shfl_xor_sync(0xffffffffu, bsum1, 16);
    if (lane < 16 && oq > 0) {
      atomicAdd(&db[2 * cp], bsum0);
      atomicAdd(&db[2 * cp + 1], bsum1);
    }
  }
  if (!ok) {
    if (lane == 0) atomicOr(error, kErrorBit);
    // the MMA groups still in flight complete before tensor memory is freed (bounded waits)
    if (tid == 0) {
      for (uint32_t w = waited; w < oq; ++w) mbar_wait(bar0 + 8u * (w & 1u), (w >> 1) & 1u);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kWgTmemCols));
  }
}

}  // namespace

cudaError_t launch_wgrad32(const __nv_bfloat16* x, const __nv_bfloat16* g, float* dw, float* db, int batch, int width,
                           int height, unsigned int* error, cudaStream_t s) {
  static int ctas = 0;
  if (ctas == 0) {
    const cudaError_t e =
        cudaFuncSetAttribute(wgrad32_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kWgSmem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    ctas = kWgCtasPerSm * (sms > 0 ? sms : 152);
  }
  if (reinterpret_cast<uintptr_t>(x) % 4 != 0 || reinterpret_cast<uintptr_t>(g) % 4 != 0) return cudaErrorInvalidValue;
  const long long nitems = static_cast<long long>(batch) * ((height + kWgRows - 1) / kWgRows) *
                           ((width + kWgStrip - 1) / kWgStrip);
  if (nitems > 0x7fffffffLL) return cudaErrorInvalidValue;  // the item arithmetic is 32-bit
  const int grid = static_cast<int>(nitems < ctas ? nitems : ctas);
  if (grid <= 0) return cudaSuccess;
  wgrad32_tc_kernel<<<grid, kWgThreads, kWgSmem, s>>>(x, g, dw, db, batch, width, height, error);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- the rest of the net (CUDA cores)
//
// Parameters, one FP32 array (kParamCount): w1[32][4][3][3] b1[32] w2[32][32][3][3] b2[32] w3[32][32][3][3] b3[32]
// w4[32][3][3] b4.  Input channels per pixel (FP32): the depth's local high-pass (d - m) * 100 (centimetres;
// m = mean of the valid depths of the 3x3 neighbourhood), the validity mask, and m / 4 (the depth level); the
// output is the residual r in centimetres, depth' = d + r / 100 on valid pixels (clamped at 0).  The
// high-pass keeps the BF16 activations' 8 significant bits on the noise rather than on metres of depth.
namespace {

constexpr int kCin = 4;
constexpr float kScale = 100.0f, kInvScale = 0.01f;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kC * kCin * 9, kOffW2 = kOffB1 + kC, kOffB2 = kOffW2 + kC * kC * 9;
constexpr int kOffW3 = kOffB2 + kC, kOffB3 = kOffW3 + kC * kC * 9, kOffW4 = kOffB3 + kC, kOffB4 = kOffW4 + kC * 9;
constexpr int kParams = kOffB4 + 1;
// depth-discontinuity threshold max(base, rel * depth) of the reference's GPU path (cuda_tsdf_integrator.cu:27-28):
// training ignores pixels whose raw depth and target differ by more (they see different surfaces), and at
// inference a correction larger than it falls back to the bilateral filter's value
constexpr float kGateBase = 0.012f, kGateRel = 0.025f;

__device__ __forceinline__ float gate(float d) { return fmaxf(kGateBase, kGateRel * d); }

__device__ __forceinline__ bool inside(int x, int y, int w, int h) { return x >= 0 && x < w && y >= 0 && y < h; }

__global__ void pack_input_kernel(const float* __restrict__ depth, float4* __restrict__ X, int batch, int w, int h) {
  const long long n = static_cast<long long>(batch) * w * h;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int x = static_cast<int>(i % w), y = static_cast<int>((i / w) % h);
    const long long img = i / (static_cast<long long>(w) * h);
    const float d = depth[i];
    float sum = 0.0f;
    int cnt = 0;
    for (int dy = -1; dy <= 1; ++dy) {
      for (int dx = -1; dx <= 1; ++dx) {
        if (!inside(x + dx, y + dy, w, h)) continue;
        const float v = depth[(img * h + y + dy) * w + x + dx];
        if (v > 0.0f) {
          sum += v;
          ++cnt;
        }
      }
    }
    const bool valid = d > 0.0f;
    const float m = cnt ? sum / static_cast<float>(cnt) : 0.0f;
    X[i] = valid ? make_float4((d - m) * kScale, 1.0f, m * 0.25f, 0.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
}

// layer 1: 4 -> 32, ReLU, one thread per pixel; weights staged tap-major as float4 over the 4 input channels
// (sw4[t][co] = w1[co][0..3][t]) so that one 16-byte shared load feeds 4 multiply-adds.  The 9 taps' loads
// are issued together, and each warp writes its 32 pixels x 64 bytes through its shared-memory buffer
// (epi_pos), 512 contiguous bytes per store instruction; the loop runs over whole warps so that every lane
// takes part in the buffer's warp-synchronous steps.
__global__ void __launch_bounds__(256) conv_in_kernel(const float4* __restrict__ X, const float* __restrict__ params,
                                                      __nv_bfloat16* __restrict__ A1, int batch, int w, int h) {
  __shared__ float4 sw4[9][kC];
  __shared__ float sb[kC];
  __shared__ uint4 sbuf[8][128];  // one 2 KB transpose buffer per warp of the 256 threads
  for (int i = threadIdx.x; i < 9 * kC; i += blockDim.x) {
    const int t = i / kC, co = i % kC;
    const float* wc = params + kOffW1 + co * kCin * 9;
    sw4[t][co] = make_float4(wc[0 * 9 + t], wc[1 * 9 + t], wc[2 * 9 + t], wc[3 * 9 + t]);
  }
  for (int i = threadIdx.x; i < kC; i += blockDim.x) sb[i] = params[kOffB1 + i];
  __syncthreads();
  const long long n = static_cast<long long>(batch) * w * h;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint4* buf = sbuf[warp];
  const long long warps = static_cast<long long>(gridDim.x) * (blockDim.x >> 5);
  for (long long base = (blockIdx.x * static_cast<long long>(blockDim.x >> 5) + warp) * 32; base < n;
       base += warps * 32) {
    const long long i = base + lane;
    float4 in[9];
    if (i < n) {
      // 32-bit coordinates (the launcher keeps the pixel count below 2^31)
      const uint32_t i32 = static_cast<uint32_t>(i), row = i32 / static_cast<uint32_t>(w);
      const int x = static_cast<int>(i32 - row * static_cast<uint32_t>(w));
      const uint32_t im = row / static_cast<uint32_t>(h);
      const int y = static_cast<int>(row - im * static_cast<uint32_t>(h));
      const long long img = im;
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const int sx = x + t % 3 - 1, sy = y + t / 3 - 1;
        in[t] = inside(sx, sy, w, h) ? X[(img * h + sy) * w + sx] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
    } else {
#pragma unroll
      for (int t = 0; t < 9; ++t) in[t] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    float acc[kC];
#pragma unroll
    for (int co = 0; co < kC; ++co) acc[co] = sb[co];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
#pragma unroll
      for (int co = 0; co < kC; ++co) {
        const float4 wv = sw4[t][co];
        acc[co] += wv.x * in[t].x + wv.y * in[t].y + wv.z * in[t].z + wv.w * in[t].w;
      }
    }
    __align__(16) __nv_bfloat162 res[kC / 2];
#pragma unroll
    for (int c = 0; c < kC / 2; ++c) res[c] = __floats2bfloat162_rn(fmaxf(acc[2 * c], 0.0f), fmaxf(acc[2 * c + 1], 0.0f));
#pragma unroll
    for (int q = 0; q < 4; ++q) buf[epi_pos(lane, q)] = reinterpret_cast<const uint4*>(res)[q];
    __syncwarp();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int p = 8 * u + (lane >> 2), q = lane & 3;
      if (base + p < n) *reinterpret_cast<uint4*>(A1 + (base + p) * kC + 8 * q) = buf[epi_pos(p, q)];
    }
    __syncwarp();  // the buffer is rewritten by the next group
  }
}

__device__ __forceinline__ void load32(const __nv_bfloat16* p, float* v) {
  __align__(16) __nv_bfloat16 b[kC];
#pragma unroll
  for (int q = 0; q < 4; ++q) reinterpret_cast<uint4*>(b)[q] = reinterpret_cast<const uint4*>(p)[q];
#pragma unroll
  for (int c = 0; c < kC; ++c) v[c] = __bfloat162float(b[c]);
}

// layer 4: 32 -> 1 residual, depth' = d + r / 100 on valid pixels; weights staged tap-major (sw[t][c]) and
// read as float4.  Four lanes per pixel, lane q = lane % 4 summing channels 8q..8q+7 over the taps: a warp
// covers 8 consecutive pixels, so its 16-byte loads of their 64-byte channel vectors are contiguous, and the
// 9 taps' loads are issued together.  The pixel's four lanes then add their sums; the loop runs over
// warp-sized groups of 8 pixels so that every lane takes part in the shuffles.
__global__ void __launch_bounds__(256) conv_out_kernel(const __nv_bfloat16* __restrict__ A3,
                                                       const float* __restrict__ params,
                                                       const float* __restrict__ depth,
                                                       const float* __restrict__ fallback, float* __restrict__ out,
                                                       int batch, int w, int h) {
  __shared__ float4 sw4[9][kC / 4];
  __shared__ float sb;
  for (int i = threadIdx.x; i < 9 * kC; i += blockDim.x) {
    const int t = i / kC, c = i % kC;
    reinterpret_cast<float*>(&sw4[t][0])[c] = params[kOffW4 + c * 9 + t];
  }
  if (threadIdx.x == 0) sb = params[kOffB4];
  __syncthreads();
  const long long n = static_cast<long long>(batch) * w * h;
  const int lane = threadIdx.x & 31, q = lane & 3;
  const long long warps = static_cast<long long>(gridDim.x) * (blockDim.x >> 5);
  for (long long base = (blockIdx.x * static_cast<long long>(blockDim.x >> 5) + (threadIdx.x >> 5)) * 8; base < n;
       base += warps * 8) {
    const long long i = base + (lane >> 2);
    const float d = i < n ? depth[i] : 0.0f;
    float r = 0.0f;
    if (d > 0.0f) {
      const uint32_t i32 = static_cast<uint32_t>(i), row = i32 / static_cast<uint32_t>(w);  // 32-bit, as in conv_in
      const int x = static_cast<int>(i32 - row * static_cast<uint32_t>(w));
      const uint32_t im = row / static_cast<uint32_t>(h);
      const int y = static_cast<int>(row - im * static_cast<uint32_t>(h));
      const long long img = im;
      // the 9 taps' loads are issued together (zero outside the image, which adds nothing), then used
      uint4 raw9[9];
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const int sx = x + t % 3 - 1, sy = y + t / 3 - 1;
        raw9[t] = inside(sx, sy, w, h) ? *reinterpret_cast<const uint4*>(A3 + ((img * h + sy) * w + sx) * kC + 8 * q)
                                       : make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const __nv_bfloat162* b2 = reinterpret_cast<const __nv_bfloat162*>(&raw9[t]);
        const float4 wa = sw4[t][2 * q], wb = sw4[t][2 * q + 1];
        const float2 a0 = __bfloat1622float2(b2[0]), a1 = __bfloat1622float2(b2[1]);
        const float2 a2 = __bfloat1622float2(b2[2]), a3 = __bfloat1622float2(b2[3]);
        r += wa.x * a0.x + wa.y * a0.y + wa.z * a1.x + wa.w * a1.y + wb.x * a2.x + wb.y * a2.y + wb.z * a3.x +
             wb.w * a3.y;
      }
    }
    r += __shfl_xor_sync(0xffffffffU, r, 1);
    r += __shfl_xor_sync(0xffffffffU, r, 2);
    if (q == 0 && i < n) {
      if (!(d > 0.0f)) {
        out[i] = 0.0f;
      } else {
        const float corr = (sb + r) * kInvScale;
        out[i] = (fallback && fabsf(corr) > gate(d)) ? fallback[i] : fmaxf(d + corr, 0.0f);
      }
    }
  }
}

// loss = sum over pixels valid in input, target and output whose input and target agree within the
// discontinuity threshold, of (out - target)^2 / n_pixels; dr = dloss/dr
__global__ void loss_grad_kernel(const float* __restrict__ out, const float* __restrict__ target,
                                 const float* __restrict__ depth, float* __restrict__ dr, long long n,
                                 float* __restrict__ loss) {
  float se = 0.0f, cnt = 0.0f;
  const float inv_n = 1.0f / static_cast<float>(n);
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const bool m = depth[i] > 0.0f && target[i] > 0.0f && out[i] > 0.0f && fabsf(depth[i] - target[i]) <= gate(target[i]);
    const float diff = m ? out[i] - target[i] : 0.0f;
    dr[i] = 2.0f * diff * kInvScale * inv_n;
    se += diff * diff;
    cnt += m ? 1.0f : 0.0f;
  }
  for (int o = 16; o > 0; o >>= 1) {
    se += __shfl_down_sync(0xffffffffU, se, o);
    cnt += __shfl_down_sync(0xffffffffU, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&loss[0], se);
    atomicAdd(&loss[1], cnt);
  }
}

// dA3[q][c] = (A3[q][c] > 0) * sum_t w4[c][t] dr[q - off(t)]
__global__ void __launch_bounds__(256) dgrad_out_kernel(const float* __restrict__ dr, const float* __restrict__ params,
                                                        const __nv_bfloat16* __restrict__ A3,
                                                        __nv_bfloat16* __restrict__ dA3, int batch, int w, int h) {
  __shared__ float sw[kC * 9];
  for (int i = threadIdx.x; i < kC * 9; i += blockDim.x) sw[i] = params[kOffW4 + i];
  __syncthreads();
  const long long n = static_cast<long long>(batch) * w * h;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int x = static_cast<int>(i % w), y = static_cast<int>((i / w) % h);
    const long long img = i / (static_cast<long long>(w) * h);
    float g[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int sx = x - (t % 3 - 1), sy = y - (t / 3 - 1);
      g[t] = inside(sx, sy, w, h) ? dr[(img * h + sy) * w + sx] : 0.0f;
    }
    float a[kC];
    load32(A3 + i * kC, a);
    __align__(16) __nv_bfloat16 res[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
      float acc = 0.0f;
#pragma unroll
      for (int t = 0; t < 9; ++t) acc += sw[c * 9 + t] * g[t];
      res[c] = __float2bfloat16_rn(a[c] > 0.0f ? acc : 0.0f);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) reinterpret_cast<uint4*>(dA3 + i * kC)[q] = reinterpret_cast<const uint4*>(res)[q];
  }
}

// Weight gradients of the input and output layers (CUDA cores): dW[co][ci][t] = sum_p dY[p][co] X[p + off(t)][ci],
// db[co] = sum_p dY[p][co].  X: BF16 with 32 channels (read as 16-byte vectors) or FP32 float4 (CI = 4); dY:
// BF16 with 32 channels or FP32 with 1.  Each CTA stages row segments of kSeg pixels (three input rows with a
// one-pixel halo, one gradient row) in shared memory as floats.  Thread (rep, co, ci) keeps 9 accumulators (and
// the bias sum) over the rep-th of kRep contiguous runs of each segment, so that CI x CO x kRep threads share a
// segment; the kRep partial sums are added in shared memory and flushed with one atomic per weight per CTA.
constexpr int kSeg = 64;

template <int CI, int CO, bool kXBf16, bool kDyBf16, int kRep>
__global__ void __launch_bounds__(CI * CO * kRep) wgrad_kernel(const void* __restrict__ Xv, const void* __restrict__ dYv,
                                                               float* __restrict__ dW, float* __restrict__ db,
                                                               int batch, int w, int h) {
  static_assert(!kXBf16 || CI == 32, "BF16 inputs carry 32 channels");
  static_assert(kXBf16 || CI == 4, "FP32 inputs are float4 pixels");
  static_assert(!kDyBf16 || CO == 32, "BF16 gradients carry 32 channels");
  static_assert(kDyBf16 || CO == 1, "FP32 gradients carry one channel");
  static_assert(kSeg % kRep == 0, "replicas take equal runs of a segment");
  constexpr int kPairs = CI * CO, kT = kPairs * kRep;
  __shared__ __align__(16) float sX[3][kSeg + 2][CI];
  __shared__ __align__(16) float sG[kSeg][CO];
  __shared__ float sRed[kRep > 1 ? kRep - 1 : 1][10][kPairs];
  const int tid = threadIdx.x;
  const int pair = tid % kPairs, rep = tid / kPairs;
  const int co = pair / CI, ci = pair % CI;
  float acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float bacc = 0.0f;
  const int segs_x = (w + kSeg - 1) / kSeg;
  const long long nseg = static_cast<long long>(batch) * h * segs_x;
  for (long long sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
    const int x0 = static_cast<int>(sgi % segs_x) * kSeg;
    const int y = static_cast<int>((sgi / segs_x) % h);
    const long long img = sgi / (static_cast<long long>(segs_x) * h);
    if (kXBf16) {  // 4 vectors of 8 channels per pixel
      for (int i = tid; i < 3 * (kSeg + 2) * 4; i += kT) {
        const int q = i & 3, px = (i >> 2) % (kSeg + 2), r = (i >> 2) / (kSeg + 2);
        const int sx = x0 - 1 + px, sy = y - 1 + r;
        uint4 u = make_uint4(0u, 0u, 0u, 0u);
        if (inside(sx, sy, w, h)) {
          u = reinterpret_cast<const uint4*>(static_cast<const __nv_bfloat16*>(Xv) + ((img * h + sy) * w + sx) * CI)[q];
        }
        const __nv_bfloat162* b2 = reinterpret_cast<const __nv_bfloat162*>(&u);
        float4* dst = reinterpret_cast<float4*>(&sX[r][px][8 * q]);
        const float2 f0 = __bfloat1622float2(b2[0]), f1 = __bfloat1622float2(b2[1]);
        const float2 f2 = __bfloat1622float2(b2[2]), f3 = __bfloat1622float2(b2[3]);
        dst[0] = make_float4(f0.x, f0.y, f1.x, f1.y);
        dst[1] = make_float4(f2.x, f2.y, f3.x, f3.y);
      }
    } else {  // one float4 per pixel
      for (int i = tid; i < 3 * (kSeg + 2); i += kT) {
        const int px = i % (kSeg + 2), r = i / (kSeg + 2);
        const int sx = x0 - 1 + px, sy = y - 1 + r;
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (inside(sx, sy, w, h)) v = static_cast<const float4*>(Xv)[(img * h + sy) * w + sx];
        *reinterpret_cast<float4*>(&sX[r][px][0]) = v;
      }
    }
    if (kDyBf16) {
      for (int i = tid; i < kSeg * 4; i += kT) {
        const int q = i & 3, px = i >> 2;
        const int sx = x0 + px;
        uint4 u = make_uint4(0u, 0u, 0u, 0u);
        if (sx < w) u = reinterpret_cast<const uint4*>(static_cast<const __nv_bfloat16*>(dYv) + ((img * h + y) * w + sx) * CO)[q];
        const __nv_bfloat162* b2 = reinterpret_cast<const __nv_bfloat162*>(&u);
        float4* dst = reinterpret_cast<float4*>(&sG[px][8 * q]);
        const float2 f0 = __bfloat1622float2(b2[0]), f1 = __bfloat1622float2(b2[1]);
        const float2 f2 = __bfloat1622float2(b2[2]), f3 = __bfloat1622float2(b2[3]);
        dst[0] = make_float4(f0.x, f0.y, f1.x, f1.y);
        dst[1] = make_float4(f2.x, f2.y, f3.x, f3.y);
      }
    } else {
      for (int i = tid; i < kSeg; i += kT) {
        const int sx = x0 + i;
        sG[i][0] = sx < w ? static_cast<const float*>(dYv)[(img * h + y) * w + sx] : 0.0f;
      }
    }
    __syncthreads();
    // replica rep takes a contiguous run of the segment's pixels, so each tap row's three inputs slide along it:
    // one new shared-memory read per row and pixel instead of three
    constexpr int kRun = kSeg / kRep;
    const int p0 = rep * kRun;
    float w0[3], w1[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      w0[r] = sX[r][p0][ci];
      w1[r] = sX[r][p0 + 1][ci];
    }
    for (int px = p0; px < p0 + kRun; ++px) {
      const float g = sG[px][co];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const float w2 = sX[r][px + 2][ci];
        acc[3 * r] += g * w0[r];
        acc[3 * r + 1] += g * w1[r];
        acc[3 * r + 2] += g * w2;
        w0[r] = w1[r];
        w1[r] = w2;
      }
      bacc += g;
    }
    __syncthreads();
  }
  if (kRep > 1) {
    if (rep > 0) {
#pragma unroll
      for (int t = 0; t < 9; ++t) sRed[rep - 1][t][pair] = acc[t];
      sRed[rep - 1][9][pair] = bacc;
    }
    __syncthreads();
    if (rep == 0) {
      for (int r = 0; r < kRep - 1; ++r) {
#pragma unroll
        for (int t = 0; t < 9; ++t) acc[t] += sRed[r][t][pair];
        bacc += sRed[r][9][pair];
      }
    }
  }
  if (rep == 0) {
#pragma unroll
    for (int t = 0; t < 9; ++t) atomicAdd(&dW[(co * CI + ci) * 9 + t], acc[t]);
    if (ci == 0) atomicAdd(&db[co], bacc);
  }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

int grid_for_elems(long long n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (n + 255) / 256;
  const long long cap = 8LL * (sms > 0 ? sms : 152);
  return static_cast<int>(want < cap ? (want > 0 ? want : 1) : cap);
}

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 152;
}

}  // namespace

int param_count() { return kParams; }

size_t workspace_bytes(int batch, int width, int height) {
  const size_t n = static_cast<size_t>(batch) * width * height;
  // X (float4), A1, A2, A3 (32 x BF16), r / dr (float), dA x 2 (32 x BF16)
  return n * (16 + 3 * 64 + 4 + 2 * 64) + 4096;
}

static void carve(unsigned char* ws, size_t n, float4** X, __nv_bfloat16** A1, __nv_bfloat16** A2,
                  __nv_bfloat16** A3, float** r, __nv_bfloat16** G1, __nv_bfloat16** G2) {
  size_t o = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = ws + o;
    o += (bytes + 255) & ~static_cast<size_t>(255);
    return p;
  };
  *X = reinterpret_cast<float4*>(take(n * 16));
  *A1 = reinterpret_cast<__nv_bfloat16*>(take(n * 64));
  *A2 = reinterpret_cast<__nv_bfloat16*>(take(n * 64));
  *A3 = reinterpret_cast<__nv_bfloat16*>(take(n * 64));
  *r = reinterpret_cast<float*>(take(n * 4));
  *G1 = reinterpret_cast<__nv_bfloat16*>(take(n * 64));
  *G2 = reinterpret_cast<__nv_bfloat16*>(take(n * 64));
}

cudaError_t pack_weights(const float* params, __nv_bfloat16* packed, cudaStream_t s) {
  cudaError_t e = launch_pack_w32(params + kOffW2, packed, 0, s);
  if (e == cudaSuccess) e = launch_pack_w32(params + kOffW3, packed + 9 * kC * kC, 0, s);
  if (e == cudaSuccess) e = launch_pack_w32(params + kOffW2, packed + 2 * 9 * kC * kC, 1, s);
  if (e == cudaSuccess) e = launch_pack_w32(params + kOffW3, packed + 3 * 9 * kC * kC, 1, s);
  return e;
}

cudaError_t forward(const float* params, const __nv_bfloat16* packed, const float* depth, const float* fallback,
                    float* out, int batch, int width, int height, unsigned char* ws, unsigned int* error,
                    cudaStream_t s) {
  const size_t n = static_cast<size_t>(batch) * width * height;
  if (n > 0x7fffffffULL) return cudaErrorInvalidValue;  // the layers' pixel arithmetic is 32-bit
  float4* X;
  __nv_bfloat16 *A1, *A2, *A3, *G1, *G2;
  float* r;
  carve(ws, n, &X, &A1, &A2, &A3, &r, &G1, &G2);
  const int grid = grid_for_elems(static_cast<long long>(n));
  pack_input_kernel<<<grid, 256, 0, s>>>(depth, X, batch, width, height);
  conv_in_kernel<<<grid, 256, 0, s>>>(X, params, A1, batch, width, height);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_conv32(A1, packed, params + kOffB2, nullptr, A2, batch, width, height, kForward, 1, error, s);
  if (e == cudaSuccess) {
    e = launch_conv32(A2, packed + 9 * kC * kC, params + kOffB3, nullptr, A3, batch, width, height, kForward, 1, error, s);
  }
  if (e != cudaSuccess) return e;
  conv_out_kernel<<<grid, 256, 0, s>>>(A3, params, depth, fallback, out, batch, width, height);
  return cudaGetLastError();
}

cudaError_t backward(const float* params, const __nv_bfloat16* packed, const float* depth, const float* target,
                     const float* out, int batch, int width, int height, unsigned char* ws, float* grads, float* loss,
                     unsigned int* error, cudaStream_t s) {
  const size_t n = static_cast<size_t>(batch) * width * height;
  float4* X;
  __nv_bfloat16 *A1, *A2, *A3, *G1, *G2;
  float* dr;
  carve(ws, n, &X, &A1, &A2, &A3, &dr, &G1, &G2);
  const int grid = grid_for_elems(static_cast<long long>(n));
  cudaError_t e = cudaMemsetAsync(grads, 0, kParams * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(loss, 0, 2 * sizeof(float), s);
  if (e != cudaSuccess) return e;
  const int wg = 4 * sm_count();  // CUDA-core weight gradients: 256-thread CTAs, four per SM
  loss_grad_kernel<<<grid, 256, 0, s>>>(out, target, depth, dr, static_cast<long long>(n), loss);
  // layer 4: weights, then the gradient into A3
  wgrad_kernel<kC, 1, true, false, 8><<<wg, kC * 8, 0, s>>>(A3, dr, grads + kOffW4, grads + kOffB4, batch, width,
                                                             height);
  dgrad_out_kernel<<<grid, 256, 0, s>>>(dr, params, A3, G1, batch, width, height);
  // layer 3
  e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_wgrad32(A2, G1, grads + kOffW3, grads + kOffB3, batch, width, height, error, s);
  if (e == cudaSuccess) {
    e = launch_conv32(G1, packed + 3 * 9 * kC * kC, nullptr, A2, G2, batch, width, height, kGrad, 0, error, s);
  }
  if (e != cudaSuccess) return e;
  // layer 2
  e = launch_wgrad32(A1, G2, grads + kOffW2, grads + kOffB2, batch, width, height, error, s);
  if (e == cudaSuccess) {
    e = launch_conv32(G2, packed + 2 * 9 * kC * kC, nullptr, A1, G1, batch, width, height, kGrad, 0, error, s);
  }
  if (e != cudaSuccess) return e;
  // layer 1
  wgrad_kernel<kCin, kC, false, true, 2><<<wg, kCin * kC * 2, 0, s>>>(X, G1, grads + kOffW1, grads + kOffB1, batch, width,
                                                              height);
  return cudaGetLastError();
}

cudaError_t adam(float* params, const float* grads, float* m, float* v, float lr, float b1, float b2, float eps,
                 int step, cudaStream_t s) {
  const float c1 = 1.0f - powf(b1, static_cast<float>(step)), c2 = 1.0f - powf(b2, static_cast<float>(step));
  adam_kernel<<<(kParams + 255) / 256, 256, 0, s>>>(params, grads, m, v, kParams, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

}  // namespace nn
}  // namespace vh
