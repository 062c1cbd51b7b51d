// vh_common.cuh -- device-side layout, parameters and exact-order math shared by the GB300 kernels.
//
// Every floating-point expression below is written in the operation order of the reference CUDA
// sources (src/cuda_tsdf_integrator.cu, src/cuda_block_allocator.cu, src/cuda_mesh_extractor.cu) and
// the library is compiled with -fmad=false, so each a*b+c rounds twice exactly as the source reads;
// IEEE division and square root are the nvcc defaults (-prec-div=true -prec-sqrt=true), and vh_expf returns
// the C library's expf bit for bit (see below), so the plain FP32 form reproduces the reference compiled for
// a host bit for bit.
#pragma once

#include <cstdint>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace vh {

constexpr int kBlockSide = 8;
constexpr int kBlockVoxels = 512;
constexpr int kDirs = 6;
constexpr int kLayers = 3;
constexpr unsigned long long kEmptyKey = ~0ULL;  // cuda_block_allocator.cu:19
constexpr uint32_t kInvalidBlock = 0xffffffffu;
constexpr int kKeyBits = 21;                      // cuda_block_allocator.cu:20-22
constexpr int kKeyBias = 1 << (kKeyBits - 1);
constexpr unsigned long long kKeyMask = (1ULL << kKeyBits) - 1ULL;

// sticky error bits in Counters::error
constexpr uint32_t kErrKeyRange = 1u;  // block coordinate outside the 21-bit packed range
constexpr uint32_t kErrHashFull = 2u;  // no free slot within `capacity` probes
constexpr uint32_t kErrPoolFull = 4u;  // more blocks than the pool holds
constexpr uint32_t kErrTimeout = 8u;   // a bounded wait on the tensor cores gave up (the denoiser's convolution)

// Device-resident counters of one volume (64 bytes; read back with one D2H copy).
struct Counters {
  uint32_t num_blocks;         // blocks ever allocated (pool high-water mark)
  uint32_t visible_count;      // unique blocks touched by the current frame
  uint32_t error;              // sticky kErr* bits
  uint32_t frame;              // frame stamp of the current frame (starts at 1)
  unsigned long long observed_voxels;  // voxels with any layer weight > 0
  uint32_t new_blocks;         // blocks allocated by the current frame
  uint32_t integrated_voxels;  // voxel layer updates applied by the current frame
  uint32_t active_voxels;      // voxels of the current frame that reached the layer update stage
  uint32_t update_queue;       // next chunk of the fused layer update (a device work queue; reset per frame)
  uint32_t pad[6];
};
static_assert(sizeof(Counters) == 64, "Counters is read back as one 64-byte copy");

// Device view of one volume.  HBM layout:
//   slot_keys   u64[capacity]           packed block keys (open addressing, linear probing)
//   slot_block  u32[capacity]           pool index of the key in the slot
//   slot_stamp  u32[capacity]           last frame that put the slot on the visible list
//   layers      float4[max_blocks][6][512][3]   {weight, surface_coord, plane_offset, packed_normal bits}
//                                       direction-major inside a block so that a warp of voxels with the
//                                       same dominant direction reads/writes 32 x 48 contiguous bytes
//   block_keys  int4[max_blocks]        {x, y, z, frame the block was allocated in}
//   obs_mask    u32[max_blocks][16]     one bit per voxel: any layer observed
//   dir_mask    u32[max_blocks]         bit d set once any voxel of the block has an observed layer in bin d
//   visible     u32[capacity]           slots touched by the current frame (unordered)
//   visible_keys int4[capacity]         per visible entry {x, y, z, pool index}: written after the allocation
//                                       by the normal-map pass, read once per chunk by the fused update
//   active      u32[max_blocks * 512]   (block << 9 | voxel) of the current frame's voxels that pass the
//                                       projection / depth / truncation tests (unordered)
struct Volume {
  unsigned long long* slot_keys;
  uint32_t* slot_block;
  uint32_t* slot_stamp;
  float4* layers;    // FP32 layer records (layer_format 0), nullptr otherwise
  uint4* layers16;   // FP16 bins (layer_format 1), nullptr otherwise
  int4* block_keys;
  uint32_t* obs_mask;
  uint32_t* dir_mask;
  uint32_t* block_stamp;  // per pool block: the last frame that ran the layer update over it
  uint32_t* visible;
  int4* visible_keys;
  uint32_t* active;
  Counters* counters;
  uint32_t capacity;
  uint32_t mask;
  uint32_t max_blocks;
  float voxel_size;      // metres (the FP16 codec's unit)
  float inv_voxel_size;  // 1 / voxel_size, rounded once on the host
  uint32_t pad[3];
};

struct Mat34 {
  float r[9];
  float t[3];
};

// Per-call algorithm parameters (constants of cuda_tsdf_integrator.cu:16-35 and cuda_mesh_extractor.cu:14-23,
// with the derived 1/(2 sigma^2) factors computed on the host in float exactly as the reference's constexprs).
struct Params {
  int width, height;
  float fx, fy, cx, cy;
  Mat34 T_wc;  // camera -> world
  Mat34 T_cw;  // world -> camera, Pose::inverse() computed on the host (math_types.h:192-197)
  float voxel_size;
  float truncation;
  float block_world_size;  // voxel_size * 8 (cuda_block_allocator.cu:342)
  int stride;
  int sample_width, sample_height;
  float disc_base, disc_rel;
  int filter_radius;
  float filter_k_spatial, filter_k_range, filter_k_angular, filter_min_cos;
  int normal_radius;
  float normal_k_spatial, normal_k_range, normal_k_angular;
  float merge_tol, layer_normal_cos, extract_tol;
  float max_weight, depth_sigma, huber_delta, min_obs_weight, min_view_weight;
  float iso;
  int alloc_mode;  // 0: reference rule (3 points x 27 neighbours), 1: truncation band (blocks crossed by the band)
  int normal_mode;  // 0: bilateral normal per voxel (reference), 1: per-pixel normal map, interpolated per voxel
};

// One scene of a multi-scene batch step (device memory, rewritten by the host every step).  Items are the
// work-queue units of the three batch kernels: filter tiles, allocation tiles, normal-map tiles (32x8 each).
struct SceneDesc {
  Volume V;
  Params p;
  const float* depth_in;  // raw depth, device
  float* depth;           // filtered depth, device
  float4* nmap;           // per-pixel normal map, device
  uint32_t filter_first, filter_items;  // [first, first + items) in the filter + allocation kernel's item space
  uint32_t map_first, map_items;        // in the normal-map kernel's item space
  uint32_t active, pad;
};

// Step header of a batch (device memory): scene count and item totals.
struct BatchHeader {
  uint32_t nscenes;
  uint32_t filter_total;  // filter + allocation items
  uint32_t stage2_total;  // normal-map items
  uint32_t pad;
};

constexpr int kMaxBatchScenes = 256;

struct f3 {
  float x, y, z;
};

__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 mul3(f3 v, float s) { return mk3(v.x * s, v.y * s, v.z * s); }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float norm3(f3 v) { return sqrtf(dot3(v, v)); }
// cuda_tsdf_integrator.cu:201-209
__device__ __forceinline__ f3 normalize3(f3 v) {
  const float len = norm3(v);
  if (len <= 1e-6f) return mk3(0.0f, 0.0f, 0.0f);
  const float inv = 1.0f / len;
  return mk3(v.x * inv, v.y * inv, v.z * inv);
}
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(hi, fmaxf(lo, v)); }

__device__ __forceinline__ f3 xform_point(const Mat34& P, f3 p) {
  return mk3(P.r[0] * p.x + P.r[1] * p.y + P.r[2] * p.z + P.t[0], P.r[3] * p.x + P.r[4] * p.y + P.r[5] * p.z + P.t[1],
             P.r[6] * p.x + P.r[7] * p.y + P.r[8] * p.z + P.t[2]);
}
__device__ __forceinline__ f3 xform_vector(const Mat34& P, f3 p) {
  return mk3(P.r[0] * p.x + P.r[1] * p.y + P.r[2] * p.z, P.r[3] * p.x + P.r[4] * p.y + P.r[5] * p.z,
             P.r[6] * p.x + P.r[7] * p.y + P.r[8] * p.z);
}
// cuda_tsdf_integrator.cu:570-579
__device__ __forceinline__ f3 backproject(float u, float v, float d, const Params& p) {
  return mk3((u - p.cx) * d / p.fx, (v - p.cy) * d / p.fy, d);
}

// ---- Single-precision exponential, bit-identical to the C library's expf ----
//
// The reference weighs its bilateral taps with expf (cuda_tsdf_integrator.cu:173-175).  Compiled for a host,
// that is the GNU C library's expf (glibc >= 2.28, the table-driven algorithm of ARM's optimized-routines):
//   z = x * 32/ln2 (double), k = z rounded to the nearest integer (ties to even), r = fma(32/ln2, x, -k),
//   y = 2^(k/32) * (1 + C2 r + C1 r^2 + C0 r^3) in double arithmetic (2^(j/32) from a 32-entry table),
//   result = (float) y.
// vh_expf returns exactly that float for every argument.  The GB300 runs FP64 at a small fraction of its FP32
// rate, so the common path evaluates the same polynomial in float-float arithmetic (error below 2^-45.7 of
// the result over every finite float argument) and rounds it itself; only when that value lies within 2^-40
// of a rounding boundary (about 5 arguments in a million) does it run the double-precision sequence
// (expf_double).  Every operation is an explicit round-to-nearest intrinsic, so the fast-math compile
// evaluates it identically.
namespace expf_detail {
// bits of the double nearest 2^(j/32), minus j << 47 (so that adding k << 47 scales by 2^floor(k/32))
static __device__ const unsigned long long kTab[32] = {
    0x3ff0000000000000ULL, 0x3fefd9b0d3158574ULL, 0x3fefb5586cf9890fULL, 0x3fef9301d0125b51ULL,
    0x3fef72b83c7d517bULL, 0x3fef54873168b9aaULL, 0x3fef387a6e756238ULL, 0x3fef1e9df51fdee1ULL,
    0x3fef06fe0a31b715ULL, 0x3feef1a7373aa9cbULL, 0x3feedea64c123422ULL, 0x3feece086061892dULL,
    0x3feebfdad5362a27ULL, 0x3feeb42b569d4f82ULL, 0x3feeab07dd485429ULL, 0x3feea47eb03a5585ULL,
    0x3feea09e667f3bcdULL, 0x3fee9f75e8ec5f74ULL, 0x3feea11473eb0187ULL, 0x3feea589994cce13ULL,
    0x3feeace5422aa0dbULL, 0x3feeb737b0cdc5e5ULL, 0x3feec49182a3f090ULL, 0x3feed503b23e255dULL,
    0x3feee89f995ad3adULL, 0x3feeff76f2fb5e47ULL, 0x3fef199bdd85529cULL, 0x3fef3720dcef9069ULL,
    0x3fef5818dcfba487ULL, 0x3fef7c97337b9b5fULL, 0x3fefa4afa2a490daULL, 0x3fefd0765b6e4540ULL};
// the same 2^(j/32) as a float pair (high part, next 24 bits)
static __device__ const float2 kTabF[32] = {
    {0x1.000000p+0f, 0.0f},           {0x1.059b0ep+0f, -0x1.9d4f52p-25f}, {0x1.0b5586p+0f, 0x1.9f3122p-25f},
    {0x1.11301ep+0f, -0x1.fdb496p-25f}, {0x1.172b84p+0f, -0x1.c15742p-27f}, {0x1.1d4874p+0f, -0x1.d2e8cap-25f},
    {0x1.2387a6p+0f, 0x1.ceac48p-25f},  {0x1.29e9e0p+0f, -0x1.5c0424p-25f}, {0x1.306fe0p+0f, 0x1.4636e2p-25f},
    {0x1.371a74p+0f, -0x1.18aac6p-25f}, {0x1.3dea64p+0f, 0x1.824684p-25f},  {0x1.44e086p+0f, 0x1.8624b4p-30f},
    {0x1.4bfdaep+0f, -0x1.593abcp-25f}, {0x1.5342b6p+0f, -0x1.2c5610p-25f}, {0x1.5ab07ep+0f, -0x1.5bd5ecp-27f},
    {0x1.6247ecp+0f, -0x1.f8b550p-25f}, {0x1.6a09e6p+0f, 0x1.9fcef4p-26f},  {0x1.71f75ep+0f, 0x1.1d8beep-25f},
    {0x1.7a1148p+0f, -0x1.829fd0p-25f}, {0x1.82589ap+0f, -0x1.accc7cp-26f}, {0x1.8ace54p+0f, 0x1.15506ep-27f},
    {0x1.93737cp+0f, -0x1.e64744p-25f}, {0x1.9c4918p+0f, 0x1.51f848p-27f},  {0x1.a5503cp+0f, -0x1.b83b54p-25f},
    {0x1.ae89fap+0f, -0x1.a94b14p-26f}, {0x1.b7f770p+0f, -0x1.a09438p-25f}, {0x1.c199bep+0f, -0x1.3d56b2p-27f},
    {0x1.cb720ep+0f, -0x1.8837ccp-27f}, {0x1.d5818ep+0f, -0x1.822dbcp-27f}, {0x1.dfc974p+0f, -0x1.908c94p-25f},
    {0x1.ea4afap+0f, 0x1.52486cp-27f},  {0x1.f50766p+0f, -0x1.246eb0p-26f}};
constexpr double kInvLn2N = 0x1.71547652b82fep+0 * 32.0;
constexpr double kShift = 0x1.8p+52;
constexpr double kC0 = 0x1.c6af84b912394p-20, kC1 = 0x1.ebfce50fac4f3p-13, kC2 = 0x1.62e42ff0c52d6p-6;
constexpr float kLo = -0x1.9fe368p6f;  // below: the result rounds to 0 (log 2^-150)
constexpr float kHi = 0x1.62e42ep6f;   // above: +inf (log 2^128)
// float splits: kInvLn2N = kIH + kIM + kIL exactly; kCi = kCiH + kCiM (+ < 2^-48 relative)
constexpr float kIH = 0x1.715476p+5f, kIM = 0x1.4ae0c0p-21f, kIL = -0x1p-46f;
constexpr float kC0H = 0x1.c6af84p-20f, kC0M = 0x1.722472p-45f;
constexpr float kC1H = 0x1.ebfce6p-13f, kC1M = -0x1.e0a762p-38f;
constexpr float kC2H = 0x1.62e430p-6f, kC2M = -0x1.e75a54p-35f;
constexpr float kWindow = 0x1p-40f;

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}
}  // namespace expf_detail

// The C library's double-precision sequence, operation for operation.
static __device__ __noinline__ float expf_double(float x) {
  using namespace expf_detail;
  if (!(x >= kLo)) return x != x ? __fadd_rn(x, x) : 0.0f;
  if (x > kHi) return __int_as_float(0x7f800000);
  const double xd = static_cast<double>(x);
  const double z = __dmul_rn(kInvLn2N, xd);
  double kd = __dadd_rn(z, kShift);
  const unsigned long long ki = static_cast<unsigned long long>(__double_as_longlong(kd));
  kd = __dsub_rn(kd, kShift);
  const double r = __fma_rn(kInvLn2N, xd, -kd);
  const double s = __longlong_as_double(static_cast<long long>(kTab[ki % 32] + (ki << 47)));
  const double c = __fma_rn(kC0, r, kC1);
  const double r2 = __dmul_rn(r, r);
  double y = __fma_rn(kC2, r, 1.0);
  y = __fma_rn(c, r2, y);
  y = __dmul_rn(y, s);
  return __double2float_rn(y);
}

__device__ __forceinline__ float vh_expf(float x) {
  using namespace expf_detail;
  if (!(x >= kLo && x <= kHi)) return expf_double(x);
  // P = x * 32/ln2 exactly, as p0 + e0 + p1 + e1 + p2 (the last product's rounding is below 2^-59)
  float p0, e0, p1, e1;
  two_prod(x, kIH, p0, e0);
  two_prod(x, kIM, p1, e1);
  const float p2 = __fmul_rn(x, kIL);
  float k = rintf(p0);
  float s1, t1, rh, rl;
  two_sum(e0, p1, s1, t1);
  two_sum(__fsub_rn(p0, k), s1, rh, rl);  // p0 - k is exact
  rl = __fadd_rn(rl, __fadd_rn(__fadd_rn(t1, e1), p2));
  // k = the nearest integer to P; P within 2^-20 of a half-integer: the double sequence decides the tie
  if (fabsf(__fsub_rn(fabsf(rh), 0.5f)) < 0x1p-20f) return expf_double(x);
  if (rh > 0.5f) {
    k = __fadd_rn(k, 1.0f);
    rh = __fsub_rn(rh, 1.0f);
  } else if (rh < -0.5f) {
    k = __fsub_rn(k, 1.0f);
    rh = __fadd_rn(rh, 1.0f);
  }
  // q = C2 r + C1 r^2 + C0 r^3 = r (C2 + r (C1 + r C0)), float-float
  float t, te, vh, vl, m, me, wh, wl, qh, ql;
  two_prod(kC0H, rh, t, te);
  te = __fmaf_rn(kC0H, rl, __fmaf_rn(kC0M, rh, te));
  two_sum(kC1H, t, vh, vl);
  vl = __fadd_rn(vl, __fadd_rn(te, kC1M));
  two_prod(rh, vh, m, me);
  me = __fmaf_rn(rh, vl, __fmaf_rn(rl, vh, me));
  fast_two_sum(kC2H, m, wh, wl);
  wl = __fadd_rn(wl, __fadd_rn(me, kC2M));
  two_prod(rh, wh, qh, ql);
  ql = __fmaf_rn(rh, wl, __fmaf_rn(rl, wh, ql));
  // Z = 2^(j/32) (1 + q), result = Z * 2^e with k = 32 e + j
  const int ki = static_cast<int>(k);
  const int e = ki >> 5;
  const float2 T = kTabF[ki & 31];
  float zh1, zl1, Zh, Zl;
  two_prod(T.x, qh, zh1, zl1);
  zl1 = __fadd_rn(zl1, __fmaf_rn(T.x, ql, __fmaf_rn(T.y, qh, T.y)));
  fast_two_sum(T.x, zh1, Zh, Zl);
  fast_two_sum(Zh, __fadd_rn(Zl, zl1), Zh, Zl);
  const uint32_t zb = __float_as_uint(Zh);
  const int ez = static_cast<int>(zb >> 23) - 127;
  if (ez + e >= -126) {  // normal result: Zh unless Z lies within the window of a rounding boundary
    const float ulp_up = __uint_as_float(static_cast<uint32_t>(ez + 104) << 23);
    const float ulp_dn = (zb & 0x7fffffU) == 0U ? __fmul_rn(ulp_up, 0.5f) : ulp_up;
    const float half = __fmul_rn(0.5f, Zl >= 0.0f ? ulp_up : ulp_dn);
    if (__fsub_rn(half, fabsf(Zl)) <= kWindow) return expf_double(x);
    return __uint_as_float(zb + (static_cast<uint32_t>(e) << 23));
  }
  // subnormal result: round Z * 2^(149 + e) to an integer n, the result's bit pattern
  const float f = __uint_as_float(static_cast<uint32_t>(149 + e + 127) << 23);
  const float zsh = __fmul_rn(Zh, f);
  float n = rintf(zsh);
  const float frac = __fadd_rn(__fsub_rn(zsh, n), __fmul_rn(Zl, f));
  if (fabsf(__fsub_rn(fabsf(frac), 0.5f)) <= __fmul_rn(kWindow, f)) return expf_double(x);
  if (frac > 0.5f) n = __fadd_rn(n, 1.0f);
  else if (frac < -0.5f) n = __fsub_rn(n, 1.0f);
  return __uint_as_float(static_cast<uint32_t>(static_cast<int>(n)));
}

// x / 65535.0f for x in {0, 1, ..., 65535}: reciprocal multiply plus one fused correction step (Markstein's
// method).  Equal to the IEEE quotient on all 65536 inputs (checked exhaustively on the host), at 3 instructions.
__device__ __forceinline__ float div65535(float x) {
  const float inv = 1.0f / 65535.0f;
  const float q = x * inv;
  return __fmaf_rn(__fmaf_rn(-q, 65535.0f, x), inv, q);
}

// cuda_tsdf_integrator.cu:173-179.  The fast-math build of the update pass (VH_FAST_MATH) uses the hardware
// exponential instead.
#ifdef VH_FAST_MATH
__device__ __forceinline__ float gaussian(float sq, float k) { return __expf(-sq * k); }
#else
__device__ __forceinline__ float gaussian(float sq, float k) { return vh_expf(-sq * k); }
#endif
__device__ __forceinline__ float disc_threshold(const Params& p, float ref) {
  return fmaxf(p.disc_base, p.disc_rel * fmaxf(ref, 0.0f));
}
// cuda_tsdf_integrator.cu:219-226
__device__ __forceinline__ f3 orient_toward_camera(f3 n, f3 pc) {
  if (norm3(n) <= 1e-6f || norm3(pc) <= 1e-6f) return n;
  const f3 view = normalize3(pc);
  return dot3(n, view) > 0.0f ? mul3(n, -1.0f) : n;
}
// The same for an n that already passed norm3(n) > 1e-6 (a normalised base normal): norm3(n) is recomputed
// from the same components, so the first test is known to be false and is skipped.
__device__ __forceinline__ f3 orient_unit_toward_camera(f3 n, f3 pc) {
  if (norm3(pc) <= 1e-6f) return n;
  const f3 view = normalize3(pc);
  return dot3(n, view) > 0.0f ? mul3(n, -1.0f) : n;
}

// unpackNormalOctahedralGpu of the mesh extractor (cuda_mesh_extractor.cu:237-257): degenerate -> (0,0,1)
__device__ __forceinline__ f3 unpack_normal_mesh(uint32_t packed) {
  f3 n = mk3(div65535(static_cast<float>(packed & 0xffffU)) * 2.0f - 1.0f,
             div65535(static_cast<float>((packed >> 16U) & 0xffffU)) * 2.0f - 1.0f, 0.0f);
  n.z = 1.0f - fabsf(n.x) - fabsf(n.y);
  if (n.z < 0.0f) {
    const float fx = (1.0f - fabsf(n.y)) * (n.x >= 0.0f ? 1.0f : -1.0f);
    const float fy = (1.0f - fabsf(n.x)) * (n.y >= 0.0f ? 1.0f : -1.0f);
    n.x = fx;
    n.y = fy;
  }
  const float len = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
  if (len <= 1e-6f) return mk3(0.0f, 0.0f, 1.0f);
  const float inv = 1.0f / len;
  return mk3(n.x * inv, n.y * inv, n.z * inv);
}

// cuda_block_allocator.cu:153-159
__device__ __forceinline__ uint32_t hash_block_key(int x, int y, int z) {
  uint32_t seed = 0U;
  // unsigned multiply: the same bits as the reference's wrapping int product, without signed overflow
  seed ^= static_cast<uint32_t>(x) * 73856093U + 0x9e3779b9U + (seed << 6U) + (seed >> 2U);
  seed ^= static_cast<uint32_t>(y) * 19349663U + 0x9e3779b9U + (seed << 6U) + (seed >> 2U);
  seed ^= static_cast<uint32_t>(z) * 83492791U + 0x9e3779b9U + (seed << 6U) + (seed >> 2U);
  return seed;
}
// cuda_block_allocator.cu:161-174
__device__ __forceinline__ bool pack_block_key(int x, int y, int z, unsigned long long& packed) {
  if (x < -kKeyBias || x > kKeyBias - 1 || y < -kKeyBias || y > kKeyBias - 1 || z < -kKeyBias || z > kKeyBias - 1) {
    return false;
  }
  packed = static_cast<unsigned long long>(x + kKeyBias) |
           (static_cast<unsigned long long>(y + kKeyBias) << kKeyBits) |
           (static_cast<unsigned long long>(z + kKeyBias) << (2 * kKeyBits));
  return true;
}
__device__ __forceinline__ void unpack_block_key(unsigned long long k, int& x, int& y, int& z) {
  x = static_cast<int>(k & kKeyMask) - kKeyBias;
  y = static_cast<int>((k >> kKeyBits) & kKeyMask) - kKeyBias;
  z = static_cast<int>((k >> (2 * kKeyBits)) & kKeyMask) - kKeyBias;
}

// Hash lookup (read-only): pool index of block (x,y,z) or kInvalidBlock.  Probes at most `capacity` slots.
__device__ __forceinline__ uint32_t lookup_block(const Volume& V, int x, int y, int z) {
  unsigned long long key;
  if (!pack_block_key(x, y, z, key)) return kInvalidBlock;
  uint32_t slot = hash_block_key(x, y, z) & V.mask;
  for (uint32_t probe = 0; probe < V.capacity; ++probe) {
    const unsigned long long cur = V.slot_keys[slot];
    if (cur == key) return V.slot_block[slot];
    if (cur == kEmptyKey) return kInvalidBlock;
    slot = (slot + 1U) & V.mask;
  }
  return kInvalidBlock;
}

// float4 index of layer l of voxel li, direction d, block b
__device__ __forceinline__ size_t layer_index(uint32_t b, int d, int li, int l) {
  return ((static_cast<size_t>(b) * kDirs + d) * kBlockVoxels + li) * kLayers + l;
}

// ---- FP16 layer storage (vh_params.layer_format 1) ----
//
// One (block, direction, voxel) bin is 32 bytes, two uint4 words:
//   A = {w0 | s0 << 16, p0 | w1 << 16, s1 | p1 << 16, w2 | s2 << 16},  B = {p2, n0, n1, n2}
// per layer l: w = weight (binary16), n = the octahedral normal word of the FP32 record (unchanged),
// s = (surface_coord - c_d) / voxel_size and p = (plane_offset - dot(bin_normal(n), c)) / voxel_size
// (binary16), c the voxel centre and c_d its coordinate along the bin's direction.  Coordinates are stored
// relative to the voxel they belong to because absolute world metres would have a 4 mm binary16 step at
// 4 m; relative to the voxel, |s|, |p| stay below a few truncation distances and the step is <= 1/64 voxel.
// Empty layers are all-zero.  The update arithmetic stays FP32: a bin is decoded to three FP32 records,
// updated, and encoded back.  The codec's products and sums are explicit round-to-nearest intrinsics; its
// normalisation is the correctly rounded reciprocal square root in the exact compile, which a host restatement
// (the oracle's layer_format 1) reproduces bit for bit, and the hardware one in the fast-math compile.
constexpr int kBinWords16 = 2;

__device__ __forceinline__ size_t bin16_index(uint32_t b, int d, int li) {
  return ((static_cast<size_t>(b) * kDirs + d) * kBlockVoxels + li) * kBinWords16;
}

// voxel centre in world coordinates, ((block * 8 + local) + 0.5) * voxel_size per axis
__device__ __forceinline__ f3 voxel_centre(const int4& bk, int li, float vs) {
  const int lx = li & 7, ly = (li >> 3) & 7, lz = li >> 6;
  return mk3(__fmul_rn(__fadd_rn(static_cast<float>(bk.x * kBlockSide + lx), 0.5f), vs),
             __fmul_rn(__fadd_rn(static_cast<float>(bk.y * kBlockSide + ly), 0.5f), vs),
             __fmul_rn(__fadd_rn(static_cast<float>(bk.z * kBlockSide + lz), 0.5f), vs));
}

__device__ __forceinline__ float axis_coordinate(f3 p, int d) {
  const float a = (d >> 1) == 0 ? p.x : ((d >> 1) == 1 ? p.y : p.z);
  return (d & 1) ? -a : a;
}

// octahedral decode of a packed normal word, normalised (the codec's reference direction for p)
__device__ __forceinline__ f3 bin_normal(uint32_t packed) {
  float x = __fadd_rn(__fmul_rn(div65535(static_cast<float>(packed & 0xffffU)), 2.0f), -1.0f);
  float y = __fadd_rn(__fmul_rn(div65535(static_cast<float>(packed >> 16U)), 2.0f), -1.0f);
  const float z = __fadd_rn(__fadd_rn(1.0f, -fabsf(x)), -fabsf(y));
  if (z < 0.0f) {
    const float fx = copysignf(__fadd_rn(1.0f, -fabsf(y)), x >= 0.0f ? 1.0f : -1.0f);
    const float fy = copysignf(__fadd_rn(1.0f, -fabsf(x)), y >= 0.0f ? 1.0f : -1.0f);
    x = fx;
    y = fy;
  }
  // |(x, y, z)|_1 = 1, so the squared length is in [1/3, 1]: no degenerate case.  The exact compile uses the
  // correctly rounded reciprocal square root (reproducible on a host: the oracle's layer_format 1); the
  // fast-math compile the hardware one (4.5 % of the fused update's time), which moves a decoded plane offset
  // by about one unit in the last place of the normal times |c|, well below the FP16 step.
#ifdef VH_FAST_MATH
  const float inv = rsqrtf(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
#else
  const float inv = __frsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
#endif
  return mk3(__fmul_rn(x, inv), __fmul_rn(y, inv), __fmul_rn(z, inv));
}

__device__ __forceinline__ float dot_rn(f3 a, f3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}

__device__ __forceinline__ float h2f(uint32_t h) { return __half2float(__ushort_as_half(static_cast<uint16_t>(h))); }
__device__ __forceinline__ uint32_t f2h(float x) { return __half_as_ushort(__float2half_rn(x)); }

// layer record from its binary16 triplet (n: unit normal of the packed word, from bin_normal)
__device__ __forceinline__ float4 decode_layer16(uint32_t w, uint32_t s, uint32_t p, uint32_t packed, f3 n, f3 c,
                                                 float cd, float vs) {
  return make_float4(h2f(w), __fadd_rn(cd, __fmul_rn(h2f(s), vs)), __fadd_rn(dot_rn(n, c), __fmul_rn(h2f(p), vs)),
                     __uint_as_float(packed));
}

// binary16 triplet of an observed layer record, packed as w | s << 16 and p
__device__ __forceinline__ void encode_layer16(const float4& L, f3 n, f3 c, float cd, float inv_vs, uint32_t& ws,
                                               uint32_t& p) {
  uint32_t w = f2h(L.x);
  if (w == 0U) w = 1U;  // a positive weight below the binary16 range keeps the layer observed
  ws = w | (f2h(__fmul_rn(__fadd_rn(L.y, -cd), inv_vs)) << 16);
  p = f2h(__fmul_rn(__fadd_rn(L.z, -dot_rn(n, c)), inv_vs));
}

__device__ __forceinline__ void decode_bin16(const uint4& A, const uint4& B, f3 c, int d, float vs, float4& L0,
                                             float4& L1, float4& L2) {
  const float cd = axis_coordinate(c, d);
  const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  L0 = (A.x & 0xffffU) ? decode_layer16(A.x & 0xffffU, A.x >> 16, A.y & 0xffffU, B.y, bin_normal(B.y), c, cd, vs) : z;
  L1 = (A.y >> 16) ? decode_layer16(A.y >> 16, A.z & 0xffffU, A.z >> 16, B.z, bin_normal(B.z), c, cd, vs) : z;
  L2 = (A.w & 0xffffU) ? decode_layer16(A.w & 0xffffU, A.w >> 16, B.x & 0xffffU, B.w, bin_normal(B.w), c, cd, vs) : z;
}

__device__ __forceinline__ void encode_bin16(const float4& L0, const float4& L1, const float4& L2, f3 c, int d,
                                             float inv_vs, uint4& A, uint4& B) {
  const float cd = axis_coordinate(c, d);
  uint32_t ws[3] = {0U, 0U, 0U}, pp[3] = {0U, 0U, 0U}, nn[3] = {0U, 0U, 0U};
  const float4* L[3] = {&L0, &L1, &L2};
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    if (L[l]->x > 0.0f) {
      nn[l] = __float_as_uint(L[l]->w);
      encode_layer16(*L[l], bin_normal(nn[l]), c, cd, inv_vs, ws[l], pp[l]);
    }
  }
  A = make_uint4(ws[0], pp[0] | ((ws[1] & 0xffffU) << 16), (ws[1] >> 16) | (pp[1] << 16), ws[2]);
  B = make_uint4(pp[2], nn[0], nn[1], nn[2]);
}

// the three layer records of one bin, in the FP32 record form, whichever storage the volume uses
__device__ __forceinline__ void load_bin(const Volume& V, uint32_t b, int d, int li, const int4& bk, float vs,
                                         float4& L0, float4& L1, float4& L2) {
  if (V.layers16 == nullptr) {
    const float4* base = V.layers + layer_index(b, d, li, 0);
    L0 = base[0];
    L1 = base[1];
    L2 = base[2];
    return;
  }
  const uint4* q = V.layers16 + bin16_index(b, d, li);
  decode_bin16(q[0], q[1], voxel_centre(bk, li, vs), d, vs, L0, L1, L2);
}

__device__ __forceinline__ void store_bin(const Volume& V, uint32_t b, int d, int li, const int4& bk, float vs,
                                          const float4& L0, const float4& L1, const float4& L2) {
  if (V.layers16 == nullptr) {
    float4* base = V.layers + layer_index(b, d, li, 0);
    base[0] = L0;
    base[1] = L1;
    base[2] = L2;
    return;
  }
  uint4 A, B;
  encode_bin16(L0, L1, L2, voxel_centre(bk, li, vs), d, V.inv_voxel_size, A, B);
  uint4* q = V.layers16 + bin16_index(b, d, li);
  q[0] = A;
  q[1] = B;
}

// any layer of the bin observed (weight > 0)
__device__ __forceinline__ bool bin_observed(const Volume& V, uint32_t b, int d, int li) {
  if (V.layers16 == nullptr) {
    const float4* L = V.layers + layer_index(b, d, li, 0);
    return L[0].x > 0.0f || L[1].x > 0.0f || L[2].x > 0.0f;
  }
  const uint4 A = V.layers16[bin16_index(b, d, li)];
  return (A.x & 0xffffU) != 0U || (A.y >> 16) != 0U || (A.w & 0xffffU) != 0U;
}

}  // namespace vh
