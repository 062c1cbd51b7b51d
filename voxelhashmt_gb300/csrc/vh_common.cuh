// vh_common.cuh -- device-side layout, parameters and exact-order math shared by the GB300 kernels.
//
// Every floating-point expression below is written in the operation order of the reference CUDA
// sources (src/cuda_tsdf_integrator.cu, src/cuda_block_allocator.cu, src/cuda_mesh_extractor.cu) and
// the library is compiled with -fmad=false, so each a*b+c rounds twice exactly as the source reads;
// IEEE division and square root are the nvcc defaults (-prec-div=true -prec-sqrt=true).  The only
// deliberate difference from the reference is vh_expf (see below), which makes the plain FP32 form
// reproducible bit-for-bit on the host.
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

// Single-precision exp: Cody-Waite reduction x = k ln2 + r (ln2 split in an 11-trailing-zero high part and a
// low part), e^r by the degree-7 Taylor polynomial in Horner form with fused multiply-adds (|r| <= ln2/2,
// truncation error < 6e-9 relative), scaling by 2^k through the exponent field (two steps below 2^-126).
// The host oracle evaluates the identical fmaf sequence, so results agree bit-for-bit.
__device__ __forceinline__ float vh_expf(float x) {
  if (!(x > -104.0f)) return 0.0f;
  if (x > 0x1.62e42ep+6f) return __int_as_float(0x7f800000);
  const float k = rintf(x * 0x1.715476p+0f);
  float r = __fmaf_rn(k, -0x1.62e400p-1f, x);
  r = __fmaf_rn(k, -0x1.7f7d1cp-20f, r);
  float q = 0x1.a01a02p-13f;
  q = __fmaf_rn(q, r, 0x1.6c16c2p-10f);
  q = __fmaf_rn(q, r, 0x1.111112p-7f);
  q = __fmaf_rn(q, r, 0x1.555556p-5f);
  q = __fmaf_rn(q, r, 0x1.555556p-3f);
  q = __fmaf_rn(q, r, 0x1.000000p-1f);
  q = __fmaf_rn(q, r, 1.0f);
  q = __fmaf_rn(q, r, 1.0f);
  const int ki = static_cast<int>(k);
  if (ki > 127) return (q * __int_as_float((127 + 127) << 23)) * 2.0f;
  if (ki >= -126) return q * __int_as_float((ki + 127) << 23);
  return (q * __int_as_float((ki + 127 + 64) << 23)) * 0x1p-64f;
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
// updated, and encoded back.  The codec's products and sums are explicit round-to-nearest intrinsics and
// its one approximation is the hardware reciprocal square root, so the exact and the fast-math compiles
// encode and decode alike.
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
  // |(x, y, z)|_1 = 1, so the squared length is in [1/3, 1]: no degenerate case
  const float inv = rsqrtf(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
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
