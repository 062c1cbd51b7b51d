// vh_weld.cu -- the indexed mesh of a marching-cubes triangle soup, built on the device.
//
// The directional multi-layer marching cubes computes the vertex of an edge separately in each cell that
// uses it (from that cell's cluster centres, src/cuda_mesh_extractor.cu:358-437), so two soup vertices are
// the same point exactly when their float32 coordinates are bit-identical; the weld merges those and nothing
// else.  Vertices are numbered in the order of their first use in the soup, faces keep the soup's order, and a
// face is dropped when two of its vertices merged or its area test fails: |cross(v1 - v0, v2 - v0)| <= 1e-8 in
// float32, the test of the reference's PLY writer (src/main.cpp:337-398).  The result is deterministic.
//
// 1. weld_insert_kernel: every soup vertex goes into an open-addressing table keyed by its 96 coordinate bits;
//    a slot keeps the smallest soup index of its key (atomicMin), each vertex remembers its slot.
// 2. weld_first_kernel flags the first use of each key; an exclusive scan of the flags numbers the vertices.
// 3. weld_vertex_kernel gives every soup vertex its key's number and writes the vertex array.
// 4. weld_face_flag_kernel flags the faces kept; a scan places them; weld_face_kernel writes them.
//
// The scan is three kernels: per-tile sums, one CTA scanning the tile sums, and per-tile scans with the
// tile's carry.  Every index is 32-bit: the host limits a weld to fewer than 2^30 soup vertices (the table
// to at most 2^31 slots).
#include "vh_common.cuh"
#include "vh_kernels.h"

namespace vh {
namespace {

constexpr uint32_t kEmptySlot = 0xFFFFFFFFu;
constexpr int kWeldThreads = 256;
constexpr int kScanThreads = 1024;
constexpr int kScanPerThread = 4;
constexpr uint32_t kScanTile = kScanThreads * kScanPerThread;

// hash of a vertex's three coordinate words: a multiplicative combine, then the MurmurHash3 32-bit finaliser
__device__ __forceinline__ uint32_t vertex_hash(uint32_t x, uint32_t y, uint32_t z) {
  uint32_t h = x * 0x9E3779B1u;
  h ^= y * 0x85EBCA77u + 0x7F4A7C15u + (h << 6) + (h >> 2);
  h ^= z * 0xC2B2AE3Du + 0x7F4A7C15u + (h << 6) + (h >> 2);
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}

__device__ __forceinline__ bool same_vertex(const float* __restrict__ tris, uint32_t r, uint32_t x, uint32_t y,
                                            uint32_t z) {
  return __float_as_uint(tris[3 * static_cast<size_t>(r)]) == x &&
         __float_as_uint(tris[3 * static_cast<size_t>(r) + 1]) == y &&
         __float_as_uint(tris[3 * static_cast<size_t>(r) + 2]) == z;
}

// Slots only ever hold soup indices of one key once non-empty, so a stale read of an occupied slot still
// compares correctly, and a stale empty read is corrected by the compare-and-swap.  A table of more than nv
// slots cannot fill; the probe count is bounded by its size (at most 2^31 slots) all the same.
__global__ void __launch_bounds__(kWeldThreads) weld_insert_kernel(const float* __restrict__ tris, uint32_t nv,
                                                                   uint32_t* __restrict__ slot_first, uint32_t mask,
                                                                   uint32_t* __restrict__ vslot,
                                                                   uint32_t* __restrict__ error) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
    const uint32_t x = __float_as_uint(tris[3 * static_cast<size_t>(i)]);
    const uint32_t y = __float_as_uint(tris[3 * static_cast<size_t>(i) + 1]);
    const uint32_t z = __float_as_uint(tris[3 * static_cast<size_t>(i) + 2]);
    uint32_t s = vertex_hash(x, y, z) & mask;
    bool placed = false;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
      uint32_t r = slot_first[s];
      if (r == kEmptySlot) {
        r = atomicCAS(&slot_first[s], kEmptySlot, i);
        if (r == kEmptySlot) {
          placed = true;
          break;
        }
      }
      if (same_vertex(tris, r, x, y, z)) {
        if (i < r) atomicMin(&slot_first[s], i);
        placed = true;
        break;
      }
      s = (s + 1U) & mask;
    }
    if (placed) {
      vslot[i] = s;
    } else {
      vslot[i] = 0U;
      atomicOr(error, 1U);
    }
  }
}

__global__ void __launch_bounds__(kWeldThreads) weld_first_kernel(uint32_t nv, const uint32_t* __restrict__ slot_first,
                                                                  const uint32_t* __restrict__ vslot,
                                                                  uint32_t* __restrict__ flags) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
    flags[i] = slot_first[vslot[i]] == i ? 1U : 0U;
  }
}

__global__ void __launch_bounds__(kWeldThreads) weld_vertex_kernel(const float* __restrict__ tris, uint32_t nv,
                                                                   const uint32_t* __restrict__ slot_first,
                                                                   const uint32_t* __restrict__ vslot,
                                                                   const uint32_t* __restrict__ number,
                                                                   uint32_t* __restrict__ vid,
                                                                   float* __restrict__ verts) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
    const uint32_t first = slot_first[vslot[i]];
    vid[i] = number[first];
    if (first == i) {
      const size_t o = 3 * static_cast<size_t>(number[i]);
      verts[o] = tris[3 * static_cast<size_t>(i)];
      verts[o + 1] = tris[3 * static_cast<size_t>(i) + 1];
      verts[o + 2] = tris[3 * static_cast<size_t>(i) + 2];
    }
  }
}

// a face is kept when its three vertex numbers differ and sqrt(cross . cross) > 1e-8, every operation rounded
// to float32 in the order (x*x + y*y) + z*z (no contraction)
__device__ __forceinline__ bool face_kept(const float* __restrict__ tris, const uint32_t* __restrict__ vid,
                                          uint32_t t) {
  const uint32_t a = vid[3 * static_cast<size_t>(t)], b = vid[3 * static_cast<size_t>(t) + 1],
                 c = vid[3 * static_cast<size_t>(t) + 2];
  if (a == b || b == c || a == c) return false;
  const float* q = tris + 9 * static_cast<size_t>(t);
  const float e1x = __fsub_rn(q[3], q[0]), e1y = __fsub_rn(q[4], q[1]), e1z = __fsub_rn(q[5], q[2]);
  const float e2x = __fsub_rn(q[6], q[0]), e2y = __fsub_rn(q[7], q[1]), e2z = __fsub_rn(q[8], q[2]);
  const float cx = __fsub_rn(__fmul_rn(e1y, e2z), __fmul_rn(e1z, e2y));
  const float cy = __fsub_rn(__fmul_rn(e1z, e2x), __fmul_rn(e1x, e2z));
  const float cz = __fsub_rn(__fmul_rn(e1x, e2y), __fmul_rn(e1y, e2x));
  const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)), __fmul_rn(cz, cz)));
  return len > 1e-8f;
}

__global__ void __launch_bounds__(kWeldThreads) weld_face_flag_kernel(const float* __restrict__ tris, uint32_t nt,
                                                                      const uint32_t* __restrict__ vid,
                                                                      uint32_t* __restrict__ flags) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    flags[t] = face_kept(tris, vid, t) ? 1U : 0U;
  }
}

__global__ void __launch_bounds__(kWeldThreads) weld_face_kernel(uint32_t nt, const uint32_t* __restrict__ vid,
                                                                 const uint32_t* __restrict__ flags,
                                                                 const uint32_t* __restrict__ position,
                                                                 int32_t* __restrict__ faces) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    if (flags[t]) {
      const size_t o = 3 * static_cast<size_t>(position[t]);
      faces[o] = static_cast<int32_t>(vid[3 * static_cast<size_t>(t)]);
      faces[o + 1] = static_cast<int32_t>(vid[3 * static_cast<size_t>(t) + 1]);
      faces[o + 2] = static_cast<int32_t>(vid[3 * static_cast<size_t>(t) + 2]);
    }
  }
}

// exclusive scan of one value per thread over the CTA (kScanThreads threads); *total = the CTA's sum.
// s_warp: 33 words of shared memory, free again when the call returns.
__device__ __forceinline__ uint32_t cta_exclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffU, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = s_warp[lane];  // kScanThreads / 32 = 32 warps
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffU, wi, o);
      if (lane >= o) wi += t;
    }
    s_warp[lane] = wi - w;
    if (lane == 31) s_warp[32] = wi;
  }
  __syncthreads();
  const uint32_t res = s_warp[warp] + incl - v;
  *total = s_warp[32];
  __syncthreads();
  return res;
}

static_assert(kScanThreads == 32 * 32, "the CTA scan keeps one warp total per lane of warp 0");

__global__ void __launch_bounds__(kScanThreads) scan_tile_sums_kernel(const uint32_t* __restrict__ in, uint32_t n,
                                                                      uint32_t* __restrict__ sums) {
  __shared__ uint32_t s_warp[33];
  const size_t base = static_cast<size_t>(blockIdx.x) * kScanTile;
  uint32_t v = 0U;
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
    const size_t i = base + static_cast<size_t>(k) * kScanThreads + threadIdx.x;
    if (i < n) v += in[i];
  }
  uint32_t total;
  cta_exclusive_scan(v, s_warp, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(uint32_t* __restrict__ sums, uint32_t ntiles,
                                                                 uint32_t* __restrict__ total_out) {
  __shared__ uint32_t s_warp[33];
  uint32_t carry = 0U;
  for (uint32_t start = 0; start < ntiles; start += kScanThreads) {
    const uint32_t i = start + threadIdx.x;
    const uint32_t v = i < ntiles ? sums[i] : 0U;
    uint32_t total;
    const uint32_t ex = cta_exclusive_scan(v, s_warp, &total);
    if (i < ntiles) sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *total_out = carry;
}

__global__ void __launch_bounds__(kScanThreads) scan_tile_apply_kernel(const uint32_t* __restrict__ in, uint32_t n,
                                                                       const uint32_t* __restrict__ sums,
                                                                       uint32_t* __restrict__ out) {
  __shared__ uint32_t s_warp[33];
  const size_t base = static_cast<size_t>(blockIdx.x) * kScanTile + static_cast<size_t>(threadIdx.x) * kScanPerThread;
  uint32_t v[kScanPerThread];
  uint32_t sum = 0U;
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
    v[k] = base + k < n ? in[base + k] : 0U;
    sum += v[k];
  }
  uint32_t total;
  uint32_t run = sums[blockIdx.x] + cta_exclusive_scan(sum, s_warp, &total);
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

int grid_for(uint32_t n) {
  const uint32_t blocks = (n + kWeldThreads - 1) / kWeldThreads;
  return static_cast<int>(blocks < 152U * 8U ? (blocks > 0U ? blocks : 1U) : 152U * 8U);
}

// exclusive scan of in[0, n) into out; *total = the sum.  sums: scan_tiles(n) words.
cudaError_t scan(const uint32_t* in, uint32_t n, uint32_t* sums, uint32_t* out, uint32_t* total, cudaStream_t s) {
  const uint32_t ntiles = weld_scan_tiles(n);
  scan_tile_sums_kernel<<<ntiles, kScanThreads, 0, s>>>(in, n, sums);
  scan_sums_kernel<<<1, kScanThreads, 0, s>>>(sums, ntiles, total);
  scan_tile_apply_kernel<<<ntiles, kScanThreads, 0, s>>>(in, n, sums, out);
  return cudaGetLastError();
}

}  // namespace

uint32_t weld_scan_tiles(uint32_t n) { return n == 0U ? 1U : (n + kScanTile - 1U) / kScanTile; }

cudaError_t launch_weld(const float* tris, uint32_t ntri, const WeldBuffers& W, cudaStream_t s) {
  const uint32_t nv = 3U * ntri;
  cudaError_t e = cudaMemsetAsync(W.slot_first, 0xFF, (static_cast<size_t>(W.slot_mask) + 1U) * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(W.counts, 0, 3 * sizeof(uint32_t), s);
  if (e != cudaSuccess || ntri == 0U) return e;
  weld_insert_kernel<<<grid_for(nv), kWeldThreads, 0, s>>>(tris, nv, W.slot_first, W.slot_mask, W.vslot,
                                                          W.counts + 2);
  weld_first_kernel<<<grid_for(nv), kWeldThreads, 0, s>>>(nv, W.slot_first, W.vslot, W.flags);
  e = scan(W.flags, nv, W.sums, W.number, W.counts, s);
  if (e != cudaSuccess) return e;
  weld_vertex_kernel<<<grid_for(nv), kWeldThreads, 0, s>>>(tris, nv, W.slot_first, W.vslot, W.number, W.vid,
                                                          W.verts);
  weld_face_flag_kernel<<<grid_for(ntri), kWeldThreads, 0, s>>>(tris, ntri, W.vid, W.flags);
  e = scan(W.flags, ntri, W.sums, W.number, W.counts + 1, s);
  if (e != cudaSuccess) return e;
  weld_face_kernel<<<grid_for(ntri), kWeldThreads, 0, s>>>(ntri, W.vid, W.flags, W.number, W.faces);
  return cudaGetLastError();
}

}  // namespace vh
