// vh_mesh.cu -- directional multi-layer marching cubes, two passes with block-level prefix sums.
//
// Reference: extractMeshCuda (src/cuda_mesh_extractor.cu:636-720) rebuilds a host lookup table per call and
// runs count + extract kernels once per direction (12 launches, 12 syncs, 6 readbacks); every cell copies
// its 8 corner voxels whole (288 B each) through a device hash lookup, twice.  Here each CTA owns one block:
// it resolves its 7 (+x, +y, +z) neighbour blocks once through the persistent hash, then for each of the 6
// directions stages that direction's bin of the 9x9x9 voxel region (block + one-voxel halo) in shared
// memory with the octahedral normals decoded once per layer, and every thread processes one cell from shared
// memory.  Pass 1 records every cell's triangle count, a scan turns the block totals into offsets, and pass 2
// re-stages only the blocks and directions that produce triangles and evaluates only the cells with a non-zero
// count, writing each block's triangles at its offset: the output is deterministic (block, direction, cell,
// cluster, table order) and needs no atomics.
//
// Per cell the arithmetic is the reference's collectSurfaceClusters / loadCubeForSurface /
// completeCubeValuesWithFallbackGpu / emitCubeTriangles (:259-551) in the same operation order.
#include "vh_common.cuh"
#include "vh_kernels.h"

#define VH_MC_TABLE_QUALIFIER static __constant__
#include "vh_mc_tables.h"

namespace vh {
namespace {

constexpr int kThreads = 512;  // one per cell
constexpr int kSide = 9;
constexpr int kStaged = kSide * kSide * kSide;
constexpr int kMaxCand = 24;  // 8 corners x 3 layers (cuda_mesh_extractor.cu:18)

__constant__ int c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                   {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
__constant__ int c_edge_corners[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                          {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

struct Shared {
  float4 plane[3][kStaged];  // {n.x, n.y, n.z, plane_offset} per layer
  float cand[kMaxCand][kThreads];  // per-thread candidate keys, then cluster centres (thread = fast index)
  uint8_t valid[3][kStaged];
  int8_t tri[256][16];
  uint16_t edge[256];
  uint32_t nbr[8];
  uint32_t warp_sums[kThreads / 32];
  uint32_t total;
};

// planeSignedDistanceGpu (:259-262)
__device__ __forceinline__ float plane_sd(const float4& pl, f3 p) {
  return pl.x * p.x + pl.y * p.y + pl.z * p.z - pl.w;
}

__device__ __forceinline__ int staged_index(int x, int y, int z) { return (z * kSide + y) * kSide + x; }

// FP16 bins: one thread decodes the three layers of a voxel.  Kept out of line so the codec's registers do
// not add to the marching-cubes body's.
__device__ __noinline__ void stage_direction16(Shared& S, const Volume& V, float vs, int d, int tid) {
  for (int vi = tid; vi < kStaged; vi += kThreads) {
    const int sx = vi % kSide, sy = (vi / kSide) % kSide, sz = vi / (kSide * kSide);
    const uint32_t nb = S.nbr[(sx >> 3) | ((sy >> 3) << 1) | ((sz >> 3) << 2)];
    float4 L[kLayers] = {make_float4(0.0f, 0.0f, 0.0f, 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f),
                         make_float4(0.0f, 0.0f, 0.0f, 0.0f)};
    if (nb != kInvalidBlock) {
      const int li = (sx & 7) + kBlockSide * ((sy & 7) + kBlockSide * (sz & 7));
      load_bin(V, nb, d, li, V.block_keys[nb], vs, L[0], L[1], L[2]);
    }
#pragma unroll
    for (int l = 0; l < kLayers; ++l) {
      float4 pl = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      const bool ok = L[l].x > 0.0f;
      if (ok) {
        const f3 n = unpack_normal_mesh(__float_as_uint(L[l].w));
        pl = make_float4(n.x, n.y, n.z, L[l].z);
      }
      S.plane[l][vi] = pl;
      S.valid[l][vi] = ok ? 1 : 0;
    }
  }
}

__device__ void stage_direction(Shared& S, const Volume& V, const Params& p, int d, int tid) {
  if (V.layers16 != nullptr) {
    stage_direction16(S, V, p.voxel_size, d, tid);
    return;
  }
  for (int i = tid; i < kStaged * kLayers; i += kThreads) {
    const int l = i % kLayers;
    const int vi = i / kLayers;
    const int sx = vi % kSide, sy = (vi / kSide) % kSide, sz = vi / (kSide * kSide);
    const uint32_t nb = S.nbr[(sx >> 3) | ((sy >> 3) << 1) | ((sz >> 3) << 2)];
    float4 pl = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint8_t ok = 0;
    if (nb != kInvalidBlock) {
      const int li = (sx & 7) + kBlockSide * ((sy & 7) + kBlockSide * (sz & 7));
      const float4 L = V.layers[layer_index(nb, d, li, l)];
      if (L.x > 0.0f) {
        const f3 n = unpack_normal_mesh(__float_as_uint(L.w));
        pl = make_float4(n.x, n.y, n.z, L.z);
        ok = 1;
      }
    }
    S.plane[l][vi] = pl;
    S.valid[l][vi] = ok;
  }
}

// interpolateVertexGpu (:358-374)
__device__ __forceinline__ f3 interp(f3 p0, f3 p1, float v0, float v1, float iso) {
  const float delta = v1 - v0;
  if (fabsf(delta) < 1e-6f) return p0;
  const float t = fminf(1.0f, fmaxf(0.0f, (iso - v0) / delta));
  return mk3(p0.x + (p1.x - p0.x) * t, p0.y + (p1.y - p0.y) * t, p0.z + (p1.z - p0.z) * t);
}

// value k of an 8-value register array, selected without indexing it (a run-time index would move the array
// to local memory)
__device__ __forceinline__ float pick8(const float (&a)[8], int k) {
  float r = a[0];
#pragma unroll
  for (int i = 1; i < 8; ++i) r = k == i ? a[i] : r;
  return r;
}

// corner k of the cell at grid (gx, gy, gz): ((g + corner) + 0.5) * vs per axis (loadCubeForSurface, :276-303)
__device__ __forceinline__ f3 corner_pos(int gx, int gy, int gz, int k, float vs) {
  return mk3((static_cast<float>(gx + c_corner[k][0]) + 0.5f) * vs, (static_cast<float>(gy + c_corner[k][1]) + 0.5f) * vs,
             (static_cast<float>(gz + c_corner[k][2]) + 0.5f) * vs);
}

// One cell of one direction: returns its triangle count; with kEmit writes them to out (9 floats each).
template <bool kEmit>
__device__ int process_cell(const Shared& S, const Params& p, int gx, int gy, int gz, int lx, int ly, int lz, int t,
                            float* __restrict__ out) {
  const float vs = p.voxel_size;
  const f3 cc = mk3((static_cast<float>(gx) + 1.0f) * vs, (static_cast<float>(gy) + 1.0f) * vs,
                    (static_cast<float>(gz) + 1.0f) * vs);
  const int s0 = staged_index(lx, ly, lz);
  // staged index of corner k: s0 + (dx + 9 dy + 81 dz)
  auto si = [&](int k) { return s0 + c_corner[k][0] + kSide * c_corner[k][1] + kSide * kSide * c_corner[k][2]; };

  // collectSurfaceClusters (:439-507); candidates in shared memory, column `t` of S.cand
  float* cand = const_cast<float*>(&S.cand[0][0]) + t;
  int nc = 0;
  float nearest = 3.0e38f;  // smallest |candidate - iso|
#pragma unroll
  for (int k = 0; k < 8; ++k) {
#pragma unroll
    for (int l = 0; l < kLayers; ++l) {
      if (S.valid[l][si(k)]) {
        const float c = plane_sd(S.plane[l][si(k)], cc);
        cand[nc * kThreads] = c;
        nearest = fminf(nearest, fabsf(c - p.iso));
        ++nc;
      }
    }
  }
  if (nc == 0) return 0;
  // Every corner value below is a candidate's plane evaluated at a corner, at most sqrt(3)/2 voxel from the
  // cell centre, so it has the candidate's sign relative to iso when the candidate is farther than that (plus
  // a rounding margin for the two float evaluations); means of same-sign values keep the sign.  Such a cell
  // has cube index 0 or 255 for every cluster: no triangles, skipped without changing the output.
  const float reject = 0.8660254f * vs * 1.00001f + 1e-5f * (1.0f + fabsf(cc.x) + fabsf(cc.y) + fabsf(cc.z));
  if (nearest > reject) return 0;
  for (int i = 1; i < nc; ++i) {  // insertion sort (:264-274)
    const float x = cand[i * kThreads];
    int j = i - 1;
    while (j >= 0 && cand[j * kThreads] > x) {
      cand[(j + 1) * kThreads] = cand[j * kThreads];
      --j;
    }
    cand[(j + 1) * kThreads] = x;
  }
  // greedy clustering with running means; centre c is written to slot c <= i after slot i has been read,
  // and only the last cluster's size is ever used
  const float tol = p.extract_tol;
  int ncl = 0;
  int last_size = 0;
  for (int i = 0; i < nc; ++i) {
    const float key = cand[i * kThreads];
    if (ncl == 0 || fabsf(key - cand[(ncl - 1) * kThreads]) > tol) {
      cand[ncl * kThreads] = key;
      last_size = 1;
      ++ncl;
      continue;
    }
    const int last = ncl - 1;
    cand[last * kThreads] = (cand[last * kThreads] * static_cast<float>(last_size) + key) /
                            static_cast<float>(last_size + 1);
    last_size += 1;
  }

  // A cluster's corner values are planes within tol of its key at the cell centre, evaluated at most sqrt(3)/2
  // voxel away (and means of such values): a key farther than tol + that from iso (with the rounding margin)
  // gives cube index 0 or 255, no triangles.  Skipped without changing the output.
  const float cluster_reject = tol * 1.00001f + reject;
  int total = 0;
  for (int ci = 0; ci < ncl; ++ci) {
    const float key = cand[ci * kThreads];
    if (fabsf(key - p.iso) > cluster_reject) continue;
    // loadCubeForSurface + selectClosestLayerForSurfaceGpu (:276-303, :509-551)
    float val[8];
    uint32_t mask = 0U;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      int best = -1;
      float best_delta = 1e30f;
#pragma unroll
      for (int l = 0; l < kLayers; ++l) {
        if (!S.valid[l][si(k)]) continue;
        const float delta = fabsf(plane_sd(S.plane[l][si(k)], cc) - key);
        if (delta <= tol && delta < best_delta) {
          best_delta = delta;
          best = l;
        }
      }
      val[k] = 0.0f;
      if (best >= 0) {
        val[k] = plane_sd(S.plane[best][si(k)], corner_pos(gx, gy, gz, k, vs));
        mask |= 1U << k;
      }
    }
    // completeCubeValuesWithFallbackGpu (:305-356)
    if (mask != 0xffU) {
      int cnt = 0;
      float sum = 0.0f;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (!(mask & (1U << k))) continue;
        ++cnt;
        sum += val[k];
      }
      if (cnt < 6) continue;
      const float global = sum / static_cast<float>(cnt);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (mask & (1U << k)) continue;
        float ns = 0.0f;
        int nn = 0;
#pragma unroll
        for (int e = 0; e < 12; ++e) {
          const int c0 = c_edge_corners[e][0], c1 = c_edge_corners[e][1];
          const int nb = c0 == k ? c1 : (c1 == k ? c0 : -1);
          if (nb < 0 || !(mask & (1U << nb))) continue;
          ns += val[nb];
          ++nn;
        }
        val[k] = nn > 0 ? (ns / static_cast<float>(nn)) : global;
        mask |= 1U << k;
      }
    }
    // computeCubeIndex / countCubeTriangles / emitCubeTriangles (:376-437)
    int cube = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (val[k] < p.iso) cube |= 1 << k;
    const int em = S.edge[cube];
    if (em == 0) continue;
    int ntri = 0;
    while (ntri < 5 && S.tri[cube][3 * ntri] >= 0) ++ntri;
    if (kEmit) {
      for (int t = 0; t < ntri; ++t) {
        float* o = out + static_cast<size_t>(total + t) * 9;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          // the vertex on edge e (interpolateVertexGpu, :358-374), computed where it is used: the same
          // operations on the same values wherever an edge's vertex is needed
          const int e = S.tri[cube][3 * t + q];
          const int c0 = c_edge_corners[e][0], c1 = c_edge_corners[e][1];
          const f3 v = interp(corner_pos(gx, gy, gz, c0, vs), corner_pos(gx, gy, gz, c1, vs), pick8(val, c0),
                              pick8(val, c1), p.iso);
          o[3 * q] = v.x;
          o[3 * q + 1] = v.y;
          o[3 * q + 2] = v.z;
        }
      }
    }
    total += ntri;
  }
  return total;
}

// exclusive scan of one value per thread over the CTA; returns the prefix, S.total = CTA sum
__device__ __forceinline__ uint32_t block_scan(Shared& S, uint32_t v, int tid) {
  const int lane = tid & 31, warp = tid >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffU, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) S.warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kThreads / 32 ? S.warp_sums[lane] : 0U;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffU, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kThreads / 32) S.warp_sums[lane] = wi - w;
    if (lane == 31) S.total = wi;
  }
  __syncthreads();
  const uint32_t r = S.warp_sums[warp] + incl - v;
  return r;
}

// sum of one value per thread over the CTA (S.total)
__device__ __forceinline__ void block_sum(Shared& S, uint32_t v, int tid) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffU, v, o);
  if ((tid & 31) == 0) S.warp_sums[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) {
    uint32_t w = tid < kThreads / 32 ? S.warp_sums[tid] : 0U;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffU, w, o);
    if (tid == 0) S.total = w;
  }
  __syncthreads();
}

__device__ __forceinline__ void load_neighbours(Shared& S, const Volume& V, uint32_t b, const int4& bk, int tid) {
  __syncthreads();  // previous block's readers are done with S.nbr / S.plane
  if (tid < 8) {
    S.nbr[tid] = tid == 0 ? b : lookup_block(V, bk.x + (tid & 1), bk.y + ((tid >> 1) & 1), bk.z + (tid >> 2));
  }
  __syncthreads();
}

// Pass 1: every cell of every direction with an observed layer in the block's neighbourhood; stores the
// cell's triangle count (cell_counts, one byte: at most 5 triangles x 24 clusters), the per-direction totals
// and the block total.
// list / list_count: optional subset of pool blocks (incremental meshing); all allocated blocks when null
__global__ void __launch_bounds__(kThreads, 2) mc_count_kernel(const Volume V, const Params p,
                                                               uint32_t* __restrict__ counts,
                                                               uint32_t* __restrict__ dir_totals,
                                                               uint8_t* __restrict__ cell_counts,
                                                               const uint32_t* __restrict__ list,
                                                               const uint32_t* __restrict__ list_count) {
  extern __shared__ __align__(16) unsigned char mc_smem[];
  Shared& S = *reinterpret_cast<Shared*>(mc_smem);
  const int tid = threadIdx.x;
  for (int i = tid; i < 256 * 16; i += kThreads) S.tri[i / 16][i % 16] = vh_mc_tri_table[i / 16][i % 16];
  for (int i = tid; i < 256; i += kThreads) S.edge[i] = vh_mc_edge_table[i];
  const uint32_t nitems = list ? *list_count : min(V.counters->num_blocks, V.max_blocks);
  const int lx = tid & 7, ly = (tid >> 3) & 7, lz = tid >> 6;
  for (uint32_t item = blockIdx.x; item < nitems; item += gridDim.x) {
    const uint32_t b = list ? list[item] : item;
    const int4 bk = V.block_keys[b];
    load_neighbours(S, V, b, bk, tid);
    // directions with an observed layer anywhere in the block or its +x/+y/+z neighbours; a cell of the
    // block only has corners there, so in any other direction no cell has a candidate surface
    uint32_t dirs = 0U;
#pragma unroll
    for (int k = 0; k < 8; ++k) dirs |= S.nbr[k] != kInvalidBlock ? V.dir_mask[S.nbr[k]] : 0U;
    const int gx = bk.x * kBlockSide + lx, gy = bk.y * kBlockSide + ly, gz = bk.z * kBlockSide + lz;
    uint32_t run = 0U;
    for (int d = 0; d < kDirs; ++d) {
      uint32_t total = 0U;
      if (dirs & (1U << d)) {  // uniform across the CTA
        stage_direction(S, V, p, d, tid);
        __syncthreads();
        const uint32_t n = static_cast<uint32_t>(process_cell<false>(S, p, gx, gy, gz, lx, ly, lz, tid, nullptr));
        cell_counts[(static_cast<size_t>(b) * kDirs + d) * kBlockVoxels + tid] = static_cast<uint8_t>(n);
        block_sum(S, n, tid);
        total = S.total;
        __syncthreads();  // S.total / S.plane reused by the next direction
      }
      if (tid == 0) dir_totals[static_cast<size_t>(b) * kDirs + d] = total;
      run += total;
    }
    if (tid == 0) counts[b] = run;
  }
}

// Pass 2: only blocks and directions that produce triangles are staged again, and only the cells whose
// pass-1 count is non-zero are evaluated, writing at offset + direction run + exclusive scan of the counts.
__global__ void __launch_bounds__(kThreads, 2) mc_emit_kernel(const Volume V, const Params p,
                                                              const uint32_t* __restrict__ counts,
                                                              const uint32_t* __restrict__ dir_totals,
                                                              const uint8_t* __restrict__ cell_counts,
                                                              const unsigned long long* __restrict__ offsets,
                                                              float* __restrict__ tris,
                                                              const uint32_t* __restrict__ list,
                                                              const uint32_t* __restrict__ list_count) {
  extern __shared__ __align__(16) unsigned char mc_smem[];
  Shared& S = *reinterpret_cast<Shared*>(mc_smem);
  const int tid = threadIdx.x;
  for (int i = tid; i < 256 * 16; i += kThreads) S.tri[i / 16][i % 16] = vh_mc_tri_table[i / 16][i % 16];
  for (int i = tid; i < 256; i += kThreads) S.edge[i] = vh_mc_edge_table[i];
  const uint32_t nitems = list ? *list_count : min(V.counters->num_blocks, V.max_blocks);
  const int lx = tid & 7, ly = (tid >> 3) & 7, lz = tid >> 6;
  for (uint32_t item = blockIdx.x; item < nitems; item += gridDim.x) {
    const uint32_t b = list ? list[item] : item;
    if (counts[b] == 0U) continue;  // uniform
    const int4 bk = V.block_keys[b];
    load_neighbours(S, V, b, bk, tid);
    const int gx = bk.x * kBlockSide + lx, gy = bk.y * kBlockSide + ly, gz = bk.z * kBlockSide + lz;
    unsigned long long run = offsets[b];
    for (int d = 0; d < kDirs; ++d) {
      const uint32_t total = dir_totals[static_cast<size_t>(b) * kDirs + d];
      if (total == 0U) continue;  // uniform
      stage_direction(S, V, p, d, tid);
      const uint32_t n = cell_counts[(static_cast<size_t>(b) * kDirs + d) * kBlockVoxels + tid];
      const uint32_t prefix = block_scan(S, n, tid);  // its barriers also publish the staged direction
      if (n > 0U) process_cell<true>(S, p, gx, gy, gz, lx, ly, lz, tid, tris + (run + prefix) * 9ULL);
      run += total;
      __syncthreads();  // S.plane / S.warp_sums reused by the next direction
    }
  }
}

// exclusive scan of counts[0..n) -> offsets, total; one CTA (the count array is a few MB at most)
// pool blocks updated in frames (frame - frames, frame]: the subset of incremental meshing
__global__ void recent_blocks_kernel(const Volume V, uint32_t frames, uint32_t* __restrict__ list,
                                     uint32_t* __restrict__ count) {
  const uint32_t n = min(V.counters->num_blocks, V.max_blocks);
  const uint32_t frame = V.counters->frame;
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
    const uint32_t st = V.block_stamp[b];
    if (st != 0U && frame - st < frames) list[atomicAdd(count, 1U)] = b;
  }
}

__global__ void __launch_bounds__(1024) scan_kernel(const Volume V, const uint32_t* __restrict__ counts,
                                                    unsigned long long* __restrict__ offsets,
                                                    unsigned long long* __restrict__ total) {
  __shared__ unsigned long long s_w[32];
  __shared__ unsigned long long s_carry;
  const uint32_t n = min(V.counters->num_blocks, V.max_blocks);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_carry = 0ULL;
  __syncthreads();
  for (uint32_t start = 0; start < n; start += 1024U) {
    const uint32_t i = start + tid;
    const unsigned long long v = i < n ? counts[i] : 0ULL;
    unsigned long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long t = __shfl_up_sync(0xffffffffU, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const unsigned long long w = s_w[lane];
      unsigned long long wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffU, wi, o);
        if (lane >= o) wi += t;
      }
      s_w[lane] = wi - w;
    }
    __syncthreads();
    const unsigned long long carry = s_carry;
    if (i < n) offsets[i] = carry + s_w[warp] + incl - v;
    __syncthreads();
    if (tid == 1023) s_carry = carry + s_w[warp] + incl;
    __syncthreads();
  }
  if (tid == 0) *total = s_carry;
}

}  // namespace

int mc_grid_size() {
  static int grid = 0;
  if (grid == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(mc_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(Shared));
    cudaFuncSetAttribute(mc_emit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(Shared));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mc_count_kernel, kThreads, sizeof(Shared));
    grid = (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 1);
  }
  return grid;
}

cudaError_t launch_mc_count(const Volume& V, const Params& p, uint32_t* counts, uint32_t* dir_totals,
                            uint8_t* cell_counts, const uint32_t* list, const uint32_t* list_count, cudaStream_t s) {
  mc_count_kernel<<<mc_grid_size(), kThreads, sizeof(Shared), s>>>(V, p, counts, dir_totals, cell_counts, list,
                                                                   list_count);
  return cudaGetLastError();
}

cudaError_t launch_recent_blocks(const Volume& V, uint32_t frames, uint32_t* list, uint32_t* count, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  recent_blocks_kernel<<<1024, 256, 0, s>>>(V, frames, list, count);
  return cudaGetLastError();
}

cudaError_t launch_mc_scan(const Volume& V, const uint32_t* counts, unsigned long long* offsets,
                           unsigned long long* total, cudaStream_t s) {
  scan_kernel<<<1, 1024, 0, s>>>(V, counts, offsets, total);
  return cudaGetLastError();
}

cudaError_t launch_mc_emit(const Volume& V, const Params& p, const uint32_t* counts, const uint32_t* dir_totals,
                           const uint8_t* cell_counts, const unsigned long long* offsets, float* tris,
                           const uint32_t* list, const uint32_t* list_count, cudaStream_t s) {
  mc_emit_kernel<<<mc_grid_size(), kThreads, sizeof(Shared), s>>>(V, p, counts, dir_totals, cell_counts, offsets,
                                                                  tris, list, list_count);
  return cudaGetLastError();
}

}  // namespace vh
