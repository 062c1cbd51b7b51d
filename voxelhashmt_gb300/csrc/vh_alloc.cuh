// vh_alloc.cuh -- device code of the block allocation, shared by the single-frame kernel (vh_alloc.cu) and the
// multi-scene batch (vh_integrate.cu).
//
// Block allocation: per sampled pixel, the surface point and the points one truncation
// distance in front of and behind it along the camera ray, each with its 27-block neighbourhood
// (src/cuda_block_allocator.cu:198-272), inserted into a persistent open-addressing spatial hash.
//
// The reference inserts all 81 keys of every pixel into a transient table with atomicCAS (memset of the
// whole table every frame), scans the table to compact it, copies the keys to the host and looks them up
// in a host map.  Here:
//   1. each CTA takes a 32x8 tile of samples, computes the 3 centre blocks per sample and de-duplicates the
//      centres in a shared-memory set;
//   2. the tile expands its unique centres to 27-neighbourhoods into a second shared-memory set;
//   3. each unique key of the tile is looked up / inserted once in the persistent device hash (plain load
//      first, atomicCAS only on an empty slot) and, the first time a frame touches a slot (atomicExch on
//      the slot's frame stamp), appended to the visible list.  New keys take the next pool index.
// Key packing, the slot hash and linear probing follow cuda_block_allocator.cu:153-196, so the table's
// key words are the reference's.  Params::alloc_mode 1 replaces the 3 x 27-neighbourhood rule by the blocks the
// +-truncation segment of each pixel's ray crosses (a 3-D DDA): the truncation band only.
#pragma once

#include "vh_common.cuh"

namespace vh {
namespace alloc {

constexpr int kTX = 32;
constexpr int kTY = 8;
constexpr int kThreads = kTX * kTY;
constexpr int kCenterSlots = 1024;  // >= 3 * kThreads centres
constexpr int kMaxSmemProbes = 64;

__device__ __forceinline__ uint32_t smem_hash(unsigned long long k, int bits) {
  return static_cast<uint32_t>((k * 0x9E3779B97F4A7C15ULL) >> (64 - bits));
}

// slot was found or inserted this frame: put it on the visible list once (the exchange both tests and sets the
// slot's frame stamp: one round trip to L2)
__device__ __forceinline__ void mark_visible(const Volume& V, uint32_t slot, uint32_t frame) {
  if (atomicExch(&V.slot_stamp[slot], frame) == frame) return;
  const uint32_t pos = atomicAdd(&V.counters->visible_count, 1U);
  V.visible[pos] = slot;
}

// insertPackedBlockKey (cuda_block_allocator.cu:180-196) into the persistent table
__device__ inline void insert_global(const Volume& V, unsigned long long key, uint32_t frame) {
  int x, y, z;
  unpack_block_key(key, x, y, z);
  uint32_t slot = hash_block_key(x, y, z) & V.mask;
  for (uint32_t probe = 0; probe < V.capacity; ++probe) {
    unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(&V.slot_keys[slot]);
    if (cur == kEmptyKey) {
      cur = atomicCAS(&V.slot_keys[slot], kEmptyKey, key);
      if (cur == kEmptyKey) {
        uint32_t idx = kInvalidBlock;
        atomicAdd(&V.counters->new_blocks, 1U);
        if (V.max_blocks > 0U) {  // a keys-only volume (max_blocks == 0) records keys without pool blocks
          idx = atomicAdd(&V.counters->num_blocks, 1U);
          if (idx >= V.max_blocks) {
            atomicOr(&V.counters->error, kErrPoolFull);
            idx = kInvalidBlock;
          } else {
            V.block_keys[idx] = make_int4(x, y, z, static_cast<int>(frame));
          }
        }
        V.slot_block[slot] = idx;
        mark_visible(V, slot, frame);
        return;
      }
    }
    if (cur == key) {
      mark_visible(V, slot, frame);
      return;
    }
    slot = (slot + 1U) & V.mask;
  }
  atomicOr(&V.counters->error, kErrHashFull);
}

// shared-memory set insert; returns 1 if inserted, 0 if present, -1 if the probe budget ran out
__device__ __forceinline__ int smem_insert(unsigned long long* set, int bits, unsigned long long key) {
  const uint32_t mask = (1U << bits) - 1U;
  uint32_t s = smem_hash(key, bits);
  for (int probe = 0; probe < kMaxSmemProbes; ++probe) {
    const unsigned long long prev = atomicCAS(&set[s], kEmptyKey, key);
    if (prev == kEmptyKey) return 1;
    if (prev == key) return 0;
    s = (s + 1U) & mask;
  }
  return -1;
}

// Blocks crossed by the segment a -> b (3-D DDA over the block grid, Amanatides & Woo 1987), each inserted into
// the tile set; returns false when a block leaves the packed key range.
__device__ inline bool insert_band_blocks(const Volume& V, unsigned long long* s_nset, int set_bits, f3 a, f3 b, float bws,
                                          uint32_t frame) {
  int c[3] = {static_cast<int>(floorf(a.x / bws)), static_cast<int>(floorf(a.y / bws)), static_cast<int>(floorf(a.z / bws))};
  const int e[3] = {static_cast<int>(floorf(b.x / bws)), static_cast<int>(floorf(b.y / bws)),
                    static_cast<int>(floorf(b.z / bws))};
  const float o[3] = {a.x, a.y, a.z};
  const float d[3] = {b.x - a.x, b.y - a.y, b.z - a.z};
  int st[3];
  float tmax[3], tdel[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    st[k] = d[k] > 0.0f ? 1 : (d[k] < 0.0f ? -1 : 0);
    tmax[k] = st[k] != 0 ? ((static_cast<float>(c[k] + (st[k] > 0 ? 1 : 0)) * bws - o[k]) / d[k]) : 3.0e38f;
    tdel[k] = st[k] != 0 ? bws / fabsf(d[k]) : 3.0e38f;
  }
  for (int it = 0; it < 64; ++it) {
    unsigned long long key;
    if (!pack_block_key(c[0], c[1], c[2], key)) return false;
    if (smem_insert(s_nset, set_bits, key) < 0) insert_global(V, key, frame);
    if (c[0] == e[0] && c[1] == e[1] && c[2] == e[2]) break;
    const int k = (tmax[0] < tmax[1]) ? (tmax[0] < tmax[2] ? 0 : 2) : (tmax[1] < tmax[2] ? 1 : 2);
    // the step on axis k, written per axis so that the arrays stay in registers (no indexing by a run-time k)
    const float tk = k == 0 ? tmax[0] : (k == 1 ? tmax[1] : tmax[2]);
    if (tk > 1.0f) break;  // rounding ended the walk one cell short of the end block
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (j == k) {
        c[j] += st[j];
        tmax[j] += tdel[j];
      }
    }
  }
  unsigned long long key;  // the end block always belongs to the band (the set drops the duplicate)
  if (!pack_block_key(e[0], e[1], e[2], key)) return false;
  if (smem_insert(s_nset, set_bits, key) < 0) insert_global(V, key, frame);
  return true;
}

// Shared-memory sets of one tile.  kBand: the truncation-band rule only (Params::alloc_mode 1), which needs
// just the tile's key set, and a small one: a tile's band crosses tens of blocks, and a key that finds the set
// full goes straight to the device table.
template <bool kBand>
struct TileSets;
template <>
struct TileSets<false> {
  static constexpr int kSetBits = 12;
  unsigned long long cset[kCenterSlots];
  unsigned long long clist[3 * kThreads];
  unsigned long long nset[1 << kSetBits];
  uint32_t ccount;
};
template <>
struct TileSets<true> {
  static constexpr int kSetBits = 10;
  unsigned long long nset[1 << kSetBits];
  unsigned long long klist[1 << kSetBits];  // the set's keys, compacted
  uint32_t nkeys;
};
using Smem = TileSets<false>;

// buildActiveBlockHashKernel (cuda_block_allocator.cu:231-272) for one tile of kThreads samples; every thread
// of the CTA calls it (it synchronises).  Thread tid holds one sample: has = it exists and lies in the image,
// (u, v) its pixel, d its depth.  kBand = false runs the rule p.alloc_mode selects; kBand = true requires
// p.alloc_mode == 1.
template <bool kBand>
__device__ __forceinline__ void alloc_samples(const Volume& V, const Params& p, bool has, int u, int v, float d, int tid,
                                              TileSets<kBand>& S) {
  constexpr int kSetBits = TileSets<kBand>::kSetBits;
  unsigned long long* s_nset = S.nset;
  const uint32_t frame = V.counters->frame;
  for (int i = tid; i < (1 << kSetBits); i += kThreads) s_nset[i] = kEmptyKey;
  if constexpr (!kBand) {
    for (int i = tid; i < kCenterSlots; i += kThreads) S.cset[i] = kEmptyKey;
    if (tid == 0) S.ccount = 0U;
  } else {
    if (tid == 0) S.nkeys = 0U;
  }
  __syncthreads();

  // 1. centre blocks of this sample (buildActiveBlockHashKernel, cuda_block_allocator.cu:231-272)
  if (has && d > 0.0f) {
    const f3 pc = mk3((static_cast<float>(u) - p.cx) * d / p.fx, (static_cast<float>(v) - p.cy) * d / p.fy, d);
    const f3 pw = xform_point(p.T_wc, pc);
    const f3 ray = normalize3(mk3(pw.x - p.T_wc.t[0], pw.y - p.T_wc.t[1], pw.z - p.T_wc.t[2]));
    const f3 pts[3] = {
        pw,
        mk3(pw.x - ray.x * p.truncation, pw.y - ray.y * p.truncation, pw.z - ray.z * p.truncation),
        mk3(pw.x + ray.x * p.truncation, pw.y + ray.y * p.truncation, pw.z + ray.z * p.truncation),
    };
    if (kBand || p.alloc_mode == 1) {
      if (!insert_band_blocks(V, s_nset, kSetBits, pts[1], pts[2], p.block_world_size, frame)) {
        atomicOr(&V.counters->error, kErrKeyRange);
      }
    } else {
      if constexpr (!kBand) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const int bx = static_cast<int>(floorf(pts[k].x / p.block_world_size));
          const int by = static_cast<int>(floorf(pts[k].y / p.block_world_size));
          const int bz = static_cast<int>(floorf(pts[k].z / p.block_world_size));
          // every neighbour must pack (the reference flags overflow on the first one that does not)
          unsigned long long lo, hi;
          if (!pack_block_key(bx - 1, by - 1, bz - 1, lo) || !pack_block_key(bx + 1, by + 1, bz + 1, hi)) {
            atomicOr(&V.counters->error, kErrKeyRange);
            continue;
          }
          unsigned long long key;
          pack_block_key(bx, by, bz, key);
          const int r = smem_insert(S.cset, 10, key);
          if (r == 1) {
            const uint32_t pos = atomicAdd(&S.ccount, 1U);
            S.clist[pos] = key;
          } else if (r < 0) {  // centre set saturated: expand this centre straight into the table
            for (int o = 0; o < 27; ++o) {
              unsigned long long nk;
              pack_block_key(bx + (o % 3) - 1, by + ((o / 3) % 3) - 1, bz + (o / 9) - 1, nk);
              insert_global(V, nk, frame);
            }
          }
        }
      }
    }
  }
  __syncthreads();

  if constexpr (!kBand) {
    // 2. 27-neighbourhoods of the unique centres (insertNeighborhood, :198-220)
    const int ncent = static_cast<int>(S.ccount);
    for (int w = tid; w < ncent * 27; w += kThreads) {
      const int c = w / 27, o = w - c * 27;
      int x, y, z;
      unpack_block_key(S.clist[c], x, y, z);
      unsigned long long key;
      pack_block_key(x + (o % 3) - 1, y + ((o / 3) % 3) - 1, z + (o / 9) - 1, key);
      if (smem_insert(s_nset, kSetBits, key) < 0) insert_global(V, key, frame);  // tile set saturated
    }
    __syncthreads();
  }

  // 3. one persistent-hash insert per unique key of the tile.  The band's set is sparse (tens of keys in 1,024
  // slots): its keys are compacted first, so that every insert (a chain of dependent L2/DRAM round trips) runs
  // on its own thread at once instead of one after another in the threads that own several set slots.
  if constexpr (kBand) {
    for (int s = tid; s < (1 << kSetBits); s += kThreads) {
      const unsigned long long key = s_nset[s];
      if (key != kEmptyKey) S.klist[atomicAdd(&S.nkeys, 1U)] = key;
    }
    __syncthreads();
    const int n = static_cast<int>(S.nkeys);
    for (int i = tid; i < n; i += kThreads) insert_global(V, S.klist[i], frame);
  } else {
    for (int s = tid; s < (1 << kSetBits); s += kThreads) {
      const unsigned long long key = s_nset[s];
      if (key != kEmptyKey) insert_global(V, key, frame);
    }
  }
}

// the tile of samples at (sx0, sy0) (sample (sx, sy) = pixel (sx * stride, sy * stride)), depth from global memory
__device__ __forceinline__ void alloc_tile(const float* __restrict__ depth, const Volume& V, const Params& p, int sx0,
                                           int sy0, int tid, Smem& S) {
  const int sx = sx0 + tid % kTX, sy = sy0 + tid / kTX;
  const int u = sx * p.stride, v = sy * p.stride;
  const bool has = sx < p.sample_width && sy < p.sample_height && u < p.width && v < p.height;
  const float d = has ? __ldg(&depth[static_cast<size_t>(v) * p.width + u]) : 0.0f;
  alloc_samples<false>(V, p, has, u, v, d, tid, S);
}

}  // namespace alloc
}  // namespace vh
