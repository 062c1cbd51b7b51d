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
constexpr int kNbrSlots = 4096;
constexpr int kMaxSmemProbes = 64;

__device__ __forceinline__ uint32_t smem_hash(unsigned long long k, int bits) {
  return static_cast<uint32_t>((k * 0x9E3779B97F4A7C15ULL) >> (64 - bits));
}

// slot was found or inserted this frame: put it on the visible list once
__device__ __forceinline__ void mark_visible(const Volume& V, uint32_t slot, uint32_t frame) {
  if (*reinterpret_cast<volatile uint32_t*>(&V.slot_stamp[slot]) == frame) return;
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
__device__ inline bool insert_band_blocks(const Volume& V, unsigned long long* s_nset, f3 a, f3 b, float bws, uint32_t frame) {
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
    if (smem_insert(s_nset, 12, key) < 0) insert_global(V, key, frame);
    if (c[0] == e[0] && c[1] == e[1] && c[2] == e[2]) break;
    const int k = (tmax[0] < tmax[1]) ? (tmax[0] < tmax[2] ? 0 : 2) : (tmax[1] < tmax[2] ? 1 : 2);
    if (tmax[k] > 1.0f) break;  // rounding ended the walk one cell short of the end block
    c[k] += st[k];
    tmax[k] += tdel[k];
  }
  unsigned long long key;  // the end block always belongs to the band (the set drops the duplicate)
  if (!pack_block_key(e[0], e[1], e[2], key)) return false;
  if (smem_insert(s_nset, 12, key) < 0) insert_global(V, key, frame);
  return true;
}

struct Smem {
  unsigned long long cset[kCenterSlots];
  unsigned long long clist[3 * kThreads];
  unsigned long long nset[kNbrSlots];
  uint32_t ccount;
};

// buildActiveBlockHashKernel (cuda_block_allocator.cu:231-272) for the 32x8 tile of samples at (sx0, sy0);
// every thread of the CTA calls it (it synchronises).
__device__ __forceinline__ void alloc_tile(const float* __restrict__ depth, const Volume& V, const Params& p, int sx0,
                                           int sy0, int tid, Smem& S) {
  unsigned long long* s_cset = S.cset;
  unsigned long long* s_clist = S.clist;
  unsigned long long* s_nset = S.nset;
  uint32_t& s_ccount = S.ccount;
  const int tx = tid % kTX, ty = tid / kTX;
  const uint32_t frame = V.counters->frame;
  for (int i = tid; i < kCenterSlots; i += kThreads) s_cset[i] = kEmptyKey;
  for (int i = tid; i < kNbrSlots; i += kThreads) s_nset[i] = kEmptyKey;
  if (tid == 0) s_ccount = 0U;
  __syncthreads();

  // 1. centre blocks of this sample (buildActiveBlockHashKernel, cuda_block_allocator.cu:231-272)
  const int sx = sx0 + tx;
  const int sy = sy0 + ty;
  if (sx < p.sample_width && sy < p.sample_height) {
    const int u = sx * p.stride, v = sy * p.stride;
    if (u < p.width && v < p.height) {
      const float d = __ldg(&depth[static_cast<size_t>(v) * p.width + u]);
      if (d > 0.0f) {
        const f3 pc = mk3((static_cast<float>(u) - p.cx) * d / p.fx, (static_cast<float>(v) - p.cy) * d / p.fy, d);
        const f3 pw = xform_point(p.T_wc, pc);
        const f3 ray = normalize3(mk3(pw.x - p.T_wc.t[0], pw.y - p.T_wc.t[1], pw.z - p.T_wc.t[2]));
        const f3 pts[3] = {
            pw,
            mk3(pw.x - ray.x * p.truncation, pw.y - ray.y * p.truncation, pw.z - ray.z * p.truncation),
            mk3(pw.x + ray.x * p.truncation, pw.y + ray.y * p.truncation, pw.z + ray.z * p.truncation),
        };
        if (p.alloc_mode == 1) {
          if (!insert_band_blocks(V, s_nset, pts[1], pts[2], p.block_world_size, frame)) {
            atomicOr(&V.counters->error, kErrKeyRange);
          }
        } else
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
          const int r = smem_insert(s_cset, 10, key);
          if (r == 1) {
            const uint32_t pos = atomicAdd(&s_ccount, 1U);
            s_clist[pos] = key;
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

  // 2. 27-neighbourhoods of the unique centres (insertNeighborhood, :198-220)
  const int ncent = static_cast<int>(s_ccount);
  for (int w = tid; w < ncent * 27; w += kThreads) {
    const int c = w / 27, o = w - c * 27;
    int x, y, z;
    unpack_block_key(s_clist[c], x, y, z);
    unsigned long long key;
    pack_block_key(x + (o % 3) - 1, y + ((o / 3) % 3) - 1, z + (o / 9) - 1, key);
    if (smem_insert(s_nset, 12, key) < 0) insert_global(V, key, frame);  // tile set saturated
  }
  __syncthreads();

  // 3. one persistent-hash insert per unique key of the tile
  for (int s = tid; s < kNbrSlots; s += kThreads) {
    const unsigned long long key = s_nset[s];
    if (key != kEmptyKey) insert_global(V, key, frame);
  }
}

}  // namespace alloc
}  // namespace vh
