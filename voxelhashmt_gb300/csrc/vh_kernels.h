// vh_kernels.h -- host-side launchers of the GB300 kernels (internal to the library).
#pragma once

#include <cuda_runtime.h>

#include "vh_common.cuh"

namespace vh {

// depth bilateral filter (normals + 5x5 joint bilateral in one kernel); begin_frame != nullptr also
// starts a new frame on that volume's counters (frame stamp + 1, per-frame counters cleared).
cudaError_t launch_filter(const float* in, float* out, const Params& p, Counters* begin_frame, cudaStream_t s);
// per-pixel normals of the filter, for kernel-level parity checks: normals[3*W*H], valid[W*H]
cudaError_t launch_depth_normals(const float* in, float* normals, unsigned char* valid, const Params& p,
                                 cudaStream_t s);
cudaError_t launch_begin_frame(Counters* c, cudaStream_t s);
// allocation: 3 points x 27-neighbourhood per sampled pixel -> persistent hash + visible list
cudaError_t launch_alloc(const float* depth, const Volume& V, const Params& p, cudaStream_t s);
// directional multi-layer update of every visible block; grid = persistent CTAs.  exact: the bit-reproducible
// FP32 form; fast: the same source compiled with fused multiply-adds and hardware approximations.  With
// Params::normal_mode 1, nmap (width x height float4) receives the per-pixel normal map.
namespace exact {
// the depth filter of one frame, begin_frame as in vh::launch_filter (the fast compile is the fast-math form's)
cudaError_t launch_frame_filter(const float* in, float* out, const Params& p, Counters* begin_frame, cudaStream_t s);
// starts a frame, then filters it and allocates its blocks in one kernel (out: the filtered depth)
cudaError_t launch_filter_alloc(const float* in, float* out, const Volume& V, const Params& p, cudaStream_t s);
// one step of a multi-scene batch: filter + allocation, normal map, update, each a work-queue kernel over all
// scenes (queue: 3 counters, cleared here); band: every scene uses the truncation-band allocation rule
cudaError_t launch_batch(const SceneDesc* descs, const BatchHeader* hdr, uint32_t* queue, bool band, cudaStream_t s);
// the same step as one cooperative launch of a persistent kernel (bar: two zeroed words kept by the batch)
cudaError_t launch_batch_persistent(const SceneDesc* descs, const BatchHeader* hdr, uint32_t* queue, uint32_t* bar,
                                    bool band, cudaStream_t s);
cudaError_t launch_integrate(const float* depth, const Volume& V, const Params& p, int grid, float4* nmap,
                             cudaStream_t s);
cudaError_t launch_integrate_prepare(const float* depth, const Volume& V, const Params& p, float4* nmap,
                                     cudaStream_t s);
cudaError_t launch_integrate_update(const float* depth, const Volume& V, const Params& p, int grid,
                                    const float4* nmap, cudaStream_t s, int variant);
int fused_variant_count();
void fused_variant_shape(int variant, int* threads, int* min_blocks);
cudaError_t launch_pixel_normals(const float* depth, const Params& p, float4* nmap, cudaStream_t s);
int integrate_grid_size();
}  // namespace exact
namespace fast {
// the depth filter of one frame, begin_frame as in vh::launch_filter (the fast compile is the fast-math form's)
cudaError_t launch_frame_filter(const float* in, float* out, const Params& p, Counters* begin_frame, cudaStream_t s);
// starts a frame, then filters it and allocates its blocks in one kernel (out: the filtered depth)
cudaError_t launch_filter_alloc(const float* in, float* out, const Volume& V, const Params& p, cudaStream_t s);
// one step of a multi-scene batch: filter + allocation, normal map, update, each a work-queue kernel over all
// scenes (queue: 3 counters, cleared here); band: every scene uses the truncation-band allocation rule
cudaError_t launch_batch(const SceneDesc* descs, const BatchHeader* hdr, uint32_t* queue, bool band, cudaStream_t s);
// the same step as one cooperative launch of a persistent kernel (bar: two zeroed words kept by the batch)
cudaError_t launch_batch_persistent(const SceneDesc* descs, const BatchHeader* hdr, uint32_t* queue, uint32_t* bar,
                                    bool band, cudaStream_t s);
cudaError_t launch_integrate(const float* depth, const Volume& V, const Params& p, int grid, float4* nmap,
                             cudaStream_t s);
cudaError_t launch_integrate_prepare(const float* depth, const Volume& V, const Params& p, float4* nmap,
                                     cudaStream_t s);
cudaError_t launch_integrate_update(const float* depth, const Volume& V, const Params& p, int grid,
                                    const float4* nmap, cudaStream_t s, int variant);
int fused_variant_count();
void fused_variant_shape(int variant, int* threads, int* min_blocks);
cudaError_t launch_pixel_normals(const float* depth, const Params& p, float4* nmap, cudaStream_t s);
int integrate_grid_size();
}  // namespace fast
// marching cubes over all allocated blocks (or the blocks of `list`, *list_count entries, device memory): pass 1
// writes per-block, per-direction and per-cell triangle
// counts, the scan turns the block counts into offsets (+ total), pass 2 writes triangles (9 floats each)
cudaError_t launch_mc_count(const Volume& V, const Params& p, uint32_t* counts, uint32_t* dir_totals,
                            uint8_t* cell_counts, const uint32_t* list, const uint32_t* list_count, cudaStream_t s);
// pool blocks updated within the last `frames` frames -> list (count on the device, reset here)
cudaError_t launch_recent_blocks(const Volume& V, uint32_t frames, uint32_t* list, uint32_t* count, cudaStream_t s);
cudaError_t launch_mc_scan(const Volume& V, const uint32_t* counts, unsigned long long* offsets,
                           unsigned long long* total, cudaStream_t s);
cudaError_t launch_mc_emit(const Volume& V, const Params& p, const uint32_t* counts, const uint32_t* dir_totals,
                           const uint8_t* cell_counts, const unsigned long long* offsets, float* tris,
                           const uint32_t* list, const uint32_t* list_count, cudaStream_t s);
int mc_grid_size();
// full recount of observed voxels (any layer weight > 0) over the pool
cudaError_t launch_recount(const Volume& V, unsigned long long* out, cudaStream_t s);
// keys of the current frame's visible blocks (int3 each, unordered)
cudaError_t launch_visible_keys(const Volume& V, int* keys, cudaStream_t s);
// copy blocks [first, first+count) to the reference layout: keys int32[count][3],
// voxels [count][512][6][3] x {f32 weight, f32 surface_coord, f32 plane_offset, u32 packed_normal}
cudaError_t launch_export(const Volume& V, uint32_t first, uint32_t count, int* keys, float4* voxels,
                          cudaStream_t s);

// import blocks in the reference layout (insert or overwrite); idx: n scratch words
cudaError_t launch_import(const Volume& V, const int* keys, const float4* voxels, uint32_t n, uint32_t* idx,
                          cudaStream_t s);
// insert (or find) n keys; idx[i] receives the pool block of key i (kInvalidBlock when the pool is full)
cudaError_t launch_import_keys(const Volume& V, const int* keys, uint32_t n, uint32_t* idx, cudaStream_t s);

// ---- eviction (vh_evict.cu) ----
constexpr int kAgeBins = 4096;  // block-age histogram: ages 0..4094 frames, the last bin everything older
cudaError_t launch_age_hist(const Volume& V, uint32_t* hist, cudaStream_t s);
// Which blocks an eviction removes.  age = frames since the block's last layer update (never updated: oldest),
// bin = min(age, kAgeBins - 1).  A block is a victim when age >= min_age, or bin > tie_bin, or bin == tie_bin
// and its pool index is below cut (ties at the boundary bin go in pool order).  {min_age, kAgeBins, 0}: every
// block of age >= min_age.
struct EvictRule {
  uint32_t min_age, tie_bin, cut;
};
// pool blocks of [0, n) in ascending order into list, their number into *total (device); what 0: the victims;
// what 1: the blocks of [lo, n) that are not; what 2: the blocks of bin tie_bin that are not victims by age.
// cta_scratch: ceil(n / 1024) words.
cudaError_t launch_select(const Volume& V, uint32_t n, const EvictRule& rule, int what, uint32_t lo,
                          uint32_t* cta_scratch, uint32_t* total, uint32_t* list, cudaStream_t s);
// listed blocks with their keys into a staging buffer: native 1 the pool's own block image, 0 the reference layout
cudaError_t launch_copy_out(const Volume& V, const uint32_t* list, uint32_t n, int native, int* keys, void* out,
                            cudaStream_t s);
// observed voxels of the n listed victim blocks -> *out (zeroed here); the volume's count less *out
cudaError_t launch_victim_observed(const Volume& V, const uint32_t* list, uint32_t n, unsigned long long* out,
                                   cudaStream_t s);
cudaError_t launch_subtract_observed(const Volume& V, const unsigned long long* removed, cudaStream_t s);
cudaError_t launch_move_blocks(const Volume& V, const uint32_t* src, const uint32_t* dst, uint32_t n, cudaStream_t s);
// empties the hash and inserts the keys of pool blocks [0, live)
cudaError_t launch_rehash(const Volume& V, uint32_t live, cudaStream_t s);
// block images in into the pool blocks idx[0..n) (kInvalidBlock: skipped), masks rebuilt, stamped with the frame
cudaError_t launch_restore_native(const Volume& V, const void* in, uint32_t n, const uint32_t* idx, cudaStream_t s);
// depth ray-cast of the fused volume from pose p.T_wc: out[W*H] camera depth of the first plane crossing, 0 = none
cudaError_t launch_raycast(const Volume& V, const Params& p, float min_depth, float max_depth, float step, float* out,
                           cudaStream_t s);
// indexed mesh of a triangle soup (vertices merged when bit-identical, numbered by first use; faces in soup
// order, collapsed and zero-area ones dropped).  Buffers for a soup of up to `capacity` triangles: slot_first
// (slot_mask + 1 >= 6 * capacity slots, a power of two), vslot / vid / flags / number (3 * capacity words),
// sums (weld_scan_tiles(3 * capacity) words), verts (9 * capacity floats), faces (3 * capacity ints), counts
// (3 words: vertices, faces, table-full flag).  3 * ntri must be below 2^30.
struct WeldBuffers {
  uint32_t* slot_first;
  uint32_t slot_mask;
  uint32_t* vslot;
  uint32_t* vid;
  uint32_t* flags;
  uint32_t* number;
  uint32_t* sums;
  float* verts;
  int32_t* faces;
  uint32_t* counts;
};
uint32_t weld_scan_tiles(uint32_t n);
cudaError_t launch_weld(const float* tris, uint32_t ntri, const WeldBuffers& W, cudaStream_t s);
// synthetic depth for the analytic benchmark scenes (prims: n x 10 floats, device memory)
cudaError_t launch_render(const float* prims, int n_prims, const Params& p, uint32_t seed, uint32_t frame,
                          float sigma_z2, float dropout, float max_depth, float* out, cudaStream_t s);

}  // namespace vh
