/*
 * vh_oracle.h -- CPU restatement of the voxelhashmt depth-fusion path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle for the CUDA product in
 * voxelhashmt_gb300/; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The product never links or calls it.
 *
 * It restates, in plain C with every float operation written in the reference's
 * order, two flavours of the same algorithm:
 *
 *   VO_FLAVOR_REF_GPU  the reference CUDA path
 *                      src/cuda_tsdf_integrator.cu:169-903 (filter, integrate)
 *                      src/cuda_block_allocator.cu:123-272 (allocation)
 *                      src/cuda_mesh_extractor.cu:144-632 (marching cubes)
 *   VO_FLAVOR_REF_CPU  the reference CPU path
 *                      src/reconstruction_backend.cpp:26-189 (filter)
 *                      include/tsdfmc/voxel_hash_tsdf.h:206-1060 (volume)
 *                      include/tsdfmc/marching_cubes.h:34-94 (polygoniser)
 *
 * Exponentials: VO_EXP_LIBM calls expf() like both reference paths do on their
 * own compilers; VO_EXP_OWN calls vo_expf_own(), a restatement of the C library's
 * expf algorithm (glibc >= 2.28) that returns the same float for every argument on
 * the host the reference was compiled on.  The CUDA product evaluates that same
 * function on the device, so it is compared bit-for-bit with both.
 *
 * Build with -ffp-contract=off (no fused multiply-add contraction) and without
 * -ffast-math: every a*b+c must round twice, as in the reference source.
 *
 * Pins: the REF_CPU flavour is checked bit-exactly against the reference CPU
 * sources compiled from the reference tree; the REF_GPU flavour (with
 * VO_EXP_LIBM) against the reference .cu sources compiled as host C++ under a
 * CUDA emulation prelude (oracle/build.py), and both through the committed
 * fixtures in tests/golden/.
 *
 * FP64 transcription: the same source built with -DVO_FP64 (liboracle64.so)
 * computes in double with libm's double functions; this interface, the inputs
 * and the stored voxel records stay float.
 */
#ifndef VH_ORACLE_H
#define VH_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { VO_FLAVOR_REF_GPU = 0, VO_FLAVOR_REF_CPU = 1 };
enum { VO_EXP_LIBM = 0, VO_EXP_OWN = 1 };

/* math_types.h:200-207 */
typedef struct {
  int32_t width, height;
  float fx, fy, cx, cy;
} vo_intrinsics;

/* math_types.h:180-198: camera->world, row-major R */
typedef struct {
  float R[9];
  float t[3];
} vo_pose;

/* voxel_hash_tsdf.h:18-23 */
typedef struct {
  float weight;
  float surface_coord;
  float plane_offset;
  uint32_t packed_normal;
} vo_layer;

/* voxel_hash_tsdf.h:25-31: 6 signed dominant-axis bins x 3 layers */
typedef struct {
  vo_layer layers[6][3];
} vo_voxel;

typedef struct {
  int32_t x, y, z;
} vo_key;

typedef struct {
  float v[9];
} vo_triangle;

typedef struct {
  int32_t flavor;
  int32_t exp_impl;
  /* depth discontinuity gate: max(base, rel * depth) */
  float disc_base, disc_rel;
  /* depth bilateral filter */
  int32_t filter_radius;
  float filter_sigma_spatial, filter_sigma_range, filter_sigma_angular;
  float filter_min_cos;
  /* per-voxel normal bilateral blend */
  int32_t normal_radius;
  float normal_sigma_spatial, normal_sigma_range, normal_sigma_angular;
  /* layer merge / extraction */
  float layer_merge_scale, layer_normal_cos, layer_extract_scale;
  /* observation weight */
  float max_weight, depth_sigma, huber_delta, min_obs_weight, min_view_weight;
  /* worker threads for the embarrassingly parallel loops (1 = literal serial order) */
  int32_t threads;
  /* The GPU library's opt-in switches in their exact compile (no reference counterpart; all 0 = the reference):
   * alloc_mode 1: truncation-band allocation (vo_collect_band_blocks); normal_mode 1: the per-pixel normal
   * map (surface_normal at every pixel centre) interpolated bilinearly per voxel; layer_format 1: FP16 bins
   * (32 bytes per voxel and direction), decoded into the voxel records after every update. */
  int32_t alloc_mode, normal_mode, layer_format;
} vo_config;

/* Fills the constant set of the given reference flavour
 * (cuda_tsdf_integrator.cu:16-35 / voxel_hash_tsdf.h:194-204 + reconstruction_backend.cpp:26-32). */
void vo_config_default(vo_config* cfg, int32_t flavor);

float vo_expf_own(float x);
void vo_expf_array(const float* x, float* y, size_t n);
void vo_expf_compare_libm(uint32_t first, uint64_t count, int threads, uint64_t* mismatches, uint32_t* first_mismatch);
/* The device renderer (vh_render_depth) restated: prims n x 10 floats, out width*height floats. */
void vo_render_depth(const float* prims, int32_t n_prims, const vo_intrinsics* K, const vo_pose* T_wc, uint32_t seed,
                     uint32_t frame, float sigma_z2, float dropout, float max_depth, float* out);

/* depth bilateral filter (both flavours): out[W*H] */
void vo_filter_depth(const vo_config* cfg, const float* depth, const vo_intrinsics* K, float* out);
/* per-pixel normals of the filter (for kernel-level parity): normals[3*W*H], valid[W*H] */
void vo_depth_normals(const vo_config* cfg, const float* depth, const vo_intrinsics* K, float* normals,
                      uint8_t* valid);

/* Active-block collection for one frame (allocation rule only, no volume).
 * Returns the number of unique keys written to out (sorted x,y,z ascending),
 * -1 if a key is outside the 21-bit packed range (REF_GPU overflow), -2 if max is too small. */
int64_t vo_collect_blocks(const vo_config* cfg, const float* depth, const vo_intrinsics* K, const vo_pose* T_wc,
                          float voxel_size, float truncation, int32_t stride, vo_key* out, int64_t max_out);

/* The truncation-band rule (the library's opt-in allocation mode): the blocks crossed by each valid pixel's
 * [p - trunc*ray, p + trunc*ray] segment.  Same return convention as vo_collect_blocks. */
int64_t vo_collect_band_blocks(const float* depth, const vo_intrinsics* K, const vo_pose* T_wc, float voxel_size,
                               float truncation, int32_t stride, vo_key* out, int64_t max_out);

typedef struct vo_volume vo_volume;
vo_volume* vo_volume_new(const vo_config* cfg, float voxel_size, float truncation);
void vo_volume_free(vo_volume* vol);
/* one frame through the flavour's pipeline: filter -> collect -> ensure blocks -> integrate.
 * returns number of active blocks this frame, or -1 on allocation overflow. */
int64_t vo_volume_integrate_frame(vo_volume* vol, const float* depth, const vo_intrinsics* K,
                                  const vo_pose* T_wc, int32_t stride);
/* ensure + integrate a given key list with the given (already filtered) depth */
void vo_volume_integrate_blocks(vo_volume* vol, const vo_key* keys, int64_t n, const float* depth,
                                const vo_intrinsics* K, const vo_pose* T_wc);
int64_t vo_volume_block_count(const vo_volume* vol);
int64_t vo_volume_observed_voxels(const vo_volume* vol);
/* block i in insertion order: key + 512 voxels (x fastest) */
void vo_volume_get_block(const vo_volume* vol, int64_t i, vo_key* key, vo_voxel* voxels);
int64_t vo_volume_find_block(const vo_volume* vol, int32_t x, int32_t y, int32_t z);
/* inserts/overwrites a block (applyFlatBlocks, voxel_hash_tsdf.h:183-188) */
void vo_volume_set_block(vo_volume* vol, vo_key key, const vo_voxel* voxels);
/* applyFlatBlocks: n records (keys[i], voxels[i * 512 ...]) applied in order */
void vo_volume_apply_flat_blocks(vo_volume* vol, const vo_key* keys, const vo_voxel* voxels, int64_t n);
/* removes the given keys (the state after the library evicts those blocks) */
void vo_volume_remove_blocks(vo_volume* vol, const vo_key* keys, int64_t n);
/* marching cubes over all blocks and 6 directions; *out is malloc'd (free with vo_free) */
int64_t vo_volume_extract_mesh(const vo_volume* vol, float iso, vo_triangle** out);
void vo_free(void* p);

/* small kernels exposed for known-answer tests */
/* depth ray-cast of the fused volume (restates voxelhashmt_gb300/csrc/vh_raycast.cu): out[W*H], 0 = no hit */
void vo_raycast_depth(const vo_volume* vol, const vo_intrinsics* K, const vo_pose* T_wc, float min_depth,
                      float max_depth, float step_voxels, float* out);
int32_t vo_surface_normal(const vo_config* cfg, const float* depth, const vo_intrinsics* K, float u, float v,
                          float n[3]);
uint32_t vo_pack_normal(int32_t flavor, const float n[3]);
void vo_unpack_normal(int32_t flavor, int32_t mesh_variant, uint32_t packed, float n[3]);
uint32_t vo_hash_block_key(int32_t x, int32_t y, int32_t z);
int32_t vo_pack_block_key(int32_t x, int32_t y, int32_t z, uint64_t* packed);
float vo_observation_weight(const vo_config* cfg, float depth, float sd, float trunc, float view);

#ifdef __cplusplus
}
#endif
#endif
