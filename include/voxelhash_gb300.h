/*
 * voxelhash_gb300.h -- C ABI of the GB300-native voxelhashmt depth-fusion path.
 *
 * One opaque handle (vh_volume) owns one voxel-hashed volume in device memory: a persistent spatial hash
 * of 8^3-voxel blocks and a pool of directional multi-layer voxels (6 signed dominant-axis bins x 3 layers
 * of {weight, surface_coord, plane_offset, packed octahedral normal}, 288 bytes per voxel).  The entry
 * points replace the reference's CUDA interfaces (paths relative to the reference project):
 *
 *   vh_integrate            integrateDepthFrameCuda            src/cuda_tsdf_integrator.h:16-19
 *   vh_allocate             allocateActiveBlocksCuda           src/cuda_block_allocator.h:17-22
 *   vh_visible_block_keys   the active block list integrateDepthFrameCuda builds (src/cuda_tsdf_integrator.cu:985-994)
 *   vh_extract_mesh/_copy   extractMeshCuda                    src/cuda_mesh_extractor.h:9
 *   vh_query_device         queryCudaBackendStatus             src/cuda_tsdf_integrator.h:9-14
 *   vh_block_count          gpuVolumeCacheBlockCount           src/cuda_tsdf_integrator.h:22
 *   vh_observed_voxel_count gpuVolumeCacheObservedVoxelCount   src/cuda_tsdf_integrator.h:23
 *   vh_export_blocks        gpuVolumeCacheBlockKeys / gpuVolumeCacheFlatBlocks  src/cuda_tsdf_integrator.h:24-25
 *   vh_import_blocks        VoxelHashTSDF::applyFlatBlocks     include/tsdfmc/voxel_hash_tsdf.h:183-188
 *   vh_filter_depth         estimateDepthNormalsKernel + bilateralFilterDepthKernel (src/cuda_tsdf_integrator.cu:629-725)
 *
 * Conventions (include/tsdfmc/math_types.h:180-244): depth is row-major float32 metres, index v*width+u,
 * <= 0 means no measurement; vh_pose is camera->world with R row-major; pinhole intrinsics without
 * distortion; camera x right, y down, z forward.  Block key = floor(world / (8 * voxel_size)).
 *
 * Execution model: calls that take a `stream` (a cudaStream_t, NULL = legacy default stream) only
 * enqueue device work and return; errors detected on the device (hash full, pool full, key range)
 * accumulate in the volume and are returned -- and cleared -- by vh_synchronize().  Calls that return
 * host-visible results (counts, keys, meshes) synchronise the stream first.  A volume is not
 * thread-safe; use one stream per volume at a time.  Results of the plain FP32 form are bit-identical
 * to a host evaluation of the reference CUDA algorithm (see oracle/).
 */
#ifndef VOXELHASH_GB300_H
#define VOXELHASH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VH_ABI_VERSION 1

typedef enum vh_status {
  VH_OK = 0,
  VH_ERR_INVALID_ARGUMENT = 1,
  VH_ERR_CUDA = 2,              /* a CUDA runtime call failed (reference: std::runtime_error, src/cuda_support.h:11-19) */
  VH_ERR_NO_DEVICE = 3,         /* no usable CUDA device (reference: TsdfIntegrationBackend(kGpu) throws) */
  VH_ERR_OUT_OF_MEMORY = 4,
  VH_ERR_KEY_RANGE = 5,         /* a block coordinate left the 21-bit packed range (reference: CudaActiveBlockAllocationFallback) */
  VH_ERR_HASH_FULL = 6,         /* no free hash slot (reference: CudaActiveBlockAllocationFallback) */
  VH_ERR_POOL_FULL = 7,         /* more blocks than vh_params.max_blocks */
  VH_ERR_BUFFER_TOO_SMALL = 8,  /* caller's output buffer is smaller than the result; *count holds the size */
  VH_ERR_CAPACITY = 9,          /* request larger than the fixed scratch of vh_allocate_static_scratch */
  VH_ERR_IO = 10,               /* dataset file missing, unreadable or unparsable (vh_dataset_last_error) */
  VH_ERR_FORMAT = 11,           /* unsupported or corrupt PNG / metadata layout (vh_dataset_last_error) */
  VH_ERR_TIMEOUT = 12           /* a bounded device-side wait gave up (the denoiser's tensor-core convolution) */
} vh_status;

typedef struct vh_volume vh_volume;

/* include/tsdfmc/math_types.h:200-207 */
typedef struct vh_intrinsics {
  int32_t width, height;
  float fx, fy, cx, cy;
} vh_intrinsics;

/* include/tsdfmc/math_types.h:180-198: camera -> world, R row-major */
typedef struct vh_pose {
  float R[9];
  float t[3];
} vh_pose;

/* VoxelHashTSDF(voxel_size, truncation_distance), include/tsdfmc/voxel_hash_tsdf.h:67-68, plus the device sizing */
typedef struct vh_params {
  float voxel_size;
  float truncation_distance;
  uint32_t hash_buckets; /* power of two; slots of the persistent block hash */
  uint32_t max_blocks;   /* pool capacity in blocks (<= 2^23); 0 = keys-only volume (vh_allocate only) */
  int32_t device;        /* CUDA device ordinal */
  /* 0 (default): FP32 layer records, 147,456 bytes per block, bit-identical to the reference;
   * 1: FP16 storage, 98,304 bytes per block: weight, surface coordinate and plane offset in binary16 (the two
   * coordinates relative to the voxel centre, in voxel units), normal word unchanged; FP32 update arithmetic.
   * Export and import always use the reference's FP32 Voxel layout. */
  int32_t layer_format;
} vh_params;

/* Algorithm constants; defaults are the reference CUDA path's (src/cuda_tsdf_integrator.cu:18-35,
 * src/cuda_mesh_extractor.cu:20).  The filter radius may not exceed 2. */
typedef struct vh_algorithm {
  float depth_discontinuity_base, depth_discontinuity_relative;
  int32_t filter_radius;
  float filter_sigma_spatial, filter_sigma_range, filter_sigma_angular, filter_min_cosine;
  int32_t normal_radius;
  float normal_sigma_spatial, normal_sigma_range, normal_sigma_angular;
  float layer_merge_voxel_scale, layer_normal_cosine, layer_extract_voxel_scale;
  float max_voxel_weight, depth_sigma, huber_delta, min_observation_weight, min_view_angle_weight;
  /* 0 (default): the reference's allocation rule, 3 points x 27-block neighbourhood per pixel;
   * 1: truncation band, the blocks crossed by each pixel's [depth - trunc, depth + trunc] ray segment. */
  int32_t allocation_mode;
  /* 0 (default): plain FP32, bit-reproducible; 1: the depth filter and the update pass with fused
   * multiply-adds and hardware approximations of exp, division and square root (results differ in the last
   * bits). */
  int32_t fast_math;
  /* 0 (default): the reference's bilateral surface normal evaluated at each voxel's projection (50 subpixel
   * depth samples); 1: the same normal evaluated once per pixel, bilinearly interpolated per voxel. */
  int32_t normal_mode;
  /* 1 (default): with normal_mode 1, the first frames cycle the layer-update kernel through its launch shapes
   * (threads per CTA x minimum resident CTAs per SM x voxel slots a thread tests per pass), time each with CUDA
   * events and keep the fastest
   * (results do not depend on the shape); 0: the shape launch_variant. */
  int32_t autotune;
  int32_t launch_variant; /* the layer-update launch shape used without autotuning (0..9, default 0) */
  /* 0 (default): the reference's bilateral depth filter; 1: the learned depth denoiser set with
   * vh_set_depth_denoiser (the bilateral filter until weights are set). */
  int32_t depth_filter;
} vh_algorithm;

/* per-frame statistics of the last integrated/allocated frame */
typedef struct vh_frame_stats {
  uint64_t visible_blocks;   /* unique blocks the frame touched (the reference's active block list) */
  uint64_t new_blocks;       /* blocks the frame allocated */
  uint64_t active_voxels;    /* voxels that passed projection, depth and truncation tests (reached the update) */
  uint64_t updated_voxels;   /* voxel layer updates the frame applied */
  uint64_t total_blocks;     /* blocks in the volume */
  uint64_t observed_voxels;  /* voxels with any layer weight > 0 */
} vh_frame_stats;

void vh_params_default(vh_params* params);
void vh_algorithm_default(vh_algorithm* algorithm);
const char* vh_status_string(vh_status status);

/* queryCudaBackendStatus: VH_OK and a "N CUDA device(s) detected" message, or VH_ERR_NO_DEVICE */
vh_status vh_query_device(char* message, size_t message_len);

/* Allocates the hash, the zeroed block pool and the counters on params->device.  algorithm may be NULL. */
vh_status vh_create(const vh_params* params, const vh_algorithm* algorithm, vh_volume** out);
void vh_destroy(vh_volume* volume);
/* Empties the volume (all blocks removed, pool re-zeroed); keeps the allocations. */
vh_status vh_reset(vh_volume* volume, void* stream);
/* Last error message of the volume (never NULL). */
const char* vh_last_error(const vh_volume* volume);

/* integrateDepthFrameCuda: bilateral filter -> block allocation on the filtered depth -> layer update.
 * depth: width*height floats, in host memory (depth_on_device = 0) or device memory (1). */
vh_status vh_integrate(vh_volume* volume, const float* depth, int32_t depth_on_device, const vh_intrinsics* K,
                       const vh_pose* T_wc, int32_t allocation_stride, void* stream);

/* allocateActiveBlocksCuda: allocation only, on the given (unfiltered) depth; adds the blocks to the volume
 * and returns the frame's unique block keys (3 int32 each, unordered) in keys_out (host memory).  With
 * keys_out == NULL only *count is returned.  Synchronises. */
vh_status vh_allocate(vh_volume* volume, const float* depth, int32_t depth_on_device, const vh_intrinsics* K,
                      const vh_pose* T_wc, int32_t allocation_stride, int32_t* keys_out, size_t max_keys,
                      size_t* count, void* stream);

/* Unique block keys (3 int32 each, unordered, host memory) the last vh_integrate / vh_allocate frame touched
 * -- the reference's per-frame active block list.  *count receives the number of keys.  Synchronises. */
vh_status vh_visible_block_keys(vh_volume* volume, int32_t* keys_out, size_t max_keys, size_t* count, void* stream);

/* vh_allocate without any allocation -- no counterpart in the reference.  For callers that cannot call
 * cudaMalloc once running (real-time tracking loops that forbid allocator calls, applications whose own pool
 * owns the whole device): the same keys-only allocation as vh_allocate, with the hash table, visible list and
 * counters in a fixed static device array of the library (20 MiB per GPU, held until the process exits).
 * depth: device memory, width*height floats, already written when the stream reaches this call (a producer on
 * another stream records an event that this stream waits for; the call orders itself against nothing else).
 * keys_out: DEVICE memory, 3 int32 per key (unlike vh_allocate, whose keys_out is host memory); NULL: count
 * only.  Runs on `stream` (NULL = the legacy default stream) and synchronises it.
 * Limit: at most 32,768 sampled pixels per call (e.g. 640x480 at allocation_stride 4, 181x181 at stride 1);
 * larger requests return VH_ERR_CAPACITY.  Each call looks up the array's device address
 * (cudaGetSymbolAddress) with the call's device current -- a host-side query, so the address stays right after
 * a cudaDeviceReset; the first call on a device may load the library's device code, so make it before any
 * stream capture.  Every call clears the table it uses, so no state carries over, but all calls share the one
 * array: calls that overlap on the same GPU race.  *count is 0 on every error except VH_ERR_BUFFER_TOO_SMALL,
 * where it holds the number of keys. */
vh_status vh_allocate_static_scratch(const float* depth, const vh_intrinsics* K, const vh_pose* T_wc,
                                     float voxel_size, float truncation_distance, int32_t allocation_stride,
                                     int32_t* keys_out, size_t max_keys, size_t* count, void* stream);

/* The depth bilateral filter alone (device buffers), with the volume's algorithm constants. */
vh_status vh_filter_depth(vh_volume* volume, const float* depth_in, float* depth_out, const vh_intrinsics* K,
                          void* stream);
/* The filter's per-pixel normals (device buffers): normals 3*W*H floats, valid W*H bytes. */
vh_status vh_depth_normals(vh_volume* volume, const float* depth_in, float* normals, uint8_t* valid,
                           const vh_intrinsics* K, void* stream);

/* The per-pixel normal map of vh_algorithm.normal_mode 1 (device buffers): estimateSurfaceNormalCamera
 * (cuda_tsdf_integrator.cu:754-832) at every pixel centre of depth_in, camera frame, as normals[4*W*H] =
 * (nx, ny, nz, valid 1/0) per pixel; normals 16-byte aligned.  No reference counterpart (the reference
 * evaluates the normal per voxel). */
vh_status vh_pixel_normals(vh_volume* volume, const float* depth_in, float* normals, const vh_intrinsics* K,
                           void* stream);

/* Depth ray-cast of the fused volume (no reference counterpart: the reference renders only its analytic
 * scenes).  For every pixel of K seen from T_wc, the ray is sampled every step_voxels voxels of path length
 * between camera depths min_depth and max_depth; the surface is the one marching cubes extracts, a voxel's
 * observed layers as planes (cuda_mesh_extractor.cu:237-262): at each sample, the trilinear blend of the
 * signed distances, at the sample, of the heaviest camera-facing layer of each of the 8 surrounding voxels
 * (at least half the weight observed); the first crossing from positive to non-positive (a drop
 * of at most the truncation distance) is the hit, interpolated linearly.  depth_out: W*H floats in device
 * memory, camera depth in metres, 0 where no surface is hit.  Asynchronous on the stream. */
vh_status vh_raycast_depth(vh_volume* volume, const vh_intrinsics* K, const vh_pose* T_wc, float min_depth,
                           float max_depth, float step_voxels, float* depth_out, void* stream);

/* Waits for the stream and returns (then clears) the device-side errors accumulated since the last call. */
vh_status vh_synchronize(vh_volume* volume, void* stream);

/* extractMeshCuda: directional multi-layer marching cubes over every block; the triangle soup stays in
 * the volume's device buffer.  *triangle_count receives its size.  Synchronises. */
vh_status vh_extract_mesh(vh_volume* volume, float iso_level, size_t* triangle_count, void* stream);
/* Incremental meshing (no reference counterpart): the same extraction restricted to the blocks the layer
 * update ran over within the last `frames` frames (frames = 0: every block).  Each listed block yields exactly
 * the triangles it yields in a full extraction (neighbour blocks are read as usual); the soup replaces the
 * volume's last extracted soup. */
vh_status vh_extract_mesh_recent(vh_volume* volume, float iso_level, uint32_t frames, size_t* triangle_count,
                                 void* stream);
/* Copies the last extracted soup, 9 floats per triangle (v0, v1, v2), to host or device memory. */
vh_status vh_copy_mesh(vh_volume* volume, float* out, size_t max_triangles, int32_t out_on_device, void* stream);
/* Indexed mesh of the last extracted soup, built on the device (the indexed output of the reference demo's
 * PLY writer, src/main.cpp:337-398, has no counterpart: it writes the soup).  Soup vertices are merged when
 * their float32 coordinates are bit-identical (marching cubes computes an edge's vertex once per cell, so
 * these are exactly the shared vertices).  Vertices are numbered in the order of their first use in the soup;
 * faces keep the soup's order; faces with a repeated vertex or |cross(v1 - v0, v2 - v0)| <= 1e-8 (float32,
 * the PLY writer's test) are dropped.  Deterministic.  Synchronises.  VH_ERR_CAPACITY above about 3.1e8
 * triangles (32-bit indices). */
vh_status vh_weld_mesh(vh_volume* volume, size_t* vertex_count, size_t* face_count, void* stream);
/* Copies the last welded mesh: vertices 3 floats each, faces 3 int32 vertex numbers each. */
vh_status vh_copy_welded_mesh(vh_volume* volume, float* vertices, size_t max_vertices, int32_t* faces,
                              size_t max_faces, int32_t out_on_device, void* stream);

vh_status vh_block_count(vh_volume* volume, uint64_t* count);
vh_status vh_observed_voxel_count(vh_volume* volume, uint64_t* count);
/* Recounts observed voxels from the pool (the incremental counter's cross-check). */
vh_status vh_recount_observed_voxels(vh_volume* volume, uint64_t* count, void* stream);
vh_status vh_frame_stats_get(vh_volume* volume, vh_frame_stats* stats, void* stream);
/* Asynchronous statistics: enqueues on the stream a copy of the volume's 64-byte device counter block into
 * counters64 (host memory; pinned for the copy to be asynchronous), so a caller can read each frame's result
 * without stalling the stream; once the stream has passed that point, vh_frame_stats_decode turns the block
 * into the statistics struct, with the values vh_frame_stats_get returns at that point. */
vh_status vh_frame_stats_enqueue(vh_volume* volume, void* counters64, void* stream);
vh_status vh_frame_stats_decode(const vh_volume* volume, const void* counters64, vh_frame_stats* stats);

/* Blocks [first, first + count) in allocation order: keys (3 int32 each) and voxels in the reference's
 * Voxel layout (include/tsdfmc/voxel_hash_tsdf.h:18-31: 512 voxels x 6 directions x 3 layers x 16 bytes
 * per block), into host memory (out_on_device = 0) or device memory (1).  Either pointer may be NULL. */
vh_status vh_export_blocks(vh_volume* volume, uint64_t first, uint64_t count, int32_t* keys, void* voxels,
                           int32_t out_on_device, void* stream);

/* applyFlatBlocks (include/tsdfmc/voxel_hash_tsdf.h:183-188): inserts or overwrites blocks given as keys
 * (3 int32 each, unique within one call) and voxels in the reference Voxel layout (512 x 6 x 3 x 16 bytes per
 * block), read from host (in_on_device = 0) or device memory (1): the inverse of vh_export_blocks, for
 * checkpoint / resume and for meshing volumes built elsewhere.  New blocks take pool slots in no particular
 * order (the export order of the result may differ from the input order).  Recounts the observed voxels.
 * Synchronises. */
vh_status vh_import_blocks(vh_volume* volume, const int32_t* keys, const void* voxels, uint64_t count,
                           int32_t in_on_device, void* stream);

/* Eviction, for trajectories longer than the pool holds (no reference counterpart: the reference's volume only
 * grows, voxel_hash_tsdf.h:133-139).  Removes every block whose layer update last ran at least min_age_frames
 * frames ago (blocks not updated since they were imported count as oldest) -- and, with target_blocks > 0,
 * also the oldest further blocks until exactly target_blocks remain (blocks of equal age, and all blocks older
 * than 4,095 frames, in pool order) -- after copying them out: keys (3 int32 per
 * block) and contents, format 0 in the reference Voxel layout (147,456 bytes per block, as vh_export_blocks),
 * format 1 as the volume's own block image (147,456 bytes with FP32 layers, 98,304 with FP16 layers), which
 * vh_restore_blocks puts back bit for bit; to host memory (out_on_device = 0) or device memory (1), in
 * ascending pool order.  Either output pointer may be NULL.  *evicted receives the number of blocks; if the
 * buffers hold fewer (max_out), nothing is evicted, *evicted holds the number and the call returns
 * VH_ERR_BUFFER_TOO_SMALL.  The pool stays dense (surviving blocks move into the freed slots), the hash is
 * rebuilt from the surviving keys, the last frame's visible list is cleared and the victims' observed voxels
 * are taken off the count; the last extracted mesh is discarded.  Synchronises. */
vh_status vh_evict_blocks(vh_volume* volume, uint32_t min_age_frames, uint64_t target_blocks, int32_t format,
                          int32_t* keys_out, void* data_out, uint64_t max_out, int32_t out_on_device,
                          uint64_t* evicted, void* stream);
/* Inserts (or overwrites) blocks saved by vh_evict_blocks with format 1, into a volume of the same layer format:
 * the pool receives the saved images unchanged; the blocks count as updated in the current frame.  Recounts the
 * observed voxels.  Synchronises. */
vh_status vh_restore_blocks(vh_volume* volume, const int32_t* keys, const void* data, uint64_t count,
                            int32_t in_on_device, void* stream);

/* The launch shape the autotuner chose for the layer update (vh_algorithm.autotune): variant index (-1 while
 * still tuning or when not tuned), threads per CTA, minimum resident CTAs per SM, and the chosen shape's median
 * time in ms.  No reference counterpart. */
vh_status vh_autotune_result(vh_volume* volume, int32_t* variant, int32_t* threads_per_cta,
                             int32_t* min_ctas_per_sm, float* ms);

/* Stage timing with CUDA events (the reference times its stages with steady_clock, src/main.cpp:424-452).
 * While enabled, vh_integrate brackets each of its kernels with events on the call's stream.
 * vh_profile_read waits for the recorded frames and returns the milliseconds spent in each stage since the
 * last read -- ms[0] filter, ms[1] allocation, ms[2] update preparation (the active-voxel list, or the
 * per-pixel normal map with normal_mode 1), ms[3] layer update -- and how many frames they cover. */
vh_status vh_profile_enable(vh_volume* volume, int32_t enable);
vh_status vh_profile_read(vh_volume* volume, double ms[4], uint64_t* frames);

/* Workload generator, not a reference interface: ray-casts the analytic benchmark scenes the way the
 * reference's demo renders its synthetic frames (src/main.cpp:189-335) -- primitives `prims` (device memory,
 * n_prims x 10 floats: type, a.xyz, b.xyz, r, h, 0; types plane / sphere / box / vertical cylinder / room
 * interior) seen from T_wc, depth = camera-space z, plus N(0, (sigma_z2 z^2)^2) noise and `dropout` zeroed
 * pixels from a counter-based hash of (seed, frame, pixel); returns outside (0.1, max_depth) are zeroed.
 * depth_out: width*height floats in device memory. */
vh_status vh_render_depth(const float* prims, int32_t n_prims, const vh_intrinsics* K, const vh_pose* T_wc,
                          uint32_t seed, uint32_t frame, float sigma_z2, float dropout, float max_depth,
                          float* depth_out, void* stream);

/* ---- The device exponential (diagnostics) ----
 * The reference's Gaussian weights call expf (src/cuda_tsdf_integrator.cu:173-175); on a host that is the C
 * library's expf.  The plain form evaluates them with a device restatement of that function which returns the
 * same float for every argument.  vh_expf_eval: y[i] = that exponential of x[i] (device buffers, n floats),
 * asynchronous on the stream.  vh_expf_check: for every float whose bit pattern lies in
 * [first_bits, first_bits + count), compares the restatement's fast single-precision path with its
 * double-precision sequence (the C library's operations) on the device; *mismatches receives the number of
 * arguments (NaNs excluded) whose results differ and *first_mismatch the smallest such bit pattern
 * (0xffffffff if none).  Synchronises. */
vh_status vh_expf_eval(const float* x, float* y, uint64_t n, void* stream);
vh_status vh_expf_check(uint32_t first_bits, uint64_t count, uint64_t* mismatches, uint32_t* first_mismatch,
                        void* stream);

/* ---- Multi-scene batch (no reference counterpart) ----
 * Many independent volumes fused together: each vh_batch_integrate call is one step in which every active
 * scene integrates one depth frame.  The step runs as three work-queue kernels over all scenes' work (filter
 * tiles; allocation and normal-map tiles; chunks of visible voxels), so small and large scenes share the GPU
 * without per-scene launches.  use_graph 0: the step's kernels are launched one after another; 1: the step
 * (descriptor upload, queue reset, three kernels) is one CUDA graph launch; 2: the step is one persistent
 * cooperative launch whose phases are separated by grid-wide barriers (waits bounded to about a second; a wait
 * that gives up sets VH_ERR_TIMEOUT on the step's volumes).  Volumes: same device, vh_algorithm.normal_mode 1
 * (the per-pixel normal map) and the same
 * fast_math setting; at most 256 per batch; a volume keeps its own counters and statistics
 * (vh_frame_stats_get, vh_synchronize).  Results equal integrating each scene alone with the same settings. */
typedef struct vh_batch vh_batch;
vh_status vh_batch_create(vh_volume* const* volumes, int32_t count, int32_t use_graph, vh_batch** out);
void vh_batch_destroy(vh_batch* batch);
/* depth_device[i]: device pointer of scene i's depth (K[i].width x K[i].height floats); active may be NULL (all
 * active), else scenes with active[i] == 0 skip the step.  Asynchronous on the stream. */
vh_status vh_batch_integrate(vh_batch* batch, const float* const* depth_device, const vh_intrinsics* K,
                             const vh_pose* T_wc, const int32_t* active, int32_t stride, void* stream);

/* ---- Learned depth denoiser: building blocks (no reference counterpart) ----
 * Activations are NHWC BF16 with 32 channels (64 bytes per pixel), device memory, 16-byte aligned.
 * vh_nn_pack_conv32_weights: FP32 weights w[co][ci][3][3] (32 x 32) -> the packed BF16 tensor-core operand
 * (18,432 bytes); transpose_flip packs w[ci][co][2-ky][2-kx], the weights of the input gradient.
 * vh_nn_conv32: 3x3 convolution with zero padding on the tensor cores (tcgen05, FP32 accumulation); mode 0:
 * out = conv(in) + bias, then ReLU if relu; mode 1: out = conv(in) where mask > 0, else 0.  *error gets
 * the timeout bit (8) if a wait on the loads or the tensor cores gave up (about a second). */
vh_status vh_nn_pack_conv32_weights(const float* w, void* packed, int32_t transpose_flip, void* stream);
vh_status vh_nn_conv32(const void* in, const void* packed_w, const float* bias, const void* mask, void* out,
                       int32_t batch, int32_t width, int32_t height, int32_t mode, int32_t relu, uint32_t* error,
                       void* stream);
/* vh_nn_wgrad32: weight and bias gradients of a 32 -> 32 3x3 convolution with zero padding on the tensor cores
 * (tcgen05, FP32 accumulation): dw[co][ci][ky][kx] += sum_p grad[p][co] x[p + (ky - 1, kx - 1)][ci] and
 * db[co] += sum_p grad[p][co] over the batch (x: the layer input, grad: the gradient at the layer output, NHWC
 * BF16 with 32 channels; dw: 9,216 and db: 32 FP32, device memory, accumulated into).  *error: as vh_nn_conv32. */
vh_status vh_nn_wgrad32(const void* x, const void* grad, float* dw, float* db, int32_t batch, int32_t width,
                        int32_t height, uint32_t* error, void* stream);
/* vh_nn_conv32 whose input loads start only once *gate (device memory) is nonzero.  A gate that stays zero
 * makes every wait of the kernel give up after about a second: *error gets the timeout bit (8, which the
 * volume calls report as VH_ERR_TIMEOUT), `out` is left unwritten and the CUDA context stays usable.  This is
 * how the bounded-wait path is tested without a GPU fault; with an open gate the result equals vh_nn_conv32's. */
vh_status vh_nn_conv32_gated(const void* in, const void* packed_w, const float* bias, const void* mask, void* out,
                             int32_t batch, int32_t width, int32_t height, int32_t mode, int32_t relu,
                             const uint32_t* gate, uint32_t* error, void* stream);

/* The whole denoiser (3x3 convolutions 4 -> 32 -> 32 -> 32 -> 1, ReLU, residual output; the two 32 -> 32 layers
 * on the tensor cores).  params: FP32 [vh_nn_param_count()] = w1[32][4][3][3] b1[32] w2[32][32][3][3] b2[32]
 * w3[32][32][3][3] b3[32] w4[32][3][3] b4; packed: 73,728 bytes (vh_nn_pack); workspace: vh_nn_workspace_bytes;
 * depth, out, target: batch x height x width FP32, device memory.  vh_nn_backward reads the activations
 * vh_nn_forward left in the same workspace and writes the FP32 gradients of the loss
 * sum((out - target)^2) / (batch * height * width) over pixels valid in depth, target and out, and
 * loss[0..1] = (sum of squared errors, pixel count); pixels whose depth and target differ by more than the
 * reference's discontinuity threshold max(0.012, 0.025 * target) are left out (they see different surfaces).
 * Inside vh_integrate, a correction larger than that threshold falls back to the bilateral filter's value.
 * error: as vh_nn_conv32. */
int32_t vh_nn_param_count(void);
uint64_t vh_nn_workspace_bytes(int32_t batch, int32_t width, int32_t height);
vh_status vh_nn_pack(const float* params, void* packed, void* stream);
vh_status vh_nn_forward(const float* params, const void* packed, const float* depth, float* out, int32_t batch,
                        int32_t width, int32_t height, void* workspace, uint32_t* error, void* stream);
vh_status vh_nn_backward(const float* params, const void* packed, const float* depth, const float* target,
                         const float* out, int32_t batch, int32_t width, int32_t height, void* workspace, float* grads,
                         float* loss, uint32_t* error, void* stream);
/* one Adam step (FP32 moments m, v; step counts from 1) */
vh_status vh_nn_adam(float* params, const float* grads, float* m, float* v, float lr, float beta1, float beta2,
                     float eps, int32_t step, void* stream);
/* Uses the denoiser with these parameters (host memory, vh_nn_param_count() floats) in place of the bilateral
 * filter in vh_integrate when vh_algorithm.depth_filter is 1; params NULL clears it. */
vh_status vh_set_depth_denoiser(vh_volume* volume, const float* params);

/* ---- Dataset reader: include/tsdfmc/dataset_io.h, portable ----
 * Layout: <root>/<frame id>/depth.png and <root>/<frame id>/<pose file>; the frame ids are the all-digit
 * directory names, ascending (listDatasetFrameIds, :135-152).  These calls touch no GPU.  On failure they
 * return VH_ERR_IO / VH_ERR_FORMAT / VH_ERR_INVALID_ARGUMENT and vh_dataset_last_error() holds the message
 * the reference would throw (thread-local). */
const char* vh_dataset_last_error(void);
/* listDatasetFrameIds: ids may be NULL (count only); VH_ERR_BUFFER_TOO_SMALL when max_ids < *count. */
vh_status vh_dataset_list_frames(const char* root, int32_t* ids, size_t max_ids, size_t* count);
/* loadDatasetIntrinsics (:382-395): metadata of 5 (fx fy cx cy depth_scale), 6 (fx fy cx cy width height) or
 * 7 (fx fy cx cy width height depth_scale) numbers; a missing file falls back to the first
 * <root>/<frame>/params.txt; without a resolution, the size of the first depth.png completes it. */
vh_status vh_dataset_load_intrinsics(const char* metadata_path, vh_intrinsics* K, float* depth_scale);
/* loadPoseFromFile (:154-188): 7 numbers (quaternion w x y z, translation) or 12/16 (row-major 3x4 / 4x4). */
vh_status vh_dataset_load_pose(const char* path, vh_pose* T_wc);
/* Any grayscale PNG (bit depth 1-16, optional alpha, optional Adam7) as 16-bit gray, the conversion the
 * reference requests from WIC (:321-330).  pixels may be NULL (size probe); else max_pixels >= W*H. */
vh_status vh_png_read_gray16(const char* path, uint16_t* pixels, size_t max_pixels, int32_t* width, int32_t* height);
/* loadDepthPng (:276-361): depth[i] = raw[i] * depth_scale where raw != 0 and the product > 0, else 0 (host
 * buffer of K->width * K->height floats); the PNG size must equal K's.  *valid_samples = nonzero depths. */
vh_status vh_dataset_load_depth_png(const char* path, const vh_intrinsics* K, float depth_scale, float* depth,
                                    uint64_t* valid_samples);

#ifdef __cplusplus
}
#endif
#endif /* VOXELHASH_GB300_H */
