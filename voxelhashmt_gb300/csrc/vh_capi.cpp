// vh_capi.cpp -- the C ABI of include/voxelhash_gb300.h: volume lifetime, buffers, launch sequences.
//
// Host code is compiled with -ffp-contract=off: the world->camera pose (Pose::inverse, math_types.h:192-197)
// and the 1/(2 sigma^2) factors are float expressions whose rounding must match the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/voxelhash_gb300.h"
#include "vh_common.cuh"
#include "vh_kernels.h"
#include "vh_nn.h"

struct vh_volume {
  vh_params params{};
  vh_algorithm algo{};
  vh::Volume dev{};
  vh::Counters* h_counters = nullptr;  // pinned mirror for read-back
  float* d_depth_in = nullptr;
  // vh_integrate's host depth is staged through two device buffers filled on an internal copy stream: the copy
  // of the next frame overlaps this frame's kernels.  stage_copied[k]: buffer k holds its frame; stage_free[k]:
  // the kernels that read buffer k are done (recorded once stage_used[k]).
  float* d_depth_stage[2] = {nullptr, nullptr};
  size_t stage_capacity = 0;  // pixels
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t stage_copied[2] = {nullptr, nullptr};
  cudaEvent_t stage_free[2] = {nullptr, nullptr};
  bool stage_used[2] = {false, false};
  int stage_next = 0;
  float* d_depth_filtered = nullptr;
  float4* d_normal_map = nullptr;  // per-pixel normals (vh_algorithm.normal_mode 1)
  // learned depth denoiser (vh_algorithm.depth_filter 1)
  float* d_nn_params = nullptr;
  float* d_depth_bilateral = nullptr;  // the fallback of the learned filter
  __nv_bfloat16* d_nn_packed = nullptr;
  unsigned char* d_nn_ws = nullptr;
  size_t nn_ws_bytes = 0;
  // launch-shape autotuner of the fused update (vh_algorithm.autotune): frames cycle through the variants,
  // each timed with a pair of events, until every variant has kTuneRounds samples; then the fastest is kept
  int tuned_variant = -1;
  int tune_frames = 0;
  std::vector<std::array<cudaEvent_t, 2>> tune_events;
  std::vector<int> tune_variant_of;
  float tune_best_ms = 0.0f;
  size_t depth_capacity = 0;  // pixels
  uint32_t* d_mc_counts = nullptr;
  uint32_t* d_mc_dir_totals = nullptr;
  uint8_t* d_mc_cell_counts = nullptr;
  unsigned long long* d_mc_offsets = nullptr;
  uint32_t* d_mc_list = nullptr;        // incremental meshing: the selected pool blocks
  uint32_t* d_mc_list_count = nullptr;
  unsigned long long* d_scalar = nullptr;  // [0] mesh total, [1] recount
  float* d_tris = nullptr;
  size_t tri_capacity = 0;
  size_t mesh_triangles = 0;
  // indexed mesh of the last extraction (vh_weld_mesh)
  vh::WeldBuffers weld{};
  size_t weld_capacity = 0;  // triangles
  size_t weld_vertices = 0;
  size_t weld_faces = 0;
  int* d_keys = nullptr;
  float4* d_export = nullptr;
  int* d_export_keys = nullptr;
  uint32_t* d_import_idx = nullptr;
  size_t export_capacity = 0;  // blocks
  // eviction scratch (vh_evict_blocks): victim and source lists (max_blocks words each), per-CTA scan counts,
  // age histogram, two totals
  uint32_t* d_evict_list = nullptr;
  uint32_t* d_evict_src = nullptr;
  uint32_t* d_evict_cta = nullptr;
  uint32_t* d_evict_hist = nullptr;
  uint32_t* d_evict_total = nullptr;
  bool profile = false;
  std::vector<cudaEvent_t> event_pool;
  std::vector<std::vector<cudaEvent_t>> profiled;  // 4 events per recorded frame
  std::string error;
};

namespace {

// one block in the reference Voxel layout / the FP32 pool (16-byte layer records)
constexpr size_t kBlockBytes = static_cast<size_t>(vh::kDirs) * vh::kBlockVoxels * vh::kLayers * sizeof(float4);
// one block of the FP16 pool (32-byte bins)
constexpr size_t kBlockBytes16 = static_cast<size_t>(vh::kDirs) * vh::kBlockVoxels * vh::kBinWords16 * sizeof(uint4);
constexpr size_t kExportChunk = 1024;  // blocks per export staging pass

class DeviceGuard {
 public:
  explicit DeviceGuard(int device) {
    if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
    if (prev_ != device) cudaSetDevice(device);
  }
  ~DeviceGuard() {
    if (prev_ >= 0) cudaSetDevice(prev_);
  }

 private:
  int prev_ = -1;
};

vh_status fail(vh_volume* v, vh_status s, const std::string& msg) {
  if (v) v->error = msg;
  return s;
}

vh_status cuda_fail(vh_volume* v, cudaError_t e, const char* what) {
  const vh_status s = e == cudaErrorMemoryAllocation ? VH_ERR_OUT_OF_MEMORY : VH_ERR_CUDA;
  return fail(v, s, std::string(what) + " failed: " + cudaGetErrorString(e));
}

#define VH_CUDA(v, call)                                        \
  do {                                                          \
    const cudaError_t vh_e_ = (call);                           \
    if (vh_e_ != cudaSuccess) return cuda_fail((v), vh_e_, #call); \
  } while (0)

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

template <class T>
cudaError_t dalloc(T** p, size_t count) {
  return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T));
}

template <class T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

bool valid_intrinsics(const vh_intrinsics* K) {
  return K && K->width > 0 && K->height > 0 && K->fx != 0.0f && K->fy != 0.0f;
}

vh::Params make_params(const vh_volume* v, const vh_intrinsics* K, const vh_pose* T, int stride) {
  vh::Params p{};
  const vh_algorithm& a = v->algo;
  p.width = K->width;
  p.height = K->height;
  p.fx = K->fx;
  p.fy = K->fy;
  p.cx = K->cx;
  p.cy = K->cy;
  if (T) {
    for (int i = 0; i < 9; ++i) p.T_wc.r[i] = T->R[i];
    for (int i = 0; i < 3; ++i) p.T_wc.t[i] = T->t[i];
    // Pose::inverse: R' = R^T, t' = R' * (t * -1)
    const float* R = T->R;
    const float Rt[9] = {R[0], R[3], R[6], R[1], R[4], R[7], R[2], R[5], R[8]};
    const float nt[3] = {T->t[0] * -1.0f, T->t[1] * -1.0f, T->t[2] * -1.0f};
    for (int i = 0; i < 9; ++i) p.T_cw.r[i] = Rt[i];
    for (int i = 0; i < 3; ++i) p.T_cw.t[i] = Rt[3 * i] * nt[0] + Rt[3 * i + 1] * nt[1] + Rt[3 * i + 2] * nt[2];
  }
  const float vs = v->params.voxel_size;
  p.voxel_size = vs;
  p.truncation = v->params.truncation_distance;
  p.block_world_size = vs * 8.0f;
  p.stride = std::max(1, stride);
  p.sample_width = (K->width + p.stride - 1) / p.stride;
  p.sample_height = (K->height + p.stride - 1) / p.stride;
  p.disc_base = a.depth_discontinuity_base;
  p.disc_rel = a.depth_discontinuity_relative;
  p.filter_radius = a.filter_radius;
  p.filter_k_spatial = 1.0f / (2.0f * a.filter_sigma_spatial * a.filter_sigma_spatial);
  p.filter_k_range = 1.0f / (2.0f * a.filter_sigma_range * a.filter_sigma_range);
  p.filter_k_angular = 1.0f / (2.0f * a.filter_sigma_angular * a.filter_sigma_angular);
  p.filter_min_cos = a.filter_min_cosine;
  p.normal_radius = a.normal_radius;
  p.normal_k_spatial = 1.0f / (2.0f * a.normal_sigma_spatial * a.normal_sigma_spatial);
  p.normal_k_range = 1.0f / (2.0f * a.normal_sigma_range * a.normal_sigma_range);
  p.normal_k_angular = 1.0f / (2.0f * a.normal_sigma_angular * a.normal_sigma_angular);
  p.merge_tol = std::max(1e-6f, vs * a.layer_merge_voxel_scale);
  p.layer_normal_cos = a.layer_normal_cosine;
  p.extract_tol = std::max(1e-6f, vs * a.layer_extract_voxel_scale);
  p.max_weight = a.max_voxel_weight;
  p.depth_sigma = a.depth_sigma;
  p.huber_delta = a.huber_delta;
  p.min_obs_weight = a.min_observation_weight;
  p.min_view_weight = a.min_view_angle_weight;
  p.iso = 0.0f;
  p.alloc_mode = a.allocation_mode;
  p.normal_mode = a.normal_mode;
  return p;
}

size_t pool_block_bytes(const vh_volume* v) { return v->dev.layers16 ? kBlockBytes16 : kBlockBytes; }
void* pool_base(const vh_volume* v) {
  return v->dev.layers16 ? static_cast<void*>(v->dev.layers16) : static_cast<void*>(v->dev.layers);
}

vh_status ensure_depth(vh_volume* v, size_t pixels) {
  if (pixels <= v->depth_capacity) return VH_OK;
  dfree(v->d_depth_in);
  dfree(v->d_depth_filtered);
  dfree(v->d_normal_map);
  dfree(v->d_depth_bilateral);
  v->depth_capacity = 0;
  VH_CUDA(v, dalloc(&v->d_depth_in, pixels));
  VH_CUDA(v, dalloc(&v->d_depth_filtered, pixels));
  if (v->algo.depth_filter == 1) VH_CUDA(v, dalloc(&v->d_depth_bilateral, pixels));
  if (v->algo.normal_mode == 1) VH_CUDA(v, dalloc(&v->d_normal_map, pixels));
  v->depth_capacity = pixels;
  return VH_OK;
}

vh_status read_counters(vh_volume* v, cudaStream_t s) {
  VH_CUDA(v, cudaMemcpyAsync(v->h_counters, v->dev.counters, sizeof(vh::Counters), cudaMemcpyDeviceToHost, s));
  VH_CUDA(v, cudaStreamSynchronize(s));
  return VH_OK;
}

vh_status stage_depth(vh_volume* v, const float* depth, int on_device, const vh_intrinsics* K, cudaStream_t s,
                      const float** src) {
  const size_t pixels = static_cast<size_t>(K->width) * static_cast<size_t>(K->height);
  const vh_status st = ensure_depth(v, pixels);
  if (st != VH_OK) return st;
  if (on_device) {
    *src = depth;
  } else {
    VH_CUDA(v, cudaMemcpyAsync(v->d_depth_in, depth, pixels * sizeof(float), cudaMemcpyHostToDevice, s));
    *src = v->d_depth_in;
  }
  return VH_OK;
}

// vh_integrate's staging of host depth (see vh_volume::d_depth_stage): the copy runs on the copy stream into
// the buffer whose last readers have finished, and stream s waits for it.  *slot: the buffer, whose readers
// record stage_free[*slot] on s when they have been enqueued (stage_release).
vh_status stage_depth_overlapped(vh_volume* v, const float* depth, const vh_intrinsics* K, cudaStream_t s,
                                 const float** src, int* slot) {
  const size_t pixels = static_cast<size_t>(K->width) * static_cast<size_t>(K->height);
  const vh_status st = ensure_depth(v, pixels);
  if (st != VH_OK) return st;
  if (!v->copy_stream) {
    VH_CUDA(v, cudaStreamCreateWithFlags(&v->copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      VH_CUDA(v, cudaEventCreateWithFlags(&v->stage_copied[k], cudaEventDisableTiming));
      VH_CUDA(v, cudaEventCreateWithFlags(&v->stage_free[k], cudaEventDisableTiming));
    }
  }
  if (pixels > v->stage_capacity) {
    for (int k = 0; k < 2; ++k) {
      if (v->stage_used[k]) VH_CUDA(v, cudaEventSynchronize(v->stage_free[k]));
      dfree(v->d_depth_stage[k]);
    }
    VH_CUDA(v, cudaStreamSynchronize(v->copy_stream));
    v->stage_capacity = 0;
    for (int k = 0; k < 2; ++k) VH_CUDA(v, dalloc(&v->d_depth_stage[k], pixels));
    v->stage_capacity = pixels;
  }
  const int k = v->stage_next;
  v->stage_next ^= 1;
  if (v->stage_used[k]) VH_CUDA(v, cudaStreamWaitEvent(v->copy_stream, v->stage_free[k], 0));
  VH_CUDA(v, cudaMemcpyAsync(v->d_depth_stage[k], depth, pixels * sizeof(float), cudaMemcpyHostToDevice,
                             v->copy_stream));
  VH_CUDA(v, cudaEventRecord(v->stage_copied[k], v->copy_stream));
  VH_CUDA(v, cudaStreamWaitEvent(s, v->stage_copied[k], 0));
  *src = v->d_depth_stage[k];
  *slot = k;
  return VH_OK;
}

// the kernels reading staging buffer slot (all enqueued on s) are done when s reaches this point
vh_status stage_release(vh_volume* v, int slot, cudaStream_t s) {
  if (slot < 0) return VH_OK;
  VH_CUDA(v, cudaEventRecord(v->stage_free[slot], s));
  v->stage_used[slot] = true;
  return VH_OK;
}

uint64_t block_total(const vh_volume* v) {
  return std::min<uint64_t>(v->h_counters->num_blocks, v->dev.max_blocks);
}

constexpr int kTuneStart = 24;  // frames before tuning starts: the first frames of a volume update far more
                                // voxels (everything is new) than the steady state the choice is for
constexpr int kTuneRounds = 4;

// Chooses the fused-update variant of this frame.  Until kTuneStart frames have run, the first variant; then,
// while tuning, the next variant in the cycle and a pair of events to record around its launch; once every
// variant has kTuneRounds samples, waits for the last one, keeps the variant with the smallest median time
// and frees the events.
vh_status autotune_step(vh_volume* v, int* variant, cudaEvent_t ev[2]) {
  ev[0] = ev[1] = nullptr;
  if (v->tuned_variant >= 0) {
    *variant = v->tuned_variant;
    return VH_OK;
  }
  const int nvar = v->algo.fast_math ? vh::fast::fused_variant_count() : vh::exact::fused_variant_count();
  if (v->tune_frames < kTuneStart) {
    *variant = 0;
    ++v->tune_frames;
    return VH_OK;
  }
  if (v->tune_frames < kTuneStart + nvar * kTuneRounds) {
    *variant = (v->tune_frames - kTuneStart) % nvar;
    std::array<cudaEvent_t, 2> pair{};
    VH_CUDA(v, cudaEventCreate(&pair[0]));
    VH_CUDA(v, cudaEventCreate(&pair[1]));
    v->tune_events.push_back(pair);
    v->tune_variant_of.push_back(*variant);
    ev[0] = pair[0];
    ev[1] = pair[1];
    ++v->tune_frames;
    return VH_OK;
  }
  VH_CUDA(v, cudaEventSynchronize(v->tune_events.back()[1]));
  std::vector<std::vector<float>> times(nvar);
  for (size_t i = 0; i < v->tune_events.size(); ++i) {
    float ms = 0.0f;
    VH_CUDA(v, cudaEventElapsedTime(&ms, v->tune_events[i][0], v->tune_events[i][1]));
    times[v->tune_variant_of[i]].push_back(ms);
  }
  int best = 0;
  float best_ms = 0.0f;
  for (int k = 0; k < nvar; ++k) {
    std::sort(times[k].begin(), times[k].end());
    const float med = times[k][times[k].size() / 2];
    if (k == 0 || med < best_ms) {
      best = k;
      best_ms = med;
    }
  }
  for (auto& pair : v->tune_events) {
    cudaEventDestroy(pair[0]);
    cudaEventDestroy(pair[1]);
  }
  v->tune_events.clear();
  v->tune_variant_of.clear();
  v->tuned_variant = best;
  v->tune_best_ms = best_ms;
  *variant = best;
  return VH_OK;
}

void free_weld(vh_volume* v) {
  vh::WeldBuffers& W = v->weld;
  dfree(W.slot_first);
  dfree(W.vslot);
  dfree(W.vid);
  dfree(W.flags);
  dfree(W.number);
  dfree(W.sums);
  dfree(W.verts);
  dfree(W.faces);
  dfree(W.counts);
  W.slot_mask = 0U;
  v->weld_capacity = 0;
}

// weld buffers for a soup of `triangles` triangles (3 * triangles < 2^30)
vh_status ensure_weld(vh_volume* v, size_t triangles) {
  if (triangles <= v->weld_capacity && v->weld.counts) return VH_OK;
  free_weld(v);
  const size_t cap = std::max<size_t>(triangles + triangles / 8, 1024);
  const size_t nv = 3 * cap;
  size_t slots = 1024;
  while (slots < 2 * nv) slots <<= 1;  // load factor <= 1/2
  vh::WeldBuffers& W = v->weld;
  VH_CUDA(v, dalloc(&W.slot_first, slots));
  VH_CUDA(v, dalloc(&W.vslot, nv));
  VH_CUDA(v, dalloc(&W.vid, nv));
  VH_CUDA(v, dalloc(&W.flags, nv));
  VH_CUDA(v, dalloc(&W.number, nv));
  VH_CUDA(v, dalloc(&W.sums, vh::weld_scan_tiles(static_cast<uint32_t>(nv))));
  VH_CUDA(v, dalloc(&W.verts, 3 * nv));
  VH_CUDA(v, dalloc(&W.faces, nv));
  VH_CUDA(v, dalloc(&W.counts, 3));
  W.slot_mask = static_cast<uint32_t>(slots - 1);
  v->weld_capacity = cap;
  return VH_OK;
}

}  // namespace

extern "C" {

void vh_params_default(vh_params* p) {
  if (!p) return;
  p->voxel_size = 0.01f;
  p->truncation_distance = 0.04f;
  p->hash_buckets = 1u << 16;
  p->max_blocks = 1u << 14;
  p->device = 0;
  p->layer_format = 0;
}

void vh_algorithm_default(vh_algorithm* a) {
  if (!a) return;
  a->depth_discontinuity_base = 0.012f;     // cuda_tsdf_integrator.cu:27
  a->depth_discontinuity_relative = 0.025f; // :28
  a->filter_radius = 2;                     // :31
  a->filter_sigma_spatial = 1.5f;           // :32
  a->filter_sigma_range = 0.0012f;          // :33
  a->filter_sigma_angular = 0.35f;          // :34
  a->filter_min_cosine = 0.9f;              // :35
  a->normal_radius = 1;                     // :23
  a->normal_sigma_spatial = 1.0f;           // :24
  a->normal_sigma_range = 0.0012f;          // :25
  a->normal_sigma_angular = 0.35f;          // :26
  a->layer_merge_voxel_scale = 0.25f;       // :29
  a->layer_normal_cosine = 0.9f;            // :30
  a->layer_extract_voxel_scale = 0.55f;     // cuda_mesh_extractor.cu:20
  a->max_voxel_weight = 100.0f;             // cuda_tsdf_integrator.cu:18
  a->depth_sigma = 1.5f;                    // :19
  a->huber_delta = 0.35f;                   // :20
  a->min_observation_weight = 0.05f;        // :21
  a->min_view_angle_weight = 0.15f;         // :22
  a->allocation_mode = 0;
  a->fast_math = 0;
  a->normal_mode = 0;
  a->autotune = 1;
  a->launch_variant = 0;
  a->depth_filter = 0;
}

const char* vh_status_string(vh_status s) {
  switch (s) {
    case VH_OK: return "ok";
    case VH_ERR_INVALID_ARGUMENT: return "invalid argument";
    case VH_ERR_CUDA: return "CUDA error";
    case VH_ERR_NO_DEVICE: return "no CUDA device";
    case VH_ERR_OUT_OF_MEMORY: return "out of device memory";
    case VH_ERR_KEY_RANGE: return "block coordinate outside the 21-bit packed key range";
    case VH_ERR_HASH_FULL: return "block hash table full";
    case VH_ERR_POOL_FULL: return "block pool full";
    case VH_ERR_BUFFER_TOO_SMALL: return "output buffer too small";
    case VH_ERR_CAPACITY: return "request larger than the fixed static scratch";
    case VH_ERR_IO: return "dataset file missing, unreadable or unparsable";
    case VH_ERR_FORMAT: return "unsupported or corrupt PNG or metadata layout";
    case VH_ERR_TIMEOUT: return "a bounded device-side wait gave up";
  }
  return "unknown status";
}

vh_status vh_query_device(char* message, size_t len) {
  int count = 0;
  const cudaError_t e = cudaGetDeviceCount(&count);
  char buf[256];
  vh_status st = VH_OK;
  if (e != cudaSuccess) {
    std::snprintf(buf, sizeof(buf), "%s", cudaGetErrorString(e));
    st = VH_ERR_NO_DEVICE;
  } else if (count <= 0) {
    std::snprintf(buf, sizeof(buf), "no CUDA device detected");
    st = VH_ERR_NO_DEVICE;
  } else {
    std::snprintf(buf, sizeof(buf), "%d CUDA device(s) detected", count);
  }
  if (message && len) {
    std::strncpy(message, buf, len - 1);
    message[len - 1] = '\0';
  }
  return st;
}

vh_status vh_create(const vh_params* params, const vh_algorithm* algo, vh_volume** out) {
  if (!params || !out) return VH_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const uint32_t buckets = params->hash_buckets;
  if (!(params->voxel_size > 0.0f) || !(params->truncation_distance > 0.0f) || buckets < 2 ||
      (buckets & (buckets - 1)) != 0 || params->max_blocks > (1u << 23) || params->layer_format < 0 ||
      params->layer_format > 1) {
    return VH_ERR_INVALID_ARGUMENT;  // pool indices are packed with the voxel index in 32 bits
  }
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || params->device < 0 || params->device >= count) {
    return VH_ERR_NO_DEVICE;
  }
  vh_volume* v = new (std::nothrow) vh_volume();
  if (!v) return VH_ERR_OUT_OF_MEMORY;
  v->params = *params;
  if (algo) {
    v->algo = *algo;
  } else {
    vh_algorithm_default(&v->algo);
  }
  if (v->algo.filter_radius < 0 || v->algo.filter_radius > 2 || v->algo.normal_radius != 1 ||
      v->algo.allocation_mode < 0 || v->algo.allocation_mode > 1 || v->algo.fast_math < 0 || v->algo.fast_math > 1 ||
      v->algo.normal_mode < 0 || v->algo.normal_mode > 1 || v->algo.autotune < 0 || v->algo.autotune > 1 ||
      v->algo.launch_variant < 0 || v->algo.launch_variant >= vh::exact::fused_variant_count() ||
      v->algo.depth_filter < 0 || v->algo.depth_filter > 1) {
    delete v;
    return VH_ERR_INVALID_ARGUMENT;
  }
  DeviceGuard guard(params->device);
  vh::Volume& V = v->dev;
  V.capacity = buckets;
  V.mask = buckets - 1;
  V.max_blocks = params->max_blocks;
  const size_t nb = params->max_blocks;
  cudaError_t e = cudaSuccess;
  auto step = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  step(dalloc(&V.slot_keys, buckets));
  step(dalloc(&V.slot_block, buckets));
  step(dalloc(&V.slot_stamp, buckets));
  step(dalloc(&V.visible, buckets));
  step(dalloc(&V.visible_keys, buckets));
  step(dalloc(&V.active, nb * vh::kBlockVoxels));
  V.voxel_size = params->voxel_size;
  V.inv_voxel_size = 1.0f / params->voxel_size;
  if (params->layer_format == 1) {
    step(cudaMalloc(reinterpret_cast<void**>(&V.layers16), std::max<size_t>(nb, 1) * kBlockBytes16));
  } else {
    step(cudaMalloc(reinterpret_cast<void**>(&V.layers), std::max<size_t>(nb, 1) * kBlockBytes));
  }
  step(dalloc(&V.block_keys, nb));
  step(dalloc(&V.obs_mask, nb * (vh::kBlockVoxels / 32)));
  step(dalloc(&V.dir_mask, nb));
  step(dalloc(&V.block_stamp, nb));
  step(dalloc(&V.counters, 1));
  step(cudaMallocHost(reinterpret_cast<void**>(&v->h_counters), sizeof(vh::Counters)));
  step(dalloc(&v->d_scalar, 2));
  if (e == cudaSuccess) {
    step(cudaMemset(V.slot_keys, 0xFF, buckets * sizeof(unsigned long long)));
    step(cudaMemset(V.slot_block, 0xFF, buckets * sizeof(uint32_t)));
    step(cudaMemset(V.slot_stamp, 0, buckets * sizeof(uint32_t)));
    step(cudaMemset(pool_base(v), 0, std::max<size_t>(nb, 1) * pool_block_bytes(v)));
    step(cudaMemset(V.obs_mask, 0, nb * (vh::kBlockVoxels / 32) * sizeof(uint32_t)));
    step(cudaMemset(V.dir_mask, 0, std::max<size_t>(nb, 1) * sizeof(uint32_t)));
    step(cudaMemset(V.block_stamp, 0, std::max<size_t>(nb, 1) * sizeof(uint32_t)));
    step(cudaMemset(V.counters, 0, sizeof(vh::Counters)));
    step(cudaDeviceSynchronize());
  }
  if (e != cudaSuccess) {
    const vh_status st = e == cudaErrorMemoryAllocation ? VH_ERR_OUT_OF_MEMORY : VH_ERR_CUDA;
    cudaGetLastError();
    vh_destroy(v);
    return st;
  }
  std::memset(v->h_counters, 0, sizeof(vh::Counters));
  *out = v;
  return VH_OK;
}

void vh_destroy(vh_volume* v) {
  if (!v) return;
  DeviceGuard guard(v->params.device);
  vh::Volume& V = v->dev;
  dfree(V.slot_keys);
  dfree(V.slot_block);
  dfree(V.slot_stamp);
  dfree(V.visible);
  dfree(V.visible_keys);
  dfree(V.active);
  dfree(V.layers);
  dfree(V.layers16);
  dfree(V.block_keys);
  dfree(V.obs_mask);
  dfree(V.dir_mask);
  dfree(V.block_stamp);
  dfree(V.counters);
  dfree(v->d_evict_list);
  dfree(v->d_evict_src);
  dfree(v->d_evict_cta);
  dfree(v->d_evict_hist);
  dfree(v->d_evict_total);
  if (v->h_counters) cudaFreeHost(v->h_counters);
  dfree(v->d_depth_in);
  if (v->copy_stream) {
    cudaStreamSynchronize(v->copy_stream);
    cudaStreamDestroy(v->copy_stream);
  }
  for (int k = 0; k < 2; ++k) {
    dfree(v->d_depth_stage[k]);
    if (v->stage_copied[k]) cudaEventDestroy(v->stage_copied[k]);
    if (v->stage_free[k]) cudaEventDestroy(v->stage_free[k]);
  }
  dfree(v->d_depth_filtered);
  dfree(v->d_normal_map);
  dfree(v->d_nn_params);
  dfree(v->d_nn_packed);
  dfree(v->d_nn_ws);
  dfree(v->d_depth_bilateral);
  for (auto& pair : v->tune_events) {
    cudaEventDestroy(pair[0]);
    cudaEventDestroy(pair[1]);
  }
  dfree(v->d_mc_counts);
  dfree(v->d_mc_dir_totals);
  dfree(v->d_mc_cell_counts);
  dfree(v->d_mc_offsets);
  dfree(v->d_mc_list);
  dfree(v->d_mc_list_count);
  dfree(v->d_scalar);
  dfree(v->d_tris);
  free_weld(v);
  dfree(v->d_keys);
  dfree(v->d_export);
  dfree(v->d_export_keys);
  dfree(v->d_import_idx);
  for (auto& fr : v->profiled)
    for (cudaEvent_t e : fr) cudaEventDestroy(e);
  for (cudaEvent_t e : v->event_pool) cudaEventDestroy(e);
  delete v;
}

const char* vh_last_error(const vh_volume* v) { return v ? v->error.c_str() : "null volume"; }

vh_status vh_reset(vh_volume* v, void* stream) {
  if (!v) return VH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  const vh_status st = read_counters(v, s);
  if (st != VH_OK) return st;
  vh::Volume& V = v->dev;
  const size_t used = block_total(v);
  VH_CUDA(v, cudaMemsetAsync(V.slot_keys, 0xFF, V.capacity * sizeof(unsigned long long), s));
  VH_CUDA(v, cudaMemsetAsync(V.slot_block, 0xFF, V.capacity * sizeof(uint32_t), s));
  VH_CUDA(v, cudaMemsetAsync(V.slot_stamp, 0, V.capacity * sizeof(uint32_t), s));
  VH_CUDA(v, cudaMemsetAsync(pool_base(v), 0, used * pool_block_bytes(v), s));
  VH_CUDA(v, cudaMemsetAsync(V.obs_mask, 0, used * (vh::kBlockVoxels / 32) * sizeof(uint32_t), s));
  VH_CUDA(v, cudaMemsetAsync(V.dir_mask, 0, used * sizeof(uint32_t), s));
  VH_CUDA(v, cudaMemsetAsync(V.block_stamp, 0, used * sizeof(uint32_t), s));
  VH_CUDA(v, cudaMemsetAsync(V.counters, 0, sizeof(vh::Counters), s));
  VH_CUDA(v, cudaStreamSynchronize(s));
  v->mesh_triangles = 0;
  return VH_OK;
}

// the bilateral filter of a frame that also starts it: exact, or the fast-math compile's (vh_algorithm.fast_math 1)
static cudaError_t frame_filter(vh_volume* v, const float* in, float* out, const vh::Params& p, cudaStream_t s) {
  return v->algo.fast_math ? vh::fast::launch_frame_filter(in, out, p, v->dev.counters, s)
                           : vh::launch_filter(in, out, p, v->dev.counters, s);
}

vh_status vh_integrate(vh_volume* v, const float* depth, int32_t on_device, const vh_intrinsics* K,
                       const vh_pose* T_wc, int32_t stride, void* stream) {
  if (!v || !depth || !valid_intrinsics(K) || !T_wc) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_integrate: bad argument");
  if (v->dev.max_blocks == 0) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_integrate: keys-only volume (max_blocks 0)");
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  const float* src = nullptr;
  int slot = -1;  // staging buffer of host depth
  vh_status st = on_device ? stage_depth(v, depth, on_device, K, s, &src)
                           : stage_depth_overlapped(v, depth, K, s, &src, &slot);
  if (st != VH_OK) return st;
  const vh::Params p = make_params(v, K, T_wc, stride);
  std::vector<cudaEvent_t> ev;
  if (v->profile) {
    for (int i = 0; i < 5; ++i) {
      cudaEvent_t e = nullptr;
      if (!v->event_pool.empty()) {
        e = v->event_pool.back();
        v->event_pool.pop_back();
      } else {
        VH_CUDA(v, cudaEventCreate(&e));
      }
      ev.push_back(e);
    }
    VH_CUDA(v, cudaEventRecord(ev[0], s));
  }
  if (v->algo.depth_filter == 1 && v->d_nn_params) {
    const size_t need = vh::nn::workspace_bytes(1, K->width, K->height);
    if (need > v->nn_ws_bytes) {
      dfree(v->d_nn_ws);
      v->nn_ws_bytes = 0;
      VH_CUDA(v, cudaMalloc(reinterpret_cast<void**>(&v->d_nn_ws), need));
      v->nn_ws_bytes = need;
    }
    // the bilateral filter (which also starts the frame) is the per-pixel fallback of the learned filter
    VH_CUDA(v, frame_filter(v, src, v->d_depth_bilateral, p, s));
    VH_CUDA(v, vh::nn::forward(v->d_nn_params, v->d_nn_packed, src, v->d_depth_bilateral, v->d_depth_filtered, 1,
                               K->width, K->height, v->d_nn_ws, &v->dev.counters->error, s));
    st = stage_release(v, slot, s);  // the raw depth's last readers
    if (st != VH_OK) return st;
    if (v->profile) VH_CUDA(v, cudaEventRecord(ev[1], s));
    VH_CUDA(v, vh::launch_alloc(v->d_depth_filtered, v->dev, p, s));
  } else {
    // the bilateral filter and the allocation in one kernel: the profile's allocation stage is then empty
    VH_CUDA(v, v->algo.fast_math ? vh::fast::launch_filter_alloc(src, v->d_depth_filtered, v->dev, p, s)
                                  : vh::exact::launch_filter_alloc(src, v->d_depth_filtered, v->dev, p, s));
    st = stage_release(v, slot, s);  // the raw depth's last reader
    if (st != VH_OK) return st;
    if (v->profile) VH_CUDA(v, cudaEventRecord(ev[1], s));
  }
  if (v->profile) VH_CUDA(v, cudaEventRecord(ev[2], s));
  VH_CUDA(v, v->algo.fast_math ? vh::fast::launch_integrate_prepare(v->d_depth_filtered, v->dev, p, v->d_normal_map, s)
                                : vh::exact::launch_integrate_prepare(v->d_depth_filtered, v->dev, p, v->d_normal_map, s));
  if (v->profile) VH_CUDA(v, cudaEventRecord(ev[3], s));
  int variant = v->algo.launch_variant;
  cudaEvent_t tune[2] = {nullptr, nullptr};
  if (v->algo.normal_mode == 1 && v->algo.autotune) {
    st = autotune_step(v, &variant, tune);
    if (st != VH_OK) return st;
    if (tune[0]) VH_CUDA(v, cudaEventRecord(tune[0], s));
  }
  VH_CUDA(v, v->algo.fast_math
                 ? vh::fast::launch_integrate_update(v->d_depth_filtered, v->dev, p, 0, v->d_normal_map, s, variant)
                 : vh::exact::launch_integrate_update(v->d_depth_filtered, v->dev, p, 0, v->d_normal_map, s, variant));
  if (tune[1]) VH_CUDA(v, cudaEventRecord(tune[1], s));
  if (v->profile) {
    VH_CUDA(v, cudaEventRecord(ev[4], s));
    v->profiled.push_back(std::move(ev));
  }
  return VH_OK;
}

// ---- eviction and restore ----

namespace {

size_t native_block_bytes(const vh_volume* v) {
  return v->dev.layers16 != nullptr
             ? static_cast<size_t>(vh::kDirs) * vh::kBlockVoxels * vh::kBinWords16 * sizeof(uint4)
             : kBlockBytes;
}

vh_status ensure_staging(vh_volume* v) {
  if (!v->d_export) {
    VH_CUDA(v, cudaMalloc(reinterpret_cast<void**>(&v->d_export), kExportChunk * kBlockBytes));
    VH_CUDA(v, dalloc(&v->d_export_keys, 3 * kExportChunk));
    v->export_capacity = kExportChunk;
  }
  if (!v->d_import_idx) VH_CUDA(v, dalloc(&v->d_import_idx, kExportChunk));
  return VH_OK;
}

vh_status ensure_evict_scratch(vh_volume* v) {
  if (v->d_evict_list) return VH_OK;
  const size_t nb = std::max<size_t>(v->dev.max_blocks, 1);
  VH_CUDA(v, dalloc(&v->d_evict_list, nb));
  VH_CUDA(v, dalloc(&v->d_evict_src, nb));
  VH_CUDA(v, dalloc(&v->d_evict_cta, nb / 1024 + 2));
  VH_CUDA(v, dalloc(&v->d_evict_hist, vh::kAgeBins));
  VH_CUDA(v, dalloc(&v->d_evict_total, 2));
  return VH_OK;
}

vh_status recount_into_counters(vh_volume* v, cudaStream_t s) {
  VH_CUDA(v, vh::launch_recount(v->dev, v->d_scalar + 1, s));
  VH_CUDA(v, cudaMemcpyAsync(&v->dev.counters->observed_voxels, v->d_scalar + 1, sizeof(unsigned long long),
                             cudaMemcpyDeviceToDevice, s));
  return VH_OK;
}

}  // namespace

vh_status vh_evict_blocks(vh_volume* v, uint32_t min_age_frames, uint64_t target_blocks, int32_t format,
                          int32_t* keys_out, void* data_out, uint64_t max_out, int32_t out_on_device,
                          uint64_t* evicted, void* stream) {
  if (!v || !evicted || (format != 0 && format != 1)) {
    return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_evict_blocks: bad argument");
  }
  *evicted = 0;
  if (v->dev.max_blocks == 0) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_evict_blocks: keys-only volume");
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  vh_status st = ensure_evict_scratch(v);
  if (st == VH_OK) st = ensure_staging(v);
  if (st == VH_OK) st = read_counters(v, s);
  if (st != VH_OK) return st;
  const uint32_t n = static_cast<uint32_t>(block_total(v));
  if (n == 0) return VH_OK;
  // the rule: age >= min_age_frames; with a target, the oldest further blocks until exactly target_blocks remain
  // (the boundary age bin is found through the age histogram, its blocks taken in pool order up to the count)
  vh::EvictRule rule{min_age_frames, static_cast<uint32_t>(vh::kAgeBins), 0U};
  if (target_blocks > 0 && target_blocks < n) {
    std::vector<uint32_t> hist(vh::kAgeBins);
    VH_CUDA(v, vh::launch_age_hist(v->dev, v->d_evict_hist, s));
    VH_CUDA(v, cudaMemcpyAsync(hist.data(), v->d_evict_hist, vh::kAgeBins * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    VH_CUDA(v, cudaStreamSynchronize(s));
    const uint64_t need = n - target_blocks;
    uint64_t acc = 0;
    uint32_t t = vh::kAgeBins - 1;
    for (int bin = vh::kAgeBins - 1; bin >= 0; --bin) {
      acc += hist[bin];
      t = static_cast<uint32_t>(bin);
      if (acc >= need) break;
    }
    if (t < min_age_frames) {
      // victims whatever the cut: age >= min_age_frames or a bin above t
      rule.tie_bin = t;
      uint32_t sure = 0, ties = 0;
      VH_CUDA(v, vh::launch_select(v->dev, n, rule, 0, 0U, v->d_evict_cta, v->d_evict_total, v->d_evict_list, s));
      VH_CUDA(v, vh::launch_select(v->dev, n, rule, 2, 0U, v->d_evict_cta, v->d_evict_total + 1, v->d_evict_src, s));
      VH_CUDA(v, cudaMemcpyAsync(&sure, v->d_evict_total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      VH_CUDA(v, cudaMemcpyAsync(&ties, v->d_evict_total + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      VH_CUDA(v, cudaStreamSynchronize(s));
      if (sure < need && ties > 0) {
        // the boundary bin's blocks below `cut` make up the count: cut = 1 + the (need - sure)-th of them
        const uint64_t take = std::min<uint64_t>(need - sure, ties);
        uint32_t last = 0;
        VH_CUDA(v, cudaMemcpyAsync(&last, v->d_evict_src + (take - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        VH_CUDA(v, cudaStreamSynchronize(s));
        rule.cut = last + 1U;
      }
    }
  }
  VH_CUDA(v, vh::launch_select(v->dev, n, rule, 0, 0U, v->d_evict_cta, v->d_evict_total, v->d_evict_list, s));
  uint32_t nv = 0;
  VH_CUDA(v, cudaMemcpyAsync(&nv, v->d_evict_total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  VH_CUDA(v, cudaStreamSynchronize(s));
  if (nv == 0) return VH_OK;
  if ((keys_out || data_out) && nv > max_out) {
    *evicted = nv;
    return fail(v, VH_ERR_BUFFER_TOO_SMALL, "vh_evict_blocks: output buffers hold fewer blocks than are evicted");
  }
  // 1. copy the victims out: into device memory directly (16-byte aligned), else through the staging buffer
  const size_t bytes = format == 1 ? native_block_bytes(v) : kBlockBytes;
  const cudaMemcpyKind kind = out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  // device (or managed) memory only: the copy kernel then stores into it; anything else goes through cudaMemcpy
  auto device_memory = [](const void* ptr) {
    if (!ptr) return true;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
  };
  const bool direct = out_on_device && reinterpret_cast<uintptr_t>(data_out) % 16 == 0 && device_memory(data_out) &&
                      device_memory(keys_out);
  if (keys_out || data_out) {
    for (uint64_t done = 0; done < nv; done += kExportChunk) {
      const uint32_t c = static_cast<uint32_t>(std::min<uint64_t>(kExportChunk, nv - done));
      if (direct) {
        // the copy kernel writes the caller's buffers (a NULL one's part goes to the staging buffer)
        VH_CUDA(v, vh::launch_copy_out(v->dev, v->d_evict_list + done, c, format,
                                       keys_out ? keys_out + 3 * done : v->d_export_keys,
                                       data_out ? static_cast<void*>(static_cast<char*>(data_out) + done * bytes)
                                                : static_cast<void*>(v->d_export),
                                       s));
        continue;
      }
      VH_CUDA(v, vh::launch_copy_out(v->dev, v->d_evict_list + done, c, format, v->d_export_keys, v->d_export, s));
      if (data_out) {
        VH_CUDA(v, cudaMemcpyAsync(static_cast<char*>(data_out) + done * bytes, v->d_export, c * bytes, kind, s));
      }
      if (keys_out) {
        VH_CUDA(v, cudaMemcpyAsync(keys_out + 3 * done, v->d_export_keys, 3 * c * sizeof(int32_t), kind, s));
      }
    }
  }
  // the victims' observed voxels, counted while their masks are still in place
  VH_CUDA(v, vh::launch_victim_observed(v->dev, v->d_evict_list, nv, v->d_scalar + 1, s));
  // 2. the survivors above the new block count move into the victims' slots below it
  const uint32_t live = n - nv;
  VH_CUDA(v, vh::launch_select(v->dev, n, rule, 1, live, v->d_evict_cta, v->d_evict_total + 1, v->d_evict_src, s));
  uint32_t nmove = 0;
  VH_CUDA(v, cudaMemcpyAsync(&nmove, v->d_evict_total + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  VH_CUDA(v, cudaStreamSynchronize(s));
  // the victims below `live` are the first nmove entries of the ascending victim list
  VH_CUDA(v, vh::launch_move_blocks(v->dev, v->d_evict_src, v->d_evict_list, nmove, s));
  // 3. the freed tail [live, n) back to zero, the hash rebuilt from the live keys
  vh::Volume& V = v->dev;
  const size_t tail = n - live;
  const size_t nb_bytes = native_block_bytes(v);
  char* pool = V.layers16 != nullptr ? reinterpret_cast<char*>(V.layers16) : reinterpret_cast<char*>(V.layers);
  VH_CUDA(v, cudaMemsetAsync(pool + static_cast<size_t>(live) * nb_bytes, 0, tail * nb_bytes, s));
  VH_CUDA(v, cudaMemsetAsync(V.block_keys + live, 0, tail * sizeof(int4), s));
  VH_CUDA(v, cudaMemsetAsync(V.obs_mask + static_cast<size_t>(live) * (vh::kBlockVoxels / 32), 0,
                             tail * (vh::kBlockVoxels / 32) * sizeof(uint32_t), s));
  VH_CUDA(v, cudaMemsetAsync(V.dir_mask + live, 0, tail * sizeof(uint32_t), s));
  VH_CUDA(v, cudaMemsetAsync(V.block_stamp + live, 0, tail * sizeof(uint32_t), s));
  VH_CUDA(v, vh::launch_rehash(V, live, s));
  // 4. counters: the new block count, no visible list, the victims' observed voxels taken off
  vh::Counters c = *v->h_counters;
  c.num_blocks = live;
  c.visible_count = 0;
  c.new_blocks = 0;
  VH_CUDA(v, cudaMemcpyAsync(V.counters, &c, sizeof(c), cudaMemcpyHostToDevice, s));
  VH_CUDA(v, vh::launch_subtract_observed(V, v->d_scalar + 1, s));
  *evicted = nv;
  v->mesh_triangles = 0;
  return vh_synchronize(v, stream);
}

vh_status vh_restore_blocks(vh_volume* v, const int32_t* keys, const void* data, uint64_t count, int32_t in_on_device,
                            void* stream) {
  if (!v || (count && (!keys || !data))) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_restore_blocks: bad argument");
  if (v->dev.max_blocks == 0) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_restore_blocks: keys-only volume");
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  vh_status st = ensure_staging(v);
  if (st != VH_OK) return st;
  const size_t bytes = native_block_bytes(v);
  const cudaMemcpyKind kind = in_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  for (uint64_t done = 0; done < count; done += kExportChunk) {
    const uint32_t n = static_cast<uint32_t>(std::min<uint64_t>(kExportChunk, count - done));
    VH_CUDA(v, cudaMemcpyAsync(v->d_export_keys, keys + 3 * done, 3 * n * sizeof(int32_t), kind, s));
    VH_CUDA(v, cudaMemcpyAsync(v->d_export, static_cast<const char*>(data) + done * bytes, n * bytes, kind, s));
    VH_CUDA(v, vh::launch_import_keys(v->dev, v->d_export_keys, n, v->d_import_idx, s));
    VH_CUDA(v, vh::launch_restore_native(v->dev, v->d_export, n, v->d_import_idx, s));
  }
  st = recount_into_counters(v, s);
  if (st != VH_OK) return st;
  return vh_synchronize(v, stream);
}

vh_status vh_autotune_result(vh_volume* v, int32_t* variant, int32_t* threads_per_cta, int32_t* min_ctas_per_sm,
                             float* ms) {
  if (!v) return VH_ERR_INVALID_ARGUMENT;
  int t = 0, b = 0;
  vh::exact::fused_variant_shape(v->tuned_variant, &t, &b);
  if (variant) *variant = v->tuned_variant;
  if (threads_per_cta) *threads_per_cta = v->tuned_variant >= 0 ? t : 0;
  if (min_ctas_per_sm) *min_ctas_per_sm = v->tuned_variant >= 0 ? b : 0;
  if (ms) *ms = v->tune_best_ms;
  return VH_OK;
}

vh_status vh_profile_enable(vh_volume* v, int32_t enable) {
  if (!v) return VH_ERR_INVALID_ARGUMENT;
  v->profile = enable != 0;
  return VH_OK;
}

vh_status vh_profile_read(vh_volume* v, double ms[4], uint64_t* frames) {
  if (!v || !ms) return VH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(v->params.device);
  ms[0] = ms[1] = ms[2] = ms[3] = 0.0;
  const uint64_t n = v->profiled.size();
  for (auto& fr : v->profiled) {
    VH_CUDA(v, cudaEventSynchronize(fr[4]));
    for (int k = 0; k < 4; ++k) {
      float t = 0.0f;
      VH_CUDA(v, cudaEventElapsedTime(&t, fr[k], fr[k + 1]));
      ms[k] += t;
    }
    for (cudaEvent_t e : fr) v->event_pool.push_back(e);
  }
  v->profiled.clear();
  if (frames) *frames = n;
  return VH_OK;
}

vh_status vh_allocate(vh_volume* v, const float* depth, int32_t on_device, const vh_intrinsics* K, const vh_pose* T_wc,
                      int32_t stride, int32_t* keys_out, size_t max_keys, size_t* count, void* stream) {
  if (!v || !depth || !valid_intrinsics(K) || !T_wc || !count) {
    return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_allocate: bad argument");
  }
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  const float* src = nullptr;
  vh_status st = stage_depth(v, depth, on_device, K, s, &src);
  if (st != VH_OK) return st;
  const vh::Params p = make_params(v, K, T_wc, stride);
  VH_CUDA(v, vh::launch_begin_frame(v->dev.counters, s));
  VH_CUDA(v, vh::launch_alloc(src, v->dev, p, s));
  st = vh_synchronize(v, stream);
  if (st != VH_OK) return st;
  return vh_visible_block_keys(v, keys_out, max_keys, count, stream);
}

vh_status vh_visible_block_keys(vh_volume* v, int32_t* keys_out, size_t max_keys, size_t* count, void* stream) {
  if (!v || !count) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_visible_block_keys: bad argument");
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  const vh_status st = read_counters(v, s);
  if (st != VH_OK) return st;
  const size_t n = v->h_counters->visible_count;
  *count = n;
  if (!keys_out || n == 0) return VH_OK;
  if (n > max_keys) return fail(v, VH_ERR_BUFFER_TOO_SMALL, "vh_visible_block_keys: keys_out too small");
  dfree(v->d_keys);
  VH_CUDA(v, dalloc(&v->d_keys, 3 * n));
  VH_CUDA(v, vh::launch_visible_keys(v->dev, v->d_keys, s));
  VH_CUDA(v, cudaMemcpyAsync(keys_out, v->d_keys, 3 * n * sizeof(int), cudaMemcpyDeviceToHost, s));
  VH_CUDA(v, cudaStreamSynchronize(s));
  return VH_OK;
}

vh_status vh_filter_depth(vh_volume* v, const float* in, float* out, const vh_intrinsics* K, void* stream) {
  if (!v || !in || !out || !valid_intrinsics(K)) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_filter_depth: bad argument");
  DeviceGuard guard(v->params.device);
  const vh::Params p = make_params(v, K, nullptr, 1);
  VH_CUDA(v, vh::launch_filter(in, out, p, nullptr, as_stream(stream)));
  return VH_OK;
}

vh_status vh_depth_normals(vh_volume* v, const float* in, float* normals, uint8_t* valid, const vh_intrinsics* K,
                           void* stream) {
  if (!v || !in || !normals || !valid || !valid_intrinsics(K)) {
    return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_depth_normals: bad argument");
  }
  DeviceGuard guard(v->params.device);
  const vh::Params p = make_params(v, K, nullptr, 1);
  VH_CUDA(v, vh::launch_depth_normals(in, normals, valid, p, as_stream(stream)));
  return VH_OK;
}

vh_status vh_pixel_normals(vh_volume* v, const float* in, float* normals, const vh_intrinsics* K, void* stream) {
  if (!v || !in || !normals || !valid_intrinsics(K)) {
    return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_pixel_normals: bad argument");
  }
  if ((reinterpret_cast<uintptr_t>(normals) & 15U) != 0U) {
    return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_pixel_normals: normals must be 16-byte aligned");
  }
  DeviceGuard guard(v->params.device);
  const vh::Params p = make_params(v, K, nullptr, 1);
  float4* out = reinterpret_cast<float4*>(normals);
  VH_CUDA(v, v->algo.fast_math ? vh::fast::launch_pixel_normals(in, p, out, as_stream(stream))
                                : vh::exact::launch_pixel_normals(in, p, out, as_stream(stream)));
  return VH_OK;
}

vh_status vh_raycast_depth(vh_volume* v, const vh_intrinsics* K, const vh_pose* T_wc, float min_depth, float max_depth,
                           float step_voxels, float* depth_out, void* stream) {
  if (!v || !valid_intrinsics(K) || !T_wc || !depth_out || !(min_depth >= 0.0f) || !(max_depth > min_depth) ||
      !(step_voxels > 0.0f) || v->dev.max_blocks == 0) {
    return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_raycast_depth: bad argument");
  }
  DeviceGuard guard(v->params.device);
  const vh::Params p = make_params(v, K, T_wc, 1);
  VH_CUDA(v, vh::launch_raycast(v->dev, p, min_depth, max_depth, step_voxels, depth_out, as_stream(stream)));
  return VH_OK;
}

vh_status vh_synchronize(vh_volume* v, void* stream) {
  if (!v) return VH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  vh_status st = read_counters(v, s);
  if (st != VH_OK) return st;
  const uint32_t err = v->h_counters->error;
  if (err == 0U) return VH_OK;
  VH_CUDA(v, cudaMemsetAsync(&v->dev.counters->error, 0, sizeof(uint32_t), s));
  VH_CUDA(v, cudaStreamSynchronize(s));
  if (err & vh::kErrKeyRange) return fail(v, VH_ERR_KEY_RANGE, "block coordinate outside the 21-bit packed key range");
  if (err & vh::kErrTimeout) return fail(v, VH_ERR_TIMEOUT, "the tensor cores did not signal completion in time");
  if (err & vh::kErrHashFull) return fail(v, VH_ERR_HASH_FULL, "block hash table full (raise hash_buckets)");
  return fail(v, VH_ERR_POOL_FULL, "block pool full (raise max_blocks)");
}

// marching cubes over every allocated block (frames == 0) or over the blocks updated within the last `frames`
// frames (incremental meshing)
static vh_status extract(vh_volume* v, float iso, uint32_t frames, size_t* triangle_count, void* stream) {
  if (!v || !triangle_count || v->dev.max_blocks == 0) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_extract_mesh: bad argument");
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  if (!v->d_mc_counts) {
    VH_CUDA(v, dalloc(&v->d_mc_counts, v->dev.max_blocks));
    VH_CUDA(v, dalloc(&v->d_mc_offsets, v->dev.max_blocks));
    VH_CUDA(v, dalloc(&v->d_mc_dir_totals, static_cast<size_t>(v->dev.max_blocks) * vh::kDirs));
    VH_CUDA(v, dalloc(&v->d_mc_cell_counts, static_cast<size_t>(v->dev.max_blocks) * vh::kDirs * vh::kBlockVoxels));
  }
  const uint32_t* list = nullptr;
  const uint32_t* list_count = nullptr;
  if (frames > 0) {
    if (!v->d_mc_list) {
      VH_CUDA(v, dalloc(&v->d_mc_list, v->dev.max_blocks));
      VH_CUDA(v, dalloc(&v->d_mc_list_count, 1));
    }
    VH_CUDA(v, vh::launch_recent_blocks(v->dev, frames, v->d_mc_list, v->d_mc_list_count, s));
    // blocks outside the list contribute nothing to the scan
    VH_CUDA(v, cudaMemsetAsync(v->d_mc_counts, 0, static_cast<size_t>(v->dev.max_blocks) * sizeof(uint32_t), s));
    list = v->d_mc_list;
    list_count = v->d_mc_list_count;
  }
  vh_intrinsics K{1, 1, 1.0f, 1.0f, 0.0f, 0.0f};
  vh::Params p = make_params(v, &K, nullptr, 1);
  p.iso = iso;
  VH_CUDA(v, vh::launch_mc_count(v->dev, p, v->d_mc_counts, v->d_mc_dir_totals, v->d_mc_cell_counts, list, list_count,
                                 s));
  VH_CUDA(v, vh::launch_mc_scan(v->dev, v->d_mc_counts, v->d_mc_offsets, v->d_scalar, s));
  unsigned long long total = 0;
  VH_CUDA(v, cudaMemcpyAsync(&total, v->d_scalar, sizeof(total), cudaMemcpyDeviceToHost, s));
  VH_CUDA(v, cudaStreamSynchronize(s));
  if (total > v->tri_capacity) {
    dfree(v->d_tris);
    v->tri_capacity = 0;
    const size_t cap = static_cast<size_t>(total) + static_cast<size_t>(total) / 8 + 1024;
    VH_CUDA(v, dalloc(&v->d_tris, cap * 9));
    v->tri_capacity = cap;
  }
  if (total > 0) {
    VH_CUDA(v, vh::launch_mc_emit(v->dev, p, v->d_mc_counts, v->d_mc_dir_totals, v->d_mc_cell_counts,
                                  v->d_mc_offsets, v->d_tris, list, list_count, s));
  }
  VH_CUDA(v, cudaStreamSynchronize(s));
  v->mesh_triangles = static_cast<size_t>(total);
  *triangle_count = v->mesh_triangles;
  return VH_OK;
}

vh_status vh_extract_mesh(vh_volume* v, float iso, size_t* triangle_count, void* stream) {
  return extract(v, iso, 0U, triangle_count, stream);
}

vh_status vh_extract_mesh_recent(vh_volume* v, float iso, uint32_t frames, size_t* triangle_count, void* stream) {
  return extract(v, iso, frames, triangle_count, stream);
}

vh_status vh_copy_mesh(vh_volume* v, float* out, size_t max_triangles, int32_t on_device, void* stream) {
  if (!v || (!out && v->mesh_triangles)) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_copy_mesh: bad argument");
  if (max_triangles < v->mesh_triangles) return fail(v, VH_ERR_BUFFER_TOO_SMALL, "vh_copy_mesh: buffer too small");
  if (v->mesh_triangles == 0) return VH_OK;
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  VH_CUDA(v, cudaMemcpyAsync(out, v->d_tris, v->mesh_triangles * 9 * sizeof(float),
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
  VH_CUDA(v, cudaStreamSynchronize(s));
  return VH_OK;
}

vh_status vh_weld_mesh(vh_volume* v, size_t* vertex_count, size_t* face_count, void* stream) {
  if (!v || !vertex_count || !face_count) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_weld_mesh: bad argument");
  const size_t nt = v->mesh_triangles;
  // 32-bit vertex indices and a table of at most 2^31 slots: fewer than 2^30 soup vertices
  if (3 * nt >= (static_cast<size_t>(1) << 30) / 9 * 8) {
    return fail(v, VH_ERR_CAPACITY, "vh_weld_mesh: soup too large for 32-bit vertex indices");
  }
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  const vh_status st = ensure_weld(v, nt);
  if (st != VH_OK) return st;
  VH_CUDA(v, vh::launch_weld(v->d_tris, static_cast<uint32_t>(nt), v->weld, s));
  uint32_t counts[3] = {0U, 0U, 0U};
  VH_CUDA(v, cudaMemcpyAsync(counts, v->weld.counts, sizeof(counts), cudaMemcpyDeviceToHost, s));
  VH_CUDA(v, cudaStreamSynchronize(s));
  if (counts[2] != 0U) return fail(v, VH_ERR_HASH_FULL, "vh_weld_mesh: vertex table full");
  v->weld_vertices = counts[0];
  v->weld_faces = counts[1];
  *vertex_count = v->weld_vertices;
  *face_count = v->weld_faces;
  return VH_OK;
}

vh_status vh_copy_welded_mesh(vh_volume* v, float* vertices, size_t max_vertices, int32_t* faces, size_t max_faces,
                              int32_t on_device, void* stream) {
  if (!v || (!vertices && v->weld_vertices) || (!faces && v->weld_faces)) {
    return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_copy_welded_mesh: bad argument");
  }
  if (max_vertices < v->weld_vertices || max_faces < v->weld_faces) {
    return fail(v, VH_ERR_BUFFER_TOO_SMALL, "vh_copy_welded_mesh: buffer too small");
  }
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (v->weld_vertices) {
    VH_CUDA(v, cudaMemcpyAsync(vertices, v->weld.verts, v->weld_vertices * 3 * sizeof(float), kind, s));
  }
  if (v->weld_faces) {
    VH_CUDA(v, cudaMemcpyAsync(faces, v->weld.faces, v->weld_faces * 3 * sizeof(int32_t), kind, s));
  }
  VH_CUDA(v, cudaStreamSynchronize(s));
  return VH_OK;
}

vh_status vh_block_count(vh_volume* v, uint64_t* count) {
  if (!v || !count) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_block_count: bad argument");
  DeviceGuard guard(v->params.device);
  const vh_status st = read_counters(v, nullptr);
  if (st != VH_OK) return st;
  *count = block_total(v);
  return VH_OK;
}

vh_status vh_observed_voxel_count(vh_volume* v, uint64_t* count) {
  if (!v || !count) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_observed_voxel_count: bad argument");
  DeviceGuard guard(v->params.device);
  const vh_status st = read_counters(v, nullptr);
  if (st != VH_OK) return st;
  *count = v->h_counters->observed_voxels;
  return VH_OK;
}

vh_status vh_recount_observed_voxels(vh_volume* v, uint64_t* count, void* stream) {
  if (!v || !count) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_recount_observed_voxels: bad argument");
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  VH_CUDA(v, vh::launch_recount(v->dev, v->d_scalar + 1, s));
  unsigned long long n = 0;
  VH_CUDA(v, cudaMemcpyAsync(&n, v->d_scalar + 1, sizeof(n), cudaMemcpyDeviceToHost, s));
  VH_CUDA(v, cudaStreamSynchronize(s));
  *count = n;
  return VH_OK;
}

vh_status vh_frame_stats_get(vh_volume* v, vh_frame_stats* stats, void* stream) {
  if (!v || !stats) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_frame_stats_get: bad argument");
  DeviceGuard guard(v->params.device);
  const vh_status st = read_counters(v, as_stream(stream));
  if (st != VH_OK) return st;
  stats->visible_blocks = v->h_counters->visible_count;
  stats->new_blocks = v->h_counters->new_blocks;
  stats->active_voxels = v->h_counters->active_voxels;
  stats->updated_voxels = v->h_counters->integrated_voxels;
  stats->total_blocks = block_total(v);
  stats->observed_voxels = v->h_counters->observed_voxels;
  return VH_OK;
}

vh_status vh_frame_stats_enqueue(vh_volume* v, void* counters64, void* stream) {
  if (!v || !counters64) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_frame_stats_enqueue: bad argument");
  DeviceGuard guard(v->params.device);
  VH_CUDA(v, cudaMemcpyAsync(counters64, v->dev.counters, sizeof(vh::Counters), cudaMemcpyDeviceToHost,
                             as_stream(stream)));
  return VH_OK;
}

vh_status vh_frame_stats_decode(const vh_volume* v, const void* counters64, vh_frame_stats* stats) {
  if (!v || !counters64 || !stats) return VH_ERR_INVALID_ARGUMENT;
  vh::Counters c;
  std::memcpy(&c, counters64, sizeof(c));
  stats->visible_blocks = c.visible_count;
  stats->new_blocks = c.new_blocks;
  stats->active_voxels = c.active_voxels;
  stats->updated_voxels = c.integrated_voxels;
  stats->total_blocks = std::min<uint64_t>(c.num_blocks, v->dev.max_blocks);
  stats->observed_voxels = c.observed_voxels;
  return VH_OK;
}

vh_status vh_export_blocks(vh_volume* v, uint64_t first, uint64_t count, int32_t* keys, void* voxels,
                           int32_t on_device, void* stream) {
  if (!v) return VH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  vh_status st = read_counters(v, s);
  if (st != VH_OK) return st;
  if (first + count > block_total(v)) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_export_blocks: range beyond block count");
  if (count == 0 || (!keys && !voxels)) return VH_OK;
  if (!v->d_export) {
    VH_CUDA(v, cudaMalloc(reinterpret_cast<void**>(&v->d_export), kExportChunk * kBlockBytes));
    VH_CUDA(v, dalloc(&v->d_export_keys, 3 * kExportChunk));
    v->export_capacity = kExportChunk;
  }
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  for (uint64_t done = 0; done < count; done += kExportChunk) {
    const uint32_t n = static_cast<uint32_t>(std::min<uint64_t>(kExportChunk, count - done));
    VH_CUDA(v, vh::launch_export(v->dev, static_cast<uint32_t>(first + done), n, v->d_export_keys, v->d_export, s));
    if (voxels) {
      VH_CUDA(v, cudaMemcpyAsync(static_cast<char*>(voxels) + done * kBlockBytes, v->d_export, n * kBlockBytes, kind, s));
    }
    if (keys) {
      VH_CUDA(v, cudaMemcpyAsync(keys + 3 * done, v->d_export_keys, 3 * n * sizeof(int32_t), kind, s));
    }
  }
  VH_CUDA(v, cudaStreamSynchronize(s));
  return VH_OK;
}

vh_status vh_import_blocks(vh_volume* v, const int32_t* keys, const void* voxels, uint64_t count, int32_t on_device,
                           void* stream) {
  if (!v || (count && (!keys || !voxels))) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_import_blocks: bad argument");
  if (v->dev.max_blocks == 0) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_import_blocks: keys-only volume");
  DeviceGuard guard(v->params.device);
  const cudaStream_t s = as_stream(stream);
  if (!v->d_export) {
    VH_CUDA(v, cudaMalloc(reinterpret_cast<void**>(&v->d_export), kExportChunk * kBlockBytes));
    VH_CUDA(v, dalloc(&v->d_export_keys, 3 * kExportChunk));
    v->export_capacity = kExportChunk;
  }
  if (!v->d_import_idx) VH_CUDA(v, dalloc(&v->d_import_idx, kExportChunk));
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  for (uint64_t done = 0; done < count; done += kExportChunk) {
    const uint32_t n = static_cast<uint32_t>(std::min<uint64_t>(kExportChunk, count - done));
    VH_CUDA(v, cudaMemcpyAsync(v->d_export_keys, keys + 3 * done, 3 * n * sizeof(int32_t), kind, s));
    VH_CUDA(v, cudaMemcpyAsync(v->d_export, static_cast<const char*>(voxels) + done * kBlockBytes, n * kBlockBytes,
                               kind, s));
    VH_CUDA(v, vh::launch_import(v->dev, v->d_export_keys, v->d_export, n, v->d_import_idx, s));
  }
  VH_CUDA(v, vh::launch_recount(v->dev, v->d_scalar + 1, s));
  VH_CUDA(v, cudaMemcpyAsync(&v->dev.counters->observed_voxels, v->d_scalar + 1, sizeof(unsigned long long),
                             cudaMemcpyDeviceToDevice, s));
  return vh_synchronize(v, stream);
}

vh_status vh_render_depth(const float* prims, int32_t n_prims, const vh_intrinsics* K, const vh_pose* T_wc,
                          uint32_t seed, uint32_t frame, float sigma_z2, float dropout, float max_depth,
                          float* depth_out, void* stream) {
  if (!prims || n_prims <= 0 || n_prims > 1024 || !valid_intrinsics(K) || !T_wc || !depth_out) {
    return VH_ERR_INVALID_ARGUMENT;
  }
  vh::Params p{};
  p.width = K->width;
  p.height = K->height;
  p.fx = K->fx;
  p.fy = K->fy;
  p.cx = K->cx;
  p.cy = K->cy;
  for (int i = 0; i < 9; ++i) p.T_wc.r[i] = T_wc->R[i];
  for (int i = 0; i < 3; ++i) p.T_wc.t[i] = T_wc->t[i];
  const cudaError_t e = vh::launch_render(prims, n_prims, p, seed, frame, sigma_z2, dropout, max_depth, depth_out,
                                          as_stream(stream));
  return e == cudaSuccess ? VH_OK : VH_ERR_CUDA;
}

// ---- multi-scene batch ----

struct vh_batch {
  std::vector<vh_volume*> vols;
  int device = 0;
  int fast = 0;
  bool band = false;  // every volume allocates by the truncation-band rule (smaller tile sets)
  bool use_graph = false;
  bool persistent = false;          // the step as one cooperative launch (use_graph 2)
  size_t bytes = 0;                 // header + descriptors
  unsigned char* d_buf = nullptr;   // [BatchHeader][SceneDesc x n]
  uint32_t* d_queue = nullptr;      // 3 work-queue counters, then (at 4) the persistent step's 2 barrier words
  unsigned char* h_stage[2] = {nullptr, nullptr};  // pinned, alternate steps
  cudaEvent_t done[2] = {nullptr, nullptr};         // step that last used h_stage[k] has finished
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  cudaStream_t capture = nullptr;
  int next = 0;
};

static uint32_t tiles(int w, int h, int tx, int ty) {
  if (w <= 0 || h <= 0) return 0U;
  return static_cast<uint32_t>(((w + tx - 1) / tx) * ((h + ty - 1) / ty));
}

static cudaError_t batch_launch(vh_batch* b, int slot, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(b->d_buf, b->h_stage[slot], b->bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  const auto* hdr = reinterpret_cast<const vh::BatchHeader*>(b->d_buf);
  const auto* desc = reinterpret_cast<const vh::SceneDesc*>(b->d_buf + sizeof(vh::BatchHeader));
  if (b->persistent) {
    return b->fast ? vh::fast::launch_batch_persistent(desc, hdr, b->d_queue, b->d_queue + 4, b->band, s)
                   : vh::exact::launch_batch_persistent(desc, hdr, b->d_queue, b->d_queue + 4, b->band, s);
  }
  return b->fast ? vh::fast::launch_batch(desc, hdr, b->d_queue, b->band, s)
                 : vh::exact::launch_batch(desc, hdr, b->d_queue, b->band, s);
}

void vh_batch_destroy(vh_batch* b) {
  if (!b) return;
  DeviceGuard guard(b->device);
  cudaDeviceSynchronize();
  for (int k = 0; k < 2; ++k) {
    if (b->exec[k]) cudaGraphExecDestroy(b->exec[k]);
    if (b->done[k]) cudaEventDestroy(b->done[k]);
    if (b->h_stage[k]) cudaFreeHost(b->h_stage[k]);
  }
  if (b->capture) cudaStreamDestroy(b->capture);
  if (b->d_buf) cudaFree(b->d_buf);
  if (b->d_queue) cudaFree(b->d_queue);
  delete b;
}

vh_status vh_batch_create(vh_volume* const* volumes, int32_t count, int32_t use_graph, vh_batch** out) {
  if (!volumes || !out || count <= 0 || count > vh::kMaxBatchScenes || use_graph < 0 || use_graph > 2) {
    return VH_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  for (int i = 0; i < count; ++i) {
    const vh_volume* v = volumes[i];
    if (!v || v->dev.max_blocks == 0 || v->algo.normal_mode != 1 || v->params.device != volumes[0]->params.device ||
        v->algo.fast_math != volumes[0]->algo.fast_math) {
      return VH_ERR_INVALID_ARGUMENT;
    }
  }
  vh_batch* b = new (std::nothrow) vh_batch();
  if (!b) return VH_ERR_OUT_OF_MEMORY;
  b->vols.assign(volumes, volumes + count);
  b->device = volumes[0]->params.device;
  b->fast = volumes[0]->algo.fast_math;
  b->band = true;
  for (int i = 0; i < count; ++i) b->band = b->band && volumes[i]->algo.allocation_mode == 1;
  b->use_graph = use_graph == 1;
  b->persistent = use_graph == 2;
  b->bytes = sizeof(vh::BatchHeader) + static_cast<size_t>(count) * sizeof(vh::SceneDesc);
  DeviceGuard guard(b->device);
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&b->d_buf), b->bytes);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&b->d_queue), 8 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(b->d_queue, 0, 8 * sizeof(uint32_t));
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
    e = cudaMallocHost(reinterpret_cast<void**>(&b->h_stage[k]), b->bytes);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done[k], cudaEventDisableTiming);
  }
  if (e == cudaSuccess && b->use_graph) e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cudaGetLastError();
    vh_batch_destroy(b);
    return e == cudaErrorMemoryAllocation ? VH_ERR_OUT_OF_MEMORY : VH_ERR_CUDA;
  }
  *out = b;
  return VH_OK;
}

vh_status vh_batch_integrate(vh_batch* b, const float* const* depth_device, const vh_intrinsics* K, const vh_pose* T_wc,
                             const int32_t* active, int32_t stride, void* stream) {
  if (!b || !depth_device || !K || !T_wc || stride < 1) return VH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(b->device);
  const cudaStream_t s = as_stream(stream);
  const int slot = b->next;
  b->next ^= 1;
  // the step two calls ago read this staging buffer: wait until it has finished
  if (cudaEventSynchronize(b->done[slot]) != cudaSuccess) return VH_ERR_CUDA;
  auto* hdr = reinterpret_cast<vh::BatchHeader*>(b->h_stage[slot]);
  auto* desc = reinterpret_cast<vh::SceneDesc*>(b->h_stage[slot] + sizeof(vh::BatchHeader));
  const int n = static_cast<int>(b->vols.size());
  uint32_t filter_total = 0, map_total = 0;
  for (int i = 0; i < n; ++i) {
    vh_volume* v = b->vols[i];
    vh::SceneDesc& d = desc[i];
    std::memset(&d, 0, sizeof(d));
    d.V = v->dev;
    const bool on = !active || active[i] != 0;
    if (on) {
      if (!valid_intrinsics(&K[i]) || !depth_device[i]) return fail(v, VH_ERR_INVALID_ARGUMENT, "vh_batch_integrate: bad scene");
      const vh_status st = ensure_depth(v, static_cast<size_t>(K[i].width) * K[i].height);
      if (st != VH_OK) return st;
      d.V = v->dev;
      d.p = make_params(v, &K[i], &T_wc[i], stride);
      d.depth_in = depth_device[i];
      d.depth = v->d_depth_filtered;
      d.nmap = v->d_normal_map;
      d.filter_items = tiles(K[i].width, K[i].height, 32, 8);
      d.map_items = tiles(K[i].width, K[i].height, 32, 8);
      d.active = 1U;
    }
    d.filter_first = filter_total;
    d.map_first = map_total;
    filter_total += d.filter_items;
    map_total += d.map_items;
  }
  hdr->nscenes = static_cast<uint32_t>(n);
  hdr->filter_total = filter_total;
  hdr->stage2_total = map_total;
  hdr->pad = 0U;
  cudaError_t e = cudaSuccess;
  if (b->use_graph) {
    if (!b->exec[slot]) {
      cudaGraph_t g = nullptr;
      e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeRelaxed);
      if (e == cudaSuccess) {
        const cudaError_t le = batch_launch(b, slot, b->capture);
        e = cudaStreamEndCapture(b->capture, &g);
        if (le != cudaSuccess) e = le;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec[slot], g, 0);
      if (g) cudaGraphDestroy(g);
    }
    if (e == cudaSuccess) e = cudaGraphLaunch(b->exec[slot], s);
  } else {
    e = batch_launch(b, slot, s);
  }
  if (e == cudaSuccess) e = cudaEventRecord(b->done[slot], s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return VH_ERR_CUDA;
  }
  return VH_OK;
}

// ---- denoiser building blocks (device pointers; no reference counterpart) ----

vh_status vh_nn_pack_conv32_weights(const float* w, void* packed, int32_t transpose_flip, void* stream) {
  if (!w || !packed) return VH_ERR_INVALID_ARGUMENT;
  return vh::nn::launch_pack_w32(w, static_cast<__nv_bfloat16*>(packed), transpose_flip, as_stream(stream)) == cudaSuccess
             ? VH_OK
             : VH_ERR_CUDA;
}

vh_status vh_nn_conv32(const void* in, const void* packed_w, const float* bias, const void* mask, void* out, int32_t batch,
                       int32_t width, int32_t height, int32_t mode, int32_t relu, uint32_t* error, void* stream) {
  if (!in || !packed_w || !out || !error || batch <= 0 || width <= 0 || height <= 0 || (mode != 0 && mode != 1) ||
      (mode == 1 && !mask)) {
    return VH_ERR_INVALID_ARGUMENT;
  }
  const cudaError_t e = vh::nn::launch_conv32(static_cast<const __nv_bfloat16*>(in),
                                              static_cast<const __nv_bfloat16*>(packed_w), bias,
                                              static_cast<const __nv_bfloat16*>(mask), static_cast<__nv_bfloat16*>(out),
                                              batch, width, height, mode, relu, error, as_stream(stream));
  return e == cudaSuccess ? VH_OK : VH_ERR_CUDA;
}

vh_status vh_nn_conv32_gated(const void* in, const void* packed_w, const float* bias, const void* mask, void* out,
                             int32_t batch, int32_t width, int32_t height, int32_t mode, int32_t relu,
                             const uint32_t* gate, uint32_t* error, void* stream) {
  if (!in || !packed_w || !out || !gate || !error || batch <= 0 || width <= 0 || height <= 0 ||
      (mode != 0 && mode != 1) || (mode == 1 && !mask)) {
    return VH_ERR_INVALID_ARGUMENT;
  }
  const cudaError_t e = vh::nn::launch_conv32(static_cast<const __nv_bfloat16*>(in),
                                              static_cast<const __nv_bfloat16*>(packed_w), bias,
                                              static_cast<const __nv_bfloat16*>(mask), static_cast<__nv_bfloat16*>(out),
                                              batch, width, height, mode, relu, error, as_stream(stream), gate);
  return e == cudaSuccess ? VH_OK : VH_ERR_CUDA;
}

vh_status vh_nn_wgrad32(const void* x, const void* grad, float* dw, float* db, int32_t batch, int32_t width,
                        int32_t height, uint32_t* error, void* stream) {
  if (!x || !grad || !dw || !db || !error || batch <= 0 || width <= 0 || height <= 0) return VH_ERR_INVALID_ARGUMENT;
  const cudaError_t e = vh::nn::launch_wgrad32(static_cast<const __nv_bfloat16*>(x),
                                               static_cast<const __nv_bfloat16*>(grad), dw, db, batch, width, height,
                                               error, as_stream(stream));
  return e == cudaSuccess ? VH_OK : VH_ERR_CUDA;
}

int32_t vh_nn_param_count(void) { return vh::nn::param_count(); }

uint64_t vh_nn_workspace_bytes(int32_t batch, int32_t width, int32_t height) {
  if (batch <= 0 || width <= 0 || height <= 0) return 0;
  return vh::nn::workspace_bytes(batch, width, height);
}

vh_status vh_nn_pack(const float* params, void* packed, void* stream) {
  if (!params || !packed) return VH_ERR_INVALID_ARGUMENT;
  return vh::nn::pack_weights(params, static_cast<__nv_bfloat16*>(packed), as_stream(stream)) == cudaSuccess ? VH_OK
                                                                                                            : VH_ERR_CUDA;
}

vh_status vh_nn_forward(const float* params, const void* packed, const float* depth, float* out, int32_t batch,
                        int32_t width, int32_t height, void* workspace, uint32_t* error, void* stream) {
  if (!params || !packed || !depth || !out || !workspace || !error || batch <= 0 || width <= 0 || height <= 0) {
    return VH_ERR_INVALID_ARGUMENT;
  }
  return vh::nn::forward(params, static_cast<const __nv_bfloat16*>(packed), depth, nullptr, out, batch, width, height,
                         static_cast<unsigned char*>(workspace), error, as_stream(stream)) == cudaSuccess
             ? VH_OK
             : VH_ERR_CUDA;
}

vh_status vh_nn_backward(const float* params, const void* packed, const float* depth, const float* target,
                         const float* out, int32_t batch, int32_t width, int32_t height, void* workspace, float* grads,
                         float* loss, uint32_t* error, void* stream) {
  if (!params || !packed || !depth || !target || !out || !workspace || !grads || !loss || !error || batch <= 0 ||
      width <= 0 || height <= 0) {
    return VH_ERR_INVALID_ARGUMENT;
  }
  return vh::nn::backward(params, static_cast<const __nv_bfloat16*>(packed), depth, target, out, batch, width, height,
                          static_cast<unsigned char*>(workspace), grads, loss, error, as_stream(stream)) == cudaSuccess
             ? VH_OK
             : VH_ERR_CUDA;
}

vh_status vh_nn_adam(float* params, const float* grads, float* m, float* v, float lr, float beta1, float beta2, float eps,
                     int32_t step, void* stream) {
  if (!params || !grads || !m || !v || step < 1) return VH_ERR_INVALID_ARGUMENT;
  return vh::nn::adam(params, grads, m, v, lr, beta1, beta2, eps, step, as_stream(stream)) == cudaSuccess ? VH_OK
                                                                                                          : VH_ERR_CUDA;
}

vh_status vh_set_depth_denoiser(vh_volume* v, const float* params) {
  if (!v) return VH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(v->params.device);
  if (!params) {
    dfree(v->d_nn_params);
    dfree(v->d_nn_packed);
    return VH_OK;
  }
  const size_t n = static_cast<size_t>(vh::nn::param_count());
  if (!v->d_nn_params) VH_CUDA(v, dalloc(&v->d_nn_params, n));
  if (!v->d_nn_packed) VH_CUDA(v, cudaMalloc(reinterpret_cast<void**>(&v->d_nn_packed), 4 * 9 * 32 * 32 * sizeof(__nv_bfloat16)));
  VH_CUDA(v, cudaMemcpy(v->d_nn_params, params, n * sizeof(float), cudaMemcpyHostToDevice));
  VH_CUDA(v, vh::nn::pack_weights(v->d_nn_params, v->d_nn_packed, nullptr));
  VH_CUDA(v, cudaDeviceSynchronize());
  return VH_OK;
}

}  // extern "C"
