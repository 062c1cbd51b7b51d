// tsdfmc_gb300_adapter.cpp -- the reference's CUDA interfaces, implemented over the GB300 C ABI.
//
// Build the reference with this file in place of src/cuda_block_allocator.cu, src/cuda_tsdf_integrator.cu and
// src/cuda_mesh_extractor.cu (TSDFMC_HAVE_CUDA=1, include paths: the reference's include/ and src/, and this
// repository's include/), and link libvoxelhash_gb300.so.  reconstruction_backend.cpp and main.cpp compile
// unchanged: every function they call keeps the signature declared in src/cuda_block_allocator.h,
// src/cuda_tsdf_integrator.h and src/cuda_mesh_extractor.h.
//
// Behaviour mirrored from the reference:
//   * one device volume bound to one VoxelHashTSDF at a time, reset when another volume is passed
//     (the reference's GpuVolumeCache singleton, src/cuda_tsdf_integrator.cu:114-130);
//   * allocateActiveBlocksCuda is stateless, with a keys-only table sized by the reference's rule
//     nextPow2(2 * max(2048, 16 * samples)) (src/cuda_block_allocator.cu:322-323);
//   * allocation overflow (key range, full table) throws CudaActiveBlockAllocationFallback, a
//     std::runtime_error; where the reference catches it and re-allocates the frame on the CPU
//     (src/cuda_tsdf_integrator.cu:984-989), integrateDepthFrameCuda lets it propagate: the device volume
//     cannot hold the keys the CPU allocator would add;
//   * extractMeshCuda meshes the bound device volume, or uploads the host volume's observed blocks
//     (src/cuda_mesh_extractor.cu:640-653).
// Differences: gpuVolumeCacheFlatBlocks returns host memory (the reference returns device memory; its only
// caller is the mesh extractor this file replaces).  Device sizing comes from the environment:
// VH_HASH_BUCKETS (default 2^22) and VH_MAX_BLOCKS (default 2^17 blocks = 19 GB); the opt-in forms too:
// VH_LAYER_FORMAT, VH_ALLOCATION_MODE, VH_NORMAL_MODE, VH_FAST_MATH (all default 0, the reference's form).
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "cuda_block_allocator.h"
#include "cuda_mesh_extractor.h"
#include "cuda_tsdf_integrator.h"
#include "voxelhash_gb300.h"

namespace tsdfmc {

static_assert(sizeof(Triangle) == 9 * sizeof(float), "Triangle must be three packed Vec3f");
static_assert(sizeof(Voxel) == 6 * 3 * 16, "Voxel must be 6 x 3 layers of 16 bytes");

namespace {

vh_intrinsics to_intrinsics(const Intrinsics& K) { return vh_intrinsics{K.width, K.height, K.fx, K.fy, K.cx, K.cy}; }

vh_pose to_pose(const Pose& P) {
  vh_pose p{};
  for (int i = 0; i < 9; ++i) p.R[i] = P.R.data[static_cast<std::size_t>(i)];
  p.t[0] = P.t.x;
  p.t[1] = P.t.y;
  p.t[2] = P.t.z;
  return p;
}

uint32_t env_u32(const char* name, uint32_t fallback) {
  const char* s = std::getenv(name);
  if (!s || !*s) return fallback;
  return static_cast<uint32_t>(std::strtoul(s, nullptr, 0));
}

void check(vh_status st, const vh_volume* v, const char* what) {
  if (st == VH_OK) return;
  const std::string msg = std::string(what) + " failed: " + (v ? vh_last_error(v) : vh_status_string(st));
  if (st == VH_ERR_KEY_RANGE || st == VH_ERR_HASH_FULL) throw CudaActiveBlockAllocationFallback(msg);
  throw std::runtime_error(msg);
}

struct DeviceVolume {
  const VoxelHashTSDF* attached = nullptr;
  vh_volume* handle = nullptr;
  std::vector<BlockKey> keys;
  std::vector<VoxelHashTSDF::FlatBlockRecord> flat;
  ~DeviceVolume() {
    if (handle) vh_destroy(handle);
  }
};

DeviceVolume& device_volume() {
  static DeviceVolume dv;
  return dv;
}

vh_volume* create_volume(float voxel_size, float truncation, uint32_t buckets, uint32_t max_blocks) {
  vh_params p;
  vh_params_default(&p);
  p.voxel_size = voxel_size;
  p.truncation_distance = truncation;
  p.hash_buckets = buckets;
  p.max_blocks = max_blocks;
  p.layer_format = static_cast<int32_t>(env_u32("VH_LAYER_FORMAT", 0));
  vh_algorithm a;
  vh_algorithm_default(&a);  // the reference's constants; the opt-in switches default off
  a.allocation_mode = static_cast<int32_t>(env_u32("VH_ALLOCATION_MODE", 0));
  a.normal_mode = static_cast<int32_t>(env_u32("VH_NORMAL_MODE", 0));
  a.fast_math = static_cast<int32_t>(env_u32("VH_FAST_MATH", 0));
  vh_volume* v = nullptr;
  check(vh_create(&p, &a, &v), nullptr, "vh_create");
  return v;
}

vh_volume* bind(const VoxelHashTSDF& volume) {
  DeviceVolume& dv = device_volume();
  if (dv.attached != &volume || !dv.handle) {
    if (dv.handle) vh_destroy(dv.handle);
    dv.handle = create_volume(volume.voxelSize(), volume.truncationDistance(), env_u32("VH_HASH_BUCKETS", 1u << 22),
                              env_u32("VH_MAX_BLOCKS", 1u << 17));
    dv.attached = &volume;
    dv.keys.clear();
  }
  return dv.handle;
}

uint64_t block_count(vh_volume* v) {
  uint64_t n = 0;
  check(vh_block_count(v, &n), v, "vh_block_count");
  return n;
}

std::size_t next_pow2(std::size_t x) {
  std::size_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

}  // namespace

CudaBackendStatus queryCudaBackendStatus() {
  char msg[256];
  const vh_status st = vh_query_device(msg, sizeof(msg));
  return CudaBackendStatus{st == VH_OK, std::string(msg)};
}

std::vector<BlockKey> allocateActiveBlocksCuda(const DepthFrame& frame, const Pose& T_wc, const float voxel_size,
                                               const float truncation_distance, const int allocation_stride,
                                               const float* device_depth) {
  if (frame.depth.empty() && device_depth == nullptr) return {};
  const int stride = allocation_stride > 1 ? allocation_stride : 1;
  const std::size_t samples = static_cast<std::size_t>((frame.intrinsics.width + stride - 1) / stride) *
                              static_cast<std::size_t>((frame.intrinsics.height + stride - 1) / stride);
  if (samples == 0) return {};
  const std::size_t capacity = next_pow2(2 * std::max<std::size_t>(2048, samples * 16));
  if (capacity > 0xffffffffULL) {
    throw CudaActiveBlockAllocationFallback("GPU active block allocation requested an oversized device hash table.");
  }
  static vh_volume* table = nullptr;
  static std::size_t table_capacity = 0;
  static float table_vs = 0.0f, table_trunc = 0.0f;
  if (!table || table_capacity != capacity || table_vs != voxel_size || table_trunc != truncation_distance) {
    if (table) vh_destroy(table);
    table = create_volume(voxel_size, truncation_distance, static_cast<uint32_t>(capacity), 0);
    table_capacity = capacity;
    table_vs = voxel_size;
    table_trunc = truncation_distance;
  } else {
    check(vh_reset(table, nullptr), table, "vh_reset");
  }
  const vh_intrinsics K = to_intrinsics(frame.intrinsics);
  const vh_pose P = to_pose(T_wc);
  std::size_t n = 0;
  const float* depth = device_depth ? device_depth : frame.depth.data();
  check(vh_allocate(table, depth, device_depth ? 1 : 0, &K, &P, stride, nullptr, 0, &n, nullptr), table,
        "vh_allocate");
  std::vector<int32_t> raw(3 * n);
  check(vh_visible_block_keys(table, raw.data(), n, &n, nullptr), table, "vh_visible_block_keys");
  std::vector<BlockKey> keys(n);
  for (std::size_t i = 0; i < n; ++i) keys[i] = BlockKey{raw[3 * i], raw[3 * i + 1], raw[3 * i + 2]};
  return keys;
}

void integrateDepthFrameCuda(VoxelHashTSDF& volume, const DepthFrame& frame, const Pose& T_wc,
                             const int allocation_stride) {
  if (frame.depth.empty()) return;
  vh_volume* v = bind(volume);
  const vh_intrinsics K = to_intrinsics(frame.intrinsics);
  const vh_pose P = to_pose(T_wc);
  check(vh_integrate(v, frame.depth.data(), 0, &K, &P, allocation_stride, nullptr), v, "vh_integrate");
  check(vh_synchronize(v, nullptr), v, "vh_synchronize");
  device_volume().keys.clear();
}

bool hasGpuVolumeCache(const VoxelHashTSDF& volume) {
  DeviceVolume& dv = device_volume();
  return dv.attached == &volume && dv.handle && block_count(dv.handle) > 0;
}

std::size_t gpuVolumeCacheBlockCount(const VoxelHashTSDF& volume) {
  return hasGpuVolumeCache(volume) ? static_cast<std::size_t>(block_count(device_volume().handle))
                                   : volume.blockCount();
}

std::size_t gpuVolumeCacheObservedVoxelCount(const VoxelHashTSDF& volume) {
  if (!hasGpuVolumeCache(volume)) return volume.observedVoxelCount();
  uint64_t n = 0;
  check(vh_observed_voxel_count(device_volume().handle, &n), device_volume().handle, "vh_observed_voxel_count");
  return static_cast<std::size_t>(n);
}

const std::vector<BlockKey>& gpuVolumeCacheBlockKeys(const VoxelHashTSDF& volume) {
  static const std::vector<BlockKey> kEmpty;
  if (!hasGpuVolumeCache(volume)) return kEmpty;
  DeviceVolume& dv = device_volume();
  const uint64_t n = block_count(dv.handle);
  std::vector<int32_t> raw(3 * n);
  check(vh_export_blocks(dv.handle, 0, n, raw.data(), nullptr, 0, nullptr), dv.handle, "vh_export_blocks");
  dv.keys.resize(n);
  for (uint64_t i = 0; i < n; ++i) dv.keys[i] = BlockKey{raw[3 * i], raw[3 * i + 1], raw[3 * i + 2]};
  return dv.keys;
}

const VoxelHashTSDF::FlatBlockRecord* gpuVolumeCacheFlatBlocks(const VoxelHashTSDF& volume) {
  if (!hasGpuVolumeCache(volume)) return nullptr;
  DeviceVolume& dv = device_volume();
  const std::vector<BlockKey>& keys = gpuVolumeCacheBlockKeys(volume);
  const std::size_t per_block = VoxelHashTSDF::kBlockVolume * sizeof(Voxel);
  std::vector<unsigned char> vox(keys.size() * per_block);
  check(vh_export_blocks(dv.handle, 0, keys.size(), nullptr, vox.data(), 0, nullptr), dv.handle,
        "vh_export_blocks");
  dv.flat.resize(keys.size());
  for (std::size_t i = 0; i < keys.size(); ++i) {
    dv.flat[i].key = keys[i];
    std::memcpy(dv.flat[i].voxels, vox.data() + i * per_block, per_block);
  }
  return dv.flat.data();
}

std::vector<Triangle> extractMeshCuda(const VoxelHashTSDF& volume, const float iso_level) {
  vh_volume* v = nullptr;
  vh_volume* temporary = nullptr;
  if (hasGpuVolumeCache(volume)) {
    v = device_volume().handle;
  } else {
    const std::vector<VoxelHashTSDF::FlatBlockRecord> host = volume.copyObservedBlocksToFlat();
    if (host.empty()) return {};
    temporary = create_volume(volume.voxelSize(), volume.truncationDistance(),
                              static_cast<uint32_t>(next_pow2(2 * host.size() + 64)),
                              static_cast<uint32_t>(host.size()));
    std::vector<int32_t> keys(3 * host.size());
    std::vector<unsigned char> vox(host.size() * sizeof(host[0].voxels));
    for (std::size_t i = 0; i < host.size(); ++i) {
      keys[3 * i] = host[i].key.x;
      keys[3 * i + 1] = host[i].key.y;
      keys[3 * i + 2] = host[i].key.z;
      std::memcpy(vox.data() + i * sizeof(host[i].voxels), host[i].voxels, sizeof(host[i].voxels));
    }
    check(vh_import_blocks(temporary, keys.data(), vox.data(), host.size(), 0, nullptr), temporary,
          "vh_import_blocks");
    v = temporary;
  }
  std::size_t n = 0;
  std::vector<Triangle> tris;
  try {
    check(vh_extract_mesh(v, iso_level, &n, nullptr), v, "vh_extract_mesh");
    tris.resize(n);
    if (n) check(vh_copy_mesh(v, reinterpret_cast<float*>(tris.data()), n, 0, nullptr), v, "vh_copy_mesh");
  } catch (...) {
    if (temporary) vh_destroy(temporary);
    throw;
  }
  if (temporary) vh_destroy(temporary);
  return tris;
}

}  // namespace tsdfmc
