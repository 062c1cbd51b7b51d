// vh_dataset.cpp -- the reference's dataset reader (include/tsdfmc/dataset_io.h) behind the C ABI, portable:
// the reference decodes depth PNGs through Windows WIC only; here vh_png.cpp does it on any host.  Metadata
// parsing, pose conversion and the frame-id listing follow dataset_io.h and math_types.h in the same
// arithmetic (doubles parsed by the standard stream, then narrowed to float; quaternion normalised and
// expanded in the reference's operation order), so poses and intrinsics are bit-identical to the reference's.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/voxelhash_gb300.h"
#include "vh_png.h"

namespace fs = std::filesystem;

namespace {

thread_local std::string g_error;

vh_status dfail(vh_status s, const std::string& msg) {
  g_error = msg;
  return s;
}

// readNumericValuesFromFile (dataset_io.h:38-55)
vh_status read_numbers(const fs::path& path, std::vector<double>& values) {
  std::ifstream input(path);
  if (!input) return dfail(VH_ERR_IO, "Failed to open metadata file: " + path.string());
  values.clear();
  double value = 0.0;
  while (input >> value) values.push_back(value);
  if (values.empty()) return dfail(VH_ERR_FORMAT, "Failed to parse numeric metadata from file: " + path.string());
  return VH_OK;
}

// listDatasetFrameIds (dataset_io.h:135-152)
vh_status frame_ids(const fs::path& root, std::vector<int>& ids) {
  ids.clear();
  std::error_code ec;
  fs::directory_iterator it(root, ec), end;
  if (ec) return dfail(VH_ERR_IO, "Failed to list dataset directory: " + root.string());
  for (; it != end; it.increment(ec)) {
    if (ec) return dfail(VH_ERR_IO, "Failed to list dataset directory: " + root.string());
    if (!it->is_directory()) continue;
    const std::string name = it->path().filename().string();
    if (!std::all_of(name.begin(), name.end(), [](unsigned char c) { return std::isdigit(c) != 0; })) continue;
    try {
      ids.push_back(std::stoi(name));
    } catch (const std::exception&) {
      return dfail(VH_ERR_FORMAT, "Frame directory name out of range: " + name);
    }
  }
  std::sort(ids.begin(), ids.end());
  return VH_OK;
}

// findDatasetIntrinsicsMetadataPath (dataset_io.h:64-79)
vh_status find_metadata(const fs::path& preferred, fs::path& out) {
  if (fs::exists(preferred)) {
    out = preferred;
    return VH_OK;
  }
  const fs::path root = preferred.parent_path();
  std::vector<int> ids;
  const vh_status st = frame_ids(root, ids);
  if (st != VH_OK) return st;
  for (int id : ids) {
    const fs::path params = root / std::to_string(id) / "params.txt";
    if (fs::exists(params)) {
      out = params;
      return VH_OK;
    }
  }
  return dfail(VH_ERR_IO, "Failed to locate dataset intrinsics metadata. Expected " + preferred.string() +
                              " or <frame>/params.txt under " + root.string());
}

// findFirstDatasetDepthImage (dataset_io.h:81-90)
vh_status first_depth_image(const fs::path& root, fs::path& out) {
  std::vector<int> ids;
  const vh_status st = frame_ids(root, ids);
  if (st != VH_OK) return st;
  for (int id : ids) {
    const fs::path p = root / std::to_string(id) / "depth.png";
    if (fs::exists(p)) {
      out = p;
      return VH_OK;
    }
  }
  return dfail(VH_ERR_IO, "Failed to locate any dataset depth.png under " + root.string());
}

vh_status decode_png(const std::string& path, vh::png::Image& img) {
  std::vector<uint8_t> file;
  std::string err;
  if (!vh::png::read_file(path, file, err)) return dfail(VH_ERR_IO, "Failed to open depth PNG: " + path);
  if (!vh::png::decode_gray16(file, img, err)) return dfail(VH_ERR_FORMAT, "Failed to decode depth PNG: " + path + " (" + err + ")");
  return VH_OK;
}

}  // namespace

extern "C" {

const char* vh_dataset_last_error(void) { return g_error.c_str(); }

vh_status vh_dataset_list_frames(const char* root, int32_t* ids, size_t max_ids, size_t* count) {
  if (!root || !count) return dfail(VH_ERR_INVALID_ARGUMENT, "vh_dataset_list_frames: bad argument");
  std::vector<int> v;
  const vh_status st = frame_ids(root, v);
  if (st != VH_OK) return st;
  *count = v.size();
  if (!ids) return VH_OK;
  if (max_ids < v.size()) return dfail(VH_ERR_BUFFER_TOO_SMALL, "vh_dataset_list_frames: ids too small");
  for (size_t i = 0; i < v.size(); ++i) ids[i] = v[i];
  return VH_OK;
}

// loadPoseFromFile (dataset_io.h:154-188)
vh_status vh_dataset_load_pose(const char* path, vh_pose* T) {
  if (!path || !T) return dfail(VH_ERR_INVALID_ARGUMENT, "vh_dataset_load_pose: bad argument");
  std::vector<double> v;
  const vh_status st = read_numbers(path, v);
  if (st != VH_OK) return st;
  if (v.size() == 7U) {
    // quaternionToMatrix (math_types.h:158-178) of the normalised quaternion (:148-156)
    const float qw = static_cast<float>(v[0]), qx = static_cast<float>(v[1]), qy = static_cast<float>(v[2]),
                qz = static_cast<float>(v[3]);
    const float length = std::sqrt(qw * qw + qx * qx + qy * qy + qz * qz);
    float w = 1.0f, x = 0.0f, y = 0.0f, z = 0.0f;
    if (!(length <= 1e-8f)) {
      w = qw / length;
      x = qx / length;
      y = qy / length;
      z = qz / length;
    }
    const float ww = w * w, xx = x * x, yy = y * y, zz = z * z;
    const float wx = w * x, wy = w * y, wz = w * z, xy = x * y, xz = x * z, yz = y * z;
    const float R[9] = {ww + xx - yy - zz, 2.0f * (xy - wz),  2.0f * (xz + wy),
                        2.0f * (xy + wz),  ww - xx + yy - zz, 2.0f * (yz - wx),
                        2.0f * (xz - wy),  2.0f * (yz + wx),  ww - xx - yy + zz};
    std::memcpy(T->R, R, sizeof(R));
    T->t[0] = static_cast<float>(v[4]);
    T->t[1] = static_cast<float>(v[5]);
    T->t[2] = static_cast<float>(v[6]);
    return VH_OK;
  }
  if (v.size() == 12U || v.size() == 16U) {
    const int r[9] = {0, 1, 2, 4, 5, 6, 8, 9, 10};
    for (int i = 0; i < 9; ++i) T->R[i] = static_cast<float>(v[r[i]]);
    T->t[0] = static_cast<float>(v[3]);
    T->t[1] = static_cast<float>(v[7]);
    T->t[2] = static_cast<float>(v[11]);
    return VH_OK;
  }
  return dfail(VH_ERR_FORMAT, "Unsupported pose format in " + std::string(path) + " (expected 7, 12, or 16 numeric values)");
}

vh_status vh_png_read_gray16(const char* path, uint16_t* pixels, size_t max_pixels, int32_t* width, int32_t* height) {
  if (!path || !width || !height) return dfail(VH_ERR_INVALID_ARGUMENT, "vh_png_read_gray16: bad argument");
  vh::png::Image img;
  const vh_status st = decode_png(path, img);
  if (st != VH_OK) return st;
  *width = img.width;
  *height = img.height;
  if (!pixels) return VH_OK;
  if (max_pixels < img.pixels.size()) return dfail(VH_ERR_BUFFER_TOO_SMALL, "vh_png_read_gray16: pixels too small");
  std::memcpy(pixels, img.pixels.data(), img.pixels.size() * sizeof(uint16_t));
  return VH_OK;
}

vh_status vh_dataset_load_intrinsics(const char* metadata_path, vh_intrinsics* K, float* depth_scale) {
  if (!metadata_path || !K || !depth_scale) return dfail(VH_ERR_INVALID_ARGUMENT, "vh_dataset_load_intrinsics: bad argument");
  fs::path path;
  vh_status st = find_metadata(metadata_path, path);
  if (st != VH_OK) return st;
  std::vector<double> v;
  st = read_numbers(path, v);
  if (st != VH_OK) return st;
  // parseIntrinsicsMetadataValues (dataset_io.h:92-133)
  vh_intrinsics k{};
  bool has_resolution = false;
  float scale = 1.0f;
  if (v.size() == 5U || v.size() == 6U || v.size() == 7U) {
    k.fx = static_cast<float>(v[0]);
    k.fy = static_cast<float>(v[1]);
    k.cx = static_cast<float>(v[2]);
    k.cy = static_cast<float>(v[3]);
    if (v.size() == 5U) {
      scale = static_cast<float>(v[4]);
    } else {
      k.width = static_cast<int32_t>(v[4]);
      k.height = static_cast<int32_t>(v[5]);
      scale = v.size() == 7U ? static_cast<float>(v[6]) : 1.0f;
      has_resolution = true;
    }
  } else {
    return dfail(VH_ERR_FORMAT, "Unsupported intrinsics metadata format in " + path.string() +
                                    " (expected 5, 6, or 7 numeric values)");
  }
  if (!has_resolution) {
    // resolveDatasetRootFromMetadataPath (dataset_io.h:57-62) + completeIntrinsicsResolutionFromDepth (:240-274)
    const fs::path root = path.filename() == "params.txt" ? path.parent_path().parent_path() : path.parent_path();
    fs::path depth;
    st = first_depth_image(root, depth);
    if (st != VH_OK) return st;
    vh::png::Image img;
    st = decode_png(depth.string(), img);
    if (st != VH_OK) return st;
    k.width = img.width;
    k.height = img.height;
  }
  *K = k;
  *depth_scale = scale;
  return VH_OK;
}

// loadDepthPng (dataset_io.h:276-361)
vh_status vh_dataset_load_depth_png(const char* path, const vh_intrinsics* K, float depth_scale, float* depth,
                                    uint64_t* valid_samples) {
  if (!path || !K || !depth || K->width <= 0 || K->height <= 0) {
    return dfail(VH_ERR_INVALID_ARGUMENT, "vh_dataset_load_depth_png: bad argument");
  }
  vh::png::Image img;
  const vh_status st = decode_png(path, img);
  if (st != VH_OK) return st;
  if (img.width != K->width || img.height != K->height) {
    return dfail(VH_ERR_FORMAT, "Depth image resolution does not match dataset intrinsics metadata: " + std::string(path) +
                                    " (detail=" + std::to_string(img.width) + "x" + std::to_string(img.height) + " vs " +
                                    std::to_string(K->width) + "x" + std::to_string(K->height) + ")");
  }
  uint64_t valid = 0;
  for (size_t i = 0; i < img.pixels.size(); ++i) {
    depth[i] = 0.0f;
    const uint16_t raw = img.pixels[i];
    if (raw == 0U) continue;
    const float d = static_cast<float>(raw) * depth_scale;
    if (d <= 0.0f) continue;
    depth[i] = d;
    ++valid;
  }
  if (valid_samples) *valid_samples = valid;
  return VH_OK;
}

}  // extern "C"
