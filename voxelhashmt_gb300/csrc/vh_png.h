// vh_png.h -- portable grayscale PNG decoding for depth images (host code).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace vh {
namespace png {

struct Image {
  int width = 0, height = 0;
  std::vector<uint16_t> pixels;  // row-major, 16-bit gray
};

// Decodes a PNG held in memory to 16-bit gray (grayscale colour types only); false + err on failure.
bool decode_gray16(const std::vector<uint8_t>& file, Image& img, std::string& err);
bool read_file(const std::string& path, std::vector<uint8_t>& out, std::string& err);

}  // namespace png
}  // namespace vh
