// PNG decoding for glTF textures (png.cpp).
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace cr {

struct Image {
  int width = 0, height = 0;
  int bits = 8;               // bits per sample of the file (8 or 16)
  std::vector<uint8_t> rgba;  // width * height * 4, row 0 first (high bytes of 16-bit samples)
};

bool isPng(const uint8_t* data, size_t size);
// Throws std::runtime_error on malformed or unsupported input.
Image decodePng(const uint8_t* data, size_t size);

}  // namespace cr
