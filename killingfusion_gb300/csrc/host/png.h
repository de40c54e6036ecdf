// PNG reading for the reference's dataset layout (16-bit depth and 8-bit
// mask images, read by cv::imread in DatasetReader.cpp:49-66), without
// OpenCV or zlib: a decoder of the zlib/DEFLATE stream (RFC 1950/1951) and of
// PNG's scanline filters (PNG specification, ISO/IEC 15948), written from
// those documents.  Non-interlaced grey, grey+alpha, RGB and RGBA images of
// bit depth 8 or 16.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace kf {
namespace png {

struct Image {
  int width = 0, height = 0;
  int channels = 0;   // 1 grey, 2 grey+alpha, 3 RGB, 4 RGBA
  int bit_depth = 0;  // 8 or 16
  // samples, row-major, channel-interleaved; 16-bit samples in host order
  std::vector<uint16_t> samples;
};

// Decodes a PNG file held in memory; throws std::runtime_error on malformed
// or unsupported input.
Image decode(const std::vector<uint8_t> &file);
Image read(const std::string &path);

// Inflates a zlib stream (RFC 1950 wrapper around RFC 1951 DEFLATE).
std::vector<uint8_t> inflate_zlib(const uint8_t *data, size_t size);

}  // namespace png
}  // namespace kf
