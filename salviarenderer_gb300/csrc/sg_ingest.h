// sg_ingest.h -- host-side image codecs of the ingest path (sg_ingest.cpp),
// shared with the device-side entry points in sg_api.cu.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace sg::ingest {

// A decoded 8-bit image in FreeImage's scanline order (row 0 = the image's
// bottom line), `channels` bytes per pixel (3 = RGB, 4 = RGBA).
struct Image {
  uint32_t w = 0, h = 0, channels = 0;
  std::vector<uint8_t> px;
};

// PNG -> Image.  SG_OK, or SG_FAILED for anything not decodable (the format
// rules are those of sg_image_decode in salvia_gb300.h).
int32_t decode_png(uint8_t const* file, size_t size, Image& out);
// Image rows (FreeImage order, 3 or 4 channels) -> PNG bytes, 8-bit RGB / RGBA.
std::vector<uint8_t> encode_png(uint8_t const* px, uint32_t w, uint32_t h, uint32_t channels);
// RGB float rows (FreeImage order) -> Radiance RGBE bytes.
std::vector<uint8_t> encode_hdr(float const* rgb, uint32_t w, uint32_t h);

// zlib (RFC 1950) around DEFLATE (RFC 1951): the decoder fills `out`, whose
// size is the exact number of bytes the stream must produce; false on any
// malformed, short or long stream.
bool zlib_inflate(uint8_t const* src, size_t n, std::vector<uint8_t>& out);
std::vector<uint8_t> zlib_deflate(uint8_t const* src, size_t n);

}  // namespace sg::ingest
