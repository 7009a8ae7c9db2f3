// Minimal PNG reader / writer for the headless compute_disp tool (no third-party dependency).
// Reads 8-bit PNGs of color type 0 (gray), 2 (RGB), 4 (gray + alpha) and 6 (RGBA), non-interlaced, with
// the five standard row filters; writes 8- or 16-bit gray PNGs using stored (uncompressed) deflate blocks.
// The decoder implements DEFLATE (RFC 1951) inside a zlib stream (RFC 1950) and the PNG chunk format
// (ISO/IEC 15948).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace pngio {

struct Image {
    int width = 0, height = 0, channels = 0; // channels 1 (gray) or 3 (B, G, R: OpenCV's imread order)
    std::vector<uint8_t> pixels;             // row-major, interleaved
};

// Returns an empty string on success, else the reason.
std::string read_png(const std::string &path, Image &out);
std::string write_png_gray(const std::string &path, int width, int height, int bit_depth, const void *pixels);

// Inflate a zlib stream (exposed for the self test).
std::string zlib_inflate(const uint8_t *data, size_t n, std::vector<uint8_t> &out);
// Store-only zlib stream of `data`.
std::vector<uint8_t> zlib_store(const uint8_t *data, size_t n);

} // namespace pngio
