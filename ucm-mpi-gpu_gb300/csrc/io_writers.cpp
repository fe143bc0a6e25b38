// io_writers.cpp -- the on-disk formats the reference writes for each piece
// (src/main.cpp:444-452): the non-max gPb as an OpenCV FileStorage YAML
// matrix (OpenCVFileWriter, src/utilities.cpp:33-37) and every plane as an
// 8-bit greyscale PNG scaled min..max to 0..255 (OpenCVImageWriter,
// src/utilities.cpp:21-31), so files from this library drop in where the
// reference's are read (UCM, visualisation).  No image library: the PNG is
// written with stored (uncompressed) deflate blocks, its CRC-32 and
// Adler-32 computed here.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <string>
#include <vector>

#include "../../include/gpb.h"
#include "gpb_internal.h"

namespace {

// CRC-32 (ISO 3309 / PNG), table-driven, polynomial 0xEDB88320 reflected
uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {
  static const std::array<uint32_t, 256> table = [] {  // built once, thread-safe
    std::array<uint32_t, 256> t{};
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t c = i;
      for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      t[i] = c;
    }
    return t;
  }();
  crc = ~crc;
  for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 255] ^ (crc >> 8);
  return ~crc;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24));
  v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t>& out, const char type[4], const std::vector<uint8_t>& data) {
  put_be32(out, (uint32_t)data.size());
  std::vector<uint8_t> td(type, type + 4);
  td.insert(td.end(), data.begin(), data.end());
  out.insert(out.end(), td.begin(), td.end());
  put_be32(out, crc32_update(0, td.data(), td.size()));
}

}  // namespace

extern "C" gpb_status gpb_write_yml(const char* path, const char* name, const float* data, uint32_t rows,
                                    uint32_t cols) {
  return gpb::guarded(nullptr, [&]() -> gpb_status {
    if (!path || !name || !data || rows == 0 || cols == 0) return GPB_ERR_ARG;
    FILE* f = fopen(path, "w");
    if (!f) return GPB_ERR_ARG;
    // the layout of cv::FileStorage for a CV_64FC1 matrix; values printed
    // with 17 significant digits so that every value reads back exactly
    fprintf(f, "%%YAML:1.0\n---\n%s: !!opencv-matrix\n   rows: %u\n   cols: %u\n   dt: d\n   data: [", name, rows,
            cols);
    const size_t n = (size_t)rows * cols;
    for (size_t i = 0; i < n; i++) {
      fprintf(f, "%s%.17g", i ? ", " : " ", (double)data[i]);
      if (i % 4 == 3 && i + 1 < n) fprintf(f, "\n       ");
    }
    fprintf(f, " ]\n");
    const bool ok = ferror(f) == 0;
    fclose(f);
    return ok ? GPB_OK : GPB_ERR_ARG;
  });
}

extern "C" gpb_status gpb_write_png_minmax(const char* path, const float* data, uint32_t rows, uint32_t cols) {
  return gpb::guarded(nullptr, [&]() -> gpb_status {
    if (!path || !data || rows == 0 || cols == 0) return GPB_ERR_ARG;
    const size_t n = (size_t)rows * cols;
    double mn = data[0], mx = data[0];
    for (size_t i = 1; i < n; i++) {
      mn = std::min(mn, (double)data[i]);
      mx = std::max(mx, (double)data[i]);
    }
    // convertTo(CV_8U, alpha, beta): saturate(round-to-nearest-even(v * alpha + beta))
    const double alpha = mx > mn ? 255.0 / (mx - mn) : 0.0, beta = mx > mn ? -mn * 255.0 / (mx - mn) : 0.0;
    std::vector<uint8_t> raw;  // filter byte 0, then the row
    raw.reserve((size_t)rows * (cols + 1));
    for (uint32_t y = 0; y < rows; y++) {
      raw.push_back(0);
      for (uint32_t x = 0; x < cols; x++) {
        double v = nearbyint((double)data[(size_t)y * cols + x] * alpha + beta);
        v = v < 0 ? 0 : (v > 255 ? 255 : v);
        raw.push_back((uint8_t)v);
      }
    }
    // zlib stream: header 0x78 0x01, stored deflate blocks of <= 65535 bytes, Adler-32
    std::vector<uint8_t> z = {0x78, 0x01};
    for (size_t off = 0;;) {  // raw holds at least one row
      const size_t len = std::min<size_t>(65535, raw.size() - off);
      const bool last = off + len >= raw.size();
      z.push_back(last ? 1 : 0);
      z.push_back((uint8_t)len);
      z.push_back((uint8_t)(len >> 8));
      z.push_back((uint8_t)~len);
      z.push_back((uint8_t)(~len >> 8));
      z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
      off += len;
      if (last) break;
    }
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
      a = (a + c) % 65521;
      b = (b + a) % 65521;
    }
    put_be32(z, (b << 16) | a);
    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, cols);
    put_be32(ihdr, rows);
    ihdr.push_back(8);  // bit depth
    ihdr.push_back(0);  // greyscale
    ihdr.push_back(0);  // deflate
    ihdr.push_back(0);  // adaptive filtering (every row: filter 0)
    ihdr.push_back(0);  // no interlace
    chunk(png, "IHDR", ihdr);
    chunk(png, "IDAT", z);
    chunk(png, "IEND", {});
    FILE* f = fopen(path, "wb");
    if (!f) return GPB_ERR_ARG;
    const bool ok = fwrite(png.data(), 1, png.size(), f) == png.size();
    fclose(f);
    return ok ? GPB_OK : GPB_ERR_ARG;
  });
}
