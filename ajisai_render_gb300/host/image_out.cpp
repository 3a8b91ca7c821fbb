#include "image_out.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

namespace ajh {
namespace {

void pixel(const float* rgbw, uint64_t i, float out[3]) {
  const float* p = rgbw + 4 * i;
  for (int k = 0; k < 3; ++k) out[k] = p[3] != 0.f ? p[k] / p[3] : 0.f;
}

// Color3::toSrgb (math/color.h:52-58)
float to_srgb(float c) {
  const float a = 0.055f;
  if (c > 0.0031308f) return (1.0f + a) * std::pow(c, 1.0f / 2.4f) - a;
  return c * 12.92f;
}

uint32_t crc32(const uint8_t* d, size_t n, uint32_t c = 0) {
  static uint32_t table[256];
  static bool ready = false;
  if (!ready) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t v = i;
      for (int k = 0; k < 8; ++k) v = (v & 1u) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
      table[i] = v;
    }
    ready = true;
  }
  c = ~c;
  for (size_t i = 0; i < n; ++i) c = table[(c ^ d[i]) & 0xffu] ^ (c >> 8);
  return ~c;
}

void be32(std::vector<uint8_t>& o, uint32_t v) {
  o.push_back((uint8_t)(v >> 24));
  o.push_back((uint8_t)(v >> 16));
  o.push_back((uint8_t)(v >> 8));
  o.push_back((uint8_t)v);
}

void chunk(std::vector<uint8_t>& png, const char* type,
           const std::vector<uint8_t>& data) {
  be32(png, (uint32_t)data.size());
  std::vector<uint8_t> td(type, type + 4);
  td.insert(td.end(), data.begin(), data.end());
  png.insert(png.end(), td.begin(), td.end());
  be32(png, crc32(td.data(), td.size()));
}

void write_file(const std::string& path, const void* data, size_t n) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  const size_t w = std::fwrite(data, 1, n, f);
  std::fclose(f);
  if (w != n) throw std::runtime_error("short write to " + path);
}

void write_pfm(const std::string& path, const float* rgbw, uint32_t w,
               uint32_t h) {
  char hdr[64];
  const int hn = std::snprintf(hdr, sizeof(hdr), "PF\n%u %u\n-1.0\n", w, h);
  std::vector<uint8_t> out(hdr, hdr + hn);
  std::vector<float> row(3 * (size_t)w);
  for (uint32_t y = 0; y < h; ++y) {
    const uint32_t src = h - 1 - y;  // bottom row first
    for (uint32_t x = 0; x < w; ++x)
      pixel(rgbw, (uint64_t)src * w + x, &row[3 * (size_t)x]);
    for (size_t i = 0; i < row.size(); ++i) {  // little endian
      uint32_t u;
      std::memcpy(&u, &row[i], 4);
      const uint8_t le[4] = {(uint8_t)u, (uint8_t)(u >> 8), (uint8_t)(u >> 16),
                             (uint8_t)(u >> 24)};
      out.insert(out.end(), le, le + 4);
    }
  }
  write_file(path, out.data(), out.size());
}

void write_png(const std::string& path, const float* rgbw, uint32_t w,
               uint32_t h) {
  // filtered scanlines: filter type 0, RGB bytes; rows flipped
  std::vector<uint8_t> raw;
  raw.reserve((size_t)h * (1 + 3 * (size_t)w));
  for (uint32_t y = 0; y < h; ++y) {
    const uint32_t src = h - 1 - y;
    raw.push_back(0);
    for (uint32_t x = 0; x < w; ++x) {
      float c[3];
      pixel(rgbw, (uint64_t)src * w + x, c);
      for (int k = 0; k < 3; ++k) {
        const float s = std::clamp(to_srgb(c[k]), 0.f, 1.f);
        raw.push_back((uint8_t)std::clamp<int>((int)std::round(s * 255.5), 0,
                                               255));
      }
    }
  }
  // zlib stream of stored deflate blocks
  std::vector<uint8_t> z = {0x78, 0x01};
  size_t pos = 0;
  do {
    const size_t n = std::min<size_t>(65535, raw.size() - pos);
    const bool last = pos + n == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((uint8_t)n);
    z.push_back((uint8_t)(n >> 8));
    z.push_back((uint8_t)~n);
    z.push_back((uint8_t)(~n >> 8));
    z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
    pos += n;
  } while (pos < raw.size());
  uint32_t a = 1, b = 0;  // Adler-32
  for (uint8_t v : raw) {
    a = (a + v) % 65521u;
    b = (b + a) % 65521u;
  }
  be32(z, (b << 16) | a);
  std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  std::vector<uint8_t> ihdr;
  be32(ihdr, w);
  be32(ihdr, h);
  ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit RGB
  chunk(png, "IHDR", ihdr);
  chunk(png, "IDAT", z);
  chunk(png, "IEND", {});
  write_file(path, png.data(), png.size());
}

bool ends_with(const std::string& s, const char* suf) {
  const size_t n = std::strlen(suf);
  return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

}  // namespace

void WriteImage(const std::string& path, const float* rgbw, uint32_t width,
                uint32_t height) {
  if (ends_with(path, ".pfm"))
    write_pfm(path, rgbw, width, height);
  else if (ends_with(path, ".png"))
    write_png(path, rgbw, width, height);
  else
    throw std::runtime_error("unsupported image format: " + path +
                             " (.pfm or .png)");
}

}  // namespace ajh
