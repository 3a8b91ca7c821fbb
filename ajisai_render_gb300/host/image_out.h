// Film output.  `rgbw` is the C ABI's film: [h][w][4] = (sum of radiance,
// sum of weights) per pixel; the image is rgb / w (0 where w is 0), as
// Film::WriteImage forms it (film.h:131-152; the PT path leaves the splat
// image empty).
//   .pfm  float32 RGB, little endian, bottom row first -- the HDR output
//   .png  8-bit RGB as ImageWriter::Write makes it (image.cpp:32-62): the
//         sRGB transfer curve, clamp to [0,1], round(v * 255.5) clamped to
//         [0, 255], rows written flipped (stbi_flip_vertically_on_write);
//         stored (uncompressed) deflate blocks
#pragma once
#include <cstdint>
#include <string>

namespace ajh {

// Throws std::runtime_error when the file cannot be written or the
// extension is neither .pfm nor .png.
void WriteImage(const std::string& path, const float* rgbw, uint32_t width,
                uint32_t height);

}  // namespace ajh
