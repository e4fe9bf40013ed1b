// cr_io.h -- host-side file formats: image codecs (cr_image.cpp) and the
// XML + OBJ/MTL scene importer (cr_import.cpp).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace cr {

void clearError();
int fail(int code, const char* fmt, ...);

namespace io {

// An image as the reference's Image holds it, interleaved: pixel (x, y)
// channel c at pixels[(y * width + x) * channels + c], row 0 first.
struct Image {
    uint32_t width = 0, height = 0, channels = 0;
    std::vector<float> pixels;
};

bool readFile(const std::string& path, std::vector<uint8_t>& data);
bool inflateRaw(const uint8_t* p, size_t n, std::vector<uint8_t>& out);
bool zlibDecompress(const uint8_t* p, size_t n, std::vector<uint8_t>& out);
uint16_t floatToHalf(float f);
float halfToFloat(uint16_t h);

int writeExr(const std::string& path, uint32_t w, uint32_t h, uint32_t ch, const float* px, std::string& err);
int readExr(const std::vector<uint8_t>& d, Image& img, std::string& err);
int writePng(const std::string& path, uint32_t w, uint32_t h, uint32_t ch, const float* px, bool gamma,
             std::string& err);
int readPng(const std::vector<uint8_t>& d, bool toLinear, Image& img, std::string& err);
// Image::load (Utils/Image.cpp:262-270): ".exr" by extension, PNG otherwise.
int loadImage(const std::string& path, bool toLinear, Image& img, std::string& err);

}  // namespace io
}  // namespace cr
