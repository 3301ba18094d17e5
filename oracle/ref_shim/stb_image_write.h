// In-memory stand-in for stb_image_write.h (see stb_image.h): HDR writes are captured into
// the shim's float table, PNG writes (8-bit RGB rows) into its byte table, both keyed by path.
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include <string>
#include <vector>
#include "stb_image.h"

inline int stbi_write_hdr(const char* name, int w, int h, int comp, const float* data) {
    stb_shim::Img img;
    img.w = w;
    img.h = h;
    img.comp = comp;
    img.data.assign(data, data + size_t(w) * h * comp);
    stb_shim::table()[name ? name : ""] = img;
    return 1;
}
namespace stb_shim {
struct Png { int w = 0, h = 0, comp = 0; std::vector<unsigned char> data; };
inline std::map<std::string, Png>& png_table() {
    static std::map<std::string, Png> t;
    return t;
}
}  // namespace stb_shim

inline int stbi_write_png(const char* name, int w, int h, int comp, const void* data, int stride) {
    stb_shim::Png img;
    img.w = w;
    img.h = h;
    img.comp = comp;
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (int y = 0; y < h; ++y) img.data.insert(img.data.end(), p + size_t(y) * stride, p + size_t(y) * stride + size_t(w) * comp);
    stb_shim::png_table()[name ? name : ""] = img;
    return 1;
}
