// In-memory stand-in for stb_image_write.h (see stb_image.h): HDR writes are captured
// into the shim's table, PNG writes are accepted and dropped. TEST INFRASTRUCTURE ONLY.
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
inline int stbi_write_png(const char*, int, int, int, const void*, int) { return 1; }
