// In-memory stand-in for stb_image.h used when compiling the reference sources.
//
// TEST INFRASTRUCTURE ONLY. The reference's post-filters (denoising/*.cpp) read their
// inputs with stbi_loadf(path) and write results with stbi_write_hdr(path). This shim
// serves loads from, and captures writes into, an in-process table keyed by path, so the
// harness can run the reference's filter() functions on arrays without any files.
#pragma once
// The real header includes <math.h> (for ldexp/pow); in C++ that also brings the float
// overloads of exp/acos into the global namespace, which the reference filters rely on.
#include <math.h>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace stb_shim {
struct Img { int w = 0, h = 0, comp = 0; std::vector<float> data; };
inline std::map<std::string, Img>& table() {
    static std::map<std::string, Img> t;
    return t;
}
}  // namespace stb_shim

inline float* stbi_loadf(const char* name, int* w, int* h, int* comp, int) {
    auto& t = stb_shim::table();
    auto it = t.find(name ? name : "");
    if (it == t.end()) {
        if (w) *w = 0;
        if (h) *h = 0;
        if (comp) *comp = 0;
        return nullptr;
    }
    const auto& img = it->second;
    float* out = static_cast<float*>(std::malloc(img.data.size() * sizeof(float)));
    std::memcpy(out, img.data.data(), img.data.size() * sizeof(float));
    if (w) *w = img.w;
    if (h) *h = img.h;
    if (comp) *comp = img.comp;
    return out;
}
inline void stbi_image_free(void* p) { std::free(p); }
// 8-bit loads (the evaluation tool's PNG comparison): the table holds float images only, so
// every 8-bit load fails as for a missing file.
inline unsigned char* stbi_load(const char*, int* w, int* h, int* comp, int) {
    if (w) *w = 0;
    if (h) *h = 0;
    if (comp) *comp = 0;
    return nullptr;
}
