// Reference post-filter harness: one of the reference's own denoising/*.cpp translation
// units (selected with -DRPD_REF_FILTER_SOURCE) compiled against oracle/ref_shim, its CLI
// main() renamed away, driven through the in-memory stb shim.
//
// TEST INFRASTRUCTURE ONLY. Built into oracle/_ref/ by oracle/Makefile; used by the tests
// to pin the C restatement of the filters and to produce the filter golden vectors.
#define main rpd_reference_filter_cli_main
#include RPD_REF_FILTER_SOURCE
#undef main

#include <filesystem>

namespace {
void put(const char* name, const float* data, int w, int h) {
    stb_shim::Img img;
    img.w = w;
    img.h = h;
    img.comp = 3;
    img.data.assign(data, data + size_t(w) * h * 3);
    stb_shim::table()[name] = img;
}
bool take(const std::string& name, float* out, int w, int h) {
    auto& t = stb_shim::table();
    auto it = t.find(name);
    if (it == t.end() || it->second.w != w || it->second.h != h) return false;
    std::copy(it->second.data.begin(), it->second.data.end(), out);
    return true;
}
}  // namespace

extern "C" {

#ifdef RPD_REF_ATROUS
// filter() of denoising/atrous_wavelet.cpp:151-218 on in-memory images.
int ref_atrous(const float* raw, const float* normal, const float* albedo, int w, int h, float sigma_c, float sigma_n,
               float sigma_a, int iterations, float* out) {
    put("raw", raw, w, h);
    put("normal", normal, w, h);
    put("albedo", albedo, w, h);
    if (!filter("raw", "normal", "albedo", sigma_c, sigma_n, sigma_a, iterations, std::filesystem::path("mem")))
        return 1;
    return take((std::filesystem::path("mem") / "atrous_wavelet.hdr").string(), out, w, h) ? 0 : 2;
}
#else
// filter() of denoising/joint_bilateral.cpp:15-170 on in-memory images.
int ref_joint_bilateral(const float* raw, const float* normal, const float* albedo, int w, int h, float sigma_c,
                        float sigma_n, float sigma_p, float sigma_a, float* gaussian, float* bilateral, float* joint) {
    put("raw", raw, w, h);
    put("normal", normal, w, h);
    put("albedo", albedo, w, h);
    if (!filter("raw", "normal", "albedo", sigma_c, sigma_n, sigma_p, sigma_a, std::filesystem::path("mem"))) return 1;
    const auto dir = std::filesystem::path("mem");
    return (take((dir / "gaussian.hdr").string(), gaussian, w, h) && take((dir / "bilateral.hdr").string(), bilateral, w, h) &&
            take((dir / "joint.hdr").string(), joint, w, h)) ? 0 : 2;
}
#endif

}  // extern "C"
