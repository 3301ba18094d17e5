// rpd_statmc.hpp — header-only C++ layer over the C ABI of rpd_gb300.h.
//
// The reference runs the denoise stage as free functions over process globals
// (path_tracer/main.cpp):
//
//     void recompute_sensitivity(const RenderConfig&);                 // main.cpp:741
//     void statmc_denoise(const RenderConfig&);                        // main.cpp:957
//     void variance_denoise(const RenderConfig&);                      // main.cpp:1166
//     std::vector<int> compute_adaptive_sample_counts(const RenderConfig&);  // main.cpp:1273
//
// This header gives the same four names over a "current job" (one per host thread), so a
// clone of render() (main.cpp:1543-1564) links against the GPU stage unchanged: it sets the
// current job once, pushes each pass's samples where the reference accumulated them, and
// calls the four functions as before. The configuration type is a template parameter read by
// field name, so the reference's own RenderConfig (path_tracer/core/config.h:15-49) works as
// is. Errors, which the reference never reports (its functions return void), throw
// rpd::Error with the library's message.
//
// The RAII wrappers Context and Job own an rpd_ctx / rpd_job.
#ifndef RPD_STATMC_HPP
#define RPD_STATMC_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "rpd_gb300.h"

namespace rpd {

struct Error : std::runtime_error {
    int status;
    Error(int st, const std::string& msg) : std::runtime_error(msg), status(st) {}
};

inline void check(int status) {
    if (status != RPD_OK) {
        const char* m = rpd_last_error();
        throw Error(status, std::string(rpd_status_string(status)) + ": " + (m ? m : ""));
    }
}

// The stage knobs of a RenderConfig-like object (core/config.h:27-48), plus the sampler seed
// the adaptive allocation hashes (g_sampler_base_seed, main.cpp:43,1427).
template <class Config>
rpd_config to_rpd_config(const Config& c, uint32_t seed) {
    rpd_config r;
    rpd_config_defaults(&r);
    r.image_width = c.image_width;
    r.image_height = c.image_height;
    r.rpf_tile_size = c.rpf_tile_size;
    r.rpf_shrinkage_scale = c.rpf_shrinkage_scale;
    r.rpf_confidence_samples = c.rpf_confidence_samples;
    r.color_window_radius = c.color_window_radius;
    r.color_normal_threshold = c.color_normal_threshold;
    r.color_depth_threshold = c.color_depth_threshold;
    r.color_compat_alpha = c.color_compat_alpha;
    r.color_sigma_max = c.color_sigma_max;
    r.var_window_radius = c.var_window_radius;
    r.var_normal_threshold = c.var_normal_threshold;
    r.var_depth_threshold = c.var_depth_threshold;
    r.var_compat_sigma = c.var_compat_sigma;
    r.var_shrinkage_k = c.var_shrinkage_k;
    r.var_iterations = c.var_iterations;
    r.adaptive_base_samples = c.adaptive_base_samples;
    r.adaptive_spp = c.adaptive_spp;
    r.adaptive_sigma_max = c.adaptive_sigma_max;
    r.adaptive_passes = c.adaptive_passes;
    r.adaptive_importance_smoothing_radius = c.adaptive_importance_smoothing_radius;
    r.debug_statmc_outputs = c.debug_statmc_outputs ? 1 : 0;
    r.seed = seed;
    return r;
}

class Context {
public:
    explicit Context(int device = 0, uint64_t hbm_budget_bytes = 0) {
        check(rpd_ctx_create(device, hbm_budget_bytes, &ctx_));
    }
    ~Context() { if (ctx_) rpd_ctx_destroy(ctx_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    rpd_ctx* get() const { return ctx_; }

private:
    rpd_ctx* ctx_ = nullptr;
};

class Job {
public:
    Job(Context& ctx, const rpd_config& cfg) : cfg_(cfg) { check(rpd_job_create(ctx.get(), &cfg_, &job_)); }
    ~Job() { if (job_) rpd_job_destroy(job_); }
    Job(const Job&) = delete;
    Job& operator=(const Job&) = delete;
    rpd_job* get() const { return job_; }
    const rpd_config& config() const { return cfg_; }

    // Re-read the knobs (only when they changed: the reference re-reads its config per call).
    void apply(const rpd_config& cfg) {
        const unsigned char* a = reinterpret_cast<const unsigned char*>(&cfg);
        const unsigned char* b = reinterpret_cast<const unsigned char*>(&cfg_);
        for (size_t i = 0; i < sizeof(rpd_config); ++i)
            if (a[i] != b[i]) {
                check(rpd_job_set_config(job_, &cfg));
                cfg_ = cfg;
                return;
            }
    }
    void begin_frame() { check(rpd_job_begin_frame(job_)); }
    // One pass's samples for pixels [first, first + count): `spp` each, or counts[i] each.
    void push(const rpd_sample_soa& s, int64_t first, int64_t count, int32_t spp, const int32_t* counts = nullptr,
              rpd_memory where = RPD_MEM_HOST) {
        check(rpd_job_push_samples(job_, &s, first, count, spp, counts, where));
    }
    void end_pass() { check(rpd_job_end_pass(job_)); }
    void finalize() { check(rpd_finalize(job_)); }
    template <class T>
    std::vector<T> read(rpd_field field) {
        std::vector<T> out(rpd_field_bytes(job_, field) / sizeof(T));
        check(rpd_job_read(job_, field, out.data(), out.size() * sizeof(T), RPD_MEM_HOST));
        return out;
    }

private:
    rpd_config cfg_;
    rpd_job* job_ = nullptr;
};

// The job the free functions below act on, per host thread (the reference's globals).
inline Job*& current_job() {
    static thread_local Job* job = nullptr;
    return job;
}
inline void set_current_job(Job* job) { current_job() = job; }
// The sampler seed the free functions pass on (the reference sets g_sampler_base_seed from
// its command line, main.cpp:1875).
inline uint32_t& current_seed() {
    static thread_local uint32_t seed = 0;
    return seed;
}

namespace detail {
template <class Config>
Job& job_for(const Config& config) {
    Job* j = current_job();
    if (!j) throw Error(RPD_ERR_STATE, "no current rpd job: call rpd::set_current_job first");
    j->apply(to_rpd_config(config, current_seed()));
    return *j;
}
}  // namespace detail

// main.cpp:741
template <class Config>
void recompute_sensitivity(const Config& config) {
    check(rpd_recompute_sensitivity(detail::job_for(config).get()));
}

// main.cpp:957
template <class Config>
void statmc_denoise(const Config& config) {
    check(rpd_statmc_denoise(detail::job_for(config).get()));
}

// main.cpp:1166
template <class Config>
void variance_denoise(const Config& config) {
    check(rpd_variance_denoise(detail::job_for(config).get()));
}

// main.cpp:1273: the extra samples per pixel, row-major W*H.
template <class Config>
std::vector<int> compute_adaptive_sample_counts(const Config& config) {
    Job& j = detail::job_for(config);
    std::vector<int> counts(size_t(j.config().image_width) * size_t(j.config().image_height));
    check(rpd_compute_adaptive_sample_counts(j.get(), counts.data(), RPD_MEM_HOST));
    return counts;
}

}  // namespace rpd

#endif  // RPD_STATMC_HPP
