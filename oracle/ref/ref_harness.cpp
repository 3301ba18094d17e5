// Reference harness: the reference's own denoise-stage code, compiled from its sources
// (path_tracer/main.cpp and the headers it includes) against the shims in
// oracle/ref_shim, exposed through a small C interface for the tests.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product links or loads this file; it is built
// into oracle/_ref/ by oracle/Makefile when the reference sources are present, and it is
// used to (1) trace the reference's cornell_box scene and record each camera sample,
// (2) replay recorded samples through the reference's accumulate_sample /
// accumulate_rpf_sample_to_grid / merge_rpf_grids_into, and (3) run the reference's
// recompute_sensitivity, statmc_denoise, variance_denoise and
// compute_adaptive_sample_counts on the result. Its outputs pin the C restatement in
// oracle/rpd_oracle.c and the golden fixtures under tests/golden/.

#define main rpd_reference_cli_main
#include "main.cpp"
#undef main

#include <chrono>
#include <cstring>

#include "rpd_gb300.h"

namespace {

RenderConfig g_cfg{};
bool g_have_cfg = false;
std::vector<rpf::Grid> g_pass_grids;  // thread-local grids of the open pass
std::vector<int> g_last_counts;
double g_stage_ms[RPD_STAGE_COUNT_] = {0, 0, 0, 0, 0};

RenderConfig to_render_config(const rpd_config* c) {
    RenderConfig r{};
    r.image_width = c->image_width;
    r.image_height = c->image_height;
    r.samples_per_pixel = 1;
    r.fov = 45.0f;
    r.focus_distance = 1.0f;
    r.aperture = 0.0f;
    r.camera_position = Vec3f::Zero();
    r.camera_direction = Vec3f::UnitZ();
    r.camera_up = Vec3f::UnitY();
    r.use_statmc = true;
    r.rpf_tile_size = c->rpf_tile_size;
    r.rpf_shrinkage_scale = c->rpf_shrinkage_scale;
    r.rpf_confidence_samples = c->rpf_confidence_samples;
    r.color_window_radius = c->color_window_radius;
    r.color_normal_threshold = c->color_normal_threshold;
    r.color_depth_threshold = c->color_depth_threshold;
    r.color_compat_alpha = c->color_compat_alpha;
    r.color_sigma_max = c->color_sigma_max;
    r.var_window_radius = c->var_window_radius;
    r.var_normal_threshold = c->var_normal_threshold;
    r.var_depth_threshold = c->var_depth_threshold;
    r.var_compat_sigma = c->var_compat_sigma;
    r.var_shrinkage_k = c->var_shrinkage_k;
    r.var_iterations = c->var_iterations;
    r.adaptive_base_samples = c->adaptive_base_samples;
    r.adaptive_spp = c->adaptive_spp;
    r.adaptive_sigma_max = c->adaptive_sigma_max;
    r.adaptive_passes = c->adaptive_passes;
    r.adaptive_importance_smoothing_radius = c->adaptive_importance_smoothing_radius;
    r.debug_statmc_outputs = false;
    return r;
}

template <typename F>
double timed_ms(F&& f) {
    const auto t0 = std::chrono::steady_clock::now();
    f();
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void set_threads(int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
}

int max_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int thread_id() {
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

rpf::Sample decode_sample(const rpd_sample_soa* s, int64_t k) {
    rpf::Sample r{};
    const uint8_t f = s->flags ? s->flags[k] : 0;
    const uint8_t c = s->category ? s->category[k] : 0;
    if ((f & RPD_SAMPLE_PIXEL_VALID) && s->pixel_u[0]) r.capture_pixel(Vec2f(s->pixel_u[0][k], s->pixel_u[1][k]));
    if ((f & RPD_SAMPLE_LENS_VALID) && s->lens_u[0]) r.capture_lens(Vec2f(s->lens_u[0][k], s->lens_u[1][k]));
    if (f & RPD_SAMPLE_LIGHT_SELECT_VALID) r.capture_light_select(int(c & RPD_CATEGORY_LIGHT_INDEX_MASK), true);
    if ((f & RPD_SAMPLE_LIGHT_VALID) && s->light_u[0]) r.capture_light_uv(Vec2f(s->light_u[0][k], s->light_u[1][k]), true);
    if ((f & RPD_SAMPLE_ENV_VALID) && s->env_u[0]) r.capture_environment(Vec2f(s->env_u[0][k], s->env_u[1][k]));
    if ((f & RPD_SAMPLE_BRDF_VALID) && s->brdf_u[0]) r.capture_brdf(Vec2f(s->brdf_u[0][k], s->brdf_u[1][k]));
    if (f & RPD_SAMPLE_RR_VALID) r.capture_rr((c & RPD_CATEGORY_RR_SURVIVED) != 0);
    return r;
}

template <typename T>
int copy_out(void* dst, size_t bytes, const std::vector<T>& v) {
    if (bytes != v.size() * sizeof(T)) return RPD_ERR_INVALID_ARGUMENT;
    std::memcpy(dst, v.data(), bytes);
    return RPD_OK;
}

int copy_image(void* dst, size_t bytes, const Image& img) {
    if (bytes != img.pixels.size() * 3 * sizeof(float)) return RPD_ERR_INVALID_ARGUMENT;
    float* out = static_cast<float*>(dst);
    for (size_t i = 0; i < img.pixels.size(); ++i)
        for (int c = 0; c < 3; ++c) out[3 * i + c] = img.pixels[i][c];
    return RPD_OK;
}

}  // namespace

extern "C" {

int ref_max_threads(void) { return max_threads(); }

// Parse a reference YAML render config with the reference's own parse_render_config
// (path_tracer/core/config.h:51) and return the stage knobs. Returns 0 on success.
int ref_parse_yaml(const char* path, rpd_config* out, char* msg, size_t cap) {
    try {
        const RenderConfig r = parse_render_config(YAML::LoadFile(path));
        out->image_width = r.image_width;
        out->image_height = r.image_height;
        out->rpf_tile_size = r.rpf_tile_size;
        out->rpf_shrinkage_scale = r.rpf_shrinkage_scale;
        out->rpf_confidence_samples = r.rpf_confidence_samples;
        out->color_window_radius = r.color_window_radius;
        out->color_normal_threshold = r.color_normal_threshold;
        out->color_depth_threshold = r.color_depth_threshold;
        out->color_compat_alpha = r.color_compat_alpha;
        out->color_sigma_max = r.color_sigma_max;
        out->var_window_radius = r.var_window_radius;
        out->var_normal_threshold = r.var_normal_threshold;
        out->var_depth_threshold = r.var_depth_threshold;
        out->var_compat_sigma = r.var_compat_sigma;
        out->var_shrinkage_k = r.var_shrinkage_k;
        out->var_iterations = r.var_iterations;
        out->adaptive_base_samples = r.adaptive_base_samples;
        out->adaptive_spp = r.adaptive_spp;
        out->adaptive_sigma_max = r.adaptive_sigma_max;
        out->adaptive_passes = r.adaptive_passes;
        out->adaptive_importance_smoothing_radius = r.adaptive_importance_smoothing_radius;
        out->debug_statmc_outputs = r.debug_statmc_outputs ? 1 : 0;
        return 0;
    } catch (const std::exception& e) {
        if (msg && cap) {
            std::strncpy(msg, e.what(), cap - 1);
            msg[cap - 1] = 0;
        }
        return 1;
    }
}

// Trace the reference's cornell_box scene (camera from the YAML at `yaml_path`, size
// w x h) and record every camera sample in reference order, exactly as
// render_image_statmc (main.cpp:685-719) / render_image_adaptive (1488-1519) draw them:
// pixel idx is seeded with pixel_sample_seed(idx, start_n[idx]) and traced counts[idx]
// times (spp when counts is NULL). The primary-hit features mis_path_trace adds to
// FrameBuffers (main.cpp:572-576) are captured through a one-pixel scratch buffer.
// Returns the number of samples written, or -1 when capacity is too small.
int64_t ref_trace_cornell(const char* yaml_path, int32_t w, int32_t h, int32_t spp, uint32_t seed,
                          const int32_t* start_n, const int32_t* counts, rpd_sample_soa* out,
                          int64_t capacity) {
    RenderConfig rc = parse_render_config(YAML::LoadFile(yaml_path));
    rc.image_width = w;
    rc.image_height = h;
    scene = scenes::load_scene("cornell_box");
    bvh = BVH{};
    bvh.build_bvh(scene.triangles);
    Camera camera;
    camera.init(rc.camera_position, rc.camera_direction, rc.fov, float(w) / h, rc.focus_distance,
                rc.aperture, rc.camera_up);
    g_sampler_base_seed = seed;

    int64_t total = 0;
    for (int64_t i = 0; i < int64_t(w) * h; ++i) total += counts ? counts[i] : spp;
    if (total > capacity) return -1;

    FrameBuffers saved = std::move(buffers);
    buffers = FrameBuffers{};
    buffers.init(1, 1);
    float* o_rad[3] = {const_cast<float*>(out->radiance[0]), const_cast<float*>(out->radiance[1]), const_cast<float*>(out->radiance[2])};
    int64_t k = 0;
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            const int idx = y * w + x;
            Sampler::init_thread(pixel_sample_seed(idx, start_n ? start_n[idx] : 0));
            const int n = counts ? counts[idx] : spp;
            for (int s = 0; s < n; ++s, ++k) {
                const Vec2f pixel_u = Sampler::next2d();
                const float u = (x + pixel_u.x()) / float(w);
                const float v = (y + pixel_u.y()) / float(h);
                const Vec2f lens_u = Sampler::next2d();
                const Vec2f lens_sample = camera.lens_radius > 0.0f ? Sampler::sample_disk(lens_u) : Vec2f::Zero();
                rpf::Sample rs{};
                rs.capture_pixel(pixel_u);
                if (camera.lens_radius > 0.0f) rs.capture_lens(lens_u);
                buffers.hit_count[0] = 0;
                buffers.normal[0] = Vec3f::Zero();
                buffers.albedo[0] = Vec3f::Zero();
                buffers.world_pos[0] = Vec3f::Zero();
                buffers.depth[0] = 0.0f;
                Ray ray = camera.generate_ray(u, (1.0f - v), lens_sample);
                const Vec3f L = mis_path_trace(ray, 0, &rs);
                for (int c = 0; c < 3; ++c) o_rad[c][k] = L[c];
                const bool hit = buffers.hit_count[0] > 0;
                for (int c = 0; c < 3; ++c) {
                    const_cast<float*>(out->normal[c])[k] = buffers.normal[0][c];
                    const_cast<float*>(out->albedo[c])[k] = buffers.albedo[0][c];
                }
                const_cast<float*>(out->depth)[k] = buffers.depth[0];
                uint8_t f = hit ? RPD_SAMPLE_HIT : 0;
                uint8_t cat = 0;
                if (rs.pixel_valid) f |= RPD_SAMPLE_PIXEL_VALID;
                if (rs.lens_valid) f |= RPD_SAMPLE_LENS_VALID;
                if (rs.brdf_valid) f |= RPD_SAMPLE_BRDF_VALID;
                if (rs.light_valid) f |= RPD_SAMPLE_LIGHT_VALID;
                if (rs.light_select_valid) {
                    f |= RPD_SAMPLE_LIGHT_SELECT_VALID;
                    cat |= uint8_t(rs.light_index & RPD_CATEGORY_LIGHT_INDEX_MASK);
                }
                if (rs.environment_valid) f |= RPD_SAMPLE_ENV_VALID;
                if (rs.rr_valid) {
                    f |= RPD_SAMPLE_RR_VALID;
                    if (rs.rr_survived) cat |= RPD_CATEGORY_RR_SURVIVED;
                }
                const_cast<uint8_t*>(out->flags)[k] = f;
                const_cast<uint8_t*>(out->category)[k] = cat;
                const_cast<float*>(out->pixel_u[0])[k] = rs.pixel_u.x();
                const_cast<float*>(out->pixel_u[1])[k] = rs.pixel_u.y();
                const_cast<float*>(out->lens_u[0])[k] = rs.lens_u.x();
                const_cast<float*>(out->lens_u[1])[k] = rs.lens_u.y();
                const_cast<float*>(out->brdf_u[0])[k] = rs.brdf_u.x();
                const_cast<float*>(out->brdf_u[1])[k] = rs.brdf_u.y();
                const_cast<float*>(out->light_u[0])[k] = rs.light_u.x();
                const_cast<float*>(out->light_u[1])[k] = rs.light_u.y();
                const_cast<float*>(out->env_u[0])[k] = rs.environment_u.x();
                const_cast<float*>(out->env_u[1])[k] = rs.environment_u.y();
            }
        }
    }
    buffers = std::move(saved);
    return k;
}

// render_image_statmc's set-up (main.cpp:650-655) for a frame of the given config.
int ref_begin_frame(const rpd_config* c) {
    g_cfg = to_render_config(c);
    g_have_cfg = true;
    g_sampler_base_seed = c->seed;
    buffers = FrameBuffers{};
    buffers.init(g_cfg.image_width, g_cfg.image_height);
    pixel_stats.assign(g_cfg.image_width * g_cfg.image_height, PixelStats{});
    rpf_grid.init(g_cfg.image_width, g_cfg.image_height, g_cfg.rpf_tile_size);
    rpf_grid.reset();
    invalidate_postprocess_caches();
    g_pass_grids.clear();
    g_last_counts.clear();
    return 0;
}

// Replace the stage knobs of later calls (image size and tile size stay).
int ref_set_config(const rpd_config* c) {
    const int w = g_cfg.image_width, h = g_cfg.image_height, t = g_cfg.rpf_tile_size;
    g_cfg = to_render_config(c);
    g_cfg.image_width = w;
    g_cfg.image_height = h;
    g_cfg.rpf_tile_size = t;
    g_sampler_base_seed = c->seed;
    return 0;
}

// Replay recorded samples for pixels [first, first+count) through the reference's own
// per-sample hooks, in the same OpenMP row loop with thread-local grids as
// render_image_statmc (main.cpp:664-719). threads = 1 gives a fixed summation order.
int ref_push_samples(const rpd_sample_soa* s, int64_t first, int64_t count, int32_t spp,
                     const int32_t* counts, int threads) {
    if (!g_have_cfg) return RPD_ERR_STATE;
    set_threads(threads);
    const int w = g_cfg.image_width;
    const bool capture_rpd = g_cfg.rpf_shrinkage_scale > 0.0f;
    const int nthreads = max_threads();
    if (capture_rpd && g_pass_grids.size() != size_t(nthreads)) {
        g_pass_grids.assign(nthreads, rpf::Grid{});
        for (auto& g : g_pass_grids) {
            g.init(g_cfg.image_width, g_cfg.image_height, g_cfg.rpf_tile_size);
            g.reset();
        }
    }
    std::vector<int64_t> offset(count + 1, 0);
    for (int64_t i = 0; i < count; ++i) offset[i + 1] = offset[i] + (counts ? counts[i] : spp);
    const int64_t row_first = first / w;
    const int64_t row_last = (first + count - 1) / w;
    const double ms = timed_ms([&] {
#ifdef _OPENMP
#pragma omp parallel
        {
            const int gi = thread_id();
#pragma omp for schedule(dynamic, 1)
#else
        const int gi = 0;
#endif
        for (int64_t row = row_first; row <= row_last; ++row) {
            const int y = int(row);
            for (int x = 0; x < w; ++x) {
                const int64_t idx = int64_t(y) * w + x;
                if (idx < first || idx >= first + count) continue;
                const int64_t local = idx - first;
                for (int64_t k = offset[local]; k < offset[local + 1]; ++k) {
                    const uint8_t f = s->flags ? s->flags[k] : 0;
                    if (f & RPD_SAMPLE_HIT) {
                        const Vec3f n(s->normal[0][k], s->normal[1][k], s->normal[2][k]);
                        const Vec3f a = s->albedo[0]
                            ? Vec3f(s->albedo[0][k], s->albedo[1][k], s->albedo[2][k])
                            : Vec3f(s->pixel_albedo[0][local], s->pixel_albedo[1][local], s->pixel_albedo[2][local]);
                        buffers.hit_count[idx]++;
                        buffers.normal[idx] += n;
                        buffers.albedo[idx] += a;
                        buffers.depth[idx] += s->depth[k];
                    }
                    const Vec3f L(s->radiance[0][k], s->radiance[1][k], s->radiance[2][k]);
                    if (!L.allFinite()) continue;
                    if (capture_rpd) {
                        accumulate_rpf_sample_to_grid(g_pass_grids[gi], x, y, decode_sample(s, k), calc_luminance(L));
                    }
                    accumulate_sample(pixel_stats[idx], L);
                    buffers.radiance(x, y) += L;
                    buffers.sample_count[idx]++;
                }
            }
        }
#ifdef _OPENMP
        }
#endif
    });
    g_stage_ms[RPD_STAGE_ACCUMULATE] = ms;
    return 0;
}

// End of a render pass: merge_rpf_grids_into (main.cpp:730 / 1531) and the cache
// invalidation of render_image_adaptive (main.cpp:1533).
int ref_end_pass(int threads) {
    set_threads(threads);
    if (!g_pass_grids.empty()) {
        g_stage_ms[RPD_STAGE_ACCUMULATE] += timed_ms([&] { merge_rpf_grids_into(rpf_grid, g_pass_grids); });
        g_pass_grids.clear();
    }
    invalidate_postprocess_caches();
    return 0;
}

int ref_recompute_sensitivity(int threads) {
    set_threads(threads);
    g_stage_ms[RPD_STAGE_SENSITIVITY] = timed_ms([&] { recompute_sensitivity(g_cfg); });
    return 0;
}

int ref_statmc_denoise(int threads) {
    set_threads(threads);
    g_stage_ms[RPD_STAGE_STATMC] = timed_ms([&] { statmc_denoise(g_cfg); });
    return 0;
}

int ref_variance_denoise(int threads) {
    set_threads(threads);
    g_stage_ms[RPD_STAGE_VARIANCE] = timed_ms([&] { variance_denoise(g_cfg); });
    return 0;
}

int ref_compute_adaptive_sample_counts(int32_t* out, int threads) {
    set_threads(threads);
    g_stage_ms[RPD_STAGE_ADAPTIVE] = timed_ms([&] { g_last_counts = compute_adaptive_sample_counts(g_cfg); });
    if (out) std::memcpy(out, g_last_counts.data(), g_last_counts.size() * sizeof(int32_t));
    return 0;
}

int ref_finalize(int threads) {
    set_threads(threads);
    buffers.finalize();
    return 0;
}

double ref_stage_ms(int stage) {
    return (stage >= 0 && stage < RPD_STAGE_COUNT_) ? g_stage_ms[stage] : -1.0;
}

int ref_nodes(int32_t* nx, int32_t* ny) {
    *nx = rpf_grid.nodes_x;
    *ny = rpf_grid.nodes_y;
    return 0;
}

int ref_read(int field, void* dst, size_t bytes) {
    const auto& t = buffers.sensitivity_tiles;
    const int w = g_cfg.image_width, h = g_cfg.image_height;
    const size_t np = size_t(w) * h;
    switch (field) {
    case RPD_FIELD_DENOISED: return copy_image(dst, bytes, buffers.denoised);
    case RPD_FIELD_UNCERTAINTY: return copy_out(dst, bytes, buffers.uncertainty);
    case RPD_FIELD_ALPHA: return copy_out(dst, bytes, buffers.alpha);
    case RPD_FIELD_VAR_TOTAL_DEBUG: return copy_out(dst, bytes, buffers.var_total_debug);
    case RPD_FIELD_VAR_EFF_DEBUG: return copy_out(dst, bytes, buffers.var_eff_debug);
    case RPD_FIELD_VAR_RATIO_DEBUG: return copy_out(dst, bytes, buffers.var_ratio_debug);
    case RPD_FIELD_VARIANCE_DENOISED: return copy_out(dst, bytes, buffers.variance_denoised);
    case RPD_FIELD_ADAPTIVE_IMPORTANCE: return copy_out(dst, bytes, buffers.adaptive_importance);
    case RPD_FIELD_SENSITIVITY_CONFIDENCE: return copy_out(dst, bytes, buffers.sensitivity_confidence);
    case RPD_FIELD_SENSITIVITY_GRADIENT: return copy_out(dst, bytes, buffers.sensitivity_gradient);
    case RPD_FIELD_HIT_COUNT: return copy_out(dst, bytes, buffers.hit_count);
    case RPD_FIELD_SAMPLE_COUNT: return copy_out(dst, bytes, buffers.sample_count);
    case RPD_FIELD_RADIANCE_SUM: return copy_image(dst, bytes, buffers.radiance);
    case RPD_FIELD_NORMAL_SUM: return copy_image(dst, bytes, buffers.normal);
    case RPD_FIELD_ALBEDO_SUM: return copy_image(dst, bytes, buffers.albedo);
    case RPD_FIELD_DEPTH_SUM: return copy_out(dst, bytes, buffers.depth);
    case RPD_FIELD_STATS_MEAN:
    case RPD_FIELD_STATS_SQUARE_DIFF:
    case RPD_FIELD_STATS_N: {
        if (bytes != np * 4) return RPD_ERR_INVALID_ARGUMENT;
        for (size_t i = 0; i < np; ++i) {
            if (field == RPD_FIELD_STATS_N) static_cast<int32_t*>(dst)[i] = pixel_stats[i].n;
            else static_cast<float*>(dst)[i] = field == RPD_FIELD_STATS_MEAN ? pixel_stats[i].mean : pixel_stats[i].square_diff;
        }
        return RPD_OK;
    }
    case RPD_FIELD_STATS_COLOR_MEAN:
    case RPD_FIELD_STATS_SQRT_MEAN:
    case RPD_FIELD_STATS_SQRT_SQUARE_DIFF: {
        if (bytes != np * 12) return RPD_ERR_INVALID_ARGUMENT;
        float* o = static_cast<float*>(dst);
        for (size_t i = 0; i < np; ++i) {
            const Vec3f& v = field == RPD_FIELD_STATS_COLOR_MEAN ? pixel_stats[i].color_mean
                : field == RPD_FIELD_STATS_SQRT_MEAN ? pixel_stats[i].sqrt_color_mean
                : pixel_stats[i].sqrt_color_square_diff;
            for (int c = 0; c < 3; ++c) o[3 * i + c] = v[c];
        }
        return RPD_OK;
    }
    case RPD_FIELD_NODE_ALL: return copy_out(dst, bytes, t.all);
    case RPD_FIELD_NODE_ALL_CONF: return copy_out(dst, bytes, t.all_conf);
    case RPD_FIELD_NODE_PIXEL: return copy_out(dst, bytes, t.pixel);
    case RPD_FIELD_NODE_PIXEL_CONF: return copy_out(dst, bytes, t.pixel_conf);
    case RPD_FIELD_NODE_BRDF: return copy_out(dst, bytes, t.brdf);
    case RPD_FIELD_NODE_BRDF_CONF: return copy_out(dst, bytes, t.brdf_conf);
    case RPD_FIELD_NODE_LENS: return copy_out(dst, bytes, t.lens);
    case RPD_FIELD_NODE_LENS_CONF: return copy_out(dst, bytes, t.lens_conf);
    case RPD_FIELD_NODE_LIGHT: return copy_out(dst, bytes, t.light);
    case RPD_FIELD_NODE_LIGHT_CONF: return copy_out(dst, bytes, t.light_conf);
    case RPD_FIELD_NODE_LIGHT_UV: return copy_out(dst, bytes, t.light_uv);
    case RPD_FIELD_NODE_LIGHT_UV_CONF: return copy_out(dst, bytes, t.light_uv_conf);
    case RPD_FIELD_NODE_LIGHT_SELECT: return copy_out(dst, bytes, t.light_select);
    case RPD_FIELD_NODE_LIGHT_SELECT_CONF: return copy_out(dst, bytes, t.light_select_conf);
    case RPD_FIELD_NODE_ENVIRONMENT: return copy_out(dst, bytes, t.environment);
    case RPD_FIELD_NODE_ENVIRONMENT_CONF: return copy_out(dst, bytes, t.environment_conf);
    case RPD_FIELD_NODE_RR: return copy_out(dst, bytes, t.rr);
    case RPD_FIELD_NODE_RR_CONF: return copy_out(dst, bytes, t.rr_conf);
    case RPD_FIELD_GRID: {
        const size_t nodes = rpf_grid.nodes.size();
        if (bytes != nodes * RPD_GRID_DEPENDENCIES * RPD_GRID_DEP_STRIDE * sizeof(double)) return RPD_ERR_INVALID_ARGUMENT;
        double* o = static_cast<double*>(dst);
        std::memset(o, 0, bytes);
        for (size_t n = 0; n < nodes; ++n) {
            const rpf::Tile& tile = rpf_grid.nodes[n];
            double* base = o + n * RPD_GRID_DEPENDENCIES * RPD_GRID_DEP_STRIDE;
            auto put = [&](int dep, const auto& b) {
                double* d = base + dep * RPD_GRID_DEP_STRIDE;
                const int bins = int(b.weight.size());
                for (int i = 0; i < bins; ++i) {
                    d[i] = b.weight[i];
                    d[16 + i] = b.sum_y[i];
                }
                d[32] = b.w_sum;
                d[33] = b.w2_sum;
                d[34] = b.y_sum;
                d[35] = b.y2_sum;
            };
            put(0, tile.pixel.nonlinear);
            put(1, tile.brdf.nonlinear);
            put(2, tile.screen_brdf.nonlinear);
            put(3, tile.lens.nonlinear);
            put(4, tile.screen_lens.nonlinear);
            put(5, tile.light_uv.nonlinear);
            put(6, tile.screen_light_uv.nonlinear);
            put(7, tile.environment.nonlinear);
            put(8, tile.screen_environment.nonlinear);
            put(9, tile.light_select);
            put(10, tile.screen_light_select.nonlinear);
            put(11, tile.rr);
            put(12, tile.screen_rr.nonlinear);
        }
        return RPD_OK;
    }
    case RPD_FIELD_EXPANDED_ALL: return copy_out(dst, bytes, t.expand_values(t.all, w, h));
    case RPD_FIELD_EXPANDED_PIXEL: return copy_out(dst, bytes, t.expand_values(t.pixel, w, h));
    case RPD_FIELD_EXPANDED_BRDF: return copy_out(dst, bytes, t.expand_values(t.brdf, w, h));
    case RPD_FIELD_EXPANDED_LENS: return copy_out(dst, bytes, t.expand_values(t.lens, w, h));
    case RPD_FIELD_EXPANDED_LIGHT: return copy_out(dst, bytes, t.expand_values(t.light, w, h));
    case RPD_FIELD_EXPANDED_LIGHT_UV: return copy_out(dst, bytes, t.expand_values(t.light_uv, w, h));
    case RPD_FIELD_EXPANDED_LIGHT_SELECT: return copy_out(dst, bytes, t.expand_values(t.light_select, w, h));
    case RPD_FIELD_EXPANDED_ENVIRONMENT: return copy_out(dst, bytes, t.expand_values(t.environment, w, h));
    case RPD_FIELD_EXPANDED_RR: return copy_out(dst, bytes, t.expand_values(t.rr, w, h));
    case RPD_FIELD_ADAPTIVE_COUNTS: return copy_out(dst, bytes, g_last_counts);
    default: return RPD_ERR_INVALID_ARGUMENT;
    }
}

// The reference's own full StatMC render of cornell_box (render(), main.cpp:1543-1564),
// used to check that trace + replay + stages reproduce it. Fields are then readable
// with ref_read (note render() ends with finalize and the radiance/denoised swap).
int ref_render_cornell(const char* yaml_path, const rpd_config* c, int32_t spp, int threads) {
    set_threads(threads);
    RenderConfig rc = parse_render_config(YAML::LoadFile(yaml_path));
    const RenderConfig knobs = to_render_config(c);
    rc.image_width = c->image_width;
    rc.image_height = c->image_height;
    rc.samples_per_pixel = spp;
    rc.use_statmc = true;
    rc.rpf_tile_size = knobs.rpf_tile_size;
    rc.rpf_shrinkage_scale = knobs.rpf_shrinkage_scale;
    rc.rpf_confidence_samples = knobs.rpf_confidence_samples;
    rc.color_window_radius = knobs.color_window_radius;
    rc.color_normal_threshold = knobs.color_normal_threshold;
    rc.color_depth_threshold = knobs.color_depth_threshold;
    rc.color_compat_alpha = knobs.color_compat_alpha;
    rc.color_sigma_max = knobs.color_sigma_max;
    rc.var_window_radius = knobs.var_window_radius;
    rc.var_normal_threshold = knobs.var_normal_threshold;
    rc.var_depth_threshold = knobs.var_depth_threshold;
    rc.var_compat_sigma = knobs.var_compat_sigma;
    rc.var_shrinkage_k = knobs.var_shrinkage_k;
    rc.var_iterations = knobs.var_iterations;
    rc.adaptive_base_samples = knobs.adaptive_base_samples;
    rc.adaptive_spp = knobs.adaptive_spp;
    rc.adaptive_sigma_max = knobs.adaptive_sigma_max;
    rc.adaptive_passes = knobs.adaptive_passes;
    rc.adaptive_importance_smoothing_radius = knobs.adaptive_importance_smoothing_radius;
    scene = scenes::load_scene("cornell_box");
    bvh = BVH{};
    bvh.build_bvh(scene.triangles);
    Camera camera;
    camera.init(rc.camera_position, rc.camera_direction, rc.fov, float(rc.image_width) / rc.image_height,
                rc.focus_distance, rc.aperture, rc.camera_up);
    g_sampler_base_seed = c->seed;
    g_cfg = rc;
    g_have_cfg = true;
    render(rc, camera);
    return 0;
}

// render()'s last step (main.cpp:1557-1559: the finalized radiance becomes raw_radiance, the
// denoised image the radiance; with `swap`) and output_buffers (core/buffers.h:197-250) with
// this prefix and tonemapping preset: every image the reference writes is captured by the stb
// shim.
int ref_output_buffers(const char* prefix, int tonemap, int swap) {
    stb_shim::table().clear();
    stb_shim::png_table().clear();
    if (swap) {
        buffers.raw_radiance = buffers.radiance;
        buffers.radiance = buffers.denoised;
    }
    return output_buffers(buffers, prefix, static_cast<Image::ToneMapping>(tonemap), true) ? 0 : 1;
}

// Image::save_with_tonemapping (shared/image.h:129-139) of n RGB values as one row; out gets
// the 3 n bytes it writes.
int ref_tonemap(const float* rgb, int n, int tonemap, unsigned char* out) {
    Image img(n, 1);
    for (int i = 0; i < n; ++i) img[i] = Vec3f(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
    stb_shim::png_table().clear();
    if (!img.save_with_tonemapping("tonemap.png", static_cast<Image::ToneMapping>(tonemap))) return 1;
    const auto& png = stb_shim::png_table()["tonemap.png"];
    std::memcpy(out, png.data.data(), png.data.size());
    return 0;
}

// Names of the captured images, '\n'-separated: HDR writes first, then "png:" + each PNG write.
int ref_output_names(char* buf, size_t cap) {
    std::string all;
    for (const auto& kv : stb_shim::table()) all += kv.first + "\n";
    for (const auto& kv : stb_shim::png_table()) all += "png:" + kv.first + "\n";
    if (all.size() + 1 > cap) return -1;
    std::memcpy(buf, all.c_str(), all.size() + 1);
    return int(all.size());
}

// One captured image: HDR floats (comp per pixel) or PNG bytes; w, h, comp out.
int ref_output_image(const char* name, int png, void* dst, size_t cap, int32_t* w, int32_t* h, int32_t* comp) {
    if (png) {
        auto it = stb_shim::png_table().find(name);
        if (it == stb_shim::png_table().end() || it->second.data.size() > cap) return 1;
        std::memcpy(dst, it->second.data.data(), it->second.data.size());
        *w = it->second.w, *h = it->second.h, *comp = it->second.comp;
        return 0;
    }
    auto it = stb_shim::table().find(name);
    if (it == stb_shim::table().end() || it->second.data.size() * sizeof(float) > cap) return 1;
    std::memcpy(dst, it->second.data.data(), it->second.data.size() * sizeof(float));
    *w = it->second.w, *h = it->second.h, *comp = it->second.comp;
    return 0;
}

}  // extern "C"
