// A clone of the reference's render() StatMC sequence (path_tracer/main.cpp:1543-1564) written
// against include/rpd_statmc.hpp: the four stage functions keep their reference names and
// signatures, and the render loops (render_image_statmc, 649-737; render_image_adaptive,
// 1451-1538) trace on host threads — here the seeded synthetic generator stands in for
// mis_path_trace — and hand each sample's record to an emitter, which streams the rows to the
// GPU band by band while the threads go on; the adaptive passes trace the counts the GPU
// computed.
//
//   render_clone W H SPP PASSES [OUT]   -> prints the mean denoised value and the adaptive total;
//                                        OUT gets each pass's counts (W*H int32 per pass) and
//                                        the denoised image (W*H*3 float)
#include <atomic>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "rpd_statmc.hpp"
#include "rpd_synth.h"

// The RenderConfig fields the stage reads, named as in path_tracer/core/config.h:15-49.
struct RenderConfig {
    int image_width = 64, image_height = 48;
    int rpf_tile_size = 16, color_window_radius = 5;
    float color_normal_threshold = 0.6f, color_depth_threshold = 0.2f, color_compat_alpha = 0.01f;
    float color_sigma_max = 4.0f;
    int var_window_radius = 3;
    float var_normal_threshold = 0.6f, var_depth_threshold = 0.25f, var_compat_sigma = 3.0f, var_shrinkage_k = 0.7f;
    int var_iterations = 2, adaptive_base_samples = 1, adaptive_spp = 4;
    float adaptive_sigma_max = 4.0f;
    int adaptive_passes = 2, adaptive_importance_smoothing_radius = 1;
    float rpf_shrinkage_scale = 1.0f, rpf_confidence_samples = 128.0f;
    bool debug_statmc_outputs = false;
};

// The render loop of one pass: `threads` host threads take rows in increasing order (OpenMP's
// dynamic schedule over rows, main.cpp:678-681 and 1488-1490) and trace each row's samples into
// the emitter's row planes; counts: the adaptive pass's per-pixel counts, or null for spp each.
void trace_pass(rpd_ctx* ctx, rpd_emitter* em, const rpd_synth_params& prm, int w, int h, int spp,
                const int32_t* counts, const int32_t* start_n, int threads) {
    rpd::check(rpd_emitter_begin_pass(em, spp, counts));
    std::atomic<int> next_row{0};
    std::atomic<int> status{RPD_OK};
    auto worker = [&]() {
        for (int y = next_row++; y < h && status == RPD_OK; y = next_row++) {
            rpd_sample_soa row{};
            const int64_t* offsets = nullptr;
            int st = rpd_emitter_row(em, y, &row, &offsets);
            const int64_t p0 = int64_t(y) * w;
            if (st == RPD_OK)
                st = rpd_synth_fill(ctx, &prm, p0, w, spp, counts ? counts + p0 : nullptr, start_n ? start_n + p0 : nullptr,
                                    &row, RPD_MEM_HOST);
            if (st == RPD_OK) st = rpd_emitter_row_done(em, y);
            if (st != RPD_OK) status = st;
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    rpd::check(status.load());
    rpd::check(rpd_emitter_end_pass(em));
}

int main(int argc, char** argv) {
    RenderConfig config;
    int spp = 4;
    if (argc > 3) {
        config.image_width = std::atoi(argv[1]);
        config.image_height = std::atoi(argv[2]);
        spp = std::atoi(argv[3]);
    }
    if (argc > 4) config.adaptive_passes = std::atoi(argv[4]);
    const char* out_path = argc > 5 ? argv[5] : nullptr;
    std::vector<int32_t> all_counts;
    const int w = config.image_width, h = config.image_height;
    const int64_t np = int64_t(w) * h;
    try {
        rpd::Context ctx(0, 0);
        rpd::current_seed() = 1234;
        rpd::Job job(ctx, rpd::to_rpd_config(config, rpd::current_seed()));
        rpd::set_current_job(&job);
        rpd_synth_params prm;
        rpd_synth_defaults(&prm, w, h, 1234);

        // render_image_statmc (main.cpp:649-737): the first pass, traced on 4 host threads
        rpd_emitter* em = nullptr;
        rpd::check(rpd_emitter_create(job.get(), 8, 3, std::max(spp, 8 * config.adaptive_spp), &em));
        job.begin_frame();
        trace_pass(ctx.get(), em, prm, w, h, spp, nullptr, nullptr, 4);
        rpd::recompute_sensitivity(config);
        std::vector<int32_t> n_so_far(size_t(np), spp);
        int64_t adaptive_total = 0;
        for (int i = 0; i < config.adaptive_passes && config.adaptive_spp > 0; ++i) {  // main.cpp:1547-1552
            rpd::statmc_denoise(config);
            rpd::variance_denoise(config);
            std::vector<int> counts = rpd::compute_adaptive_sample_counts(config);
            all_counts.insert(all_counts.end(), counts.begin(), counts.end());
            for (int c : counts) adaptive_total += c;
            // render_image_adaptive (main.cpp:1451-1538): the extra samples the GPU asked for
            trace_pass(ctx.get(), em, prm, w, h, 0, counts.data(), n_so_far.data(), 4);
            for (int64_t p = 0; p < np; ++p) n_so_far[size_t(p)] += counts[size_t(p)];
            rpd::recompute_sensitivity(config);
        }
        rpd_emitter_destroy(em);
        rpd::recompute_sensitivity(config);
        rpd::statmc_denoise(config);
        rpd::variance_denoise(config);
        job.finalize();
        const std::vector<float> den = job.read<float>(RPD_FIELD_DENOISED);
        double mean = 0.0;
        for (float v : den) mean += v;
        mean /= double(den.size());
        std::printf("denoised_mean %.9g adaptive_total %lld\n", mean, (long long)adaptive_total);
        if (out_path) {
            std::FILE* fo = std::fopen(out_path, "wb");
            if (!fo) return 2;
            const bool ok = std::fwrite(all_counts.data(), sizeof(int32_t), all_counts.size(), fo) == all_counts.size() &&
                            std::fwrite(den.data(), sizeof(float), den.size(), fo) == den.size();
            std::fclose(fo);
            if (!ok) return 2;
        }
        rpd::set_current_job(nullptr);
    } catch (const rpd::Error& e) {
        std::fprintf(stderr, "rpd error %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}
