/*
 * rpd_oracle.h — CPU restatement of the reference's StatMC / RPD denoise stage.
 *
 * TEST INFRASTRUCTURE ONLY. Only the tests, the smoke check and the CPU-baseline leg of
 * bench.py load this library; the product never does. It restates, in plain C with
 * OpenMP, the algorithm of path_tracer/main.cpp:94-185, 188-231, 266-281, 292-388 and
 * 741-1446, path_tracer/core/stats.h:25-141 and 161-329, path_tracer/core/buffers.h:68-101
 * and 152-167, following the reference's IEEE operation order (see oracle/rpd_oracle.c).
 * Its entry points mirror include/rpd_gb300.h one for one, on host memory.
 *
 * Parity pin: on x86-64 it is checked bit for bit against the reference's own sources
 * compiled in oracle/_ref (tests/test_oracle_vs_reference.py) and against the golden
 * vectors under tests/golden/ (produced by the compiled reference).
 */
#ifndef RPD_ORACLE_H
#define RPD_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "rpd_gb300.h"
#include "rpd_synth.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_job orc_job;

void orc_config_defaults(rpd_config* cfg);
int orc_config_validate(const rpd_config* cfg, char* msg, size_t cap);

orc_job* orc_job_create(const rpd_config* cfg);
void orc_job_destroy(orc_job* job);
/* OpenMP threads used by later calls (0 = all). The grid accumulation uses static row
 * blocks per thread and merges thread grids in thread order, so results depend only on
 * the thread count; 1 thread reproduces the reference's single-thread order. */
void orc_set_threads(orc_job* job, int threads);
int orc_job_set_config(orc_job* job, const rpd_config* cfg);
int orc_job_begin_frame(orc_job* job);
int orc_job_push_samples(orc_job* job, const rpd_sample_soa* s, int64_t first_pixel,
                         int64_t pixel_count, int32_t spp, const int32_t* counts);
int orc_job_end_pass(orc_job* job);
int orc_recompute_sensitivity(orc_job* job);
int orc_statmc_denoise(orc_job* job);
int orc_variance_denoise(orc_job* job);
/* compute_adaptive_sample_counts' allocation (main.cpp:1372-1438) on a final importance map:
 * counts holds the floor per pixel on entry; sum_importance is the in-order double sum. */
void orc_allocate_counts(const float* importance, int64_t np, const rpd_config* cfg, double sum_importance,
                         int32_t* counts);
/* The same from the map alone: counts is set to the floor, the sum taken in pixel order. */
void orc_allocate_counts_map(const float* importance, int64_t np, const rpd_config* cfg, int32_t* counts);
int orc_compute_adaptive_sample_counts(orc_job* job, int32_t* counts_out);
int orc_finalize(orc_job* job);
int orc_job_read(orc_job* job, int field, void* dst, size_t bytes);
uint64_t orc_field_bytes(const orc_job* job, int field);
double orc_stage_ms(const orc_job* job, int stage);
int orc_nodes(const orc_job* job, int32_t* nodes_x, int32_t* nodes_y);

/* Standalone filters (denoising/atrous_wavelet.cpp:54-197, denoising/joint_bilateral.cpp:15-132). */
int orc_atrous_wavelet(const float* raw, const float* normal, const float* albedo, int32_t w, int32_t h,
                       float sigma_c, float sigma_n, float sigma_a, int32_t iterations, float* out,
                       int threads);
int orc_joint_bilateral(const float* raw, const float* normal, const float* albedo, int32_t w, int32_t h,
                        float sigma_c, float sigma_n, float sigma_p, float sigma_a,
                        float* gaussian, float* bilateral, float* joint, int threads);

/* eval_tools hdr-metrics (shared/tools/eval_tools.cpp:121-213, 232-286) on interleaved RGB
 * float images, single-threaded in the reference's order. */
int orc_hdr_metrics(const float* ref, const float* tst, int32_t w, int32_t h, rpd_image_metrics* out);

/* Synthetic samples (include/rpd_synth.h) for pixels [first, first+count): pixel i gets
 * counts[i] (or spp) samples with ordinals start_n[i] (or 0) onward, written to the
 * planes of `out` (which must all be non-NULL except albedo, env_u; pixel_albedo gets the
 * per-pixel albedo). Returns the number of samples. */
int64_t orc_synth_fill(const rpd_synth_params* p, int64_t first_pixel, int64_t pixel_count,
                       int32_t spp, const int32_t* counts, const int32_t* start_n,
                       rpd_sample_soa* out, int threads);

#ifdef __cplusplus
}
#endif

#endif
