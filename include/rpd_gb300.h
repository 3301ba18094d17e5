/*
 * rpd_gb300.h — C ABI of the GB300 (sm_103a) StatMC / RPD denoise stage.
 *
 * The reference (andersonliu1/rpd-statmc-denoiser) runs this stage as free C++ functions
 * over process globals in path_tracer/main.cpp. This header replaces them with explicit
 * job handles whose state lives in HBM; every entry point below names the reference
 * function it stands in for. Plain C types only: no CUDA or C++ types cross the boundary.
 *
 * Threading: one host thread per job handle at a time. Jobs of one context may be driven
 * from different host threads. Every call is asynchronous on the job's CUDA stream unless
 * it returns host data (rpd_job_read, rpd_compute_adaptive_sample_counts with a host
 * destination, rpd_job_sync).
 *
 * Errors: every function returns an rpd_status. rpd_last_error() gives the message of the
 * last failure on the calling thread. Configuration errors use the reference's messages
 * (path_tracer/core/config.h:116-195).
 */
#ifndef RPD_GB300_H
#define RPD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RPD_ABI_VERSION 1

typedef enum rpd_status {
    RPD_OK = 0,
    RPD_ERR_INVALID_CONFIG = 1,   /* config.h:116-195 validation failed */
    RPD_ERR_INVALID_ARGUMENT = 2, /* null handle, bad size, out-of-range pixel span */
    RPD_ERR_OUT_OF_MEMORY = 3,    /* device or pinned-host allocation failed */
    RPD_ERR_OVER_BUDGET = 4,      /* job would exceed the context's HBM budget */
    RPD_ERR_CUDA = 5,             /* CUDA runtime error (message has the CUDA text) */
    RPD_ERR_TIMEOUT = 6,          /* a bounded device-side wait gave up */
    RPD_ERR_STATE = 7,            /* call out of order (e.g. denoise before any samples) */
    RPD_ERR_NO_DEVICE = 8,        /* no CUDA device, or the device is not sm_103 */
    RPD_ERR_CANCELLED = 9         /* a queued serving request was cancelled */
} rpd_status;

/* Where the pointers handed to a call live. */
typedef enum rpd_memory {
    RPD_MEM_HOST = 0,   /* host memory (pinned or pageable); the call copies it to HBM */
    RPD_MEM_DEVICE = 1  /* device memory of the context's GPU; used in place */
} rpd_memory;

/*
 * Denoise-stage knobs. Field names, meanings and defaults are those of RenderConfig
 * (path_tracer/core/config.h:15-49); only the fields the stage reads are kept.
 * seed plays the role of g_sampler_base_seed (main.cpp:43), which the adaptive
 * allocation hashes for its systematic-sampling offset (main.cpp:1427).
 */
typedef struct rpd_config {
    int32_t image_width;
    int32_t image_height;
    int32_t rpf_tile_size;                 /* default 8 */
    float rpf_shrinkage_scale;             /* default 1.0; 0 disables all RPD influence */
    float rpf_confidence_samples;          /* default 128 */
    int32_t color_window_radius;           /* default 7 */
    float color_normal_threshold;          /* default 0.5 */
    float color_depth_threshold;           /* default 0.25 */
    float color_compat_alpha;              /* default 0.05 */
    float color_sigma_max;                 /* default 6 */
    int32_t var_window_radius;             /* default 1 */
    float var_normal_threshold;            /* default 0.5 */
    float var_depth_threshold;             /* default 0.25 */
    float var_compat_sigma;                /* default 30 */
    float var_shrinkage_k;                 /* default 1e-3 */
    int32_t var_iterations;                /* default 2 */
    int32_t adaptive_base_samples;         /* default 0 */
    int32_t adaptive_spp;                  /* default 0 */
    float adaptive_sigma_max;              /* default 3 */
    int32_t adaptive_passes;               /* default 1 */
    int32_t adaptive_importance_smoothing_radius; /* default 1 */
    int32_t debug_statmc_outputs;          /* default 0; accepted, no files are written */
    uint32_t seed;                         /* g_sampler_base_seed */
} rpd_config;

/*
 * Per-sample record, structure of arrays. One entry per traced camera sample, in the
 * order the tracer produced them: all samples of a pixel are contiguous and pixels are
 * in increasing index order (the reference's render loops, main.cpp:685-719 and
 * 1488-1519, consume them in the same order).
 *
 * The fields are what the reference's per-sample hooks see:
 *   radiance        path radiance returned by mis_path_trace (main.cpp:706); a sample whose
 *                   radiance is not finite is dropped from the statistics and the grid
 *                   (main.cpp:707) but its primary-hit features still count (572-576).
 *   normal/depth/albedo   primary-hit features accumulated into FrameBuffers
 *                   (main.cpp:572-576); ignored when RPD_SAMPLE_HIT is clear.
 *   pixel_u, lens_u, brdf_u, light_u, env_u, category   the first-valid record
 *                   rpf::Sample (core/stats.h:331-399).
 *
 * A NULL plane means "never valid": the matching valid bit is treated as clear.
 * albedo may be NULL when pixel_albedo is given: every hit sample of a pixel then
 * contributes that pixel's albedo (indexed by pixel - first_pixel).
 */
#define RPD_SAMPLE_HIT                 0x01u
#define RPD_SAMPLE_PIXEL_VALID         0x02u
#define RPD_SAMPLE_LENS_VALID          0x04u
#define RPD_SAMPLE_BRDF_VALID          0x08u
#define RPD_SAMPLE_LIGHT_VALID         0x10u /* light_u (light_valid) */
#define RPD_SAMPLE_LIGHT_SELECT_VALID  0x20u
#define RPD_SAMPLE_ENV_VALID           0x40u
#define RPD_SAMPLE_RR_VALID            0x80u

#define RPD_CATEGORY_LIGHT_INDEX_MASK  0x0Fu /* light_index, valid only when < 16 (main.cpp:407) */
#define RPD_CATEGORY_RR_SURVIVED       0x10u

typedef struct rpd_sample_soa {
    const float* radiance[3];
    const float* normal[3];
    const float* depth;
    const float* albedo[3];
    const float* pixel_albedo[3];
    const float* pixel_u[2];
    const float* lens_u[2];
    const float* brdf_u[2];
    const float* light_u[2];
    const float* env_u[2];
    const uint8_t* flags;
    const uint8_t* category;
} rpd_sample_soa;

/* Readable per-job fields (rpd_job_read). Per-pixel fields are row-major W*H; RGB fields
 * are interleaved W*H*3 floats like the reference's Image; node fields are
 * nodes_x*nodes_y floats; the grid is nodes*13*36 doubles (see RPD_FIELD_GRID). */
typedef enum rpd_field {
    RPD_FIELD_DENOISED = 0,          /* buffers.denoised (main.cpp:1125) */
    RPD_FIELD_UNCERTAINTY,           /* buffers.uncertainty */
    RPD_FIELD_ALPHA,                 /* buffers.alpha */
    RPD_FIELD_VAR_TOTAL_DEBUG,       /* buffers.var_total_debug */
    RPD_FIELD_VAR_EFF_DEBUG,         /* buffers.var_eff_debug */
    RPD_FIELD_VAR_RATIO_DEBUG,       /* buffers.var_ratio_debug */
    RPD_FIELD_VARIANCE_DENOISED,     /* buffers.variance_denoised (main.cpp:1264) */
    RPD_FIELD_ADAPTIVE_IMPORTANCE,   /* buffers.adaptive_importance (main.cpp:1373) */
    RPD_FIELD_SENSITIVITY_CONFIDENCE,/* buffers.sensitivity_confidence (main.cpp:932) */
    RPD_FIELD_SENSITIVITY_GRADIENT,  /* buffers.sensitivity_gradient (main.cpp:945) */
    RPD_FIELD_HIT_COUNT,             /* int32 buffers.hit_count */
    RPD_FIELD_SAMPLE_COUNT,          /* int32 buffers.sample_count */
    RPD_FIELD_RADIANCE_SUM,          /* RGB sum of finite samples (buffers.radiance before finalize) */
    RPD_FIELD_NORMAL_SUM,            /* RGB buffers.normal before finalize */
    RPD_FIELD_ALBEDO_SUM,            /* RGB buffers.albedo before finalize */
    RPD_FIELD_DEPTH_SUM,             /* buffers.depth before finalize */
    RPD_FIELD_STATS_MEAN,            /* PixelStats::mean (core/stats.h:7) */
    RPD_FIELD_STATS_SQUARE_DIFF,     /* PixelStats::square_diff */
    RPD_FIELD_STATS_N,               /* int32 PixelStats::n */
    RPD_FIELD_STATS_COLOR_MEAN,      /* RGB PixelStats::color_mean */
    RPD_FIELD_STATS_SQRT_MEAN,       /* RGB PixelStats::sqrt_color_mean */
    RPD_FIELD_STATS_SQRT_SQUARE_DIFF,/* RGB PixelStats::sqrt_color_square_diff */
    RPD_FIELD_NODE_ALL,              /* sensitivity_tiles.all ... (core/buffers.h:23-40) */
    RPD_FIELD_NODE_ALL_CONF,
    RPD_FIELD_NODE_PIXEL,
    RPD_FIELD_NODE_PIXEL_CONF,
    RPD_FIELD_NODE_BRDF,
    RPD_FIELD_NODE_BRDF_CONF,
    RPD_FIELD_NODE_LENS,
    RPD_FIELD_NODE_LENS_CONF,
    RPD_FIELD_NODE_LIGHT,
    RPD_FIELD_NODE_LIGHT_CONF,
    RPD_FIELD_NODE_LIGHT_UV,
    RPD_FIELD_NODE_LIGHT_UV_CONF,
    RPD_FIELD_NODE_LIGHT_SELECT,
    RPD_FIELD_NODE_LIGHT_SELECT_CONF,
    RPD_FIELD_NODE_ENVIRONMENT,
    RPD_FIELD_NODE_ENVIRONMENT_CONF,
    RPD_FIELD_NODE_RR,
    RPD_FIELD_NODE_RR_CONF,
    /* rpf::Grid (core/stats.h:305-329): per node the 13 Tile dependencies in member order
     * (pixel, brdf, screen_brdf, lens, screen_lens, light_uv, screen_light_uv,
     * environment, screen_environment, light_select, screen_light_select, rr, screen_rr),
     * each as 36 doubles: weight[16], sum_y[16], w_sum, w2_sum, y_sum, y2_sum
     * (rr uses bins 0-1 of weight and sum_y; the rest are zero). */
    RPD_FIELD_GRID,
    /* Per-pixel bilinear expansions written by output_buffers (core/buffers.h:221-229). */
    RPD_FIELD_EXPANDED_ALL,
    RPD_FIELD_EXPANDED_PIXEL,
    RPD_FIELD_EXPANDED_BRDF,
    RPD_FIELD_EXPANDED_LENS,
    RPD_FIELD_EXPANDED_LIGHT,
    RPD_FIELD_EXPANDED_LIGHT_UV,
    RPD_FIELD_EXPANDED_LIGHT_SELECT,
    RPD_FIELD_EXPANDED_ENVIRONMENT,
    RPD_FIELD_EXPANDED_RR,
    RPD_FIELD_ADAPTIVE_COUNTS,       /* int32 last compute_adaptive_sample_counts result */
    RPD_FIELD_SQRT_VARIANCE_STABLE,  /* rgb: the StatMC window's sqrt-variance, max of the pixel's and its
                                      * 3x3 average (main.cpp:972-990), of the last statmc_denoise */
    RPD_FIELD_COUNT_
} rpd_field;

#define RPD_GRID_DEPENDENCIES 13
#define RPD_GRID_DEP_STRIDE 36

/* Stage timers (CUDA events on the job stream), like the reference's ms log lines
 * (main.cpp:952,1161,1267,1444). */
typedef enum rpd_stage {
    RPD_STAGE_ACCUMULATE = 0,       /* per-sample statistics + RPD grid (push) */
    RPD_STAGE_SENSITIVITY,          /* recompute_sensitivity */
    RPD_STAGE_STATMC,               /* statmc_denoise */
    RPD_STAGE_VARIANCE,             /* variance_denoise */
    RPD_STAGE_ADAPTIVE,             /* compute_adaptive_sample_counts */
    RPD_STAGE_COUNT_
} rpd_stage;

/* Kernel families, for per-kernel device timing (rpd_job_kernel_time). */
typedef enum rpd_kernel {
    RPD_KERNEL_OFFSETS = 0,         /* per-pixel sample offsets of a push */
    RPD_KERNEL_ACCUMULATE_PIXELS,   /* Welford statistics + features */
    RPD_KERNEL_GRID,                /* RPD grid: totals and screen bins */
    RPD_KERNEL_GRID_RANDOM,         /* RPD grid: random-dimension bins */
    RPD_KERNEL_MERGE,               /* pass grid merge (the exact grid mode's passes) */
    RPD_KERNEL_FEATURES,            /* feature cache */
    RPD_KERNEL_NODE_STATS,          /* per-node sensitivities, confidences, features */
    RPD_KERNEL_NODE_COMBINE,        /* prior smoothing + combine */
    RPD_KERNEL_SENS_PIXELS,         /* per-pixel confidence + gradient */
    RPD_KERNEL_RPD_CACHE,           /* per-pixel RPD components */
    RPD_KERNEL_SQRT_VARIANCE,       /* sqrt-domain variance of the mean + stabilisation */
    RPD_KERNEL_STATMC_WINDOW,       /* the StatMC Welch window */
    RPD_KERNEL_VARIANCE,            /* variance stabilisation iterations */
    RPD_KERNEL_ADAPTIVE,            /* importance + allocation */
    RPD_KERNEL_OTHER,               /* finalize, reads, fills */
    RPD_KERNEL_SYNTH,               /* the serving loop's sample generation */
    RPD_KERNEL_COUNT_
} rpd_kernel;

typedef struct rpd_ctx rpd_ctx;
typedef struct rpd_job rpd_job;

/* ---- configuration (core/config.h) ------------------------------------------------ */

/* RenderConfig defaults (core/config.h:27-48); image size 0, seed 0. */
void rpd_config_defaults(rpd_config* cfg);
/* parse_render_config's checks on the stage's fields (core/config.h:116-195), plus a
 * positive image size. Writes the reference's message into msg. */
int rpd_config_validate(const rpd_config* cfg, char* msg, size_t msg_capacity);

/* ---- context and jobs ------------------------------------------------------------- */

/* Opens the CUDA device and sets the HBM budget that jobs are admitted against
 * (0 = all free memory at creation). */
int rpd_ctx_create(int device, uint64_t hbm_budget_bytes, rpd_ctx** out);
void rpd_ctx_destroy(rpd_ctx* ctx);
/* Bytes of HBM a job with this config would hold. */
uint64_t rpd_job_footprint(const rpd_config* cfg);
uint64_t rpd_ctx_bytes_in_use(const rpd_ctx* ctx);

/* buffers.init + pixel_stats.assign + rpf_grid.init/reset (main.cpp:651-655), in HBM. */
int rpd_job_create(rpd_ctx* ctx, const rpd_config* cfg, rpd_job** out);
void rpd_job_destroy(rpd_job* job);
/* Replace the knobs of later calls (the reference passes RenderConfig to every stage).
 * Image size and rpf_tile_size are fixed at job creation. */
int rpd_job_set_config(rpd_job* job, const rpd_config* cfg);

/* Exact modes. By default the RPD grid is accumulated in double-float (pairs of floats,
 * ~2^-44 relative) and the StatMC window is evaluated in single precision with every
 * threshold decision (q > 25, the accepted-neighbour test, the t-table branch, the
 * weight-sum test) confirmed in double near its threshold. The exact modes instead run
 * the reference's double-precision operations in its order: RPD_EXACT_GRID makes the grid
 * bit-identical to the reference's single-thread run; RPD_EXACT_WINDOW evaluates every
 * neighbour in double. Both are slower on GB300, whose double-precision rate is 1/55 of
 * its single-precision rate. */
#define RPD_EXACT_GRID   0x1
#define RPD_EXACT_WINDOW 0x2
int rpd_job_set_exact(rpd_job* job, int flags);
/* Launch-shape knobs (no counterpart in the reference; results do not depend on them).
 * RPD_TUNE_GRID_SHAPE: warps per node of the random-dimension grid pass, as row groups x
 * dimension sets: 1 = 2x1, 2 = 2x2, 3 = 2x3, 4 = 1x2, 5 = 1x3, 6 = 1x1 (default). More dimension sets
 * keep fewer bins per warp (more resident warps) but walk the samples once per set. */
#define RPD_TUNE_GRID_SHAPE 0
/* RPD_TUNE_HOST_BAND_MB: a host-memory push is copied to HBM in row bands of about this many
 * megabytes (default 768, measured: fewer, larger copies keep the host link busier), each band's copy
 * overlapping the previous band's passes. */
#define RPD_TUNE_HOST_BAND_MB 1
/* RPD_TUNE_STATMC_ROWS: pixel rows per block of the StatMC window kernel: 2, 4 or 8 (0, the
 * default: 8 where the halo tile fits in shared memory, else the tallest that fits). */
#define RPD_TUNE_STATMC_ROWS 2
/* RPD_TUNE_ALLOCATOR: 0 (default) the parallel allocation of the adaptive counts on one block
 * per SM, N >= 2 the same on at most N blocks, 1 the one-thread kernel in the reference's order.
 * All give the same counts. */
#define RPD_TUNE_ALLOCATOR 3
/* RPD_TUNE_SMOOTHING: 0 (default) the adaptive importance smoothing's double-precision products
 * carried out exactly in integer instructions, 1 all of it in double-precision instructions. Both
 * give the same bits. */
#define RPD_TUNE_SMOOTHING 4
/* RPD_TUNE_WINDOW_GUARD: the fast StatMC window recomputes in double every neighbour whose
 * compatibility q (or Welch-Satterthwaite df) lies within 2^-g, relative, of a decision point,
 * and every pixel whose weight sum lies within 2^-(g+1) of the blend's 1.1 test; g = 15 by
 * default, 0..15 allowed. A smaller g sends more decisions to double; results stay within the
 * plain-form bar for every g (tested). */
#define RPD_TUNE_WINDOW_GUARD 5
int rpd_job_set_tuning(rpd_job* job, int knob, int value);
int rpd_job_get_tuning(rpd_job* job, int knob, int* value);
/* Start a new frame: clears every accumulator, like render_image_statmc's set-up. */
int rpd_job_begin_frame(rpd_job* job);

/*
 * Accumulate traced samples: per-pixel Welford statistics (accumulate_sample,
 * core/stats.h:25-41), primary-hit features (main.cpp:572-576) and the RPD grid
 * (accumulate_rpf_sample_to_grid, main.cpp:329-376) for pixels
 * [first_pixel, first_pixel + pixel_count). counts == NULL means every pixel has spp
 * samples; otherwise counts[i] is the number of samples of pixel first_pixel + i.
 * Pushes of one pass must come in increasing pixel order and cover each pixel once.
 * The planes of s and counts live in `where` memory.
 */
int rpd_job_push_samples(rpd_job* job, const rpd_sample_soa* s, int64_t first_pixel,
                         int64_t pixel_count, int32_t spp, const int32_t* counts,
                         rpd_memory where);
/*
 * Compact per-sample storage (the precision form; no counterpart in the reference): the same
 * record in 32 bytes per sample instead of 62-74, decoded to float by the statistics pass,
 * which then accumulates in single precision exactly as for rpd_sample_soa:
 *   sqrt_radiance   IEEE binary16 of sqrt(max(radiance, 0)) per channel (a non-finite
 *                   radiance stays non-finite and drops the sample); radiance = s * s
 *   normal          snorm16, n = max(q / 32767, -1)
 *   depth           binary16 of depth / depth_scale; depth = d * depth_scale
 *   pixel_albedo    binary16 per pixel (per-sample albedo is not carried)
 *   *_u             unorm16, u = q / 65536 (the 4x4 bins of Dependency2D::add are those
 *                   of the unquantised u: floor(u * 4) == floor(q / 16384))
 *   flags, category as in rpd_sample_soa.
 */
typedef struct rpd_sample_soa16 {
    const uint16_t* sqrt_radiance[3];
    const int16_t* normal[3];
    const uint16_t* depth;
    const uint16_t* pixel_albedo[3];
    const uint16_t* pixel_u[2];
    const uint16_t* lens_u[2];
    const uint16_t* brdf_u[2];
    const uint16_t* light_u[2];
    const uint16_t* env_u[2];
    const uint8_t* flags;
    const uint8_t* category;
    float depth_scale;
} rpd_sample_soa16;
int rpd_job_push_samples16(rpd_job* job, const rpd_sample_soa16* s, int64_t first_pixel,
                           int64_t pixel_count, int32_t spp, const int32_t* counts,
                           rpd_memory where);
/* Encode device-resident rpd_sample_soa planes (n_samples samples, n_pixels pixels) into
 * device-resident rpd_sample_soa16 planes (out's pointers; out->depth_scale is used). The
 * per-pixel albedo comes from in->pixel_albedo. */
int rpd_encode_samples16(rpd_ctx* ctx, const rpd_sample_soa* in, int64_t n_samples, int64_t n_pixels,
                         const rpd_sample_soa16* out);

/* End of a render pass: merge_rpf_grids_into (main.cpp:378-388, 730, 1531) and cache
 * invalidation (main.cpp:1533). In the exact grid mode the pass grid is added to the frame grid
 * here; in the default double-float mode the pushes add straight into the frame grid (the
 * frame's first push clears it), so a GRID read already reflects the pushes of an open pass. */
int rpd_job_end_pass(rpd_job* job);

/* The four stage entry points (main.cpp:741, 957, 1166, 1273). */
int rpd_recompute_sensitivity(rpd_job* job);
int rpd_statmc_denoise(rpd_job* job);
int rpd_variance_denoise(rpd_job* job);
/* Extra sample count per pixel for one adaptive pass; written to counts_out (W*H int32
 * in `where` memory; may be NULL, the result stays readable as RPD_FIELD_ADAPTIVE_COUNTS). */
int rpd_compute_adaptive_sample_counts(rpd_job* job, int32_t* counts_out, rpd_memory where);
/* Outcome of the job's last adaptive allocation (synchronises the job's stream): out[0] 1 when
 * the parallel allocation finished, out[1] 1 when it handed the allocation to the serial
 * kernel, out[2] 1 when a grid barrier timed out, out[3] water-filling passes, out[4]
 * fixed-point rounds beyond the first of each pass, out[5] chunks walked exactly, out[6] why
 * it handed over (0 it did not, 1 an importance outside [0, FLT_MAX], 2 no room for exact
 * chunk values, 3 a pass that did not settle, 4 a barrier timeout, 5 no cooperative launch). */
int rpd_job_allocator_stats(rpd_job* job, int32_t* out7);
/* Device timestamps (ns since its launch) of the last parallel allocation at each of its grid
 * barriers: up to max values into ns, the count in *n_out. */
int rpd_job_allocator_timeline(rpd_job* job, uint64_t* ns, int32_t max, int32_t* n_out);
/* The allocation step of compute_adaptive_sample_counts (main.cpp:1372-1438) on a caller's
 * importance map (W*H floats, the map after any smoothing; finite and >= 0): counts_out gets
 * the floor plus the extra samples exactly as the reference allocates them from that map. The
 * map becomes the job's RPD_FIELD_ADAPTIVE_IMPORTANCE. */
int rpd_adaptive_allocate(rpd_job* job, const float* importance, rpd_memory where, int32_t* counts_out,
                          rpd_memory out_where);
/* FrameBuffers::finalize (core/buffers.h:152-167) on the radiance/feature sums. */
int rpd_finalize(rpd_job* job);

/* rpd_job_push_samples / rpd_job_push_samples16 of host planes (RPD_MEM_HOST) that return once
 * the copies are enqueued (no counterpart in the reference, whose push has read its input when it
 * returns): the planes and counts must be page-locked (rpd_host_alloc) and stay unchanged until
 * rpd_job_sync returns. The copies overlap whatever the caller does next, such as the stages of
 * another job or the next frame's push into another job. */
int rpd_job_push_samples_async(rpd_job* job, const rpd_sample_soa* s, int64_t first_pixel,
                               int64_t pixel_count, int32_t spp, const int32_t* counts);
int rpd_job_push_samples16_async(rpd_job* job, const rpd_sample_soa16* s, int64_t first_pixel,
                                 int64_t pixel_count, int32_t spp, const int32_t* counts);

/* Copy a field to `where` memory. bytes must equal the field's size. */
int rpd_job_read(rpd_job* job, rpd_field field, void* dst, size_t bytes, rpd_memory where);
/* rpd_job_read enqueued on the job's stream without waiting: dst (page-locked host memory from
 * rpd_host_alloc, or device memory) holds the field once rpd_job_sync returns or the job's later
 * work has run. The copy overlaps the caller's next push into another job. */
int rpd_job_read_async(rpd_job* job, rpd_field field, void* dst, size_t bytes, rpd_memory where);
uint64_t rpd_field_bytes(const rpd_job* job, rpd_field field);
int rpd_job_sync(rpd_job* job);
/* Device milliseconds of the last run of a stage on this job. */
float rpd_job_stage_ms(const rpd_job* job, rpd_stage stage);
/* Kernel launches issued by this job since creation (for launch accounting). */
uint64_t rpd_job_launch_count(const rpd_job* job);
/* Per-kernel device timing: with profiling on, every launch of the job is bracketed by
 * CUDA events on the job's stream. rpd_job_kernel_time synchronises the job and returns
 * the summed milliseconds and launch count of one kernel family since the last reset. */
int rpd_job_set_profiling(rpd_job* job, int enable);
int rpd_job_kernel_time(rpd_job* job, rpd_kernel kernel, double* total_ms, uint64_t* launches);
int rpd_job_reset_kernel_times(rpd_job* job);
const char* rpd_kernel_name(rpd_kernel kernel);
/* Device-time markers on the job's stream (slots 0..7): record, then read the elapsed
 * milliseconds between two recorded slots (synchronises on the later one). */
int rpd_job_mark(rpd_job* job, int slot);
int rpd_job_mark_elapsed(rpd_job* job, int from_slot, int to_slot, float* ms);

/* Device-side counters of a job, no counterpart in the reference (its statmc_denoise,
 * main.cpp:957-1162, evaluates every neighbour in double precision). The fast StatMC window
 * evaluates neighbours in single precision and recomputes in double, exactly as the reference
 * does, the decisions that fall inside its guard bands; these counters show how often. */
typedef enum rpd_counter {
    RPD_COUNTER_WINDOW_PAIR_RECHECKS = 0,  /* neighbour pairs whose compatibility q was recomputed in
                                            * double (last statmc_denoise) */
    RPD_COUNTER_WINDOW_PIXEL_RECHECKS,     /* pixels whose whole window was recomputed in double
                                            * (weight sum within the 1.1 test's band; last statmc_denoise) */
    RPD_COUNTER_DEVICE_WAIT_TIMEOUTS,      /* bounded device-side waits that gave up (since job creation);
                                            * rpd_job_sync returns RPD_ERR_TIMEOUT while it is non-zero */
    RPD_COUNTER_WINDOW_SLOW_PIXELS,        /* pixels the fast loop handed to the slow pass: a decision
                                            * inside a guard band, or the weight sum inside the 1.1
                                            * test's band (last statmc_denoise) */
    RPD_COUNTER_COUNT_ = 8
} rpd_counter;
/* Waits for the job's stream and copies min(n, RPD_COUNTER_COUNT_) counters to out. */
int rpd_job_counters(rpd_job* job, uint64_t* out, int32_t n);

/* FP32 issue-rate probe (no counterpart in the reference): times a microkernel in which every
 * thread of a grid filling all SMs runs independent chains of single-precision fused
 * multiply-adds, with CUDA events, best of `repeats` launches. *per_second gets the FP32
 * lane instructions issued per second (one fused multiply-add = one instruction), *ms the
 * best launch's time. Changes no clock or power setting. */
int rpd_probe_fp32_issue(int device, int32_t repeats, double* per_second, double* ms);

/* ---- standalone filters (denoising/atrous_wavelet.cpp, denoising/joint_bilateral.cpp) ---- */

/* atrous_wavelet filter() core (denoising/atrous_wavelet.cpp:151-197): `iterations`
 * passes of atrous_filter_pass with step 2^i. raw/normal/albedo/out are interleaved RGB
 * W*H*3 floats in `where` memory. */
int rpd_atrous_wavelet(rpd_ctx* ctx, const float* raw, const float* normal, const float* albedo,
                       int32_t width, int32_t height, float sigma_c, float sigma_n, float sigma_a,
                       int32_t iterations, float* out, rpd_memory where);
/* joint_bilateral filter() core (denoising/joint_bilateral.cpp:15-132): writes the
 * gaussian, colour-bilateral and joint outputs in one pass. */
int rpd_joint_bilateral(rpd_ctx* ctx, const float* raw, const float* normal, const float* albedo,
                        int32_t width, int32_t height, float sigma_c, float sigma_n,
                        float sigma_p, float sigma_a, float* gaussian, float* bilateral,
                        float* joint, rpd_memory where);

/* ---- the tracer side: streaming per-sample records (main.cpp:649-737, 1451-1538) ---------
 *
 * The reference's render loops fold each traced sample into the pixel statistics and a
 * thread-local RPD grid from an OpenMP row loop (accumulate_sample,
 * accumulate_rpf_sample_to_grid, main.cpp:701-717 and 1509-1519). An emitter replaces those
 * calls: the loop's threads write each sample's record into page-locked ring buffers, row by
 * row, and every band of `band_rows` rows is copied to HBM and accumulated on the GPU as soon as
 * its rows are done, while tracing continues. Rows must be taken in increasing order across the
 * threads (as a dynamic schedule over rows hands them out); rows inside the ring's window of
 * `ring_slots` bands may be done in any order. A pass through an emitter accumulates exactly as
 * one rpd_job_push_samples of the whole image. */
typedef struct rpd_emitter rpd_emitter;
/* A ring of ring_slots (>= 2) bands of band_rows rows, each band holding up to
 * band_rows * width * max_spp samples (page-locked host and device copies of every plane). */
int rpd_emitter_create(rpd_job* job, int32_t band_rows, int32_t ring_slots, int32_t max_spp, rpd_emitter** out);
/* Open a pass: spp samples per pixel, or counts[i] (host memory, W*H) for pixel i, e.g. the
 * counts of rpd_compute_adaptive_sample_counts (render_image_adaptive). */
int rpd_emitter_begin_pass(rpd_emitter* em, int32_t spp, const int32_t* counts);
/* Where row y's samples go: the planes of `planes` point at the row's first sample (every plane
 * of rpd_sample_soa is present; albedo per sample); pixel x of the row owns the samples
 * [pixel_offsets[x] - pixel_offsets[0], pixel_offsets[x + 1] - pixel_offsets[0]), in the order
 * the tracer draws them. Waits (bounded) while the row's ring slot still holds an earlier band. */
int rpd_emitter_row(rpd_emitter* em, int32_t y, rpd_sample_soa* planes, const int64_t** pixel_offsets);
/* Row y is written. The band's last row sends the band (and every complete band after it). */
int rpd_emitter_row_done(rpd_emitter* em, int32_t y);
/* Every row done: waits for the last copies and closes the pass (rpd_job_end_pass). */
int rpd_emitter_end_pass(rpd_emitter* em);
void rpd_emitter_destroy(rpd_emitter* em);

/* ---- evaluation metrics (shared/tools/eval_tools.cpp) --------------------------------- */

/* What `eval_tools hdr-metrics <ref> <test>` reports (eval_tools.cpp:215-286, with
 * compute_extended_metrics 121-213), for interleaved RGB float images. */
typedef struct rpd_image_metrics {
    double mae;                 /* mean |ref - test| over pixels and channels */
    double rmse;                /* sqrt(mean (ref - test)^2) */
    double psnr;                /* 20 log10(peak / rmse); +inf when rmse is 0 */
    double peak;                /* max |ref| (1 when that is 0) */
    double ssim[3];             /* the global per-channel SSIM diagnostic */
    double ssim_mean;           /* (ssim[0] + ssim[1] + ssim[2]) / 3 */
    double nrmse;               /* sqrt(sum (ref - test)^2 / max(1e-18, sum ref^2)) */
    double log_ssim11;          /* mean SSIM over 11x11 windows (clipped at the edges) of
                                 * log1p(max(0, luminance)), constants from the reference's peak */
    double log_gradient_nrmse;  /* NRMSE of the forward x and y differences of that log luminance */
} rpd_image_metrics;
/* The metrics of `test` against `reference` (w x h, interleaved RGB floats in `where` memory),
 * computed on the context's GPU in double precision. Scalars agree with the reference's to
 * about 1e-12 relative (the sums are taken in another order). */
int rpd_hdr_metrics(rpd_ctx* ctx, const float* reference, const float* test, int32_t width, int32_t height,
                    rpd_memory where, rpd_image_metrics* out);
/* The same for a job's denoised image (RPD_FIELD_DENOISED) against `reference`, on the job's
 * stream without copying the image out: a caller scores each frame where it was denoised. */
int rpd_job_hdr_metrics(rpd_job* job, const float* reference, rpd_memory where, rpd_image_metrics* out);

/* ---- output writers (core/buffers.h:197-250, shared/image.h) --------------------------- */

/* Tonemapping presets of Image::ToneMapping (shared/image.h:20), in its order. */
typedef enum rpd_tonemap {
    RPD_TONEMAP_AGX = 0,         /* AGXDefault */
    RPD_TONEMAP_AGX_GOLDEN = 1,
    RPD_TONEMAP_AGX_PUNCHY = 2,
    RPD_TONEMAP_ACES = 3
} rpd_tonemap;
/* Image::save (a Radiance RGBE .hdr file) and Image::save_with_tonemapping (an 8-bit RGB .png)
 * of an interleaved RGB float image in `where` memory; the pixel encoding runs on the context's
 * GPU, the file is written from host memory. RGBE has no sign: negative components are written
 * as 0. */
int rpd_write_hdr(rpd_ctx* ctx, const float* rgb, int32_t width, int32_t height, rpd_memory where,
                  const char* path);
int rpd_write_png(rpd_ctx* ctx, const float* rgb, int32_t width, int32_t height, rpd_memory where,
                  int tonemap, const char* path);
/* output_buffers (core/buffers.h:197-250) for a finalized job (rpd_finalize): the files the
 * reference writes under `prefix` (its directory + name; file names are prefix + suffix), from
 * the job's device buffers: prefix.png / prefix.hdr (the denoised image when statmc is set,
 * else the radiance), and with statmc the raw radiance (_raw.png, _raw.hdr), the expanded
 * sensitivity maps (_sensitivity.hdr, _sensitivity_pixel.hdr ... _sensitivity_rr.hdr),
 * _sensitivity_confidence, _sensitivity_gradient, _uncertainty, _alpha, _vardenoised,
 * _adaptive_importance, _sample_fraction; always _albedo, _normal, _depth; with statmc
 * _var_total, _var_eff, _var_ratio. The per-sample record carries no world position, so the
 * reference's _worldpos.hdr has no counterpart here. */
int rpd_job_write_outputs(rpd_job* job, const char* prefix, int tonemap, int statmc);

/* No counterpart in the reference: the a-trous filter above for callers that may not
 * allocate device memory while they run (all HBM reserved up front, no device-wide
 * synchronisation from cudaFree allowed, or an allocator that forbids library-internal
 * allocations). Its ping-pong scratch is a fixed device array of the library holding
 * RPD_NOALLOC_MAX_PIXELS pixels; larger images fail with RPD_ERR_INVALID_ARGUMENT.
 * raw/normal/albedo/out are device pointers on the calling thread's current device, out
 * must not overlap the inputs, and the call is asynchronous on `stream` (a cudaStream_t,
 * NULL for the legacy default stream). One scratch per device: overlapping calls on a
 * device race. The first call on a device looks the scratch up and should precede any
 * stream capture; the address is kept for the life of the process, so the entry point must
 * not be called on a device after cudaDeviceReset. The 48 MiB array is part of the library's
 * module: every context that loads the module reserves it (with lazy loading at first use,
 * with CUDA_MODULE_LOADING=EAGER at context creation), whether or not this is called. */
#define RPD_NOALLOC_MAX_PIXELS 4194304 /* 2048 x 2048; 48 MiB of FP32 RGB scratch */
int rpd_atrous_wavelet_noalloc(const float* raw, const float* normal, const float* albedo,
                               int32_t width, int32_t height, float sigma_c, float sigma_n,
                               float sigma_a, int32_t iterations, float* out, void* stream);

/* ---- the batched form (no counterpart in the reference) ------------------------------ */

/* Autotune a job's launch shapes (RPD_TUNE_GRID_SHAPE, RPD_TUNE_STATMC_ROWS) on the frame in
 * device-resident planes (exactly one of s32 / s16; spp samples per pixel): every candidate is
 * timed on this frame and the fastest kept. The choice is cached per frame class (size, spp,
 * tile, window radii, storage) for the process, so later jobs of the class skip the timing.
 * Leaves the frame denoised (begin_frame .. variance_denoise). */
int rpd_job_autotune(rpd_job* job, const rpd_sample_soa* s32, const rpd_sample_soa16* s16, int32_t spp);

/* A batch: frames of different jobs (uneven sizes allowed) run as one CUDA graph. */
typedef struct rpd_batch_s rpd_batch;
int rpd_batch_create(rpd_ctx* ctx, rpd_batch** out);
/* Add a frame: `job` runs begin_frame, one push of device-resident planes (exactly one of s32 /
 * s16, spp samples per pixel), end_pass, recompute_sensitivity, statmc_denoise and
 * variance_denoise. A job appears once per batch. */
int rpd_batch_add(rpd_batch* b, rpd_job* job, const rpd_sample_soa* s32, const rpd_sample_soa16* s16,
                  int32_t spp);
/* Run every frame. The first run executes the frames once directly (sizing every buffer), then
 * captures all of them, each on its job's stream, into one CUDA graph; every run launches that
 * graph: one launch for the whole batch, frames of different jobs running concurrently. The
 * graph keeps the planes' addresses (update their contents, not the pointers). Asynchronous;
 * rpd_batch_sync waits, rpd_batch_last_ms gives the device time of the last launch. */
int rpd_batch_run(rpd_batch* b);
int rpd_batch_sync(rpd_batch* b);
int rpd_batch_last_ms(rpd_batch* b, float* ms);
uint64_t rpd_batch_kernel_count(rpd_batch* b);  /* kernel nodes in one run */
/* Frames run in `lanes` concurrent chains (default 4), largest frames first, each frame to the
 * least-loaded chain. Set before the first run. */
int rpd_batch_set_lanes(rpd_batch* b, int lanes);
void rpd_batch_destroy(rpd_batch* b);

/* ---- memory helpers for callers without a CUDA toolchain ---------------------------- */

/* HBM owned by the caller (sample planes for RPD_MEM_DEVICE pushes). Counts against the
 * context's budget. */
int rpd_device_alloc(rpd_ctx* ctx, uint64_t bytes, void** out);
int rpd_device_free(rpd_ctx* ctx, void* ptr);
/* Page-locked host memory (fast host->HBM pushes). */
int rpd_host_alloc(uint64_t bytes, void** out);
int rpd_host_free(void* ptr);
/* Synchronous copy; kind 0 = host->device, 1 = device->host, 2 = device->device. */
int rpd_memcpy(rpd_ctx* ctx, void* dst, const void* src, uint64_t bytes, int kind);

/* ---- synthetic samples (include/rpd_synth.h) ---------------------------------------- */

struct rpd_synth_params;
/* Fill the planes of `out` (radiance, normal, depth, pixel_u, lens_u, brdf_u, light_u,
 * flags, category; albedo and pixel_albedo when non-NULL) with the seeded synthetic
 * samples of pixels [first_pixel, first_pixel + pixel_count): spp each, or counts[i],
 * with sample ordinals starting at start_n[i] (0 when NULL). Host and device fills are
 * bit-identical. counts/start_n live in `where` memory like the planes. */
int rpd_synth_fill(rpd_ctx* ctx, const struct rpd_synth_params* params, int64_t first_pixel,
                   int64_t pixel_count, int32_t spp, const int32_t* counts, const int32_t* start_n,
                   const rpd_sample_soa* out, rpd_memory where);

const char* rpd_last_error(void);
const char* rpd_status_string(int status);

/* ---- serving: continuous batching of denoise requests (serve.cu) ----------------------
 *
 * A request loop over one GPU. Requests of any size and first-pass spp are submitted at any
 * time; a scheduler thread admits them in arrival order as slots (max_inflight) and HBM budget
 * free up, runs each one's whole pipeline — the first pass, config.adaptive_passes adaptive
 * passes, the final StatMC and variance passes (render(), main.cpp:1543-1564) — on its own
 * stream with its state resident in HBM, and copies the denoised image to host memory. Requests
 * overlap on the device. The per-sample source is the seeded generator of rpd_synth.h evaluated
 * on the device (the first pass draws ordinals 0..spp-1 of each pixel, adaptive pass p draws
 * from p << 16 on), so a request is fully described by its size, spp and seed. A request's
 * result does not depend on what else runs. */
typedef struct rpd_server rpd_server;

typedef enum rpd_storage {
    RPD_STORAGE_FP32 = 0,   /* rpd_sample_soa planes */
    RPD_STORAGE_FP16 = 1    /* rpd_sample_soa16 planes (sqrt-radiance binary16, snorm16 normals, ...) */
} rpd_storage;

typedef struct rpd_server_config {
    rpd_config knobs;            /* stage knobs of every request; the image size comes per request */
    uint64_t hbm_budget_bytes;   /* admission budget for request state and buffers (0: the context's) */
    int32_t max_inflight;        /* requests on the GPU at once, 1..256 */
    int32_t storage;             /* rpd_storage of the sample buffers */
    int32_t profile;             /* nonzero: time every kernel family of every request (CUDA events) */
    int32_t allocator_blocks;    /* blocks of each request's parallel adaptive allocation: 0 one on
                                  * half the SMs, N >= 2 at most N (RPD_TUNE_ALLOCATOR); fewer leave
                                  * SMs to the other requests' kernels while an allocation walks its
                                  * chain */
} rpd_server_config;

typedef struct rpd_request {
    int32_t width, height;
    int32_t spp;                 /* samples per pixel of the first pass, 0..65535 */
    uint32_t seed;               /* seed of the synthetic workload (rpd_synth_defaults at this size) */
    float* denoised_out;         /* width*height*3 floats (interleaved RGB), page-locked host memory
                                  * (rpd_host_alloc) or device memory; NULL: the result is copied to
                                  * a buffer of the server and not kept */
    int32_t out_where;           /* rpd_memory of denoised_out */
    uint64_t tag;                /* returned in the completion */
} rpd_request;

typedef struct rpd_completion {
    uint64_t id, tag;
    int32_t status;              /* RPD_OK, RPD_ERR_CANCELLED or the error that stopped the request */
    int32_t width, height, spp;
    int64_t samples;             /* samples denoised: the first pass plus every adaptive pass */
    double submit_ms, admit_ms, done_ms;  /* server clock (ms since rpd_server_create) */
} rpd_completion;

typedef struct rpd_server_stats {
    int64_t submitted, completed, rejected, queued, inflight;
    uint64_t bytes_reserved, bytes_peak, bytes_budget;
    int64_t jobs_cached;
    double now_ms;               /* server clock */
    int64_t launches;            /* kernels enqueued for requests so far */
    int64_t jobs_created;        /* jobs (per-size arenas) created so far */
    int64_t jobs_destroyed;      /* cached jobs destroyed to make room for other sizes */
    int64_t scratch_grown;       /* cached jobs whose push scratch had to grow on reuse */
} rpd_server_stats;

void rpd_server_config_defaults(rpd_server_config* cfg);
int rpd_server_create(rpd_ctx* ctx, const rpd_server_config* cfg, rpd_server** out);
/* Queues a request. A request that cannot fit the budget even alone is refused here with
 * RPD_ERR_OVER_BUDGET; a bad size or config with RPD_ERR_INVALID_ARGUMENT / _CONFIG. */
int rpd_server_submit(rpd_server* srv, const rpd_request* req, uint64_t* id_out);
/* Moves up to max finished requests (in completion order) to out; *n_out gets the number. */
int rpd_server_poll(rpd_server* srv, rpd_completion* out, int32_t max, int32_t* n_out);
/* Waits until nothing is queued or running (timeout_ms < 0: no limit); RPD_ERR_TIMEOUT else. */
int rpd_server_drain(rpd_server* srv, int32_t timeout_ms);
/* Cancels a queued request (its completion carries RPD_ERR_CANCELLED); one already on the GPU
 * runs to the end (RPD_ERR_STATE). */
int rpd_server_cancel(rpd_server* srv, uint64_t id);
int rpd_server_get_stats(rpd_server* srv, rpd_server_stats* out);
/* With profile set: the summed device time and launches of each kernel family (RPD_KERNEL_COUNT_
 * entries each) over the requests finished so far. The times include waits behind other requests'
 * work on a busy GPU. */
int rpd_server_kernel_times(rpd_server* srv, double* ms_out, uint64_t* launches_out);
/* Finishes every submitted request, then releases the server. */
void rpd_server_destroy(rpd_server* srv);

#ifdef __cplusplus
}
#endif

#endif /* RPD_GB300_H */
