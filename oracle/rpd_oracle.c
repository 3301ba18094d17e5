/*
 * rpd_oracle.c — CPU restatement of the reference's StatMC / RPD denoise stage.
 *
 * TEST INFRASTRUCTURE ONLY (see rpd_oracle.h). Each function cites the reference lines it
 * restates. Floating-point conventions, which the CUDA kernels follow as well:
 *   - single-precision where the reference uses float, double where it uses double,
 *     evaluated left to right in the reference's order, no FMA contraction
 *     (built with -ffp-contract=off);
 *   - 3-vector reductions (dot, squaredNorm, norm) as c0 + (c1 + c2), the order of
 *     Eigen's scalar unroller (oracle/ref_shim/Eigen/Dense);
 *   - std::max(a,b) = (a < b) ? b : a, std::min(a,b) = (b < a) ? b : a,
 *     std::clamp(v,lo,hi) = (v < lo) ? lo : (hi < v) ? hi : v.
 */
#include "rpd_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EPS_SMALL 1e-8f      /* shared/global.h:4 */
#define EPS_F 1e-4f          /* path_tracer/core/common.h:5 */
#define BASE_ALBEDO_THRESH 0.12f  /* core/stats.h:45 */
#define NDEP 13
#define DSTRIDE 36

/* ---- scalar helpers with the C++ standard library's semantics ---------------------- */

static inline float fmaxs(float a, float b) { return (a < b) ? b : a; }
static inline float fmins(float a, float b) { return (b < a) ? b : a; }
static inline float fclamps(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }
static inline double dmaxs(double a, double b) { return (a < b) ? b : a; }
static inline double dmins(double a, double b) { return (b < a) ? b : a; }
static inline double dclamps(double v, double lo, double hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }
static inline int imaxs(int a, int b) { return (a < b) ? b : a; }
static inline int imins(int a, int b) { return (b < a) ? b : a; }
static inline int iclamps(int v, int lo, int hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }
/* global.h:45-48 */
/* The template lerp of shared/global.h:45-48; main.cpp calls it for Vec3f only
 * (main.cpp:1115). */
static inline float lerpf(float a, float b, float t) { return a + (b - a) * t; }
/* Every lerp(float, float, float) call of the reference (main.cpp:196,869-879,
 * core/buffers.h:84-86, core/stats.h:90) resolves to std::lerp instead: stb_image.h, which
 * shared/image.h:10-11 includes with its implementation, includes <math.h>, and in C++20
 * libstdc++'s <math.h> brings std::lerp into the global namespace, where the non-template
 * float overload beats the template above. This is the C++20 algorithm (P0811R3) as
 * libstdc++ evaluates it: when a and b do not share a sign, t*b + (1-t)*a; t == 1 gives b
 * exactly; otherwise a + t*(b-a), kept from passing b. */
static inline float lerp_std(float a, float b, float t) {
    if ((a <= 0.0f && b >= 0.0f) || (a >= 0.0f && b <= 0.0f)) return t * b + (1.0f - t) * a;
    if (t == 1.0f) return b;
    const float x = a + t * (b - a);
    if ((t > 1.0f) == (b > a)) return (b < x) ? x : b;
    return (b > x) ? x : b;
}
/* Eigen 3-vector reduction order */
static inline float dot3(const float* a, const float* b) {
    return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]);
}
static inline float norm3(const float* a) { return sqrtf(dot3(a, a)); }
static inline void normalize3(float* v) {
    const float z = dot3(v, v);
    if (z > 0.0f) {
        const float s = sqrtf(z);
        v[0] = v[0] / s; v[1] = v[1] / s; v[2] = v[2] / s;
    }
}
/* common.h:39-41 */
static inline float calc_luminance(float r, float g, float b) {
    return 0.2126f * r + 0.7152f * g + 0.0722f * b;
}
/* main.cpp:266-268 */
static inline float relative_depth_delta(float a, float b) {
    float m = fabsf(a);
    if (m < fabsf(b)) m = fabsf(b);
    if (m < EPS_SMALL) m = EPS_SMALL;
    return fabsf(a - b) / m;
}
/* main.cpp:270-281 */
static inline uint32_t hash_u32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
static inline float hash_to_unit_float(uint32_t x) {
    return (float)(hash_u32(x) & 0x00ffffffu) / (float)0x01000000u;
}

static double now_ms(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec * 1e3 + (double)ts.tv_nsec * 1e-6;
}

/* ---- state ------------------------------------------------------------------------- */

typedef struct {              /* core/stats.h:6-23 */
    float mean, square_diff;
    int n;
    float color_mean[3], sqrt_mean[3], sqrt_sq[3];
} pstats;

/* rpf::Tile (core/stats.h:184-230) as 13 dependencies of 36 doubles:
 * weight[16], sum_y[16], w_sum, w2_sum, y_sum, y2_sum. */
enum { D_PIXEL = 0, D_BRDF, D_SCREEN_BRDF, D_LENS, D_SCREEN_LENS, D_LIGHT_UV, D_SCREEN_LIGHT_UV,
       D_ENV, D_SCREEN_ENV, D_LIGHT_SELECT, D_SCREEN_LIGHT_SELECT, D_RR, D_SCREEN_RR };
static const int dep_bins[NDEP] = {16, 16, 16, 16, 16, 16, 16, 16, 16, 16, 16, 2, 16};

enum { N_ALL = 0, N_ALL_CONF, N_PIXEL, N_PIXEL_CONF, N_BRDF, N_BRDF_CONF, N_LENS, N_LENS_CONF,
       N_LIGHT, N_LIGHT_CONF, N_LIGHT_UV, N_LIGHT_UV_CONF, N_LIGHT_SELECT, N_LIGHT_SELECT_CONF,
       N_ENV, N_ENV_CONF, N_RR, N_RR_CONF, N_FIELDS };

/* main.cpp:54-76 SensitivityImageCache order */
enum { C_ALL = 0, C_PIXEL, C_PIXEL_CONF, C_BRDF, C_BRDF_CONF, C_LENS, C_LENS_CONF, C_LIGHT,
       C_LIGHT_CONF, C_LIGHT_UV, C_LIGHT_UV_CONF, C_LIGHT_SELECT, C_LIGHT_SELECT_CONF, C_ENV,
       C_ENV_CONF, C_RR, C_RR_CONF, C_GRADIENT, C_FIELDS };
static const int cache_from_node[C_GRADIENT] = {
    N_ALL, N_PIXEL, N_PIXEL_CONF, N_BRDF, N_BRDF_CONF, N_LENS, N_LENS_CONF, N_LIGHT, N_LIGHT_CONF,
    N_LIGHT_UV, N_LIGHT_UV_CONF, N_LIGHT_SELECT, N_LIGHT_SELECT_CONF, N_ENV, N_ENV_CONF, N_RR, N_RR_CONF};

struct orc_job {
    rpd_config cfg;
    int w, h, threads;
    int support, step, nodes_x, nodes_y;
    size_t np, nn;
    pstats* stats;
    int32_t* hit_count;
    int32_t* sample_count;
    float* radiance;      /* 3 per pixel */
    float* normal;        /* 3 per pixel */
    float* albedo;        /* 3 per pixel */
    float* depth;
    double* grid;         /* nn * NDEP * DSTRIDE */
    double** pass_grids;  /* one per thread of the open pass */
    int n_pass_grids;
    float* node[N_FIELDS];
    float* sens_confidence;
    float* sens_gradient;
    int features_valid;
    float* f_normal;      /* 3 per pixel */
    float* f_depth;
    float* f_albedo;      /* 3 per pixel */
    int cache_valid;
    float* cache[C_FIELDS];
    float* denoised;      /* 3 per pixel */
    float* uncertainty;
    float* alpha;
    float* var_total;
    float* var_eff;
    float* var_ratio;
    float* variance_denoised;
    float* sqrt_var_stable;  /* rgb interleaved, the last statmc_denoise's */
    float* adaptive_importance;
    int32_t* last_counts;
    double stage_ms[RPD_STAGE_COUNT_];
};

static void set_omp(int threads) {
#ifdef _OPENMP
    omp_set_num_threads(threads > 0 ? threads : omp_get_num_procs());
#else
    (void)threads;
#endif
}

/* ---- configuration (core/config.h:27-48, 116-195) ----------------------------------- */

void orc_config_defaults(rpd_config* c) {
    memset(c, 0, sizeof(*c));
    c->rpf_tile_size = 8;
    c->rpf_shrinkage_scale = 1.0f;
    c->rpf_confidence_samples = 128.0f;
    c->color_window_radius = 7;
    c->color_normal_threshold = 0.5f;
    c->color_depth_threshold = 0.25f;
    c->color_compat_alpha = 0.05f;
    c->color_sigma_max = 6.0f;
    c->var_window_radius = 1;
    c->var_normal_threshold = 0.5f;
    c->var_depth_threshold = 0.25f;
    c->var_compat_sigma = 30.0f;
    c->var_shrinkage_k = 1e-3f;
    c->var_iterations = 2;
    c->adaptive_base_samples = 0;
    c->adaptive_spp = 0;
    c->adaptive_sigma_max = 3.0f;
    c->adaptive_passes = 1;
    c->adaptive_importance_smoothing_radius = 1;
    c->debug_statmc_outputs = 0;
}

static int fail(char* msg, size_t cap, const char* text) {
    if (msg && cap) { strncpy(msg, text, cap - 1); msg[cap - 1] = 0; }
    return RPD_ERR_INVALID_CONFIG;
}

int orc_config_validate(const rpd_config* c, char* msg, size_t cap) {
    if (c->image_width <= 0 || c->image_height <= 0) return fail(msg, cap, "image_width and image_height must be positive");
    if (c->rpf_tile_size <= 0) return fail(msg, cap, "rpf_tile_size must be positive");
    if (c->color_window_radius <= 0) return fail(msg, cap, "color_window_radius must be positive");
    if (!isfinite(c->color_normal_threshold) || c->color_normal_threshold <= 0.0f || c->color_normal_threshold > 1.0f)
        return fail(msg, cap, "color_normal_threshold must be finite and in (0,1]");
    if (!isfinite(c->color_depth_threshold) || c->color_depth_threshold < 0.0f)
        return fail(msg, cap, "color_depth_threshold must be finite and non-negative");
    if (!isfinite(c->color_compat_alpha) || c->color_compat_alpha <= 0.0f || c->color_compat_alpha >= 1.0f)
        return fail(msg, cap, "color_compat_alpha must be finite and in (0,1)");
    if (!isfinite(c->color_sigma_max) || c->color_sigma_max <= 0.0f)
        return fail(msg, cap, "color_sigma_max must be finite and positive");
    if (c->var_window_radius <= 0) return fail(msg, cap, "var_window_radius must be positive");
    if (!isfinite(c->var_normal_threshold) || c->var_normal_threshold <= 0.0f || c->var_normal_threshold > 1.0f)
        return fail(msg, cap, "var_normal_threshold must be finite and in (0,1]");
    if (!isfinite(c->var_depth_threshold) || c->var_depth_threshold < 0.0f)
        return fail(msg, cap, "var_depth_threshold must be finite and non-negative");
    if (!isfinite(c->var_compat_sigma) || c->var_compat_sigma <= 0.0f)
        return fail(msg, cap, "var_compat_sigma must be finite and positive");
    if (!isfinite(c->var_shrinkage_k) || c->var_shrinkage_k <= 0.0f)
        return fail(msg, cap, "var_shrinkage_k must be finite and positive");
    if (c->adaptive_base_samples < 0) return fail(msg, cap, "adaptive_base_samples must be non-negative");
    if (c->adaptive_spp < 0) return fail(msg, cap, "adaptive_spp must be non-negative");
    if (c->adaptive_base_samples > c->adaptive_spp) return fail(msg, cap, "adaptive_base_samples cannot exceed adaptive_spp");
    if (!isfinite(c->adaptive_sigma_max) || c->adaptive_sigma_max <= 0.0f)
        return fail(msg, cap, "adaptive_sigma_max must be finite and positive");
    if (c->adaptive_passes < 0) return fail(msg, cap, "adaptive_passes must be non-negative");
    if (c->adaptive_importance_smoothing_radius < 0)
        return fail(msg, cap, "adaptive_importance_smoothing_radius must be non-negative");
    if (c->var_iterations <= 0) return fail(msg, cap, "var_iterations must be positive");
    if (!isfinite(c->rpf_shrinkage_scale) || c->rpf_shrinkage_scale < 0.0f)
        return fail(msg, cap, "rpf_shrinkage_scale must be finite and non-negative");
    if (!isfinite(c->rpf_confidence_samples) || c->rpf_confidence_samples <= 0.0f)
        return fail(msg, cap, "rpf_confidence_samples must be finite and positive");
    if (msg && cap) msg[0] = 0;
    return RPD_OK;
}

/* ---- job lifetime (main.cpp:650-655, core/buffers.h:121-150, core/stats.h:312-318) -- */

static void* zalloc(size_t n) { return calloc(n ? n : 1, 1); }

orc_job* orc_job_create(const rpd_config* cfg) {
    if (orc_config_validate(cfg, NULL, 0) != RPD_OK) return NULL;
    orc_job* j = (orc_job*)zalloc(sizeof(orc_job));
    j->cfg = *cfg;
    j->w = cfg->image_width;
    j->h = cfg->image_height;
    j->threads = 0;
    j->support = cfg->rpf_tile_size;
    j->step = imaxs(1, j->support / 2);
    j->nodes_x = imaxs(2, (j->w + j->step - 1) / j->step + 1);
    j->nodes_y = imaxs(2, (j->h + j->step - 1) / j->step + 1);
    j->np = (size_t)j->w * (size_t)j->h;
    j->nn = (size_t)j->nodes_x * (size_t)j->nodes_y;
    const size_t np = j->np, nn = j->nn;
    j->stats = (pstats*)zalloc(np * sizeof(pstats));
    j->hit_count = (int32_t*)zalloc(np * 4);
    j->sample_count = (int32_t*)zalloc(np * 4);
    j->radiance = (float*)zalloc(np * 3 * sizeof(float));
    j->normal = (float*)zalloc(np * 3 * sizeof(float));
    j->albedo = (float*)zalloc(np * 3 * sizeof(float));
    j->depth = (float*)zalloc(np * sizeof(float));
    j->grid = (double*)zalloc(nn * NDEP * DSTRIDE * sizeof(double));
    for (int f = 0; f < N_FIELDS; ++f) j->node[f] = (float*)zalloc(nn * sizeof(float));
    j->sens_confidence = (float*)zalloc(np * sizeof(float));
    j->sens_gradient = (float*)zalloc(np * sizeof(float));
    j->f_normal = (float*)zalloc(np * 3 * sizeof(float));
    j->f_depth = (float*)zalloc(np * sizeof(float));
    j->f_albedo = (float*)zalloc(np * 3 * sizeof(float));
    for (int f = 0; f < C_FIELDS; ++f) j->cache[f] = (float*)zalloc(np * sizeof(float));
    j->denoised = (float*)zalloc(np * 3 * sizeof(float));
    j->uncertainty = (float*)zalloc(np * sizeof(float));
    j->alpha = (float*)zalloc(np * sizeof(float));
    j->var_total = (float*)zalloc(np * sizeof(float));
    j->var_eff = (float*)zalloc(np * sizeof(float));
    j->var_ratio = (float*)zalloc(np * sizeof(float));
    j->variance_denoised = (float*)zalloc(np * sizeof(float));
    j->sqrt_var_stable = (float*)zalloc(np * 3 * sizeof(float));
    j->adaptive_importance = (float*)zalloc(np * sizeof(float));
    j->last_counts = (int32_t*)zalloc(np * 4);
    return j;
}

static void free_pass_grids(orc_job* j) {
    for (int i = 0; i < j->n_pass_grids; ++i) free(j->pass_grids[i]);
    free(j->pass_grids);
    j->pass_grids = NULL;
    j->n_pass_grids = 0;
}

void orc_job_destroy(orc_job* j) {
    if (!j) return;
    free_pass_grids(j);
    free(j->stats); free(j->hit_count); free(j->sample_count); free(j->radiance); free(j->normal);
    free(j->albedo); free(j->depth); free(j->grid);
    for (int f = 0; f < N_FIELDS; ++f) free(j->node[f]);
    free(j->sens_confidence); free(j->sens_gradient); free(j->f_normal); free(j->f_depth); free(j->f_albedo);
    for (int f = 0; f < C_FIELDS; ++f) free(j->cache[f]);
    free(j->denoised); free(j->uncertainty); free(j->alpha); free(j->var_total); free(j->var_eff);
    free(j->var_ratio); free(j->variance_denoised); free(j->sqrt_var_stable); free(j->adaptive_importance); free(j->last_counts);
    free(j);
}

void orc_set_threads(orc_job* j, int threads) { j->threads = threads; }

int orc_job_set_config(orc_job* j, const rpd_config* cfg) {
    rpd_config c = *cfg;
    c.image_width = j->w;
    c.image_height = j->h;
    c.rpf_tile_size = j->support;
    const int st = orc_config_validate(&c, NULL, 0);
    if (st != RPD_OK) return st;
    j->cfg = c;
    return RPD_OK;
}

int orc_job_begin_frame(orc_job* j) {
    const size_t np = j->np, nn = j->nn;
    memset(j->stats, 0, np * sizeof(pstats));
    memset(j->hit_count, 0, np * 4);
    memset(j->sample_count, 0, np * 4);
    memset(j->radiance, 0, np * 3 * sizeof(float));
    memset(j->normal, 0, np * 3 * sizeof(float));
    memset(j->albedo, 0, np * 3 * sizeof(float));
    memset(j->depth, 0, np * sizeof(float));
    memset(j->grid, 0, nn * NDEP * DSTRIDE * sizeof(double));
    for (int f = 0; f < N_FIELDS; ++f) memset(j->node[f], 0, nn * sizeof(float));
    memset(j->sens_confidence, 0, np * sizeof(float));
    memset(j->sens_gradient, 0, np * sizeof(float));
    memset(j->uncertainty, 0, np * sizeof(float));
    memset(j->alpha, 0, np * sizeof(float));
    memset(j->var_total, 0, np * sizeof(float));
    memset(j->var_eff, 0, np * sizeof(float));
    memset(j->var_ratio, 0, np * sizeof(float));
    memset(j->variance_denoised, 0, np * sizeof(float));
    memset(j->adaptive_importance, 0, np * sizeof(float));
    memset(j->denoised, 0, np * 3 * sizeof(float));
    free_pass_grids(j);
    j->features_valid = 0;
    j->cache_valid = 0;
    return RPD_OK;
}

/* ---- per-sample accumulation -------------------------------------------------------- */

/* accumulate_sample (core/stats.h:25-41) */
static void accumulate_sample(pstats* s, const float L[3]) {
    const float lum = calc_luminance(L[0], L[1], L[2]);
    const float delta = lum - s->mean;
    s->n += 1;
    s->mean += delta / (float)s->n;
    const float delta2 = lum - s->mean;
    s->square_diff += delta * delta2;
    for (int c = 0; c < 3; ++c) {
        const float cd = L[c] - s->color_mean[c];
        s->color_mean[c] += cd / (float)s->n;
    }
    for (int c = 0; c < 3; ++c) {
        const float sc = sqrtf(fmaxs(0.0f, L[c]));
        const float sd = sc - s->sqrt_mean[c];
        s->sqrt_mean[c] += sd / (float)s->n;
        s->sqrt_sq[c] += sd * (sc - s->sqrt_mean[c]);
    }
}

/* BinnedDependency::add (core/stats.h:102-113) */
static inline void dep_add(double* d, int bins, int bin, float y, float w) {
    if (w <= EPS_SMALL) return;
    const int b = iclamps(bin, 0, bins - 1);
    const double wd = (double)w;
    const double yd = (double)y;
    d[b] += wd;
    d[16 + b] += wd * yd;
    d[32] += wd;
    d[33] += wd * wd;
    d[34] += wd * yd;
    d[35] += wd * yd * yd;
}

/* Dependency2D::add (core/stats.h:165-169) */
static inline void dep2d_add(double* d, float u, float v, float y, float w) {
    const int x = iclamps((int)(u * 4.0f), 0, 3);
    const int z = iclamps((int)(v * 4.0f), 0, 3);
    dep_add(d, 16, z * 4 + x, y, w);
}

typedef struct {
    uint8_t flags, category;
    float pu[2], lu[2], bu[2], liu[2], eu[2];
} rsample;

static inline rsample read_rsample(const rpd_sample_soa* s, int64_t k) {
    rsample r;
    uint8_t f = s->flags ? s->flags[k] : 0;
    if (!s->pixel_u[0]) f &= (uint8_t)~RPD_SAMPLE_PIXEL_VALID;
    if (!s->lens_u[0]) f &= (uint8_t)~RPD_SAMPLE_LENS_VALID;
    if (!s->brdf_u[0]) f &= (uint8_t)~RPD_SAMPLE_BRDF_VALID;
    if (!s->light_u[0]) f &= (uint8_t)~RPD_SAMPLE_LIGHT_VALID;
    if (!s->env_u[0]) f &= (uint8_t)~RPD_SAMPLE_ENV_VALID;
    r.flags = f;
    r.category = s->category ? s->category[k] : 0;
    r.pu[0] = (f & RPD_SAMPLE_PIXEL_VALID) ? s->pixel_u[0][k] : 0.0f;
    r.pu[1] = (f & RPD_SAMPLE_PIXEL_VALID) ? s->pixel_u[1][k] : 0.0f;
    r.lu[0] = (f & RPD_SAMPLE_LENS_VALID) ? s->lens_u[0][k] : 0.0f;
    r.lu[1] = (f & RPD_SAMPLE_LENS_VALID) ? s->lens_u[1][k] : 0.0f;
    r.bu[0] = (f & RPD_SAMPLE_BRDF_VALID) ? s->brdf_u[0][k] : 0.0f;
    r.bu[1] = (f & RPD_SAMPLE_BRDF_VALID) ? s->brdf_u[1][k] : 0.0f;
    r.liu[0] = (f & RPD_SAMPLE_LIGHT_VALID) ? s->light_u[0][k] : 0.0f;
    r.liu[1] = (f & RPD_SAMPLE_LIGHT_VALID) ? s->light_u[1][k] : 0.0f;
    r.eu[0] = (f & RPD_SAMPLE_ENV_VALID) ? s->env_u[0][k] : 0.0f;
    r.eu[1] = (f & RPD_SAMPLE_ENV_VALID) ? s->env_u[1][k] : 0.0f;
    return r;
}

/* accumulate_rpf_sample_to_grid (main.cpp:329-376) */
static void accumulate_rpf_sample_to_grid(const orc_job* j, double* grid, int x, int y, const rsample* s, float lum) {
    const uint8_t f = s->flags;
    const int pixel_valid = (f & RPD_SAMPLE_PIXEL_VALID) != 0;
    const int lens_valid = (f & RPD_SAMPLE_LENS_VALID) != 0;
    const int shading = (f & (RPD_SAMPLE_LIGHT_SELECT_VALID | RPD_SAMPLE_BRDF_VALID | RPD_SAMPLE_LIGHT_VALID |
                              RPD_SAMPLE_ENV_VALID | RPD_SAMPLE_RR_VALID)) != 0;
    if (!pixel_valid && !lens_valid && !shading) return;
    const float gx = (float)x / (float)j->step;
    const float gy = (float)y / (float)j->step;
    const int x0 = iclamps((int)floorf(gx), 0, j->nodes_x - 1);
    const int y0 = iclamps((int)floorf(gy), 0, j->nodes_y - 1);
    const int x1 = imins(x0 + 1, j->nodes_x - 1);
    const int y1 = imins(y0 + 1, j->nodes_y - 1);
    const float tx = fclamps(gx - (float)x0, 0.0f, 1.0f);
    const float ty = fclamps(gy - (float)y0, 0.0f, 1.0f);
    const int nxs[4] = {x0, x1, x0, x1};
    const int nys[4] = {y0, y0, y1, y1};
    const float ws[4] = {(1.0f - tx) * (1.0f - ty), tx * (1.0f - ty), (1.0f - tx) * ty, tx * ty};
    for (int e = 0; e < 4; ++e) {
        const float w = ws[e];
        if (w <= EPS_SMALL) continue;
        double* node = grid + ((size_t)nys[e] * j->nodes_x + nxs[e]) * NDEP * DSTRIDE;
        if (pixel_valid) {
            const float half_support = 0.5f * (float)j->support;
            const float support_left = (float)(nxs[e] * j->step) - half_support;
            const float support_top = (float)(nys[e] * j->step) - half_support;
            const float su = fclamps(((float)x + s->pu[0] - support_left) / (float)j->support, 0.0f, 1.0f);
            const float sv = fclamps(((float)y + s->pu[1] - support_top) / (float)j->support, 0.0f, 1.0f);
            dep2d_add(node + D_PIXEL * DSTRIDE, su, sv, lum, w);
            if (f & RPD_SAMPLE_BRDF_VALID) dep2d_add(node + D_SCREEN_BRDF * DSTRIDE, su, sv, lum, w);
            if (f & RPD_SAMPLE_LENS_VALID) dep2d_add(node + D_SCREEN_LENS * DSTRIDE, su, sv, lum, w);
            if (f & RPD_SAMPLE_LIGHT_VALID) dep2d_add(node + D_SCREEN_LIGHT_UV * DSTRIDE, su, sv, lum, w);
            if (f & RPD_SAMPLE_LIGHT_SELECT_VALID) dep2d_add(node + D_SCREEN_LIGHT_SELECT * DSTRIDE, su, sv, lum, w);
            if (f & RPD_SAMPLE_ENV_VALID) dep2d_add(node + D_SCREEN_ENV * DSTRIDE, su, sv, lum, w);
            if (f & RPD_SAMPLE_RR_VALID) dep2d_add(node + D_SCREEN_RR * DSTRIDE, su, sv, lum, w);
        }
        if (f & RPD_SAMPLE_LENS_VALID) dep2d_add(node + D_LENS * DSTRIDE, s->lu[0], s->lu[1], lum, w);
        if (f & RPD_SAMPLE_BRDF_VALID) dep2d_add(node + D_BRDF * DSTRIDE, s->bu[0], s->bu[1], lum, w);
        if (f & RPD_SAMPLE_LIGHT_VALID) dep2d_add(node + D_LIGHT_UV * DSTRIDE, s->liu[0], s->liu[1], lum, w);
        if (f & RPD_SAMPLE_ENV_VALID) dep2d_add(node + D_ENV * DSTRIDE, s->eu[0], s->eu[1], lum, w);
        if (f & RPD_SAMPLE_LIGHT_SELECT_VALID)
            dep_add(node + D_LIGHT_SELECT * DSTRIDE, 16, (int)(s->category & RPD_CATEGORY_LIGHT_INDEX_MASK), lum, w);
        if (f & RPD_SAMPLE_RR_VALID)
            dep_add(node + D_RR * DSTRIDE, 2, (s->category & RPD_CATEGORY_RR_SURVIVED) ? 1 : 0, lum, w);
    }
}

static int nthreads_now(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* The render loops' per-sample bookkeeping (main.cpp:572-576, 706-717, 1509-1518), with
 * rows split into static blocks per thread (the reference uses dynamic,1 over rows). */
int orc_job_push_samples(orc_job* j, const rpd_sample_soa* s, int64_t first, int64_t count, int32_t spp,
                         const int32_t* counts) {
    if (first < 0 || count < 0 || first + count > (int64_t)j->np) return RPD_ERR_INVALID_ARGUMENT;
    if (count == 0) return RPD_OK;
    const double t0 = now_ms();
    set_omp(j->threads);
    const int capture_rpd = j->cfg.rpf_shrinkage_scale > 0.0f;
    const int nt = nthreads_now();
    const size_t gsize = j->nn * NDEP * DSTRIDE * sizeof(double);
    if (capture_rpd && j->n_pass_grids != nt) {
        free_pass_grids(j);
        j->pass_grids = (double**)zalloc(sizeof(double*) * (size_t)nt);
        for (int i = 0; i < nt; ++i) j->pass_grids[i] = (double*)zalloc(gsize);
        j->n_pass_grids = nt;
    }
    int64_t* offset = (int64_t*)malloc(sizeof(int64_t) * (size_t)(count + 1));
    offset[0] = 0;
    for (int64_t i = 0; i < count; ++i) offset[i + 1] = offset[i] + (counts ? counts[i] : spp);
    const int64_t row_first = first / j->w;
    const int64_t row_last = (first + count - 1) / j->w;
    const int64_t rows = row_last - row_first + 1;
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
#ifdef _OPENMP
        const int tid = omp_get_thread_num();
        const int tn = omp_get_num_threads();
#else
        const int tid = 0, tn = 1;
#endif
        const int64_t r0 = row_first + rows * tid / tn;
        const int64_t r1 = row_first + rows * (tid + 1) / tn;
        double* grid = capture_rpd ? j->pass_grids[tid] : NULL;
        for (int64_t row = r0; row < r1; ++row) {
            const int y = (int)row;
            for (int x = 0; x < j->w; ++x) {
                const int64_t idx = (int64_t)y * j->w + x;
                if (idx < first || idx >= first + count) continue;
                const int64_t local = idx - first;
                for (int64_t k = offset[local]; k < offset[local + 1]; ++k) {
                    const uint8_t f = s->flags ? s->flags[k] : 0;
                    if (f & RPD_SAMPLE_HIT) {
                        j->hit_count[idx]++;
                        for (int c = 0; c < 3; ++c) j->normal[3 * idx + c] += s->normal[c][k];
                        for (int c = 0; c < 3; ++c)
                            j->albedo[3 * idx + c] += s->albedo[0] ? s->albedo[c][k] : s->pixel_albedo[c][local];
                        j->depth[idx] += s->depth[k];
                    }
                    const float L[3] = {s->radiance[0][k], s->radiance[1][k], s->radiance[2][k]};
                    if (!isfinite(L[0]) || !isfinite(L[1]) || !isfinite(L[2])) continue;
                    if (capture_rpd) {
                        const rsample rs = read_rsample(s, k);
                        accumulate_rpf_sample_to_grid(j, grid, x, y, &rs, calc_luminance(L[0], L[1], L[2]));
                    }
                    accumulate_sample(&j->stats[idx], L);
                    for (int c = 0; c < 3; ++c) j->radiance[3 * idx + c] += L[c];
                    j->sample_count[idx]++;
                }
            }
        }
    }
    free(offset);
    j->stage_ms[RPD_STAGE_ACCUMULATE] = now_ms() - t0;
    return RPD_OK;
}

/* merge_rpf_grids_into (main.cpp:378-388) + invalidate_postprocess_caches (main.cpp:1533) */
int orc_job_end_pass(orc_job* j) {
    const double t0 = now_ms();
    set_omp(j->threads);
    if (j->n_pass_grids > 0) {
        const int64_t total = (int64_t)(j->nn * NDEP * DSTRIDE);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t nidx = 0; nidx < (int64_t)j->nn; ++nidx) {
            double* dst = j->grid + nidx * NDEP * DSTRIDE;
            for (int t = 0; t < j->n_pass_grids; ++t) {
                const double* src = j->pass_grids[t] + nidx * NDEP * DSTRIDE;
                for (int d = 0; d < NDEP; ++d) {
                    /* BinnedDependency::merge (core/stats.h:149-158) */
                    double* a = dst + d * DSTRIDE;
                    const double* b = src + d * DSTRIDE;
                    for (int bin = 0; bin < dep_bins[d]; ++bin) {
                        a[bin] += b[bin];
                        a[16 + bin] += b[16 + bin];
                    }
                    a[32] += b[32];
                    a[33] += b[33];
                    a[34] += b[34];
                    a[35] += b[35];
                }
            }
        }
        (void)total;
        free_pass_grids(j);
    }
    j->features_valid = 0;
    j->cache_valid = 0;
    j->stage_ms[RPD_STAGE_ACCUMULATE] += now_ms() - t0;
    return RPD_OK;
}

/* ---- caches (main.cpp:94-154) ------------------------------------------------------- */

static void ensure_feature_cache(orc_job* j) {
    if (j->features_valid) return;
    const int64_t np = (int64_t)j->np;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < np; ++i) {
        if (j->hit_count[i] > 0) {
            const float hc = (float)j->hit_count[i];
            float n[3] = {j->normal[3 * i] / hc, j->normal[3 * i + 1] / hc, j->normal[3 * i + 2] / hc};
            if (dot3(n, n) > EPS_SMALL) normalize3(n);
            for (int c = 0; c < 3; ++c) j->f_normal[3 * i + c] = n[c];
            j->f_depth[i] = j->depth[i] / hc;
            for (int c = 0; c < 3; ++c) j->f_albedo[3 * i + c] = j->albedo[3 * i + c] / hc;
        } else {
            for (int c = 0; c < 3; ++c) j->f_normal[3 * i + c] = j->normal[3 * i + c];
            j->f_depth[i] = j->depth[i];
            for (int c = 0; c < 3; ++c) j->f_albedo[3 * i + c] = j->albedo[3 * i + c];
        }
    }
    j->features_valid = 1;
}

/* SensitivityTiles::lookup (core/buffers.h:68-87) */
static inline float tiles_lookup(const orc_job* j, const float* tiles, int64_t idx) {
    const int y = (int)(idx / j->w);
    const int x = (int)(idx - (int64_t)y * j->w);
    const float gx = (float)x / (float)j->step;
    const float gy = (float)y / (float)j->step;
    const int x0 = iclamps((int)floorf(gx), 0, j->nodes_x - 1);
    const int y0 = iclamps((int)floorf(gy), 0, j->nodes_y - 1);
    const int x1 = imins(x0 + 1, j->nodes_x - 1);
    const int y1 = imins(y0 + 1, j->nodes_y - 1);
    const float tx = fclamps(gx - (float)x0, 0.0f, 1.0f);
    const float ty = fclamps(gy - (float)y0, 0.0f, 1.0f);
    const float v00 = tiles[(size_t)y0 * j->nodes_x + x0];
    const float v10 = tiles[(size_t)y0 * j->nodes_x + x1];
    const float v01 = tiles[(size_t)y1 * j->nodes_x + x0];
    const float v11 = tiles[(size_t)y1 * j->nodes_x + x1];
    const float top = lerp_std(v00, v10, tx);
    const float bottom = lerp_std(v01, v11, tx);
    return lerp_std(top, bottom, ty);
}

/* SensitivityTiles::expand_values (core/buffers.h:89-101) */
static void expand_values(const orc_job* j, const float* tiles, float* out) {
    const int64_t np = (int64_t)j->np;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < np; ++i) out[i] = tiles_lookup(j, tiles, i);
}

static void ensure_sensitivity_cache(orc_job* j) {
    if (j->cache_valid) return;
    for (int f = 0; f < C_GRADIENT; ++f) expand_values(j, j->node[cache_from_node[f]], j->cache[f]);
    memcpy(j->cache[C_GRADIENT], j->sens_gradient, j->np * sizeof(float));
    j->cache_valid = 1;
}

/* main.cpp:156-169 */
static float sample_scalar_local_average(const float* v, int w, int h, int cx, int cy, int radius) {
    double accum = 0.0, weight_sum = 0.0;
    for (int dy = -radius; dy <= radius; ++dy) {
        const int y = iclamps(cy + dy, 0, h - 1);
        for (int dx = -radius; dx <= radius; ++dx) {
            const int x = iclamps(cx + dx, 0, w - 1);
            const double weight = 1.0 / (1.0 + (double)(dx * dx + dy * dy));
            accum += weight * (double)v[(size_t)y * w + x];
            weight_sum += weight;
        }
    }
    return (weight_sum > 0.0) ? (float)(accum / weight_sum) : 0.0f;
}

/* main.cpp:171-185 */
static void sample_vec3_local_average(const float* v, int w, int h, int cx, int cy, int radius, float out[3]) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, weight_sum = 0.0;
    for (int dy = -radius; dy <= radius; ++dy) {
        const int y = iclamps(cy + dy, 0, h - 1);
        for (int dx = -radius; dx <= radius; ++dx) {
            const int x = iclamps(cx + dx, 0, w - 1);
            const double weight = 1.0 / (1.0 + (double)(dx * dx + dy * dy));
            const float* p = v + 3 * ((size_t)y * w + x);
            a0 += (double)p[0] * weight;
            a1 += (double)p[1] * weight;
            a2 += (double)p[2] * weight;
            weight_sum += weight;
        }
    }
    if (weight_sum <= 0.0) { out[0] = out[1] = out[2] = 0.0f; return; }
    out[0] = (float)(a0 / weight_sum);
    out[1] = (float)(a1 / weight_sum);
    out[2] = (float)(a2 / weight_sum);
}

/* ---- recompute_sensitivity (main.cpp:741-953) ---------------------------------------- */

/* BinnedDependency::sample_mass / compute_sensitivity (core/stats.h:115-141) */
static double sample_mass(const double* d) { return d[33] > 0.0 ? d[32] * d[32] / d[33] : 0.0; }

static float compute_sensitivity(const double* d, int bins) {
    const double kEps = 1e-18;
    const double effective_n = sample_mass(d);
    if (effective_n <= 2.0) return 0.0f;
    const double mean = d[34] / d[32];
    const double total = d[35] - d[32] * mean * mean;
    if (total <= kEps) return 0.0f;
    int active = 0;
    double between = 0.0;
    for (int b = 0; b < bins; ++b) {
        if (d[b] <= kEps) continue;
        ++active;
        const double delta = d[16 + b] / d[b] - mean;
        between += d[b] * delta * delta;
    }
    if (active < 2 || effective_n <= (double)active) return 0.0f;
    const double eta2 = dclamps(between / total, 0.0, 1.0);
    const double adjusted = dmaxs(0.0, 1.0 - (1.0 - eta2) * (effective_n - 1.0) / (effective_n - active));
    return (float)sqrt(adjusted);
}

/* Order in which main.cpp:779-806 reads the Tile dependencies:
 * raw/conf for pixel, brdf, lens, light_uv, light_select, environment, rr and the six
 * screen comparators (screen_brdf, screen_lens, screen_light_uv, screen_light_select,
 * screen_environment, screen_rr). */
enum { R_PIXEL = 0, R_BRDF, R_LENS, R_LIGHT_UV, R_LIGHT_SELECT, R_ENV, R_RR,
       R_S_BRDF, R_S_LENS, R_S_LIGHT_UV, R_S_LIGHT_SELECT, R_S_ENV, R_S_RR, R_FIELDS };
static const int raw_dep[R_FIELDS] = {D_PIXEL, D_BRDF, D_LENS, D_LIGHT_UV, D_LIGHT_SELECT, D_ENV, D_RR,
                                      D_SCREEN_BRDF, D_SCREEN_LENS, D_SCREEN_LIGHT_UV,
                                      D_SCREEN_LIGHT_SELECT, D_SCREEN_ENV, D_SCREEN_RR};

int orc_recompute_sensitivity(orc_job* j) {
    const double t0 = now_ms();
    set_omp(j->threads);
    const int w = j->w, h = j->h, nx = j->nodes_x, ny = j->nodes_y, step = j->step;
    const int64_t nn = (int64_t)j->nn, np = (int64_t)j->np;
    j->cache_valid = 0;
    if (j->cfg.rpf_shrinkage_scale <= 0.0f) {
        memset(j->sens_confidence, 0, j->np * sizeof(float));
        memset(j->sens_gradient, 0, j->np * sizeof(float));
        ensure_sensitivity_cache(j);
        j->stage_ms[RPD_STAGE_SENSITIVITY] = now_ms() - t0;
        return RPD_OK;
    }
    ensure_feature_cache(j);
    float* raw[R_FIELDS];
    float* conf[R_FIELDS];
    float* prior[R_FIELDS];
    for (int f = 0; f < R_FIELDS; ++f) {
        raw[f] = (float*)zalloc((size_t)nn * sizeof(float));
        conf[f] = (float*)zalloc((size_t)nn * sizeof(float));
        prior[f] = (float*)zalloc((size_t)nn * sizeof(float));
    }
    float* nnorm = (float*)zalloc((size_t)nn * 3 * sizeof(float));
    float* ndepth = (float*)zalloc((size_t)nn * sizeof(float));
    float* nalb = (float*)zalloc((size_t)nn * 3 * sizeof(float));
    const double n0d = (double)j->cfg.rpf_confidence_samples;

    /* main.cpp:773-815 */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t idx = 0; idx < nn; ++idx) {
        const int ix = (int)(idx % nx), iy = (int)(idx / nx);
        const double* tile = j->grid + idx * NDEP * DSTRIDE;
        for (int f = 0; f < R_FIELDS; ++f) {
            const double* d = tile + raw_dep[f] * DSTRIDE;
            raw[f][idx] = compute_sensitivity(d, dep_bins[raw_dep[f]]);
            const double mass = sample_mass(d);
            conf[f][idx] = (float)(mass / (mass + n0d));
        }
        const int px = iclamps(ix * step, 0, w - 1);
        const int py = iclamps(iy * step, 0, h - 1);
        sample_vec3_local_average(j->f_normal, w, h, px, py, 1, nnorm + 3 * idx);
        if (dot3(nnorm + 3 * idx, nnorm + 3 * idx) > EPS_SMALL) normalize3(nnorm + 3 * idx);
        ndepth[idx] = sample_scalar_local_average(j->f_depth, w, h, px, py, 1);
        sample_vec3_local_average(j->f_albedo, w, h, px, py, 1, nalb + 3 * idx);
    }

    /* prior_smooth (main.cpp:817-851), applied to each of the 13 fields (853-863) */
    for (int f = 0; f < R_FIELDS; ++f) {
        const float* rv = raw[f];
        const float* cv = conf[f];
        float* pv = prior[f];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t idx = 0; idx < nn; ++idx) {
            const int ix = (int)(idx % nx), iy = (int)(idx / nx);
            double weight_sum = 0.0, accum = 0.0;
            for (int dy = -1; dy <= 1; ++dy) {
                const int sy = iy + dy;
                if (sy < 0 || sy >= ny) continue;
                for (int dx = -1; dx <= 1; ++dx) {
                    const int sx = ix + dx;
                    if (sx < 0 || sx >= nx) continue;
                    const int64_t sidx = (int64_t)sy * nx + sx;
                    const float spatial_w = 1.0f / (1.0f + (float)(dx * dx + dy * dy));
                    const float normal_w = fclamps((dot3(nnorm + 3 * idx, nnorm + 3 * sidx) + 1.0f) * 0.5f, 0.0f, 1.0f);
                    const float depth_w = expf(-4.0f * relative_depth_delta(ndepth[idx], ndepth[sidx]));
                    const float da[3] = {nalb[3 * idx] - nalb[3 * sidx], nalb[3 * idx + 1] - nalb[3 * sidx + 1],
                                         nalb[3 * idx + 2] - nalb[3 * sidx + 2]};
                    const float albedo_w = expf(-2.5f * norm3(da));
                    const double w_neighbor = (double)spatial_w * (double)normal_w * (double)depth_w *
                                              (double)albedo_w * (double)fmaxs(0.05f, cv[sidx]);
                    accum += w_neighbor * (double)rv[sidx];
                    weight_sum += w_neighbor;
                }
            }
            pv[idx] = (weight_sum > (double)EPS_SMALL) ? (float)(accum / weight_sum) : rv[idx];
        }
    }

    /* main.cpp:865-928 */
    float** T = j->node;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t idx = 0; idx < nn; ++idx) {
        float fin[7];
        for (int f = 0; f < 7; ++f) fin[f] = lerp_std(prior[f][idx], raw[f][idx], conf[f][idx]);
        float screen[6];
        for (int c = 0; c < 6; ++c) screen[c] = lerp_std(prior[7 + c][idx], raw[7 + c][idx], conf[7 + c][idx]);
        T[N_PIXEL][idx] = fclamps(fin[R_PIXEL], 0.0f, 1.0f);
        T[N_BRDF][idx] = fclamps(fin[R_BRDF], 0.0f, 1.0f);
        T[N_LENS][idx] = fclamps(fin[R_LENS], 0.0f, 1.0f);
        T[N_LIGHT_UV][idx] = fclamps(fin[R_LIGHT_UV], 0.0f, 1.0f);
        T[N_LIGHT_SELECT][idx] = fclamps(fin[R_LIGHT_SELECT], 0.0f, 1.0f);
        T[N_ENV][idx] = fclamps(fin[R_ENV], 0.0f, 1.0f);
        T[N_RR][idx] = fclamps(fin[R_RR], 0.0f, 1.0f);
        T[N_PIXEL_CONF][idx] = fclamps(conf[R_PIXEL][idx], 0.0f, 1.0f);
        T[N_BRDF_CONF][idx] = fclamps(conf[R_BRDF][idx], 0.0f, 1.0f);
        T[N_LENS_CONF][idx] = fclamps(conf[R_LENS][idx], 0.0f, 1.0f);
        T[N_LIGHT_UV_CONF][idx] = fclamps(conf[R_LIGHT_UV][idx], 0.0f, 1.0f);
        T[N_LIGHT_SELECT_CONF][idx] = fclamps(conf[R_LIGHT_SELECT][idx], 0.0f, 1.0f);
        T[N_ENV_CONF][idx] = fclamps(conf[R_ENV][idx], 0.0f, 1.0f);
        T[N_RR_CONF][idx] = fclamps(conf[R_RR][idx], 0.0f, 1.0f);
        const float rnd[6] = {T[N_BRDF][idx], T[N_LENS][idx], T[N_LIGHT_UV][idx], T[N_LIGHT_SELECT][idx],
                              T[N_ENV][idx], T[N_RR][idx]};
        const float rc[6] = {T[N_BRDF_CONF][idx], T[N_LENS_CONF][idx], T[N_LIGHT_UV_CONF][idx],
                             T[N_LIGHT_SELECT_CONF][idx], T[N_ENV_CONF][idx], T[N_RR_CONF][idx]};
        float rel[6];
        for (int c = 0; c < 6; ++c) {
            /* rpf::relative_random_sensitivity (core/stats.h:48-50) */
            const float relative = rnd[c] / fmaxs(EPS_SMALL, rnd[c] + screen[c]);
            rel[c] = relative * fmins(rc[c], conf[7 + c][idx]);
        }
        int dominant = 0;
        for (int c = 1; c < 6; ++c) if (rel[dominant] < rel[c]) dominant = c;
        T[N_BRDF][idx] = rel[0];
        T[N_LENS][idx] = rel[1];
        T[N_LIGHT_UV][idx] = rel[2];
        T[N_LIGHT_SELECT][idx] = rel[3];
        T[N_LIGHT][idx] = fmaxs(rel[2], rel[3]);
        T[N_ENV][idx] = rel[4];
        T[N_RR][idx] = rel[5];
        T[N_LIGHT_CONF][idx] = rel[2] >= rel[3] ? rc[2] : rc[3];
        T[N_ALL][idx] = rel[dominant];
        T[N_ALL_CONF][idx] = fmins(rc[dominant], conf[7 + dominant][idx]);
    }

    /* main.cpp:930-947 */
    float* expanded = (float*)zalloc((size_t)np * sizeof(float));
    expand_values(j, T[N_ALL], expanded);
    expand_values(j, T[N_ALL_CONF], j->sens_confidence);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < np; ++i) {
        const int y = (int)(i / w), x = (int)(i % w);
        const float left = expanded[(size_t)y * w + imaxs(0, x - 1)];
        const float right = expanded[(size_t)y * w + imins(w - 1, x + 1)];
        const float up = expanded[(size_t)imaxs(0, y - 1) * w + x];
        const float down = expanded[(size_t)imins(h - 1, y + 1) * w + x];
        const float grad = sqrtf((right - left) * (right - left) + (down - up) * (down - up));
        j->sens_gradient[i] = fclamps(0.5f * grad, 0.0f, 1.0f);
    }
    free(expanded);
    ensure_sensitivity_cache(j);

    for (int f = 0; f < R_FIELDS; ++f) { free(raw[f]); free(conf[f]); free(prior[f]); }
    free(nnorm); free(ndepth); free(nalb);
    j->stage_ms[RPD_STAGE_SENSITIVITY] = now_ms() - t0;
    return RPD_OK;
}

/* ---- statmc_denoise (main.cpp:957-1162) ---------------------------------------------- */

/* lookup_t_critical (main.cpp:188-231) */
static const float t05_table[30] = {
    12.706f, 4.303f, 3.182f, 2.776f, 2.571f, 2.447f, 2.365f, 2.306f, 2.262f, 2.228f,
    2.201f, 2.179f, 2.160f, 2.145f, 2.131f, 2.120f, 2.110f, 2.101f, 2.093f, 2.086f,
    2.080f, 2.074f, 2.069f, 2.064f, 2.060f, 2.056f, 2.052f, 2.048f, 2.045f, 2.042f};
static const float t01_table[30] = {
    63.657f, 9.925f, 5.841f, 4.604f, 4.032f, 3.707f, 3.499f, 3.355f, 3.250f, 3.169f,
    3.106f, 3.055f, 3.012f, 2.977f, 2.947f, 2.921f, 2.898f, 2.878f, 2.861f, 2.845f,
    2.831f, 2.819f, 2.807f, 2.797f, 2.787f, 2.779f, 2.771f, 2.763f, 2.756f, 2.750f};

static float interpolate_table(const float* table, float df) {
    const int lo = iclamps((int)floorf(df), 1, 30);
    const int hi = iclamps((int)ceilf(df), 1, 30);
    if (lo == hi) return table[lo - 1];
    return lerp_std(table[lo - 1], table[hi - 1], (df - (float)lo) / (float)(hi - lo));
}

static float lookup_t_critical(float df, float alpha) {
    df = fmaxs(df, 1.0f);
    alpha = fclamps(alpha, EPS_SMALL, 0.999999f);
    if (df < 30.5f && fabsf(alpha - 0.05f) < EPS_F) return interpolate_table(t05_table, df);
    if (df < 30.5f && fabsf(alpha - 0.01f) < EPS_F) return interpolate_table(t01_table, df);
    float z;
    if (alpha <= 0.001f) z = 3.29f;
    else if (alpha <= 0.005f) z = 2.81f;
    else if (alpha <= 0.01f) z = 2.58f;
    else if (alpha <= 0.02f) z = 2.33f;
    else if (alpha <= 0.05f) z = 1.96f;
    else if (alpha <= 0.10f) z = 1.64f;
    else z = 1.28f;
    if (df < 30.0f) {
        const float adj = sqrtf(df / fmaxs(1.0f, df - 1.0f));
        z *= adj;
    }
    return z;
}

/* sample_sensitivity + components_denoise (main.cpp:297-327) */
static void rpd_components(const orc_job* j, int64_t idx, float out[6]) {
    const float* const* C = (const float* const*)j->cache;
    const float comps[6] = {fclamps(C[C_BRDF][idx], 0.0f, 1.0f), fclamps(C[C_LENS][idx], 0.0f, 1.0f),
                            fclamps(C[C_LIGHT_UV][idx], 0.0f, 1.0f), fclamps(C[C_LIGHT_SELECT][idx], 0.0f, 1.0f),
                            fclamps(C[C_ENV][idx], 0.0f, 1.0f), fclamps(C[C_RR][idx], 0.0f, 1.0f)};
    const float gradient = fclamps(C[C_GRADIENT][idx], 0.0f, 1.0f);
    const float attenuation = 1.0f - gradient;
    for (int c = 0; c < 6; ++c) out[c] = fclamps(comps[c] * attenuation, 0.0f, 1.0f);
}

static inline float pixel_variance(const pstats* s) {    /* core/stats.h:14-16 */
    return (s->n > 1) ? s->square_diff / (float)(s->n - 1) : 0.0f;
}

int orc_statmc_denoise(orc_job* j) {
    const double t0 = now_ms();
    set_omp(j->threads);
    const int w = j->w, h = j->h, r = j->cfg.color_window_radius;
    const float normal_threshold = j->cfg.color_normal_threshold;
    const float depth_threshold = j->cfg.color_depth_threshold;
    const float rpd_scale = j->cfg.rpf_shrinkage_scale;
    const float alpha_cfg = j->cfg.color_compat_alpha;
    const int64_t np = (int64_t)j->np;
    ensure_feature_cache(j);
    ensure_sensitivity_cache(j);
    float* svm = (float*)zalloc((size_t)np * 3 * sizeof(float));  /* sqrt_variance_mean */
    float* svs = j->sqrt_var_stable;  /* sqrt_variance_stable, kept for reads */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < np; ++i) {
        const pstats* s = &j->stats[i];
        for (int c = 0; c < 3; ++c) {
            const float var = (s->n <= 1) ? 0.0f : s->sqrt_sq[c] / (float)(s->n - 1);
            svm[3 * i + c] = fmaxs(var / (float)imaxs(1, s->n), EPS_SMALL);
        }
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < np; ++i) {
        float avg[3];
        sample_vec3_local_average(svm, w, h, (int)(i % w), (int)(i / w), 1, avg);
        for (int c = 0; c < 3; ++c) svs[3 * i + c] = fmaxs(svm[3 * i + c], avg[c]);
    }
    const float var2_max = j->cfg.color_sigma_max * j->cfg.color_sigma_max;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t idx = 0; idx < np; ++idx) {
        const int y = (int)(idx / w), x = (int)(idx % w);
        const pstats* si = &j->stats[idx];
        if (j->hit_count[idx] == 0) {
            for (int c = 0; c < 3; ++c) j->denoised[3 * idx + c] = si->color_mean[c];
            j->uncertainty[idx] = pixel_variance(si) / (float)imaxs(1, si->n);
            j->alpha[idx] = 1.0f;
            continue;
        }
        const float* normal_i = j->f_normal + 3 * idx;
        const float depth_i = j->f_depth[idx];
        float var_i = pixel_variance(si);
        if (!isfinite(var_i)) var_i = EPS_SMALL;
        var_i = fclamps(var_i, EPS_SMALL, var2_max);
        const int n_i = imaxs(1, si->n);
        float rpd_i[6];
        rpd_components(j, idx, rpd_i);
        const float var_mean_i = fmaxs(EPS_SMALL, var_i / (float)n_i);
        const float* sqrt_mean_i = si->sqrt_mean;
        const float* svi = svs + 3 * idx;
        j->var_total[idx] = var_i;
        j->var_eff[idx] = var_mean_i;
        j->var_ratio[idx] = (var_i > EPS_SMALL) ? (var_mean_i * (float)n_i) / var_i : 0.0f;

        double weight_sum = 0.0, weight_square_sum = 0.0, weighted_variance_sum = 0.0;
        double cs0 = 0.0, cs1 = 0.0, cs2 = 0.0, accepted = 0.0;
        const double center_weight = 1.0;
        for (int dy = -r; dy <= r; ++dy) {
            const int yy = y + dy;
            if (yy < 0 || yy >= h) continue;
            for (int dx = -r; dx <= r; ++dx) {
                const int xx = x + dx;
                if (xx < 0 || xx >= w) continue;
                const int64_t jn = (int64_t)yy * w + xx;
                if (j->hit_count[jn] == 0) continue;
                if (dot3(normal_i, j->f_normal + 3 * jn) < normal_threshold) continue;
                const float depth_delta = relative_depth_delta(depth_i, j->f_depth[jn]);
                if (depth_delta > depth_threshold) continue;
                const float* ai = j->f_albedo + 3 * idx;
                const float* aj = j->f_albedo + 3 * jn;
                const float da[3] = {ai[0] - aj[0], ai[1] - aj[1], ai[2] - aj[2]};
                if (norm3(da) > BASE_ALBEDO_THRESH) continue;
                const pstats* sj = &j->stats[jn];
                float var_j = pixel_variance(sj);
                if (!isfinite(var_j)) var_j = EPS_SMALL;
                var_j = fclamps(var_j, EPS_SMALL, var2_max);
                const int n_j = imaxs(1, sj->n);
                const float var_mean_j = fmaxs(EPS_SMALL, var_j / (float)n_j);
                const float* svj = svs + 3 * jn;
                double max_t2 = 0.0;
                for (int c = 0; c < 3; ++c) {
                    const double v_i = (double)svi[c];
                    const double v_j = (double)svj[c];
                    const double variance_sum = v_i + v_j;
                    const double mean_diff = (double)(sqrt_mean_i[c] - sj->sqrt_mean[c]);
                    const double t2 = mean_diff * mean_diff / dmaxs((double)EPS_SMALL, variance_sum);
                    const double denom_df = (v_i * v_i) / dmaxs((double)(n_i - 1), 1.0) +
                                            (v_j * v_j) / dmaxs((double)(n_j - 1), 1.0);
                    const double df = (denom_df > (double)EPS_SMALL) ? (variance_sum * variance_sum) / denom_df
                                                                     : (double)(n_i + n_j - 2);
                    const double t_crit = (double)lookup_t_critical((float)df, alpha_cfg);
                    max_t2 = dmaxs(max_t2, t2 / (t_crit * t_crit));
                }
                float rpd_j[6];
                rpd_components(j, jn, rpd_j);
                /* rpf::shared_reliability + relax_compatibility (core/stats.h:56-78) */
                float shared = 0.0f;
                for (int c = 0; c < 6; ++c) shared = fmaxs(shared, fmins(rpd_i[c], rpd_j[c]));
                shared = fclamps(shared, 0.0f, 1.0f);
                const float adjustment = fclamps(rpd_scale * shared, 0.0f, 1.0f);
                const double q = max_t2 / (1.0 + (double)adjustment);
                if (q > 25.0) continue;
                const double dist2 = (double)(dx * dx + dy * dy);
                const double spatial_w = 1.0 / (1.0 + dist2);
                const double weight_j = spatial_w * exp(-0.5 * q);
                cs0 += (double)sj->color_mean[0] * weight_j;
                cs1 += (double)sj->color_mean[1] * weight_j;
                cs2 += (double)sj->color_mean[2] * weight_j;
                weight_sum += weight_j;
                weight_square_sum += weight_j * weight_j;
                weighted_variance_sum += weight_j * weight_j * (double)var_mean_j;
                if ((dx != 0 || dy != 0) && weight_j > 0.05 * spatial_w) accepted += 1.0;
            }
        }
        float mean_nb[3] = {si->color_mean[0], si->color_mean[1], si->color_mean[2]};
        double var_neighbors = (double)var_mean_i;
        if (weight_sum > (double)EPS_SMALL) {
            mean_nb[0] = (float)(cs0 / weight_sum);
            mean_nb[1] = (float)(cs1 / weight_sum);
            mean_nb[2] = (float)(cs2 / weight_sum);
            var_neighbors = weighted_variance_sum / (weight_sum * weight_sum);
        }
        const double effective = weight_sum * weight_sum / dmaxs((double)EPS_SMALL, weight_square_sum);
        const double blend = (accepted >= 2.0 && weight_sum >= 1.1 * center_weight)
                                 ? dclamps(1.0 - 1.0 / sqrt(effective), 0.0, 0.8) : 0.0;
        const float alpha = (float)(1.0 - blend);
        const float fb = (float)blend;
        for (int c = 0; c < 3; ++c) j->denoised[3 * idx + c] = lerpf(si->color_mean[c], mean_nb[c], fb);
        const float uncertainty = (float)((double)alpha * (double)alpha * (double)var_mean_i +
                                          blend * blend * var_neighbors +
                                          2.0 * (double)alpha * blend *
                                              (center_weight / dmaxs(weight_sum, (double)EPS_SMALL)) *
                                              (double)var_mean_i);
        j->alpha[idx] = alpha;
        j->uncertainty[idx] = uncertainty;
    }
    free(svm);

    j->stage_ms[RPD_STAGE_STATMC] = now_ms() - t0;
    return RPD_OK;
}

/* ---- variance_denoise (main.cpp:1166-1268) ------------------------------------------- */

/* rpf::conservative_variance_update (core/stats.h:85-91) */
static inline float conservative_variance_update(float value, float neighbor, float stabilizer) {
    const float blend = fclamps(fmaxs(0.0f, neighbor - value) / fmaxs(EPS_SMALL, value + neighbor + stabilizer),
                                0.0f, 1.0f);
    return lerp_std(value, neighbor, blend);
}

int orc_variance_denoise(orc_job* j) {
    const double t0 = now_ms();
    set_omp(j->threads);
    const int w = j->w, h = j->h, radius = j->cfg.var_window_radius;
    const float normal_threshold = j->cfg.var_normal_threshold;
    const float depth_threshold = j->cfg.var_depth_threshold;
    const float compat_sigma = j->cfg.var_compat_sigma;
    const float shrinkage_k = j->cfg.var_shrinkage_k;
    const int iterations = j->cfg.var_iterations;
    const float max_variance = j->cfg.adaptive_sigma_max * j->cfg.adaptive_sigma_max;
    const int64_t np = (int64_t)j->np;
    float* curr = (float*)zalloc((size_t)np * sizeof(float));
    float* next = (float*)zalloc((size_t)np * sizeof(float));
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < np; ++i) {
        float v = pixel_variance(&j->stats[i]);
        if (!isfinite(v)) v = EPS_SMALL;
        curr[i] = fclamps(v, EPS_SMALL, max_variance);
    }
    ensure_feature_cache(j);
    for (int it = 0; it < iterations; ++it) {
        const float* src = curr;
        float* dst = next;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t idx = 0; idx < np; ++idx) {
            const int y = (int)(idx / w), x = (int)(idx % w);
            if (j->hit_count[idx] == 0) { dst[idx] = src[idx]; continue; }
            const float* normal_i = j->f_normal + 3 * idx;
            const float depth_i = j->f_depth[idx];
            const float var_i = fmaxs(EPS_SMALL, src[idx]);
            float weight_sum = 0.0f, weighted_sum = 0.0f;
            for (int dy = -radius; dy <= radius; ++dy) {
                const int yy = y + dy;
                if (yy < 0 || yy >= h) continue;
                for (int dx = -radius; dx <= radius; ++dx) {
                    const int xx = x + dx;
                    if (xx < 0 || xx >= w || (dx == 0 && dy == 0)) continue;
                    const int64_t jn = (int64_t)yy * w + xx;
                    if (j->hit_count[jn] == 0) continue;
                    if (dot3(normal_i, j->f_normal + 3 * jn) < normal_threshold) continue;
                    if (relative_depth_delta(depth_i, j->f_depth[jn]) > depth_threshold) continue;
                    const float var_j = fmaxs(EPS_SMALL, src[jn]);
                    const float relative_difference = fabsf(var_i - var_j) / fmaxs(EPS_SMALL, sqrtf(var_i * var_j));
                    if (relative_difference > compat_sigma) continue;
                    const float dist2 = (float)(dx * dx + dy * dy);
                    const float w_j = 1.0f / (1.0f + dist2);
                    weighted_sum += w_j * var_j;
                    weight_sum += w_j;
                }
            }
            float neighbor_mean = var_i;
            if (weight_sum > EPS_SMALL) neighbor_mean = weighted_sum / weight_sum;
            dst[idx] = conservative_variance_update(var_i, neighbor_mean, shrinkage_k);
        }
        float* t = curr; curr = next; next = t;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < np; ++i) {
        float raw = pixel_variance(&j->stats[i]);
        if (!isfinite(raw)) raw = EPS_SMALL;
        raw = fclamps(raw, EPS_SMALL, max_variance);
        j->variance_denoised[i] = fmaxs(curr[i], raw);
    }
    free(curr);
    free(next);
    j->stage_ms[RPD_STAGE_VARIANCE] = now_ms() - t0;
    return RPD_OK;
}

/* ---- compute_adaptive_sample_counts (main.cpp:1273-1446) ------------------------------ */
#ifndef ORC_F64

/* The budget-preserving allocation of compute_adaptive_sample_counts (main.cpp:1372-1438) on a
 * final importance map: counts holds the floor per pixel on entry and the counts on return.
 * sum_importance is std::accumulate over the map (main.cpp:1370), in pixel order. */
void orc_allocate_counts(const float* importance, int64_t np, const rpd_config* cfg, double sum_importance,
                         int32_t* sc) {
    const int extra_sample_total = (int)(cfg->adaptive_spp * np);
    const int floor_per_pixel = iclamps(cfg->adaptive_base_samples, 0, cfg->adaptive_spp);
    const int reserved_samples = (int)(floor_per_pixel * np);
    if (extra_sample_total <= 0) return;
    {
        int remaining_samples = imaxs(0, extra_sample_total - reserved_samples);
        if (sum_importance <= 0.0 || remaining_samples <= 0) {
            return;
        }
        float* desired_add = (float*)zalloc((size_t)np * sizeof(float));
        int32_t* active = (int32_t*)malloc((size_t)np * 4);
        int32_t* next_active = (int32_t*)malloc((size_t)np * 4);
        int64_t n_active = np;
        for (int64_t i = 0; i < np; ++i) active[i] = (int32_t)i;
        double remaining_importance = sum_importance;
        const int max_extra_per_pixel = imaxs(4, 8 * imaxs(1, cfg->adaptive_spp));
        while (n_active > 0 && remaining_samples > 0 && remaining_importance > (double)EPS_SMALL) {
            int clipped = 0;
            int64_t n_next = 0;
            for (int64_t a = 0; a < n_active; ++a) {
                const int32_t idx = active[a];
                const double share = (double)importance[idx] / remaining_importance;
                const double desired = share * (double)remaining_samples;
                if (desired > (double)max_extra_per_pixel) {
                    desired_add[idx] = (float)max_extra_per_pixel;
                    remaining_samples -= max_extra_per_pixel;
                    remaining_importance -= (double)importance[idx];
                    clipped = 1;
                } else {
                    next_active[n_next++] = idx;
                }
            }
            if (!clipped) {
                for (int64_t a = 0; a < n_next; ++a) {
                    const int32_t idx = next_active[a];
                    desired_add[idx] = (float)((double)importance[idx] / remaining_importance * (double)remaining_samples);
                }
                break;
            }
            int32_t* t = active; active = next_active; next_active = t;
            n_active = n_next;
        }
        int assigned = 0;
        float* residual = (float*)zalloc((size_t)np * sizeof(float));
        double residual_sum = 0.0;
        for (int64_t i = 0; i < np; ++i) {
            const int add = (int)floorf(desired_add[i]);
            sc[i] += add;
            assigned += add;
            residual[i] = fmaxs(0.0f, desired_add[i] - (float)add);
            residual_sum += (double)residual[i];
        }
        const int remaining = imaxs(0, extra_sample_total - reserved_samples - assigned);
        if (remaining > 0 && residual_sum > (double)EPS_SMALL) {
            const double offset = (double)hash_to_unit_float(cfg->seed ^ 0x4d595df4u);
            double cumulative = 0.0;
            int64_t cursor = 0;
            for (int k = 0; k < remaining; ++k) {
                const double target = (((double)k + offset) / (double)remaining) * residual_sum;
                while (cursor < np && cumulative + (double)residual[cursor] < target) {
                    cumulative += (double)residual[cursor];
                    ++cursor;
                }
                if (cursor < np) sc[cursor]++;
            }
        }
        free(residual); free(desired_add); free(active); free(next_active);
    }
}

/* orc_allocate_counts with the sum taken here, for callers holding only the map. */
void orc_allocate_counts_map(const float* importance, int64_t np, const rpd_config* cfg, int32_t* counts) {
    const int floor_per_pixel = iclamps(cfg->adaptive_base_samples, 0, cfg->adaptive_spp);
    for (int64_t i = 0; i < np; ++i) counts[i] = floor_per_pixel;
    double sum_importance = 0.0;
    for (int64_t i = 0; i < np; ++i) sum_importance = sum_importance + (double)importance[i];
    orc_allocate_counts(importance, np, cfg, sum_importance, counts);
}

int orc_compute_adaptive_sample_counts(orc_job* j, int32_t* counts_out) {
    const double t0 = now_ms();
    set_omp(j->threads);
    const int w = j->w, h = j->h;
    const int64_t np = (int64_t)j->np;
    const int extra_sample_total = j->cfg.adaptive_spp * w * h;
    const int floor_per_pixel = iclamps(j->cfg.adaptive_base_samples, 0, j->cfg.adaptive_spp);
    int32_t* sc = j->last_counts;
    for (int64_t i = 0; i < np; ++i) sc[i] = floor_per_pixel;
    if (extra_sample_total <= 0) goto done;
    {
        const float SIGMA_MAX = j->cfg.adaptive_sigma_max;
        ensure_feature_cache(j);
        float* importance = (float*)zalloc((size_t)np * sizeof(float));
        float* vs = (float*)zalloc((size_t)np * sizeof(float));
        memcpy(vs, j->variance_denoised, (size_t)np * sizeof(float));
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t i = 0; i < np; ++i) {
            float raw = pixel_variance(&j->stats[i]);
            if (!isfinite(raw)) raw = EPS_SMALL;
            raw = fmaxs(EPS_SMALL, raw);
            float dsv = vs[i];
            if (!isfinite(dsv) || dsv <= 0.0f) dsv = raw;
            vs[i] = fclamps(fmaxs(raw, dsv), EPS_SMALL, SIGMA_MAX * SIGMA_MAX);
        }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t i = 0; i < np; ++i) importance[i] = sqrtf(vs[i]);
        double sum_importance = 0.0;
        for (int64_t i = 0; i < np; ++i) sum_importance = sum_importance + (double)importance[i];

        const int radius = j->cfg.adaptive_importance_smoothing_radius;
        if (radius > 0) {
            float* smoothed = (float*)zalloc((size_t)np * sizeof(float));
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
            for (int64_t idx = 0; idx < np; ++idx) {
                const int y = (int)(idx / w), x = (int)(idx % w);
                if (j->hit_count[idx] == 0) { smoothed[idx] = importance[idx]; continue; }
                double accum = 0.0, weight_sum = 0.0;
                for (int dy = -radius; dy <= radius; ++dy) {
                    const int yy = y + dy;
                    if (yy < 0 || yy >= h) continue;
                    for (int dx = -radius; dx <= radius; ++dx) {
                        const int xx = x + dx;
                        if (xx < 0 || xx >= w) continue;
                        const int64_t nidx = (int64_t)yy * w + xx;
                        if (j->hit_count[nidx] == 0) continue;
                        const float spatial_w = 1.0f / (1.0f + (float)(dx * dx + dy * dy));
                        const float normal_w = fclamps((dot3(j->f_normal + 3 * idx, j->f_normal + 3 * nidx) + 1.0f) * 0.5f,
                                                       0.0f, 1.0f);
                        const float depth_w = expf(-4.0f * relative_depth_delta(j->f_depth[idx], j->f_depth[nidx]));
                        const double w_neighbor = (double)spatial_w * (double)normal_w * (double)depth_w;
                        accum += w_neighbor * (double)importance[nidx];
                        weight_sum += w_neighbor;
                    }
                }
                smoothed[idx] = (weight_sum > (double)EPS_SMALL) ? (float)(accum / weight_sum) : importance[idx];
            }
            free(importance);
            importance = smoothed;
            sum_importance = 0.0;
            for (int64_t i = 0; i < np; ++i) sum_importance = sum_importance + (double)importance[i];
        }
        memcpy(j->adaptive_importance, importance, (size_t)np * sizeof(float));

        orc_allocate_counts(importance, np, &j->cfg, sum_importance, sc);
        free(importance); free(vs);
    }
done:
    if (counts_out) memcpy(counts_out, sc, (size_t)np * 4);
    j->stage_ms[RPD_STAGE_ADAPTIVE] = now_ms() - t0;
    return RPD_OK;
}

#endif /* ORC_F64 */

/* ---- FrameBuffers::finalize (core/buffers.h:152-167) --------------------------------- */

int orc_finalize(orc_job* j) {
    set_omp(j->threads);
    const int64_t np = (int64_t)j->np;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < np; ++i) {
        const int samples = imaxs(1, j->sample_count[i]);
        const int hits = imaxs(1, j->hit_count[i]);
        for (int c = 0; c < 3; ++c) j->radiance[3 * i + c] /= (float)samples;
        for (int c = 0; c < 3; ++c) j->albedo[3 * i + c] /= (float)hits;
        for (int c = 0; c < 3; ++c) j->normal[3 * i + c] /= (float)hits;
        if (dot3(j->normal + 3 * i, j->normal + 3 * i) > EPS_SMALL) normalize3(j->normal + 3 * i);
        j->depth[i] /= (float)hits;
    }
    j->features_valid = 0;
    return RPD_OK;
}

/* ---- reads ------------------------------------------------------------------------- */

uint64_t orc_field_bytes(const orc_job* j, int field) {
    const uint64_t np = j->np, nn = j->nn;
    switch (field) {
    case RPD_FIELD_DENOISED: case RPD_FIELD_RADIANCE_SUM: case RPD_FIELD_NORMAL_SUM: case RPD_FIELD_ALBEDO_SUM:
    case RPD_FIELD_STATS_COLOR_MEAN: case RPD_FIELD_STATS_SQRT_MEAN: case RPD_FIELD_STATS_SQRT_SQUARE_DIFF:
    case RPD_FIELD_SQRT_VARIANCE_STABLE:
        return np * 12;
    case RPD_FIELD_GRID: return nn * NDEP * DSTRIDE * 8;
    default:
        if (field >= RPD_FIELD_NODE_ALL && field <= RPD_FIELD_NODE_RR_CONF) return nn * 4;
        if (field >= 0 && field < RPD_FIELD_COUNT_) return np * 4;
        return 0;
    }
}

static int put(void* dst, size_t bytes, const void* src, uint64_t need) {
    if (bytes != need) return RPD_ERR_INVALID_ARGUMENT;
    memcpy(dst, src, bytes);
    return RPD_OK;
}

#ifndef ORC_F64
int orc_job_read(orc_job* j, int field, void* dst, size_t bytes) {
    const uint64_t need = orc_field_bytes(j, field);
    const int64_t np = (int64_t)j->np;
    if (need == 0 || bytes != need) return RPD_ERR_INVALID_ARGUMENT;
    switch (field) {
    case RPD_FIELD_DENOISED: return put(dst, bytes, j->denoised, need);
    case RPD_FIELD_UNCERTAINTY: return put(dst, bytes, j->uncertainty, need);
    case RPD_FIELD_ALPHA: return put(dst, bytes, j->alpha, need);
    case RPD_FIELD_VAR_TOTAL_DEBUG: return put(dst, bytes, j->var_total, need);
    case RPD_FIELD_VAR_EFF_DEBUG: return put(dst, bytes, j->var_eff, need);
    case RPD_FIELD_VAR_RATIO_DEBUG: return put(dst, bytes, j->var_ratio, need);
    case RPD_FIELD_VARIANCE_DENOISED: return put(dst, bytes, j->variance_denoised, need);
    case RPD_FIELD_ADAPTIVE_IMPORTANCE: return put(dst, bytes, j->adaptive_importance, need);
    case RPD_FIELD_SENSITIVITY_CONFIDENCE: return put(dst, bytes, j->sens_confidence, need);
    case RPD_FIELD_SENSITIVITY_GRADIENT: return put(dst, bytes, j->sens_gradient, need);
    case RPD_FIELD_HIT_COUNT: return put(dst, bytes, j->hit_count, need);
    case RPD_FIELD_SAMPLE_COUNT: return put(dst, bytes, j->sample_count, need);
    case RPD_FIELD_RADIANCE_SUM: return put(dst, bytes, j->radiance, need);
    case RPD_FIELD_NORMAL_SUM: return put(dst, bytes, j->normal, need);
    case RPD_FIELD_ALBEDO_SUM: return put(dst, bytes, j->albedo, need);
    case RPD_FIELD_DEPTH_SUM: return put(dst, bytes, j->depth, need);
    case RPD_FIELD_STATS_MEAN: case RPD_FIELD_STATS_SQUARE_DIFF: case RPD_FIELD_STATS_N:
        for (int64_t i = 0; i < np; ++i) {
            const pstats* s = &j->stats[i];
            if (field == RPD_FIELD_STATS_N) ((int32_t*)dst)[i] = s->n;
            else ((float*)dst)[i] = field == RPD_FIELD_STATS_MEAN ? s->mean : s->square_diff;
        }
        return RPD_OK;
    case RPD_FIELD_STATS_COLOR_MEAN: case RPD_FIELD_STATS_SQRT_MEAN: case RPD_FIELD_STATS_SQRT_SQUARE_DIFF:
        for (int64_t i = 0; i < np; ++i) {
            const pstats* s = &j->stats[i];
            const float* v = field == RPD_FIELD_STATS_COLOR_MEAN ? s->color_mean
                           : field == RPD_FIELD_STATS_SQRT_MEAN ? s->sqrt_mean : s->sqrt_sq;
            for (int c = 0; c < 3; ++c) ((float*)dst)[3 * i + c] = v[c];
        }
        return RPD_OK;
    case RPD_FIELD_GRID: return put(dst, bytes, j->grid, need);
    case RPD_FIELD_ADAPTIVE_COUNTS: return put(dst, bytes, j->last_counts, need);
    case RPD_FIELD_SQRT_VARIANCE_STABLE: return put(dst, bytes, j->sqrt_var_stable, need);
    default:
        break;
    }
    if (field >= RPD_FIELD_NODE_ALL && field <= RPD_FIELD_NODE_RR_CONF)
        return put(dst, bytes, j->node[field - RPD_FIELD_NODE_ALL], need);
    if (field >= RPD_FIELD_EXPANDED_ALL && field <= RPD_FIELD_EXPANDED_RR) {
        static const int map[9] = {N_ALL, N_PIXEL, N_BRDF, N_LENS, N_LIGHT, N_LIGHT_UV, N_LIGHT_SELECT, N_ENV, N_RR};
        expand_values(j, j->node[map[field - RPD_FIELD_EXPANDED_ALL]], (float*)dst);
        return RPD_OK;
    }
    return RPD_ERR_INVALID_ARGUMENT;
}

#endif /* ORC_F64 */

double orc_stage_ms(const orc_job* j, int stage) {
    return (stage >= 0 && stage < RPD_STAGE_COUNT_) ? j->stage_ms[stage] : -1.0;
}

int orc_nodes(const orc_job* j, int32_t* nodes_x, int32_t* nodes_y) {
    *nodes_x = j->nodes_x;
    *nodes_y = j->nodes_y;
    return RPD_OK;
}

#ifndef ORC_F64
/* ---- standalone filters ------------------------------------------------------------- */

/* normalize + luminance helpers (denoising/atrous_wavelet.cpp:37-52) */
static inline void filt_normalize(float* x, float* y, float* z) {
    const float len_sq = *x * *x + *y * *y + *z * *z;
    if (len_sq > EPS_SMALL) {
        const float inv_len = 1.0f / sqrtf(len_sq);
        *x *= inv_len; *y *= inv_len; *z *= inv_len;
    }
}

/* atrous_filter_pass (denoising/atrous_wavelet.cpp:54-149) */
static void atrous_pass(const float* input, float* output, const float* normal, const float* albedo, int w, int h,
                        int step_width, float sigma_c, float sigma_n, float sigma_a) {
    static const float hk[5] = {1 / 16.0f, 1 / 4.0f, 3 / 8.0f, 1 / 4.0f, 1 / 16.0f};
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            const int idx = y * w + x;
            const float c_r = input[3 * idx], c_g = input[3 * idx + 1], c_b = input[3 * idx + 2];
            const float c_lum = calc_luminance(c_r, c_g, c_b);
            float n_r = normal[3 * idx], n_g = normal[3 * idx + 1], n_b = normal[3 * idx + 2];
            filt_normalize(&n_r, &n_g, &n_b);
            const float a_r = albedo[3 * idx], a_g = albedo[3 * idx + 1], a_b = albedo[3 * idx + 2];
            float sum_r = 0.0f, sum_g = 0.0f, sum_b = 0.0f, sum_weight = 0.0f;
            for (int k = 0; k < 25; k++) {
                const int kx = k % 5 - 2, ky = k / 5 - 2;
                const int ox = kx * step_width, oy = ky * step_width;
                const int nx = iclamps(x + ox, 0, w - 1);
                const int ny = iclamps(y + oy, 0, h - 1);
                const int n_idx = ny * w + nx;
                const float p_r = input[3 * n_idx], p_g = input[3 * n_idx + 1], p_b = input[3 * n_idx + 2];
                const float p_lum = calc_luminance(p_r, p_g, p_b);
                float pn_r = normal[3 * n_idx], pn_g = normal[3 * n_idx + 1], pn_b = normal[3 * n_idx + 2];
                filt_normalize(&pn_r, &pn_g, &pn_b);
                const float pa_r = albedo[3 * n_idx], pa_g = albedo[3 * n_idx + 1], pa_b = albedo[3 * n_idx + 2];
                const float w_spatial = hk[ky + 2] * hk[kx + 2];
                const float lum_diff = c_lum - p_lum;
                const float w_color = expf(-lum_diff * lum_diff / (2.0f * sigma_c * sigma_c));
                float dot_n = n_r * pn_r + n_g * pn_g + n_b * pn_b;
                dot_n = fclamps(dot_n, -1.0f, 1.0f);
                const float angle = acosf(dot_n);
                const float w_normal = expf(-angle * angle / (2.0f * sigma_n * sigma_n));
                const float da_r = a_r - pa_r, da_g = a_g - pa_g, da_b = a_b - pa_b;
                const float dist_sq_albedo = da_r * da_r + da_g * da_g + da_b * da_b;
                const float w_albedo = expf(-dist_sq_albedo / (2.0f * sigma_a * sigma_a));
                const float weight = w_spatial * w_color * w_normal * w_albedo;
                sum_r += weight * p_r;
                sum_g += weight * p_g;
                sum_b += weight * p_b;
                sum_weight += weight;
            }
            if (sum_weight > EPS_SMALL) {
                output[3 * idx] = sum_r / sum_weight;
                output[3 * idx + 1] = sum_g / sum_weight;
                output[3 * idx + 2] = sum_b / sum_weight;
            } else {
                output[3 * idx] = c_r;
                output[3 * idx + 1] = c_g;
                output[3 * idx + 2] = c_b;
            }
        }
    }
}

/* filter() (denoising/atrous_wavelet.cpp:175-199) */
int orc_atrous_wavelet(const float* raw, const float* normal, const float* albedo, int32_t w, int32_t h,
                       float sigma_c, float sigma_n, float sigma_a, int32_t iterations, float* out, int threads) {
    set_omp(threads);
    const size_t n = (size_t)w * h * 3;
    float* a = (float*)malloc(n * 4);
    float* b = (float*)malloc(n * 4);
    memcpy(a, raw, n * 4);
    float* in = a;
    float* o = b;
    for (int it = 0; it < iterations; ++it) {
        atrous_pass(in, o, normal, albedo, w, h, 1 << it, sigma_c, sigma_n, sigma_a);
        float* t = in; in = o; o = t;
    }
    memcpy(out, in, n * 4);
    free(a);
    free(b);
    return RPD_OK;
}

/* filter() loop (denoising/joint_bilateral.cpp:43-132) */
int orc_joint_bilateral(const float* raw, const float* normal, const float* albedo, int32_t w, int32_t h,
                        float sigma_c, float sigma_n, float sigma_p, float sigma_a,
                        float* gaussian, float* bilateral, float* joint, int threads) {
    set_omp(threads);
    const int radius = imaxs(1, (int)ceilf(3.0f * sigma_p));
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < h; i++) {
        for (int jx = 0; jx < w; jx++) {
            float ws_g = 0.0f, vr_g = 0.0f, vg_g = 0.0f, vb_g = 0.0f;
            float ws_c = 0.0f, vr_c = 0.0f, vg_c = 0.0f, vb_c = 0.0f;
            float ws_j = 0.0f, vr_j = 0.0f, vg_j = 0.0f, vb_j = 0.0f;
            const int ci = 3 * (i * w + jx);
            const float red = raw[ci], green = raw[ci + 1], blue = raw[ci + 2];
            float n_i_r = normal[ci] * 2.0f - 1.0f;
            float n_i_g = normal[ci + 1] * 2.0f - 1.0f;
            float n_i_b = normal[ci + 2] * 2.0f - 1.0f;
            filt_normalize(&n_i_r, &n_i_g, &n_i_b);
            const float a_i_r = albedo[ci], a_i_g = albedo[ci + 1], a_i_b = albedo[ci + 2];
            for (int y = i - radius; y < i + radius + 1; y++) {
                for (int x = jx - radius; x < jx + radius + 1; x++) {
                    const int c = (int)(fmins(fmaxs(0.0f, (float)y), (float)h - 1));
                    const int r = (int)(fmins(fmaxs(0.0f, (float)x), (float)w - 1));
                    const float alpha = 0.5f;
                    const float beta = 2.0f - alpha;
                    const float dist_square_pixel = (float)((i - c) * (i - c) + (jx - r) * (jx - r));
                    const int q = 3 * (c * w + r);
                    const float red_diff = (red - raw[q]);
                    const float green_diff = (green - raw[q + 1]);
                    const float blue_diff = (blue - raw[q + 2]);
                    float dist_square_color = red_diff * red_diff + green_diff * green_diff + blue_diff * blue_diff;
                    dist_square_color *= alpha;
                    float n_j_r = normal[q] * 2.0f - 1.0f;
                    float n_j_g = normal[q + 1] * 2.0f - 1.0f;
                    float n_j_b = normal[q + 2] * 2.0f - 1.0f;
                    filt_normalize(&n_j_r, &n_j_g, &n_j_b);
                    const float a_red_diff = (a_i_r - albedo[q]);
                    const float a_green_diff = (a_i_g - albedo[q + 1]);
                    const float a_blue_diff = (a_i_b - albedo[q + 2]);
                    const float dist_square_albedo =
                        a_red_diff * a_red_diff + a_green_diff * a_green_diff + a_blue_diff * a_blue_diff;
                    float dot_product = n_i_r * n_j_r + n_i_g * n_j_g + n_i_b * n_j_b;
                    dot_product = fclamps(dot_product, -1.0f, 1.0f);
                    const float n_val = acosf(dot_product);
                    float n_val_square = n_val * n_val;
                    n_val_square *= beta;
                    const float weight_gauss = expf(-dist_square_pixel / (2.0f * sigma_p * sigma_p));
                    vr_g += weight_gauss * raw[q];
                    vg_g += weight_gauss * raw[q + 1];
                    vb_g += weight_gauss * raw[q + 2];
                    const float weight_color = expf(-dist_square_pixel / (2.0f * sigma_p * sigma_p) -
                                                    dist_square_color / (2.0f * sigma_c * sigma_c));
                    vr_c += weight_color * raw[q];
                    vg_c += weight_color * raw[q + 1];
                    vb_c += weight_color * raw[q + 2];
                    const float weight_joint = expf(-dist_square_pixel / (2.0f * sigma_p * sigma_p) -
                                                    dist_square_color / (2.0f * sigma_c * sigma_c) -
                                                    n_val_square / (2.0f * sigma_n * sigma_n) -
                                                    dist_square_albedo / (2.0f * sigma_a * sigma_a));
                    vr_j += weight_joint * raw[q];
                    vg_j += weight_joint * raw[q + 1];
                    vb_j += weight_joint * raw[q + 2];
                    ws_g += weight_gauss;
                    ws_c += weight_color;
                    ws_j += weight_joint;
                }
            }
            gaussian[ci] = vr_g / ws_g; gaussian[ci + 1] = vg_g / ws_g; gaussian[ci + 2] = vb_g / ws_g;
            bilateral[ci] = vr_c / ws_c; bilateral[ci + 1] = vg_c / ws_c; bilateral[ci + 2] = vb_c / ws_c;
            joint[ci] = vr_j / ws_j; joint[ci + 1] = vg_j / ws_j; joint[ci + 2] = vb_j / ws_j;
        }
    }
    return RPD_OK;
}

/* compute_extended_metrics (shared/tools/eval_tools.cpp:121-213): NRMSE, the 11x11 box-window
 * SSIM of log1p luminance from integral images, and the NRMSE of its forward differences, in
 * double precision and the reference's order. */
static double orc_box_sum(const double* s, int stride, int x0, int y0, int x1, int y1) {
    return s[y1 * stride + x1] - s[y0 * stride + x1] - s[y1 * stride + x0] + s[y0 * stride + x0];
}

static double orc_maxd(double a, double b) { return (a < b) ? b : a; }

static void orc_extended_metrics(const float* ref, const float* tst, int w, int h, rpd_image_metrics* m) {
    const int pixels = w * h;
    double* ref_log = (double*)malloc(sizeof(double) * (size_t)pixels);
    double* tst_log = (double*)malloc(sizeof(double) * (size_t)pixels);
    double ref_energy = 0.0, error_energy = 0.0, log_peak = 0.0;
    static const double weights[3] = {0.2126, 0.7152, 0.0722};
    for (int i = 0; i < pixels; ++i) {
        double ref_lum = 0.0, tst_lum = 0.0;
        for (int c = 0; c < 3; ++c) {
            const double a = ref[3 * i + c];
            const double b = tst[3 * i + c];
            ref_energy += a * a;
            error_energy += (a - b) * (a - b);
            ref_lum += weights[c] * a;
            tst_lum += weights[c] * b;
        }
        ref_log[i] = log1p(orc_maxd(0.0, ref_lum));
        tst_log[i] = log1p(orc_maxd(0.0, tst_lum));
        log_peak = orc_maxd(log_peak, ref_log[i]);
    }
    m->nrmse = sqrt(error_energy / orc_maxd(1e-18, ref_energy));

    const int stride = w + 1;
    const size_t isz = (size_t)stride * (size_t)(h + 1);
    double* sr = (double*)calloc(isz, sizeof(double));
    double* st = (double*)calloc(isz, sizeof(double));
    double* sr2 = (double*)calloc(isz, sizeof(double));
    double* st2 = (double*)calloc(isz, sizeof(double));
    double* sx = (double*)calloc(isz, sizeof(double));
    for (int y = 0; y < h; ++y) {
        double row_ref = 0.0, row_tst = 0.0, row_ref2 = 0.0, row_tst2 = 0.0, row_cross = 0.0;
        for (int x = 0; x < w; ++x) {
            const double a = ref_log[y * w + x];
            const double b = tst_log[y * w + x];
            row_ref += a;
            row_tst += b;
            row_ref2 += a * a;
            row_tst2 += b * b;
            row_cross += a * b;
            const int out = (y + 1) * stride + x + 1;
            sr[out] = sr[out - stride] + row_ref;
            st[out] = st[out - stride] + row_tst;
            sr2[out] = sr2[out - stride] + row_ref2;
            st2[out] = st2[out - stride] + row_tst2;
            sx[out] = sx[out - stride] + row_cross;
        }
    }
    log_peak = orc_maxd(1e-6, log_peak);
    const double c1 = pow(0.01 * log_peak, 2.0);
    const double c2 = pow(0.03 * log_peak, 2.0);
    double ssim_sum = 0.0;
    for (int y = 0; y < h; ++y) {
        const int y0 = y - 5 > 0 ? y - 5 : 0;
        const int y1 = y + 6 < h ? y + 6 : h;
        for (int x = 0; x < w; ++x) {
            const int x0 = x - 5 > 0 ? x - 5 : 0;
            const int x1 = x + 6 < w ? x + 6 : w;
            const double n = (double)((x1 - x0) * (y1 - y0));
            const double mean_ref = orc_box_sum(sr, stride, x0, y0, x1, y1) / n;
            const double mean_tst = orc_box_sum(st, stride, x0, y0, x1, y1) / n;
            const double var_ref = orc_maxd(0.0, orc_box_sum(sr2, stride, x0, y0, x1, y1) / n - mean_ref * mean_ref);
            const double var_tst = orc_maxd(0.0, orc_box_sum(st2, stride, x0, y0, x1, y1) / n - mean_tst * mean_tst);
            const double cov = orc_box_sum(sx, stride, x0, y0, x1, y1) / n - mean_ref * mean_tst;
            const double num = (2.0 * mean_ref * mean_tst + c1) * (2.0 * cov + c2);
            const double den = (mean_ref * mean_ref + mean_tst * mean_tst + c1) * (var_ref + var_tst + c2);
            ssim_sum += (den > 0.0) ? num / den : 1.0;
        }
    }
    m->log_ssim11 = ssim_sum / (double)pixels;

    double gerr = 0.0, gref = 0.0;
    for (int y = 0; y < h - 1; ++y) {
        for (int x = 0; x < w - 1; ++x) {
            const int i = y * w + x;
            const double rdx = ref_log[i + 1] - ref_log[i];
            const double rdy = ref_log[i + w] - ref_log[i];
            const double tdx = tst_log[i + 1] - tst_log[i];
            const double tdy = tst_log[i + w] - tst_log[i];
            gerr += (rdx - tdx) * (rdx - tdx) + (rdy - tdy) * (rdy - tdy);
            gref += rdx * rdx + rdy * rdy;
        }
    }
    m->log_gradient_nrmse = sqrt(gerr / orc_maxd(1e-18, gref));
    free(ref_log);
    free(tst_log);
    free(sr);
    free(st);
    free(sr2);
    free(st2);
    free(sx);
}

/* hdr_metrics (shared/tools/eval_tools.cpp:232-286) without the file I/O and the residual image. */
int orc_hdr_metrics(const float* ref, const float* tst, int32_t w, int32_t h, rpd_image_metrics* out) {
    if (!ref || !tst || !out || w <= 0 || h <= 0) return RPD_ERR_INVALID_ARGUMENT;
    const int pixels = w * h;
    double sum_sq = 0.0, sum_abs = 0.0, peak = 0.0;
    double mean_ref[3] = {0.0, 0.0, 0.0}, mean_tst[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < pixels; ++i) {
        for (int c = 0; c < 3; ++c) {
            const double a = ref[3 * i + c];
            const double b = tst[3 * i + c];
            sum_sq += (a - b) * (a - b);
            sum_abs += fabs(a - b);
            peak = orc_maxd(peak, fabs(a));
            mean_ref[c] += a;
            mean_tst[c] += b;
        }
    }
    for (int c = 0; c < 3; ++c) {
        mean_ref[c] /= pixels;
        mean_tst[c] /= pixels;
    }
    if (peak <= 0.0) peak = 1.0;
    const double C1 = (0.01 * peak) * (0.01 * peak);
    const double C2 = (0.03 * peak) * (0.03 * peak);
    for (int c = 0; c < 3; ++c) {
        double var_ref = 0.0, var_tst = 0.0, cov = 0.0;
        for (int i = 0; i < pixels; ++i) {
            const double a = ref[3 * i + c];
            const double b = tst[3 * i + c];
            var_ref += (a - mean_ref[c]) * (a - mean_ref[c]);
            var_tst += (b - mean_tst[c]) * (b - mean_tst[c]);
            cov += (a - mean_ref[c]) * (b - mean_tst[c]);
        }
        var_ref /= pixels;
        var_tst /= pixels;
        cov /= pixels;
        const double num = (2.0 * mean_ref[c] * mean_tst[c] + C1) * (2.0 * cov + C2);
        const double den = (mean_ref[c] * mean_ref[c] + mean_tst[c] * mean_tst[c] + C1) * (var_ref + var_tst + C2);
        out->ssim[c] = (den > 0.0) ? num / den : 0.0;
    }
    const double mse = sum_sq / (pixels * 3);
    out->mae = sum_abs / (pixels * 3);
    out->rmse = sqrt(mse);
    out->peak = peak;
    out->psnr = (out->rmse > 0.0) ? 20.0 * log10(peak / out->rmse) : INFINITY;
    out->ssim_mean = (out->ssim[0] + out->ssim[1] + out->ssim[2]) / 3.0;
    orc_extended_metrics(ref, tst, w, h, out);
    return RPD_OK;
}
#endif /* ORC_F64 */
