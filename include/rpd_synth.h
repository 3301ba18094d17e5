/*
 * rpd_synth.h — seeded synthetic per-sample generator for the denoise stage.
 *
 * The reference measures the stage on samples traced from its scenes. At 1080p/16 spp
 * that needs a tracer this project does not ship, so the full-size workloads use this
 * generator instead. It stands in for a tracer's output with the structure stated for
 * the full-size benchmark: a Voronoi partition of the image into `regions` cells, each
 * with a constant unit normal, a planar depth in [1, 10], a constant albedo and a
 * log-normal luminance (mu uniform in [mu_min, mu_max], sigma `sigma`); in
 * `dependent_regions` of them the luminance is scaled by (1 + slope * (u_a + u_b - 1)) for
 * two of the eight random dimensions; `firefly_rate` of the samples are multiplied by
 * `firefly_scale`. The random dimensions are lens uv, BRDF uv, light select (mapped to one
 * of `lights` equal-power lights with the reference's lower_bound rule, core/scene.h:54-61),
 * light uv and Russian roulette (survived = u < 0.8, main.cpp:517-519).
 *
 * Everything here is evaluated with IEEE single-precision +, -, *, / and floor only (the
 * normal draw is an Irwin-Hall sum and exp is a fixed polynomial in powers of two), so
 * host C and device CUDA produce bit-identical samples when built without FMA
 * contraction. Header-only; usable from C11 and CUDA.
 */
#ifndef RPD_SYNTH_H
#define RPD_SYNTH_H

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define RPD_HD __host__ __device__ __forceinline__
#else
#define RPD_HD static inline
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define RPD_SYNTH_MAX_REGIONS 256

typedef struct rpd_synth_params {
    int32_t width;
    int32_t height;
    uint32_t seed;
    int32_t regions;            /* Voronoi cells (48) */
    int32_t dependent_regions;  /* cells whose luminance depends on two random dims (24) */
    float mu_min, mu_max;       /* log-luminance mean range (-2, 1) */
    float sigma;                /* log-luminance sigma (0.8) */
    float slope;                /* dependency slope (0.5) */
    float firefly_rate;         /* fraction of firefly samples (0.001) */
    float firefly_scale;        /* firefly multiplier (100) */
    int32_t lights;             /* equal-power lights for light select (4, must be < 16) */
    int32_t miss_regions;       /* cells that are background (no primary hit); 0 for the benchmark */
    float nan_rate;             /* fraction of samples with non-finite radiance (tests only) */
} rpd_synth_params;

typedef struct rpd_synth_region {
    int32_t cx, cy;             /* seed point */
    float normal[3];            /* unit normal */
    float d0, gx, gy;           /* depth plane: d0 + gx*(x/W-0.5) + gy*(y/H-0.5), clamped to [1,10] */
    float albedo[3];
    float tint[3];              /* colour with luminance 1 */
    float mu;                   /* log-luminance mean */
    int32_t dim_a, dim_b;       /* random dims the luminance depends on, or -1 */
    int32_t miss;               /* background cell */
} rpd_synth_region;

/* Defaults of the full-size benchmark workload. */
RPD_HD void rpd_synth_defaults(rpd_synth_params* p, int32_t width, int32_t height, uint32_t seed) {
    p->width = width;
    p->height = height;
    p->seed = seed;
    p->regions = 48;
    p->dependent_regions = 24;
    p->mu_min = -2.0f;
    p->mu_max = 1.0f;
    p->sigma = 0.8f;
    p->slope = 0.5f;
    p->firefly_rate = 0.001f;
    p->firefly_scale = 100.0f;
    p->lights = 4;
    p->miss_regions = 0;
    p->nan_rate = 0.0f;
}

/* 32-bit integer finaliser (xorshift-multiply, constants from the public "hash
 * prospector" search). */
RPD_HD uint32_t rpd_synth_mix(uint32_t x) {
    x ^= x >> 16;
    x *= 0x21f0aaadu;
    x ^= x >> 15;
    x *= 0x735a2d97u;
    x ^= x >> 15;
    return x;
}

/* Uniform in [0,1) with 24 random bits (exact in float). */
RPD_HD float rpd_synth_unit(uint32_t h) {
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}

RPD_HD uint32_t rpd_synth_key(uint32_t seed, uint32_t a, uint32_t b) {
    return rpd_synth_mix(rpd_synth_mix(seed ^ 0x5bd1e995u) ^ rpd_synth_mix(a * 0x9e3779b1u + b));
}

RPD_HD float rpd_synth_dim(uint32_t key, uint32_t dim) {
    return rpd_synth_unit(rpd_synth_mix(key + dim * 0x632be5abu));
}

/* exp(x) for |x| < 80 as 2^k * P(f): k = floor(x*log2(e)), f in [0,1), P the degree-7
 * Taylor polynomial of 2^f (relative error < 2e-6). Only +,-,* and floor. */
RPD_HD float rpd_synth_exp(float x) {
    if (x > 80.0f) x = 80.0f;
    if (x < -80.0f) x = -80.0f;
    const float t = x * 1.44269504f;
    const float k = floorf(t);
    const float f = t - k;
    float p = 1.52527338e-5f;
    p = p * f;
    p = p + 1.54035304e-4f;
    p = p * f;
    p = p + 1.33335581e-3f;
    p = p * f;
    p = p + 9.61812911e-3f;
    p = p * f;
    p = p + 5.55041087e-2f;
    p = p * f;
    p = p + 2.40226507e-1f;
    p = p * f;
    p = p + 6.93147181e-1f;
    p = p * f;
    p = p + 1.0f;
    /* scale by 2^k with exact power-of-two multiplications */
    int32_t ki = (int32_t)k;
    while (ki > 60) { p = p * 1152921504606846976.0f; ki -= 60; }
    while (ki < -60) { p = p * 8.67361737988403547e-19f; ki += 60; }
    float s = 1.0f;
    if (ki >= 0) { for (int32_t i = 0; i < ki; ++i) s = s * 2.0f; }
    else { for (int32_t i = 0; i < -ki; ++i) s = s * 0.5f; }
    return p * s;
}

RPD_HD float rpd_synth_lum(float r, float g, float b) {
    return 0.2126f * r + 0.7152f * g + 0.0722f * b;
}

/* Region table entry r (0 <= r < p->regions). */
RPD_HD void rpd_synth_region_make(const rpd_synth_params* p, int32_t r, rpd_synth_region* o) {
    const uint32_t key = rpd_synth_key(p->seed, 0xfffffff0u, (uint32_t)r);
    o->cx = (int32_t)(rpd_synth_dim(key, 0) * (float)p->width);
    o->cy = (int32_t)(rpd_synth_dim(key, 1) * (float)p->height);
    if (o->cx >= p->width) o->cx = p->width - 1;
    if (o->cy >= p->height) o->cy = p->height - 1;
    float nx = rpd_synth_dim(key, 2) * 2.0f - 1.0f;
    float ny = rpd_synth_dim(key, 3) * 2.0f - 1.0f;
    float nz = 0.3f + rpd_synth_dim(key, 4);
    const float len = sqrtf(nx * nx + (ny * ny + nz * nz));
    o->normal[0] = nx / len;
    o->normal[1] = ny / len;
    o->normal[2] = nz / len;
    o->d0 = 3.0f + 5.0f * rpd_synth_dim(key, 5);
    o->gx = 4.0f * rpd_synth_dim(key, 6) - 2.0f;
    o->gy = 4.0f * rpd_synth_dim(key, 7) - 2.0f;
    for (int c = 0; c < 3; ++c) o->albedo[c] = 0.05f + 0.9f * rpd_synth_dim(key, 8u + (uint32_t)c);
    float t0 = 0.2f + rpd_synth_dim(key, 11);
    float t1 = 0.2f + rpd_synth_dim(key, 12);
    float t2 = 0.2f + rpd_synth_dim(key, 13);
    const float tl = rpd_synth_lum(t0, t1, t2);
    o->tint[0] = t0 / tl;
    o->tint[1] = t1 / tl;
    o->tint[2] = t2 / tl;
    o->mu = p->mu_min + (p->mu_max - p->mu_min) * rpd_synth_dim(key, 14);
    /* every other cell (up to dependent_regions of them) depends on two distinct dims */
    if ((r & 1) == 1 && (r >> 1) < p->dependent_regions) {
        const int32_t a = (int32_t)(rpd_synth_dim(key, 15) * 8.0f);
        int32_t b = (int32_t)(rpd_synth_dim(key, 16) * 7.0f);
        if (b >= a) b += 1;
        o->dim_a = a > 7 ? 7 : a;
        o->dim_b = b > 7 ? 7 : b;
    } else {
        o->dim_a = -1;
        o->dim_b = -1;
    }
    o->miss = (r < p->miss_regions) ? 1 : 0;
}

/* Index of the Voronoi cell of pixel (x, y): nearest seed in integer distance, ties to
 * the lower index. */
RPD_HD int32_t rpd_synth_pixel_region(const rpd_synth_params* p, const rpd_synth_region* table,
                                      int32_t x, int32_t y) {
    int32_t best = 0;
    int64_t best_d = INT64_MAX;
    for (int32_t r = 0; r < p->regions; ++r) {
        const int64_t dx = (int64_t)(x - table[r].cx);
        const int64_t dy = (int64_t)(y - table[r].cy);
        const int64_t d = dx * dx + dy * dy;
        if (d < best_d) { best_d = d; best = r; }
    }
    return best;
}

typedef struct rpd_synth_sample {
    float radiance[3];
    float normal[3];
    float depth;
    float pixel_u[2];
    float lens_u[2];
    float brdf_u[2];
    float light_u[2];
    uint8_t flags;
    uint8_t category;
} rpd_synth_sample;

/* Sample number `ordinal` (0-based over the pixel's whole life, so adaptive passes keep
 * drawing fresh samples) of pixel (x, y) in cell `reg`. */
RPD_HD void rpd_synth_sample_make(const rpd_synth_params* p, const rpd_synth_region* reg,
                                  int32_t x, int32_t y, uint32_t ordinal, rpd_synth_sample* o) {
    const uint32_t pixel = (uint32_t)y * (uint32_t)p->width + (uint32_t)x;
    const uint32_t key = rpd_synth_key(p->seed, pixel, ordinal);
    float dims[8];
    o->pixel_u[0] = rpd_synth_dim(key, 0);
    o->pixel_u[1] = rpd_synth_dim(key, 1);
    for (uint32_t d = 0; d < 8; ++d) dims[d] = rpd_synth_dim(key, 2u + d);
    o->lens_u[0] = dims[0];
    o->lens_u[1] = dims[1];
    o->brdf_u[0] = dims[2];
    o->brdf_u[1] = dims[3];
    o->light_u[0] = dims[5];
    o->light_u[1] = dims[6];
    if (reg->miss) {
        o->flags = (uint8_t)(0x02u | 0x04u); /* pixel + lens only: no shading data */
        o->category = 0;
        for (int c = 0; c < 3; ++c) {
            o->radiance[c] = 0.5f * reg->tint[c];
            o->normal[c] = 0.0f;
        }
        o->depth = 0.0f;
    } else {
        /* light select: lower_bound over the cumulative equal powers 1..L (scene.h:54-61) */
        const float target = dims[4] * (float)p->lights;
        int32_t light = 0;
        while (light < p->lights - 1 && (float)(light + 1) < target) ++light;
        const int rr = dims[7] < 0.8f;
        o->flags = (uint8_t)(0x01u | 0x02u | 0x04u | 0x08u | 0x10u | 0x20u | 0x80u);
        o->category = (uint8_t)((light & 0x0f) | (rr ? 0x10 : 0));
        const float z = (rpd_synth_dim(key, 10) + rpd_synth_dim(key, 11) + rpd_synth_dim(key, 12) +
                         rpd_synth_dim(key, 13) - 2.0f) * 1.7320508f;
        float lum = rpd_synth_exp(reg->mu + p->sigma * z);
        if (reg->dim_a >= 0) lum = lum * (1.0f + p->slope * (dims[reg->dim_a] + dims[reg->dim_b] - 1.0f));
        if (rpd_synth_dim(key, 14) < p->firefly_rate) lum = lum * p->firefly_scale;
        for (int c = 0; c < 3; ++c) {
            o->radiance[c] = lum * reg->tint[c];
            o->normal[c] = reg->normal[c];
        }
        const float sx = ((float)x + o->pixel_u[0]) / (float)p->width - 0.5f;
        const float sy = ((float)y + o->pixel_u[1]) / (float)p->height - 0.5f;
        float d = reg->d0 + reg->gx * sx + reg->gy * sy;
        if (d < 1.0f) d = 1.0f;
        if (d > 10.0f) d = 10.0f;
        o->depth = d;
    }
    if (p->nan_rate > 0.0f && rpd_synth_dim(key, 15) < p->nan_rate) o->radiance[1] = NAN;
}

#ifdef __cplusplus
}
#endif

#endif /* RPD_SYNTH_H */
