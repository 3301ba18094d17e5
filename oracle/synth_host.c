/*
 * synth_host.c — host fill of the synthetic per-sample generator (include/rpd_synth.h)
 * for the oracle and the tests. TEST INFRASTRUCTURE ONLY.
 */
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "rpd_oracle.h"

int64_t orc_synth_fill(const rpd_synth_params* p, int64_t first, int64_t count, int32_t spp,
                       const int32_t* counts, const int32_t* start_n, rpd_sample_soa* out, int threads) {
    rpd_synth_region table[RPD_SYNTH_MAX_REGIONS];
    const int regions = p->regions < RPD_SYNTH_MAX_REGIONS ? p->regions : RPD_SYNTH_MAX_REGIONS;
    rpd_synth_params pp = *p;
    pp.regions = regions;
    for (int r = 0; r < regions; ++r) rpd_synth_region_make(&pp, r, &table[r]);
    int64_t* offset = (int64_t*)malloc(sizeof(int64_t) * (size_t)(count + 1));
    offset[0] = 0;
    for (int64_t i = 0; i < count; ++i) offset[i + 1] = offset[i] + (counts ? counts[i] : spp);
#ifdef _OPENMP
    omp_set_num_threads(threads > 0 ? threads : omp_get_num_procs());
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < count; ++i) {
        const int64_t pix = first + i;
        const int32_t x = (int32_t)(pix % pp.width), y = (int32_t)(pix / pp.width);
        const rpd_synth_region* reg = &table[rpd_synth_pixel_region(&pp, table, x, y)];
        if (out->pixel_albedo[0])
            for (int c = 0; c < 3; ++c) ((float*)out->pixel_albedo[c])[i] = reg->albedo[c];
        const uint32_t n0 = start_n ? (uint32_t)start_n[i] : 0u;
        for (int64_t k = offset[i]; k < offset[i + 1]; ++k) {
            rpd_synth_sample s;
            rpd_synth_sample_make(&pp, reg, x, y, n0 + (uint32_t)(k - offset[i]), &s);
            for (int c = 0; c < 3; ++c) {
                ((float*)out->radiance[c])[k] = s.radiance[c];
                ((float*)out->normal[c])[k] = s.normal[c];
            }
            ((float*)out->depth)[k] = s.depth;
            for (int c = 0; c < 2; ++c) {
                ((float*)out->pixel_u[c])[k] = s.pixel_u[c];
                ((float*)out->lens_u[c])[k] = s.lens_u[c];
                ((float*)out->brdf_u[c])[k] = s.brdf_u[c];
                ((float*)out->light_u[c])[k] = s.light_u[c];
            }
            ((uint8_t*)out->flags)[k] = s.flags;
            ((uint8_t*)out->category)[k] = s.category;
            if (out->albedo[0])
                for (int c = 0; c < 3; ++c) ((float*)out->albedo[c])[k] = reg->albedo[c];
        }
    }
    const int64_t total = offset[count];
    free(offset);
    return total;
}
