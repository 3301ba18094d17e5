/*
 * rpd_oracle64.c — the double-precision form of the restatement (test infrastructure only).
 *
 * oracle/rpd_oracle.c compiled with every single-precision quantity of the stage held in
 * double: the Welford statistics, the feature sums and caches, the sensitivities, the StatMC
 * window and the variance stabilisation (the reference's own double-precision sums stay
 * double). The public structures (sample planes, rpd_config) keep their float types, so the
 * inputs are the same floats the single-precision paths see. This is the ideal-arithmetic
 * reference the forms' errors are stated against; it is not expected to match the reference's
 * bits. The float-interface entry points (allocation, reads, filters) are not built here;
 * orc64_read converts a result plane to float.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "rpd_gb300.h"
#include "rpd_synth.h"
#include "rpd_oracle.h"

#define ORC_F64 1
#define float double
#define sqrtf sqrt
#define expf exp
#define fabsf fabs
#define floorf floor
#define ceilf ceil
#include "rpd_oracle.c"
#undef float

/* DENOISED (3 per pixel), UNCERTAINTY, ALPHA or VARIANCE_DENOISED of a job as floats. */
int orc64_read(orc_job* j, int field, float* out) {
    const int64_t np = (int64_t)j->np;
    const double* src;
    int64_t n = np;
    switch (field) {
    case RPD_FIELD_DENOISED: src = j->denoised; n = 3 * np; break;
    case RPD_FIELD_UNCERTAINTY: src = j->uncertainty; break;
    case RPD_FIELD_ALPHA: src = j->alpha; break;
    case RPD_FIELD_VARIANCE_DENOISED: src = j->variance_denoised; break;
    default: return RPD_ERR_INVALID_ARGUMENT;
    }
    for (int64_t i = 0; i < n; ++i) out[i] = (float)src[i];
    return RPD_OK;
}
