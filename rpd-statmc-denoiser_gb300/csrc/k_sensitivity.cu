// recompute_sensitivity (main.cpp:741-953) on the node grid.
//
//   k_node_stats    per node: the 13 bias-adjusted explained-variance sensitivities and
//                   confidences (core/stats.h:115-141, 264-302; main.cpp:776-806) and the
//                   3x3 pixel-feature averages at the node centre (main.cpp:808-813).
//   k_node_combine  per node: the 3x3 feature-aware prior smoothing of all 13 fields
//                   (main.cpp:817-863) and the confidence-lerp / relative-sensitivity /
//                   dominant-component combine (main.cpp:865-928). The depth and albedo
//                   edge weights are identical for every field, so each neighbour's weight
//                   is evaluated once and reused for the 13 fields.
//   k_sens_pixels   bilinear expansion of all / all_conf to pixels and the central-
//                   difference gradient (main.cpp:930-947, core/buffers.h:68-101).
//   k_rpd_cache     the per-pixel view statmc_denoise takes of the sensitivity cache:
//                   components_denoise() of sample_sensitivity() (main.cpp:297-327).
#include "rpd_internal.h"
#include "device_math.cuh"

namespace rpd {

namespace {

// ---- the per-bin sums of compute_sensitivity in double-float ---------------------------------
// GB300 executes double precision at a small fraction of its single-precision rate, and the
// sixteen bins' quotients and squares are most of this pass's double work. With the grid in
// its double-float mode (itself within 1e-9 of the reference's double sums) the bin loop runs on
// pairs of floats (about 2^-44 relative), the scalars around it stay in double.
struct F2 {
    float h, l;
};
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }  // k in [-126, 127]
// |a| >= |b|
__device__ __forceinline__ F2 f2_fast(float a, float b) {
    const float s = a + b;
    return F2{s, b - (s - a)};
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float e = ((a.h - (s - bb)) + (b.h - bb)) + (a.l + b.l);
    return f2_fast(s, e);
}
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
    const float p = a.h * b.h;
    const float e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, __fmaf_rn(a.h, b.h, -p)));
    return f2_fast(p, e);
}
// a / b: a quotient from the float reciprocal, corrected once by the double-float remainder
__device__ __forceinline__ F2 f2_div(F2 a, F2 b) {
    float rb;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rb) : "f"(b.h));
    const float q1 = a.h * rb;
    const F2 bq = f2_mul(b, F2{q1, 0.0f});
    const F2 r = f2_add(a, F2{-bq.h, -bq.l});
    return f2_fast(q1, r.h * rb);
}
// d as hi + lo, hi = RN_float(d), lo = RN_float(d - hi), in integer operations; false when
// |d| lies outside [2^-60, 2^61) (the double loop then takes the dependency)
__device__ __forceinline__ bool f2_split(double d, F2& out) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
    if ((b << 1) == 0ull) {
        out = F2{0.0f, 0.0f};
        return true;
    }
    const int e = int((b >> 52) & 0x7ffull) - 1023;
    if (e < -60 || e > 60) return false;
    const unsigned sign = unsigned(b >> 63);
    const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);  // 53-bit significand
    unsigned long long mh = m >> 29;                                     // its top 24 bits
    long long rem = static_cast<long long>(m & ((1ull << 29) - 1ull));   // the rest, units of 2^(e-52)
    if (rem > (1ll << 28) || (rem == (1ll << 28) && (mh & 1ull))) {      // round to nearest, ties to even
        ++mh;
        rem -= 1ll << 29;
    }
    int eh = e;
    if (mh == (1ull << 24)) {
        mh >>= 1;
        ++eh;
    }
    out.h = __int_as_float(int((sign << 31) | (unsigned(eh + 127) << 23) | unsigned(mh & 0x7fffffull)));
    out.l = __ll2float_rn(sign ? -rem : rem) * pow2f(e - 52);
    return true;
}

__device__ __forceinline__ double sample_mass(const double* d) {
    return d[33] > 0.0 ? d[32] * d[32] / d[33] : 0.0;
}

// BinnedDependency::compute_sensitivity (core/stats.h:115-137), in double as the reference sums it.
__device__ float compute_sensitivity(const double* d, int bins) {
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
    if (active < 2 || effective_n <= double(active)) return 0.0f;
    const double eta2 = dclamps(between / total, 0.0, 1.0);
    const double adjusted = dmaxs(0.0, 1.0 - (1.0 - eta2) * (effective_n - 1.0) / (effective_n - active));
    return float(sqrt(adjusted));
}

__device__ __forceinline__ bool f2_le(F2 a, float c) { return a.h < c || (a.h == c && a.l <= 0.0f); }
__device__ __forceinline__ F2 f2_sub(F2 a, F2 b) { return f2_add(a, F2{-b.h, -b.l}); }
__device__ __forceinline__ double f2_double(F2 a) { return double(a.h) + double(a.l); }

// compute_sensitivity and the node's confidence, sample_mass / (sample_mass + n0), with every
// quotient, product and the square root in double-float (about 2^-44 relative; the results are
// floats). GRID_DF: the frame grid holds double-float pairs (the grid's fast mode merges them so);
// else its doubles are split into pairs, and false comes back when one lies outside the split's
// range (the caller then takes the double path). Decisions follow the reference's tests in its
// order.
template <bool GRID_DF>
__device__ bool sensitivity_df(const double* d, int bins, float n0, float& sens, float& conf) {
    const double kEps = 1e-18;
    const float2* dp = reinterpret_cast<const float2*>(d);
    auto get = [&](int k, F2& out) -> bool {
        if (GRID_DF) {
            const float2 v = dp[k];
            out = F2{v.x, v.y};
            return true;
        }
        return f2_split(d[k], out);
    };
    // value > kEps (or > 0) as the double test decides it: on the pairs, against kEps as a pair
    const F2 eps2{1.0e-18f, float(1e-18 - double(1.0e-18f))};
    auto above = [&](int k, F2 v, double t) {
        if (!GRID_DF) return d[k] > t;
        const F2 tt = t > 0.0 ? eps2 : F2{0.0f, 0.0f};
        return v.h > tt.h || (v.h == tt.h && v.l > tt.l);
    };
    F2 w, w2, ys, y2;
    if (!(get(32, w) && get(33, w2) && get(34, ys) && get(35, y2))) return false;
    const F2 en = above(33, w2, 0.0) ? f2_div(f2_mul(w, w), w2) : F2{0.0f, 0.0f};  // sample_mass
    const F2 c = f2_div(en, f2_add(en, F2{n0, 0.0f}));
    conf = c.h + c.l;
    sens = 0.0f;
    if (f2_le(en, 2.0f)) return true;
    const F2 mean = f2_div(ys, w);
    const F2 total = f2_sub(y2, f2_mul(w, f2_mul(mean, mean)));
    if (f2_double(total) <= kEps) return true;
    const F2 nmean{-mean.h, -mean.l};
    F2 between{0.0f, 0.0f};
    int active = 0;
    for (int b = 0; b < bins; ++b) {
        F2 wb, sb;
        if (!get(b, wb)) return false;
        if (!above(b, wb, kEps)) continue;
        ++active;
        if (!get(16 + b, sb)) return false;
        const F2 delta = f2_add(f2_div(sb, wb), nmean);
        between = f2_add(between, f2_mul(wb, f2_mul(delta, delta)));
    }
    if (active < 2 || f2_le(en, float(active))) return true;
    F2 eta2 = f2_div(between, total);
    if (eta2.h < 0.0f) eta2 = F2{0.0f, 0.0f};
    if (eta2.h > 1.0f || (eta2.h == 1.0f && eta2.l > 0.0f)) eta2 = F2{1.0f, 0.0f};
    const F2 one{1.0f, 0.0f};
    const F2 fa = f2_div(f2_sub(en, one), f2_sub(en, F2{float(active), 0.0f}));
    const F2 adj = f2_sub(one, f2_mul(f2_sub(one, eta2), fa));
    if (!(adj.h > 0.0f)) return true;  // max(0, adjusted)
    // sqrt(hi + lo) from the float root of hi and one correction
    const float s0 = sqrtf(adj.h);
    const float r = __fmaf_rn(-s0, s0, adj.h) + adj.l;
    sens = __fmaf_rn(r, 0.5f / s0, s0);
    return true;
}

__constant__ int c_raw_dep[R_FIELDS] = {D_PIXEL, D_BRDF, D_LENS, D_LIGHT_UV, D_LIGHT_SELECT, D_ENV, D_RR,
                                        D_SCREEN_BRDF, D_SCREEN_LENS, D_SCREEN_LIGHT_UV,
                                        D_SCREEN_LIGHT_SELECT, D_SCREEN_ENV, D_SCREEN_RR};

// sample_scalar_local_average / sample_vec3_local_average with radius 1 (main.cpp:156-185)
__device__ float local_avg1(const float* v, int w, int h, int cx, int cy) {
    double accum = 0.0, weight_sum = 0.0;
    for (int dy = -1; dy <= 1; ++dy) {
        const int y = iclamps(cy + dy, 0, h - 1);
        for (int dx = -1; dx <= 1; ++dx) {
            const int x = iclamps(cx + dx, 0, w - 1);
            const double weight = 1.0 / (1.0 + double(dx * dx + dy * dy));
            accum += weight * double(v[int64_t(y) * w + x]);
            weight_sum += weight;
        }
    }
    return (weight_sum > 0.0) ? float(accum / weight_sum) : 0.0f;
}

__device__ void local_avg3(float* const* v, int w, int h, int cx, int cy, float out[3]) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, weight_sum = 0.0;
    for (int dy = -1; dy <= 1; ++dy) {
        const int y = iclamps(cy + dy, 0, h - 1);
        for (int dx = -1; dx <= 1; ++dx) {
            const int x = iclamps(cx + dx, 0, w - 1);
            const double weight = 1.0 / (1.0 + double(dx * dx + dy * dy));
            const int64_t i = int64_t(y) * w + x;
            a0 += double(v[0][i]) * weight;
            a1 += double(v[1][i]) * weight;
            a2 += double(v[2][i]) * weight;
            weight_sum += weight;
        }
    }
    if (weight_sum <= 0.0) {
        out[0] = out[1] = out[2] = 0.0f;
        return;
    }
    out[0] = float(a0 / weight_sum);
    out[1] = float(a1 / weight_sum);
    out[2] = float(a2 / weight_sum);
}

// local_avg3 / local_avg1 in double-float (the grid's fast mode): C planes, the weights
// 1 / (1 + d^2) as pairs of floats, the quotient by their sum rounded to float.
template <int C>
__device__ void local_avg_df(const float* const* v, int w, int h, int cx, int cy, float* out) {
    // 1, 1/2 and the double 1/3 as hi + lo
    const F2 wts[3] = {F2{1.0f, 0.0f}, F2{0.5f, 0.0f}, F2{0.333333343f, -9.934107758624577e-09f}};
    F2 acc[C], ws{0.0f, 0.0f};
    for (int c = 0; c < C; ++c) acc[c] = F2{0.0f, 0.0f};
    for (int dy = -1; dy <= 1; ++dy) {
        const int y = iclamps(cy + dy, 0, h - 1);
        for (int dx = -1; dx <= 1; ++dx) {
            const int x = iclamps(cx + dx, 0, w - 1);
            const F2 wt = wts[dx * dx + dy * dy];
            const int64_t i = int64_t(y) * w + x;
            for (int c = 0; c < C; ++c) acc[c] = f2_add(acc[c], f2_mul(wt, F2{v[c][i], 0.0f}));
            ws = f2_add(ws, wt);
        }
    }
    for (int c = 0; c < C; ++c) {
        const F2 q = f2_div(acc[c], ws);
        out[c] = q.h + q.l;
    }
}

// One thread per (node, task): tasks 0 .. R_FIELDS-1 are the dependencies' sensitivity and
// confidence, task R_FIELDS the node's features (blockIdx.y). The tasks are independent, so the
// double-precision chains of a node run side by side instead of one after another.
// df_bins: 0 the reference's double arithmetic (exact grid), 1 double-float on the split doubles
// of the grid, 2 double-float on a grid that holds double-float pairs
__global__ void k_node_stats(Geometry g, NodePlanes n, PixelPlanes p, float n0, int df_bins) {
    const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= g.nn) return;
    const int f = int(blockIdx.y);
    if (f < R_FIELDS) {
        const int d = c_raw_dep[f];
        const double* dep = n.grid + idx * kDeps * kDepStride + d * kDepStride;
        float sens, conf;
        const bool done = df_bins == 2   ? sensitivity_df<true>(dep, d == D_RR ? 2 : 16, n0, sens, conf)
                          : df_bins == 1 ? sensitivity_df<false>(dep, d == D_RR ? 2 : 16, n0, sens, conf)
                                         : false;
        if (!done) {
            sens = compute_sensitivity(dep, d == D_RR ? 2 : 16);
            const double mass = sample_mass(dep);
            conf = float(mass / (mass + double(n0)));
        }
        n.raw[f][idx] = sens;
        n.conf[f][idx] = conf;
        return;
    }
    const int ix = int(idx % g.nodes_x), iy = int(idx / g.nodes_x);
    const int px = iclamps(ix * g.step, 0, g.w - 1);
    const int py = iclamps(iy * g.step, 0, g.h - 1);
    float nn3[3], na3[3], nd1;
    if (df_bins) {
        local_avg_df<3>(p.f_normal, g.w, g.h, px, py, nn3);
        local_avg_df<1>(&p.f_depth, g.w, g.h, px, py, &nd1);
        local_avg_df<3>(p.f_albedo, g.w, g.h, px, py, na3);
    } else {
        local_avg3(p.f_normal, g.w, g.h, px, py, nn3);
        nd1 = local_avg1(p.f_depth, g.w, g.h, px, py);
        local_avg3(p.f_albedo, g.w, g.h, px, py, na3);
    }
    const float z = dot3(nn3[0], nn3[1], nn3[2], nn3[0], nn3[1], nn3[2]);
    if (z > 1e-8f) {
        const float sn = sqrtf(z);
        nn3[0] = nn3[0] / sn;
        nn3[1] = nn3[1] / sn;
        nn3[2] = nn3[2] / sn;
    }
    for (int c = 0; c < 3; ++c) n.n_normal[c][idx] = nn3[c];
    n.n_depth[idx] = nd1;
    for (int c = 0; c < 3; ++c) n.n_albedo[c][idx] = na3[c];
}

// The prior smoothing's weighted sums (main.cpp:817-851) in double-float (df) or in double as the
// reference sums them; the prior is their quotient rounded to float either way.
template <bool DF>
__device__ __forceinline__ void prior_sums(const Geometry& g, const NodePlanes& n, int ix, int iy, int64_t idx,
                                           float prior[R_FIELDS]) {
    const float ni0 = n.n_normal[0][idx], ni1 = n.n_normal[1][idx], ni2 = n.n_normal[2][idx];
    const float di = n.n_depth[idx];
    const float ai0 = n.n_albedo[0][idx], ai1 = n.n_albedo[1][idx], ai2 = n.n_albedo[2][idx];
    double accum[R_FIELDS], wsum[R_FIELDS];
    F2 acc2[R_FIELDS], ws2[R_FIELDS];
    for (int f = 0; f < R_FIELDS; ++f) {
        if (DF) acc2[f] = ws2[f] = F2{0.0f, 0.0f};
        else accum[f] = wsum[f] = 0.0;
    }
    for (int dy = -1; dy <= 1; ++dy) {
        const int sy = iy + dy;
        if (sy < 0 || sy >= g.nodes_y) continue;
        for (int dx = -1; dx <= 1; ++dx) {
            const int sx = ix + dx;
            if (sx < 0 || sx >= g.nodes_x) continue;
            const int64_t sidx = int64_t(sy) * g.nodes_x + sx;
            const float spatial_w = 1.0f / (1.0f + float(dx * dx + dy * dy));
            const float normal_w = fclamps(
                (dot3(ni0, ni1, ni2, n.n_normal[0][sidx], n.n_normal[1][sidx], n.n_normal[2][sidx]) + 1.0f) * 0.5f,
                0.0f, 1.0f);
            const float depth_w = expf(-4.0f * relative_depth_delta(di, n.n_depth[sidx]));
            const float albedo_w = expf(-2.5f * norm3(ai0 - n.n_albedo[0][sidx], ai1 - n.n_albedo[1][sidx],
                                                      ai2 - n.n_albedo[2][sidx]));
            if (DF) {
                // the product of the four float weights, exact in its first step
                const float p = spatial_w * normal_w;
                const F2 b2 = f2_mul(f2_mul(F2{p, __fmaf_rn(spatial_w, normal_w, -p)}, F2{depth_w, 0.0f}),
                                     F2{albedo_w, 0.0f});
                for (int f = 0; f < R_FIELDS; ++f) {
                    const F2 wn = f2_mul(b2, F2{fmaxs(0.05f, n.conf[f][sidx]), 0.0f});
                    acc2[f] = f2_add(acc2[f], f2_mul(wn, F2{n.raw[f][sidx], 0.0f}));
                    ws2[f] = f2_add(ws2[f], wn);
                }
            } else {
                const double base = double(spatial_w) * double(normal_w) * double(depth_w) * double(albedo_w);
                for (int f = 0; f < R_FIELDS; ++f) {
                    const double w_neighbor = base * double(fmaxs(0.05f, n.conf[f][sidx]));
                    accum[f] += w_neighbor * double(n.raw[f][sidx]);
                    wsum[f] += w_neighbor;
                }
            }
        }
    }
    for (int f = 0; f < R_FIELDS; ++f) {
        if (DF) {
            const bool some = ws2[f].h > 1e-8f || (ws2[f].h == 1e-8f && ws2[f].l > 0.0f);
            const F2 q = some ? f2_div(acc2[f], ws2[f]) : F2{0.0f, 0.0f};
            prior[f] = some ? q.h + q.l : n.raw[f][idx];
        } else {
            prior[f] = (wsum[f] > double(1e-8f)) ? float(accum[f] / wsum[f]) : n.raw[f][idx];
        }
    }
}

__global__ void k_node_combine(Geometry g, NodePlanes n, int df) {
    const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= g.nn) return;
    const int ix = int(idx % g.nodes_x), iy = int(idx / g.nodes_x);
    float prior[R_FIELDS], raw[R_FIELDS], conf[R_FIELDS];
    if (df) prior_sums<true>(g, n, ix, iy, idx, prior);
    else prior_sums<false>(g, n, ix, iy, idx, prior);
    for (int f = 0; f < R_FIELDS; ++f) {
        raw[f] = n.raw[f][idx];
        conf[f] = n.conf[f][idx];
        n.prior[f][idx] = prior[f];
    }
    float fin[7];
    for (int f = 0; f < 7; ++f) fin[f] = lerp_std(prior[f], raw[f], conf[f]);
    float screen[6];
    for (int c = 0; c < 6; ++c) screen[c] = lerp_std(prior[7 + c], raw[7 + c], conf[7 + c]);
    float** T = n.field;
    T[N_PIXEL][idx] = fclamps(fin[R_PIXEL], 0.0f, 1.0f);
    const float rnd[6] = {fclamps(fin[R_BRDF], 0.0f, 1.0f), fclamps(fin[R_LENS], 0.0f, 1.0f),
                          fclamps(fin[R_LIGHT_UV], 0.0f, 1.0f), fclamps(fin[R_LIGHT_SELECT], 0.0f, 1.0f),
                          fclamps(fin[R_ENV], 0.0f, 1.0f), fclamps(fin[R_RR], 0.0f, 1.0f)};
    const float rc[6] = {fclamps(conf[R_BRDF], 0.0f, 1.0f), fclamps(conf[R_LENS], 0.0f, 1.0f),
                         fclamps(conf[R_LIGHT_UV], 0.0f, 1.0f), fclamps(conf[R_LIGHT_SELECT], 0.0f, 1.0f),
                         fclamps(conf[R_ENV], 0.0f, 1.0f), fclamps(conf[R_RR], 0.0f, 1.0f)};
    T[N_PIXEL_CONF][idx] = fclamps(conf[R_PIXEL], 0.0f, 1.0f);
    T[N_BRDF_CONF][idx] = rc[0];
    T[N_LENS_CONF][idx] = rc[1];
    T[N_LIGHT_UV_CONF][idx] = rc[2];
    T[N_LIGHT_SELECT_CONF][idx] = rc[3];
    T[N_ENV_CONF][idx] = rc[4];
    T[N_RR_CONF][idx] = rc[5];
    float rel[6];
    for (int c = 0; c < 6; ++c) {
        const float relative = rnd[c] / fmaxs(1e-8f, rnd[c] + screen[c]);  // core/stats.h:48-50
        rel[c] = relative * fmins(rc[c], conf[7 + c]);
    }
    int dominant = 0;
    for (int c = 1; c < 6; ++c)
        if (rel[dominant] < rel[c]) dominant = c;
    T[N_BRDF][idx] = rel[0];
    T[N_LENS][idx] = rel[1];
    T[N_LIGHT_UV][idx] = rel[2];
    T[N_LIGHT_SELECT][idx] = rel[3];
    T[N_LIGHT][idx] = fmaxs(rel[2], rel[3]);
    T[N_ENV][idx] = rel[4];
    T[N_RR][idx] = rel[5];
    T[N_LIGHT_CONF][idx] = rel[2] >= rel[3] ? rc[2] : rc[3];
    T[N_ALL][idx] = rel[dominant];
    T[N_ALL_CONF][idx] = fmins(rc[dominant], conf[7 + dominant]);
}

// SensitivityTiles::lookup (core/buffers.h:68-87)
__device__ __forceinline__ float tiles_lookup(const Geometry& g, const float* tiles, int x, int y) {
    const float gx = float(x) / float(g.step);
    const float gy = float(y) / float(g.step);
    const int x0 = iclamps(int(floorf(gx)), 0, g.nodes_x - 1);
    const int y0 = iclamps(int(floorf(gy)), 0, g.nodes_y - 1);
    const int x1 = imins(x0 + 1, g.nodes_x - 1);
    const int y1 = imins(y0 + 1, g.nodes_y - 1);
    const float tx = fclamps(gx - float(x0), 0.0f, 1.0f);
    const float ty = fclamps(gy - float(y0), 0.0f, 1.0f);
    const float v00 = tiles[int64_t(y0) * g.nodes_x + x0];
    const float v10 = tiles[int64_t(y0) * g.nodes_x + x1];
    const float v01 = tiles[int64_t(y1) * g.nodes_x + x0];
    const float v11 = tiles[int64_t(y1) * g.nodes_x + x1];
    const float top = lerp_std(v00, v10, tx);
    const float bottom = lerp_std(v01, v11, tx);
    return lerp_std(top, bottom, ty);
}

__global__ void k_sens_pixels(Geometry g, NodePlanes n, PixelPlanes p) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= g.np) return;
    const int y = int(i / g.w), x = int(i % g.w);
    p.sens_confidence[i] = tiles_lookup(g, n.field[N_ALL_CONF], x, y);
    const float left = tiles_lookup(g, n.field[N_ALL], imaxs(0, x - 1), y);
    const float right = tiles_lookup(g, n.field[N_ALL], imins(g.w - 1, x + 1), y);
    const float up = tiles_lookup(g, n.field[N_ALL], x, imaxs(0, y - 1));
    const float down = tiles_lookup(g, n.field[N_ALL], x, imins(g.h - 1, y + 1));
    const float grad = sqrtf((right - left) * (right - left) + (down - up) * (down - up));
    p.sens_gradient[i] = fclamps(0.5f * grad, 0.0f, 1.0f);
}

__global__ void k_sens_zero(PixelPlanes p, int64_t np) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    p.sens_confidence[i] = 0.0f;
    p.sens_gradient[i] = 0.0f;
}

__constant__ int c_rpd_field[6] = {N_BRDF, N_LENS, N_LIGHT_UV, N_LIGHT_SELECT, N_ENV, N_RR};

__global__ void k_rpd_cache(Geometry g, NodePlanes n, PixelPlanes p) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= g.np) return;
    const int y = int(i / g.w), x = int(i % g.w);
    const float gradient = fclamps(p.sens_gradient[i], 0.0f, 1.0f);
    const float attenuation = 1.0f - gradient;
    for (int c = 0; c < 6; ++c) {
        const float v = fclamps(tiles_lookup(g, n.field[c_rpd_field[c]], x, y), 0.0f, 1.0f);
        p.rpd[c][i] = fclamps(v * attenuation, 0.0f, 1.0f);
    }
}

__global__ void k_expand(Geometry g, const float* tiles, float* out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= g.np) return;
    out[i] = tiles_lookup(g, tiles, int(i % g.w), int(i / g.w));
}

}  // namespace

cudaError_t launch_sensitivity(Job& j) {
    {
        KernelScope ks(j, RPD_KERNEL_NODE_STATS);
        k_node_stats<<<dim3(grid_for(j.g.nn, 128), R_FIELDS + 1), 128, 0, j.stream>>>(
            j.g, j.n, j.p, j.cfg.rpf_confidence_samples, j.grid_pairs ? 2 : j.exact_grid ? 0 : 1);
    }
    {
        KernelScope ks(j, RPD_KERNEL_NODE_COMBINE);
        k_node_combine<<<grid_for(j.g.nn, 128), 128, 0, j.stream>>>(j.g, j.n, j.exact_grid ? 0 : 1);
    }
    {
        KernelScope ks(j, RPD_KERNEL_SENS_PIXELS);
        k_sens_pixels<<<grid_for(j.g.np, 256), 256, 0, j.stream>>>(j.g, j.n, j.p);
    }
    j.launches += 3;
    return cudaGetLastError();
}

cudaError_t launch_sensitivity_zero(Job& j) {
    KernelScope ks(j, RPD_KERNEL_SENS_PIXELS);
    k_sens_zero<<<grid_for(j.g.np, 256), 256, 0, j.stream>>>(j.p, j.g.np);
    j.launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_rpd_cache(Job& j) {
    KernelScope ks(j, RPD_KERNEL_RPD_CACHE);
    k_rpd_cache<<<grid_for(j.g.np, 256), 256, 0, j.stream>>>(j.g, j.n, j.p);
    j.launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_expand(Job& j, const float* node_field, float* out) {
    KernelScope ks(j, RPD_KERNEL_OTHER);
    k_expand<<<grid_for(j.g.np, 256), 256, 0, j.stream>>>(j.g, node_field, out);
    j.launches += 1;
    return cudaGetLastError();
}

}  // namespace rpd
