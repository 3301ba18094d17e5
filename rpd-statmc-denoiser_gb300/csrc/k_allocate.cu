// The budget-preserving allocation of compute_adaptive_sample_counts (main.cpp:1329-1438)
// in parallel, with the reference's integers bit for bit.
//
// The reference's counts come out of three sequential double-precision chains over float
// addends in pixel order:
//   sum_importance        = std::accumulate(importance, 0.0)                     (1370)
//   remaining_importance -= importance[idx] at each pixel a water-filling pass
//                           clips                                                 (1387-1402)
//   cumulative           += residual_weights[cursor] in the systematic sampling   (1425-1437)
// A tree sum rounds differently, so the chains cannot be reassociated. They can still be
// evaluated exactly in parallel. While a chain value s stays inside one binade
// [2^E, 2^(E+1)), s is an integer multiple S of g = 2^(E-52), and s + x (or s - x) rounds to
// g * (S +- round(x / g)) where a tie goes to the even multiple. So each addend acts on S as a
// map from the parity of S to (integer step, new parity): two states. These maps compose
// associatively, so a chunk of 4096 addends reduces to one map by a block scan, for the
// binade (or two) the chunk is predicted to lie in. One warp then walks the chunk maps in
// order and gets the exact chain value at every chunk start. A chunk whose prediction was
// wrong, or that crosses a binade, is walked exactly by one block instead: block scans up to
// the crossing addend, that addend added in double precision as the reference adds it, and
// on from there. Every chain value the later phases need is recomputed from the chunk start
// by the same scan (or read back from the walk for a chunk walked exactly).
//
// A water-filling pass visits the active pixels in order and clips a pixel when
// importance / remaining_importance * remaining_samples > max_extra_per_pixel, with the state
// left by the clips before it. The pass's clip set is found as a fixed point: start from the
// decisions at the pass's start state, evaluate the remaining_importance chain over the
// current clip set, decide every pixel again with the chain value and sample count before it,
// and repeat until nothing changes. A pixel's decision depends only on the clips before it,
// so the fixed point is unique and equals the sequential result: each round settles at least
// one more pixel, and in practice every pixel settles in a few rounds. The active list of the
// reference keeps pixel order, so it is kept here as an alive bit per pixel (a pixel that left
// the list adds 0 to the chain, which changes no value).
//
// The systematic residual sampling gives target k, t_k = ((k + offset) / remaining) *
// residual_sum, to the first pixel whose inclusive cumulative C_j >= t_k. With C_j exact, pixel
// j receives N(C_j) - N(C_{j-1}) extra samples, where N(c) counts the t_k <= c; t_k is evaluated
// with the reference's expression wherever a cheaper estimate cannot decide the comparison.
//
// All of it is one cooperative launch (every block resident at once) whose blocks meet at
// grid barriers. Each wait there is bounded; a barrier that runs out of time, a non-finite or
// negative importance, a full pool of exactly walked chunks or a pass that does not settle
// sets a flag, and the serial allocation kernel launched behind this one then redoes the
// whole allocation in the reference's order.
#include <algorithm>
#include <cfloat>
#include <climits>

#include "rpd_internal.h"
#include "device_math.cuh"

namespace rpd {

namespace {

constexpr int kAT = 256;                // threads per block
constexpr int kAV = 8;                  // consecutive pixels per thread
constexpr int kAL = kAT * kAV;          // pixels per chunk
constexpr int kAWarps = kAT / 32;
constexpr int kTile = 128;              // chunk records staged in shared memory by the walk
constexpr int kMaxOwned = 128;          // chunks per block
constexpr int kDefaultBlocks = 1 << 20;  // blocks of the cooperative launch: one per SM unless capped
constexpr int kMaxRounds = 64;          // fixed-point rounds per water-filling pass
constexpr long long kTwo52 = 1ll << 52;
constexpr long long kTwo53 = 1ll << 53;
constexpr unsigned long long kSat = 1ull << 62;  // saturation of exact integer sums
constexpr long long kBarrierCycles = 4000000000ll;  // about two seconds at the SM clock
constexpr int kNoExp = INT_MIN;
constexpr int kNoRegion = INT_MIN;  // a chain without an exact region
constexpr int kStamps = 96;

// The action of one addend (or a run of them) on S: for input parity p, S += step[p] and the
// parity becomes bit p of `o`. Bit 2 of `o` marks an addend the binade arithmetic cannot
// take (|x / g| >= 2^52).
struct EF {
    long long i0, i1;
    unsigned o;
};

__device__ __forceinline__ EF ef_identity() { return EF{0, 0, 2u}; }

// f, then g.
__device__ __forceinline__ EF ef_compose(const EF& f, const EF& g) {
    const unsigned a0 = f.o & 1u, a1 = (f.o >> 1) & 1u;
    EF r;
    r.i0 = f.i0 + (a0 ? g.i1 : g.i0);
    r.i1 = f.i1 + (a1 ? g.i1 : g.i0);
    r.o = ((g.o >> a0) & 1u) | (((g.o >> a1) & 1u) << 1) | ((f.o | g.o) & 4u);
    // a valid run moves S by less than 2^53; far beyond that it is marked unusable and
    // clamped, so that no composition can wrap around
    constexpr long long kBig = 1ll << 60;
    if (r.i0 >= kBig || r.i0 <= -kBig || r.i1 >= kBig || r.i1 <= -kBig) {
        r.i0 = r.i0 >= kBig ? kBig : (r.i0 <= -kBig ? -kBig : r.i0);
        r.i1 = r.i1 >= kBig ? kBig : (r.i1 <= -kBig ? -kBig : r.i1);
        r.o |= 4u;
    }
    return r;
}

// s -> s + sign * x rounded to nearest-even, for s in the binade of exponent E, as an action
// on S = s / 2^(E-52). x >= 0 and finite.
__device__ __forceinline__ EF ef_make(float x, int E, int sign) {
    EF f;
    const unsigned bits = __float_as_uint(x) & 0x7fffffffu;
    if (bits == 0u) return ef_identity();
    const unsigned eb = bits >> 23;
    const long long m = eb ? (long long)((bits & 0x7fffffu) | 0x800000u) : (long long)bits;
    const int e = eb ? int(eb) - 150 : -149;  // x = m * 2^e
    const int sh = e - (E - 52);              // x / g = m * 2^sh
    long long q;
    int cls;                                  // 0: below half, 1: above half, 2: tie
    if (sh >= 0) {
        if (sh > 40) {
            f.i0 = f.i1 = 0;
            f.o = 6u;
            return f;
        }
        q = m << sh;
        cls = 0;
    } else {
        const int k = -sh;
        if (k > 25) return ef_identity();     // x < g / 2: s is unchanged
        q = m >> k;
        const long long rem = m & ((1ll << k) - 1);
        const long long half = 1ll << (k - 1);
        cls = rem > half ? 1 : (rem == half ? 2 : 0);
    }
    if (q >= kTwo52) {
        f.i0 = f.i1 = 0;
        f.o = 6u;
        return f;
    }
    if (cls == 2) {
        // the rounded result is the even one of S + q and S + q + 1 (or S - q, S - q - 1)
        const long long v0 = q + (q & 1), v1 = q + ((q + 1) & 1);
        f.i0 = sign > 0 ? v0 : -v0;
        f.i1 = sign > 0 ? v1 : -v1;
        f.o = 0u;
    } else {
        const long long v = q + cls;
        f.i0 = f.i1 = sign > 0 ? v : -v;
        f.o = (v & 1) ? 1u : 2u;
    }
    return f;
}

__device__ __forceinline__ double pow2d(int k) {  // 2^k for -1022 <= k <= 1023
    return __longlong_as_double((long long)(k + 1023) << 52);
}
// The binade arithmetic works on the bits of the double, with no double-precision instruction
// (GB300 issues those at 2 per SM per clock): a positive normal s = S * 2^(E-52) with S in
// [2^52, 2^53) has exponent field E + 1023 and mantissa field S - 2^52.
__device__ __forceinline__ int exponent_of(double s) {
    return int((__double_as_longlong(s) >> 52) & 0x7ff) - 1023;
}
// A value the binade arithmetic handles: positive and normal, far from the ends of the range.
__device__ __forceinline__ bool binade_ok(double s) {
    const long long b = __double_as_longlong(s);
    const int e = int((b >> 52) & 0x7ff) - 1023;  // the sign bit lands in bit 11 of the field
    return b > 0 && e > -900 && e < 900;
}
__device__ __forceinline__ bool stays_in_binade(long long S, int sign) {
    // adding: every exact sum stays below 2^(E+1); subtracting: every exact difference stays
    // at or above 2^E (S >= 2^52 + 1 keeps the unrounded value above the binade's floor)
    return sign > 0 ? S < kTwo53 : S > kTwo52;
}
// S of s, for s in the binade of exponent E
__device__ __forceinline__ long long scaled(double s, int) {
    return (__double_as_longlong(s) & (kTwo52 - 1)) | kTwo52;
}
// the double S * 2^(E-52), for S in [2^52, 2^53)
__device__ __forceinline__ double unscaled(long long S, int E) {
    return __longlong_as_double((static_cast<long long>(E + 1023) << 52) | (S - kTwo52));
}
// float(s) rounded toward zero, from the bits (the clip test's screen only needs 2^-23)
__device__ __forceinline__ float float_trunc(double s) {
    const long long b = __double_as_longlong(s);
    const int e = int((b >> 52) & 0x7ff) - 1023;
    if (b <= 0 || e < -126 || e > 127) return float(s);
    return __uint_as_float((unsigned(e + 127) << 23) | unsigned((b >> 29) & 0x7fffff));
}

// ---- the exact region of a sum from zero -------------------------------------------------------
// While every partial sum of nonnegative floats from 0 stays below 2^(53-F), where 2^-F is the
// smallest unit in last place among the addends, no addition rounds: every partial sum is an
// integer multiple of 2^-F below 2^53 units, which a double holds exactly. There the chain value is
// the exact sum, evaluated as a 64-bit integer count of 2^-F units in any order.
__device__ __forceinline__ int float_exp(float x) {  // x = m * 2^e with the integer mantissa m
    const unsigned eb = (__float_as_uint(x) >> 23) & 0xffu;
    return eb ? int(eb) - 150 : -149;
}
// x * 2^F for x >= 0 (F >= -e for every addend), saturated at 2^62
__device__ __forceinline__ unsigned long long int_units(float x, int F) {
    const unsigned bits = __float_as_uint(x) & 0x7fffffffu;
    if (bits == 0u) return 0ull;
    const unsigned eb = bits >> 23;
    const unsigned long long m = eb ? (unsigned long long)((bits & 0x7fffffu) | 0x800000u) : bits;
    const int sh = float_exp(x) + F;
    if (sh < 0 || sh > 38) return kSat;
    return m << sh;
}
__device__ __forceinline__ unsigned long long sat_add(unsigned long long a, unsigned long long b) {
    const unsigned long long t = a + b;  // both at most 2^62: no wrap
    return t > kSat ? kSat : t;
}
// P * 2^-F for P < 2^53 (exact), from the bits
__device__ __forceinline__ double units_to_double(unsigned long long P, int F) {
    if (P == 0ull) return 0.0;
    const int top = 63 - __clzll((long long)P);
    const unsigned long long mant = (P << (52 - top)) & (unsigned long long)(kTwo52 - 1);
    return __longlong_as_double(((long long)(top - F + 1023) << 52) | (long long)mant);
}
// F of a chain from the largest (1000 - e) the addends reported (0: no nonzero addend)
__device__ __forceinline__ int region_f(int code) {
    const int F = code - 1000;
    return (code > 0 && F >= -900 && F <= 900) ? F : kNoRegion;
}

struct __align__(16) ChunkRec {
    long long i0[2];   // chunk action for the candidate exponents E[0], E[1]
    long long i1[2];
    unsigned o[2];
    int E[2];
    double approx;     // approximate sum of the chunk's addends (predictions only)
    int clips;         // clipped pixels of the chunk (water-filling chain)
    int len;           // pixels in the chunk
    unsigned long long isum;  // exact sum of the chunk's addends in units of 2^-F (saturated)
    // written by the walk
    double start;      // exact chain value before the chunk
    int mode;          // 0/1: walked with candidate mode; 2: walked exactly, values in the pool;
                       // 3: inside the exact region; 4: split at a binade crossing
    int slot;          // pool slot of an exactly walked chunk
    int nb;            // clipped pixels before the chunk
    int pad;
    unsigned long long pstart;  // units before the chunk (mode 3)
    int split;         // >= 0: the chunk crosses into the next binade at this pixel; action 0 covers
                       // the pixels before it (binade E[0]) and action 1 the pixels after (E[1])
    float xval;        // the addend at the split pixel
    double xstart;     // written by the walk: the chain value after the split pixel (mode 4)
};

static_assert(sizeof(ChunkRec) % 16 == 0, "the walk copies records as 16-byte words");

struct AllocScalars {
    unsigned bar_count;
    unsigned bar_gen;
    int error;
    int fallback;
    unsigned long long changed;  // running count of decisions that changed between rounds
    unsigned long long start_clips;  // running count of the clips decided at the passes' start states
    double walk_final;
    long long assigned;
    int walk_clips;
    int passes;
    int rounds;
    int exact_chunks;
    int done;                    // the parallel allocation finished
    int reason;                  // why it handed over: 1 input, 2 pool, 3 rounds, 4 barrier, 5 no launch
    int n_stamps;
    int region_code[2];          // largest 1000 - e over the nonzero importances (0) and residuals (1)
    int pad;
    unsigned long long stamps[kStamps];  // %globaltimer (ns) at the start and after each barrier
};

constexpr uint64_t kScalarBytes = (sizeof(AllocScalars) + 255) & ~uint64_t(255);

struct CoopArgs {
    const float* importance;
    float* desired_add;
    float* residual;
    int32_t* counts;
    uint8_t* state;       // per pixel: bit 0 alive, bits 1 and 2 the two clip-flag buffers
    ChunkRec* rec;
    double* pool;
    AllocScalars* sc;
    int64_t np;
    int nch;
    int pool_chunks;
    int extra_sample_total;
    int reserved_samples;
    int max_extra;
    uint32_t seed;
};

// ---- grid barrier (bounded) ----------------------------------------------------------------
__device__ bool grid_sync(AllocScalars* sc) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &sc->bar_gen;
        volatile int* verr = &sc->error;
        const unsigned g = *vgen;
        __threadfence();
        if (atomicAdd(&sc->bar_count, 1u) == gridDim.x - 1) {
            atomicExch(&sc->bar_count, 0u);
            __threadfence();
            atomicAdd(&sc->bar_gen, 1u);
        } else {
            const long long t0 = clock64();
            while (*vgen == g && *verr == 0) {
                __nanosleep(64);
                if (clock64() - t0 > kBarrierCycles) {
                    atomicExch(&sc->error, 1);
                    atomicExch(&sc->reason, 4);
                    atomicExch(&sc->fallback, 1);
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0 && sc->n_stamps < kStamps) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        sc->stamps[sc->n_stamps++] = t;
    }
    return *(volatile int*)&sc->error == 0;
}

__device__ __forceinline__ bool fell_back(AllocScalars* sc) { return *(volatile int*)&sc->fallback != 0; }

// ---- block-level helpers --------------------------------------------------------------------
struct Shared {
    EF warp_ef[2][kAWarps];
    float2 warp_f2[kAWarps];
    long long warp_l[kAWarps];
    int warp_i[kAWarps];
    double own_pred[kMaxOwned];
    ChunkRec tile[kTile];
    float xs[kAL];  // the addends of the chunk an exact walk is on
    double bcast_d;
    int bcast_i;
    int bcast_j;
    int bcast_k;
};

__device__ __forceinline__ EF shfl_up_ef(const EF& f, int d) {
    EF o;
    o.i0 = __shfl_up_sync(0xffffffffu, f.i0, d);
    o.i1 = __shfl_up_sync(0xffffffffu, f.i1, d);
    o.o = __shfl_up_sync(0xffffffffu, f.o, d);
    return o;
}

// Exclusive scan of the threads' actions in thread order; *total gets the block's action.
// Two independent scans (two candidate exponents) share the synchronisation.
template <int N>
__device__ void block_scan_ef(EF (&tf)[N], EF (&ex)[N], EF (&total)[N], Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    EF inc[N];
#pragma unroll
    for (int n = 0; n < N; ++n) inc[n] = tf[n];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
        for (int n = 0; n < N; ++n) {
            const EF o = shfl_up_ef(inc[n], d);
            if (lane >= d) inc[n] = ef_compose(o, inc[n]);
        }
    }
    if (lane == 31)
#pragma unroll
        for (int n = 0; n < N; ++n) sh.warp_ef[n][warp] = inc[n];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int n = 0; n < N; ++n) {
            EF w = lane < kAWarps ? sh.warp_ef[n][lane] : ef_identity();
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const EF o = shfl_up_ef(w, d);
                if (lane >= d) w = ef_compose(o, w);
            }
            if (lane < kAWarps) sh.warp_ef[n][lane] = w;
        }
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < N; ++n) {
        EF lane_ex = shfl_up_ef(inc[n], 1);
        if (lane == 0) lane_ex = ef_identity();
        ex[n] = warp ? ef_compose(sh.warp_ef[n][warp - 1], lane_ex) : lane_ex;
        total[n] = sh.warp_ef[n][kAWarps - 1];
    }
    __syncthreads();
}

// Double-float (h + l) sums for the approximate chain values: the chunk sums, their prefix and the
// split prediction need about 2^-40 relative accuracy, which pairs of floats give on the FP32 pipes
// (a chain of double-precision additions waits on each one at 2 per SM per clock).
struct DF {
    float h, l;
};

__device__ __forceinline__ void df_acc(DF& a, float x) {  // a += x, the rounding error kept in l
    const float s = a.h + x;
    const float bb = s - a.h;
    a.l += (a.h - (s - bb)) + (x - bb);
    a.h = s;
}

__device__ __forceinline__ DF df_sum(DF a, DF b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b.h - bb);
    const float l = e + (a.l + b.l);
    const float h = s + l;
    return DF{h, l - (h - s)};
}

__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }
__device__ __forceinline__ double df_value(DF a) { return double(a.h) + double(a.l); }
__device__ __forceinline__ DF df_of(double v) {
    const float h = __double2float_rn(v);
    return DF{h, __double2float_rn(v - double(h))};
}
__device__ __forceinline__ DF shfl_down_df(DF a, int d) {
    return DF{__shfl_down_sync(0xffffffffu, a.h, d), __shfl_down_sync(0xffffffffu, a.l, d)};
}
__device__ __forceinline__ DF shfl_up_df(DF a, int d) {
    return DF{__shfl_up_sync(0xffffffffu, a.h, d), __shfl_up_sync(0xffffffffu, a.l, d)};
}

__device__ DF block_sum_df(DF v, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = df_sum(v, shfl_down_df(v, d));
    if (lane == 0) sh.warp_f2[warp] = make_float2(v.h, v.l);
    __syncthreads();
    DF t{0.0f, 0.0f};
    for (int w = 0; w < kAWarps; ++w) t = df_sum(t, DF{sh.warp_f2[w].x, sh.warp_f2[w].y});
    __syncthreads();
    return t;
}

// Exclusive scan of double-floats over the block's threads; *total gets the block's sum.
__device__ DF block_exscan_df(DF v, DF* total, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    DF inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const DF o = shfl_up_df(inc, d);
        if (lane >= d) inc = df_sum(o, inc);
    }
    DF ex = shfl_up_df(inc, 1);
    if (lane == 0) ex = DF{0.0f, 0.0f};
    if (lane == 31) sh.warp_f2[warp] = make_float2(inc.h, inc.l);
    __syncthreads();
    DF before{0.0f, 0.0f}, all{0.0f, 0.0f};
    for (int w = 0; w < kAWarps; ++w) {
        const DF t{sh.warp_f2[w].x, sh.warp_f2[w].y};
        if (w < warp) before = df_sum(before, t);
        all = df_sum(all, t);
    }
    __syncthreads();
    *total = all;
    return df_sum(before, ex);
}

__device__ float block_sum_f(float v, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    if (lane == 0) sh.warp_i[warp] = __float_as_int(v);
    __syncthreads();
    float t = 0.0f;
    for (int w = 0; w < kAWarps; ++w) t += __int_as_float(sh.warp_i[w]);
    __syncthreads();
    return t;
}

__device__ int block_max_i(int v, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, d));
    if (lane == 0) sh.warp_i[warp] = v;
    __syncthreads();
    int t = INT_MIN;
    for (int w = 0; w < kAWarps; ++w) t = max(t, sh.warp_i[w]);
    __syncthreads();
    return t;
}

__device__ long long block_sum_l(long long v, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    if (lane == 0) sh.warp_l[warp] = v;
    __syncthreads();
    long long t = 0;
    for (int w = 0; w < kAWarps; ++w) t += sh.warp_l[w];
    __syncthreads();
    return t;
}

// Exclusive scan of an int over threads; *total gets the sum.
__device__ int block_scan_i(int v, int* total, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += o;
    }
    if (lane == 31) sh.warp_i[warp] = inc;
    __syncthreads();
    int before = 0, all = 0;
    for (int w = 0; w < kAWarps; ++w) {
        if (w < warp) before += sh.warp_i[w];
        all += sh.warp_i[w];
    }
    __syncthreads();
    *total = all;
    return before + inc - v;
}

// Exclusive scan of an unsigned 64-bit value over threads (values small enough not to wrap).
__device__ unsigned long long block_scan_u64(unsigned long long v, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long o = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += o;
    }
    if (lane == 31) sh.warp_l[warp] = (long long)inc;
    __syncthreads();
    unsigned long long before = 0;
    for (int w = 0; w < warp; ++w) before += (unsigned long long)sh.warp_l[w];
    __syncthreads();
    return before + inc - v;
}

__device__ int block_min_i(int v, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = min(v, __shfl_down_sync(0xffffffffu, v, d));
    if (lane == 0) sh.warp_i[warp] = v;
    __syncthreads();
    int t = INT_MAX;
    for (int w = 0; w < kAWarps; ++w) t = min(t, sh.warp_i[w]);
    __syncthreads();
    return t;
}

// ---- per-thread pixel loads -------------------------------------------------------------------
__device__ __forceinline__ void load_f8(const float* p, int64_t k0, int64_t np, float (&x)[kAV]) {
    if (k0 + kAV <= np) {
        const float4 a = __ldcg(reinterpret_cast<const float4*>(p + k0));
        const float4 b = __ldcg(reinterpret_cast<const float4*>(p + k0 + 4));
        x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
        x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
    } else {
#pragma unroll
        for (int e = 0; e < kAV; ++e) x[e] = (k0 + e < np) ? __ldcg(p + k0 + e) : 0.0f;
    }
}
__device__ __forceinline__ void load_u8(const uint8_t* p, int64_t k0, int64_t np, uint8_t (&s)[kAV]) {
    if (k0 + kAV <= np) {
        const uint2 v = __ldcg(reinterpret_cast<const uint2*>(p + k0));
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            s[e] = uint8_t(v.x >> (8 * e));
            s[e + 4] = uint8_t(v.y >> (8 * e));
        }
    } else {
#pragma unroll
        for (int e = 0; e < kAV; ++e) s[e] = (k0 + e < np) ? __ldcg(p + k0 + e) : uint8_t(0);
    }
}
__device__ __forceinline__ void store_u8(uint8_t* p, int64_t k0, int64_t np, const uint8_t (&s)[kAV]) {
    if (k0 + kAV <= np) {
        uint2 v;
        v.x = uint32_t(s[0]) | uint32_t(s[1]) << 8 | uint32_t(s[2]) << 16 | uint32_t(s[3]) << 24;
        v.y = uint32_t(s[4]) | uint32_t(s[5]) << 8 | uint32_t(s[6]) << 16 | uint32_t(s[7]) << 24;
        *reinterpret_cast<uint2*>(p + k0) = v;
    } else {
#pragma unroll
        for (int e = 0; e < kAV; ++e)
            if (k0 + e < np) p[k0 + e] = s[e];
    }
}

// The chain's addends: 0 importance, 1 importance of alive pixels flagged in buffer `fbit`,
// 2 residual weights.
struct Src {
    int kind;
    unsigned fbit;
    __device__ __forceinline__ void load(const CoopArgs& a, int64_t k0, float (&x)[kAV]) const {
        if (kind == 2) {
            load_f8(a.residual, k0, a.np, x);
            return;
        }
        load_f8(a.importance, k0, a.np, x);
        if (kind == 1) {
            uint8_t s[kAV];
            load_u8(a.state, k0, a.np, s);
#pragma unroll
            for (int e = 0; e < kAV; ++e)
                if (!((s[e] & 1u) && (s[e] & fbit))) x[e] = 0.0f;
        }
    }
};

// Chunk actions for up to two candidate exponents; writes them to the record.
__device__ void chunk_actions(const float (&x)[kAV], int E0, int E1, int sign, ChunkRec* r, Shared& sh) {
    if (E1 == kNoExp) {  // one candidate: one scan
        EF tf[1], ex[1], tot[1];
        tf[0] = ef_identity();
        if (E0 != kNoExp)
#pragma unroll
            for (int e = 0; e < kAV; ++e) tf[0] = ef_compose(tf[0], ef_make(x[e], E0, sign));
        block_scan_ef<1>(tf, ex, tot, sh);
        if (threadIdx.x == 0) {
            r->i0[0] = tot[0].i0;
            r->i1[0] = tot[0].i1;
            r->o[0] = E0 == kNoExp ? 6u : tot[0].o;
            r->E[0] = E0;
            r->i0[1] = r->i1[1] = 0;
            r->o[1] = 6u;
            r->E[1] = kNoExp;
            r->split = -1;
        }
        return;
    }
    EF tf[2], ex[2], tot[2];
    tf[0] = ef_identity();
    tf[1] = ef_identity();
#pragma unroll
    for (int e = 0; e < kAV; ++e) {
        if (E0 != kNoExp) tf[0] = ef_compose(tf[0], ef_make(x[e], E0, sign));
        tf[1] = ef_compose(tf[1], ef_make(x[e], E1, sign));
    }
    block_scan_ef<2>(tf, ex, tot, sh);
    if (threadIdx.x == 0) {
        for (int n = 0; n < 2; ++n) {
            const int En = n ? E1 : E0;
            r->i0[n] = tot[n].i0;
            r->i1[n] = tot[n].i1;
            r->o[n] = En == kNoExp ? 6u : tot[n].o;
            r->E[n] = En;
        }
        r->split = -1;
    }
}

// The exact chain values (inclusive) of this thread's pixels in chunk c after the walk, and
// the value before the thread's first pixel. F is the chain's exact-region unit (kNoRegion: none).
__device__ void chain_values(const CoopArgs& a, int c, const float (&x)[kAV], int sign, int F, double (&v)[kAV],
                             double* before, Shared& sh) {
    const int mode = __ldcg(&a.rec[c].mode);
    const double start = __ldcg(&a.rec[c].start);
    const int base = threadIdx.x * kAV;
    if (mode == 3) {
        unsigned long long u[kAV], t = 0;
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            u[e] = int_units(x[e], F);
            t += u[e];
        }
        unsigned long long P = __ldcg(&a.rec[c].pstart) + block_scan_u64(t, sh);
        *before = units_to_double(P, F);
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            P += u[e];
            v[e] = units_to_double(P, F);
        }
    } else if (mode == 4) {
        // before the split pixel kx in binade E[0] from the start, kx itself, after it in E[1]
        const int kx = __ldcg(&a.rec[c].split);
        const int EA = __ldcg(&a.rec[c].E[0]), EB = __ldcg(&a.rec[c].E[1]);
        const double sx = __ldcg(&a.rec[c].xstart);
        EF fa[kAV], fb[kAV], tf[2], ex[2], tot[2];
        tf[0] = ef_identity();
        tf[1] = ef_identity();
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            fa[e] = base + e < kx ? ef_make(x[e], EA, sign) : ef_identity();
            fb[e] = base + e > kx ? ef_make(x[e], EB, sign) : ef_identity();
            tf[0] = ef_compose(tf[0], fa[e]);
            tf[1] = ef_compose(tf[1], fb[e]);
        }
        block_scan_ef<2>(tf, ex, tot, sh);
        long long SA = scaled(start, EA);
        const unsigned pa0 = unsigned(SA & 1);
        SA += pa0 ? ex[0].i1 : ex[0].i0;
        unsigned pa = (ex[0].o >> pa0) & 1u;
        long long SB = scaled(sx, EB);
        const unsigned pb0 = unsigned(SB & 1);
        SB += pb0 ? ex[1].i1 : ex[1].i0;
        unsigned pb = (ex[1].o >> pb0) & 1u;
        *before = base <= kx ? unscaled(SA, EA) : unscaled(SB, EB);
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            const int idx = base + e;
            if (idx < kx) {
                SA += pa ? fa[e].i1 : fa[e].i0;
                pa = (fa[e].o >> pa) & 1u;
                v[e] = unscaled(SA, EA);
            } else if (idx == kx) {
                v[e] = sx;
            } else {
                SB += pb ? fb[e].i1 : fb[e].i0;
                pb = (fb[e].o >> pb) & 1u;
                v[e] = unscaled(SB, EB);
            }
        }
    } else if (mode < 2) {
        const int E = __ldcg(&a.rec[c].E[mode]);
        EF tf[1], ex[1], tot[1];
        EF f[kAV];
        tf[0] = ef_identity();
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            f[e] = ef_make(x[e], E, sign);
            tf[0] = ef_compose(tf[0], f[e]);
        }
        block_scan_ef<1>(tf, ex, tot, sh);
        long long S = scaled(start, E);
        const unsigned p0 = unsigned(S & 1);
        S += p0 ? ex[0].i1 : ex[0].i0;
        unsigned p = (ex[0].o >> p0) & 1u;
        *before = unscaled(S, E);
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            S += p ? f[e].i1 : f[e].i0;
            p = (f[e].o >> p) & 1u;
            v[e] = unscaled(S, E);
        }
    } else {
        const int slot = __ldcg(&a.rec[c].slot);
        const double* pv = a.pool + int64_t(slot) * kAL;
        *before = base == 0 ? start : __ldcg(pv + base - 1);
#pragma unroll
        for (int e = 0; e < kAV; ++e) v[e] = __ldcg(pv + base + e);
    }
}

// ---- the walk (block 0) -----------------------------------------------------------------------
// Chunk c walked exactly from value s: block scans within the binade, the crossing addend in
// double precision. Stores every inclusive value in the pool slot when `slot` >= 0.
// After a binade crossing that came within kDenseGap addends of the previous position, the next
// kBurst addends are added one at a time by one thread (a sum from near zero crosses a binade
// every few addends, and a block scan per crossing costs more than the additions).
constexpr int kDenseGap = 64;
constexpr int kBurst = 128;

__device__ double walk_exact(const CoopArgs& a, const Src& src, int c, double s, int sign, int slot, Shared& sh) {
    const int len = __ldcg(&a.rec[c].len);
    const int64_t k0 = int64_t(c) * kAL + threadIdx.x * kAV;
    const int base = threadIdx.x * kAV;
    float x[kAV];
    src.load(a, k0, x);
#pragma unroll
    for (int e = 0; e < kAV; ++e) sh.xs[base + e] = x[e];
    __syncthreads();
    double* pv = slot >= 0 ? a.pool + int64_t(slot) * kAL : nullptr;
    int pos = 0;  // first pixel not yet walked
    bool dense = false;
    while (pos < len) {
        if (dense && binade_ok(s)) {
            const int end = min(pos + kBurst, len);
            if (threadIdx.x == 0) {
                double t = s;
                for (int k = pos; k < end; ++k) {
                    const double xe = double(sh.xs[k]);
                    t = sign > 0 ? t + xe : t - xe;
                    if (pv) pv[k] = t;
                }
                sh.bcast_d = t;
            }
            __syncthreads();
            s = sh.bcast_d;
            __syncthreads();
            pos = end;
            dense = false;
            continue;
        }
        if (!binade_ok(s)) {
            // s is zero, negative or extreme: walk to the next nonzero addend one at a time
            int first = INT_MAX;
#pragma unroll
            for (int e = 0; e < kAV; ++e)
                if (base + e >= pos && base + e < len && x[e] != 0.0f) first = min(first, base + e);
            const int kz = min(block_min_i(first, sh), len);
            if (pv)
#pragma unroll
                for (int e = 0; e < kAV; ++e)
                    if (base + e >= pos && base + e < kz) pv[base + e] = s;
            if (kz < len) {
                if (kz / kAV == int(threadIdx.x)) {
                    const double xe = double(x[kz % kAV]);
                    const double t = sign > 0 ? s + xe : s - xe;
                    sh.bcast_d = t;
                    if (pv) pv[kz] = t;
                }
                __syncthreads();
                s = sh.bcast_d;
                __syncthreads();
            }
            pos = kz + 1;
            continue;
        }
        const int E = exponent_of(s);
        const long long S0 = scaled(s, E);
        const unsigned p0 = unsigned(S0 & 1);
        EF f[kAV];
        EF tf[1], ex[1], tot[1];
        tf[0] = ef_identity();
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            f[e] = (base + e >= pos && base + e < len) ? ef_make(x[e], E, sign) : ef_identity();
            tf[0] = ef_compose(tf[0], f[e]);
        }
        block_scan_ef<1>(tf, ex, tot, sh);
        long long S = S0 + (p0 ? ex[0].i1 : ex[0].i0);
        unsigned p = (ex[0].o >> p0) & 1u;
        bool bad = (ex[0].o & 4u) != 0;
        int first_bad = INT_MAX;
        double vals[kAV];
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            vals[e] = 0.0;
            if (base + e < pos || base + e >= len) continue;
            bad = bad || (f[e].o & 4u);
            S += p ? f[e].i1 : f[e].i0;
            p = (f[e].o >> p) & 1u;
            if (!bad && !stays_in_binade(S, sign)) bad = true;
            if (bad) {
                first_bad = min(first_bad, base + e);
            } else {
                vals[e] = unscaled(S, E);
            }
        }
        const int kb = min(block_min_i(first_bad, sh), len);
        // the pixels before kb are exact; kb (if any) crosses the binade
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            const int idx = base + e;
            if (idx >= pos && idx < kb) {
                if (pv) pv[idx] = vals[e];
                if (idx == kb - 1) sh.bcast_d = vals[e];
            }
        }
        __syncthreads();
        const double prev = kb > pos ? sh.bcast_d : s;
        __syncthreads();
        if (kb < len) {
            if (kb / kAV == int(threadIdx.x)) {
                const double xe = double(x[kb % kAV]);
                const double t = sign > 0 ? prev + xe : prev - xe;
                sh.bcast_d = t;
                if (pv) pv[kb] = t;
            }
            __syncthreads();
            s = sh.bcast_d;
            __syncthreads();
            dense = kb - pos < kDenseGap;
            pos = kb + 1;
        } else {
            s = prev;
            pos = len;
        }
    }
    __syncthreads();  // sh.xs is rewritten by the next exact walk
    return s;
}

// Walks every chunk in order from s0. Block 0 only; writes start/mode/slot/nb of each chunk
// and the final value and clip count to the scalars.
__device__ void walk(const CoopArgs& a, const Src& src, double s0, int sign, bool keep_values, int F, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double s = s0;
    // the exact region of a sum from zero (warp 0's state only)
    bool region = F != kNoRegion && sign > 0 && s0 == 0.0;
    unsigned long long P = 0;
    int clips = 0;
    int pool_used = 0;
    int exact = 0;
    bool full = false;
    for (int t0 = 0; t0 < a.nch && !full; t0 += kTile) {
        const int tn = min(kTile, a.nch - t0);
        __syncthreads();
        {
            const int words = tn * int(sizeof(ChunkRec) / 16);
            const int4* srcw = reinterpret_cast<const int4*>(a.rec + t0);
            int4* dstw = reinterpret_cast<int4*>(sh.tile);
            for (int w = threadIdx.x; w < words; w += kAT) dstw[w] = __ldcg(srcw + w);
        }
        __syncthreads();
        int c = 0;
        while (c < tn) {
            if (warp == 0) {
                // 32 chunks per step: every lane takes the next chunk, the lanes' chunk maps are
                // composed by a warp scan, and the chunks before the first one that does not fit
                // (a missed binade, a crossing) are committed together
                while (c < tn) {
                    const int cl = c + lane;
                    const bool have = cl < tn;
                    const ChunkRec* r = &sh.tile[have ? cl : c];
                    int cinc = have ? r->clips : 0;  // inclusive clip count over the lanes
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const int o = __shfl_up_sync(0xffffffffu, cinc, d);
                        if (lane >= d) cinc += o;
                    }
                    const int cexc = cinc - (have ? r->clips : 0);
                    int k;
                    if (region) {
                        unsigned long long u = have ? r->isum : kSat;
#pragma unroll
                        for (int d = 1; d < 32; d <<= 1) {
                            const unsigned long long o = __shfl_up_sync(0xffffffffu, u, d);
                            if (lane >= d) u = sat_add(u, o);
                        }
                        const unsigned long long uexc = sat_add(u, 0) - (have && r->isum < kSat ? r->isum : 0);
                        const bool fits = have && u < kSat && P + u < (unsigned long long)kTwo53;
                        const unsigned bad = __ballot_sync(0xffffffffu, !fits);
                        k = bad ? __ffs(bad) - 1 : 32;
                        if (lane < k) {
                            ChunkRec* g = a.rec + t0 + cl;
                            g->start = units_to_double(P + uexc, F);
                            g->mode = 3;
                            g->slot = -1;
                            g->nb = clips + cexc;
                            g->pstart = P + uexc;
                        }
                        if (k > 0) {
                            P += __shfl_sync(0xffffffffu, u, k - 1);
                            s = units_to_double(P, F);
                            clips += __shfl_sync(0xffffffffu, cinc, k - 1);
                            c += k;
                        }
                        // a chunk that does not fit ends the region (not the end of the tile); s holds
                        // the exact sum so far and the binade walk goes on from it
                        if (k < 32 && c < tn) region = false;
                        continue;
                    } else {
                        if (!binade_ok(s)) break;
                        const int E = exponent_of(s);
                        const long long S = scaled(s, E);
                        const unsigned p0 = unsigned(S & 1);
                        int q = -1;
                        if (have && r->split < 0)
                            q = (r->E[0] == E && !(r->o[0] & 4u)) ? 0 : ((r->E[1] == E && !(r->o[1] & 4u)) ? 1 : -1);
                        EF f;
                        if (q >= 0) {
                            f.i0 = r->i0[q];
                            f.i1 = r->i1[q];
                            f.o = r->o[q];
                        } else {
                            f.i0 = f.i1 = 0;
                            f.o = 6u;
                        }
#pragma unroll
                        for (int d = 1; d < 32; d <<= 1) {
                            const EF o = shfl_up_ef(f, d);
                            if (lane >= d) f = ef_compose(o, f);
                        }
                        const long long Se = S + (p0 ? f.i1 : f.i0);
                        const bool ok = have && !(f.o & 4u) && stays_in_binade(Se, sign);
                        const unsigned bad = __ballot_sync(0xffffffffu, !ok);
                        k = bad ? __ffs(bad) - 1 : 32;
                        long long Sx = __shfl_up_sync(0xffffffffu, Se, 1);
                        if (lane == 0) Sx = S;
                        if (lane < k) {
                            ChunkRec* g = a.rec + t0 + cl;
                            g->start = unscaled(Sx, E);
                            g->mode = q;
                            g->slot = -1;
                            g->nb = clips + cexc;
                        }
                        if (k > 0) s = unscaled(__shfl_sync(0xffffffffu, Se, k - 1), E);
                    }
                    if (k > 0) clips += __shfl_sync(0xffffffffu, cinc, k - 1);
                    c += k;
                    if (k == 0) {
                        // a split chunk: the pixels before the predicted crossing in binade E, the
                        // crossing pixel added as the reference adds it, the rest in binade E + 1
                        const ChunkRec& r0 = sh.tile[c];
                        bool ok = false;
                        if (r0.split >= 0 && sign > 0 && binade_ok(s) && exponent_of(s) == r0.E[0] &&
                            !((r0.o[0] | r0.o[1]) & 4u)) {
                            const int E = r0.E[0];
                            const long long S = scaled(s, E);
                            const long long SA = S + ((S & 1) ? r0.i1[0] : r0.i0[0]);
                            if (stays_in_binade(SA, 1)) {
                                const double sx = unscaled(SA, E) + double(r0.xval);
                                if (binade_ok(sx) && exponent_of(sx) == E + 1) {
                                    const long long Sx = scaled(sx, E + 1);
                                    const long long SB = Sx + ((Sx & 1) ? r0.i1[1] : r0.i0[1]);
                                    if (stays_in_binade(SB, 1)) {
                                        ok = true;
                                        if (lane == 0) {
                                            ChunkRec* g = a.rec + t0 + c;
                                            g->start = s;
                                            g->mode = 4;
                                            g->slot = -1;
                                            g->nb = clips;
                                            g->xstart = sx;
                                        }
                                        s = unscaled(SB, E + 1);
                                        clips += r0.clips;
                                        ++c;
                                    }
                                }
                            }
                        }
                        if (!ok) break;  // chunk c is walked exactly
                    }
                }
                if (lane == 0) {
                    sh.bcast_d = s;
                    sh.bcast_i = c;
                    sh.bcast_j = clips;
                }
            }
            __syncthreads();
            s = sh.bcast_d;
            c = sh.bcast_i;
            clips = sh.bcast_j;
            __syncthreads();
            if (c < tn) {
                const int cc = t0 + c;
                int slot = -1;
                if (keep_values) {
                    if (pool_used >= a.pool_chunks) {
                        full = true;
                        break;
                    }
                    slot = pool_used++;
                }
                if (threadIdx.x == 0) {
                    ChunkRec* g = a.rec + cc;
                    g->start = s;
                    g->mode = 2;
                    g->slot = slot;
                    g->nb = clips;
                }
                s = walk_exact(a, src, cc, s, sign, slot, sh);
                clips += sh.tile[c].clips;
                ++exact;
                ++c;
            }
        }
    }
    if (threadIdx.x == 0) {
        if (full) {
            atomicExch(&a.sc->reason, 2);
            atomicExch(&a.sc->fallback, 1);
        }
        a.sc->walk_final = s;
        a.sc->walk_clips = clips;
        a.sc->exact_chunks += exact;
    }
}

// ---- phases -----------------------------------------------------------------------------------
// Approximate prefix of the chunks' addend sums from s0 for this block's chunks, then the chunk
// actions for the predicted binade (and the neighbouring one when the prediction is close to a
// binade edge).
// Saturating sum of unsigned values over the block (at most 2^62 each).
__device__ unsigned long long block_sum_sat(unsigned long long v, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = sat_add(v, __shfl_down_sync(0xffffffffu, v, d));
    if (lane == 0) sh.warp_l[warp] = (long long)v;
    __syncthreads();
    unsigned long long t = 0;
    for (int w = 0; w < kAWarps; ++w) t = sat_add(t, (unsigned long long)sh.warp_l[w]);
    __syncthreads();
    return t;
}

// ... and, for a sum from zero with an exact region (F != kNoRegion), each chunk's exact sum in
// units of 2^-F; chunks predicted to end well inside the region get no binade actions (the walk
// takes them whole).
__device__ void phase_predicted_actions(const CoopArgs& a, const Src& src, double s0, int sign, int F, Shared& sh) {
    const int G = gridDim.x;
    DF carry = df_of(s0);
    for (int t0 = 0; t0 < a.nch; t0 += kAT) {
        const int c = t0 + threadIdx.x;
        const DF v = c < a.nch ? df_of(__ldcg(&a.rec[c].approx)) : DF{0.0f, 0.0f};
        DF all;
        const DF ex = block_exscan_df(v, &all, sh);
        if (c < a.nch && c % G == int(blockIdx.x))
            sh.own_pred[c / G] = df_value(df_sum(carry, sign > 0 ? ex : df_neg(ex)));
        carry = df_sum(carry, sign > 0 ? all : df_neg(all));
    }
    __syncthreads();
    const bool region = F != kNoRegion && sign > 0 && s0 == 0.0;
    const double region_end = region && 53 - F > -1000 && 53 - F < 1000 ? pow2d(53 - F) * (1.0 - 1.0 / 1048576.0) : 0.0;
    for (int c = blockIdx.x; c < a.nch; c += G) {
        const double pred = sh.own_pred[c / G];
        float x[kAV];
        src.load(a, int64_t(c) * kAL + threadIdx.x * kAV, x);
        if (region) {
            unsigned long long u = 0;
#pragma unroll
            for (int e = 0; e < kAV; ++e) u = sat_add(u, int_units(x[e], F));
            const unsigned long long t = block_sum_sat(u, sh);
            if (threadIdx.x == 0) a.rec[c].isum = t;
            if (pred + __ldcg(&a.rec[c].approx) < region_end) {
                if (threadIdx.x == 0) {  // the walk takes this chunk whole from the exact sum
                    a.rec[c].o[0] = a.rec[c].o[1] = 6u;
                    a.rec[c].E[0] = a.rec[c].E[1] = kNoExp;
                    a.rec[c].split = -1;
                }
                continue;
            }
        } else if (threadIdx.x == 0) {
            a.rec[c].isum = kSat;
        }
        int E0 = kNoExp, E1 = kNoExp;
        if (binade_ok(pred)) {
            E0 = exponent_of(pred);
            const double mant = pred * pow2d(-E0);  // in [1, 2)
            if (mant < 1.0 + 1.0 / 1024.0) E1 = E0 - 1;
            else if (mant > 2.0 - 1.0 / 1024.0) E1 = E0 + 1;
            // a sum that leaves its binade once inside the chunk: split the chunk at the predicted
            // crossing pixel (the walk checks the prediction and walks the chunk exactly if it missed)
            const double pend = pred + __ldcg(&a.rec[c].approx);
            if (sign > 0 && E0 < 898 && pend >= pow2d(E0 + 1) && pend < pow2d(E0 + 2)) {
                const int base = threadIdx.x * kAV;
                const int len = __ldcg(&a.rec[c].len);
                DF loc{0.0f, 0.0f};
#pragma unroll
                for (int e = 0; e < kAV; ++e) df_acc(loc, x[e]);
                DF tot;
                const DF ex = block_exscan_df(loc, &tot, sh);
                // the running sum against 2^(E0+1) (a float when E0 + 1 is within the float range)
                const bool fits = E0 + 1 >= -125 && E0 + 1 <= 126;
                const float edgef = fits ? __int_as_float((E0 + 1 + 127) << 23) : 0.0f;
                DF run = df_sum(df_of(pred), ex);
                int first = INT_MAX;
#pragma unroll
                for (int e = 0; e < kAV; ++e) {
                    df_acc(run, x[e]);
                    const float h = run.h + run.l, l = run.l - (h - run.h);
                    if (fits && first == INT_MAX && base + e < len && (h > edgef || (h == edgef && l >= 0.0f)))
                        first = base + e;
                }
                const int kx = block_min_i(first, sh);
                if (kx < len) {
                    EF tf[2], exf[2], totf[2];
                    tf[0] = ef_identity();
                    tf[1] = ef_identity();
#pragma unroll
                    for (int e = 0; e < kAV; ++e) {
                        if (base + e < kx) tf[0] = ef_compose(tf[0], ef_make(x[e], E0, sign));
                        if (base + e > kx) tf[1] = ef_compose(tf[1], ef_make(x[e], E0 + 1, sign));
                    }
                    block_scan_ef<2>(tf, exf, totf, sh);
                    ChunkRec* r = a.rec + c;
                    if (threadIdx.x == 0) {
                        r->i0[0] = totf[0].i0;
                        r->i1[0] = totf[0].i1;
                        r->o[0] = totf[0].o;
                        r->E[0] = E0;
                        r->i0[1] = totf[1].i0;
                        r->i1[1] = totf[1].i1;
                        r->o[1] = totf[1].o;
                        r->E[1] = E0 + 1;
                        r->split = kx;
                    }
                    if (kx / kAV == int(threadIdx.x)) r->xval = x[kx % kAV];
                    continue;
                }
            }
        }
        chunk_actions(x, E0, E1, sign, a.rec + c, sh);
    }
}

// float(double(I) / R * double(Rs)) (main.cpp:1405-1406) with the quotient taken through the
// reciprocal of R, computed once: the two agree to a few double ulps, so wherever the product is not
// within 64 double ulps of a midpoint between two floats both round to the same float; otherwise the
// reference's division decides.
__device__ __forceinline__ float share_of(float I, double R, double rcp, double Rsd) {
    const double t = (double(I) * rcp) * Rsd;
    const long long b = __double_as_longlong(t);
    const long long low = b & ((1ll << 29) - 1);  // the bits below a float's mantissa
    const int e = int((b >> 52) & 0x7ff) - 1023;
    if (b > 0 && e > -120 && e < 120 && llabs(low - (1ll << 28)) > 64) return __double2float_rn(t);
    return float(double(I) / R * Rsd);
}

// remaining_importance clip test of the water-filling loop (main.cpp:1391-1393), with a
// single-precision screen that leaves every undecided case to the reference's expression.
__device__ __forceinline__ bool clip_test(float I, double R, int Rs, int m) {
    if (Rs > 0 && R > 1e-30 && R < 1e30) {
        const float r = float(Rs) / float_trunc(R);
        const float d = I * r;
        const float fm = float(m);
        if (d > fm * 1.0001f) return true;
        if (d < fm * 0.9999f) return false;
    }
    const double share = double(I) / R;
    const double desired = share * double(Rs);
    return desired > double(m);
}

// Clip decisions of the alive pixels at the pass's start state into flag buffer fb, with the
// chunk's clip count and approximate clipped importance (the binade predictions of the walk).
__device__ void phase_decide_start(const CoopArgs& a, double R, int Rs, int fb, Shared& sh) {
    const unsigned fbit = 2u << fb;
    unsigned long long block_clips = 0;
    for (int c = blockIdx.x; c < a.nch; c += gridDim.x) {
        const int64_t k0 = int64_t(c) * kAL + threadIdx.x * kAV;
        float I[kAV];
        uint8_t st[kAV];
        load_f8(a.importance, k0, a.np, I);
        load_u8(a.state, k0, a.np, st);
        int n = 0;
        float acc = 0.0f;
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            const bool clip = (st[e] & 1u) && clip_test(I[e], R, Rs, a.max_extra);
            st[e] = uint8_t((st[e] & ~fbit) | (clip ? fbit : 0u));
            if (clip) acc += I[e];
            n += clip;
        }
        store_u8(a.state, k0, a.np, st);
        int total;
        block_scan_i(n, &total, sh);
        const float t = block_sum_f(acc, sh);
        if (threadIdx.x == 0) {
            a.rec[c].clips = total;
            a.rec[c].approx = double(t);
            block_clips += (unsigned long long)total;
        }
    }
    if (threadIdx.x == 0 && block_clips) atomicAdd(&a.sc->start_clips, block_clips);
}

// One fixed-point round: the chain values of clip set fb (walked), every alive pixel decided
// again with the state before it into buffer fb ^ 1, and the chunk actions of the new set.
__device__ void phase_decide_round(const CoopArgs& a, double R0, int Rs0, int fb, Shared& sh) {
    const unsigned fbit = 2u << fb, nbit = 2u << (fb ^ 1);
    unsigned long long changed = 0;
    for (int c = blockIdx.x; c < a.nch; c += gridDim.x) {
        const int64_t k0 = int64_t(c) * kAL + threadIdx.x * kAV;
        float I[kAV], x[kAV];
        uint8_t st[kAV];
        load_f8(a.importance, k0, a.np, I);
        load_u8(a.state, k0, a.np, st);
        int n = 0;
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            const bool clip = (st[e] & 1u) && (st[e] & fbit);
            x[e] = clip ? I[e] : 0.0f;
            n += clip;
        }
        int total;
        const int nb_thread = block_scan_i(n, &total, sh);
        double v[kAV], before;
        chain_values(a, c, x, -1, kNoRegion, v, &before, sh);
        const int nb_chunk = __ldcg(&a.rec[c].nb);
        const double start = __ldcg(&a.rec[c].start);
        __syncthreads();  // the record is rewritten below
        int nb = nb_chunk + nb_thread;
        double Rb = before;
        int n_new = 0;
#pragma unroll
        for (int e = 0; e < kAV; ++e) {
            const bool alive = st[e] & 1u;
            const bool was = alive && (st[e] & fbit);
            const bool now = alive && clip_test(I[e], Rb, Rs0 - a.max_extra * nb, a.max_extra);
            changed += (was != now);
            st[e] = uint8_t((st[e] & ~nbit) | (now ? nbit : 0u));
            x[e] = now ? I[e] : 0.0f;
            n_new += now;
            nb += was;
            Rb = v[e];
        }
        store_u8(a.state, k0, a.np, st);
        int total_new;
        block_scan_i(n_new, &total_new, sh);
        const double ref = binade_ok(start) ? start : R0;
        const int E0 = binade_ok(ref) ? exponent_of(ref) : kNoExp;
        // the clip set grows by little between rounds: the start stays in its binade unless it
        // sits just above the binade's floor
        const bool low = E0 != kNoExp && ((__double_as_longlong(ref) & (kTwo52 - 1)) >> 42) == 0;
        chunk_actions(x, E0, low ? E0 - 1 : kNoExp, -1, a.rec + c, sh);
        if (threadIdx.x == 0) a.rec[c].clips = total_new;
    }
    const long long ch = block_sum_l((long long)changed, sh);
    if (threadIdx.x == 0 && ch) atomicAdd(&a.sc->changed, (unsigned long long)ch);
}

}  // namespace

__global__ void __launch_bounds__(kAT, 2) k_allocate_coop(CoopArgs a) {
    __shared__ Shared sh;
    AllocScalars* sc = a.sc;
    const int G = gridDim.x;
    const int m = a.max_extra;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        sc->stamps[0] = t;
        sc->n_stamps = 1;
    }

    // importance checks, desired_add = 0, every pixel alive, approximate chunk sums
    {
        int bad = 0;
        int code = 0;  // largest 1000 - e over the nonzero importances (the exact region's unit)
        for (int c = blockIdx.x; c < a.nch; c += G) {
            const int64_t k0 = int64_t(c) * kAL + threadIdx.x * kAV;
            float I[kAV];
            load_f8(a.importance, k0, a.np, I);
            DF acc{0.0f, 0.0f};  // the split prediction needs chunk starts to ~2^-40
            uint8_t st[kAV];
#pragma unroll
            for (int e = 0; e < kAV; ++e) {
                if (!(I[e] >= 0.0f && I[e] <= FLT_MAX)) bad = 1;
                if (I[e] > 0.0f) code = max(code, 1000 - float_exp(I[e]));
                df_acc(acc, I[e]);
                st[e] = 1u;
                if (k0 + e < a.np) a.desired_add[k0 + e] = 0.0f;
            }
            store_u8(a.state, k0, a.np, st);
            const double t = df_value(block_sum_df(acc, sh));
            if (threadIdx.x == 0) {
                a.rec[c].approx = t;
                a.rec[c].len = int(min((long long)kAL, (long long)(a.np - int64_t(c) * kAL)));
                a.rec[c].clips = 0;
            }
        }
        if (__syncthreads_or(bad) && threadIdx.x == 0) {
            atomicExch(&sc->reason, 1);
            atomicExch(&sc->fallback, 1);
        }
        code = block_max_i(code, sh);
        if (threadIdx.x == 0 && code > 0) atomicMax(&sc->region_code[0], code);
    }
    if (!grid_sync(sc) || fell_back(sc)) return;
    const int F_imp = region_f(__ldcg(&sc->region_code[0]));

    // sum_importance (main.cpp:1370)
    const Src imp{0, 0u};
    phase_predicted_actions(a, imp, 0.0, 1, F_imp, sh);
    if (!grid_sync(sc)) return;
    if (blockIdx.x == 0) walk(a, imp, 0.0, 1, false, F_imp, sh);
    if (!grid_sync(sc) || fell_back(sc)) return;
    const double sum_importance = __ldcg(&sc->walk_final);
    const int remaining_samples0 = max(0, a.extra_sample_total - a.reserved_samples);
    if (sum_importance <= 0.0 || remaining_samples0 <= 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) sc->done = 1;
        return;  // the counts stay at the floor (main.cpp:1375-1379)
    }

    // water-filling (main.cpp:1381-1409)
    double R = sum_importance;
    int Rs = remaining_samples0;
    int64_t active = a.np;
    int fb = 0;
    unsigned long long changed_seen = 0, start_clips_seen = 0;
    int passes = 0, rounds = 0;
    bool shares = false;  // the alive pixels take share_of(I, R, Rs) as their desired_add
    while (active > 0 && Rs > 0 && R > double(1e-8f)) {
        ++passes;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            sc->passes = passes;
            sc->rounds = rounds;
        }
        phase_decide_start(a, R, Rs, fb, sh);
        if (!grid_sync(sc)) return;
        // No pixel clips at the pass's start state: then none clips in the reference's order
        // either (the state it tests against never leaves the start state), and the pass ends
        // with the shares of the start state.
        const unsigned long long sc_now = __ldcg(&sc->start_clips);
        const bool none_at_start = sc_now == start_clips_seen;
        start_clips_seen = sc_now;
        int nc = 0;
        double R_after = R;
        if (!none_at_start) {
            phase_predicted_actions(a, Src{1, 2u << fb}, R, -1, kNoRegion, sh);
            if (!grid_sync(sc)) return;
            if (blockIdx.x == 0) walk(a, Src{1, 2u << fb}, R, -1, true, kNoRegion, sh);
            if (!grid_sync(sc) || fell_back(sc)) return;
            for (int round = 0;; ++round) {
                phase_decide_round(a, R, Rs, fb, sh);
                if (!grid_sync(sc)) return;
                const unsigned long long ch = __ldcg(&sc->changed);
                if (ch == changed_seen) break;  // buffer fb is the pass's clip set; its walk is current
                changed_seen = ch;
                ++rounds;
                fb ^= 1;
                if (round + 1 >= kMaxRounds) {
                    if (threadIdx.x == 0) {
                        atomicExch(&sc->reason, 3);
                        atomicExch(&sc->fallback, 1);
                    }
                    return;
                }
                if (blockIdx.x == 0) walk(a, Src{1, 2u << fb}, R, -1, true, kNoRegion, sh);
                if (!grid_sync(sc) || fell_back(sc)) return;
            }
            nc = __ldcg(&sc->walk_clips);
            R_after = __ldcg(&sc->walk_final);
        }
        const unsigned fbit = 2u << fb;
        if (nc == 0) {
            // no pixel clipped: the rest share the remaining samples (main.cpp:1403-1408); the
            // shares are taken where the residual weights are formed, below
            shares = true;
            break;
        }
        // clipped pixels get the cap and leave the active list
        for (int c = blockIdx.x; c < a.nch; c += G) {
            const int64_t k0 = int64_t(c) * kAL + threadIdx.x * kAV;
            uint8_t st[kAV];
            load_u8(a.state, k0, a.np, st);
#pragma unroll
            for (int e = 0; e < kAV; ++e) {
                if ((st[e] & 1u) && (st[e] & fbit)) {
                    if (k0 + e < a.np) a.desired_add[k0 + e] = float(m);
                    st[e] = 0u;
                }
            }
            store_u8(a.state, k0, a.np, st);
        }
        R = R_after;
        Rs -= m * nc;
        active -= nc;
    }

    // floors and residual weights (main.cpp:1411-1420), approximate chunk sums of the weights
    {
        long long assigned = 0;
        int code = 0;
        const double rcp = 1.0 / R;
        const double Rsd = double(Rs);
        for (int c = blockIdx.x; c < a.nch; c += G) {
            const int64_t k0 = int64_t(c) * kAL + threadIdx.x * kAV;
            DF acc{0.0f, 0.0f};
            float I[kAV];
            uint8_t st[kAV];
            if (shares) {
                load_f8(a.importance, k0, a.np, I);
                load_u8(a.state, k0, a.np, st);
            }
#pragma unroll
            for (int e = 0; e < kAV; ++e) {
                if (k0 + e >= a.np) continue;
                const float d = (shares && (st[e] & 1u)) ? share_of(I[e], R, rcp, Rsd) : __ldcg(a.desired_add + k0 + e);
                const int add = int(floorf(d));
                a.counts[k0 + e] += add;
                assigned += add;
                const float r = fmaxs(0.0f, d - float(add));
                a.residual[k0 + e] = r;
                if (r > 0.0f) code = max(code, 1000 - float_exp(r));
                df_acc(acc, r);
            }
            const double t = df_value(block_sum_df(acc, sh));
            if (threadIdx.x == 0) {
                a.rec[c].approx = t;
                a.rec[c].clips = 0;
            }
        }
        const long long tot = block_sum_l(assigned, sh);
        if (threadIdx.x == 0 && tot) atomicAdd(reinterpret_cast<unsigned long long*>(&sc->assigned),
                                               (unsigned long long)tot);
        code = block_max_i(code, sh);
        if (threadIdx.x == 0 && code > 0) atomicMax(&sc->region_code[1], code);
    }
    if (!grid_sync(sc)) return;
    const int F_res = region_f(__ldcg(&sc->region_code[1]));
    const int assigned = int(__ldcg(&sc->assigned));
    const int remaining = max(0, a.extra_sample_total - a.reserved_samples - assigned);

    // the cumulative chain of the residual weights (main.cpp:1417-1437)
    const Src res{2, 0u};
    phase_predicted_actions(a, res, 0.0, 1, F_res, sh);
    if (!grid_sync(sc)) return;
    if (blockIdx.x == 0) walk(a, res, 0.0, 1, true, F_res, sh);
    if (!grid_sync(sc) || fell_back(sc)) return;
    const double residual_sum = __ldcg(&sc->walk_final);
    if (remaining > 0 && residual_sum > double(1e-8f)) {
        // hash_to_unit_float(g_sampler_base_seed ^ 0x4d595df4u) (main.cpp:270-281, 1427)
        uint32_t h = a.seed ^ 0x4d595df4u;
        h ^= h >> 16;
        h *= 0x7feb352du;
        h ^= h >> 15;
        h *= 0x846ca68bu;
        h ^= h >> 16;
        const double offset = double(float(h & 0x00ffffffu) / float(0x01000000u));
        const double rem_d = double(remaining);
        const double step = residual_sum / rem_d;  // estimate of the target spacing
        // t_k > c, by the estimate where it is decisive, else by main.cpp:1431's expression
        auto above = [&](long long k, double c) -> bool {
            const double kk = double(k) + offset;
            const double est = kk * step;
            const double tol = 1.0 / 1099511627776.0 * (est > c ? est : c);  // 2^-40 relative
            if (est > c + tol) return true;
            if (est < c - tol) return false;
            return (kk / rem_d) * residual_sum > c;
        };
        // N(c): the number of targets t_k <= c, k < remaining; from the estimate c / step - offset,
        // stepped to the exact boundary t_{k-1} <= c < t_k
        const double per_unit = rem_d / residual_sum;
        auto first_above = [&](double c) -> long long {
            const double e = c * per_unit - offset;
            long long k = e <= 0.0 ? 0 : (e >= rem_d ? remaining : (long long)e);
            while (k > 0 && above(k - 1, c)) --k;
            while (k < remaining && !above(k, c)) ++k;
            return k;
        };
        // A single-precision screen decides t_k > c from values relative to the thread's first
        // chain value `before`: tau_i = t_(n0+i) - before (its estimate for i = 0 in double, then
        // steps of `step`) against d = c - before. Its error is below 2^-22 of the magnitudes
        // involved plus 2^-48 of |before| (the double steps); a gap within the margin goes to
        // above(), so the screen never decides what the estimate or the reference's expression
        // would decide otherwise.
        const float stepf = float(step);
        for (int c = blockIdx.x; c < a.nch; c += G) {
            const int64_t k0 = int64_t(c) * kAL + threadIdx.x * kAV;
            float x[kAV];
            load_f8(a.residual, k0, a.np, x);
            double v[kAV], before;
            chain_values(a, c, x, 1, F_res, v, &before, sh);
            const long long n0 = k0 == 0 ? 0 : first_above(before);
            const float tau0 = float((double(n0) + offset) * step - before);
            const float mfix = float(fabs(before)) * (1.0f / 35184372088832.0f) + fabsf(tau0) * (1.0f / 1048576.0f);
            long long n_prev = n0;
#pragma unroll
            for (int e = 0; e < kAV; ++e) {
                if (k0 + e >= a.np) break;
                const float d = float(v[e] - before);
                const float md = mfix + fabsf(d) * (1.0f / 1048576.0f);
                long long n = n_prev;
                while (n < remaining) {
                    const float i = float(n - n0);
                    const float gap = (tau0 + i * stepf) - d;
                    const float m = md + (i + 1.0f) * stepf * (1.0f / 1048576.0f);
                    const bool ab = gap > m ? true : (gap < -m ? false : above(n, v[e]));
                    if (ab) break;
                    ++n;
                }
                if (n != n_prev) a.counts[k0 + e] += int(n - n_prev);
                n_prev = n;
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->passes = passes;
        sc->rounds = rounds;
        sc->done = 1;
        if (sc->n_stamps < kStamps) {
            unsigned long long t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            sc->stamps[sc->n_stamps++] = t;
        }
    }
}

uint64_t allocator_work_bytes(int64_t np) {
    const int64_t nch = (np + kAL - 1) / kAL;
    const int64_t pool = nch;  // every chunk can be walked exactly
    return kScalarBytes + uint64_t(nch) * sizeof(ChunkRec) + 256 + uint64_t(pool) * kAL * sizeof(double);
}

namespace {
struct CoopShape {
    int device = -1;
    int sms = 0;
    int per_sm = 0;
};
CoopShape g_coop_shape;
std::mutex g_coop_mu;
}  // namespace

// Launches the parallel allocation on the job's stream. *fallback_flag receives the device
// address of the flag the serial kernel checks (nonzero: redo the allocation serially).
cudaError_t launch_allocate_parallel(Job& j, const float* importance, int extra_sample_total, int reserved_samples,
                                     int max_extra, uint32_t seed, const int** fallback_flag) {
    const int64_t np = j.g.np;
    const int nch = int((np + kAL - 1) / kAL);
    char* work = reinterpret_cast<char*>(j.p.alloc_work);
    AllocScalars* sc = reinterpret_cast<AllocScalars*>(work);
    ChunkRec* rec = reinterpret_cast<ChunkRec*>(work + kScalarBytes);
    double* pool = reinterpret_cast<double*>(work + kScalarBytes + ((uint64_t(nch) * sizeof(ChunkRec) + 255) & ~uint64_t(255)));
    *fallback_flag = &sc->fallback;
    // on the job's own stream: a cooperative launch starts only when all of its blocks are
    // resident, so the allocations of jobs running side by side never wait on each other's
    // blocks (each block is built for half an SM's registers, so two share an SM)
    cudaStream_t as = j.stream;
    cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(AllocScalars), as);
    if (e != cudaSuccess) return e;
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    CoopShape shape;
    {
        std::lock_guard<std::mutex> lk(g_coop_mu);
        if (g_coop_shape.device != dev) {
            int sms = 0, coop = 0, per_sm = 0;
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_allocate_coop, kAT, 0);
            if (e != cudaSuccess) return e;
            g_coop_shape.device = dev;
            g_coop_shape.sms = coop ? sms : 0;
            g_coop_shape.per_sm = per_sm;
        }
        shape = g_coop_shape;
    }
    // one block per SM (256 threads: a block leaves room on its SM for other kernels), or the cap
    // of RPD_TUNE_ALLOCATOR; more when the frame has more chunks than the blocks can own
    const int resident = shape.sms * std::max(shape.per_sm, 0);
    int want = j.allocator_blocks >= 2 ? j.allocator_blocks : kDefaultBlocks;
    want = std::max(want, int((int64_t(nch) + kMaxOwned - 1) / kMaxOwned));
    const int G = std::min(nch, std::min(std::min(resident, shape.sms), want));
    if (G < 1 || int64_t(nch) > int64_t(kMaxOwned) * G) {
        // no cooperative launch possible here: leave it to the serial kernel
        e = cudaMemsetAsync(&sc->fallback, 1, sizeof(int), as);
        if (e == cudaSuccess) e = cudaMemsetAsync(&sc->reason, 5, 1, as);
    } else {
        CoopArgs a;
        a.importance = importance;
        a.desired_add = j.p.desired_add;
        a.residual = j.p.residual;
        a.counts = j.p.counts;
        a.state = j.p.alloc_state;
        a.rec = rec;
        a.pool = pool;
        a.sc = sc;
        a.np = np;
        a.nch = nch;
        a.pool_chunks = nch;
        a.extra_sample_total = extra_sample_total;
        a.reserved_samples = reserved_samples;
        a.max_extra = max_extra;
        a.seed = seed;
        void* args[] = {&a};
        e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_allocate_coop), dim3(G), dim3(kAT), args, 0,
                                        as);
        j.launches += 1;
    }
    return e;
}

cudaError_t allocator_stats(Job& j, int32_t* out) {
    AllocScalars h;
    cudaError_t e = cudaMemcpyAsync(&h, j.p.alloc_work, sizeof(h), cudaMemcpyDeviceToHost, j.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(j.stream);
    if (e != cudaSuccess) return e;
    out[0] = h.done;
    out[1] = h.fallback;
    out[2] = h.error;
    out[3] = h.passes;
    out[4] = h.rounds;
    out[5] = h.exact_chunks;
    out[6] = h.reason;
    return cudaSuccess;
}

int allocator_timeline(Job& j, uint64_t* ns, int32_t max, int32_t* n) {
    AllocScalars h;
    cudaError_t e = cudaMemcpyAsync(&h, j.p.alloc_work, sizeof(h), cudaMemcpyDeviceToHost, j.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(j.stream);
    if (e != cudaSuccess) return cuda_fail(e, "allocator timeline");
    const int k = std::min(std::min(h.n_stamps, kStamps), int(max));
    for (int i = 0; i < k; ++i) ns[i] = h.stamps[i] - h.stamps[0];
    *n = k;
    return RPD_OK;
}

}  // namespace rpd
