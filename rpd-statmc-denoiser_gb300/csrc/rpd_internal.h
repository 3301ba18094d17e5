// Internal state of the GB300 denoise stage: job layout in HBM, kernel launch wrappers
// and the helpers every translation unit shares. Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "rpd_gb300.h"

namespace rpd {

constexpr float kEpsSmall = 1e-8f;        // shared/global.h:4
constexpr int kClasses = 7;               // validity classes of the fast grid pass
constexpr int kDeps = RPD_GRID_DEPENDENCIES;
constexpr int kDepStride = RPD_GRID_DEP_STRIDE;

// rpf::Tile member order (core/stats.h:185-198).
enum Dep {
    D_PIXEL = 0, D_BRDF, D_SCREEN_BRDF, D_LENS, D_SCREEN_LENS, D_LIGHT_UV, D_SCREEN_LIGHT_UV,
    D_ENV, D_SCREEN_ENV, D_LIGHT_SELECT, D_SCREEN_LIGHT_SELECT, D_RR, D_SCREEN_RR
};

// Node fields of FrameBuffers::SensitivityTiles (core/buffers.h:23-40), in rpd_field order.
enum NodeField {
    N_ALL = 0, N_ALL_CONF, N_PIXEL, N_PIXEL_CONF, N_BRDF, N_BRDF_CONF, N_LENS, N_LENS_CONF,
    N_LIGHT, N_LIGHT_CONF, N_LIGHT_UV, N_LIGHT_UV_CONF, N_LIGHT_SELECT, N_LIGHT_SELECT_CONF,
    N_ENV, N_ENV_CONF, N_RR, N_RR_CONF, N_FIELDS
};

// Raw per-node sensitivity / confidence fields in the order main.cpp:781-806 fills them.
enum RawField {
    R_PIXEL = 0, R_BRDF, R_LENS, R_LIGHT_UV, R_LIGHT_SELECT, R_ENV, R_RR,
    R_S_BRDF, R_S_LENS, R_S_LIGHT_UV, R_S_LIGHT_SELECT, R_S_ENV, R_S_RR, R_FIELDS
};

// Per-pixel planes (float unless noted). Every plane holds W*H values.
struct PixelPlanes {
    // PixelStats (core/stats.h:6-23)
    float* mean;
    float* square_diff;
    int32_t* n;
    float* color_mean[3];
    float* sqrt_mean[3];
    float* sqrt_sq[3];
    // FrameBuffers sums (core/buffers.h:13-16, 114, 118-119)
    int32_t* hit_count;
    int32_t* sample_count;
    float* radiance[3];
    float* normal[3];
    float* albedo[3];
    float* depth;
    // DerivedFeatureCache (main.cpp:45-52)
    float* f_normal[3];
    float* f_depth;
    float* f_albedo[3];
    // sensitivity outputs (main.cpp:932-946) and the denoise view of the sensitivity cache:
    // rpd[c] = clamp(clamp(expanded component c) * (1 - clamp(gradient)))  (main.cpp:305-327)
    float* sens_confidence;
    float* sens_gradient;
    float* rpd[6];
    // statmc_denoise outputs (main.cpp:1021-1126)
    float* denoised[3];
    float* uncertainty;
    float* alpha;
    float* var_total;
    float* var_eff;
    float* var_ratio;
    // statmc scratch: stabilised sqrt variance of the mean (main.cpp:972-990)
    float* sqrt_var_mean[3];
    float* sqrt_var_stable[3];
    // statmc_denoise's packed neighbour records: six float4 planes of W*H, one after the other
    // (record k of pixel i at win[k * W*H + i]), written with the stabilised sqrt variance and
    // staged into shared memory tile by tile by the window kernel (k_statmc.cu)
    float4* win;
    // variance_denoise (main.cpp:1178-1264)
    float* variance_denoised;
    float* var_ping;     // rows of var_pitch(w) floats
    float* var_pong;
    float4* var_gate;    // variance_denoise's gate records: unit normal, depth
    uint64_t* var_mask;  // variance_denoise: per pixel, the neighbours that pass the geometric gates
    // compute_adaptive_sample_counts (main.cpp:1300-1438)
    float* importance;
    float* importance_tmp;
    float* desired_add;
    float* residual;
    int32_t* counts;
    int32_t* active_a;
    int32_t* active_b;
    int32_t* slow;       // pixels the StatMC window's fast loop handed to its slow pass
    // scratch of the parallel allocation (k_allocate.cu)
    uint8_t* alloc_state;
    unsigned char* alloc_work;
    // RPD_COUNTER_COUNT_ device counters (rpd_counter)
    unsigned long long* counters;
};

struct NodePlanes {
    double* grid;        // nodes * 13 * 36 doubles, merged grid (rpf_grid)
    double* pass_grid;   // grid of the open pass (the reference's thread-local grids)
    float* field[N_FIELDS];
    float* raw[R_FIELDS];
    float* conf[R_FIELDS];
    float* prior[R_FIELDS];
    float* n_normal[3];
    float* n_depth;
    float* n_albedo[3];
};

struct Geometry {
    int w, h;
    int support, step, nodes_x, nodes_y;
    int64_t np, nn;
};

struct Ctx {
    int device = 0;
    uint64_t budget = 0;
    std::atomic<uint64_t> in_use{0};
    std::mutex mu;
    cudaStream_t util_stream = nullptr;
    std::unordered_map<void*, uint64_t> user_allocs;  // rpd_device_alloc bookkeeping
};

struct Job {
    Ctx* ctx = nullptr;
    rpd_config cfg{};
    Geometry g{};
    cudaStream_t stream = nullptr;
    // set (jobs of the serving loop): the arena, the offsets and the push scratch come from this
    // memory pool in the order of the job's stream, so creating, growing and destroying them
    // never synchronises the device (cudaFree does), which would drain every other request
    cudaMemPool_t pool = nullptr;
    void* arena = nullptr;       // one allocation holding every plane
    uint64_t arena_bytes = 0;
    PixelPlanes p{};
    NodePlanes n{};
    // scalars the serial allocation kernel leaves for the host (int32 + doubles)
    void* scalars = nullptr;
    // staging for host-side pushes (grown on demand)
    void* staging = nullptr;
    uint64_t staging_bytes = 0;
    // host pushes copy row bands on their own stream into the staging buffer, so that the copy
    // of one band overlaps the statistics and grid passes of the previous ones; the staging
    // is reused by the next host push once this push's passes have read it
    static constexpr int kMaxBands = 16;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t band_copied[kMaxBands]{};
    cudaEvent_t staging_free = nullptr;
    int64_t band_bytes = int64_t(768) << 20;  // target size of a band (RPD_TUNE_HOST_BAND_MB)
    float* lum = nullptr;        // per-sample luminance of the current push (fast grid pass)
    uint64_t lum_cap = 0;
    float* cls[kClasses][5]{};   // per-pixel validity-class sums of deviant pixels (arena)
    float4* pat4 = nullptr;      // per-pixel pattern sums (count, sum y hi, lo, sum y^2 hi) (arena)
    float2* pat2 = nullptr;      // per-pixel (sum y^2 lo, pattern | flags << 8 as bits) (arena)
    int64_t* offsets = nullptr;  // per-pixel sample offsets of the current push
    int64_t offsets_cap = 0;
    bool exact_grid = false;     // RPD_EXACT_GRID: double-precision grid in the reference's order
    bool exact_window = false;   // RPD_EXACT_WINDOW: double-precision StatMC window
    int grid_shape = 6;          // launch shape of the random-dimension grid pass (row groups x dimension sets)
    int statmc_by = 0;           // StatMC tile height (0: the largest that fits)
    int window_guard = 15;       // the StatMC window's guard band is 2^-window_guard (RPD_TUNE_WINDOW_GUARD)
    bool serial_allocator = false;  // RPD_TUNE_ALLOCATOR = 1: the one-thread allocation kernel only
    bool smooth_fp64 = false;       // RPD_TUNE_SMOOTHING = 1: the importance smoothing in double-precision instructions
    int allocator_blocks = 0;       // RPD_TUNE_ALLOCATOR >= 2: blocks of the parallel allocation
    bool pass_open = false;
    bool acc_zero = false;      // the per-pixel statistics are the frame start's zeros (no push yet)
    bool host_async = false;  // the current host push returns before its copies complete
    bool grid_fresh = true;      // the frame grid has no merged pass yet (the next merge assigns)
    bool grid_pairs = false;     // the frame grid holds double-float pairs (fast grid mode), not doubles
    // the open pass's fast-mode pushes added straight into the frame grid (pairs), so the end of
    // the pass merges nothing of theirs; pass_indirect: some push of the pass wrote the pass grid
    bool pass_direct = false;
    bool pass_indirect = false;
    bool features_valid = false;
    bool cache_valid = false;
    bool have_samples = false;
    cudaEvent_t ev_start[RPD_STAGE_COUNT_]{};
    cudaEvent_t ev_stop[RPD_STAGE_COUNT_]{};
    bool ev_used[RPD_STAGE_COUNT_]{};
    std::atomic<uint64_t> launches{0};
    // per-kernel event timing (rpd_job_set_profiling)
    bool profile = false;
    struct KTiming { int kernel; cudaEvent_t a, b; };
    std::vector<KTiming> ktimes;
    std::vector<cudaEvent_t> event_pool;
    double ktotal[RPD_KERNEL_COUNT_]{};
    uint64_t kcount[RPD_KERNEL_COUNT_]{};
    cudaEvent_t marks[8]{};      // rpd_job_mark slots
    // the StatMC window's tensor map over `win` (a CUtensorMap, 64-byte aligned), for the
    // halo box of radius win_map_r and win_map_by rows per block (0: not encoded yet)
    alignas(64) unsigned char win_map[128]{};
    int win_map_r = 0, win_map_by = 0;
    // variance_denoise's tensor maps (gate records, ping, pong) for halo radius var_map_r (0: not encoded)
    alignas(64) unsigned char var_maps[3][128]{};
    int var_map_r = 0;
};

// Brackets the launches of one kernel family with CUDA events when profiling is on.
struct KernelScope {
    Job& j;
    int kernel;
    cudaEvent_t a = nullptr, b = nullptr;
    KernelScope(Job& job, int k) : j(job), kernel(k) {
        if (!j.profile) return;
        for (cudaEvent_t* e : {&a, &b}) {
            if (!j.event_pool.empty()) {
                *e = j.event_pool.back();
                j.event_pool.pop_back();
            } else if (cudaEventCreate(e) != cudaSuccess) {
                *e = nullptr;
            }
        }
        if (a) cudaEventRecord(a, j.stream);
    }
    ~KernelScope() {
        if (!j.profile || !a || !b) return;
        cudaEventRecord(b, j.stream);
        j.ktimes.push_back({kernel, a, b});
    }
};

// ---- error plumbing -------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
#define RPD_CUDA(call)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return ::rpd::cuda_fail(e_, #call); \
    } while (0)

// ---- kernels (launch wrappers; each returns cudaError_t of the launch) -------------------
struct DeviceSamples16 {         // rpd_sample_soa16 with pointers in HBM
    const uint16_t* sqrt_radiance[3];
    const int16_t* normal[3];
    const uint16_t* depth;
    const uint16_t* pixel_albedo[3];
    const uint16_t* pixel_u[2];
    const uint16_t* lens_u[2];
    const uint16_t* brdf_u[2];
    const uint16_t* light_u[2];
    const uint16_t* env_u[2];
    float depth_scale;
};

struct DeviceSamples {           // rpd_sample_soa with pointers in HBM
    int compact;                 // 1: the planes are rpd_sample_soa16's, in c16 (flags and category below)
    DeviceSamples16 c16;
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
};

// Per-pixel validity-class sums the statistics pass leaves for the fast grid pass.
// Class 0: pixel_valid samples; classes 1-6: samples with the brdf, lens, light_uv,
// environment, light_select and rr dimension valid. Each class holds count, sum y
// (hi, lo) and sum y^2 (hi, lo) over the pixel's finite samples.
constexpr uint8_t kPixUniform = 0x1;  // every screen position lies inside its pixel
constexpr uint8_t kPixMixed = 0x2;    // some sample has a random dimension but no screen position
constexpr uint8_t kPixDeviant = 0x4;  // some sample's validity pattern differs from the pixel's pattern
constexpr float kUniformMax = 1.0f - 1.0f / 4096.0f;  // largest in-pixel offset of a uniform pixel
__host__ __device__ constexpr uint8_t class_bit(int c) {
    return c == 0 ? RPD_SAMPLE_PIXEL_VALID : c == 1 ? RPD_SAMPLE_BRDF_VALID : c == 2 ? RPD_SAMPLE_LENS_VALID
         : c == 3 ? RPD_SAMPLE_LIGHT_VALID : c == 4 ? RPD_SAMPLE_ENV_VALID : c == 5 ? RPD_SAMPLE_LIGHT_SELECT_VALID
         : RPD_SAMPLE_RR_VALID;
}
// Per-pixel inputs of the grid pass, written by the statistics pass for the pixels of a push.
// A pixel's pattern is the validity-class bits (flags & 0xfe) of its first finite sample that
// has any; pat4/pat2 hold the (count, sum y, sum y^2) double-float sums over its finite samples
// with exactly that pattern, and the pattern and the pixel flags (kPix*) as the bits of
// pat2.y: pattern | flags << 8. A pixel with other patterns too is deviant (kPixDeviant) and
// then also has full per-class sums in cls[0..6].
struct GridPrep {
    float* cls[kClasses][5];  // W*H planes
    float4* pat4;             // W*H
    float2* pat2;             // W*H
    float* lum;               // per sample of the push (NaN when the radiance is not finite)
    uint32_t* key;            // per sample of the push: packed random-dimension bins + validity
    uint16_t* col;            // per sample of a push with per-pixel counts: the pixel's column
                              // (null for uniform pushes, where the column follows from the index)
    int width;
};
// Sample key: bits 0-3 lens bin, 4-7 brdf bin, 8-11 light_uv bin, 12-15 environment bin,
// 16-19 light index, 20 rr survived; bits 21-27 the valid flags of pixel, lens, brdf,
// light_uv, light_select, environment, rr (after dropping flags whose plane is absent).
constexpr int kKeyValidShift = 21;
__host__ __device__ constexpr uint32_t key_valid_bit(int group) {
    // group 0 pixel, 1 brdf, 2 lens, 3 light_uv, 4 environment, 5 light_select, 6 rr
    return group == 0 ? 1u << 21 : group == 1 ? 1u << 23 : group == 2 ? 1u << 22 : group == 3 ? 1u << 24
         : group == 4 ? 1u << 26 : group == 5 ? 1u << 25 : 1u << 27;
}
__host__ __device__ constexpr int key_bin_shift(int group) {
    return group == 1 ? 4 : group == 2 ? 0 : group == 3 ? 8 : group == 4 ? 12 : 16;
}

cudaError_t launch_encode_samples16(const DeviceSamples& in, int64_t n_samples, int64_t n_pixels,
                                    const DeviceSamples16& out, cudaStream_t stream);
cudaError_t launch_offsets_uniform(Job& j, int64_t count, int32_t spp);
// The exclusive offsets of per-pixel counts into j.offsets[0..count]; the largest count goes to
// offsets_count_max(j, count), which stays valid until the next scan.
cudaError_t launch_offsets_scan(Job& j, const int32_t* d_counts, int64_t count);
const int64_t* offsets_count_max(const Job& j, int64_t count);
cudaError_t launch_accumulate_pixels(Job& j, const DeviceSamples& s, int64_t first, int64_t count,
                                     const GridPrep& gp, int32_t spp);
cudaError_t launch_accumulate_grid(Job& j, const DeviceSamples& s, int64_t first, int64_t count);
// max_count bounds the samples of one pixel; total_samples bounds the samples of the push. Either
// bound can make the bin weights exact integers (no bin of a node can then pass 2^32 units).
// d_max_count: the push's largest per-pixel count in device memory when the host does not know it
// (max_count INT32_MAX), or nullptr.
cudaError_t launch_grid_fast(Job& j, const DeviceSamples& s, int64_t first, int64_t count, const GridPrep& gp,
                             int32_t spp, int32_t max_count, int64_t total_samples,
                             const int64_t* d_max_count = nullptr);
cudaError_t launch_merge_grid(Job& j);
// The frame grid as doubles into out (nn * kDeps * kDepStride entries) when it holds pairs.
cudaError_t launch_grid_to_double(Job& j, double* out);
cudaError_t launch_feature_cache(Job& j);
cudaError_t launch_sensitivity(Job& j);
cudaError_t launch_sensitivity_zero(Job& j);
cudaError_t launch_rpd_cache(Job& j);
cudaError_t launch_statmc(Job& j);
cudaError_t launch_variance(Job& j);
cudaError_t launch_adaptive(Job& j);
// The allocation alone, from the importance map already in j.p.importance.
cudaError_t launch_allocate_map(Job& j);
// The parallel allocation (k_allocate.cu): bytes of its scratch for np pixels, and the launch;
// *fallback_flag gets the device flag telling the serial kernel to redo the allocation.
uint64_t allocator_work_bytes(int64_t np);
cudaError_t launch_allocate_parallel(Job& j, const float* importance, int extra_sample_total, int reserved_samples,
                                     int max_extra, uint32_t seed, const int** fallback_flag);
// The last parallel allocation's outcome (rpd_job_allocator_stats), after a stream sync.
cudaError_t allocator_stats(Job& j, int32_t* out);
// Device times (ns from the launch) of the last parallel allocation's barriers.
int allocator_timeline(Job& j, uint64_t* ns, int32_t max, int32_t* n);
cudaError_t launch_finalize(Job& j);
cudaError_t launch_expand(Job& j, const float* node_field, float* out);
// `iterations` a-trous passes ping-ponging between buf_a and buf_b (interleaved RGB); *result
// gets the buffer holding the last pass (raw for 0 passes). records: scratch for 2 * w * h float4
// normal and albedo records, or nullptr to renormalise the normals at every tap instead.
cudaError_t launch_atrous(const float* raw, const float* normal, const float* albedo, int w, int h,
                          float sigma_c, float sigma_n, float sigma_a, int iterations, float* buf_a,
                          float* buf_b, float4* records, float** result, cudaStream_t stream, uint64_t* launches);
// The joint bilateral filter's scratch (its records and a copy-timeout flag), and the filter.
// The flag (an unsigned after the records) is non-zero when a tile copy's bounded wait gave up.
uint64_t joint_bilateral_scratch_bytes(int w, int h);
cudaError_t launch_joint_bilateral(const float* raw, const float* normal, const float* albedo, int w, int h,
                                   float sigma_c, float sigma_n, float sigma_p, float sigma_a, float* gaussian,
                                   float* bilateral, float* joint, void* scratch, cudaStream_t stream,
                                   uint64_t* launches);

// eval_tools hdr-metrics on the GPU (k_metrics.cu): the scratch it needs for a w x h image,
// and the launches; *d_out (device memory) gets the metrics.
// An RGB image as three channel pointers and a pixel stride: interleaved (p[c] = base + c,
// step 3) or planar (step 1).
struct Img3 {
    const float* p[3];
    int step;
    __device__ __forceinline__ double at(int64_t i, int c) const { return double(p[c][i * step]); }
};
uint64_t metrics_scratch_bytes(int w, int h);
// Image products (k_output.cu): encode src on `stream` and write the file (tonemap < 0: Radiance
// HDR, else a PNG with that preset); dev / host: scratch of 4 w h bytes (host page-locked).
int write_image(const Img3& src, int w, int h, int tonemap, const std::string& path, uint8_t* dev, uint8_t* host,
                cudaStream_t stream);
cudaError_t launch_count_fraction(const int32_t* counts, int64_t np, int* dmax, float* out, cudaStream_t stream);
cudaError_t launch_metrics(const Img3& ref, const Img3& tst, int w, int h, void* scratch, rpd_image_metrics* d_out,
                           cudaStream_t stream);

// Pushes without host synchronisation (the serving loop, serve.cu). job_reserve sizes the
// offsets for every pixel and the per-sample scratch for pushes of up to max_push_samples, so
// that later pushes allocate nothing; push_device_async takes device planes and, with device
// counts, a bound on the push's sample total instead of reading the total back.
int job_reserve(Job& j, int64_t max_push_samples);
// rpd_job_create with the job's device memory from `pool` (nullptr: cudaMalloc, as
// rpd_job_create does); rpd_job_destroy releases either kind.
int job_create(Ctx* c, const rpd_config* cfg, cudaMemPool_t pool, Job** out);
// offsets_ready: j.offsets already holds the push's offsets (a scan of the same counts).
int push_device_async(Job& j, const DeviceSamples& d, int64_t first, int64_t count, int32_t spp, const int32_t* counts,
                      int64_t total_bound, bool offsets_ready = false);

inline unsigned grid_for(int64_t n, int block) {
    return static_cast<unsigned>((n + block - 1) / block);
}

}  // namespace rpd
