// C ABI of the GB300 denoise stage (include/rpd_gb300.h): contexts, jobs, HBM layout,
// admission against the HBM budget, the stage entry points and field reads.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <new>

#include "rpd_internal.h"
#include "device_math.cuh"
#include "rpd_synth.h"

namespace rpd {

cudaError_t launch_synth(const rpd_synth_params& prm, const rpd_synth_region* d_table, int64_t first, int64_t count,
                         const int64_t* d_offsets, int64_t total, const int32_t* d_start_n, int32_t* d_region_of,
                         const rpd_sample_soa& out, cudaStream_t stream);

namespace {
thread_local std::string t_last_error;

// Deterministic placement of every plane in one arena, 256-byte aligned.
struct Layout {
    uint64_t bytes = 0;
    template <typename T>
    void add(T*& ptr, int64_t count) {
        bytes = (bytes + 255) & ~uint64_t(255);
        ptr = reinterpret_cast<T*>(static_cast<uintptr_t>(bytes));
        bytes += uint64_t(count) * sizeof(T);
    }
};

template <typename T>
void rebase(T*& ptr, char* base) {
    ptr = reinterpret_cast<T*>(base + reinterpret_cast<uintptr_t>(ptr));
}

Geometry make_geometry(const rpd_config& c) {
    Geometry g{};
    g.w = c.image_width;
    g.h = c.image_height;
    g.support = c.rpf_tile_size;
    g.step = std::max(1, g.support / 2);                          // core/stats.h:314
    g.nodes_x = std::max(2, (g.w + g.step - 1) / g.step + 1);     // core/stats.h:315
    g.nodes_y = std::max(2, (g.h + g.step - 1) / g.step + 1);
    g.np = int64_t(g.w) * g.h;
    g.nn = int64_t(g.nodes_x) * g.nodes_y;
    return g;
}

// Assigns (offset-encoded) plane pointers; returns the arena size.
uint64_t plan(const Geometry& g, PixelPlanes& p, NodePlanes& n, float* (*cls)[5] = nullptr,
              float4** pat4 = nullptr, float2** pat2 = nullptr) {
    Layout L;
    const int64_t np = g.np, nn = g.nn;
    L.add(p.mean, np);
    L.add(p.square_diff, np);
    L.add(p.n, np);
    for (int c = 0; c < 3; ++c) L.add(p.color_mean[c], np);
    for (int c = 0; c < 3; ++c) L.add(p.sqrt_mean[c], np);
    for (int c = 0; c < 3; ++c) L.add(p.sqrt_sq[c], np);
    L.add(p.hit_count, np);
    L.add(p.sample_count, np);
    for (int c = 0; c < 3; ++c) L.add(p.radiance[c], np);
    for (int c = 0; c < 3; ++c) L.add(p.normal[c], np);
    for (int c = 0; c < 3; ++c) L.add(p.albedo[c], np);
    L.add(p.depth, np);
    for (int c = 0; c < 3; ++c) L.add(p.f_normal[c], np);
    L.add(p.f_depth, np);
    for (int c = 0; c < 3; ++c) L.add(p.f_albedo[c], np);
    L.add(p.sens_confidence, np);
    L.add(p.sens_gradient, np);
    for (int c = 0; c < 6; ++c) L.add(p.rpd[c], np);
    for (int c = 0; c < 3; ++c) L.add(p.denoised[c], np);
    L.add(p.uncertainty, np);
    L.add(p.alpha, np);
    L.add(p.var_total, np);
    L.add(p.var_eff, np);
    L.add(p.var_ratio, np);
    for (int c = 0; c < 3; ++c) L.add(p.sqrt_var_mean[c], np);
    for (int c = 0; c < 3; ++c) L.add(p.sqrt_var_stable[c], np);
    L.add(p.win, 6 * np);
    L.add(p.variance_denoised, np);
    // variance_denoise's ping-pong planes: rows padded to a multiple of 4 floats (16 bytes)
    L.add(p.var_ping, int64_t((g.w + 3) & ~3) * g.h);
    L.add(p.var_pong, int64_t((g.w + 3) & ~3) * g.h);
    L.add(p.var_gate, np);
    L.add(p.var_mask, np);
    L.add(p.importance, np);
    L.add(p.importance_tmp, np);
    L.add(p.desired_add, np);
    L.add(p.residual, np);
    L.add(p.counts, np);
    L.add(p.active_a, np);
    L.add(p.active_b, np);
    L.add(p.slow, np);
    L.add(p.alloc_state, np);
    L.add(p.alloc_work, int64_t(allocator_work_bytes(np)));
    L.add(p.counters, RPD_COUNTER_COUNT_);
    L.add(n.grid, nn * kDeps * kDepStride);
    L.add(n.pass_grid, nn * kDeps * kDepStride);
    for (int f = 0; f < N_FIELDS; ++f) L.add(n.field[f], nn);
    for (int f = 0; f < R_FIELDS; ++f) L.add(n.raw[f], nn);
    for (int f = 0; f < R_FIELDS; ++f) L.add(n.conf[f], nn);
    for (int f = 0; f < R_FIELDS; ++f) L.add(n.prior[f], nn);
    for (int c = 0; c < 3; ++c) L.add(n.n_normal[c], nn);
    L.add(n.n_depth, nn);
    for (int c = 0; c < 3; ++c) L.add(n.n_albedo[c], nn);
    float* cls_tmp[kClasses][5];
    float4* pat4_tmp = nullptr;
    float2* pat2_tmp = nullptr;
    float* (*C)[5] = cls ? cls : cls_tmp;
    for (int c = 0; c < kClasses; ++c)
        for (int f = 0; f < 5; ++f) L.add(C[c][f], np);
    L.add(pat4 ? *pat4 : pat4_tmp, np);
    L.add(pat2 ? *pat2 : pat2_tmp, np);
    return (L.bytes + 255) & ~uint64_t(255);
}

void rebase_all(PixelPlanes& p, NodePlanes& n, char* base) {
    rebase(p.mean, base);
    rebase(p.square_diff, base);
    rebase(p.n, base);
    for (int c = 0; c < 3; ++c) {
        rebase(p.color_mean[c], base);
        rebase(p.sqrt_mean[c], base);
        rebase(p.sqrt_sq[c], base);
        rebase(p.radiance[c], base);
        rebase(p.normal[c], base);
        rebase(p.albedo[c], base);
        rebase(p.f_normal[c], base);
        rebase(p.f_albedo[c], base);
        rebase(p.denoised[c], base);
        rebase(p.sqrt_var_mean[c], base);
        rebase(p.sqrt_var_stable[c], base);
        if (c == 0) rebase(p.win, base);
        rebase(n.n_normal[c], base);
        rebase(n.n_albedo[c], base);
    }
    rebase(p.hit_count, base);
    rebase(p.sample_count, base);
    rebase(p.depth, base);
    rebase(p.f_depth, base);
    rebase(p.sens_confidence, base);
    rebase(p.sens_gradient, base);
    for (int c = 0; c < 6; ++c) rebase(p.rpd[c], base);
    rebase(p.uncertainty, base);
    rebase(p.alpha, base);
    rebase(p.var_total, base);
    rebase(p.var_eff, base);
    rebase(p.var_ratio, base);
    rebase(p.variance_denoised, base);
    rebase(p.var_ping, base);
    rebase(p.var_gate, base);
    rebase(p.var_pong, base);
    rebase(p.var_mask, base);
    rebase(p.importance, base);
    rebase(p.importance_tmp, base);
    rebase(p.desired_add, base);
    rebase(p.residual, base);
    rebase(p.counts, base);
    rebase(p.active_a, base);
    rebase(p.active_b, base);
    rebase(p.slow, base);
    rebase(p.alloc_state, base);
    rebase(p.alloc_work, base);
    rebase(p.counters, base);
    rebase(n.grid, base);
    rebase(n.pass_grid, base);
    for (int f = 0; f < N_FIELDS; ++f) rebase(n.field[f], base);
    for (int f = 0; f < R_FIELDS; ++f) {
        rebase(n.raw[f], base);
        rebase(n.conf[f], base);
        rebase(n.prior[f], base);
    }
    rebase(n.n_depth, base);
}

struct StageTimer {
    Job& j;
    rpd_stage s;
    StageTimer(Job& job, rpd_stage stage) : j(job), s(stage) {
        cudaEventRecord(j.ev_start[s], j.stream);
    }
    ~StageTimer() {
        cudaEventRecord(j.ev_stop[s], j.stream);
        j.ev_used[s] = true;
    }
};

__global__ void k_pack3(const float* a, const float* b, const float* c, float* out, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[3 * i] = a[i];
    out[3 * i + 1] = b[i];
    out[3 * i + 2] = c[i];
}

bool device_ok(int device, std::string* why) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) {
        *why = "no CUDA device " + std::to_string(device);
        return false;
    }
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        *why = "cannot query CUDA device";
        return false;
    }
    if (prop.major != 10 || prop.minor != 3) {
        *why = "device " + std::string(prop.name) + " is sm_" + std::to_string(prop.major) +
               std::to_string(prop.minor) + "; this build targets sm_103a (GB300)";
        return false;
    }
    return true;
}

// A job buffer: from the job's pool in stream order when it has one, else cudaMalloc.
cudaError_t job_alloc(Job& j, void** p, uint64_t bytes) {
    if (j.pool) return cudaMallocFromPoolAsync(p, bytes, j.pool, j.stream);
    return cudaMalloc(p, bytes);
}

// Frees a job buffer: after the job stream's earlier work (a pool buffer, without synchronising
// anything), or with cudaFree once that work is done.
void job_free(Job& j, void* p) {
    if (!p) return;
    if (j.pool) {
        cudaFreeAsync(p, j.stream);
    } else {
        cudaStreamSynchronize(j.stream);
        cudaFree(p);
    }
}

// stream_only: the buffer is used on the job's stream alone, so a pool job may replace it in
// stream order; a buffer that other streams use (the host-push staging) is always replaced
// after the job's work has finished.
int grow_device(Job& j, void** buf, uint64_t* cap, uint64_t need, bool stream_only = false) {
    if (*cap >= need) return RPD_OK;
    const bool ordered = stream_only && j.pool;
    if (*buf) {
        if (ordered) {
            cudaFreeAsync(*buf, j.stream);
        } else {
            cudaStreamSynchronize(j.stream);
            cudaFree(*buf);
        }
        j.ctx->in_use -= *cap;
        *buf = nullptr;
        *cap = 0;
    }
    const uint64_t want = need + need / 8;
    if (j.ctx->in_use.load() + want > j.ctx->budget)
        return fail(RPD_ERR_OVER_BUDGET, "staging buffer of " + std::to_string(want) + " bytes exceeds the HBM budget");
    cudaError_t e = ordered ? cudaMallocFromPoolAsync(buf, want, j.pool, j.stream) : cudaMalloc(buf, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(RPD_ERR_OUT_OF_MEMORY, std::string("cudaMalloc staging: ") + cudaGetErrorString(e));
    }
    j.ctx->in_use += want;
    *cap = want;
    return RPD_OK;
}

int ensure_offsets(Job& j, int64_t count) {
    // count+1 offsets plus room for the scan's block sums and block maxima
    const int64_t need = count + 1 + 2 * ((count + 1023) / 1024) + 4;
    if (j.offsets_cap >= need) return RPD_OK;
    if (j.offsets) {
        job_free(j, j.offsets);
        j.ctx->in_use -= uint64_t(j.offsets_cap) * 8;
        j.offsets = nullptr;
        j.offsets_cap = 0;
    }
    const int64_t want = need + need / 8 + 64;
    cudaError_t e = job_alloc(j, reinterpret_cast<void**>(&j.offsets), uint64_t(want) * 8);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(RPD_ERR_OUT_OF_MEMORY, std::string("cudaMalloc offsets: ") + cudaGetErrorString(e));
    }
    j.ctx->in_use += uint64_t(want) * 8;
    j.offsets_cap = want;
    return RPD_OK;
}

int ensure_features(Job& j) {
    if (j.features_valid) return RPD_OK;
    RPD_CUDA(launch_feature_cache(j));
    j.features_valid = true;
    return RPD_OK;
}

int ensure_cache(Job& j) {
    if (j.cache_valid) return RPD_OK;
    RPD_CUDA(launch_rpd_cache(j));
    j.cache_valid = true;
    return RPD_OK;
}

#define CHECK_JOB(j) \
    if (!(j)) return fail(RPD_ERR_INVALID_ARGUMENT, "null job handle")

}  // namespace

void set_error(const std::string& msg) { t_last_error = msg; }
int fail(int status, const std::string& msg) {
    t_last_error = msg;
    return status;
}
int cuda_fail(cudaError_t e, const char* what) {
    cudaGetLastError();
    t_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return RPD_ERR_CUDA;
}

}  // namespace rpd

using namespace rpd;

extern "C" {

const char* rpd_last_error(void) { return t_last_error.c_str(); }

const char* rpd_status_string(int s) {
    switch (s) {
    case RPD_OK: return "ok";
    case RPD_ERR_INVALID_CONFIG: return "invalid config";
    case RPD_ERR_INVALID_ARGUMENT: return "invalid argument";
    case RPD_ERR_OUT_OF_MEMORY: return "out of memory";
    case RPD_ERR_OVER_BUDGET: return "over HBM budget";
    case RPD_ERR_CUDA: return "CUDA error";
    case RPD_ERR_TIMEOUT: return "device wait timed out";
    case RPD_ERR_STATE: return "call out of order";
    case RPD_ERR_NO_DEVICE: return "no sm_103 device";
    case RPD_ERR_CANCELLED: return "cancelled";
    default: return "unknown status";
    }
}

void rpd_config_defaults(rpd_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    // RenderConfig defaults (core/config.h:28-47)
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

int rpd_config_validate(const rpd_config* c, char* msg, size_t cap) {
    auto bad = [&](const char* text) {
        if (msg && cap) {
            std::strncpy(msg, text, cap - 1);
            msg[cap - 1] = 0;
        }
        set_error(text);
        return int(RPD_ERR_INVALID_CONFIG);
    };
    if (!c) return bad("null config");
    // parse_render_config's checks (core/config.h:116-195) on the stage's fields
    if (c->image_width <= 0 || c->image_height <= 0) return bad("image_width and image_height must be positive");
    if (c->rpf_tile_size <= 0) return bad("rpf_tile_size must be positive");
    if (c->color_window_radius <= 0) return bad("color_window_radius must be positive");
    if (!std::isfinite(c->color_normal_threshold) || c->color_normal_threshold <= 0.0f || c->color_normal_threshold > 1.0f)
        return bad("color_normal_threshold must be finite and in (0,1]");
    if (!std::isfinite(c->color_depth_threshold) || c->color_depth_threshold < 0.0f)
        return bad("color_depth_threshold must be finite and non-negative");
    if (!std::isfinite(c->color_compat_alpha) || c->color_compat_alpha <= 0.0f || c->color_compat_alpha >= 1.0f)
        return bad("color_compat_alpha must be finite and in (0,1)");
    if (!std::isfinite(c->color_sigma_max) || c->color_sigma_max <= 0.0f)
        return bad("color_sigma_max must be finite and positive");
    if (c->var_window_radius <= 0) return bad("var_window_radius must be positive");
    if (!std::isfinite(c->var_normal_threshold) || c->var_normal_threshold <= 0.0f || c->var_normal_threshold > 1.0f)
        return bad("var_normal_threshold must be finite and in (0,1]");
    if (!std::isfinite(c->var_depth_threshold) || c->var_depth_threshold < 0.0f)
        return bad("var_depth_threshold must be finite and non-negative");
    if (!std::isfinite(c->var_compat_sigma) || c->var_compat_sigma <= 0.0f)
        return bad("var_compat_sigma must be finite and positive");
    if (!std::isfinite(c->var_shrinkage_k) || c->var_shrinkage_k <= 0.0f)
        return bad("var_shrinkage_k must be finite and positive");
    if (c->adaptive_base_samples < 0) return bad("adaptive_base_samples must be non-negative");
    if (c->adaptive_spp < 0) return bad("adaptive_spp must be non-negative");
    if (c->adaptive_base_samples > c->adaptive_spp) return bad("adaptive_base_samples cannot exceed adaptive_spp");
    if (!std::isfinite(c->adaptive_sigma_max) || c->adaptive_sigma_max <= 0.0f)
        return bad("adaptive_sigma_max must be finite and positive");
    if (c->adaptive_passes < 0) return bad("adaptive_passes must be non-negative");
    if (c->adaptive_importance_smoothing_radius < 0) return bad("adaptive_importance_smoothing_radius must be non-negative");
    if (c->var_iterations <= 0) return bad("var_iterations must be positive");
    if (!std::isfinite(c->rpf_shrinkage_scale) || c->rpf_shrinkage_scale < 0.0f)
        return bad("rpf_shrinkage_scale must be finite and non-negative");
    if (!std::isfinite(c->rpf_confidence_samples) || c->rpf_confidence_samples <= 0.0f)
        return bad("rpf_confidence_samples must be finite and positive");
    if (int64_t(c->image_width) * c->image_height > (int64_t(1) << 31) / 8)
        return bad("image is too large for 32-bit sample budgets");
    if (msg && cap) msg[0] = 0;
    return RPD_OK;
}

int rpd_ctx_create(int device, uint64_t budget, rpd_ctx** out) {
    if (!out) return fail(RPD_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    std::string why;
    if (!device_ok(device, &why)) return fail(RPD_ERR_NO_DEVICE, why);
    RPD_CUDA(cudaSetDevice(device));
    size_t free_b = 0, total_b = 0;
    RPD_CUDA(cudaMemGetInfo(&free_b, &total_b));
    Ctx* c = new (std::nothrow) Ctx();
    if (!c) return fail(RPD_ERR_OUT_OF_MEMORY, "context allocation failed");
    c->device = device;
    c->budget = budget ? budget : uint64_t(free_b);
    cudaError_t e = cudaStreamCreateWithFlags(&c->util_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        if (c->util_stream) cudaStreamDestroy(c->util_stream);
        delete c;
        return cuda_fail(e, "cudaStreamCreate");
    }
    *out = reinterpret_cast<rpd_ctx*>(c);
    return RPD_OK;
}

void rpd_ctx_destroy(rpd_ctx* ctx) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->util_stream) cudaStreamDestroy(c->util_stream);
    delete c;
}

uint64_t rpd_ctx_bytes_in_use(const rpd_ctx* ctx) {
    const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
    return c ? c->in_use.load() : 0;
}

uint64_t rpd_job_footprint(const rpd_config* cfg) {
    if (!cfg || cfg->image_width <= 0 || cfg->image_height <= 0 || cfg->rpf_tile_size <= 0) return 0;
    PixelPlanes p{};
    NodePlanes n{};
    return plan(make_geometry(*cfg), p, n);
}

int rpd_job_create(rpd_ctx* ctx, const rpd_config* cfg, rpd_job** out) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !cfg || !out) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    Job* j = nullptr;
    const int st = job_create(c, cfg, nullptr, &j);
    if (st == RPD_OK) *out = reinterpret_cast<rpd_job*>(j);
    return st;
}

}  // extern "C"

namespace rpd {

int job_create(Ctx* c, const rpd_config* cfg, cudaMemPool_t pool, Job** out) {
    *out = nullptr;
    char msg[256];
    if (rpd_config_validate(cfg, msg, sizeof(msg)) != RPD_OK) return fail(RPD_ERR_INVALID_CONFIG, msg);
    RPD_CUDA(cudaSetDevice(c->device));
    Job* j = new (std::nothrow) Job();
    if (!j) return fail(RPD_ERR_OUT_OF_MEMORY, "job allocation failed");
    j->ctx = c;
    j->cfg = *cfg;
    j->g = make_geometry(*cfg);
    j->pool = pool;
    j->arena_bytes = plan(j->g, j->p, j->n, j->cls, &j->pat4, &j->pat2);
    // the streams first: a pool job's arena is allocated in the order of its stream
    cudaError_t e = cudaStreamCreateWithFlags(&j->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete j;
        return cuda_fail(e, "job stream");
    }
    {
        std::lock_guard<std::mutex> lock(c->mu);
        if (c->in_use.load() + j->arena_bytes > c->budget) {
            const uint64_t need = j->arena_bytes;
            cudaStreamDestroy(j->stream);
            delete j;
            return fail(RPD_ERR_OVER_BUDGET, "job needs " + std::to_string(need) + " bytes of HBM; " +
                                                 std::to_string(c->budget - std::min(c->budget, c->in_use.load())) +
                                                 " left in the budget");
        }
        e = job_alloc(*j, &j->arena, j->arena_bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            j->arena = nullptr;
            cudaStreamDestroy(j->stream);
            delete j;
            return fail(RPD_ERR_OUT_OF_MEMORY, std::string("job arena: ") + cudaGetErrorString(e));
        }
        c->in_use += j->arena_bytes;
    }
    rebase_all(j->p, j->n, static_cast<char*>(j->arena));
    for (int c = 0; c < kClasses; ++c)
        for (int f = 0; f < 5; ++f) rebase(j->cls[c][f], static_cast<char*>(j->arena));
    rebase(j->pat4, static_cast<char*>(j->arena));
    rebase(j->pat2, static_cast<char*>(j->arena));
    e = cudaStreamCreateWithFlags(&j->copy_stream, cudaStreamNonBlocking);
    for (int b = 0; b < Job::kMaxBands && e == cudaSuccess; ++b)
        e = cudaEventCreateWithFlags(&j->band_copied[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j->staging_free, cudaEventDisableTiming);
    for (int s = 0; s < RPD_STAGE_COUNT_ && e == cudaSuccess; ++s) {
        e = cudaEventCreate(&j->ev_start[s]);
        if (e == cudaSuccess) e = cudaEventCreate(&j->ev_stop[s]);
    }
    if (e == cudaSuccess) e = cudaMallocHost(&j->scalars, 64);
    if (e == cudaSuccess) e = cudaMemsetAsync(j->arena, 0, j->arena_bytes, j->stream);
    if (e != cudaSuccess) {
        rpd_job_destroy(reinterpret_cast<rpd_job*>(j));
        return cuda_fail(e, "job set-up");
    }
    *out = j;
    return RPD_OK;
}

}  // namespace rpd

extern "C" {

void rpd_job_destroy(rpd_job* job) {
    Job* j = reinterpret_cast<Job*>(job);
    if (!j) return;
    cudaSetDevice(j->ctx->device);
    if (j->stream) cudaStreamSynchronize(j->stream);
    if (j->copy_stream) cudaStreamSynchronize(j->copy_stream);
    // a pool job's buffers go back to the pool in stream order (the streams are idle here)
    if (j->arena) {
        job_free(*j, j->arena);
        j->ctx->in_use -= j->arena_bytes;
    }
    if (j->staging) {
        cudaFree(j->staging);
        j->ctx->in_use -= j->staging_bytes;
    }
    if (j->offsets) {
        job_free(*j, j->offsets);
        j->ctx->in_use -= uint64_t(j->offsets_cap) * 8;
    }
    if (j->lum) {
        job_free(*j, j->lum);
        j->ctx->in_use -= j->lum_cap;
    }
    if (j->scalars) cudaFreeHost(j->scalars);
    for (int s = 0; s < RPD_STAGE_COUNT_; ++s) {
        if (j->ev_start[s]) cudaEventDestroy(j->ev_start[s]);
        if (j->ev_stop[s]) cudaEventDestroy(j->ev_stop[s]);
    }
    for (auto& t : j->ktimes) {
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    for (auto e : j->event_pool) cudaEventDestroy(e);
    for (auto e : j->marks)
        if (e) cudaEventDestroy(e);
    for (int b = 0; b < Job::kMaxBands; ++b)
        if (j->band_copied[b]) cudaEventDestroy(j->band_copied[b]);
    if (j->staging_free) cudaEventDestroy(j->staging_free);
    if (j->copy_stream) cudaStreamDestroy(j->copy_stream);
    if (j->stream) cudaStreamDestroy(j->stream);
    delete j;
}

int rpd_job_set_config(rpd_job* job, const rpd_config* cfg) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (!cfg) return fail(RPD_ERR_INVALID_ARGUMENT, "null config");
    rpd_config c = *cfg;
    c.image_width = j->cfg.image_width;
    c.image_height = j->cfg.image_height;
    c.rpf_tile_size = j->cfg.rpf_tile_size;
    char msg[256];
    if (rpd_config_validate(&c, msg, sizeof(msg)) != RPD_OK) return fail(RPD_ERR_INVALID_CONFIG, msg);
    j->cfg = c;
    return RPD_OK;
}

int rpd_job_set_exact(rpd_job* job, int flags) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (flags & ~(RPD_EXACT_GRID | RPD_EXACT_WINDOW)) return fail(RPD_ERR_INVALID_ARGUMENT, "unknown exact-mode flag");
    if (j->pass_open && bool(flags & RPD_EXACT_GRID) != j->exact_grid)
        return fail(RPD_ERR_STATE, "the grid mode cannot change while a pass is open");
    j->exact_grid = (flags & RPD_EXACT_GRID) != 0;
    j->exact_window = (flags & RPD_EXACT_WINDOW) != 0;
    return RPD_OK;
}

int rpd_job_set_tuning(rpd_job* job, int knob, int value) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (knob == RPD_TUNE_GRID_SHAPE) {
        if (value < 1 || value > 6) return fail(RPD_ERR_INVALID_ARGUMENT, "grid shape must be 1..6");
        j->grid_shape = value;
        return RPD_OK;
    }
    if (knob == RPD_TUNE_HOST_BAND_MB) {
        if (value < 1 || value > 65536) return fail(RPD_ERR_INVALID_ARGUMENT, "host band size must be 1..65536 MB");
        j->band_bytes = int64_t(value) << 20;
        return RPD_OK;
    }
    if (knob == RPD_TUNE_STATMC_ROWS) {
        if (value != 0 && value != 2 && value != 4 && value != 8)
            return fail(RPD_ERR_INVALID_ARGUMENT, "StatMC tile rows must be 0, 2, 4 or 8");
        j->statmc_by = value;
        return RPD_OK;
    }
    if (knob == RPD_TUNE_ALLOCATOR) {
        if (value < 0 || value > 4096) return fail(RPD_ERR_INVALID_ARGUMENT, "allocator must be 0..4096");
        j->serial_allocator = value == 1;
        j->allocator_blocks = value >= 2 ? value : 0;
        return RPD_OK;
    }
    if (knob == RPD_TUNE_SMOOTHING) {
        if (value != 0 && value != 1) return fail(RPD_ERR_INVALID_ARGUMENT, "smoothing must be 0 or 1");
        j->smooth_fp64 = value == 1;
        return RPD_OK;
    }
    if (knob == RPD_TUNE_WINDOW_GUARD) {
        if (value < 0 || value > 15) return fail(RPD_ERR_INVALID_ARGUMENT, "window guard must be 0..15");
        j->window_guard = value;
        return RPD_OK;
    }
    return fail(RPD_ERR_INVALID_ARGUMENT, "unknown tuning knob");
}

int rpd_job_get_tuning(rpd_job* job, int knob, int* value) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (!value) return fail(RPD_ERR_INVALID_ARGUMENT, "null value");
    if (knob == RPD_TUNE_GRID_SHAPE) *value = j->grid_shape;
    else if (knob == RPD_TUNE_HOST_BAND_MB) *value = int(j->band_bytes >> 20);
    else if (knob == RPD_TUNE_STATMC_ROWS) *value = j->statmc_by;
    else if (knob == RPD_TUNE_ALLOCATOR) *value = j->serial_allocator ? 1 : j->allocator_blocks;
    else if (knob == RPD_TUNE_SMOOTHING) *value = j->smooth_fp64 ? 1 : 0;
    else if (knob == RPD_TUNE_WINDOW_GUARD) *value = j->window_guard;
    else return fail(RPD_ERR_INVALID_ARGUMENT, "unknown tuning knob");
    return RPD_OK;
}

int rpd_job_begin_frame(rpd_job* job) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    // only the per-pixel accumulators start from zero (render_image_statmc's buffers.init and
    // pixel_stats reset): they are contiguous from the Welford mean to the depth sum. Every
    // other plane is written whole by the stage that produces it; the frame grid is assigned by
    // the first merge; the pass grid is cleared by each merge (and here if a pass was left open).
    const char* acc0 = reinterpret_cast<const char*>(j->p.mean);
    const char* acc1 = reinterpret_cast<const char*>(j->p.depth + j->g.np);
    RPD_CUDA(cudaMemsetAsync(j->p.mean, 0, size_t(acc1 - acc0), j->stream));
    if (j->pass_open)
        RPD_CUDA(cudaMemsetAsync(j->n.pass_grid, 0, size_t(j->g.nn) * kDeps * kDepStride * sizeof(double), j->stream));
    j->grid_fresh = true;
    j->pass_direct = j->pass_indirect = false;
    j->acc_zero = true;
    j->pass_open = false;
    j->features_valid = false;
    j->cache_valid = false;
    j->have_samples = false;
    return RPD_OK;
}

static int push_tail(Job* j, DeviceSamples& d, int64_t first, int64_t count, int32_t spp, const int32_t* counts,
                     rpd_memory where, int64_t total);

// One host-memory plane of a push: its source, bytes per element, whether it has one element
// per pixel (else per sample) and where its device pointer goes in a DeviceSamples.
struct HostPlane {
    const void* src;
    uint32_t elem;
    bool per_pixel;
    size_t field;
};

// A host push in row bands: every band's planes are copied on the job's copy stream into the
// staging buffer (one region per band), and each band's statistics and grid passes start on the
// job stream as soon as its copy is done, overlapping the copies of the later bands (a pass
// pushed in bands accumulates exactly as one push). The copies wait only for the previous host
// push's passes to release the staging. Returns when every copy has completed, so the caller
// may reuse its host planes; for the asynchronous pushes (j->host_async) it returns once the copies
// are enqueued, and the job stream's passes wait for them.
static int push_host_banded(Job* j, const std::vector<HostPlane>& planes, const DeviceSamples& proto, int64_t first,
                            int64_t count, int32_t spp, const int32_t* counts, int64_t total) {
    std::vector<int64_t> pre;
    if (counts) {
        pre.resize(size_t(count) + 1);
        pre[0] = 0;
        for (int64_t i = 0; i < count; ++i) pre[size_t(i) + 1] = pre[size_t(i)] + counts[i];
    }
    auto sample_at = [&](int64_t p) { return counts ? pre[size_t(p)] : p * int64_t(spp); };
    uint64_t per_sample = 0;
    for (const auto& hp : planes)
        if (!hp.per_pixel) per_sample += hp.elem;
    const uint64_t total_bytes = uint64_t(total) * per_sample;
    // bands of about j->band_bytes, at most kMaxBands, on image-row boundaries
    const int w = j->g.w;
    const int64_t rows = (first + count - 1) / w - first / w + 1;
    int64_t nbands = int64_t(total_bytes / uint64_t(j->band_bytes));
    nbands = std::max<int64_t>(1, std::min<int64_t>({nbands, int64_t(Job::kMaxBands), rows}));
    const int64_t rows_per_band = (rows + nbands - 1) / nbands;
    struct Band { int64_t p0, p1, k0, k1; uint64_t off; };
    std::vector<Band> bands;
    uint64_t need = 0;
    for (int64_t p0 = 0; p0 < count;) {
        const int64_t row0 = (first + p0) / w;
        const int64_t p1 = std::min<int64_t>(count, (row0 + rows_per_band) * w - first);
        Band b{p0, p1, sample_at(p0), sample_at(p1), (need + 255) & ~uint64_t(255)};
        need = b.off;
        for (const auto& hp : planes)
            need = ((need + 255) & ~uint64_t(255)) + uint64_t(hp.per_pixel ? p1 - p0 : b.k1 - b.k0) * hp.elem;
        if (counts) need = ((need + 255) & ~uint64_t(255)) + uint64_t(p1 - p0) * 4;
        bands.push_back(b);
        p0 = p1;
    }
    if (j->staging_bytes < need + 256) {
        RPD_CUDA(cudaStreamSynchronize(j->stream));  // the previous push's passes are done with it
        int st = grow_device(*j, &j->staging, &j->staging_bytes, need + 256);
        if (st != RPD_OK) return st;
    }
    RPD_CUDA(cudaStreamWaitEvent(j->copy_stream, j->staging_free, 0));
    char* base = static_cast<char*>(j->staging);
    std::vector<DeviceSamples> dev(bands.size(), proto);
    std::vector<const int32_t*> dcounts(bands.size(), nullptr);
    for (size_t bi = 0; bi < bands.size(); ++bi) {
        const Band& b = bands[bi];
        uint64_t off = b.off;
        for (const auto& hp : planes) {
            off = (off + 255) & ~uint64_t(255);
            const int64_t e0 = hp.per_pixel ? b.p0 : b.k0, n = hp.per_pixel ? b.p1 - b.p0 : b.k1 - b.k0;
            const uint64_t bytes = uint64_t(n) * hp.elem;
            if (bytes)
                RPD_CUDA(cudaMemcpyAsync(base + off, static_cast<const char*>(hp.src) + uint64_t(e0) * hp.elem, bytes,
                                         cudaMemcpyHostToDevice, j->copy_stream));
            *reinterpret_cast<const void**>(reinterpret_cast<char*>(&dev[bi]) + hp.field) = base + off;
            off += bytes;
        }
        if (counts) {
            off = (off + 255) & ~uint64_t(255);
            RPD_CUDA(cudaMemcpyAsync(base + off, counts + b.p0, uint64_t(b.p1 - b.p0) * 4, cudaMemcpyHostToDevice,
                                     j->copy_stream));
            dcounts[bi] = reinterpret_cast<const int32_t*>(base + off);
        }
        RPD_CUDA(cudaEventRecord(j->band_copied[bi], j->copy_stream));
    }
    for (size_t bi = 0; bi < bands.size(); ++bi) {
        const Band& b = bands[bi];
        RPD_CUDA(cudaStreamWaitEvent(j->stream, j->band_copied[bi], 0));
        if (counts) RPD_CUDA(launch_offsets_scan(*j, dcounts[bi], b.p1 - b.p0));
        else RPD_CUDA(launch_offsets_uniform(*j, b.p1 - b.p0, spp));
        const int st = push_tail(j, dev[bi], first + b.p0, b.p1 - b.p0, spp, counts ? counts + b.p0 : nullptr,
                                 RPD_MEM_HOST, b.k1 - b.k0);
        if (st != RPD_OK) return st;
    }
    RPD_CUDA(cudaEventRecord(j->staging_free, j->stream));
    if (!j->host_async) RPD_CUDA(cudaStreamSynchronize(j->copy_stream));
    return RPD_OK;
}

int rpd_job_push_samples(rpd_job* job, const rpd_sample_soa* s, int64_t first, int64_t count, int32_t spp,
                         const int32_t* counts, rpd_memory where) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (!s) return fail(RPD_ERR_INVALID_ARGUMENT, "null sample planes");
    if (first < 0 || count < 0 || first + count > j->g.np)
        return fail(RPD_ERR_INVALID_ARGUMENT, "pixel span [" + std::to_string(first) + ", " +
                                                  std::to_string(first + count) + ") is outside the image");
    if (!counts && spp < 0) return fail(RPD_ERR_INVALID_ARGUMENT, "negative spp");
    if (count == 0) return RPD_OK;
    if (!s->radiance[0] || !s->radiance[1] || !s->radiance[2])
        return fail(RPD_ERR_INVALID_ARGUMENT, "radiance planes are required");
    if (!s->flags) return fail(RPD_ERR_INVALID_ARGUMENT, "flags plane is required");
    {
        // a multi-component plane is either fully present or fully absent
        auto pair_ok = [](const float* const* v, int n) {
            int present = 0;
            for (int c = 0; c < n; ++c) present += v[c] != nullptr;
            return present == 0 || present == n;
        };
        if (!pair_ok(s->normal, 3) || !pair_ok(s->albedo, 3) || !pair_ok(s->pixel_albedo, 3) ||
            !pair_ok(s->pixel_u, 2) || !pair_ok(s->lens_u, 2) || !pair_ok(s->brdf_u, 2) || !pair_ok(s->light_u, 2) ||
            !pair_ok(s->env_u, 2))
            return fail(RPD_ERR_INVALID_ARGUMENT, "a multi-component sample plane is only partly given");
    }
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    int st = ensure_offsets(*j, count);
    if (st != RPD_OK) return st;

    StageTimer timer(*j, RPD_STAGE_ACCUMULATE);
    int64_t total = 0;
    if (counts) {
        if (where == RPD_MEM_HOST) {
            for (int64_t i = 0; i < count; ++i) {
                if (counts[i] < 0) return fail(RPD_ERR_INVALID_ARGUMENT, "negative per-pixel sample count");
                total += counts[i];
            }
        }
    } else {
        total = int64_t(count) * spp;
    }

    DeviceSamples d{};
    if (where == RPD_MEM_HOST) {
        if (!s->normal[0] || !s->depth || (!s->albedo[0] && !s->pixel_albedo[0]))
            return fail(RPD_ERR_INVALID_ARGUMENT, "normal, depth and albedo (per sample or per pixel) are required");
        if (j->cfg.rpf_shrinkage_scale > 0.0f && !s->category)
            return fail(RPD_ERR_INVALID_ARGUMENT, "category plane is required when RPD is enabled");
        std::vector<HostPlane> planes;
        auto add = [&](const void* src, uint32_t elem, bool per_pixel, const void* const& field) {
            if (src)
                planes.push_back({src, elem, per_pixel,
                                  size_t(reinterpret_cast<const char*>(&field) - reinterpret_cast<const char*>(&d))});
        };
        for (int c = 0; c < 3; ++c) {
            add(s->radiance[c], 4, false, reinterpret_cast<const void* const&>(d.radiance[c]));
            add(s->normal[c], 4, false, reinterpret_cast<const void* const&>(d.normal[c]));
            add(s->albedo[c], 4, false, reinterpret_cast<const void* const&>(d.albedo[c]));
            add(s->pixel_albedo[c], 4, true, reinterpret_cast<const void* const&>(d.pixel_albedo[c]));
        }
        add(s->depth, 4, false, reinterpret_cast<const void* const&>(d.depth));
        for (int c = 0; c < 2; ++c) {
            add(s->pixel_u[c], 4, false, reinterpret_cast<const void* const&>(d.pixel_u[c]));
            add(s->lens_u[c], 4, false, reinterpret_cast<const void* const&>(d.lens_u[c]));
            add(s->brdf_u[c], 4, false, reinterpret_cast<const void* const&>(d.brdf_u[c]));
            add(s->light_u[c], 4, false, reinterpret_cast<const void* const&>(d.light_u[c]));
            add(s->env_u[c], 4, false, reinterpret_cast<const void* const&>(d.env_u[c]));
        }
        add(s->flags, 1, false, reinterpret_cast<const void* const&>(d.flags));
        add(s->category, 1, false, reinterpret_cast<const void* const&>(d.category));
        return push_host_banded(j, planes, d, first, count, spp, counts, total);
    } else {
        for (int c = 0; c < 3; ++c) {
            d.radiance[c] = s->radiance[c];
            d.normal[c] = s->normal[c];
            d.albedo[c] = s->albedo[c];
            d.pixel_albedo[c] = s->pixel_albedo[c];
        }
        d.depth = s->depth;
        for (int c = 0; c < 2; ++c) {
            d.pixel_u[c] = s->pixel_u[c];
            d.lens_u[c] = s->lens_u[c];
            d.brdf_u[c] = s->brdf_u[c];
            d.light_u[c] = s->light_u[c];
            d.env_u[c] = s->env_u[c];
        }
        d.flags = s->flags;
        d.category = s->category;
        if (counts) RPD_CUDA(launch_offsets_scan(*j, counts, count));
        else RPD_CUDA(launch_offsets_uniform(*j, count, spp));
    }
    if (!d.normal[0] || !d.normal[1] || !d.normal[2] || !d.depth ||
        (!d.albedo[0] && !d.pixel_albedo[0]))
        return fail(RPD_ERR_INVALID_ARGUMENT, "normal, depth and albedo (per sample or per pixel) are required");
    return push_tail(j, d, first, count, spp, counts, where, total);
}

// The part of a push shared by both sample formats: the offsets are computed, d points at
// device planes. Runs the statistics pass and the grid pass.
int rpd_job_push_samples16(rpd_job* job, const rpd_sample_soa16* s, int64_t first, int64_t count, int32_t spp,
                           const int32_t* counts, rpd_memory where) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (!s) return fail(RPD_ERR_INVALID_ARGUMENT, "null sample planes");
    if (first < 0 || count < 0 || first + count > j->g.np)
        return fail(RPD_ERR_INVALID_ARGUMENT, "pixel span [" + std::to_string(first) + ", " +
                                                  std::to_string(first + count) + ") is outside the image");
    if (!counts && spp < 0) return fail(RPD_ERR_INVALID_ARGUMENT, "negative spp");
    if (j->exact_grid) return fail(RPD_ERR_STATE, "the exact grid mode needs rpd_sample_soa planes");
    if (count == 0) return RPD_OK;
    for (int c = 0; c < 3; ++c)
        if (!s->sqrt_radiance[c] || !s->normal[c] || !s->pixel_albedo[c])
            return fail(RPD_ERR_INVALID_ARGUMENT, "sqrt_radiance, normal and pixel_albedo planes are required");
    if (!s->depth || !s->flags) return fail(RPD_ERR_INVALID_ARGUMENT, "depth and flags planes are required");
    if (!(s->depth_scale > 0.0f) || !std::isfinite(s->depth_scale))
        return fail(RPD_ERR_INVALID_ARGUMENT, "depth_scale must be finite and positive");
    {
        auto pair_ok = [](const uint16_t* const* v) { return (v[0] == nullptr) == (v[1] == nullptr); };
        if (!pair_ok(s->pixel_u) || !pair_ok(s->lens_u) || !pair_ok(s->brdf_u) || !pair_ok(s->light_u) ||
            !pair_ok(s->env_u))
            return fail(RPD_ERR_INVALID_ARGUMENT, "a multi-component sample plane is only partly given");
    }
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    int st = ensure_offsets(*j, count);
    if (st != RPD_OK) return st;
    StageTimer timer(*j, RPD_STAGE_ACCUMULATE);
    int64_t total = 0;
    if (counts) {
        if (where == RPD_MEM_HOST) {
            for (int64_t i = 0; i < count; ++i) {
                if (counts[i] < 0) return fail(RPD_ERR_INVALID_ARGUMENT, "negative per-pixel sample count");
                total += counts[i];
            }
        }
    } else {
        total = int64_t(count) * spp;
    }
    DeviceSamples d{};
    d.compact = 1;
    d.c16.depth_scale = s->depth_scale;
    if (where == RPD_MEM_HOST) {
        if (j->cfg.rpf_shrinkage_scale > 0.0f && !s->category)
            return fail(RPD_ERR_INVALID_ARGUMENT, "category plane is required when RPD is enabled");
        std::vector<HostPlane> planes;
        auto add = [&](const void* src, uint32_t elem, bool per_pixel, const void* const& field) {
            if (src)
                planes.push_back({src, elem, per_pixel,
                                  size_t(reinterpret_cast<const char*>(&field) - reinterpret_cast<const char*>(&d))});
        };
        for (int c = 0; c < 3; ++c) {
            add(s->sqrt_radiance[c], 2, false, reinterpret_cast<const void* const&>(d.c16.sqrt_radiance[c]));
            add(s->normal[c], 2, false, reinterpret_cast<const void* const&>(d.c16.normal[c]));
            add(s->pixel_albedo[c], 2, true, reinterpret_cast<const void* const&>(d.c16.pixel_albedo[c]));
        }
        add(s->depth, 2, false, reinterpret_cast<const void* const&>(d.c16.depth));
        for (int c = 0; c < 2; ++c) {
            add(s->pixel_u[c], 2, false, reinterpret_cast<const void* const&>(d.c16.pixel_u[c]));
            add(s->lens_u[c], 2, false, reinterpret_cast<const void* const&>(d.c16.lens_u[c]));
            add(s->brdf_u[c], 2, false, reinterpret_cast<const void* const&>(d.c16.brdf_u[c]));
            add(s->light_u[c], 2, false, reinterpret_cast<const void* const&>(d.c16.light_u[c]));
            add(s->env_u[c], 2, false, reinterpret_cast<const void* const&>(d.c16.env_u[c]));
        }
        add(s->flags, 1, false, reinterpret_cast<const void* const&>(d.flags));
        add(s->category, 1, false, reinterpret_cast<const void* const&>(d.category));
        return push_host_banded(j, planes, d, first, count, spp, counts, total);
    } else {
        for (int c = 0; c < 3; ++c) {
            d.c16.sqrt_radiance[c] = s->sqrt_radiance[c];
            d.c16.normal[c] = s->normal[c];
            d.c16.pixel_albedo[c] = s->pixel_albedo[c];
        }
        d.c16.depth = s->depth;
        for (int c = 0; c < 2; ++c) {
            d.c16.pixel_u[c] = s->pixel_u[c];
            d.c16.lens_u[c] = s->lens_u[c];
            d.c16.brdf_u[c] = s->brdf_u[c];
            d.c16.light_u[c] = s->light_u[c];
            d.c16.env_u[c] = s->env_u[c];
        }
        d.flags = s->flags;
        d.category = s->category;
        if (counts) RPD_CUDA(launch_offsets_scan(*j, counts, count));
        else RPD_CUDA(launch_offsets_uniform(*j, count, spp));
    }
    return push_tail(j, d, first, count, spp, counts, where, total);
}

int rpd_encode_samples16(rpd_ctx* ctx, const rpd_sample_soa* in, int64_t n_samples, int64_t n_pixels,
                         const rpd_sample_soa16* out) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !in || !out || n_samples < 0 || n_pixels < 0) return fail(RPD_ERR_INVALID_ARGUMENT, "bad encode arguments");
    if (!(out->depth_scale > 0.0f) || !std::isfinite(out->depth_scale))
        return fail(RPD_ERR_INVALID_ARGUMENT, "depth_scale must be finite and positive");
    for (int k = 0; k < 3; ++k)
        if (!in->radiance[k] || !in->normal[k] || !out->sqrt_radiance[k] || !out->normal[k])
            return fail(RPD_ERR_INVALID_ARGUMENT, "radiance and normal planes are required on both sides");
    if (!in->depth || !out->depth) return fail(RPD_ERR_INVALID_ARGUMENT, "depth planes are required on both sides");
    DeviceSamples d{};
    for (int k = 0; k < 3; ++k) {
        d.radiance[k] = in->radiance[k];
        d.normal[k] = in->normal[k];
        d.pixel_albedo[k] = in->pixel_albedo[k];
    }
    d.depth = in->depth;
    DeviceSamples16 o{};
    for (int k = 0; k < 3; ++k) {
        o.sqrt_radiance[k] = out->sqrt_radiance[k];
        o.normal[k] = out->normal[k];
        o.pixel_albedo[k] = out->pixel_albedo[k];
    }
    o.depth = out->depth;
    o.depth_scale = out->depth_scale;
    auto dim = [](const float* const* a, const uint16_t* const* b, const float** da, const uint16_t** db) {
        if (a[0] && b[0]) {
            da[0] = a[0]; da[1] = a[1];
            db[0] = b[0]; db[1] = b[1];
        }
    };
    dim(in->pixel_u, out->pixel_u, d.pixel_u, o.pixel_u);
    dim(in->lens_u, out->lens_u, d.lens_u, o.lens_u);
    dim(in->brdf_u, out->brdf_u, d.brdf_u, o.brdf_u);
    dim(in->light_u, out->light_u, d.light_u, o.light_u);
    dim(in->env_u, out->env_u, d.env_u, o.env_u);
    RPD_CUDA(cudaSetDevice(c->device));
    RPD_CUDA(launch_encode_samples16(d, n_samples, n_pixels, o, c->util_stream));
    RPD_CUDA(cudaStreamSynchronize(c->util_stream));
    return RPD_OK;
}

static int push_tail(Job* j, DeviceSamples& d, int64_t first, int64_t count, int32_t spp, const int32_t* counts,
                     rpd_memory where, int64_t total) {
    int st = RPD_OK;
    const bool rpd = j->cfg.rpf_shrinkage_scale > 0.0f;
    if (rpd && !d.category) return fail(RPD_ERR_INVALID_ARGUMENT, "category plane is required when RPD is enabled");
    GridPrep gp{};
    gp.width = j->g.w;
    const bool fast_grid = rpd && !j->exact_grid;
    int64_t nsamp = total;
    if (fast_grid) {
        // the per-sample total (or a bound on it) is needed on the host to size the luminance plane
        if (counts && where != RPD_MEM_HOST && total <= 0) {
            RPD_CUDA(cudaMemcpyAsync(&nsamp, j->offsets + count, 8, cudaMemcpyDeviceToHost, j->stream));
            RPD_CUDA(cudaStreamSynchronize(j->stream));
        }
        // luminance, key (and, with per-pixel counts, column) planes of the push, one allocation
        const int64_t ns64 = ((std::max<int64_t>(nsamp, 1) + 63) / 64) * 64;
        const bool with_col = counts != nullptr && j->g.w <= 65535;
        void* lum = j->lum;
        st = grow_device(*j, &lum, &j->lum_cap, uint64_t(ns64) * (with_col ? 10 : 8) + 256, true);
        if (st != RPD_OK) return st;
        j->lum = static_cast<float*>(lum);
        gp.key = reinterpret_cast<uint32_t*>(j->lum + ns64);
        gp.col = with_col ? reinterpret_cast<uint16_t*>(gp.key + ns64) : nullptr;
        for (int c = 0; c < kClasses; ++c)
            for (int f = 0; f < 5; ++f) gp.cls[c][f] = j->cls[c][f];
        gp.pat4 = j->pat4;
        gp.pat2 = j->pat2;
        gp.lum = j->lum;
    }
    RPD_CUDA(launch_accumulate_pixels(*j, d, first, count, gp, counts ? 0 : spp));
    if (fast_grid) {
        int32_t max_count = spp;
        if (counts) {
            max_count = 0;
            if (where == RPD_MEM_HOST)
                for (int64_t i = 0; i < count; ++i) max_count = std::max(max_count, counts[i]);
            else
                max_count = INT32_MAX;  // unknown on the host: the push's total bounds the weights
        }
        // every push with per-pixel counts scanned them into j->offsets first
        const int64_t* d_max = (counts && max_count == INT32_MAX) ? offsets_count_max(*j, count) : nullptr;
        RPD_CUDA(launch_grid_fast(*j, d, first, count, gp, counts ? 0 : spp, max_count, nsamp, d_max));
    }
    else if (rpd) RPD_CUDA(launch_accumulate_grid(*j, d, first, count));
    j->pass_open = true;
    j->have_samples = true;
    j->features_valid = false;
    j->cache_valid = false;
    return RPD_OK;
}

int rpd_job_end_pass(rpd_job* job) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    if (j->pass_open && j->cfg.rpf_shrinkage_scale > 0.0f) RPD_CUDA(launch_merge_grid(*j));
    j->pass_open = false;
    j->features_valid = false;
    j->cache_valid = false;
    return RPD_OK;
}

int rpd_recompute_sensitivity(rpd_job* job) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    if (j->pass_open) {
        int st = rpd_job_end_pass(job);
        if (st != RPD_OK) return st;
    }
    StageTimer timer(*j, RPD_STAGE_SENSITIVITY);
    j->cache_valid = false;
    if (j->cfg.rpf_shrinkage_scale <= 0.0f) {
        RPD_CUDA(launch_sensitivity_zero(*j));
    } else {
        int st = ensure_features(*j);
        if (st != RPD_OK) return st;
        RPD_CUDA(launch_sensitivity(*j));
    }
    return ensure_cache(*j);
}

int rpd_statmc_denoise(rpd_job* job) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    StageTimer timer(*j, RPD_STAGE_STATMC);
    int st = ensure_features(*j);
    if (st != RPD_OK) return st;
    st = ensure_cache(*j);
    if (st != RPD_OK) return st;
    // the window's recheck counters and its slow-pixel list describe the last call
    RPD_CUDA(cudaMemsetAsync(j->p.counters + RPD_COUNTER_WINDOW_PAIR_RECHECKS, 0, 2 * sizeof(unsigned long long),
                             j->stream));
    RPD_CUDA(cudaMemsetAsync(j->p.counters + RPD_COUNTER_WINDOW_SLOW_PIXELS, 0, sizeof(unsigned long long),
                             j->stream));
    RPD_CUDA(launch_statmc(*j));
    return RPD_OK;
}

int rpd_variance_denoise(rpd_job* job) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    StageTimer timer(*j, RPD_STAGE_VARIANCE);
    int st = ensure_features(*j);
    if (st != RPD_OK) return st;
    RPD_CUDA(launch_variance(*j));
    return RPD_OK;
}

int rpd_compute_adaptive_sample_counts(rpd_job* job, int32_t* out, rpd_memory where) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    {
        StageTimer timer(*j, RPD_STAGE_ADAPTIVE);
        int st = ensure_features(*j);
        if (st != RPD_OK) return st;
        RPD_CUDA(launch_adaptive(*j));
    }
    if (out) {
        const uint64_t bytes = uint64_t(j->g.np) * 4;
        RPD_CUDA(cudaMemcpyAsync(out, j->p.counts, bytes,
                                 where == RPD_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, j->stream));
        if (where == RPD_MEM_HOST) RPD_CUDA(cudaStreamSynchronize(j->stream));
    }
    return RPD_OK;
}

int rpd_job_allocator_timeline(rpd_job* job, uint64_t* ns, int32_t max, int32_t* n_out) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (!ns || !n_out || max < 0) return fail(RPD_ERR_INVALID_ARGUMENT, "bad timeline arguments");
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    return allocator_timeline(*j, ns, max, n_out);
}

int rpd_adaptive_allocate(rpd_job* job, const float* importance, rpd_memory where, int32_t* counts_out,
                          rpd_memory out_where) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (!importance) return fail(RPD_ERR_INVALID_ARGUMENT, "null importance map");
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    const uint64_t bytes = uint64_t(j->g.np) * 4;
    RPD_CUDA(cudaMemcpyAsync(j->p.importance, importance, bytes,
                             where == RPD_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, j->stream));
    {
        StageTimer timer(*j, RPD_STAGE_ADAPTIVE);
        RPD_CUDA(launch_allocate_map(*j));
    }
    if (counts_out) {
        RPD_CUDA(cudaMemcpyAsync(counts_out, j->p.counts, bytes,
                                 out_where == RPD_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                                 j->stream));
        if (out_where == RPD_MEM_HOST) RPD_CUDA(cudaStreamSynchronize(j->stream));
    }
    return RPD_OK;
}

int rpd_job_allocator_stats(rpd_job* job, int32_t* out) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (!out) return fail(RPD_ERR_INVALID_ARGUMENT, "null output");
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    RPD_CUDA(allocator_stats(*j, out));
    return RPD_OK;
}

int rpd_finalize(rpd_job* job) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    RPD_CUDA(launch_finalize(*j));
    j->features_valid = false;
    return RPD_OK;
}

uint64_t rpd_field_bytes(const rpd_job* job, rpd_field f) {
    const Job* j = reinterpret_cast<const Job*>(job);
    if (!j) return 0;
    const uint64_t np = uint64_t(j->g.np), nn = uint64_t(j->g.nn);
    switch (f) {
    case RPD_FIELD_DENOISED: case RPD_FIELD_RADIANCE_SUM: case RPD_FIELD_NORMAL_SUM: case RPD_FIELD_ALBEDO_SUM:
    case RPD_FIELD_STATS_COLOR_MEAN: case RPD_FIELD_STATS_SQRT_MEAN: case RPD_FIELD_STATS_SQRT_SQUARE_DIFF:
    case RPD_FIELD_SQRT_VARIANCE_STABLE:
        return np * 12;
    case RPD_FIELD_GRID: return nn * kDeps * kDepStride * 8;
    default:
        if (f >= RPD_FIELD_NODE_ALL && f <= RPD_FIELD_NODE_RR_CONF) return nn * 4;
        if (f >= 0 && f < RPD_FIELD_COUNT_) return np * 4;
        return 0;
    }
}

static int job_read(rpd_job* job, rpd_field f, void* dst, size_t bytes, rpd_memory where, bool sync) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    const uint64_t need = rpd_field_bytes(job, f);
    if (need == 0 || bytes != need || !dst)
        return fail(RPD_ERR_INVALID_ARGUMENT, "field " + std::to_string(int(f)) + " needs " + std::to_string(need) +
                                                  " bytes, got " + std::to_string(bytes));
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    const int64_t np = j->g.np;
    const cudaMemcpyKind kind = where == RPD_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    const void* src = nullptr;
    float* const* rgb = nullptr;
    switch (f) {
    case RPD_FIELD_DENOISED: rgb = j->p.denoised; break;
    case RPD_FIELD_RADIANCE_SUM: rgb = j->p.radiance; break;
    case RPD_FIELD_NORMAL_SUM: rgb = j->p.normal; break;
    case RPD_FIELD_ALBEDO_SUM: rgb = j->p.albedo; break;
    case RPD_FIELD_STATS_COLOR_MEAN: rgb = j->p.color_mean; break;
    case RPD_FIELD_STATS_SQRT_MEAN: rgb = j->p.sqrt_mean; break;
    case RPD_FIELD_STATS_SQRT_SQUARE_DIFF: rgb = j->p.sqrt_sq; break;
    case RPD_FIELD_SQRT_VARIANCE_STABLE: rgb = j->p.sqrt_var_stable; break;
    case RPD_FIELD_UNCERTAINTY: src = j->p.uncertainty; break;
    case RPD_FIELD_ALPHA: src = j->p.alpha; break;
    case RPD_FIELD_VAR_TOTAL_DEBUG: src = j->p.var_total; break;
    case RPD_FIELD_VAR_EFF_DEBUG: src = j->p.var_eff; break;
    case RPD_FIELD_VAR_RATIO_DEBUG: src = j->p.var_ratio; break;
    case RPD_FIELD_VARIANCE_DENOISED: src = j->p.variance_denoised; break;
    case RPD_FIELD_ADAPTIVE_IMPORTANCE: src = j->p.importance; break;
    case RPD_FIELD_SENSITIVITY_CONFIDENCE: src = j->p.sens_confidence; break;
    case RPD_FIELD_SENSITIVITY_GRADIENT: src = j->p.sens_gradient; break;
    case RPD_FIELD_HIT_COUNT: src = j->p.hit_count; break;
    case RPD_FIELD_SAMPLE_COUNT: src = j->p.sample_count; break;
    case RPD_FIELD_DEPTH_SUM: src = j->p.depth; break;
    case RPD_FIELD_STATS_MEAN: src = j->p.mean; break;
    case RPD_FIELD_STATS_SQUARE_DIFF: src = j->p.square_diff; break;
    case RPD_FIELD_STATS_N: src = j->p.n; break;
    case RPD_FIELD_GRID: src = j->n.grid; break;
    case RPD_FIELD_ADAPTIVE_COUNTS: src = j->p.counts; break;
    default: break;
    }
    if (f >= RPD_FIELD_NODE_ALL && f <= RPD_FIELD_NODE_RR_CONF) src = j->n.field[f - RPD_FIELD_NODE_ALL];
    if (f == RPD_FIELD_GRID && j->grid_fresh) {  // no pass merged into this frame's grid yet: zeros
        if (where == RPD_MEM_HOST) std::memset(dst, 0, bytes);
        else RPD_CUDA(cudaMemsetAsync(dst, 0, bytes, j->stream));
        RPD_CUDA(cudaStreamSynchronize(j->stream));
        return RPD_OK;
    }
    if (f == RPD_FIELD_GRID && j->grid_pairs) src = nullptr;  // pairs: widened on the way out
    if (src) {
        RPD_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, j->stream));
        if (sync) RPD_CUDA(cudaStreamSynchronize(j->stream));
        return RPD_OK;
    }
    // fields computed on read go through the staging buffer
    int st = grow_device(*j, &j->staging, &j->staging_bytes, need);
    if (st != RPD_OK) return st;
    float* tmp = static_cast<float*>(j->staging);
    if (f == RPD_FIELD_GRID) {
        RPD_CUDA(launch_grid_to_double(*j, reinterpret_cast<double*>(tmp)));
    } else if (rgb) {
        k_pack3<<<grid_for(np, 256), 256, 0, j->stream>>>(rgb[0], rgb[1], rgb[2], tmp, np);
        j->launches += 1;
        RPD_CUDA(cudaGetLastError());
    } else if (f >= RPD_FIELD_EXPANDED_ALL && f <= RPD_FIELD_EXPANDED_RR) {
        static const int map[9] = {N_ALL, N_PIXEL, N_BRDF, N_LENS, N_LIGHT, N_LIGHT_UV, N_LIGHT_SELECT, N_ENV, N_RR};
        RPD_CUDA(launch_expand(*j, j->n.field[map[f - RPD_FIELD_EXPANDED_ALL]], tmp));
    } else {
        return fail(RPD_ERR_INVALID_ARGUMENT, "unknown field");
    }
    RPD_CUDA(cudaMemcpyAsync(dst, tmp, bytes, kind, j->stream));
    if (sync) {
        RPD_CUDA(cudaStreamSynchronize(j->stream));
    } else {
        RPD_CUDA(cudaEventRecord(j->staging_free, j->stream));  // the next host push waits for this copy
    }
    return RPD_OK;
}

int rpd_job_read(rpd_job* job, rpd_field f, void* dst, size_t bytes, rpd_memory where) {
    return job_read(job, f, dst, bytes, where, true);
}

int rpd_job_read_async(rpd_job* job, rpd_field f, void* dst, size_t bytes, rpd_memory where) {
    return job_read(job, f, dst, bytes, where, false);
}

int rpd_job_push_samples_async(rpd_job* job, const rpd_sample_soa* s, int64_t first, int64_t count, int32_t spp,
                               const int32_t* counts) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    j->host_async = true;
    const int st = rpd_job_push_samples(job, s, first, count, spp, counts, RPD_MEM_HOST);
    j->host_async = false;
    return st;
}

int rpd_job_push_samples16_async(rpd_job* job, const rpd_sample_soa16* s, int64_t first, int64_t count, int32_t spp,
                                 const int32_t* counts) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    j->host_async = true;
    const int st = rpd_job_push_samples16(job, s, first, count, spp, counts, RPD_MEM_HOST);
    j->host_async = false;
    return st;
}

int rpd_job_sync(rpd_job* job) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    RPD_CUDA(cudaStreamSynchronize(j->stream));
    unsigned long long timeouts = 0;
    RPD_CUDA(cudaMemcpy(&timeouts, j->p.counters + RPD_COUNTER_DEVICE_WAIT_TIMEOUTS, sizeof(timeouts),
                        cudaMemcpyDeviceToHost));
    if (timeouts)
        return fail(RPD_ERR_TIMEOUT, std::to_string(timeouts) + " bounded device wait(s) of this job gave up");
    return RPD_OK;
}

int rpd_job_counters(rpd_job* job, uint64_t* out, int32_t n) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (!out || n < 0) return fail(RPD_ERR_INVALID_ARGUMENT, "bad counter output");
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    RPD_CUDA(cudaStreamSynchronize(j->stream));
    unsigned long long c[RPD_COUNTER_COUNT_];
    RPD_CUDA(cudaMemcpy(c, j->p.counters, sizeof(c), cudaMemcpyDeviceToHost));
    for (int32_t i = 0; i < n && i < RPD_COUNTER_COUNT_; ++i) out[i] = c[i];
    return RPD_OK;
}

float rpd_job_stage_ms(const rpd_job* job, rpd_stage s) {
    const Job* j = reinterpret_cast<const Job*>(job);
    if (!j || s < 0 || s >= RPD_STAGE_COUNT_ || !j->ev_used[s]) return -1.0f;
    float ms = -1.0f;
    if (cudaEventSynchronize(j->ev_stop[s]) != cudaSuccess) return -1.0f;
    if (cudaEventElapsedTime(&ms, j->ev_start[s], j->ev_stop[s]) != cudaSuccess) return -1.0f;
    return ms;
}

uint64_t rpd_job_launch_count(const rpd_job* job) {
    const Job* j = reinterpret_cast<const Job*>(job);
    return j ? j->launches.load() : 0;
}

int rpd_job_set_profiling(rpd_job* job, int enable) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    j->profile = enable != 0;
    return RPD_OK;
}

static int fold_kernel_times(Job* j) {
    RPD_CUDA(cudaStreamSynchronize(j->stream));
    for (auto& t : j->ktimes) {
        float ms = 0.0f;
        RPD_CUDA(cudaEventElapsedTime(&ms, t.a, t.b));
        j->ktotal[t.kernel] += double(ms);
        j->kcount[t.kernel] += 1;
        j->event_pool.push_back(t.a);
        j->event_pool.push_back(t.b);
    }
    j->ktimes.clear();
    return RPD_OK;
}

int rpd_job_kernel_time(rpd_job* job, rpd_kernel k, double* total_ms, uint64_t* launches) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (k < 0 || k >= RPD_KERNEL_COUNT_) return fail(RPD_ERR_INVALID_ARGUMENT, "unknown kernel family");
    int st = fold_kernel_times(j);
    if (st != RPD_OK) return st;
    if (total_ms) *total_ms = j->ktotal[k];
    if (launches) *launches = j->kcount[k];
    return RPD_OK;
}

int rpd_job_reset_kernel_times(rpd_job* job) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    int st = fold_kernel_times(j);
    if (st != RPD_OK) return st;
    for (int k = 0; k < RPD_KERNEL_COUNT_; ++k) {
        j->ktotal[k] = 0.0;
        j->kcount[k] = 0;
    }
    return RPD_OK;
}

int rpd_job_mark(rpd_job* job, int slot) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (slot < 0 || slot >= 8) return fail(RPD_ERR_INVALID_ARGUMENT, "marker slot must be 0..7");
    if (!j->marks[slot]) RPD_CUDA(cudaEventCreate(&j->marks[slot]));
    RPD_CUDA(cudaEventRecord(j->marks[slot], j->stream));
    return RPD_OK;
}

int rpd_job_mark_elapsed(rpd_job* job, int a, int b, float* ms) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (a < 0 || a >= 8 || b < 0 || b >= 8 || !j->marks[a] || !j->marks[b] || !ms)
        return fail(RPD_ERR_INVALID_ARGUMENT, "marker slots were not recorded");
    RPD_CUDA(cudaEventSynchronize(j->marks[b]));
    RPD_CUDA(cudaEventElapsedTime(ms, j->marks[a], j->marks[b]));
    return RPD_OK;
}

const char* rpd_kernel_name(rpd_kernel k) {
    static const char* names[RPD_KERNEL_COUNT_] = {
        "offsets", "accumulate_pixels", "grid", "grid_random", "merge", "features", "node_stats", "node_combine",
        "sens_pixels", "rpd_cache", "sqrt_variance", "statmc_window", "variance", "adaptive", "other", "synth"};
    return (k >= 0 && k < RPD_KERNEL_COUNT_) ? names[k] : "unknown";
}

int rpd_device_alloc(rpd_ctx* ctx, uint64_t bytes, void** out) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !out) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    if (c->in_use.load() + bytes > c->budget) return fail(RPD_ERR_OVER_BUDGET, "allocation exceeds the HBM budget");
    RPD_CUDA(cudaSetDevice(c->device));
    cudaError_t e = cudaMalloc(out, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(RPD_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    c->in_use += bytes;
    std::lock_guard<std::mutex> lock(c->mu);
    c->user_allocs[*out] = bytes;
    return RPD_OK;
}

int rpd_device_free(rpd_ctx* ctx, void* ptr) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c) return fail(RPD_ERR_INVALID_ARGUMENT, "null context");
    if (!ptr) return RPD_OK;
    uint64_t bytes = 0;
    {
        std::lock_guard<std::mutex> lock(c->mu);
        auto it = c->user_allocs.find(ptr);
        if (it == c->user_allocs.end()) return fail(RPD_ERR_INVALID_ARGUMENT, "pointer was not allocated by rpd_device_alloc");
        bytes = it->second;
        c->user_allocs.erase(it);
    }
    RPD_CUDA(cudaSetDevice(c->device));
    RPD_CUDA(cudaFree(ptr));
    c->in_use -= bytes;
    return RPD_OK;
}

int rpd_host_alloc(uint64_t bytes, void** out) {
    if (!out) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    cudaError_t e = cudaMallocHost(out, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(RPD_ERR_OUT_OF_MEMORY, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    return RPD_OK;
}

int rpd_host_free(void* ptr) {
    if (ptr) RPD_CUDA(cudaFreeHost(ptr));
    return RPD_OK;
}

int rpd_memcpy(rpd_ctx* ctx, void* dst, const void* src, uint64_t bytes, int kind) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c) return fail(RPD_ERR_INVALID_ARGUMENT, "null context");
    RPD_CUDA(cudaSetDevice(c->device));
    const cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : kind == 1 ? cudaMemcpyDeviceToHost
                                                                             : cudaMemcpyDeviceToDevice;
    RPD_CUDA(cudaMemcpyAsync(dst, src, bytes, k, c->util_stream));
    RPD_CUDA(cudaStreamSynchronize(c->util_stream));
    return RPD_OK;
}

int rpd_synth_fill(rpd_ctx* ctx, const rpd_synth_params* prm, int64_t first, int64_t count, int32_t spp,
                   const int32_t* counts, const int32_t* start_n, const rpd_sample_soa* out, rpd_memory where) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!prm || !out) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    if (prm->regions <= 0 || prm->regions > RPD_SYNTH_MAX_REGIONS || prm->lights <= 0 || prm->lights > 15)
        return fail(RPD_ERR_INVALID_ARGUMENT, "synthetic regions must be in 1..256 and lights in 1..15");
    if (first < 0 || count < 0 || first + count > int64_t(prm->width) * prm->height)
        return fail(RPD_ERR_INVALID_ARGUMENT, "pixel span outside the synthetic image");
    std::vector<rpd_synth_region> table(size_t(prm->regions));
    for (int r = 0; r < prm->regions; ++r) rpd_synth_region_make(prm, r, &table[size_t(r)]);
    if (where == RPD_MEM_HOST) {
        int64_t k = 0;
        for (int64_t i = 0; i < count; ++i) {
            const int64_t pix = first + i;
            const int x = int(pix % prm->width), y = int(pix / prm->width);
            const rpd_synth_region& reg = table[size_t(rpd_synth_pixel_region(prm, table.data(), x, y))];
            if (out->pixel_albedo[0])
                for (int ch = 0; ch < 3; ++ch) const_cast<float*>(out->pixel_albedo[ch])[i] = reg.albedo[ch];
            const int32_t n = counts ? counts[i] : spp;
            const uint32_t n0 = start_n ? uint32_t(start_n[i]) : 0u;
            for (int32_t q = 0; q < n; ++q, ++k) {
                rpd_synth_sample sm;
                rpd_synth_sample_make(prm, &reg, x, y, n0 + uint32_t(q), &sm);
                for (int ch = 0; ch < 3; ++ch) {
                    const_cast<float*>(out->radiance[ch])[k] = sm.radiance[ch];
                    const_cast<float*>(out->normal[ch])[k] = sm.normal[ch];
                    if (out->albedo[0]) const_cast<float*>(out->albedo[ch])[k] = reg.albedo[ch];
                }
                const_cast<float*>(out->depth)[k] = sm.depth;
                for (int ch = 0; ch < 2; ++ch) {
                    const_cast<float*>(out->pixel_u[ch])[k] = sm.pixel_u[ch];
                    const_cast<float*>(out->lens_u[ch])[k] = sm.lens_u[ch];
                    const_cast<float*>(out->brdf_u[ch])[k] = sm.brdf_u[ch];
                    const_cast<float*>(out->light_u[ch])[k] = sm.light_u[ch];
                }
                const_cast<uint8_t*>(out->flags)[k] = sm.flags;
                const_cast<uint8_t*>(out->category)[k] = sm.category;
            }
        }
        return RPD_OK;
    }
    if (!c) return fail(RPD_ERR_INVALID_ARGUMENT, "a context is needed for a device fill");
    RPD_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->util_stream;
    rpd_synth_region* d_table = nullptr;
    int64_t* d_offsets = nullptr;
    int32_t* d_region = nullptr;
    const int64_t nblocks = (count + 1023) / 1024;
    RPD_CUDA(cudaMallocAsync(&d_table, table.size() * sizeof(rpd_synth_region), st));
    RPD_CUDA(cudaMallocAsync(&d_offsets, uint64_t(count + 1) * 8, st));
    RPD_CUDA(cudaMallocAsync(&d_region, uint64_t(std::max<int64_t>(count, 1)) * 4, st));
    RPD_CUDA(cudaMemcpyAsync(d_table, table.data(), table.size() * sizeof(rpd_synth_region), cudaMemcpyHostToDevice, st));
    int64_t total = 0;
    {
        // offsets through a temporary job-less scan
        Job tmp;
        tmp.ctx = c;
        tmp.stream = st;
        tmp.offsets = d_offsets;
        if (counts) {
            // launch_offsets_scan writes its block sums and maxima after offsets[count]; use a
            // dedicated buffer large enough for all of them
            int64_t* both = nullptr;
            RPD_CUDA(cudaMallocAsync(&both, uint64_t(count + 1 + 2 * nblocks + 4) * 8, st));
            tmp.offsets = both;
            RPD_CUDA(launch_offsets_scan(tmp, counts, count));
            RPD_CUDA(cudaMemcpyAsync(d_offsets, both, uint64_t(count + 1) * 8, cudaMemcpyDeviceToDevice, st));
            RPD_CUDA(cudaMemcpyAsync(&total, both + count, 8, cudaMemcpyDeviceToHost, st));
            RPD_CUDA(cudaStreamSynchronize(st));
            RPD_CUDA(cudaFreeAsync(both, st));
            tmp.offsets = d_offsets;
        } else {
            RPD_CUDA(launch_offsets_uniform(tmp, count, spp));
            total = count * int64_t(spp);
        }
    }
    RPD_CUDA(launch_synth(*prm, d_table, first, count, d_offsets, total, start_n, d_region, *out, st));
    RPD_CUDA(cudaFreeAsync(d_table, st));
    RPD_CUDA(cudaFreeAsync(d_offsets, st));
    RPD_CUDA(cudaFreeAsync(d_region, st));
    RPD_CUDA(cudaStreamSynchronize(st));
    return RPD_OK;
}

int rpd_atrous_wavelet(rpd_ctx* ctx, const float* raw, const float* normal, const float* albedo, int32_t w, int32_t h,
                       float sigma_c, float sigma_n, float sigma_a, int32_t iterations, float* out, rpd_memory where) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !raw || !normal || !albedo || !out || w <= 0 || h <= 0 || iterations < 0)
        return fail(RPD_ERR_INVALID_ARGUMENT, "bad a-trous arguments");
    RPD_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->util_stream;
    const uint64_t bytes = uint64_t(w) * h * 12;
    float *d_raw = nullptr, *d_n = nullptr, *d_a = nullptr, *b0 = nullptr, *b1 = nullptr;
    float4* records = nullptr;
    RPD_CUDA(cudaMallocAsync(&b0, bytes, st));
    RPD_CUDA(cudaMallocAsync(&b1, bytes, st));
    RPD_CUDA(cudaMallocAsync(&records, uint64_t(w) * h * 2 * sizeof(float4), st));
    if (where == RPD_MEM_HOST) {
        RPD_CUDA(cudaMallocAsync(&d_raw, bytes, st));
        RPD_CUDA(cudaMallocAsync(&d_n, bytes, st));
        RPD_CUDA(cudaMallocAsync(&d_a, bytes, st));
        RPD_CUDA(cudaMemcpyAsync(d_raw, raw, bytes, cudaMemcpyHostToDevice, st));
        RPD_CUDA(cudaMemcpyAsync(d_n, normal, bytes, cudaMemcpyHostToDevice, st));
        RPD_CUDA(cudaMemcpyAsync(d_a, albedo, bytes, cudaMemcpyHostToDevice, st));
    }
    const float* r_in = where == RPD_MEM_HOST ? d_raw : raw;
    const float* n_in = where == RPD_MEM_HOST ? d_n : normal;
    const float* a_in = where == RPD_MEM_HOST ? d_a : albedo;
    float* result = nullptr;
    uint64_t launches = 0;
    RPD_CUDA(launch_atrous(r_in, n_in, a_in, w, h, sigma_c, sigma_n, sigma_a, iterations, b0, b1, records, &result, st,
                           &launches));
    RPD_CUDA(cudaMemcpyAsync(out, result, bytes, where == RPD_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
    RPD_CUDA(cudaFreeAsync(b0, st));
    RPD_CUDA(cudaFreeAsync(b1, st));
    RPD_CUDA(cudaFreeAsync(records, st));
    if (d_raw) RPD_CUDA(cudaFreeAsync(d_raw, st));
    if (d_n) RPD_CUDA(cudaFreeAsync(d_n, st));
    if (d_a) RPD_CUDA(cudaFreeAsync(d_a, st));
    RPD_CUDA(cudaStreamSynchronize(st));
    return RPD_OK;
}

int rpd_joint_bilateral(rpd_ctx* ctx, const float* raw, const float* normal, const float* albedo, int32_t w, int32_t h,
                        float sigma_c, float sigma_n, float sigma_p, float sigma_a, float* gaussian, float* bilateral,
                        float* joint, rpd_memory where) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !raw || !normal || !albedo || !gaussian || !bilateral || !joint || w <= 0 || h <= 0)
        return fail(RPD_ERR_INVALID_ARGUMENT, "bad joint-bilateral arguments");
    RPD_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->util_stream;
    const uint64_t bytes = uint64_t(w) * h * 12;
    void* scratch = nullptr;
    RPD_CUDA(cudaMallocAsync(&scratch, joint_bilateral_scratch_bytes(w, h), st));
    float* d[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const float* in[3] = {raw, normal, albedo};
    float* outs[3] = {gaussian, bilateral, joint};
    if (where == RPD_MEM_HOST) {
        for (auto& p : d) RPD_CUDA(cudaMallocAsync(&p, bytes, st));
        for (int k = 0; k < 3; ++k) RPD_CUDA(cudaMemcpyAsync(d[k], in[k], bytes, cudaMemcpyHostToDevice, st));
        for (int k = 0; k < 3; ++k) in[k] = d[k];
    }
    float* dev_out[3] = {where == RPD_MEM_HOST ? d[3] : gaussian, where == RPD_MEM_HOST ? d[4] : bilateral,
                         where == RPD_MEM_HOST ? d[5] : joint};
    uint64_t launches = 0;
    RPD_CUDA(launch_joint_bilateral(in[0], in[1], in[2], w, h, sigma_c, sigma_n, sigma_p, sigma_a, dev_out[0], dev_out[1],
                                    dev_out[2], scratch, st, &launches));
    if (where == RPD_MEM_HOST)
        for (int k = 0; k < 3; ++k) RPD_CUDA(cudaMemcpyAsync(outs[k], dev_out[k], bytes, cudaMemcpyDeviceToHost, st));
    unsigned timeouts = 0;
    const uint64_t flag_offset = joint_bilateral_scratch_bytes(w, h) - 256;
    RPD_CUDA(cudaMemcpyAsync(&timeouts, static_cast<char*>(scratch) + flag_offset, sizeof(timeouts),
                             cudaMemcpyDeviceToHost, st));
    for (auto& p : d)
        if (p) RPD_CUDA(cudaFreeAsync(p, st));
    RPD_CUDA(cudaFreeAsync(scratch, st));
    RPD_CUDA(cudaStreamSynchronize(st));
    if (timeouts) return fail(RPD_ERR_TIMEOUT, "a joint-bilateral tile copy did not complete in time");
    return RPD_OK;
}

namespace {

// Metrics of `tst` against `ref` on `stream`: scratch from the stream-ordered pool, the result
// copied to host memory after the stream drains.
int run_metrics(const rpd::Img3& ref, const rpd::Img3& tst, int w, int h, cudaStream_t st, rpd_image_metrics* out) {
    void* scratch = nullptr;
    rpd_image_metrics* d_out = nullptr;
    RPD_CUDA(cudaMallocAsync(&scratch, metrics_scratch_bytes(w, h), st));
    RPD_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d_out), sizeof(rpd_image_metrics), st));
    RPD_CUDA(launch_metrics(ref, tst, w, h, scratch, d_out, st));
    RPD_CUDA(cudaMemcpyAsync(out, d_out, sizeof(rpd_image_metrics), cudaMemcpyDeviceToHost, st));
    RPD_CUDA(cudaFreeAsync(scratch, st));
    RPD_CUDA(cudaFreeAsync(d_out, st));
    RPD_CUDA(cudaStreamSynchronize(st));
    return RPD_OK;
}

rpd::Img3 interleaved(const float* base) { return rpd::Img3{{base, base + 1, base + 2}, 3}; }

}  // namespace

int rpd_hdr_metrics(rpd_ctx* ctx, const float* reference, const float* test, int32_t w, int32_t h, rpd_memory where,
                    rpd_image_metrics* out) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !reference || !test || !out || w <= 0 || h <= 0)
        return fail(RPD_ERR_INVALID_ARGUMENT, "bad metrics arguments");
    RPD_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->util_stream;
    const uint64_t bytes = uint64_t(w) * h * 12;
    float* d[2] = {nullptr, nullptr};
    const float* in[2] = {reference, test};
    if (where == RPD_MEM_HOST) {
        for (int k = 0; k < 2; ++k) {
            RPD_CUDA(cudaMallocAsync(&d[k], bytes, st));
            RPD_CUDA(cudaMemcpyAsync(d[k], in[k], bytes, cudaMemcpyHostToDevice, st));
            in[k] = d[k];
        }
    }
    const int r = run_metrics(interleaved(in[0]), interleaved(in[1]), w, h, st, out);
    for (float* p : d)
        if (p) cudaFreeAsync(p, st);
    if (r == RPD_OK) RPD_CUDA(cudaStreamSynchronize(st));
    return r;
}

int rpd_job_hdr_metrics(rpd_job* job, const float* reference, rpd_memory where, rpd_image_metrics* out) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (!reference || !out) return fail(RPD_ERR_INVALID_ARGUMENT, "bad metrics arguments");
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    const uint64_t bytes = uint64_t(j->g.np) * 12;
    const float* ref = reference;
    float* d_ref = nullptr;
    if (where == RPD_MEM_HOST) {
        RPD_CUDA(cudaMallocAsync(&d_ref, bytes, j->stream));
        RPD_CUDA(cudaMemcpyAsync(d_ref, reference, bytes, cudaMemcpyHostToDevice, j->stream));
        ref = d_ref;
    }
    const rpd::Img3 den{{j->p.denoised[0], j->p.denoised[1], j->p.denoised[2]}, 1};
    const int r = run_metrics(interleaved(ref), den, j->g.w, j->g.h, j->stream, out);
    if (d_ref) cudaFreeAsync(d_ref, j->stream);
    if (r == RPD_OK) RPD_CUDA(cudaStreamSynchronize(j->stream));
    return r;
}

namespace {

// Device and page-locked scratch for writing w x h images, released by the destructor.
struct WriteScratch {
    uint8_t* dev = nullptr;
    uint8_t* host = nullptr;
    float* plane = nullptr;
    int* dmax = nullptr;
    ~WriteScratch() {
        if (dev) cudaFree(dev);
        if (host) cudaFreeHost(host);
        if (plane) cudaFree(plane);
        if (dmax) cudaFree(dmax);
    }
    int init(int64_t np, bool with_plane) {
        RPD_CUDA(cudaMalloc(&dev, size_t(np) * 4));
        RPD_CUDA(cudaMallocHost(&host, size_t(np) * 4));
        if (with_plane) {
            RPD_CUDA(cudaMalloc(&plane, size_t(np) * sizeof(float)));
            RPD_CUDA(cudaMalloc(&dmax, sizeof(int)));
        }
        return RPD_OK;
    }
};

int write_rgb(rpd_ctx* ctx, const float* rgb, int32_t w, int32_t h, rpd_memory where, int tonemap, const char* path) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !rgb || !path || w <= 0 || h <= 0) return fail(RPD_ERR_INVALID_ARGUMENT, "bad image arguments");
    if (tonemap > RPD_TONEMAP_ACES) return fail(RPD_ERR_INVALID_ARGUMENT, "unknown tonemapping preset");
    RPD_CUDA(cudaSetDevice(c->device));
    const int64_t np = int64_t(w) * h;
    WriteScratch ws;
    int st = ws.init(np, false);
    if (st != RPD_OK) return st;
    float* d_rgb = nullptr;
    const float* src = rgb;
    if (where == RPD_MEM_HOST) {
        RPD_CUDA(cudaMalloc(&d_rgb, size_t(np) * 12));
        RPD_CUDA(cudaMemcpyAsync(d_rgb, rgb, size_t(np) * 12, cudaMemcpyHostToDevice, c->util_stream));
        src = d_rgb;
    }
    st = write_image(rpd::Img3{{src, src + 1, src + 2}, 3}, w, h, tonemap, path, ws.dev, ws.host, c->util_stream);
    if (d_rgb) cudaFree(d_rgb);
    return st;
}

}  // namespace

int rpd_write_hdr(rpd_ctx* ctx, const float* rgb, int32_t w, int32_t h, rpd_memory where, const char* path) {
    return write_rgb(ctx, rgb, w, h, where, -1, path);
}

int rpd_write_png(rpd_ctx* ctx, const float* rgb, int32_t w, int32_t h, rpd_memory where, int tonemap, const char* path) {
    if (tonemap < 0) return fail(RPD_ERR_INVALID_ARGUMENT, "unknown tonemapping preset");
    return write_rgb(ctx, rgb, w, h, where, tonemap, path);
}

int rpd_job_write_outputs(rpd_job* job, const char* prefix, int tonemap, int statmc) {
    Job* j = reinterpret_cast<Job*>(job);
    CHECK_JOB(j);
    if (!prefix || tonemap < 0 || tonemap > RPD_TONEMAP_ACES) return fail(RPD_ERR_INVALID_ARGUMENT, "bad output arguments");
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    const int w = j->g.w, h = j->g.h;
    const int64_t np = j->g.np;
    WriteScratch ws;
    int st = ws.init(np, true);
    if (st != RPD_OK) return st;
    const std::string base(prefix);
    auto rgb = [](float* const* p) { return rpd::Img3{{p[0], p[1], p[2]}, 1}; };
    auto grey = [](const float* p) { return rpd::Img3{{p, p, p}, 1}; };
    auto put = [&](const rpd::Img3& img, const char* suffix, int tm) {
        return write_image(img, w, h, tm, base + suffix, ws.dev, ws.host, j->stream);
    };
    // buffers.radiance after render(): the denoised image with StatMC, else the finalized radiance
    const rpd::Img3 main = statmc ? rgb(j->p.denoised) : rgb(j->p.radiance);
    if ((st = put(main, ".png", tonemap)) != RPD_OK) return st;
    if ((st = put(main, ".hdr", -1)) != RPD_OK) return st;
    if (statmc) {
        if ((st = put(rgb(j->p.radiance), "_raw.png", tonemap)) != RPD_OK) return st;
        if ((st = put(rgb(j->p.radiance), "_raw.hdr", -1)) != RPD_OK) return st;
        static const int fields[9] = {N_ALL, N_PIXEL, N_BRDF, N_LENS, N_LIGHT, N_LIGHT_UV, N_LIGHT_SELECT, N_ENV, N_RR};
        static const char* names[9] = {"_sensitivity.hdr", "_sensitivity_pixel.hdr", "_sensitivity_brdf.hdr",
                                       "_sensitivity_lens.hdr", "_sensitivity_light.hdr", "_sensitivity_light_uv.hdr",
                                       "_sensitivity_light_select.hdr", "_sensitivity_environment.hdr",
                                       "_sensitivity_rr.hdr"};
        for (int k = 0; k < 9; ++k) {
            RPD_CUDA(launch_expand(*j, j->n.field[fields[k]], ws.plane));
            if ((st = put(grey(ws.plane), names[k], -1)) != RPD_OK) return st;
        }
        const std::pair<const float*, const char*> planes[] = {
            {j->p.sens_confidence, "_sensitivity_confidence.hdr"}, {j->p.sens_gradient, "_sensitivity_gradient.hdr"},
            {j->p.uncertainty, "_uncertainty.hdr"}, {j->p.alpha, "_alpha.hdr"},
            {j->p.variance_denoised, "_vardenoised.hdr"}, {j->p.importance, "_adaptive_importance.hdr"}};
        for (const auto& pl : planes)
            if ((st = put(grey(pl.first), pl.second, -1)) != RPD_OK) return st;
        RPD_CUDA(launch_count_fraction(j->p.sample_count, np, ws.dmax, ws.plane, j->stream));
        if ((st = put(grey(ws.plane), "_sample_fraction.hdr", -1)) != RPD_OK) return st;
    }
    if ((st = put(rgb(j->p.albedo), "_albedo.hdr", -1)) != RPD_OK) return st;
    if ((st = put(rgb(j->p.normal), "_normal.hdr", -1)) != RPD_OK) return st;
    if ((st = put(grey(j->p.depth), "_depth.hdr", -1)) != RPD_OK) return st;
    if (statmc) {
        if ((st = put(grey(j->p.var_total), "_var_total.hdr", -1)) != RPD_OK) return st;
        if ((st = put(grey(j->p.var_eff), "_var_eff.hdr", -1)) != RPD_OK) return st;
        if ((st = put(grey(j->p.var_ratio), "_var_ratio.hdr", -1)) != RPD_OK) return st;
    }
    return RPD_OK;
}

}  // extern "C"

namespace rpd {

int job_reserve(Job& j, int64_t max_push_samples) {
    int st = ensure_offsets(j, j.g.np);
    if (st != RPD_OK) return st;
    if (j.cfg.rpf_shrinkage_scale > 0.0f && !j.exact_grid) {
        void* lum = j.lum;
        const int64_t ns64 = ((std::max<int64_t>(max_push_samples, 1) + 63) / 64) * 64;
        st = grow_device(j, &lum, &j.lum_cap, uint64_t(ns64) * 10 + 256, true);
        j.lum = static_cast<float*>(lum);
    }
    return st;
}

int push_device_async(Job& j, const DeviceSamples& d, int64_t first, int64_t count, int32_t spp, const int32_t* counts,
                      int64_t total_bound, bool offsets_ready) {
    int st = ensure_offsets(j, count);
    if (st != RPD_OK) return st;
    StageTimer timer(j, RPD_STAGE_ACCUMULATE);
    if (!offsets_ready) {
        if (counts) RPD_CUDA(launch_offsets_scan(j, counts, count));
        else RPD_CUDA(launch_offsets_uniform(j, count, spp));
    }
    DeviceSamples dd = d;
    return push_tail(&j, dd, first, count, spp, counts, RPD_MEM_DEVICE,
                     counts ? std::max<int64_t>(total_bound, 1) : int64_t(count) * spp);
}

}  // namespace rpd
