// The batched form: an autotuner for the launch shapes of a frame class, and batches of frames
// (one job each) captured into one CUDA graph and replayed with a single launch. No
// counterpart in the reference, which denoises one frame per process run.
#include <algorithm>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "rpd_internal.h"

using namespace rpd;

namespace {

struct Frame {
    Job* job;
    rpd_sample_soa s32;
    rpd_sample_soa16 s16;
    bool compact;
    int32_t spp;
};

int run_frame(const Frame& f) {
    rpd_job* h = reinterpret_cast<rpd_job*>(f.job);
    const int64_t np = f.job->g.np;
    int st = rpd_job_begin_frame(h);
    if (st == RPD_OK)
        st = f.compact ? rpd_job_push_samples16(h, &f.s16, 0, np, f.spp, nullptr, RPD_MEM_DEVICE)
                       : rpd_job_push_samples(h, &f.s32, 0, np, f.spp, nullptr, RPD_MEM_DEVICE);
    if (st == RPD_OK) st = rpd_job_end_pass(h);
    if (st == RPD_OK) st = rpd_recompute_sensitivity(h);
    if (st == RPD_OK) st = rpd_statmc_denoise(h);
    if (st == RPD_OK) st = rpd_variance_denoise(h);
    return st;
}

// the frame class the tuned shapes are cached for
using TuneKey = std::tuple<int, int, int, int, int, int, bool>;
std::mutex g_tune_mu;
std::map<TuneKey, std::pair<int, int>> g_tuned;  // -> (grid shape, StatMC rows)

TuneKey tune_key(const Job& j, int32_t spp, bool compact) {
    return TuneKey(j.g.w, j.g.h, spp, j.cfg.rpf_tile_size, j.cfg.color_window_radius, j.cfg.var_window_radius,
                   compact);
}

// milliseconds of one kernel family over `reps` runs of `fn`, after one untimed run
template <typename Fn>
int time_kernel(Job* j, rpd_kernel k, int reps, Fn fn, double* ms) {
    rpd_job* h = reinterpret_cast<rpd_job*>(j);
    int st = fn();
    if (st != RPD_OK) return st;
    rpd_job_reset_kernel_times(h);
    rpd_job_set_profiling(h, 1);
    for (int r = 0; r < reps && st == RPD_OK; ++r) st = fn();
    rpd_job_set_profiling(h, 0);
    if (st != RPD_OK) return st;
    uint64_t n = 0;
    st = rpd_job_kernel_time(h, k, ms, &n);
    rpd_job_reset_kernel_times(h);
    return st;
}

}  // namespace

struct rpd_batch_s {
    Ctx* ctx = nullptr;
    std::vector<Frame> frames;
    cudaStream_t origin = nullptr;
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    std::vector<cudaEvent_t> joins;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0;
    bool timed = false;
    int lanes = 4;  // frames run in this many concurrent chains
};

extern "C" {

int rpd_job_autotune(rpd_job* job, const rpd_sample_soa* s32, const rpd_sample_soa16* s16, int32_t spp) {
    Job* j = reinterpret_cast<Job*>(job);
    if (!j || (!s32 == !s16) || spp <= 0)
        return fail(RPD_ERR_INVALID_ARGUMENT, "autotune needs a job, exactly one of s32/s16 and spp > 0");
    Frame f{j, s32 ? *s32 : rpd_sample_soa{}, s16 ? *s16 : rpd_sample_soa16{}, s16 != nullptr, spp};
    const TuneKey key = tune_key(*j, spp, f.compact);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            j->grid_shape = it->second.first;
            j->statmc_by = it->second.second;
            return run_frame(f);
        }
    }
    const int64_t np = j->g.np;
    auto accumulate = [&]() {
        int st = rpd_job_begin_frame(job);
        if (st == RPD_OK)
            st = f.compact ? rpd_job_push_samples16(job, &f.s16, 0, np, spp, nullptr, RPD_MEM_DEVICE)
                           : rpd_job_push_samples(job, &f.s32, 0, np, spp, nullptr, RPD_MEM_DEVICE);
        if (st == RPD_OK) st = rpd_job_end_pass(job);
        return st;
    };
    int best_shape = j->grid_shape;
    double best = 1e30;
    for (int shape : {6, 4, 5, 1}) {
        j->grid_shape = shape;
        double ms = 0.0;
        const int st = time_kernel(j, RPD_KERNEL_GRID_RANDOM, 2, accumulate, &ms);
        if (st != RPD_OK) return st;
        if (ms < best) {
            best = ms;
            best_shape = shape;
        }
    }
    j->grid_shape = best_shape;
    int st = accumulate();
    if (st == RPD_OK) st = rpd_recompute_sensitivity(job);
    if (st != RPD_OK) return st;
    int best_by = 0;
    best = 1e30;
    for (int by : {8, 4, 2}) {
        j->statmc_by = by;
        double ms = 0.0;
        st = time_kernel(j, RPD_KERNEL_STATMC_WINDOW, 2, [&]() { return rpd_statmc_denoise(job); }, &ms);
        if (st != RPD_OK) return st;
        if (ms < best) {
            best = ms;
            best_by = by;
        }
    }
    j->statmc_by = best_by;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tuned[key] = {j->grid_shape, j->statmc_by};
    }
    return run_frame(f);
}

int rpd_batch_create(rpd_ctx* ctx, rpd_batch** out) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !out) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    rpd_batch_s* b = new (std::nothrow) rpd_batch_s();
    if (!b) return fail(RPD_ERR_OUT_OF_MEMORY, "batch allocation failed");
    b->ctx = c;
    RPD_CUDA(cudaSetDevice(c->device));
    cudaError_t e = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&b->t0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->t1);
    if (e != cudaSuccess) {
        rpd_batch_destroy(b);
        return cuda_fail(e, "batch set-up");
    }
    *out = b;
    return RPD_OK;
}

int rpd_batch_add(rpd_batch* b, rpd_job* job, const rpd_sample_soa* s32, const rpd_sample_soa16* s16, int32_t spp) {
    Job* j = reinterpret_cast<Job*>(job);
    if (!b || !j || (!s32 == !s16) || spp <= 0)
        return fail(RPD_ERR_INVALID_ARGUMENT, "a frame needs a job, exactly one of s32/s16 and spp > 0");
    if (b->exec) return fail(RPD_ERR_STATE, "the batch was already captured");
    if (j->ctx != b->ctx) return fail(RPD_ERR_INVALID_ARGUMENT, "the job belongs to another context");
    for (const Frame& f : b->frames)
        if (f.job == j) return fail(RPD_ERR_INVALID_ARGUMENT, "a job appears once in a batch");
    b->frames.push_back(Frame{j, s32 ? *s32 : rpd_sample_soa{}, s16 ? *s16 : rpd_sample_soa16{}, s16 != nullptr, spp});
    cudaEvent_t e = nullptr;
    RPD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b->joins.push_back(e);
    return RPD_OK;
}

int rpd_batch_run(rpd_batch* b) {
    if (!b) return fail(RPD_ERR_INVALID_ARGUMENT, "null batch");
    if (b->frames.empty()) return fail(RPD_ERR_STATE, "empty batch");
    RPD_CUDA(cudaSetDevice(b->ctx->device));
    if (!b->exec) {
        // one direct run sizes every buffer, so that the capture allocates nothing
        for (const Frame& f : b->frames) {
            const int st = run_frame(f);
            if (st != RPD_OK) return st;
        }
        for (const Frame& f : b->frames) RPD_CUDA(cudaStreamSynchronize(f.job->stream));
        uint64_t before = 0;
        for (const Frame& f : b->frames) before += f.job->launches;
        // chains: frames in decreasing sample count, each to the least-loaded chain; a chain
        // runs its frames one after another, the chains run concurrently
        const int lanes = std::max(1, std::min<int>(b->lanes, int(b->frames.size())));
        std::vector<size_t> order(b->frames.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        auto work = [&](size_t i) { return double(b->frames[i].job->g.np) * double(b->frames[i].spp); };
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t c) { return work(a) > work(c); });
        std::vector<double> load(size_t(lanes), 0.0);
        std::vector<int> last(size_t(lanes), -1);
        RPD_CUDA(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed));
        cudaEventRecord(b->fork, b->origin);
        int st = RPD_OK;
        for (size_t oi = 0; oi < order.size() && st == RPD_OK; ++oi) {
            const size_t i = order[oi];
            const size_t lane = size_t(std::min_element(load.begin(), load.end()) - load.begin());
            load[lane] += work(i);
            const Frame& f = b->frames[i];
            cudaStreamWaitEvent(f.job->stream, last[lane] < 0 ? b->fork : b->joins[size_t(last[lane])], 0);
            st = run_frame(f);
            cudaEventRecord(b->joins[i], f.job->stream);
            last[lane] = int(i);
        }
        for (int l = 0; l < lanes; ++l)
            if (last[size_t(l)] >= 0) cudaStreamWaitEvent(b->origin, b->joins[size_t(last[size_t(l)])], 0);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(b->origin, &g);
        if (st != RPD_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_fail(e, "batch capture");
        b->graph = g;
        RPD_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
        uint64_t after = 0;
        for (const Frame& f : b->frames) after += f.job->launches;
        b->kernels = after - before;
    }
    RPD_CUDA(cudaEventRecord(b->t0, b->origin));
    RPD_CUDA(cudaGraphLaunch(b->exec, b->origin));
    RPD_CUDA(cudaEventRecord(b->t1, b->origin));
    b->timed = true;
    return RPD_OK;
}

int rpd_batch_sync(rpd_batch* b) {
    if (!b) return fail(RPD_ERR_INVALID_ARGUMENT, "null batch");
    RPD_CUDA(cudaStreamSynchronize(b->origin));
    return RPD_OK;
}

int rpd_batch_last_ms(rpd_batch* b, float* ms) {
    if (!b || !ms) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    if (!b->timed) return fail(RPD_ERR_STATE, "the batch has not run");
    RPD_CUDA(cudaEventSynchronize(b->t1));
    RPD_CUDA(cudaEventElapsedTime(ms, b->t0, b->t1));
    return RPD_OK;
}

uint64_t rpd_batch_kernel_count(rpd_batch* b) { return b ? b->kernels : 0; }

int rpd_batch_set_lanes(rpd_batch* b, int lanes) {
    if (!b || lanes < 1) return fail(RPD_ERR_INVALID_ARGUMENT, "lanes must be at least 1");
    if (b->exec) return fail(RPD_ERR_STATE, "the batch was already captured");
    b->lanes = lanes;
    return RPD_OK;
}

void rpd_batch_destroy(rpd_batch* b) {
    if (!b) return;
    if (b->ctx) cudaSetDevice(b->ctx->device);
    if (b->origin) cudaStreamSynchronize(b->origin);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto e : b->joins) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    if (b->origin) cudaStreamDestroy(b->origin);
    delete b;
}

}  // extern "C"
