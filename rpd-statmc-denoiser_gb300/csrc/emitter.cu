// The tracer side of a pass: per-sample records written by the host render loop straight into
// page-locked ring buffers and streamed to the GPU band by band while tracing continues.
//
// The reference's render loops (render_image_statmc, main.cpp:649-737; render_image_adaptive,
// 1451-1538) fold each traced sample into the pixel's statistics and a thread-local RPD grid
// (accumulate_sample, accumulate_rpf_sample_to_grid, 701-717) from an OpenMP row loop. Here the
// loop writes the sample's record instead: rows are handed out in any order from any number of
// host threads; a band of `band_rows` rows lives in one ring slot (a page-locked host copy and a
// device copy of every plane); when the band's last row is done and every earlier band has gone,
// its planes are copied to HBM on the emitter's copy stream and the job stream runs the band's
// statistics and grid passes on them, while the tracer fills the next slots. Bands are pushed in
// band order, so the pass accumulates exactly as one push of the whole image. A thread asking for
// a row whose band has no free slot waits (bounded) until the slot's earlier band has been copied.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <mutex>
#include <string>
#include <vector>

#include "rpd_internal.h"

namespace rpd {
namespace {

// Sample planes of a slot, in one allocation: 20 float planes then flags and category.
enum EmPlane {
    E_RAD = 0, E_NRM = 3, E_DEPTH = 6, E_ALB = 7, E_PIX = 10, E_LENS = 12, E_BRDF = 14, E_LIGHT = 16, E_ENV = 18,
    E_FLOATS = 20
};
constexpr int64_t kSlotWaitMs = 600000;  // a tracer thread gives up after 10 minutes without a free slot

struct Slot {
    char* host = nullptr;  // page-locked
    char* dev = nullptr;
    int32_t* dev_counts = nullptr;  // the band's per-pixel counts (passes with counts)
    int band = -1;                  // band held, -1: free
    int rows_done = 0;
    cudaEvent_t copied = nullptr;    // the band's planes have reached HBM: the host copy is free
    cudaEvent_t consumed = nullptr;  // the job stream's passes have read the device copy
    bool in_flight = false;          // copied/consumed recorded and not yet waited on
};

}  // namespace

struct Emitter {
    Job* job = nullptr;
    int band_rows = 0, nslots = 0;
    int64_t cap = 0;  // samples per slot
    std::vector<Slot> slots;
    cudaStream_t copy = nullptr;
    std::mutex mu;
    std::condition_variable cv;
    // the open pass
    bool open = false;
    int32_t spp = 0;
    std::vector<int32_t> counts;     // per pixel, empty for a uniform pass
    std::vector<int64_t> off;        // per pixel, sample offsets within the pass (np + 1)
    int nbands = 0, next_push = 0;
    std::vector<int> band_of_slot_rows;  // rows done per band
    int error = RPD_OK;
    std::string error_msg;

    int64_t band_first(int b) const { return int64_t(b) * band_rows * job->g.w; }
    int64_t band_last(int b) const { return std::min<int64_t>(job->g.np, int64_t(b + 1) * band_rows * job->g.w); }
    int band_row_count(int b) const { return std::min(job->g.h, (b + 1) * band_rows) - b * band_rows; }
    int64_t band_samples(int b) const { return off[size_t(band_last(b))] - off[size_t(band_first(b))]; }

    size_t plane_offset(int k) const {  // byte offset of plane k in a slot
        return k < E_FLOATS ? size_t(k) * size_t(cap) * 4 : size_t(E_FLOATS) * size_t(cap) * 4 + size_t(k - E_FLOATS) * size_t(cap);
    }
    size_t slot_bytes() const { return plane_offset(E_FLOATS + 2); }

    void planes(char* base, int64_t first_sample, rpd_sample_soa* s) const {
        auto f = [&](int k) { return reinterpret_cast<float*>(base + plane_offset(k)) + first_sample; };
        for (int c = 0; c < 3; ++c) {
            s->radiance[c] = f(E_RAD + c);
            s->normal[c] = f(E_NRM + c);
            s->albedo[c] = f(E_ALB + c);
            s->pixel_albedo[c] = nullptr;
        }
        s->depth = f(E_DEPTH);
        for (int c = 0; c < 2; ++c) {
            s->pixel_u[c] = f(E_PIX + c);
            s->lens_u[c] = f(E_LENS + c);
            s->brdf_u[c] = f(E_BRDF + c);
            s->light_u[c] = f(E_LIGHT + c);
            s->env_u[c] = f(E_ENV + c);
        }
        s->flags = reinterpret_cast<uint8_t*>(base + plane_offset(E_FLOATS)) + first_sample;
        s->category = reinterpret_cast<uint8_t*>(base + plane_offset(E_FLOATS + 1)) + first_sample;
    }

    // Copy band b (complete) to HBM and enqueue its passes. Called in band order, under mu.
    int push_band(int b) {
        Slot& sl = slots[size_t(b % nslots)];
        const int64_t n = band_samples(b), p0 = band_first(b), np = band_last(b) - p0;
        // the device copy of this slot is free once the job stream consumed its earlier band
        RPD_CUDA(cudaStreamWaitEvent(copy, sl.consumed, 0));
        for (int k = 0; k < E_FLOATS + 2; ++k) {
            const size_t elem = k < E_FLOATS ? 4 : 1;
            if (n > 0)
                RPD_CUDA(cudaMemcpyAsync(sl.dev + plane_offset(k), sl.host + plane_offset(k), size_t(n) * elem,
                                         cudaMemcpyHostToDevice, copy));
        }
        if (!counts.empty())
            RPD_CUDA(cudaMemcpyAsync(sl.dev_counts, counts.data() + p0, size_t(np) * 4, cudaMemcpyHostToDevice, copy));
        RPD_CUDA(cudaEventRecord(sl.copied, copy));
        RPD_CUDA(cudaStreamWaitEvent(job->stream, sl.copied, 0));
        rpd_sample_soa s{};
        planes(sl.dev, 0, &s);
        DeviceSamples d{};
        for (int c = 0; c < 3; ++c) {
            d.radiance[c] = s.radiance[c];
            d.normal[c] = s.normal[c];
            d.albedo[c] = s.albedo[c];
        }
        d.depth = s.depth;
        for (int c = 0; c < 2; ++c) {
            d.pixel_u[c] = s.pixel_u[c];
            d.lens_u[c] = s.lens_u[c];
            d.brdf_u[c] = s.brdf_u[c];
            d.light_u[c] = s.light_u[c];
            d.env_u[c] = s.env_u[c];
        }
        d.flags = s.flags;
        d.category = s.category;
        const int st = push_device_async(*job, d, p0, np, counts.empty() ? spp : 0,
                                         counts.empty() ? nullptr : sl.dev_counts, n);
        if (st != RPD_OK) return st;
        RPD_CUDA(cudaEventRecord(sl.consumed, job->stream));
        sl.in_flight = true;
        return RPD_OK;
    }

    int fail_pass(int st) {
        if (error == RPD_OK) {
            error = st;
            error_msg = rpd_last_error();
        }
        cv.notify_all();
        return st;
    }
};

}  // namespace rpd

using rpd::Emitter;

extern "C" {

int rpd_emitter_create(rpd_job* job, int32_t band_rows, int32_t ring_slots, int32_t max_spp, rpd_emitter** out) {
    using namespace rpd;
    Job* j = reinterpret_cast<Job*>(job);
    if (!j || !out || band_rows <= 0 || ring_slots < 2 || max_spp <= 0)
        return fail(RPD_ERR_INVALID_ARGUMENT, "bad emitter arguments (band_rows > 0, ring_slots >= 2, max_spp > 0)");
    RPD_CUDA(cudaSetDevice(j->ctx->device));
    auto* em = new (std::nothrow) Emitter();
    if (!em) return fail(RPD_ERR_OUT_OF_MEMORY, "emitter");
    em->job = j;
    em->band_rows = std::min(band_rows, j->g.h);
    em->nslots = ring_slots;
    em->cap = int64_t(em->band_rows) * j->g.w * max_spp;
    em->slots.resize(size_t(ring_slots));
    cudaError_t e = cudaStreamCreateWithFlags(&em->copy, cudaStreamNonBlocking);
    for (auto& sl : em->slots) {
        if (e == cudaSuccess) e = cudaMallocHost(&sl.host, em->slot_bytes());
        if (e == cudaSuccess) e = cudaMalloc(&sl.dev, em->slot_bytes());
        if (e == cudaSuccess) e = cudaMalloc(&sl.dev_counts, size_t(em->band_rows) * j->g.w * 4);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.copied, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.consumed, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        rpd_emitter_destroy(reinterpret_cast<rpd_emitter*>(em));
        return cuda_fail(e, "emitter ring");
    }
    *out = reinterpret_cast<rpd_emitter*>(em);
    return RPD_OK;
}

void rpd_emitter_destroy(rpd_emitter* emitter) {
    auto* em = reinterpret_cast<Emitter*>(emitter);
    if (!em) return;
    cudaSetDevice(em->job->ctx->device);
    if (em->copy) cudaStreamSynchronize(em->copy);
    cudaStreamSynchronize(em->job->stream);
    for (auto& sl : em->slots) {
        if (sl.host) cudaFreeHost(sl.host);
        if (sl.dev) cudaFree(sl.dev);
        if (sl.dev_counts) cudaFree(sl.dev_counts);
        if (sl.copied) cudaEventDestroy(sl.copied);
        if (sl.consumed) cudaEventDestroy(sl.consumed);
    }
    if (em->copy) cudaStreamDestroy(em->copy);
    delete em;
}

int rpd_emitter_begin_pass(rpd_emitter* emitter, int32_t spp, const int32_t* counts) {
    using namespace rpd;
    auto* em = reinterpret_cast<Emitter*>(emitter);
    if (!em) return fail(RPD_ERR_INVALID_ARGUMENT, "null emitter");
    std::lock_guard<std::mutex> lock(em->mu);
    if (em->open) return fail(RPD_ERR_STATE, "the emitter's pass is still open");
    if (!counts && spp < 0) return fail(RPD_ERR_INVALID_ARGUMENT, "negative spp");
    Job& j = *em->job;
    RPD_CUDA(cudaSetDevice(j.ctx->device));
    const int64_t np = j.g.np;
    em->spp = counts ? 0 : spp;
    em->counts.assign(counts ? counts : nullptr, counts ? counts + np : nullptr);
    em->off.resize(size_t(np) + 1);
    em->off[0] = 0;
    for (int64_t p = 0; p < np; ++p) {
        const int32_t c = counts ? counts[p] : spp;
        if (c < 0) return fail(RPD_ERR_INVALID_ARGUMENT, "negative per-pixel sample count");
        em->off[size_t(p) + 1] = em->off[size_t(p)] + c;
    }
    em->nbands = (j.g.h + em->band_rows - 1) / em->band_rows;
    int64_t most = 0;
    for (int b = 0; b < em->nbands; ++b) most = std::max(most, em->band_samples(b));
    if (most > em->cap)
        return fail(RPD_ERR_INVALID_ARGUMENT, "a band of this pass holds " + std::to_string(most) +
                                                  " samples, more than the emitter's " + std::to_string(em->cap) +
                                                  " per slot (band_rows x width x max_spp)");
    const int st = job_reserve(j, most);
    if (st != RPD_OK) return st;
    em->band_of_slot_rows.assign(size_t(em->nbands), 0);
    em->next_push = 0;
    em->error = RPD_OK;
    for (auto& sl : em->slots) {
        sl.band = -1;
        sl.rows_done = 0;
    }
    em->open = true;
    return RPD_OK;
}

int rpd_emitter_row(rpd_emitter* emitter, int32_t y, rpd_sample_soa* planes, const int64_t** pixel_offsets) {
    using namespace rpd;
    auto* em = reinterpret_cast<Emitter*>(emitter);
    if (!em || !planes || !pixel_offsets) return fail(RPD_ERR_INVALID_ARGUMENT, "bad emitter row arguments");
    std::unique_lock<std::mutex> lock(em->mu);
    if (!em->open) return fail(RPD_ERR_STATE, "no open emitter pass");
    if (y < 0 || y >= em->job->g.h) return fail(RPD_ERR_INVALID_ARGUMENT, "row outside the image");
    const int b = y / em->band_rows;
    Slot& sl = em->slots[size_t(b % em->nslots)];
    // wait until the slot holds this band, or is free of an earlier band whose planes have gone
    const auto limit = std::chrono::steady_clock::now() + std::chrono::milliseconds(kSlotWaitMs);
    while (sl.band != b) {
        if (em->error != RPD_OK) return fail(em->error, em->error_msg);
        if (sl.band < 0 || (sl.band < b && !sl.in_flight && sl.band < em->next_push)) {
            sl.band = b;
            sl.rows_done = 0;
            break;
        }
        if (sl.band < b && sl.in_flight) {
            // the earlier band was pushed: its host copy is free once the copy completed
            lock.unlock();
            const cudaError_t e = cudaEventSynchronize(sl.copied);
            lock.lock();
            if (e != cudaSuccess) return em->fail_pass(cuda_fail(e, "emitter slot copy"));
            if (sl.in_flight && sl.band < b && sl.band < em->next_push) sl.in_flight = false;
            continue;
        }
        if (em->cv.wait_until(lock, limit) == std::cv_status::timeout)
            return fail(RPD_ERR_TIMEOUT, "no emitter slot became free for row " + std::to_string(y));
    }
    const int64_t p = int64_t(y) * em->job->g.w;
    em->planes(sl.host, em->off[size_t(p)] - em->off[size_t(em->band_first(b))], planes);
    *pixel_offsets = em->off.data() + p;
    return RPD_OK;
}

int rpd_emitter_row_done(rpd_emitter* emitter, int32_t y) {
    using namespace rpd;
    auto* em = reinterpret_cast<Emitter*>(emitter);
    if (!em) return fail(RPD_ERR_INVALID_ARGUMENT, "null emitter");
    std::lock_guard<std::mutex> lock(em->mu);
    if (!em->open) return fail(RPD_ERR_STATE, "no open emitter pass");
    if (y < 0 || y >= em->job->g.h) return fail(RPD_ERR_INVALID_ARGUMENT, "row outside the image");
    const int b = y / em->band_rows;
    if (em->slots[size_t(b % em->nslots)].band != b) return fail(RPD_ERR_STATE, "row done before it was taken");
    if (++em->band_of_slot_rows[size_t(b)] > em->band_row_count(b)) return fail(RPD_ERR_STATE, "row done twice");
    // push every complete band in order
    while (em->next_push < em->nbands &&
           em->band_of_slot_rows[size_t(em->next_push)] == em->band_row_count(em->next_push)) {
        RPD_CUDA(cudaSetDevice(em->job->ctx->device));
        const int st = em->push_band(em->next_push);
        if (st != RPD_OK) return em->fail_pass(st);
        ++em->next_push;
    }
    em->cv.notify_all();
    return RPD_OK;
}

int rpd_emitter_end_pass(rpd_emitter* emitter) {
    using namespace rpd;
    auto* em = reinterpret_cast<Emitter*>(emitter);
    if (!em) return fail(RPD_ERR_INVALID_ARGUMENT, "null emitter");
    {
        std::lock_guard<std::mutex> lock(em->mu);
        if (!em->open) return fail(RPD_ERR_STATE, "no open emitter pass");
        em->open = false;
        if (em->error != RPD_OK) return fail(em->error, em->error_msg);
        if (em->next_push != em->nbands)
            return fail(RPD_ERR_STATE, "the pass ended with " + std::to_string(em->nbands - em->next_push) +
                                           " band(s) of rows not done");
    }
    RPD_CUDA(cudaSetDevice(em->job->ctx->device));
    RPD_CUDA(cudaStreamSynchronize(em->copy));  // every band's host planes have been copied
    for (auto& sl : em->slots) sl.in_flight = false;
    return rpd_job_end_pass(reinterpret_cast<rpd_job*>(em->job));
}

}  // extern "C"
