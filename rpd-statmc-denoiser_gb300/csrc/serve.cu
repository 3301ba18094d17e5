// The serving form: a request loop over one GPU. Denoise requests of any size and sample
// count arrive at any time; a scheduler thread admits them as slots and HBM budget free up,
// enqueues each admitted request's whole pipeline on its own stream and retires it when its
// result has reached host memory. Requests therefore overlap on the device (continuous
// batching), and a request's state — the per-pixel statistics, the frame grid, the feature and
// sensitivity caches, its sample buffer — stays resident across its adaptive passes.
//
// Per request the pipeline is the reference's render() (path_tracer/main.cpp:1543-1564) with
// the tracer replaced by the seeded per-sample generator (include/rpd_synth.h) evaluated on the
// device:
//   first pass        spp samples per pixel, pushed, merged (render_image_statmc,
//                     main.cpp:649-737)
//   adaptive passes   variance_denoise, compute_adaptive_sample_counts, the extra samples
//                     generated from the counts on the device, pushed, merged (main.cpp:1547-1552,
//                     1451-1538)
//   final             recompute_sensitivity, statmc_denoise, variance_denoise, finalize
//                     (main.cpp:1554-1559)
// and the denoised image is copied to host memory. The adaptive passes' statmc_denoise and
// recompute_sensitivity calls and the final variance_denoise are dead work for the denoised
// image (see enqueue_request) and are not run. Nothing in
// the pipeline waits on the host: the counts, their offsets and the extra samples stay in HBM,
// a push with device counts sizes its scratch from the bound adaptive_spp * W * H, and every
// buffer comes from a stream-ordered pool.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <thread>
#include <vector>

#include "rpd_internal.h"
#include "device_math.cuh"
#include "compact.cuh"
#include "rpd_synth.h"

namespace rpd {

struct Server;

namespace {

// ---- device side: the generator writing the planes a push reads -----------------------------
struct SynthOut {
    int compact;
    // FP32 planes (rpd_sample_soa)
    float* radiance[3];
    float* normal[3];
    float* depth;
    float* pixel_u[2];
    float* lens_u[2];
    float* brdf_u[2];
    float* light_u[2];
    float* pixel_albedo[3];
    // compact planes (rpd_sample_soa16)
    uint16_t* sqrt_radiance[3];
    int16_t* normal16[3];
    uint16_t* depth16;
    uint16_t* pixel_u16[2];
    uint16_t* lens_u16[2];
    uint16_t* brdf_u16[2];
    uint16_t* light_u16[2];
    uint16_t* pixel_albedo16[3];
    uint8_t* flags;
    uint8_t* category;
};

__global__ void k_srv_regions(rpd_synth_params prm, rpd_synth_region* table) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < prm.regions) rpd_synth_region_make(&prm, r, &table[r]);
}

__global__ void k_srv_region_map(rpd_synth_params prm, const rpd_synth_region* table, int64_t np, uint8_t* region,
                                 SynthOut o) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int x = int(i % prm.width), y = int(i / prm.width);
    const int r = rpd_synth_pixel_region(&prm, table, x, y);
    region[i] = uint8_t(r);
    for (int c = 0; c < 3; ++c) {
        if (o.compact) o.pixel_albedo16[c][i] = f2h(table[r].albedo[c]);
        else o.pixel_albedo[c][i] = table[r].albedo[c];
    }
}

__device__ __forceinline__ void srv_write(const SynthOut& o, int64_t k, const rpd_synth_sample& s) {
    if (o.compact) {
        for (int c = 0; c < 3; ++c) {
            o.sqrt_radiance[c][k] = enc_sqrt_radiance(s.radiance[c]);
            o.normal16[c][k] = enc_snorm16(s.normal[c]);
        }
        o.depth16[k] = f2h(s.depth);  // depth_scale 1: the generator's depths lie in [1, 10]
        for (int c = 0; c < 2; ++c) {
            o.pixel_u16[c][k] = enc_unorm16(s.pixel_u[c]);
            o.lens_u16[c][k] = enc_unorm16(s.lens_u[c]);
            o.brdf_u16[c][k] = enc_unorm16(s.brdf_u[c]);
            o.light_u16[c][k] = enc_unorm16(s.light_u[c]);
        }
    } else {
        for (int c = 0; c < 3; ++c) {
            o.radiance[c][k] = s.radiance[c];
            o.normal[c][k] = s.normal[c];
        }
        o.depth[k] = s.depth;
        for (int c = 0; c < 2; ++c) {
            o.pixel_u[c][k] = s.pixel_u[c];
            o.lens_u[c][k] = s.lens_u[c];
            o.brdf_u[c][k] = s.brdf_u[c];
            o.light_u[c][k] = s.light_u[c];
        }
    }
    o.flags[k] = s.flags;
    o.category[k] = s.category;
}

// spp samples for every pixel, sample q of pixel i at index i * spp + q, ordinals start + q.
// One block row per image row (blockIdx.y): the row-local sample index splits into the column
// and q with a shift when spp is a power of two (spp_shift >= 0), else a 32-bit division.
__global__ void k_srv_synth_uniform(rpd_synth_params prm, const rpd_synth_region* table, const uint8_t* region,
                                    int32_t spp, int spp_shift, int y0, uint32_t start, SynthOut o) {
    const uint32_t rk = blockIdx.x * blockDim.x + threadIdx.x;  // sample within the row
    const uint32_t row_samples = uint32_t(prm.width) * uint32_t(spp);
    if (rk >= row_samples) return;
    const int y = y0 + int(blockIdx.y);
    const uint32_t x = spp_shift >= 0 ? rk >> spp_shift : rk / uint32_t(spp);
    const uint32_t q = rk - x * uint32_t(spp);
    const int64_t i = int64_t(y) * prm.width + x;
    rpd_synth_sample s;
    rpd_synth_sample_make(&prm, &table[region[i]], int(x), y, start + q, &s);
    srv_write(o, int64_t(y) * row_samples + rk, s);
}

// counts[i] samples for pixel i at offsets[i] + q, ordinals start + q. One block of 256
// threads per 256 pixels: each thread marks its pixel's samples among the block's first
// kSynthOwners in shared memory, and a sample past those finds its pixel by a search of the
// block's offsets.
constexpr int kSynthPix = 256;
constexpr int kSynthOwners = 4096;
__global__ void __launch_bounds__(kSynthPix) k_srv_synth_counts(rpd_synth_params prm, const rpd_synth_region* table,
                                                                const uint8_t* region, const int64_t* offsets, int64_t np,
                                                                int64_t capacity, uint32_t start, SynthOut o) {
    __shared__ int64_t off[kSynthPix + 1];
    __shared__ int xy[kSynthPix][2];
    __shared__ uint8_t owner[kSynthOwners];
    const int64_t p0 = int64_t(blockIdx.x) * kSynthPix;
    const int np_block = int(min((long long)kSynthPix, (long long)(np - p0)));
    for (int t = threadIdx.x; t <= np_block; t += blockDim.x) {
        off[t] = offsets[p0 + t];
        if (t < np_block) {
            const int64_t i = p0 + t;
            xy[t][0] = int(i % prm.width);
            xy[t][1] = int(i / prm.width);
        }
    }
    __syncthreads();
    // the counts of a pass never exceed adaptive_spp * W * H (the capacity); the bound only keeps
    // the writes inside the buffer
    const int64_t k0 = off[0], k1 = min((long long)off[np_block], (long long)capacity);
    const int64_t marked = min((long long)(k1 - k0), (long long)kSynthOwners);  // samples k0 .. k0 + marked - 1
    if (threadIdx.x < np_block) {
        const int64_t a = off[threadIdx.x] - k0, b = min((long long)(off[threadIdx.x + 1] - k0), (long long)marked);
        for (int64_t u = a; u < b; ++u) owner[u] = uint8_t(threadIdx.x);
    }
    __syncthreads();
    for (int64_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        int lo = 0, hi = np_block - 1;  // last pixel whose offset <= k
        if (k - k0 < marked) {
            lo = owner[k - k0];
        } else {
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (off[mid] <= k) lo = mid; else hi = mid - 1;
            }
        }
        const int64_t i = p0 + lo;
        rpd_synth_sample s;
        rpd_synth_sample_make(&prm, &table[region[i]], xy[lo][0], xy[lo][1], start + uint32_t(k - off[lo]), &s);
        srv_write(o, k, s);
    }
}

__global__ void k_srv_pack(const float* r, const float* g, const float* b, float* out, int64_t np) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    out[3 * i] = r[i];
    out[3 * i + 1] = g[i];
    out[3 * i + 2] = b[i];
}

// ---- host side ------------------------------------------------------------------------------
constexpr int64_t kSpanSamples = int64_t(32) << 20;  // largest push of a first pass (scratch bound)
constexpr uint32_t kPassOrdinalStride = 1u << 16;    // ordinals of adaptive pass p start at p << 16

uint64_t round256(uint64_t b) { return (b + 255) & ~uint64_t(255); }

// The layout of one request's buffer.
struct ReqLayout {
    uint64_t table = 0, region = 0, albedo = 0, planes = 0, out = 0, bytes = 0;
    uint64_t plane_stride = 0;  // bytes per per-sample plane
    int64_t max_samples = 0;
};

ReqLayout request_layout(int64_t np, int32_t spp, int32_t adaptive_spp, int passes, bool compact) {
    ReqLayout L;
    L.max_samples = std::max<int64_t>(int64_t(spp) * np, passes > 0 ? int64_t(adaptive_spp) * np : 0);
    const uint64_t e = compact ? 2 : 4;
    uint64_t at = 0;
    L.table = at;
    at = round256(at + sizeof(rpd_synth_region) * RPD_SYNTH_MAX_REGIONS);
    L.region = at;
    at = round256(at + uint64_t(np));
    L.albedo = at;
    at = round256(at + 3 * round256(uint64_t(np) * e));
    L.plane_stride = round256(uint64_t(std::max<int64_t>(L.max_samples, 1)) * e);
    L.planes = at;
    // radiance 3, normal 3, depth, four 2-component dims; flags and category take one byte each
    at += 15 * L.plane_stride + 2 * round256(uint64_t(std::max<int64_t>(L.max_samples, 1)));
    L.out = at;
    at = round256(at + uint64_t(np) * 12);
    L.bytes = at;
    return L;
}

struct Request {
    uint64_t id = 0;
    rpd_request req{};
    double t_submit = 0, t_admit = 0, t_done = 0;
    int status = RPD_OK;
    ReqLayout layout;
    uint64_t reserve = 0;      // bytes admission counted for the request's buffer
    Job* job = nullptr;
    void* mem = nullptr;
    int slot = -1;
    std::atomic<bool> gpu_done{false};
    Server* server = nullptr;
};

struct Slot {
    bool busy = false;
    int64_t* totals = nullptr;  // pinned: the sample total of each adaptive pass
    float* staging = nullptr;   // pinned result buffer for requests without an output pointer
    uint64_t staging_bytes = 0;
};

struct CachedJob {
    Job* job;
    uint64_t bytes;   // arena + offsets + scratch counted against the budget
};

}  // namespace

struct Server {
    Ctx* ctx = nullptr;
    rpd_server_config cfg{};
    uint64_t budget = 0;
    cudaMemPool_t pool = nullptr;
    std::chrono::steady_clock::time_point t0;

    std::mutex mu;                      // guards everything below this line
    std::condition_variable cv;         // submissions, GPU completions, stop
    std::deque<Request*> queue;
    std::vector<Request*> running;
    int admitting = 0;                  // popped from the queue, not yet in `running`
    std::deque<rpd_completion> done;
    std::map<uint64_t, Request*> by_id; // queued or running
    uint64_t next_id = 1;
    int64_t submitted = 0, completed = 0, rejected = 0;
    uint64_t launches = 0;              // kernels enqueued for requests
    int64_t jobs_created = 0, jobs_destroyed = 0, scratch_grown = 0;
    double kernel_ms[RPD_KERNEL_COUNT_] = {};  // profile: per kernel family over finished requests
    uint64_t kernel_n[RPD_KERNEL_COUNT_] = {};
    uint64_t reserved = 0, peak = 0;    // request buffers + cached jobs
    std::multimap<std::pair<int, int>, CachedJob> idle_jobs;
    std::map<Job*, uint64_t> busy_jobs;
    bool stop = false;
    std::string fatal;

    std::vector<Slot> slots;
    std::thread worker;

    double now_ms() const {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

// Runs on the CUDA runtime's callback thread when a request's stream reaches its end. It takes
// no lock: the scheduler may hold its mutex inside a call that waits for the device (a job's
// cudaFree), which would wait for this callback in turn. A wake-up lost between the
// scheduler's check and its wait costs at most the wait's time-out.
void CUDART_CB on_request_done(void* p) {
    Request* r = static_cast<Request*>(p);
    Server* s = r->server;
    r->gpu_done.store(true);
    s->cv.notify_all();
}

rpd_config request_config(const Server& s, const rpd_request& r) {
    rpd_config c = s.cfg.knobs;
    c.image_width = r.width;
    c.image_height = r.height;
    return c;
}

uint64_t job_bytes(const rpd_config& c, int64_t span_samples) {
    // the arena plus the offsets (8 B per pixel) and the per-sample scratch of the largest push
    const int64_t np = int64_t(c.image_width) * c.image_height;
    return rpd_job_footprint(&c) + uint64_t(np + np / 512 + 64) * 9 + uint64_t(span_samples + 64) * 12 + 512;
}

int64_t span_samples(const rpd_config& c, int32_t spp) {
    const int64_t np = int64_t(c.image_width) * c.image_height;
    // a span is whole rows: at least one row even when a row holds more than kSpanSamples
    const int64_t first = std::min<int64_t>(int64_t(spp) * np, std::max<int64_t>(kSpanSamples, int64_t(spp) * c.image_width));
    const int64_t extra = c.adaptive_passes > 0 ? int64_t(c.adaptive_spp) * np : 0;
    return std::max<int64_t>({first, extra, int64_t(spp)});
}

// Destroys idle jobs (other sizes first) until `need` more bytes fit. Caller holds mu.
bool make_room(Server& s, uint64_t need, std::pair<int, int> keep) {
    while (s.reserved + need > s.budget) {
        auto victim = s.idle_jobs.end();
        for (auto it = s.idle_jobs.begin(); it != s.idle_jobs.end(); ++it)
            if (it->first != keep) { victim = it; break; }
        if (victim == s.idle_jobs.end()) victim = s.idle_jobs.begin();
        if (victim == s.idle_jobs.end()) return false;
        rpd_job_destroy(reinterpret_cast<rpd_job*>(victim->second.job));
        ++s.jobs_destroyed;
        s.reserved -= victim->second.bytes;
        s.idle_jobs.erase(victim);
    }
    return true;
}

// Enqueues request r's whole pipeline on its job's stream. Returns an rpd_status.
int enqueue_request(Server& s, Request& r) {
    Job& j = *r.job;
    const rpd_config c = j.cfg;
    const int64_t np = j.g.np;
    const bool compact = s.cfg.storage == RPD_STORAGE_FP16;
    const ReqLayout& L = r.layout;
    cudaStream_t st = j.stream;
    RPD_CUDA(cudaMallocFromPoolAsync(&r.mem, L.bytes, s.pool, st));
    char* base = static_cast<char*>(r.mem);
    rpd_synth_params prm;
    rpd_synth_defaults(&prm, r.req.width, r.req.height, r.req.seed);
    rpd_synth_region* table = reinterpret_cast<rpd_synth_region*>(base + L.table);
    uint8_t* region = reinterpret_cast<uint8_t*>(base + L.region);
    const uint64_t e = compact ? 2 : 4;
    SynthOut o{};
    o.compact = compact ? 1 : 0;
    for (int ch = 0; ch < 3; ++ch) {
        char* a = base + L.albedo + uint64_t(ch) * round256(uint64_t(np) * e);
        o.pixel_albedo[ch] = reinterpret_cast<float*>(a);
        o.pixel_albedo16[ch] = reinterpret_cast<uint16_t*>(a);
    }
    auto plane = [&](int k) { return base + L.planes + uint64_t(k) * L.plane_stride; };
    for (int ch = 0; ch < 3; ++ch) {
        o.radiance[ch] = reinterpret_cast<float*>(plane(ch));
        o.sqrt_radiance[ch] = reinterpret_cast<uint16_t*>(plane(ch));
        o.normal[ch] = reinterpret_cast<float*>(plane(3 + ch));
        o.normal16[ch] = reinterpret_cast<int16_t*>(plane(3 + ch));
    }
    o.depth = reinterpret_cast<float*>(plane(6));
    o.depth16 = reinterpret_cast<uint16_t*>(plane(6));
    for (int ch = 0; ch < 2; ++ch) {
        o.pixel_u[ch] = reinterpret_cast<float*>(plane(7 + ch));
        o.lens_u[ch] = reinterpret_cast<float*>(plane(9 + ch));
        o.brdf_u[ch] = reinterpret_cast<float*>(plane(11 + ch));
        o.light_u[ch] = reinterpret_cast<float*>(plane(13 + ch));
        o.pixel_u16[ch] = reinterpret_cast<uint16_t*>(plane(7 + ch));
        o.lens_u16[ch] = reinterpret_cast<uint16_t*>(plane(9 + ch));
        o.brdf_u16[ch] = reinterpret_cast<uint16_t*>(plane(11 + ch));
        o.light_u16[ch] = reinterpret_cast<uint16_t*>(plane(13 + ch));
    }
    const uint64_t byte_plane = round256(uint64_t(std::max<int64_t>(L.max_samples, 1)));
    o.flags = reinterpret_cast<uint8_t*>(plane(15));
    o.category = reinterpret_cast<uint8_t*>(plane(15) + byte_plane);
    float* out = reinterpret_cast<float*>(base + L.out);

    // the planes of a push whose first sample is sample `at` of the buffer
    auto push_planes = [&](int64_t at) {
        DeviceSamples d{};
        d.compact = o.compact;
        if (compact) {
            d.c16.depth_scale = 1.0f;
            for (int ch = 0; ch < 3; ++ch) {
                d.c16.sqrt_radiance[ch] = o.sqrt_radiance[ch] + at;
                d.c16.normal[ch] = o.normal16[ch] + at;
                d.c16.pixel_albedo[ch] = o.pixel_albedo16[ch];
            }
            d.c16.depth = o.depth16 + at;
            for (int ch = 0; ch < 2; ++ch) {
                d.c16.pixel_u[ch] = o.pixel_u16[ch] + at;
                d.c16.lens_u[ch] = o.lens_u16[ch] + at;
                d.c16.brdf_u[ch] = o.brdf_u16[ch] + at;
                d.c16.light_u[ch] = o.light_u16[ch] + at;
            }
        } else {
            for (int ch = 0; ch < 3; ++ch) {
                d.radiance[ch] = o.radiance[ch] + at;
                d.normal[ch] = o.normal[ch] + at;
                d.pixel_albedo[ch] = o.pixel_albedo[ch];
            }
            d.depth = o.depth + at;
            for (int ch = 0; ch < 2; ++ch) {
                d.pixel_u[ch] = o.pixel_u[ch] + at;
                d.lens_u[ch] = o.lens_u[ch] + at;
                d.brdf_u[ch] = o.brdf_u[ch] + at;
                d.light_u[ch] = o.light_u[ch] + at;
            }
        }
        d.flags = o.flags + at;
        d.category = o.category + at;
        return d;
    };

    rpd_job* jh = reinterpret_cast<rpd_job*>(&j);
    int rc = RPD_OK;
#define SRV_TRY(x)                    \
    do {                              \
        rc = (x);                     \
        if (rc != RPD_OK) return rc;  \
    } while (0)
    {
        KernelScope ks(j, RPD_KERNEL_SYNTH);
        k_srv_regions<<<1, RPD_SYNTH_MAX_REGIONS, 0, st>>>(prm, table);
        k_srv_region_map<<<grid_for(np, 256), 256, 0, st>>>(prm, table, np, region, o);
        j.launches += 2;
    }
    SRV_TRY(rpd_job_begin_frame(jh));
    // the first pass: generated at once, pushed in spans of whole rows that bound the scratch
    const int32_t spp = r.req.spp;
    if (spp > 0) {
        {
            KernelScope ks(j, RPD_KERNEL_SYNTH);
            int spp_shift = -1;
            if ((spp & (spp - 1)) == 0)
                for (spp_shift = 0; (1 << spp_shift) < spp; ++spp_shift) {}
            for (int y0 = 0; y0 < c.image_height; y0 += 65535) {  // grid rows per launch
                const dim3 sgrid(unsigned((int64_t(c.image_width) * spp + 255) / 256),
                                 unsigned(std::min(65535, c.image_height - y0)));
                k_srv_synth_uniform<<<sgrid, 256, 0, st>>>(prm, table, region, spp, spp_shift, y0, 0u, o);
            }
            j.launches += 1;
        }
        const int64_t rows_per_span =
            std::max<int64_t>(1, (kSpanSamples / std::max<int64_t>(1, int64_t(spp) * c.image_width)) & ~int64_t(7));
        for (int64_t y0 = 0; y0 < c.image_height; y0 += rows_per_span) {
            const int64_t y1 = std::min<int64_t>(c.image_height, y0 + rows_per_span);
            const int64_t first = y0 * c.image_width, count = (y1 - y0) * c.image_width;
            SRV_TRY(push_device_async(j, push_planes(first * spp), first, count, spp, nullptr, count * spp));
        }
    }
    SRV_TRY(rpd_job_end_pass(jh));
    // render() runs statmc_denoise and recompute_sensitivity in every adaptive pass
    // (main.cpp:1547-1552) and again after the loop (1554-1556). Before that final
    // statmc_denoise nothing reads what they write: variance_denoise and
    // compute_adaptive_sample_counts read the per-pixel statistics, the feature cache and the hit
    // counts only (main.cpp:1166-1446), recompute_sensitivity starts over from the grid on every
    // call (741-953), and the final statmc_denoise overwrites every plane the earlier ones wrote.
    // So the loop runs them once, after the last pass, and the result is the same bits (the
    // tests compare it with the full sequence). The variance_denoise after the loop (1556) writes
    // only the denoised variance, which finalize does not read and the request does not return:
    // it is not run either.
    int64_t* totals = s.slots[size_t(r.slot)].totals;
    const int passes = c.adaptive_spp > 0 ? std::max(0, c.adaptive_passes) : 0;
    for (int p = 1; p <= passes; ++p) {
        SRV_TRY(rpd_variance_denoise(jh));
        SRV_TRY(rpd_compute_adaptive_sample_counts(jh, nullptr, RPD_MEM_DEVICE));
        RPD_CUDA(launch_offsets_scan(j, j.p.counts, np));
        RPD_CUDA(cudaMemcpyAsync(totals + p, j.offsets + np, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        {
            KernelScope ks(j, RPD_KERNEL_SYNTH);
            k_srv_synth_counts<<<grid_for(np, kSynthPix), 256, 0, st>>>(prm, table, region, j.offsets, np,
                                                                          L.max_samples, uint32_t(p) * kPassOrdinalStride, o);
            j.launches += 1;
        }
        // the offsets of these counts are in j.offsets already (the scan above)
        SRV_TRY(push_device_async(j, push_planes(0), 0, np, 0, j.p.counts, int64_t(c.adaptive_spp) * np, true));
        SRV_TRY(rpd_job_end_pass(jh));
    }
    SRV_TRY(rpd_recompute_sensitivity(jh));
    SRV_TRY(rpd_statmc_denoise(jh));
    SRV_TRY(rpd_finalize(jh));
    k_srv_pack<<<grid_for(np, 256), 256, 0, st>>>(j.p.denoised[0], j.p.denoised[1], j.p.denoised[2], out, np);
    j.launches += 1;
    Slot& slot = s.slots[size_t(r.slot)];
    void* dst = r.req.denoised_out ? static_cast<void*>(r.req.denoised_out) : static_cast<void*>(slot.staging);
    const cudaMemcpyKind kind =
        (r.req.denoised_out && r.req.out_where == RPD_MEM_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    RPD_CUDA(cudaMemcpyAsync(dst, out, uint64_t(np) * 12, kind, st));
    RPD_CUDA(cudaFreeAsync(r.mem, st));
    r.mem = nullptr;
    RPD_CUDA(cudaLaunchHostFunc(st, on_request_done, &r));
#undef SRV_TRY
    return RPD_OK;
}

// Takes an idle job of the request's size or creates one; caller holds mu and has checked the
// budget for `create_bytes` when no idle job exists.
int acquire_job(Server& s, Request& r, Job** out) {
    const std::pair<int, int> key{r.req.width, r.req.height};
    const rpd_config c = request_config(s, r.req);
    const int64_t need_span = span_samples(c, r.req.spp);
    auto it = s.idle_jobs.find(key);
    if (it != s.idle_jobs.end()) {
        Job* j = it->second.job;
        uint64_t bytes = it->second.bytes;
        s.idle_jobs.erase(it);
        const uint64_t caps = j->lum_cap + j->offsets_cap;
        const int st = job_reserve(*j, need_span);
        if (j->lum_cap + j->offsets_cap != caps) ++s.scratch_grown;
        if (st != RPD_OK) {
            rpd_job_destroy(reinterpret_cast<rpd_job*>(j));
            s.reserved -= bytes;
            return st;
        }
        const uint64_t now_bytes = std::max(bytes, job_bytes(c, need_span));
        s.reserved += now_bytes - bytes;
        s.busy_jobs[j] = now_bytes;
        *out = j;
        return RPD_OK;
    }
    // the job's memory from the server's pool, in the order of its stream: creating, growing and
    // destroying cached jobs then never synchronises the device while other requests run
    Job* j = nullptr;
    int st = job_create(s.ctx, &c, s.pool, &j);
    if (st != RPD_OK) return st;
    rpd_job* h = reinterpret_cast<rpd_job*>(j);
    ++s.jobs_created;
    if (s.cfg.profile) rpd_job_set_profiling(h, 1);
    // requests share the GPU: by default an allocation takes half the SMs (one block each), and
    // the other requests' kernels keep the rest while it walks its chains (measured 1 % more
    // throughput on the mixed stream than one block per SM)
    int blocks = s.cfg.allocator_blocks;
    if (blocks == 0) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s.ctx->device) == cudaSuccess)
            blocks = std::max(2, sms / 2);
    }
    if (blocks >= 2) rpd_job_set_tuning(h, RPD_TUNE_ALLOCATOR, blocks);
    st = job_reserve(*j, need_span);
    if (st != RPD_OK) {
        rpd_job_destroy(h);
        return st;
    }
    const uint64_t bytes = job_bytes(c, need_span);
    s.reserved += bytes;
    s.busy_jobs[j] = bytes;
    *out = j;
    return RPD_OK;
}

void finish(Server& s, Request* r) {  // caller holds mu
    rpd_completion cpl{};
    cpl.id = r->id;
    cpl.tag = r->req.tag;
    cpl.status = r->status;
    cpl.width = r->req.width;
    cpl.height = r->req.height;
    cpl.spp = r->req.spp;
    const int64_t np = int64_t(r->req.width) * r->req.height;
    int64_t samples = int64_t(r->req.spp) * np;
    if (r->status == RPD_OK && r->slot >= 0) {
        const rpd_config c = request_config(s, r->req);
        const int passes = c.adaptive_spp > 0 ? std::max(0, c.adaptive_passes) : 0;
        for (int p = 1; p <= passes; ++p) samples += s.slots[size_t(r->slot)].totals[p];
    }
    cpl.samples = samples;
    cpl.submit_ms = r->t_submit;
    cpl.admit_ms = r->t_admit;
    cpl.done_ms = r->t_done;
    s.done.push_back(cpl);
    ++s.completed;
    s.by_id.erase(r->id);
    delete r;
}

void retire(Server& s, Request* r) {  // caller holds mu; r's GPU work has finished
    r->t_done = s.now_ms();
    if (r->job && s.cfg.profile) {
        rpd_job* jh = reinterpret_cast<rpd_job*>(r->job);
        for (int k = 0; k < RPD_KERNEL_COUNT_; ++k) {
            double ms = 0.0;
            uint64_t n = 0;
            if (rpd_job_kernel_time(jh, rpd_kernel(k), &ms, &n) == RPD_OK) {
                s.kernel_ms[k] += ms;
                s.kernel_n[k] += n;
            }
        }
        rpd_job_reset_kernel_times(jh);
    }
    if (r->job) {
        auto it = s.busy_jobs.find(r->job);
        const uint64_t bytes = it != s.busy_jobs.end() ? it->second : 0;
        if (it != s.busy_jobs.end()) s.busy_jobs.erase(it);
        s.idle_jobs.insert({{r->req.width, r->req.height}, CachedJob{r->job, bytes}});
        r->job = nullptr;
    }
    s.reserved -= r->reserve;
    if (r->slot >= 0) s.slots[size_t(r->slot)].busy = false;
    finish(s, r);
}

void worker_loop(Server* sp) {
    Server& s = *sp;
    cudaSetDevice(s.ctx->device);
    std::unique_lock<std::mutex> lk(s.mu);
    for (;;) {
        bool progress = false;
        // retire what the GPU finished
        for (size_t i = 0; i < s.running.size();) {
            Request* r = s.running[i];
            if (r->gpu_done.load()) {
                s.running.erase(s.running.begin() + long(i));
                retire(s, r);
                progress = true;
            } else {
                ++i;
            }
        }
        // admit in arrival order while a slot and the budget allow
        while (!s.queue.empty()) {
            int slot = -1;
            for (size_t i = 0; i < s.slots.size(); ++i)
                if (!s.slots[i].busy) { slot = int(i); break; }
            if (slot < 0) break;
            Request* r = s.queue.front();
            const std::pair<int, int> key{r->req.width, r->req.height};
            const rpd_config c = request_config(s, r->req);
            const bool have_job = s.idle_jobs.count(key) != 0;
            const uint64_t need = r->reserve + (have_job ? 0 : job_bytes(c, span_samples(c, r->req.spp)));
            if (s.reserved + need > s.budget) {
                if (!make_room(s, need, key)) break;  // wait for running requests to free memory
            }
            s.queue.pop_front();
            r->slot = slot;
            Slot& sl = s.slots[size_t(slot)];
            sl.busy = true;
            const uint64_t out_bytes = uint64_t(r->req.width) * r->req.height * 12;
            int st = RPD_OK;
            if (!r->req.denoised_out && sl.staging_bytes < out_bytes) {
                // at least doubled, so a slot's staging is replaced a few times at most (freeing
                // page-locked memory may wait for the device)
                const uint64_t grow = std::max<uint64_t>(out_bytes, 2 * sl.staging_bytes);
                if (sl.staging) cudaFreeHost(sl.staging);
                sl.staging = nullptr;
                sl.staging_bytes = 0;
                if (cudaMallocHost(&sl.staging, grow) == cudaSuccess) sl.staging_bytes = grow;
                else st = cuda_fail(cudaErrorMemoryAllocation, "pinned result buffer");
            }
            if (st == RPD_OK) st = acquire_job(s, *r, &r->job);
            r->t_admit = s.now_ms();
            if (st == RPD_OK) {
                s.reserved += r->reserve;
                s.peak = std::max(s.peak, s.reserved);
                ++s.admitting;
                lk.unlock();  // the request, its slot and its job belong to this thread now
                const uint64_t l0 = r->job->launches.load();
                st = enqueue_request(s, *r);
                const uint64_t l1 = r->job->launches.load();
                lk.lock();
                --s.admitting;
                s.launches += l1 - l0;
                if (st == RPD_OK) {
                    s.running.push_back(r);
                } else {
                    // the stream holds part of the request: wait for it, then hand the job back
                    cudaStreamSynchronize(r->job->stream);
                    if (r->mem) cudaFreeAsync(r->mem, r->job->stream);
                    r->status = st;
                    retire(s, r);
                }
            } else {
                r->status = st;
                r->t_done = r->t_admit;
                sl.busy = false;
                finish(s, r);
            }
            progress = true;
        }
        if (s.stop && s.queue.empty() && s.running.empty() && s.admitting == 0) break;
        if (!progress) {
            // a stream that stopped on a device error never reaches its completion callback:
            // fail its request instead of waiting for it
            for (size_t i = 0; i < s.running.size();) {
                Request* r = s.running[i];
                const cudaError_t e = r->gpu_done.load() ? cudaSuccess : cudaStreamQuery(r->job->stream);
                if (e != cudaSuccess && e != cudaErrorNotReady) {
                    r->status = cuda_fail(e, "request stream");
                    s.fatal = rpd_last_error();
                    s.running.erase(s.running.begin() + long(i));
                    retire(s, r);
                    progress = true;
                } else {
                    ++i;
                }
            }
        }
        if (!progress) s.cv.wait_for(lk, std::chrono::microseconds(200));
    }
}

}  // namespace

}  // namespace rpd

using namespace rpd;

extern "C" {

void rpd_server_config_defaults(rpd_server_config* cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    rpd_config_defaults(&cfg->knobs);
    cfg->knobs.image_width = 1;
    cfg->knobs.image_height = 1;
    cfg->hbm_budget_bytes = 0;
    cfg->max_inflight = 16;
    cfg->storage = RPD_STORAGE_FP16;
}

int rpd_server_create(rpd_ctx* ctx, const rpd_server_config* cfg, rpd_server** out) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !cfg || !out) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (cfg->max_inflight < 1 || cfg->max_inflight > 256)
        return fail(RPD_ERR_INVALID_ARGUMENT, "max_inflight must be 1..256");
    if (cfg->storage != RPD_STORAGE_FP32 && cfg->storage != RPD_STORAGE_FP16)
        return fail(RPD_ERR_INVALID_ARGUMENT, "unknown sample storage");
    if (cfg->allocator_blocks < 0 || cfg->allocator_blocks == 1 || cfg->allocator_blocks > 4096)
        return fail(RPD_ERR_INVALID_ARGUMENT, "allocator_blocks must be 0 or 2..4096");
    {
        rpd_config probe = cfg->knobs;
        probe.image_width = std::max(probe.image_width, 1);
        probe.image_height = std::max(probe.image_height, 1);
        char msg[256];
        if (rpd_config_validate(&probe, msg, sizeof(msg)) != RPD_OK) return fail(RPD_ERR_INVALID_CONFIG, msg);
    }
    RPD_CUDA(cudaSetDevice(c->device));
    Server* s = new (std::nothrow) Server();
    if (!s) return fail(RPD_ERR_OUT_OF_MEMORY, "server allocation failed");
    s->ctx = c;
    s->cfg = *cfg;
    s->budget = cfg->hbm_budget_bytes ? std::min<uint64_t>(cfg->hbm_budget_bytes, c->budget) : c->budget;
    s->t0 = std::chrono::steady_clock::now();
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = c->device;
    cudaError_t e = cudaMemPoolCreate(&s->pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = ~uint64_t(0);  // keep freed blocks for the next requests
        e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    s->slots.resize(size_t(cfg->max_inflight));
    for (auto& sl : s->slots)
        if (e == cudaSuccess) e = cudaMallocHost(&sl.totals, 16 * sizeof(int64_t));
    if (e != cudaSuccess) {
        for (auto& sl : s->slots)
            if (sl.totals) cudaFreeHost(sl.totals);
        if (s->pool) cudaMemPoolDestroy(s->pool);
        delete s;
        return cuda_fail(e, "server set-up");
    }
    s->worker = std::thread(worker_loop, s);
    *out = reinterpret_cast<rpd_server*>(s);
    return RPD_OK;
}

int rpd_server_submit(rpd_server* srv, const rpd_request* req, uint64_t* id_out) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s || !req) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    if (req->width <= 0 || req->height <= 0 || req->spp < 0 || req->spp > 65535)
        return fail(RPD_ERR_INVALID_ARGUMENT, "request size and spp must be positive (spp at most 65535)");
    rpd_config c = s->cfg.knobs;
    c.image_width = req->width;
    c.image_height = req->height;
    char msg[256];
    if (rpd_config_validate(&c, msg, sizeof(msg)) != RPD_OK) return fail(RPD_ERR_INVALID_CONFIG, msg);
    const int64_t np = int64_t(req->width) * req->height;
    const int passes = c.adaptive_spp > 0 ? std::max(0, c.adaptive_passes) : 0;
    if (passes >= 16) return fail(RPD_ERR_INVALID_CONFIG, "the serving loop runs at most 15 adaptive passes");
    if (np > (int64_t(1) << 27)) return fail(RPD_ERR_INVALID_ARGUMENT, "request larger than 2^27 pixels");
    auto* r = new (std::nothrow) Request();
    if (!r) return fail(RPD_ERR_OUT_OF_MEMORY, "request allocation failed");
    r->req = *req;
    r->server = s;
    r->layout = request_layout(np, req->spp, c.adaptive_spp, passes, s->cfg.storage == RPD_STORAGE_FP16);
    r->reserve = r->layout.bytes;
    const uint64_t alone = r->reserve + job_bytes(c, span_samples(c, req->spp));
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
        delete r;
        return fail(RPD_ERR_STATE, "the server is shutting down");
    }
    if (alone > s->budget) {
        ++s->rejected;
        delete r;
        return fail(RPD_ERR_OVER_BUDGET, "request needs " + std::to_string(alone) + " bytes of HBM; the budget is " +
                                             std::to_string(s->budget));
    }
    r->id = s->next_id++;
    r->t_submit = s->now_ms();
    s->queue.push_back(r);
    s->by_id[r->id] = r;
    ++s->submitted;
    if (id_out) *id_out = r->id;
    s->cv.notify_all();
    return RPD_OK;
}

int rpd_server_poll(rpd_server* srv, rpd_completion* out, int32_t max, int32_t* n_out) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s || (!out && max > 0) || !n_out) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    int32_t n = 0;
    while (n < max && !s->done.empty()) {
        out[n++] = s->done.front();
        s->done.pop_front();
    }
    *n_out = n;
    return RPD_OK;
}

int rpd_server_drain(rpd_server* srv, int32_t timeout_ms) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s) return fail(RPD_ERR_INVALID_ARGUMENT, "null server");
    const auto until = std::chrono::steady_clock::now() + std::chrono::milliseconds(std::max(0, timeout_ms));
    std::unique_lock<std::mutex> lk(s->mu);
    while (!s->queue.empty() || !s->running.empty() || s->admitting > 0) {
        if (timeout_ms >= 0 && std::chrono::steady_clock::now() >= until)
            return fail(RPD_ERR_TIMEOUT, "requests still queued or running");
        s->cv.wait_for(lk, std::chrono::milliseconds(1));
    }
    if (!s->fatal.empty()) return fail(RPD_ERR_CUDA, s->fatal);
    return RPD_OK;
}

int rpd_server_cancel(rpd_server* srv, uint64_t id) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s) return fail(RPD_ERR_INVALID_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
        if ((*it)->id == id) {
            Request* r = *it;
            s->queue.erase(it);
            r->status = RPD_ERR_CANCELLED;
            r->t_admit = r->t_done = s->now_ms();
            finish(*s, r);
            return RPD_OK;
        }
    }
    if (s->by_id.count(id)) return fail(RPD_ERR_STATE, "request " + std::to_string(id) + " is already on the GPU");
    return fail(RPD_ERR_INVALID_ARGUMENT, "no queued request " + std::to_string(id));
}

int rpd_server_get_stats(rpd_server* srv, rpd_server_stats* out) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s || !out) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->rejected = s->rejected;
    out->queued = int64_t(s->queue.size());
    out->inflight = int64_t(s->running.size()) + s->admitting;
    out->bytes_reserved = s->reserved;
    out->bytes_peak = s->peak;
    out->bytes_budget = s->budget;
    out->jobs_cached = int64_t(s->idle_jobs.size() + s->busy_jobs.size());
    out->now_ms = s->now_ms();
    out->launches = int64_t(s->launches);
    out->jobs_created = s->jobs_created;
    out->jobs_destroyed = s->jobs_destroyed;
    out->scratch_grown = s->scratch_grown;
    return RPD_OK;
}

int rpd_server_kernel_times(rpd_server* srv, double* ms_out, uint64_t* launches_out) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s || !ms_out || !launches_out) return fail(RPD_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    for (int k = 0; k < RPD_KERNEL_COUNT_; ++k) {
        ms_out[k] = s->kernel_ms[k];
        launches_out[k] = s->kernel_n[k];
    }
    return RPD_OK;
}

void rpd_server_destroy(rpd_server* srv) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->ctx->device);
    cudaDeviceSynchronize();
    for (auto& kv : s->idle_jobs) rpd_job_destroy(reinterpret_cast<rpd_job*>(kv.second.job));
    for (auto& kv : s->busy_jobs) rpd_job_destroy(reinterpret_cast<rpd_job*>(kv.first));
    for (auto& sl : s->slots) {
        if (sl.totals) cudaFreeHost(sl.totals);
        if (sl.staging) cudaFreeHost(sl.staging);
    }
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
}

}  // extern "C"
