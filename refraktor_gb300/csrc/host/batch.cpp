// Batched rendering: many units (flames or animation frames) of one flame
// structure in one persistent launch of rfk_bin_batch, then density-estimation
// blur and tonemap per unit. The pipeline runs on one stream, directly or as
// a CUDA graph captured on the first run and replayed afterwards; everything a
// replay needs to change (samples, the run's Philox sub-stream) is read from
// pinned host memory by copy nodes, so the graph never has to be rebuilt.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../kernels/image_kernels.h"
#include "runtime_internal.h"

using namespace rfk::rt;

namespace {

// Host mirrors of rfk_unit / rfk_unit_counters / rfk_batch_args in rfk_iterate.cuh.
struct dev_unit {
    const float* params;
    float4* bins;
    unsigned w, h;
    unsigned long long quality_target;
    unsigned long long first_item;
    unsigned check;
    unsigned pad;
};
constexpr int kUnitWords = 4;     // quality, draws, passes, items
constexpr int kCounterWords = 6;  // rfk_counters: quality, passes, start, stop, draws, status|pad
struct dev_batch_args {
    const dev_unit* units;
    unsigned long long* uc;
    unsigned nunits;
    unsigned passes_per_item;
    unsigned long long nitems;
    unsigned long long* next_item;
    unsigned warmup;
    unsigned seed, salt;
    const unsigned* call_id;
    unsigned long long time_ns;
    const volatile unsigned* stop;
    unsigned long long* counters;
};
constexpr uint32_t kMaxMillis = 60000;

size_t pixel_bytes(int f) {
    switch (f) {
    case RFK_HALF3: return 6;
    case RFK_HALF4: return 8;
    case RFK_FLOAT3: return 12;
    case RFK_FLOAT4: return 16;
    default: return 0;
    }
}

template <typename T>
void dalloc(T*& p, size_t bytes) {
    void* v = nullptr;
    cuda_check(cudaMalloc(&v, std::max<size_t>(bytes, 16)), "cudaMalloc (batch)");
    p = static_cast<T*>(v);
}

}  // namespace

struct rfk_batch {
    std::shared_ptr<const kernel_impl> k;
    std::vector<rfk_batch_unit> units;
    rfk_batch_opts opts{};
    size_t nsamples = 0, sample_size = 0;
    std::vector<size_t> px_off, img_off;  // per unit: first pixel, first image byte
    size_t total_px = 0, img_bytes = 0;
    uint64_t nitems = 0;
    unsigned naff = 0;
    // Runs of samples [first, first + count) that fix_rotation unwraps as one
    // spline: consecutive samples j - 1 and j are in one run when a unit's
    // segment uses both (its knots seg .. seg + 3). Unwrapping across samples
    // that no segment joins (one independent flame after another) would add
    // multiples of 2 pi to the later flames' angles, which then reach FP32
    // with a coarser rounding than the same flame rendered alone; restarting
    // keeps every independent flame's prepared parameters bit-identical to the
    // single-flame path's.
    std::vector<std::pair<unsigned, unsigned>> rot_runs;

    double* d_samples = nullptr;
    float4* d_coeff = nullptr;
    unsigned* d_aff = nullptr;
    unsigned* d_seg = nullptr;
    float* d_t = nullptr;
    float* d_params = nullptr;
    float4* d_bins = nullptr;
    float4* d_blur = nullptr;
    unsigned char* d_img = nullptr;
    dev_unit* d_units = nullptr;
    unsigned long long* d_uc = nullptr;        // kUnitWords per unit
    unsigned long long* d_counters = nullptr;  // kCounterWords, then the queue head
    unsigned* d_call = nullptr;

    double* h_samples = nullptr;        // pinned staging of the samples
    unsigned long long* h_out = nullptr;  // pinned: unit counters, then kCounterWords
    unsigned* h_call = nullptr;         // pinned: this run's Philox sub-stream
    unsigned* h_stop = nullptr;         // mapped pinned stop flag
    unsigned* d_stop = nullptr;
    cudaEvent_t done = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int launches = 0;
    unsigned runs = 0;
    bool samples_set = false, pending = false;

    ~rfk_batch() {
        if (done) cudaEventSynchronize(done);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (void* p : {(void*)d_samples, (void*)d_coeff, (void*)d_aff, (void*)d_seg, (void*)d_t, (void*)d_params,
                        (void*)d_bins, (void*)d_blur, (void*)d_img, (void*)d_units, (void*)d_uc, (void*)d_counters,
                        (void*)d_call})
            if (p) cudaFree(p);
        for (void* p : {(void*)h_samples, (void*)h_out, (void*)h_call, (void*)h_stop})
            if (p) cudaFreeHost(p);
        if (done) cudaEventDestroy(done);
    }

    // The whole pipeline on stream s; returns the number of kernel launches.
    int enqueue(cudaStream_t s) {
        int n = 0;
        const size_t nu = units.size();
        cuda_check(cudaMemcpyAsync(d_call, h_call, sizeof(unsigned), cudaMemcpyHostToDevice, s), "H2D run id");
        cuda_check(cudaMemcpyAsync(d_samples, h_samples, nsamples * sample_size * sizeof(double), cudaMemcpyHostToDevice, s),
                   "H2D samples");
        for (const auto& r : rot_runs) {
            cuda_check(rfk_launch_fix_rotation(d_samples + (size_t)r.first * sample_size, r.second, (unsigned)sample_size,
                                               (unsigned)k->gen.size_reals, d_aff, naff, s),
                       "fix_rotation");
            n++;
        }
        const unsigned nseg = (unsigned)(nsamples - 3);
        cuda_check(rfk_launch_catmull(d_samples, (unsigned)sample_size, nseg, d_coeff, s), "catmull");
        n++;
        {
            unsigned ss = (unsigned)sample_size, seed = opts.seed, salt = k->salt, jitter = 0;
            float4* coeff = d_coeff;
            unsigned* seg = d_seg;
            float* t = d_t;
            float* out = d_params;
            void* args[] = {&coeff, &ss, &seg, &t, &out, &seed, &salt, &jitter};
            launch(k->f_prepare, (unsigned)nu, 256, s, args, "rfk_prepare (batch)");
            n++;
        }
        cuda_check(cudaMemsetAsync(d_bins, 0, total_px * sizeof(float4), s), "clear histograms");
        cuda_check(cudaMemsetAsync(d_uc, 0, nu * kUnitWords * sizeof(unsigned long long), s), "clear unit counters");
        cuda_check(rfk_launch_clear_counters(d_counters, s), "clear counters");
        n++;
        cuda_check(cudaMemsetAsync(d_counters + kCounterWords, 0, sizeof(unsigned long long), s), "clear queue");
        {
            dev_batch_args a{};
            a.units = d_units;
            a.uc = d_uc;
            a.nunits = (unsigned)nu;
            a.passes_per_item = opts.passes_per_item;
            a.nitems = nitems;
            a.next_item = d_counters + kCounterWords;
            a.warmup = opts.warmup;
            a.seed = opts.seed;
            a.salt = k->salt;
            a.call_id = d_call;
            const uint32_t ms = (opts.millis == 0 || opts.millis > kMaxMillis) ? kMaxMillis : opts.millis;
            a.time_ns = (unsigned long long)ms * 1000000ull;
            a.stop = d_stop;
            a.counters = d_counters;
            void* args[] = {&a};
            launch(k->f_bin_batch, (unsigned)k->grid, (unsigned)k->block, s, args, "rfk_bin_batch");
            n++;
        }
        if (opts.out_format >= 0 || opts.de_max_radius > 0.0f) {
            for (size_t u = 0; u < nu; u++) {
                const rfk_batch_unit& U = units[u];
                const float4* src = d_bins + px_off[u];
                if (opts.de_max_radius > 0.0f) {
                    cuda_check(rfk_launch_de_blur(src, d_blur + px_off[u], U.width, U.height, opts.de_max_radius,
                                                  opts.de_min_radius, opts.de_curve, s),
                               "density blur (batch)");
                    n++;
                    src = d_blur + px_off[u];
                }
                if (opts.out_format >= 0) {
                    const double per_hit = 1.0 / (255.0 * (double)U.width * (double)U.height);
                    cuda_check(rfk_launch_tonemap(src, U.width * U.height, d_img + img_off[u], opts.out_format,
                                                  opts.precise_tonemap, U.gamma, 0.0f, U.brightness, U.vibrancy,
                                                  U.highlight_power, nullptr, nullptr, d_uc + u * kUnitWords, per_hit, s),
                               "tonemap (batch)");
                    n++;
                }
            }
        }
        cuda_check(cudaMemcpyAsync(h_out, d_uc, nu * kUnitWords * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s),
                   "D2H unit counters");
        cuda_check(cudaMemcpyAsync(h_out + nu * kUnitWords, d_counters, kCounterWords * sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, s),
                   "D2H counters");
        return n;
    }
};

extern "C" {

rfk_status rfk_flames_align(const rfk_db* db, const rfk_flame* const* flames, size_t n, int by_weight, rfk_flame** out) {
    return guard([&] {
        if (!db || !flames || !out || n == 0) fail(RFK_E_INVALID, "null argument");
        std::vector<rfk::flame> in;
        for (size_t i = 0; i < n; i++) {
            if (!flames[i]) fail(RFK_E_INVALID, "null flame");
            in.push_back(flames[i]->f);
        }
        std::vector<rfk::flame> al = rfk::align_structures(db->db, in, by_weight != 0);
        std::vector<std::unique_ptr<rfk_flame>> hs;
        for (auto& f : al) {
            auto h = std::make_unique<rfk_flame>();
            h->f = std::move(f);
            hs.push_back(std::move(h));
        }
        for (size_t i = 0; i < n; i++) out[i] = hs[i].release();
    });
}

rfk_status rfk_batch_create(rfk_kernel* k, const rfk_batch_unit* units, size_t nunits, size_t nsamples,
                            const rfk_batch_opts* opts, rfk_batch** out) {
    return guard([&] {
        if (!k || !units || !out || nunits == 0) fail(RFK_E_INVALID, "null argument");
        if (nsamples < 4) fail(RFK_E_INVALID, "need at least 4 packed samples");
        if (nunits > 0x7FFFFFFF) fail(RFK_E_INVALID, "too many units");
        auto b = std::make_unique<rfk_batch>();
        b->k = k->impl;
        b->units.assign(units, units + nunits);
        if (opts) b->opts = *opts;
        rfk_batch_opts& o = b->opts;
        if (o.passes_per_item == 0) o.passes_per_item = 256;
        if (o.item_factor == 0) o.item_factor = 3;
        if (o.out_format < -1 || o.out_format > RFK_FLOAT4) fail(RFK_E_INVALID, "bad output format");
        if (o.de_max_radius < 0.0f || o.de_max_radius > (float)RFK_DE_MAX_RADIUS_CAP)
            fail(RFK_E_INVALID, "de_max_radius must be in [0, 9]");
        const unsigned nseg = (unsigned)(nsamples - 3);
        b->nsamples = nsamples;
        b->sample_size = b->k->gen.size_reals + rfk::palette_reals;
        {
            // joined[j]: samples j - 1 and j belong to one unit's segment
            std::vector<char> joined(nsamples, 0);
            for (size_t u = 0; u < nunits; u++) {
                const size_t sg = units[u].segment;
                if (sg >= nseg) continue;  // rejected below
                for (size_t j = sg + 1; j <= sg + 3; j++) joined[j] = 1;
            }
            unsigned first = 0;
            for (unsigned j = 1; j <= (unsigned)nsamples; j++)
                if (j == (unsigned)nsamples || !joined[j]) {
                    b->rot_runs.emplace_back(first, j - first);
                    first = j;
                }
        }

        // queue: items per unit from the least number of chain steps that can
        // reach the target (every step a full-opacity draw), times item_factor
        const double chains = (double)b->k->block * b->k->cpt;
        const double per_item = chains * o.passes_per_item;
        const double per_pass = chains * b->k->grid;
        std::vector<dev_unit> du(nunits);
        for (size_t u = 0; u < nunits; u++) {
            const rfk_batch_unit& U = units[u];
            if (U.width == 0 || U.height == 0) fail(RFK_E_INVALID, "image size must be positive");
            if ((uint64_t)U.width * U.height > 0xFFFFFFFFull) fail(RFK_E_INVALID, "image too large");
            if (!(U.quality > 0.0)) fail(RFK_E_INVALID, "unit quality must be positive");
            if (U.segment >= nseg) fail(RFK_E_INVALID, "unit segment out of range");
            if (!(U.t >= 0.0f && U.t <= 1.0f)) fail(RFK_E_INVALID, "unit t must be in [0, 1]");
            if (o.out_format >= 0 && !(U.gamma > 0.0f)) fail(RFK_E_INVALID, "unit gamma must be positive");
            const double px = (double)U.width * U.height;
            b->px_off.push_back(b->total_px);
            b->img_off.push_back(b->img_bytes);
            b->total_px += (size_t)px;
            b->img_bytes += (size_t)px * pixel_bytes(o.out_format);
            b->img_bytes = (b->img_bytes + 255) / 256 * 256;
            du[u].w = U.width;
            du[u].h = U.height;
            du[u].quality_target = (unsigned long long)std::ceil(U.quality * px * 255.0);
            du[u].first_item = b->nitems;
            b->nitems += (uint64_t)std::ceil(o.item_factor * U.quality * px / per_item) + 1;
            // quality checks often enough that the unit overshoots its target
            // by a few % at most when every block works on it
            du[u].check = (unsigned)std::clamp(std::floor(0.05 * U.quality * px / per_pass), 1.0, 32.0);
            du[u].pad = 0;
        }

        b->naff = (unsigned)b->k->gen.affine_indices.size();
        dalloc(b->d_samples, nsamples * b->sample_size * sizeof(double));
        dalloc(b->d_coeff, (size_t)nseg * b->sample_size * sizeof(float4));
        dalloc(b->d_aff, b->naff * sizeof(unsigned));
        dalloc(b->d_seg, nunits * sizeof(unsigned));
        dalloc(b->d_t, nunits * sizeof(float));
        dalloc(b->d_params, nunits * b->k->sample_floats * sizeof(float));
        dalloc(b->d_bins, b->total_px * sizeof(float4));
        if (o.de_max_radius > 0.0f) dalloc(b->d_blur, b->total_px * sizeof(float4));
        if (o.out_format >= 0) dalloc(b->d_img, b->img_bytes);
        dalloc(b->d_units, nunits * sizeof(dev_unit));
        dalloc(b->d_uc, nunits * kUnitWords * sizeof(unsigned long long));
        dalloc(b->d_counters, (kCounterWords + 1) * sizeof(unsigned long long));
        dalloc(b->d_call, sizeof(unsigned));
        for (size_t u = 0; u < nunits; u++) {
            du[u].params = b->d_params + u * b->k->sample_floats;
            du[u].bins = b->d_bins + b->px_off[u];
        }
        std::vector<unsigned> aff(b->k->gen.affine_indices.begin(), b->k->gen.affine_indices.end()), seg(nunits);
        std::vector<float> t(nunits);
        for (size_t u = 0; u < nunits; u++) {
            seg[u] = units[u].segment;
            t[u] = units[u].t;
        }
        cuda_check(cudaMemcpy(b->d_aff, aff.data(), aff.size() * sizeof(unsigned), cudaMemcpyHostToDevice), "H2D affines");
        cuda_check(cudaMemcpy(b->d_seg, seg.data(), nunits * sizeof(unsigned), cudaMemcpyHostToDevice), "H2D schedule");
        cuda_check(cudaMemcpy(b->d_t, t.data(), nunits * sizeof(float), cudaMemcpyHostToDevice), "H2D schedule");
        cuda_check(cudaMemcpy(b->d_units, du.data(), nunits * sizeof(dev_unit), cudaMemcpyHostToDevice), "H2D units");

        cuda_check(cudaHostAlloc(&b->h_samples, nsamples * b->sample_size * sizeof(double), cudaHostAllocDefault),
                   "pinned samples");
        cuda_check(cudaHostAlloc(&b->h_out, (nunits * kUnitWords + kCounterWords) * sizeof(unsigned long long),
                                 cudaHostAllocDefault),
                   "pinned counters");
        cuda_check(cudaHostAlloc(&b->h_call, sizeof(unsigned), cudaHostAllocDefault), "pinned run id");
        cuda_check(cudaHostAlloc(&b->h_stop, sizeof(unsigned), cudaHostAllocMapped), "stop flag");
        *b->h_stop = 0;
        cuda_check(cudaHostGetDevicePointer(reinterpret_cast<void**>(&b->d_stop), b->h_stop, 0), "stop flag");
        cuda_check(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming), "event");
        *out = b.release();
    });
}

void rfk_batch_destroy(rfk_batch* b) { delete b; }

rfk_status rfk_batch_set_samples(rfk_batch* b, const double* samples) {
    return guard([&] {
        if (!b || !samples) fail(RFK_E_INVALID, "null argument");
        if (b->pending) cuda_check(cudaEventSynchronize(b->done), "batch wait");
        std::memcpy(b->h_samples, samples, b->nsamples * b->sample_size * sizeof(double));
        b->samples_set = true;
    });
}

rfk_status rfk_batch_run(rfk_batch* b, int use_graph, void* stream) {
    return guard([&] {
        if (!b) fail(RFK_E_INVALID, "null batch");
        if (!b->samples_set) fail(RFK_E_INVALID, "rfk_batch_set_samples has not been called");
        cudaStream_t s = (cudaStream_t)stream;
        if (b->pending) cuda_check(cudaEventSynchronize(b->done), "batch wait");
        *b->h_call = b->runs++ % 0xFFF0u;
        *b->h_stop = 0;
        if (use_graph) {
            if (!b->exec) {
                // legacy default stream cannot be captured
                if (s == nullptr || s == cudaStreamLegacy) fail(RFK_E_INVALID, "graph capture needs a non-default stream");
                cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
                int n = 0;
                try {
                    n = b->enqueue(s);
                } catch (...) {
                    cudaGraph_t g = nullptr;
                    cudaStreamEndCapture(s, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                cuda_check(cudaStreamEndCapture(s, &b->graph), "end capture");
                cuda_check(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
                b->launches = n;
            }
            cuda_check(cudaGraphLaunch(b->exec, s), "graph launch");
        } else {
            b->launches = b->enqueue(s);
        }
        cuda_check(cudaEventRecord(b->done, s), "event");
        b->pending = true;
    });
}

rfk_status rfk_batch_wait(rfk_batch* b, rfk_bin_result* total, rfk_bin_result* per_unit) {
    return guard([&] {
        if (!b) fail(RFK_E_INVALID, "null batch");
        if (!b->pending) fail(RFK_E_INVALID, "no run to wait for");
        cuda_check(cudaEventSynchronize(b->done), "batch wait");
        b->pending = false;
        const size_t nu = b->units.size();
        const unsigned long long* c = b->h_out + nu * kUnitWords;
        rfk_bin_result tr{};
        tr.elapsed_ms = c[3] > c[2] ? (double)(c[3] - c[2]) / 1e6 : 0.0;
        tr.total_passes = c[1];
        tr.status = (uint32_t)(c[5] & 0xFFFFFFFFu);
        uint64_t px = 0, hits = 0, reached = 0;
        for (size_t u = 0; u < nu; u++) {
            const unsigned long long* w = b->h_out + u * kUnitWords;
            const double upx = (double)b->units[u].width * b->units[u].height;
            const unsigned long long target = (unsigned long long)std::ceil(b->units[u].quality * upx * 255.0);
            if (per_unit) {
                rfk_bin_result r{};
                r.quality = (double)w[0] / (255.0 * upx);
                r.elapsed_ms = tr.elapsed_ms;
                r.total_passes = w[2];
                r.total_draws = w[0] / 255;
                r.total_bins = (uint64_t)upx;
                r.passes_per_thread = (double)w[3] * b->opts.passes_per_item;
                r.draw_count = w[1];
                r.status = (w[0] >= target ? 1u : 0u) | tr.status;
                per_unit[u] = r;
            }
            px += (uint64_t)upx;
            hits += w[0];
            tr.draw_count += w[1];
            reached += (w[0] >= target) ? 1 : 0;
        }
        tr.total_bins = px;
        tr.total_draws = hits / 255;
        tr.quality = px ? (double)hits / (255.0 * (double)px) : 0.0;
        tr.passes_per_thread = (double)c[1] / ((double)b->k->grid * b->k->block);
        if (reached == nu) tr.status |= 1u;
        if (total) *total = tr;
    });
}

void* rfk_batch_bins(rfk_batch* b, size_t unit) {
    if (!b || unit >= b->units.size()) return nullptr;
    return b->d_bins + b->px_off[unit];
}

void* rfk_batch_image(rfk_batch* b, size_t unit) {
    if (!b || unit >= b->units.size() || !b->d_img) return nullptr;
    return b->d_img + b->img_off[unit];
}

void* rfk_batch_params(rfk_batch* b, size_t unit) {
    if (!b || unit >= b->units.size()) return nullptr;
    return b->d_params + unit * b->k->sample_floats;
}

rfk_status rfk_batch_get_info(const rfk_batch* b, rfk_batch_info* info) {
    return guard([&] {
        if (!b || !info) fail(RFK_E_INVALID, "null argument");
        info->units = b->units.size();
        info->items = b->nitems;
        info->hist_bytes = b->total_px * sizeof(float4);
        info->image_bytes = b->img_bytes;
        info->launches_per_run = b->launches;
        info->graph = b->exec ? 1 : 0;
    });
}

}  // extern "C"
