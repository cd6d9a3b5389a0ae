// Learned denoiser: a 4-level U-Net (32 / 64 / 128 / 256 channels, 3x3
// convolutions, ReLU, 2x2 average pooling, nearest upsampling with skip
// concatenations) that maps the histogram of a low-spp render to the
// tonemapped image of a converged one. bf16 activations and weights, f32
// accumulation (TMEM) and f32 master weights; every convolution - forward,
// input gradient and weight gradient - runs on the tcgen05 kernels of
// unet_tc.cu, the layers between them on unet_ops.cu, Adam on the device.
//
// The reference's denoiser interface (src/librefrakt/include/librefrakt/
// interface/denoiser.h:21-39) takes an image and returns an image through
// closed denoisers; this one takes the histogram (density, colour, alpha and
// spp as input channels) and the low-spp render's tonemapped image (the plain
// path's result, "base"), and predicts a correction of it: prediction =
// base + network output, so an untrained network starts from the plain image.
// The result comes out in the tonemapper's formats.
//
// Channel layout per level (H x W at level 1, halved per level):
//   L1  x 32 (9 live), a1 32, cat1 96 = [up(d2) 64 | s1 32], e1 32, d1 32, out f32 32 (3 live)
//   L2  p1 32, a2 64, cat2 192 = [up(d3) 128 | s2 64], e2 64, d2 64
//   L3  p2 64, a3 128, cat3 384 = [up(b2) 256 | s3 128], e3 128, d3 128
//   L4  p3 128, b1 256, b2 256
// s_l (the skip activations) are written straight into their concatenation.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <random>
#include <tuple>
#include <vector>

#include "../../../include/rfk_denoise.h"
#include "../kernels/unet_kernels.h"
#include "runtime_internal.h"

using namespace rfk::rt;

namespace {

using bf16 = __nv_bfloat16;

enum { L_IN, E1B, E2A, E2B, E3A, E3B, B1, B2, D3A, D3B, D2A, D2B, D1A, D1B, L_OUT, NLAYERS };

struct layer_def {
    int cin, cout, live_in, live_out;
};
constexpr layer_def kLayers[NLAYERS] = {
    {32, 32, 9, 32},    {32, 32, 32, 32},    {32, 64, 32, 64},    {64, 64, 64, 64},   {64, 128, 64, 128},
    {128, 128, 128, 128}, {128, 256, 128, 256}, {256, 256, 256, 256}, {384, 128, 384, 128}, {128, 128, 128, 128},
    {192, 64, 192, 64}, {64, 64, 64, 64},    {96, 32, 96, 32},    {32, 32, 32, 32},   {32, 32, 32, 3},
};

template <typename T>
T* dalloc(size_t count) {
    void* p = nullptr;
    cuda_check(cudaMalloc(&p, std::max<size_t>(count * sizeof(T), 64)), "cudaMalloc (denoiser)");
    return static_cast<T*>(p);
}

struct layer {
    layer_def d{};
    float *w = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
    float *b = nullptr, *bm = nullptr, *bv = nullptr, *bg = nullptr;
    bf16 *wf = nullptr, *wb = nullptr;
    size_t nw() const { return (size_t)d.cout * 9 * d.cin; }
};

// Activations and gradients of one (batch, height, width).
struct workspace {
    int n = 0, h = 0, w = 0;
    bool train = false;
    std::vector<void*> owned;
    bf16 *x, *a1, *cat1, *e1, *d1;
    float* out;
    bf16 *p1, *a2, *cat2, *e2, *d2;
    bf16 *p2, *a3, *cat3, *e3, *d3;
    bf16 *p3, *b1, *b2;
    // training only
    bf16 *g_out, *gl1a, *gl1b, *g_cat1;
    bf16 *gl2a, *gl2b, *g_cat2, *g_p1;
    bf16 *gl3a, *gl3b, *g_cat3, *g_p2;
    bf16 *gl4a, *gl4b, *g_p3;
    float4* target_scratch = nullptr;
    ~workspace() {
        for (void* p : owned) cudaFree(p);
    }
    template <typename T>
    T* take(size_t count) {
        T* p = dalloc<T>(count);
        owned.push_back(p);
        return p;
    }
};

}  // namespace

struct rfk_denoiser {
    layer L[NLAYERS];
    int step = 0;
    int* d_err = nullptr;
    double* d_loss = nullptr;
    std::map<std::tuple<int, int, int, bool>, std::unique_ptr<workspace>> ws;

    ~rfk_denoiser() {
        for (auto& l : L)
            for (void* p : {(void*)l.w, (void*)l.m, (void*)l.v, (void*)l.g, (void*)l.b, (void*)l.bm, (void*)l.bv,
                            (void*)l.bg, (void*)l.wf, (void*)l.wb})
                if (p) cudaFree(p);
        if (d_err) cudaFree(d_err);
        if (d_loss) cudaFree(d_loss);
    }

    workspace& get_ws(int n, int h, int w, bool train) {
        auto key = std::make_tuple(n, h, w, train);
        auto it = ws.find(key);
        if (it != ws.end()) return *it->second;
        auto s = std::make_unique<workspace>();
        s->n = n;
        s->h = h;
        s->w = w;
        s->train = train;
        const size_t P1 = (size_t)n * h * w, P2 = P1 / 4, P3 = P1 / 16, P4 = P1 / 64;
        s->x = s->take<bf16>(P1 * 32);
        s->a1 = s->take<bf16>(P1 * 32);
        s->cat1 = s->take<bf16>(P1 * 96);
        s->e1 = s->take<bf16>(P1 * 32);
        s->d1 = s->take<bf16>(P1 * 32);
        s->out = s->take<float>(P1 * 32);
        s->p1 = s->take<bf16>(P2 * 32);
        s->a2 = s->take<bf16>(P2 * 64);
        s->cat2 = s->take<bf16>(P2 * 192);
        s->e2 = s->take<bf16>(P2 * 64);
        s->d2 = s->take<bf16>(P2 * 64);
        s->p2 = s->take<bf16>(P3 * 64);
        s->a3 = s->take<bf16>(P3 * 128);
        s->cat3 = s->take<bf16>(P3 * 384);
        s->e3 = s->take<bf16>(P3 * 128);
        s->d3 = s->take<bf16>(P3 * 128);
        s->p3 = s->take<bf16>(P4 * 128);
        s->b1 = s->take<bf16>(P4 * 256);
        s->b2 = s->take<bf16>(P4 * 256);
        if (train) {
            s->g_out = s->take<bf16>(P1 * 32);
            s->gl1a = s->take<bf16>(P1 * 32);
            s->gl1b = s->take<bf16>(P1 * 32);
            s->g_cat1 = s->take<bf16>(P1 * 96);
            s->gl2a = s->take<bf16>(P2 * 64);
            s->gl2b = s->take<bf16>(P2 * 64);
            s->g_cat2 = s->take<bf16>(P2 * 192);
            s->g_p1 = s->take<bf16>(P2 * 32);
            s->gl3a = s->take<bf16>(P3 * 128);
            s->gl3b = s->take<bf16>(P3 * 128);
            s->g_cat3 = s->take<bf16>(P3 * 384);
            s->g_p2 = s->take<bf16>(P3 * 64);
            s->gl4a = s->take<bf16>(P4 * 256);
            s->gl4b = s->take<bf16>(P4 * 256);
            s->g_p3 = s->take<bf16>(P4 * 128);
        }
        workspace& r = *s;
        ws[key] = std::move(s);
        return r;
    }

    void conv(int l, const bf16* in, int h, int w, int n, int in_cstride, int in_coff, void* out, int out_cstride,
              int out_coff, int flags, cudaStream_t st) {
        const layer& y = L[l];
        cuda_check(rfk_unet_conv3x3(in, n, h, w, in_cstride, in_coff, y.d.cin, y.wf, y.d.cout, y.b, flags, out, out_cstride,
                                    out_coff, nullptr, 0, 0, 0, d_err, st),
                   "conv");
    }

    // Forward pass of the whole network on ws.x; the result in ws.out. For
    // inference (`infer`) the last convolution of each decoder level and of
    // the bottleneck writes its output straight into the next level's
    // concatenation at twice the resolution (the upsampling fused into its
    // epilogue); training keeps the low-resolution activations, which the
    // backward pass reads, and upsamples them in a pass of its own.
    void forward(workspace& s, cudaStream_t st, bool infer = false) {
        const int n = s.n, H = s.h, W = s.w;
        const int H2 = H / 2, W2 = W / 2, H3 = H / 4, W3 = W / 4, H4 = H / 8, W4 = W / 8;
        const int R = RFK_UNET_RELU;
        conv(L_IN, s.x, H, W, n, 32, 0, s.a1, 32, 0, R, st);
        conv(E1B, s.a1, H, W, n, 32, 0, s.cat1, 96, 64, R, st);
        cuda_check(rfk_unet_avgpool(s.cat1, n, H, W, 96, 64, 32, s.p1, st), "pool");
        conv(E2A, s.p1, H2, W2, n, 32, 0, s.a2, 64, 0, R, st);
        conv(E2B, s.a2, H2, W2, n, 64, 0, s.cat2, 192, 128, R, st);
        cuda_check(rfk_unet_avgpool(s.cat2, n, H2, W2, 192, 128, 64, s.p2, st), "pool");
        conv(E3A, s.p2, H3, W3, n, 64, 0, s.a3, 128, 0, R, st);
        conv(E3B, s.a3, H3, W3, n, 128, 0, s.cat3, 384, 256, R, st);
        cuda_check(rfk_unet_avgpool(s.cat3, n, H3, W3, 384, 256, 128, s.p3, st), "pool");
        conv(B1, s.p3, H4, W4, n, 128, 0, s.b1, 256, 0, R, st);
        const int U = R | RFK_UNET_UP2;
        if (infer) {
            conv(B2, s.b1, H4, W4, n, 256, 0, s.cat3, 384, 0, U, st);
        } else {
            conv(B2, s.b1, H4, W4, n, 256, 0, s.b2, 256, 0, R, st);
            cuda_check(rfk_unet_upsample(s.b2, n, H4, W4, 256, s.cat3, 384, 0, st), "upsample");
        }
        conv(D3A, s.cat3, H3, W3, n, 384, 0, s.e3, 128, 0, R, st);
        if (infer) {
            conv(D3B, s.e3, H3, W3, n, 128, 0, s.cat2, 192, 0, U, st);
        } else {
            conv(D3B, s.e3, H3, W3, n, 128, 0, s.d3, 128, 0, R, st);
            cuda_check(rfk_unet_upsample(s.d3, n, H3, W3, 128, s.cat2, 192, 0, st), "upsample");
        }
        conv(D2A, s.cat2, H2, W2, n, 192, 0, s.e2, 64, 0, R, st);
        if (infer) {
            conv(D2B, s.e2, H2, W2, n, 64, 0, s.cat1, 96, 0, U, st);
        } else {
            conv(D2B, s.e2, H2, W2, n, 64, 0, s.d2, 64, 0, R, st);
            cuda_check(rfk_unet_upsample(s.d2, n, H2, W2, 64, s.cat1, 96, 0, st), "upsample");
        }
        conv(D1A, s.cat1, H, W, n, 96, 0, s.e1, 32, 0, R, st);
        conv(D1B, s.e1, H, W, n, 32, 0, s.d1, 32, 0, R, st);
        conv(L_OUT, s.d1, H, W, n, 32, 0, s.out, 32, 0, RFK_UNET_F32OUT, st);
    }

    // Gradients of layer l from dY (dense, cout channels, pre-activation) and
    // its input X (a channel slice); dX (optional) into a slice, times
    // (mask > 0) when a mask is given.
    void back(workspace& s, int l, const bf16* dy, int n, int h, int w, const bf16* x, int x_cstride, int x_coff, bf16* dx,
              int dx_cstride, int dx_coff, const bf16* mask, cudaStream_t st) {
        const layer& y = L[l];
        const size_t P = (size_t)n * h * w;
        cuda_check(rfk_unet_bias_grad(dy, P, y.d.cout, y.bg, st), "bias grad");
        cuda_check(rfk_unet_wgrad3x3(dy, x, x_cstride, x_coff, n, h, w, y.d.cout, y.d.cin, y.g, d_err, st), "wgrad");
        if (dx)
            cuda_check(rfk_unet_conv3x3(dy, n, h, w, y.d.cout, 0, y.d.cout, y.wb, y.d.cin, nullptr, 0, dx, dx_cstride, dx_coff,
                                        mask, y.d.cin, 0, 0, d_err, st),
                       "dgrad");
    }

    void backward(workspace& s, cudaStream_t st) {
        const int n = s.n, H = s.h, W = s.w;
        const int H2 = H / 2, W2 = W / 2, H3 = H / 4, W3 = W / 4, H4 = H / 8, W4 = W / 8;
        for (auto& y : L) {
            cuda_check(cudaMemsetAsync(y.g, 0, y.nw() * sizeof(float), st), "zero grads");
            cuda_check(cudaMemsetAsync(y.bg, 0, y.d.cout * sizeof(float), st), "zero grads");
        }
        // level 1, decoder side
        back(s, L_OUT, s.g_out, n, H, W, s.d1, 32, 0, s.gl1a, 32, 0, s.d1, st);     // gl1a = gp_d1
        back(s, D1B, s.gl1a, n, H, W, s.e1, 32, 0, s.gl1b, 32, 0, s.e1, st);        // gl1b = gp_e1
        back(s, D1A, s.gl1b, n, H, W, s.cat1, 96, 0, s.g_cat1, 96, 0, nullptr, st);
        // level 2
        cuda_check(rfk_unet_up_backward(s.g_cat1, 96, 0, s.d2, n, H2, W2, 64, s.gl2a, st), "up backward");
        back(s, D2B, s.gl2a, n, H2, W2, s.e2, 64, 0, s.gl2b, 64, 0, s.e2, st);
        back(s, D2A, s.gl2b, n, H2, W2, s.cat2, 192, 0, s.g_cat2, 192, 0, nullptr, st);
        // level 3
        cuda_check(rfk_unet_up_backward(s.g_cat2, 192, 0, s.d3, n, H3, W3, 128, s.gl3a, st), "up backward");
        back(s, D3B, s.gl3a, n, H3, W3, s.e3, 128, 0, s.gl3b, 128, 0, s.e3, st);
        back(s, D3A, s.gl3b, n, H3, W3, s.cat3, 384, 0, s.g_cat3, 384, 0, nullptr, st);
        // bottleneck
        cuda_check(rfk_unet_up_backward(s.g_cat3, 384, 0, s.b2, n, H4, W4, 256, s.gl4a, st), "up backward");
        back(s, B2, s.gl4a, n, H4, W4, s.b1, 256, 0, s.gl4b, 256, 0, s.b1, st);
        back(s, B1, s.gl4b, n, H4, W4, s.p3, 128, 0, s.g_p3, 128, 0, nullptr, st);
        // encoder
        cuda_check(rfk_unet_skip_backward(s.g_cat3, 384, 256, s.g_p3, s.cat3, n, H3, W3, 128, s.gl3a, st), "skip");
        back(s, E3B, s.gl3a, n, H3, W3, s.a3, 128, 0, s.gl3b, 128, 0, s.a3, st);
        back(s, E3A, s.gl3b, n, H3, W3, s.p2, 64, 0, s.g_p2, 64, 0, nullptr, st);
        cuda_check(rfk_unet_skip_backward(s.g_cat2, 192, 128, s.g_p2, s.cat2, n, H2, W2, 64, s.gl2a, st), "skip");
        back(s, E2B, s.gl2a, n, H2, W2, s.a2, 64, 0, s.gl2b, 64, 0, s.a2, st);
        back(s, E2A, s.gl2b, n, H2, W2, s.p1, 32, 0, s.g_p1, 32, 0, nullptr, st);
        cuda_check(rfk_unet_skip_backward(s.g_cat1, 96, 64, s.g_p1, s.cat1, n, H, W, 32, s.gl1a, st), "skip");
        back(s, E1B, s.gl1a, n, H, W, s.a1, 32, 0, s.gl1b, 32, 0, s.a1, st);
        back(s, L_IN, s.gl1b, n, H, W, s.x, 32, 0, nullptr, 0, 0, nullptr, st);
    }

    void adam(float lr, cudaStream_t st) {
        step++;
        for (auto& y : L)
            cuda_check(rfk_unet_adam(y.w, y.m, y.v, y.g, y.d.cout, y.d.cin, y.d.live_out, y.d.live_in, lr, 0.9f, 0.999f,
                                     1e-8f, step, y.wf, y.wb, y.b, y.bm, y.bv, y.bg, st),
                       "adam");
    }

    // Writes the bf16 copies of the current master weights (Adam with lr 0).
    void sync_copies(cudaStream_t st) {
        for (auto& y : L) {
            cuda_check(cudaMemsetAsync(y.g, 0, y.nw() * sizeof(float), st), "zero");
            cuda_check(cudaMemsetAsync(y.bg, 0, y.d.cout * sizeof(float), st), "zero");
            cuda_check(rfk_unet_adam(y.w, y.m, y.v, y.g, y.d.cout, y.d.cin, y.d.live_out, y.d.live_in, 0.0f, 0.9f, 0.999f,
                                     1e-8f, 1, y.wf, y.wb, y.b, y.bm, y.bv, y.bg, st),
                       "weights");
        }
    }

    void check_err(cudaStream_t st) {
        int e = 0;
        cuda_check(cudaMemcpyAsync(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H");
        cuda_check(cudaStreamSynchronize(st), "denoiser");
        if (e) {
            cudaMemsetAsync(d_err, 0, sizeof(int), st);
            fail(RFK_E_CUDA, "a tensor-core kernel's pipeline wait ran out of time");
        }
    }
};

namespace {
void check_dims(uint32_t n, uint32_t w, uint32_t h, bool train) {
    if (n == 0 || w == 0 || h == 0) fail(RFK_E_INVALID, "empty batch");
    if (w % 8 || h % 8) fail(RFK_E_INVALID, "width and height must be multiples of 8 (three 2x2 poolings)");
    if (train && w % 512) fail(RFK_E_INVALID, "training width must be a multiple of 512 (weight-gradient tiles)");
    if ((uint64_t)n * w * h > (1ull << 31)) fail(RFK_E_INVALID, "batch too large");
}
}  // namespace

extern "C" {

namespace {
const char* const kDenoiserNames[] = {"rfkt::gb300_unet_denoiser"};
}  // namespace

rfk_status rfk_denoiser_name(int index, char* buf, size_t cap) {
    return guard([&] {
        if (index < 0 || index >= (int)(sizeof kDenoiserNames / sizeof kDenoiserNames[0]))
            fail(RFK_E_INVALID, "no denoiser with that index");
        if (!buf || cap == 0) fail(RFK_E_INVALID, "null buffer");
        std::snprintf(buf, cap, "%s", kDenoiserNames[index]);
    });
}

rfk_status rfk_denoiser_make(const char* name, const char* weights_path, rfk_denoiser** out) {
    if (out) *out = nullptr;
    if (!name || !out) return guard([] { fail(RFK_E_INVALID, "null argument"); });
    if (std::strcmp(name, kDenoiserNames[0]) != 0)
        return guard([&] { fail(RFK_E_INVALID, std::string("unknown denoiser '") + name + "'"); });
    std::vector<float> params;
    if (weights_path) {
        size_t n = 0;
        if (rfk_status r = rfk_denoiser_read_params(weights_path, nullptr, 0, &n)) return r;
        params.resize(n);
        if (rfk_status r = rfk_denoiser_read_params(weights_path, params.data(), n, &n)) return r;
    }
    rfk_denoiser* d = nullptr;
    if (rfk_status r = rfk_denoiser_create(0, &d)) return r;
    if (weights_path) {
        if (rfk_status r = rfk_denoiser_set_params(d, params.data(), params.size())) {
            rfk_denoiser_destroy(d);
            return r;
        }
    }
    *out = d;
    return RFK_OK;
}

rfk_status rfk_denoiser_create(uint64_t seed, rfk_denoiser** out) {
    return guard([&] {
        if (!out) fail(RFK_E_INVALID, "null argument");
        auto d = std::make_unique<rfk_denoiser>();
        std::mt19937_64 rng(seed);
        for (int l = 0; l < NLAYERS; l++) {
            layer& y = d->L[l];
            y.d = kLayers[l];
            const size_t nw = y.nw();
            y.w = dalloc<float>(nw);
            y.m = dalloc<float>(nw);
            y.v = dalloc<float>(nw);
            y.g = dalloc<float>(nw);
            y.b = dalloc<float>(y.d.cout);
            y.bm = dalloc<float>(y.d.cout);
            y.bv = dalloc<float>(y.d.cout);
            y.bg = dalloc<float>(y.d.cout);
            y.wf = dalloc<bf16>(nw);
            y.wb = dalloc<bf16>(nw);
            // He initialisation over the live fan-in; the output layer (a
            // correction of the base image) starts near zero
            const double sd = (l == L_OUT) ? 0.1 * std::sqrt(1.0 / (9.0 * y.d.live_in)) : std::sqrt(2.0 / (9.0 * y.d.live_in));
            std::normal_distribution<double> nd(0.0, sd);
            std::vector<float> w(nw, 0.0f);
            for (int co = 0; co < y.d.live_out; co++)
                for (int t = 0; t < 9; t++)
                    for (int ci = 0; ci < y.d.live_in; ci++) w[((size_t)co * 9 + t) * y.d.cin + ci] = (float)nd(rng);
            cuda_check(cudaMemcpy(y.w, w.data(), nw * sizeof(float), cudaMemcpyHostToDevice), "H2D weights");
            for (float* p : {y.m, y.v}) cuda_check(cudaMemset(p, 0, nw * sizeof(float)), "zero");
            for (float* p : {y.b, y.bm, y.bv}) cuda_check(cudaMemset(p, 0, y.d.cout * sizeof(float)), "zero");
        }
        d->d_err = dalloc<int>(1);
        d->d_loss = dalloc<double>(1);
        cuda_check(cudaMemset(d->d_err, 0, sizeof(int)), "zero");
        d->sync_copies(nullptr);
        cuda_check(cudaDeviceSynchronize(), "init");
        *out = d.release();
    });
}

void rfk_denoiser_destroy(rfk_denoiser* d) { delete d; }

size_t rfk_denoiser_param_count(const rfk_denoiser* d) {
    if (!d) return 0;
    size_t n = 0;
    for (auto& y : d->L) n += y.nw() + y.d.cout;
    return n;
}

rfk_status rfk_denoiser_get_params(const rfk_denoiser* d, float* out, size_t n) {
    return guard([&] {
        if (!d || !out) fail(RFK_E_INVALID, "null argument");
        if (n < rfk_denoiser_param_count(d)) fail(RFK_E_INVALID, "parameter buffer too small");
        cuda_check(cudaDeviceSynchronize(), "sync");
        size_t o = 0;
        for (auto& y : d->L) {
            cuda_check(cudaMemcpy(out + o, y.w, y.nw() * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
            o += y.nw();
            cuda_check(cudaMemcpy(out + o, y.b, y.d.cout * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
            o += y.d.cout;
        }
    });
}

rfk_status rfk_denoiser_set_params(rfk_denoiser* d, const float* in, size_t n) {
    return guard([&] {
        if (!d || !in) fail(RFK_E_INVALID, "null argument");
        if (n != rfk_denoiser_param_count(d)) fail(RFK_E_INVALID, "parameter count mismatch");
        size_t o = 0;
        for (auto& y : d->L) {
            cuda_check(cudaMemcpy(y.w, in + o, y.nw() * sizeof(float), cudaMemcpyHostToDevice), "H2D");
            o += y.nw();
            cuda_check(cudaMemcpy(y.b, in + o, y.d.cout * sizeof(float), cudaMemcpyHostToDevice), "H2D");
            o += y.d.cout;
        }
        d->sync_copies(nullptr);
        cuda_check(cudaDeviceSynchronize(), "set params");
    });
}

rfk_status rfk_denoiser_features(const float* bins, const float* base, uint32_t w, uint32_t h, double spp, void* out,
                                 void* stream) {
    return guard([&] {
        if (!bins || !base || !out) fail(RFK_E_INVALID, "null argument");
        cuda_check(rfk_unet_features(reinterpret_cast<const float4*>(bins), reinterpret_cast<const float4*>(base),
                                     (size_t)w * h, (float)spp, out, (cudaStream_t)stream),
                   "features");
    });
}

rfk_status rfk_denoiser_train_step(rfk_denoiser* d, const float* bins, const float* base, uint32_t n, uint32_t w, uint32_t h, double spp,
                                   const float* targets, float lr, double* loss, void* stream) {
    return guard([&] {
        if (!d || !bins || !base || !targets) fail(RFK_E_INVALID, "null argument");
        check_dims(n, w, h, true);
        cudaStream_t st = (cudaStream_t)stream;
        workspace& s = d->get_ws((int)n, (int)h, (int)w, true);
        const size_t P = (size_t)n * w * h;
        cuda_check(rfk_unet_features(reinterpret_cast<const float4*>(bins), reinterpret_cast<const float4*>(base), P,
                                     (float)spp, s.x, st),
                   "features");
        d->forward(s, st);
        cuda_check(cudaMemsetAsync(d->d_loss, 0, sizeof(double), st), "zero");
        cuda_check(rfk_unet_mse(s.out, reinterpret_cast<const float4*>(base), reinterpret_cast<const float4*>(targets), P,
                                s.g_out, d->d_loss, st),
                   "loss");
        d->backward(s, st);
        d->adam(lr, st);
        double l = 0.0;
        cuda_check(cudaMemcpyAsync(&l, d->d_loss, sizeof(double), cudaMemcpyDeviceToHost, st), "D2H loss");
        d->check_err(st);
        if (loss) *loss = l / (3.0 * (double)P);
    });
}

rfk_status rfk_denoiser_loss(rfk_denoiser* d, const float* bins, const float* base, uint32_t n, uint32_t w, uint32_t h, double spp,
                             const float* targets, double* loss, void* stream) {
    return guard([&] {
        if (!d || !bins || !base || !targets || !loss) fail(RFK_E_INVALID, "null argument");
        check_dims(n, w, h, false);
        cudaStream_t st = (cudaStream_t)stream;
        workspace& s = d->get_ws((int)n, (int)h, (int)w, true);
        const size_t P = (size_t)n * w * h;
        cuda_check(rfk_unet_features(reinterpret_cast<const float4*>(bins), reinterpret_cast<const float4*>(base), P,
                                     (float)spp, s.x, st),
                   "features");
        d->forward(s, st);
        cuda_check(cudaMemsetAsync(d->d_loss, 0, sizeof(double), st), "zero");
        cuda_check(rfk_unet_mse(s.out, reinterpret_cast<const float4*>(base), reinterpret_cast<const float4*>(targets), P,
                                s.g_out, d->d_loss, st),
                   "loss");
        double l = 0.0;
        cuda_check(cudaMemcpyAsync(&l, d->d_loss, sizeof(double), cudaMemcpyDeviceToHost, st), "D2H loss");
        d->check_err(st);
        *loss = l / (3.0 * (double)P);
    });
}

rfk_status rfk_denoiser_gradients(rfk_denoiser* d, const float* bins, const float* base, uint32_t n, uint32_t w, uint32_t h, double spp,
                                  const float* targets, float* grads, size_t count, void* stream) {
    return guard([&] {
        if (!d || !bins || !base || !targets || !grads) fail(RFK_E_INVALID, "null argument");
        if (count < rfk_denoiser_param_count(d)) fail(RFK_E_INVALID, "gradient buffer too small");
        check_dims(n, w, h, true);
        cudaStream_t st = (cudaStream_t)stream;
        workspace& s = d->get_ws((int)n, (int)h, (int)w, true);
        const size_t P = (size_t)n * w * h;
        cuda_check(rfk_unet_features(reinterpret_cast<const float4*>(bins), reinterpret_cast<const float4*>(base), P,
                                     (float)spp, s.x, st),
                   "features");
        d->forward(s, st);
        cuda_check(cudaMemsetAsync(d->d_loss, 0, sizeof(double), st), "zero");
        cuda_check(rfk_unet_mse(s.out, reinterpret_cast<const float4*>(base), reinterpret_cast<const float4*>(targets), P,
                                s.g_out, d->d_loss, st),
                   "loss");
        d->backward(s, st);
        d->check_err(st);
        size_t o = 0;
        for (auto& y : d->L) {
            cuda_check(cudaMemcpy(grads + o, y.g, y.nw() * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
            o += y.nw();
            cuda_check(cudaMemcpy(grads + o, y.bg, y.d.cout * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
            o += y.d.cout;
        }
    });
}

rfk_status rfk_denoise(rfk_denoiser* d, const float* bins, const float* base, uint32_t w, uint32_t h, double spp, void* out,
                       int format, void* stream) {
    return guard([&] {
        if (!d || !bins || !base || !out) fail(RFK_E_INVALID, "null argument");
        if (format < 0 || format > 3) fail(RFK_E_INVALID, "bad output format");
        check_dims(1, w, h, false);
        cudaStream_t st = (cudaStream_t)stream;
        workspace& s = d->get_ws(1, (int)h, (int)w, false);
        const size_t P = (size_t)w * h;
        cuda_check(rfk_unet_features(reinterpret_cast<const float4*>(bins), reinterpret_cast<const float4*>(base), P,
                                     (float)spp, s.x, st),
                   "features");
        d->forward(s, st, true);
        cuda_check(rfk_unet_to_image(s.out, reinterpret_cast<const float4*>(base), reinterpret_cast<const float4*>(bins), P,
                                     out, format, st),
                   "to image");
        d->check_err(st);
    });
}

}  // extern "C"
