// Tensor-core kernels of the learned denoiser: 3x3 convolutions (stride 1,
// zero padding 1) of bf16 NHWC activations as implicit GEMMs on tcgen05, with
// f32 accumulators in TMEM.
//
// conv3x3_tc (forward and input-gradient): persistent CTAs walk tiles of R
// image rows x 128 output pixels x BN output channels.
//   D[p, n] = sum over taps t and input channels c of A[p + t, c] * W[n, t, c]
// The K loop runs over input channel blocks of BK and, depending on MODE
// (conv_cfg), over taps, tap rows or neither: the A tile of a K block is a
// TMA box of the NHWC input at the tile's offset - the padding comes from
// TMA's zero fill outside the image - and the B tiles boxes (BK x BN) of the
// weights [cout][9][cin]. A producer warp (one lane) issues the TMA loads into
// a ring of shared-memory stages, an MMA warp (one lane) issues tcgen05.mma
// (M 128, N BN, K 16 per instruction) and frees each stage with
// tcgen05.commit; eight epilogue warps read the accumulator rows from TMEM
// (two per lane quarter) and apply the epilogue: bias, ReLU, a
// ReLU-derivative mask, accumulation into the output, bf16 or f32 store.
// The input gradient of a conv is the same kernel on the output gradient with
// the weights transposed and the taps flipped ([cin][9][cout]).
//
// wgrad3x3_tc (weight gradient): dW[n, t, c] = sum over pixels p of
// dY[p, n] * X[p + t, c], a GEMM with M = cout (up to 128 per tile), N = BN
// input channels, K = pixels; a K block is 64 pixels of one image row (W a
// multiple of 64). A is K-major from a channel-major copy of dY; B is read
// MN-major straight from the NHWC input: boxes of 32 or 64 channels x 64
// pixels at the tap's offset, the column offset dx being a pixel coordinate
// (not the innermost one, so any value is fine; zero fill outside the image).
// CTAs split K and add their partial sums into dW (f32) atomically.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "tc_ptx.cuh"
#include "unet_kernels.h"

namespace {

using bf16 = __nv_bfloat16;

// ------------------------------------------------------------------ conv ----
struct conv_args {
    int n_img, h, w, tiles_x;
    int cin, cin_off;  // K channels and their offset in the input tensor
    int cout;
    void* out;
    int out_cstride, out_coff;
    const float* bias;
    int relu;
    int out_f32;  // store f32 instead of bf16
    int up2;      // store at the 2x2 pixels of a (2h, 2w) output
    const bf16* mask;
    int mask_cstride, mask_coff;
    int accumulate;
    int* err;
};

// Tap reuse. MODE 0: one K block per (tap, input channel block), its A box
// the 128 pixels of each tile row shifted by the tap. MODE 1 (column taps): a
// K block covers one tap row dy and the three column taps; its A box holds
// 136 pixels of each image row from x0 - 1 on (130 used; 136 keeps every row
// 1024-byte aligned for 128-byte swizzle and 512-byte aligned for 64-byte
// swizzle) and the MMAs of column tap dx read it through a descriptor that
// starts dx pixel lines later. MODE 2 (all taps): a K block covers all nine
// taps of one input channel block; its A box holds the tile's R rows plus the
// row above and below (R + 2 rows of 136 pixels) and the MMAs of tap (dy, dx)
// start at row r + dy, pixel line dx; the layer's weights (up to three input
// channel blocks x nine taps, one output tile) are loaded once per CTA and
// stay in shared memory, so the stages carry only the input. The input
// crosses L2 nine, three or (R + 2) / R times per layer.
template <int BK, int BN, int MODE>
struct conv_cfg {
    // R image rows per tile (R accumulators of 128 x BN): small-N layers move
    // R times the bytes per pipeline stage, so the stage round trip is shared
    static constexpr int R = BN >= 128 ? 1 : 128 / BN;
    static constexpr int A_PIX = MODE ? 136 : 128;                // pixel lines per image row
    static constexpr int A_ROWS = MODE == 2 ? R + 2 : R;           // image rows per A box
    static constexpr uint32_t A_ROW = (uint32_t)A_PIX * BK * 2u;   // one image row segment
    static constexpr uint32_t A_BYTES = A_ROWS * A_ROW;
    static constexpr int NT = MODE == 2 ? 9 : (MODE == 1 ? 3 : 1);  // taps per K block
    static constexpr int NB = MODE == 2 ? 0 : NT;                    // weight tiles per stage
    static constexpr uint32_t B_TILE = (uint32_t)BN * BK * 2u;
    static constexpr int KB_RES = 3;                                 // resident input channel blocks (MODE 2)
    static constexpr uint32_t B_RES = MODE == 2 ? KB_RES * 9u * B_TILE : 0u;
    static constexpr uint32_t LOAD_BYTES = A_BYTES + NB * B_TILE;  // bytes the TMA writes per stage
    static constexpr uint32_t STAGE_BYTES = (LOAD_BYTES + 1023u) & ~1023u;
    static constexpr int TAPS = MODE == 2 ? 1 : (MODE == 1 ? 3 : 9);  // K blocks per input channel block
    // one persistent CTA per SM: as many stages as fit in ~208 KB, at most 8
    static constexpr uint32_t BUDGET = 212992u;
    static constexpr int STAGES = ((BUDGET - B_RES) / STAGE_BYTES > 8) ? 8 : (int)((BUDGET - B_RES) / STAGE_BYTES);
    static constexpr uint32_t SMEM = B_RES + STAGES * STAGE_BYTES + 1024u;
    static constexpr uint32_t TMEM_COLS = 2u * R * BN;  // two sets of R accumulators
    static_assert(MODE == 0 || (A_ROW % 512u == 0 && A_BYTES % 1024u == 0 && B_TILE % 1024u == 0 && B_RES % 1024u == 0),
                  "tap-reuse tiles must stay swizzle-aligned");
    static_assert(STAGES >= 2, "at least two stages");
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void store_bf16x16(bf16* dst, const float (&v)[16]) {
    uint4* d = reinterpret_cast<uint4*>(dst);
#pragma unroll
    for (int q = 0; q < 2; q++) {
        __nv_bfloat162 h[4];
#pragma unroll
        for (int j = 0; j < 4; j++) h[j] = __floats2bfloat162_rn(v[8 * q + 2 * j], v[8 * q + 2 * j + 1]);
        d[q] = *reinterpret_cast<uint4*>(h);
    }
}

__device__ __forceinline__ void load_bf16x16(const bf16* src, float (&v)[16]) {
    const uint4* s = reinterpret_cast<const uint4*>(src);
#pragma unroll
    for (int q = 0; q < 2; q++) {
        uint4 u = s[q];
        const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            float2 f = __bfloat1622float2(h[j]);
            v[8 * q + 2 * j] = f.x;
            v[8 * q + 2 * j + 1] = f.y;
        }
    }
}

constexpr int kEpiWarps = 8;  // two warps per TMEM lane quarter, each half of the columns

// Persistent: one CTA per SM walks the tiles (R rows x 128-pixel segment x BN
// output channels) t = blockIdx.x, blockIdx.x + gridDim.x, ...
// Warps 0-7: epilogue (warp w reads TMEM lane quarter w % 4, column half
// w / 4), warp 8 lane 0: TMA producer over a ring of stages that runs across
// tiles, warp 9 lane 0: MMA issuer. Two TMEM accumulators: the MMAs of tile
// i + 1 run while the epilogue drains tile i (acc_full / acc_empty barriers).
template <int BK, int BN, int MODE>
__global__ void __launch_bounds__(320, 1) conv3x3_tc(const __grid_constant__ CUtensorMap tmA,
                                                     const __grid_constant__ CUtensorMap tmB, conv_args p) {
    using C = conv_cfg<BK, BN, MODE>;
    extern __shared__ uint8_t smem_dyn[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t full[C::STAGES], empty[C::STAGES], acc_full[2], acc_empty[2], wbar;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t* const res = base;                   // resident weights (MODE 2)
    uint8_t* const stages = base + C::B_RES;

    const int ntn = p.cout / BN;                           // N tiles
    const int rows_t = (p.h + C::R - 1) / C::R;            // row groups per image
    const int ntiles = p.n_img * rows_t * p.tiles_x * ntn;
    const int kpt = p.cin / BK;                            // K blocks per tap
    const int nk = C::TAPS * kpt;

    if (warp == 0) tc::tmem_alloc(&tmem_base, C::TMEM_COLS);
    if (threadIdx.x == 32) {
        for (int s = 0; s < C::STAGES; s++) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], kEpiWarps);  // one arrival per epilogue warp
        }
        tc::mbar_init(&wbar, 1);
        s_fail = 0;
        tc::mbar_fence_init();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == kEpiWarps) {
        if (lane == 0) {
            // producer: the stage ring runs across tiles
            uint32_t g = 0;
            bool ok = true;
            if (MODE == 2) {
                // the layer's weights (one output tile: cout == BN), all taps and input blocks
                tc::mbar_expect_tx(&wbar, (uint32_t)kpt * 9u * C::B_TILE);
                for (int cb = 0; cb < kpt; cb++)
#pragma unroll
                    for (int t9 = 0; t9 < 9; t9++)
                        tc::tma_load_2d(res + (cb * 9 + t9) * C::B_TILE, &tmB, &wbar, t9 * p.cin + cb * BK, 0);
            }
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
                const int mt = t / ntn, n0 = (t - mt * ntn) * BN;
                const int xt = mt % p.tiles_x;
                const int y = ((mt / p.tiles_x) % rows_t) * C::R;
                const int img = mt / (p.tiles_x * rows_t);
                for (int kb = 0; kb < nk; kb++, g++) {
                    const uint32_t s = g % C::STAGES, r = g / C::STAGES;
                    if (r > 0 && !tc::mbar_wait(&empty[s], (r - 1) & 1)) {
                        ok = false;
                        break;
                    }
                    const int tap = kb / kpt, cb = kb - tap * kpt;
                    uint8_t* sa = stages + (size_t)s * C::STAGE_BYTES;
                    tc::mbar_expect_tx(&full[s], C::LOAD_BYTES);
                    if (MODE == 2) {
                        // rows y - 1 .. y + R, pixels x0 - 1 .. x0 + 134 (weights resident)
                        tc::tma_load_4d(sa, &tmA, &full[s], p.cin_off + cb * BK, xt * 128 - 1, y - 1, img);
                    } else if (MODE == 1) {
                        // tap = dy row: pixels x0 - 1 .. x0 + 134, the three column taps' weights
                        tc::tma_load_4d(sa, &tmA, &full[s], p.cin_off + cb * BK, xt * 128 - 1, y + tap - 1, img);
#pragma unroll
                        for (int dx = 0; dx < 3; dx++)
                            tc::tma_load_2d(sa + C::A_BYTES + dx * C::B_TILE, &tmB, &full[s], (tap * 3 + dx) * p.cin + cb * BK,
                                            n0);
                    } else {
                        tc::tma_load_4d(sa, &tmA, &full[s], p.cin_off + cb * BK, xt * 128 + tap % 3 - 1, y + tap / 3 - 1,
                                        img);
                        tc::tma_load_2d(sa + C::A_BYTES, &tmB, &full[s], tap * p.cin + cb * BK, n0);
                    }
                }
            }
            if (!ok) {
                atomicExch(&s_fail, 1);
                // let the copies in flight land before the CTA exits (bounded)
                for (uint32_t q = g >= (uint32_t)C::STAGES ? g - C::STAGES : 0; q < g; q++)
                    tc::mbar_wait(&full[q % C::STAGES], (q / C::STAGES) & 1);
            }
            if (MODE == 2 && !tc::mbar_wait(&wbar, 0)) atomicExch(&s_fail, 1);
        }
    } else if (warp == kEpiWarps + 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_bf16(128, BN);
            uint32_t g = 0;
            bool ok = MODE != 2 || tc::mbar_wait(&wbar, 0);
            const uint32_t sres = tc::smem_u32(res);
            int i = 0;
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x, i++) {
                const int b = i & 1;
                if (i >= 2 && !tc::mbar_wait(&acc_empty[b], ((i >> 1) - 1) & 1)) {
                    ok = false;
                    break;
                }
                tc::fence_after();
                const uint32_t acc = tmem + (uint32_t)(b * C::R * BN);
                for (int kb = 0; kb < nk; kb++, g++) {
                    const uint32_t s = g % C::STAGES;
                    if (!tc::mbar_wait(&full[s], (g / C::STAGES) & 1)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after();
                    const uint32_t sa = tc::smem_u32(stages + (size_t)s * C::STAGE_BYTES);
                    // MODE 2: the resident weights of input block kb, else the stage's
                    const uint32_t sb = MODE == 2 ? sres + (uint32_t)(kb * 9) * C::B_TILE : sa + C::A_BYTES;
                    // descriptors of the stage's first tiles; the others differ only in the
                    // start address field (bits 0-13, 16-byte units; shared memory < 256 KB,
                    // so adding the compile-time offset cannot carry out of it)
                    const uint64_t a0 = tc::smem_desc_at(sa, BK * 2), b0 = tc::smem_desc(sb, BK * 2);
#pragma unroll
                    for (int r = 0; r < C::R; r++)
#pragma unroll
                        for (int t = 0; t < C::NT; t++) {
                            // MODE 2: tap t = (dy, dx) reads row r + dy; MODE 1: t = dx
                            const int dy = MODE == 2 ? t / 3 : 0, dx = MODE == 2 ? t % 3 : t;
#pragma unroll
                            for (int kk = 0; kk < BK / 16; kk++)
                                tc::mma_bf16(acc + (uint32_t)(r * BN),
                                             a0 + (uint64_t)(((r + dy) * C::A_ROW + dx * (BK * 2) + kk * 32) >> 4),
                                             b0 + (uint64_t)((t * C::B_TILE + kk * 32) >> 4), idesc,
                                             (kb | t | kk) != 0 ? 1u : 0u);
                        }
                    tc::mma_commit(&empty[s]);
                }
                tc::mma_commit(&acc_full[b]);  // also on failure: arrives once the issued MMAs are done
            }
            if (!ok) atomicExch(&s_fail, 1);
        }
    } else {
        // epilogue: warps 0-7; TMEM lane 32 * (warp % 4) + lane = tile row,
        // columns [half * BN / 2, (half + 1) * BN / 2)
        const int quarter = warp & 3, half = warp >> 2;
        int i = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
            const int b = i & 1;
            bool got = tc::mbar_wait(&acc_full[b], (i >> 1) & 1);
            got = __all_sync(0xffffffffu, got);
            if (!got) {
                if (lane == 0) atomicExch(&s_fail, 1);
                break;
            }
            tc::fence_after();
            const int mt = t / ntn, n0 = (t - mt * ntn) * BN;
            const int xt = mt % p.tiles_x;
            const int y0 = ((mt / p.tiles_x) % rows_t) * C::R;
            const int img = mt / (p.tiles_x * rows_t);
            const int x = xt * 128 + quarter * 32 + lane;
#pragma unroll 1
            for (int r = 0; r < C::R; r++) {
                const int y = y0 + r;
                const bool valid = x < p.w && y < p.h;
                const size_t pix = ((size_t)img * p.h + (valid ? y : 0)) * p.w + (valid ? x : 0);
#pragma unroll 1
                for (int c = half * (BN / 2); c < (half + 1) * (BN / 2); c += 16) {
                    float v[16];
                    tc::tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((b * C::R + r) * BN + c), v);
                    const int ch = n0 + c;
                    if (!valid) continue;
                    if (p.bias) {
                        const float4* bb = reinterpret_cast<const float4*>(p.bias + ch);
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const float4 f = __ldg(bb + q);
                            v[4 * q] += f.x;
                            v[4 * q + 1] += f.y;
                            v[4 * q + 2] += f.z;
                            v[4 * q + 3] += f.w;
                        }
                    }
                    if (p.relu) {
#pragma unroll
                        for (int j = 0; j < 16; j++) v[j] = fmaxf(v[j], 0.0f);
                    }
                    if (p.mask) {
                        float m[16];
                        load_bf16x16(p.mask + pix * p.mask_cstride + p.mask_coff + ch, m);
#pragma unroll
                        for (int j = 0; j < 16; j++) v[j] = m[j] > 0.0f ? v[j] : 0.0f;
                    }
                    const size_t at = pix * p.out_cstride + p.out_coff + ch;
                    if (p.out_f32) {
                        float4* dst = reinterpret_cast<float4*>(static_cast<float*>(p.out) + at);
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            float4 o = p.accumulate ? dst[q] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                            dst[q] = make_float4(v[4 * q] + o.x, v[4 * q + 1] + o.y, v[4 * q + 2] + o.z, v[4 * q + 3] + o.w);
                        }
                    } else if (p.up2) {
                        // nearest 2x upsampling: the four pixels (2x + dx, 2y + dy) of the
                        // output image, which is (2h, 2w)
#pragma unroll
                        for (int d = 0; d < 4; d++) {
                            const size_t pix2 = ((size_t)img * 2 * p.h + 2 * y + (d >> 1)) * (2 * (size_t)p.w) + 2 * x + (d & 1);
                            store_bf16x16(static_cast<bf16*>(p.out) + pix2 * p.out_cstride + p.out_coff + ch, v);
                        }
                    } else {
                        bf16* dst = static_cast<bf16*>(p.out) + at;
                        if (p.accumulate) {
                            float o[16];
                            load_bf16x16(dst, o);
#pragma unroll
                            for (int j = 0; j < 16; j++) v[j] += o[j];
                        }
                        store_bf16x16(dst, v);
                    }
                }
            }
            // the accumulator may be overwritten once all epilogue warps have read it
            tc::fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[b]);
        }
    }
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && s_fail) atomicExch(p.err, 1);
    if (warp == 0) tc::tmem_dealloc(tmem, C::TMEM_COLS);
}

// ----------------------------------------------------------------- wgrad ----
struct wgrad_args {
    int n_img, h, w;
    int cout, cin;
    int x_coff;     // first input channel in the NHWC tensor of X
    int dx;         // tap column offset of this launch
    int kpc;        // K blocks (64-pixel row segments) per CTA
    int total_kb;   // all row segments
    int a_rows;     // output channels an A box loads (rows of the 128-row A tile; the rest is not read)
    float* dw;      // [cout][9][cin]
    int* err;
};

// DXP (input channel tiles of at most 64): the three column taps share one
// launch as three B blocks of BN channels (X at pixel offsets -1, 0, +1), so
// the MMA's N is 3 BN.
template <int BN, bool DXP>
struct wgrad_cfg {
    static constexpr int NB = DXP ? 3 * BN : BN;  // MMA N
    static constexpr uint32_t A_BYTES = 128u * 64u * 2u;
    static constexpr uint32_t B_BYTES = (uint32_t)NB * 64u * 2u;
    // B: groups of G channels (64-byte rows, 64-byte swizzle, for 32-channel
    // tiles; else 128-byte rows), each a 64-pixel box
    static constexpr int G = BN == 32 ? 32 : 64;
    static constexpr uint32_t B_ROW = (uint32_t)G * 2u;
    static constexpr uint32_t B_GROUP = B_ROW * 64u;
    static constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
    // two CTAs per SM of ~96 KB; packed column taps (bigger stages): one CTA
    // with a deeper ring
    static constexpr uint32_t BUDGET = DXP ? 196608u : 98304u;
    static constexpr int STAGES = BN == 256 ? 4 : (BUDGET / STAGE_BYTES > 8 ? 8 : (int)(BUDGET / STAGE_BYTES));
    static constexpr uint32_t SMEM = STAGES * STAGE_BYTES + 1024u;
    static constexpr uint32_t TMEM_COLS = NB <= 32 ? 32u : NB <= 64 ? 64u : NB <= 128 ? 128u : 256u;
    static_assert(!DXP || BN <= 64, "column taps packed only for tiles of at most 64 channels");
};

// grid: x = K split, y = m tile * (cin / BN) + n tile, z = tap row (dy + 1).
// PACK (32 output channels): the three tap rows share one launch, rows
// 32 d .. 32 d + 31 of the A tile holding dY at image row yy - dy (dy = d - 1)
// against X at row yy, since sum_y dY[y] X[y + dy] = sum_y' dY[y' - dy] X[y']
// (rows outside the image are TMA zero fill); the A map is then 4D over
// (x, y, image, channel). Rows of the A tile that no box writes hold stale
// data; they only reach accumulator rows the epilogue does not read.
template <int BN, bool PACK, bool DXP>
__global__ void __launch_bounds__(128) wgrad3x3_tc(const __grid_constant__ CUtensorMap tmA,
                                                   const __grid_constant__ CUtensorMap tmB, wgrad_args p) {
    using C = wgrad_cfg<BN, DXP>;
    // A (dY, MN-major from NHWC): groups of 32 output channels (64-byte rows)
    // when packed, else of 64 (128-byte rows); the 128-row tile is 16 KB
    constexpr uint32_t A_ROW = PACK ? 64u : 128u, A_GROUP = A_ROW * 64u;
    extern __shared__ uint8_t smem_dyn[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t full[C::STAGES], empty[C::STAGES], done;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const int ntiles = p.cin / BN;
    const int m0 = (blockIdx.y / ntiles) * 128;
    const int c0 = (blockIdx.y % ntiles) * BN;
    const int dy = (int)blockIdx.z - 1;
    const int segs_x = p.w / 64;
    const int kb0 = blockIdx.x * p.kpc;
    int nk = p.total_kb - kb0;
    if (nk > p.kpc) nk = p.kpc;
    if (nk < 0) nk = 0;

    if (warp == 0) tc::tmem_alloc(&tmem_base, C::TMEM_COLS);
    if (threadIdx.x == 32) {
        for (int s = 0; s < C::STAGES; s++) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(&done, 1);
        s_fail = 0;
        tc::mbar_fence_init();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == 0 && lane == 0) {
        int issued = 0;
        bool ok = true;
        for (int kb = 0; kb < nk; kb++) {
            const int s = kb % C::STAGES, r = kb / C::STAGES;
            if (r > 0 && !tc::mbar_wait(&empty[s], (r - 1) & 1)) {
                ok = false;
                break;
            }
            const int seg = kb0 + kb;
            const int xs = seg % segs_x;
            const int yy = (seg / segs_x) % p.h;
            const int im = seg / (segs_x * p.h);
            uint8_t* sa = base + (size_t)s * C::STAGE_BYTES;
            // whole boxes count, zero fill included
            tc::mbar_expect_tx(&full[s], (PACK ? 3u : (uint32_t)(p.a_rows + 63) / 64u) * A_GROUP + C::B_BYTES);
            if (PACK) {
#pragma unroll
                for (int d = 0; d < 3; d++) tc::tma_load_4d(sa + d * A_GROUP, &tmA, &full[s], 0, xs * 64, yy - (d - 1), im);
            } else {
                for (int j = 0; j * 64 < p.a_rows; j++) tc::tma_load_4d(sa + j * A_GROUP, &tmA, &full[s], m0 + j * 64, xs * 64, yy, im);
            }
#pragma unroll
            for (int xi = 0; xi < (DXP ? 3 : 1); xi++)
#pragma unroll
                for (int j = 0; j < BN / C::G; j++)
                    tc::tma_load_4d(sa + C::A_BYTES + (xi * (BN / C::G) + j) * C::B_GROUP, &tmB, &full[s],
                                    p.x_coff + c0 + j * C::G, xs * 64 + (DXP ? xi - 1 : p.dx), PACK ? yy : yy + dy, im);
            issued++;
        }
        if (!ok) {
            atomicExch(&s_fail, 1);
            for (int kb = issued - C::STAGES < 0 ? 0 : issued - C::STAGES; kb < issued; kb++)
                tc::mbar_wait(&full[kb % C::STAGES], (kb / C::STAGES) & 1);
        }
    } else if (warp == 1 && lane == 0) {
        constexpr uint32_t idesc = tc::idesc_bf16_bmn(128, C::NB) | (1u << 15);  // A MN-major too
        bool ok = true;
        for (int kb = 0; kb < nk; kb++) {
            const int s = kb % C::STAGES, r = kb / C::STAGES;
            if (!tc::mbar_wait(&full[s], r & 1)) {
                ok = false;
                break;
            }
            tc::fence_after();
            const uint32_t sa = tc::smem_u32(base + (size_t)s * C::STAGE_BYTES), sb = sa + C::A_BYTES;
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                tc::mma_bf16(tmem, tc::smem_desc_mn(sa + kk * 16 * A_ROW, A_ROW, A_GROUP),
                             tc::smem_desc_mn(sb + kk * 16 * C::B_ROW, C::B_ROW, C::B_GROUP),
                             idesc,
                             (kb | kk) != 0 ? 1u : 0u);
            tc::mma_commit(&empty[s]);
        }
        tc::mma_commit(&done);
        if (!ok) atomicExch(&s_fail, 1);
    }
    __syncwarp();

    bool got = tc::mbar_wait(&done, 0);
    got = __all_sync(0xffffffffu, got);
    tc::fence_after();
    // PACK: warp d < 3 holds tap row d of output channels lane; otherwise
    // accumulator row m is output channel m of tap row blockIdx.z. DXP:
    // columns [xi BN, (xi + 1) BN) belong to column tap xi
    if (got && nk > 0 && (!PACK || warp < 3)) {
        const int m = PACK ? lane : m0 + warp * 32 + lane;
        const int trow = PACK ? warp : dy + 1;
#pragma unroll 1
        for (int c = 0; c < C::NB; c += 32) {
            float v[32];
            tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
            const int xi = DXP ? c / BN : p.dx + 1, cc = DXP ? c % BN : c;
            if (m < p.cout) {
                float* dst = p.dw + ((size_t)m * 9 + trow * 3 + xi) * p.cin + c0 + cc;
#pragma unroll
                for (int j = 0; j < 32; j++) atomicAdd(dst + j, v[j]);
            }
        }
    }
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && (!got || s_fail)) atomicExch(p.err, 1);
    if (warp == 0) tc::tmem_dealloc(tmem, C::TMEM_COLS);
}

// ------------------------------------------------------------- tensor maps --
using encode_fn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                               const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                               CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

encode_fn encoder() {
    static encode_fn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<encode_fn>(p);
    });
    return fn;
}

bool make_map(CUtensorMap* m, const void* base, int rank, const cuuint64_t* dims, const cuuint64_t* strides_bytes,
              const cuuint32_t* box, CUtensorMapSwizzle sw) {
    encode_fn fn = encoder();
    if (!fn) return false;
    cuuint32_t es[4] = {1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(base), dims, strides_bytes, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <typename K>
cudaError_t raise_smem(K kernel, uint32_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

int sm_count_cached() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <int BK, int BN, int MODE>
cudaError_t launch_conv(const CUtensorMap& a, const CUtensorMap& b, const conv_args& p, cudaStream_t s) {
    using C = conv_cfg<BK, BN, MODE>;
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] { attr = raise_smem(conv3x3_tc<BK, BN, MODE>, C::SMEM); });
    if (attr != cudaSuccess) return attr;
    const long long tiles = (long long)p.n_img * ((p.h + C::R - 1) / C::R) * p.tiles_x * (p.cout / BN);
    if (tiles > 0x7FFFFFFFLL) return cudaErrorInvalidValue;
    const int grid = (int)std::min<long long>(tiles, sm_count_cached());
    conv3x3_tc<BK, BN, MODE><<<grid, 32 * (kEpiWarps + 2), C::SMEM, s>>>(a, b, p);
    return cudaGetLastError();
}

template <int BN, bool PACK, bool DXP>
cudaError_t launch_wgrad(const CUtensorMap& a, const CUtensorMap& b, const wgrad_args& p, int splits, cudaStream_t s) {
    using C = wgrad_cfg<BN, DXP>;
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] { attr = raise_smem(wgrad3x3_tc<BN, PACK, DXP>, C::SMEM); });
    if (attr != cudaSuccess) return attr;
    const int mtiles = (p.cout + 127) / 128;
    dim3 grid((unsigned)splits, (unsigned)(mtiles * (p.cin / BN)), PACK ? 1u : 3u);
    wgrad3x3_tc<BN, PACK, DXP><<<grid, 128, C::SMEM, s>>>(a, b, p);
    return cudaGetLastError();
}

int pick_bn(int c) {
    for (int bn : {256, 128, 64, 32})
        if (c % bn == 0) return bn;
    return 0;
}

}  // namespace

extern "C" cudaError_t rfk_unet_conv3x3(const void* in, int n_img, int h, int w, int in_cstride, int in_coff, int cin,
                                        const void* weights, int cout, const float* bias, int flags, void* out,
                                        int out_cstride, int out_coff, const void* mask, int mask_cstride, int mask_coff,
                                        int accumulate, int* err, cudaStream_t s) {
    if (cin % 32 || in_coff % 32 || in_cstride % 32 || cout % 32 || out_coff % 32 || out_cstride % 32) return cudaErrorInvalidValue;
    if (mask && (mask_coff % 32 || mask_cstride % 32)) return cudaErrorInvalidValue;
    if (in_coff + cin > in_cstride || out_coff + cout > out_cstride || n_img <= 0 || h <= 0 || w <= 0)
        return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(weights) | reinterpret_cast<uintptr_t>(out)) & 63)
        return cudaErrorMisalignedAddress;
    const int bn = pick_bn(cout);
    // tap reuse: 32 output channels (4 rows per tile) load each input channel
    // block once for all nine taps (MODE 2, 32-channel K blocks so that three
    // 70 KB stages fit); 64 (2 rows) once per tap row (MODE 1); wider tiles
    // (1 row) once per tap (MODE 0)
    // MODE 2 keeps one output tile's weights resident: cout == 32, at most 3 input blocks
    const int mode = (bn == 32 && cout == 32 && cin <= 32 * 3) ? 2 : (bn <= 64 ? 1 : 0);
    const int bk = (mode != 2 && cin % 64 == 0 && in_coff % 64 == 0) ? 64 : 32;
    CUtensorMap ma, mb;
    const CUtensorMapSwizzle sw = bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
    {
        cuuint64_t dims[4] = {(cuuint64_t)in_cstride, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n_img};
        cuuint64_t str[3] = {(cuuint64_t)in_cstride * 2, (cuuint64_t)w * in_cstride * 2, (cuuint64_t)h * w * in_cstride * 2};
        // image rows and pixel lines of an A box, as conv_cfg<BK, BN, MODE>
        const cuuint32_t rows = (bn >= 128 ? 1u : (cuuint32_t)(128 / bn)) + (mode == 2 ? 2u : 0u);
        cuuint32_t box[4] = {(cuuint32_t)bk, mode ? 136u : 128u, rows, 1};
        if (!make_map(&ma, in, 4, dims, str, box, sw)) return cudaErrorInvalidValue;
    }
    {
        cuuint64_t dims[2] = {(cuuint64_t)9 * cin, (cuuint64_t)cout};
        cuuint64_t str[1] = {(cuuint64_t)9 * cin * 2};
        cuuint32_t box[2] = {(cuuint32_t)bk, (cuuint32_t)bn};
        if (!make_map(&mb, weights, 2, dims, str, box, sw)) return cudaErrorInvalidValue;
    }
    conv_args p{};
    p.n_img = n_img;
    p.h = h;
    p.w = w;
    p.tiles_x = (w + 127) / 128;
    p.cin = cin;
    p.cin_off = in_coff;
    p.cout = cout;
    p.out = out;
    p.out_cstride = out_cstride;
    p.out_coff = out_coff;
    p.bias = bias;
    p.relu = flags & RFK_UNET_RELU;
    p.out_f32 = (flags & RFK_UNET_F32OUT) ? 1 : 0;
    p.up2 = (flags & RFK_UNET_UP2) ? 1 : 0;
    if (p.up2 && (p.out_f32 || accumulate)) return cudaErrorInvalidValue;
    p.mask = static_cast<const bf16*>(mask);
    p.mask_cstride = mask_cstride;
    p.mask_coff = mask_coff;
    p.accumulate = accumulate;
    p.err = err;
    if (bk == 64) {
        switch (bn) {
        case 256: return launch_conv<64, 256, 0>(ma, mb, p, s);
        case 128: return launch_conv<64, 128, 0>(ma, mb, p, s);
        case 64: return launch_conv<64, 64, 1>(ma, mb, p, s);
        default: return launch_conv<64, 32, 1>(ma, mb, p, s);
        }
    }
    switch (bn) {
    case 256: return launch_conv<32, 256, 0>(ma, mb, p, s);
    case 128: return launch_conv<32, 128, 0>(ma, mb, p, s);
    case 64: return launch_conv<32, 64, 1>(ma, mb, p, s);
    default: return mode == 2 ? launch_conv<32, 32, 2>(ma, mb, p, s) : launch_conv<32, 32, 1>(ma, mb, p, s);
    }
}

extern "C" cudaError_t rfk_unet_wgrad3x3(const void* dy, const void* x, int x_cstride, int x_coff, int n_img, int h, int w,
                                         int cout, int cin, float* dw, int* err, cudaStream_t s) {
    if (w % 64 || cin % 32 || cout <= 0 || cout % 32 || n_img <= 0 || h <= 0) return cudaErrorInvalidValue;
    if (x_coff % 32 || x_cstride % 32 || x_coff + cin > x_cstride) return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(dy) | reinterpret_cast<uintptr_t>(x)) & 63) return cudaErrorMisalignedAddress;
    const int bn = pick_bn(cin);
    const size_t P = (size_t)n_img * h * w;
    // 32 output channels: the three tap rows packed into one launch's M
    const bool pack = cout == 32;
    const int a_rows = cout < 128 ? cout : 128;
    CUtensorMap ma, mb;
    {
        // dY NHWC (cout channels): boxes of 32 (packed, 64-byte swizzle) or 64
        // output channels x 64 pixels, MN-major
        const cuuint32_t g = pack ? 32u : 64u;
        cuuint64_t dims[4] = {(cuuint64_t)cout, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n_img};
        cuuint64_t str[3] = {(cuuint64_t)cout * 2, (cuuint64_t)w * cout * 2, (cuuint64_t)h * w * cout * 2};
        cuuint32_t box[4] = {g, 64, 1, 1};
        if (!make_map(&ma, dy, 4, dims, str, box, pack ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B))
            return cudaErrorInvalidValue;
    }
    {
        // X NHWC: boxes of 32 (64-byte swizzle) or 64 channels x 64 pixels
        const cuuint32_t g = bn == 32 ? 32u : 64u;
        cuuint64_t dims[4] = {(cuuint64_t)x_cstride, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n_img};
        cuuint64_t str[3] = {(cuuint64_t)x_cstride * 2, (cuuint64_t)w * x_cstride * 2, (cuuint64_t)h * w * x_cstride * 2};
        cuuint32_t box[4] = {g, 64, 1, 1};
        if (!make_map(&mb, x, 4, dims, str, box, g == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B))
            return cudaErrorInvalidValue;
    }
    wgrad_args p{};
    p.n_img = n_img;
    p.h = h;
    p.w = w;
    p.cout = cout;
    p.cin = cin;
    p.x_coff = x_coff;
    p.total_kb = (int)(P / 64);
    p.a_rows = a_rows;
    // about 8 CTAs per SM over the three launches' taps and tiles
    // input channel tiles of at most 64: the column taps packed into N
    const bool dxp = bn <= 64;
    const int mtiles = (cout + 127) / 128;
    const int per_split = (pack ? 1 : 3) * (dxp ? 1 : 3) * mtiles * (cin / bn);
    int splits = (152 * 8 / 3 + per_split - 1) / per_split;
    if (splits > p.total_kb) splits = p.total_kb;
    if (splits < 1) splits = 1;
    p.kpc = (p.total_kb + splits - 1) / splits;
    splits = (p.total_kb + p.kpc - 1) / p.kpc;
    p.dw = dw;
    p.err = err;
    for (int d = 0; d < (dxp ? 1 : 3); d++) {
        p.dx = d - 1;
        cudaError_t e;
        if (dxp) {
            if (bn == 64) e = pack ? launch_wgrad<64, true, true>(ma, mb, p, splits, s) : launch_wgrad<64, false, true>(ma, mb, p, splits, s);
            else e = pack ? launch_wgrad<32, true, true>(ma, mb, p, splits, s) : launch_wgrad<32, false, true>(ma, mb, p, splits, s);
        } else if (pack) {
            e = bn == 256 ? launch_wgrad<256, true, false>(ma, mb, p, splits, s) : launch_wgrad<128, true, false>(ma, mb, p, splits, s);
        } else {
            e = bn == 256 ? launch_wgrad<256, false, false>(ma, mb, p, splits, s) : launch_wgrad<128, false, false>(ma, mb, p, splits, s);
        }
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
