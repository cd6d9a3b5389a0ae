// Chaos-game kernels, specialised per flame structure by NVRTC.
//
// The flame compiler prepends rfk_device.cuh and the generated flame code,
// which defines:
//   RFK_NX, RFK_HAS_FINAL, RFK_CHAOS, RFK_SIZE_REALS, RFK_NUM_AFFINES,
//   rfk_affine_idx[], rfk_xf_base[] (offset of each xform's weight),
//   R rfk_dispatch(int k, V2& p, R& c, const float* P, Rng& rng)   (standard xforms)
//   R rfk_final(V2& p, R& c, const float* P, Rng& rng)              (if RFK_HAS_FINAL)
//   void rfk_precalc(float* P, Rng& rng)                             (variation precalc)
// and the launch shape: RFK_BLOCK (threads per block), RFK_CPT (chains per
// thread), RFK_FLUSH (0 = one red.global.add.v4.f32 per draw, 1 = warp-
// aggregated red for lanes that hit the same pixel, 2 = warp-aggregated into a
// per-block shared-memory cache of hot pixels, 3 = the cache without warp
// aggregation, 4 = shared-memory sums for the pixels that the block's own
// draws show to be hot, one red per draw elsewhere), RFK_SORT (1 = sort each
// warp's chains by picked xform every pass, so a warp runs one xform at a
// time instead of a divergent switch).
//
// Reference behaviour restated here (assets/kernels/refactor.cu):
//   :99-117,:266-294  per temporal sample: flame = Catmull-Rom at t, affines
//                     polar -> Cartesian, palette HSV -> 8-bit RGB (:128-147)
//   :296-308          precalc, Hammersley start points mapped through the
//                     plane-space affine, colour ~ U(0,1)
//   :176-238          pass: pick xform, apply, bad-value reset
//   :347-386          final xform on a copy, screen affine, trunc, bounds,
//                     palette lerp between floor/ceil of colour*255, draw
//   :404-475          persistent loop with quality / time / stop-flag bailout
// Differences by design: each chain picks its own xform from a cumulative
// weight table in shared memory (the reference votes one xform per warp and
// shuffles iterators through the block); histogram updates are atomic
// red.global.add.v4.f32 (the reference does a racy load/add/store); the RNG is
// counter-based Philox keyed by (seed, flame salt) with counter (chain, sub,
// pass).

#ifndef RFK_BLOCK
#define RFK_BLOCK 256
#endif
#ifndef RFK_CPT
#define RFK_CPT 1
#endif
#ifndef RFK_FLUSH
#define RFK_FLUSH 0
#endif
#ifndef RFK_SORT
#define RFK_SORT 0
#endif

// Per-sample parameter block (floats): the reals, the xform pick table (an
// alias table of RFK_NX (threshold, alias) pairs), with chaos one alias table
// per previous xform, then the 256 x float4 palette.
#define RFK_OFF_ALIAS ((RFK_SIZE_REALS + 1) / 2 * 2)
#define RFK_OFF_CALIAS (RFK_OFF_ALIAS + 2 * RFK_NX)
#define RFK_OFF_PAL_RAW (RFK_OFF_CALIAS + (RFK_CHAOS ? 2 * RFK_NX * RFK_NX : 0))
#define RFK_OFF_PAL (((RFK_OFF_PAL_RAW) + 3) / 4 * 4)
#define RFK_SAMPLE_FLOATS (RFK_OFF_PAL + 1024)

// Passes between the bailout checks of the bin kernels, at most (the host
// computes at most 32; the kernels clamp it again).
#define RFK_MAX_CHECK 32u

// Status bits reported to the host.
#define RFK_ST_QUALITY 1u
#define RFK_ST_TIME 2u
#define RFK_ST_STOP 4u
#define RFK_ST_ITERS 8u

struct rfk_counters {
    unsigned long long quality;   // sum of (u32)(255 * opacity) over draws
    unsigned long long passes;    // chain steps
    unsigned long long start_ns;  // earliest block start (%globaltimer)
    unsigned long long stop_ns;   // latest block stop
    unsigned long long draws;     // in-bounds draws with opacity > 0
    unsigned int status;          // RFK_ST_* bits seen by any block
    unsigned int pad;
};

__device__ __forceinline__ unsigned long long rfk_time() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void rfk_red_v4(float4* addr, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}

// Chain state, structure of arrays over chains.
struct rfk_chains {
    float* x;
    float* y;
    float* c;
    unsigned char* last;  // previous xform (chaos), 255 = none
};

// Walker / Vose alias table of the weights wt[0..RFK_NX): entry i holds a
// threshold and an alias; a uniform u picks i = floor(u * RFK_NX) and keeps i
// when the fraction u * RFK_NX - i is below the threshold, else takes the
// alias, so xform k comes out with probability wt[k] / sum(wt) in O(1)
// (flame.tpl:110-123 picks by a linear search of the cumulative weights with
// the same distribution). Zero weights get threshold 0 and the heaviest xform
// as alias, so they are never picked; all weights zero picks xform 0, as the
// reference's fallback does.
__device__ void rfk_alias_table(const float (&wt)[RFK_NX], float* tbl) {
    float sum = 0.0f;
    int heavy = 0;
    for (int i = 0; i < RFK_NX; i++) {
        sum += wt[i];
        if (wt[i] > wt[heavy]) heavy = i;
    }
    if (!(sum > 0.0f)) {
        for (int i = 0; i < RFK_NX; i++) {
            tbl[2 * i] = 0.0f;
            tbl[2 * i + 1] = __int_as_float(0);
        }
        return;
    }
    float q[RFK_NX];
    int small[RFK_NX], large[RFK_NX];
    int ns = 0, nl = 0;
    for (int i = 0; i < RFK_NX; i++) {
        q[i] = wt[i] * (float)RFK_NX / sum;
        if (q[i] < 1.0f) small[ns++] = i;
        else large[nl++] = i;
    }
    while (ns > 0 && nl > 0) {
        const int sm = small[--ns], lg = large[nl - 1];
        tbl[2 * sm] = q[sm];
        tbl[2 * sm + 1] = __int_as_float(lg);
        q[lg] = (q[lg] + q[sm]) - 1.0f;
        if (q[lg] < 1.0f) {
            nl--;
            small[ns++] = lg;
        }
    }
    // what rounding leaves over keeps itself (zero weights: the heaviest)
    while (nl > 0) {
        const int lg = large[--nl];
        tbl[2 * lg] = 2.0f;
        tbl[2 * lg + 1] = __int_as_float(lg);
    }
    while (ns > 0) {
        const int sm = small[--ns];
        const bool zero = !(wt[sm] > 0.0f);
        tbl[2 * sm] = zero ? 0.0f : 2.0f;
        tbl[2 * sm + 1] = __int_as_float(zero ? heavy : sm);
    }
}

// ---------------------------------------------------------------- prepare --
// One block per temporal sample: evaluate the spline segment at t, convert
// affines, build the palette, run precalc, build the xform pick tables, and
// (jitter != 0) offset the screen affine by the sample's antialiasing jitter.
extern "C" __global__ void __launch_bounds__(256) rfk_prepare(const float4* __restrict__ coeff, unsigned sample_size,
                                                              const unsigned* __restrict__ seg_of, const float* __restrict__ t_of,
                                                              float* __restrict__ out, unsigned seed, unsigned salt,
                                                              unsigned jitter) {
    __shared__ float P[RFK_SAMPLE_FLOATS];
    const unsigned s = blockIdx.x;
    const float t = t_of[s];
    // the padding after the reals and before the palette is written too (as
    // 0): every float of the block that leaves this kernel is defined
    for (unsigned i = RFK_SIZE_REALS + threadIdx.x; i < RFK_OFF_ALIAS; i += blockDim.x) P[i] = 0.0f;
    for (unsigned i = RFK_OFF_PAL_RAW + threadIdx.x; i < RFK_OFF_PAL; i += blockDim.x) P[i] = 0.0f;
    const float4* seg = coeff + (size_t)seg_of[s] * sample_size;

    // Hermite basis of the segment p1 -> p2 with tangents m1, m2 (the same
    // cubic as a t^3 + b t^2 + c t + d of catmull.cu, evaluated so that t = 0
    // and t = 1 return the knots exactly)
    const float t2 = t * t;
    const float h01 = t2 * (3.0f - 2.0f * t), h00 = 1.0f - h01;
    const float h10 = t * (1.0f - t) * (1.0f - t), h11 = t2 * (t - 1.0f);
    for (unsigned i = threadIdx.x; i < RFK_SIZE_REALS; i += blockDim.x) {
        const float4 k = seg[i];  // (p1, p2, m1, m2)
        P[i] = fmaf(h00, k.x, fmaf(h01, k.y, fmaf(h10, k.z, h11 * k.w)));
    }
    for (unsigned i = threadIdx.x; i < 256; i += blockDim.x) {
        float hsv[3];
        for (int j = 0; j < 3; j++) {
            const float4 k = seg[RFK_SIZE_REALS + 3 * i + j];
            hsv[j] = fmaf(h00, k.x, fmaf(h01, k.y, fmaf(h10, k.z, h11 * k.w)));
        }
        // HSV -> RGB as refactor.cu:128-140, truncated to 8 bits
        float rgb[3];
        const float ns[3] = {5.0f, 3.0f, 1.0f};
        for (int j = 0; j < 3; j++) {
            float kk = fmodf(ns[j] + hsv[0] / 60.0f, 6.0f);
            float f = hsv[2] - hsv[2] * hsv[1] * fmaxf(0.0f, fminf(kk, fminf(4.0f - kk, 1.0f)));
            float v = f * 255.0f;
            rgb[j] = (float)(unsigned char)fminf(fmaxf(v, 0.0f), 255.0f) / 255.0f;
        }
        P[RFK_OFF_PAL + 4 * i + 0] = rgb[0];
        P[RFK_OFF_PAL + 4 * i + 1] = rgb[1];
        P[RFK_OFF_PAL + 4 * i + 2] = rgb[2];
        P[RFK_OFF_PAL + 4 * i + 3] = 0.0f;
    }
    __syncthreads();
    for (unsigned ai = threadIdx.x; ai < RFK_NUM_AFFINES; ai += blockDim.x) {
        const unsigned a = rfk_affine_idx[ai];
        const float angx = P[a], angy = P[a + 1];
        const float magx = expf(P[a + 2]), magy = expf(P[a + 3]);
        float sx, cx, sy, cy;
        sincosf(angx, &sx, &cx);
        sincosf(angy, &sy, &cy);
        P[a] = magx * cx;
        P[a + 1] = magx * sx;
        P[a + 2] = magy * cy;
        P[a + 3] = magy * sy;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        Rng rng;
        rng.start(s, 0xFFFFu, 0xFFFFFFFFFFFFFFFFull, seed, salt);
        // weight sum and pick table (flame.tpl:110-123 semantics)
        float wt[RFK_NX];
        float wsum = 0.0f;
        for (int i = 0; i < RFK_NX; i++) {
            wt[i] = P[rfk_xf_base[i]];
            wsum += wt[i];
        }
        P[12] = wsum;
        rfk_alias_table(wt, P + RFK_OFF_ALIAS);
#if RFK_CHAOS
        // chaos rows (flame.tpl:170-177): weights[j] *= xform_j.weight; the
        // interpolated rows themselves stay as they are
        for (int r = 0; r < RFK_NX; r++) {
            const unsigned row = 13 + r * (RFK_NX + 1);
            float rw[RFK_NX];
            for (int j = 0; j < RFK_NX; j++) rw[j] = P[row + 1 + j] * wt[j];
            rfk_alias_table(rw, P + RFK_OFF_CALIAS + r * (2 * RFK_NX));
        }
#endif
        // screen jitter ~ gauss(1/3 px) for antialiasing (flame.tpl:179-182)
        V2 j = rng.gauss(1.0f / 3.0f);
        if (jitter) {
            P[4] += j.x;
            P[5] += j.y;
        }
        rfk_precalc(P, rng);
    }
    __syncthreads();
    float* dst = out + (size_t)s * RFK_SAMPLE_FLOATS;
    for (unsigned i = threadIdx.x; i < RFK_SAMPLE_FLOATS; i += blockDim.x) dst[i] = P[i];
}

// ------------------------------------------------------- parameter block --
// 8-bit RGB of a palette entry (the prepared palette holds k / 255).
__device__ __forceinline__ unsigned rfk_rgb8(float4 c) {
    return (unsigned)__float2int_rn(c.x * 255.0f) | ((unsigned)__float2int_rn(c.y * 255.0f) << 8) |
           ((unsigned)__float2int_rn(c.z * 255.0f) << 16);
}

// All threads of the block: copies a prepared parameter block into shared
// memory P. The palette goes in as 8-bit RGB pairs (entry i, entry i + 1) in
// the first half of its float4 region, as the reference keeps it (uchar3,
// refactor.cu:128-140): a draw reads both ends of its colour interval with one
// 8-byte load from a 2 KB table instead of two 16-byte loads from 4 KB, which
// cuts the shared-memory wavefronts of the random palette reads.
__device__ __forceinline__ void rfk_load_params(float* P, const float* __restrict__ src) {
    for (unsigned i = threadIdx.x; i < RFK_OFF_PAL; i += RFK_BLOCK) P[i] = src[i];
    uint2* pal = reinterpret_cast<uint2*>(P + RFK_OFF_PAL);
    const float4* sp = reinterpret_cast<const float4*>(src + RFK_OFF_PAL);
    for (unsigned i = threadIdx.x; i < 256; i += RFK_BLOCK) pal[i] = make_uint2(rfk_rgb8(sp[i]), rfk_rgb8(sp[min(i + 1, 255u)]));
}

// ------------------------------------------------------------- chain step --
// Xform pick from a uniform u in [0, 1) through the alias table (of the
// previous xform's chaos row when there is one).
__device__ __forceinline__ int rfk_pick(float u, const float* __restrict__ P, unsigned last) {
    const float* tbl = P + RFK_OFF_ALIAS;
#if RFK_CHAOS
    if (last != 255u) tbl = P + RFK_OFF_CALIAS + last * (2 * RFK_NX);
#endif
    const float v = u * (float)RFK_NX;
    const int i = min((int)v, RFK_NX - 1);
    const float2 e = reinterpret_cast<const float2*>(tbl)[i];
    return (v - (float)i < e.x) ? i : __float_as_int(e.y);
}

// Moves one chain through xform k: apply, bad-value reset, final xform on a
// copy, screen projection. Returns the draw (pixel index or -1) and its RGBA
// contribution.
__device__ __forceinline__ int rfk_move(int k, float& x, float& y, float& c, Rng& rng, const float* __restrict__ P,
                                        unsigned w, unsigned h, float4& contrib, unsigned& hit) {
    V2 p = fl_vec2(x, y);
    R col = c;
    R op = rfk_dispatch(k, p, col, P, rng);
    if (rfk_badvalue(p.x) || rfk_badvalue(p.y)) {
        p.x = rng.u01() * 2.0f - 1.0f;
        p.y = rng.u01() * 2.0f - 1.0f;
        op = 0.0f;
    }
    x = p.x;
    y = p.y;
    c = col;
#if RFK_HAS_FINAL
    rfk_final(p, col, P, rng);
#endif
    // screen-space affine (a,d,b,e,c,f at P[0..5])
    float sx = fmaf(P[0], p.x, fmaf(P[2], p.y, P[4]));
    float sy = fmaf(P[1], p.x, fmaf(P[3], p.y, P[5]));
    sx = truncf(sx);
    sy = truncf(sy);
    hit = 0;
    if (sx >= 0.0f && sy >= 0.0f && sx < (float)w && sy < (float)h && op > 0.0f) {
        // lerp between the 8-bit entries at floor and floor + 1 of colour *
        // 255 (at an integer the weight of floor + 1 is 0, as the reference's
        // ceil), / 255, * opacity (refactor.cu:366-378)
        const float pi = fminf(fmaxf(col, 0.0f), 1.0f) * 255.0f;
        const float lo_f = floorf(pi);
        const float mix = pi - lo_f;
        const uint2 e = reinterpret_cast<const uint2*>(P + RFK_OFF_PAL)[(int)lo_f];
        const float s = op * (1.0f / 255.0f);
        contrib.x = ((1.0f - mix) * (float)(e.x & 0xFFu) + mix * (float)(e.y & 0xFFu)) * s;
        contrib.y = ((1.0f - mix) * (float)((e.x >> 8) & 0xFFu) + mix * (float)((e.y >> 8) & 0xFFu)) * s;
        contrib.z = ((1.0f - mix) * (float)((e.x >> 16) & 0xFFu) + mix * (float)((e.y >> 16) & 0xFFu)) * s;
        contrib.w = op;
        hit = (unsigned)(255.0f * op);
        return (int)sy * (int)w + (int)sx;
    }
    return -1;
}

// One chaos-game step of one chain: pick an xform from the cumulative weights
// (or the chaos row of the previous xform), then move.
__device__ __forceinline__ int rfk_step(float& x, float& y, float& c, unsigned& last, Rng& rng,
                                        const float* __restrict__ P, unsigned w, unsigned h, float4& contrib,
                                        unsigned& hit) {
    const int k = rfk_pick(rng.u01(), P, last);
#if RFK_CHAOS
    last = (unsigned)k;
#endif
    return rfk_move(k, x, y, c, rng, P, w, h, contrib, hit);
}

#if RFK_SORT
// Counting sort of a warp's 32 * RFK_CPT chains by their picked xform, in
// place in the warp's region of the chain array: the caller has read every
// slot of the warp (its values v and picks k) before the call, so the scatter
// may overwrite any of them. Afterwards slot q * 32 + lane of the region holds
// the lane's round-q chain, and the lanes of one round run the same xform
// except at the boundaries between xform runs. Each round's lanes with equal
// xform are grouped by __match_any_sync; the group leader reserves the group's
// places in the per-warp xform counters; a warp scan of the counters gives
// each xform's start. Only __syncwarp is needed.
__device__ __forceinline__ void rfk_sort_chains(float4* __restrict__ region, const float4 (&v)[RFK_CPT],
                                                const int (&k)[RFK_CPT], const unsigned (&bits)[RFK_CPT],
                                                unsigned* __restrict__ counts) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt = (1u << lane) - 1u;
    if (lane < RFK_NX) counts[lane] = 0u;
    __syncwarp();
    unsigned off[RFK_CPT];
#pragma unroll
    for (int q = 0; q < RFK_CPT; q++) {
        const unsigned same = __match_any_sync(0xffffffffu, k[q]);
        const int leader = __ffs(same) - 1;
        unsigned base = 0;
        if ((int)lane == leader) base = atomicAdd(&counts[k[q]], (unsigned)__popc(same));
        off[q] = __shfl_sync(0xffffffffu, base, leader) + __popc(same & lt);
    }
    __syncwarp();
    // exclusive scan of the per-xform counts across lanes 0..RFK_NX-1
    unsigned cnt = (lane < RFK_NX) ? counts[lane] : 0u;
    unsigned incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, incl, d);
        if ((int)lane >= d) incl += u;
    }
    const unsigned start = incl - cnt;
#pragma unroll
    for (int q = 0; q < RFK_CPT; q++) {
        const unsigned pos = __shfl_sync(0xffffffffu, start, k[q]) + off[q];
        region[pos] = make_float4(v[q].x, v[q].y, v[q].z, __int_as_float(k[q] | (int)(bits[q] << 8)));
    }
    __syncwarp();
}

#define RFK_NW (RFK_BLOCK / 32)
// Block-wide counting sort of the block's RFK_BLOCK * RFK_CPT chains by picked
// xform (deterministic order: xform-major, then warp, then round, then lane),
// in place in the chain array: every thread has read its own slots (positions
// and colours v, picks) before the call, and the scatter comes after a
// barrier. Two barriers per pass: after the first, every warp derives the
// starts it needs from the per-(xform, warp) counters itself (no single-warp
// scan and second barrier). counts[RFK_NX * RFK_NW] must be zero on entry.
// `next` (the other counter set) is cleared after the first barrier: every
// warp read it in the previous pass before that pass's second barrier, and its
// next-pass updates come after this pass's second barrier. Afterwards slot
// q * RFK_BLOCK + t holds thread t's round-q chain, so a warp's round covers 32
// consecutive slots of one xform run except at run ends.
// kb[q / 2] holds round q's pick | 8 spare random bits << 8 in its 16-bit half
// q % 2, and the offsets are packed the same way: two per register, so the
// sort of 8 chains per thread holds 24 + 4 + 4 registers instead of 24 + 24
// (fewer spills at the 64-register cap; 1.3% faster on the 1080p genome).
__device__ __forceinline__ void rfk_block_sort(float4* __restrict__ chains, const float3 (&v)[RFK_CPT],
                                               const unsigned (&kb)[(RFK_CPT + 1) / 2],
                                               unsigned* __restrict__ counts, unsigned* __restrict__ next) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    unsigned offp[(RFK_CPT + 1) / 2];
#pragma unroll
    for (int q = 0; q < RFK_CPT; q++) {
        const int k = (int)((kb[q >> 1] >> (16 * (q & 1))) & 0xFFu);
        const unsigned same = __match_any_sync(0xffffffffu, k);
        const int leader = __ffs(same) - 1;
        unsigned base = 0;
        if ((int)lane == leader) base = atomicAdd(&counts[k * RFK_NW + warp], (unsigned)__popc(same));
        const unsigned off = __shfl_sync(0xffffffffu, base, leader) + __popc(same & lt);
        if (q & 1) offp[q >> 1] |= off << 16;
        else offp[q >> 1] = off;
    }
    __syncthreads();
    for (unsigned i = threadIdx.x; i < RFK_NX * RFK_NW; i += RFK_BLOCK) next[i] = 0u;
    // lane x < RFK_NX: the block's count of xform x and the part of it in
    // warps before this one; an exclusive scan of the counts over lanes gives
    // the start of xform x's run, and start + part this warp's start in it
    unsigned tot = 0, part = 0;
    if (lane < RFK_NX) {
#pragma unroll
        for (unsigned w = 0; w < RFK_NW; w++) {
            const unsigned c = counts[lane * RFK_NW + w];
            tot += c;
            part += (w < warp) ? c : 0u;
        }
    }
    unsigned incl = tot;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, incl, d);
        if ((int)lane >= d) incl += u;
    }
    const unsigned start = incl - tot + part;
#pragma unroll
    for (int q = 0; q < RFK_CPT; q++) {
        const unsigned kbq = (kb[q >> 1] >> (16 * (q & 1))) & 0xFFFFu;
        const unsigned pos =
            __shfl_sync(0xffffffffu, start, (int)(kbq & 0xFFu)) + ((offp[q >> 1] >> (16 * (q & 1))) & 0xFFFFu);
        chains[pos] = make_float4(v[q].x, v[q].y, v[q].z, __int_as_float((int)kbq));
    }
    __syncthreads();
}
#endif

#if RFK_FLUSH == 2 || RFK_FLUSH == 3
// Shared-memory cache of hot pixels (one per block): direct-mapped slots keyed
// by pixel index, claimed with atomicCAS while empty and never evicted until
// the next flush, so adds into a claimed slot never race with its flush.
#define RFK_CACHE_SLOTS 1024
#define RFK_CACHE_EMPTY 0xFFFFFFFFu
struct rfk_cache {
    unsigned tag[RFK_CACHE_SLOTS];
    float val[4][RFK_CACHE_SLOTS];
};

__device__ __forceinline__ unsigned rfk_cache_slot(int idx) {
    return ((unsigned)idx * 2654435761u) >> (32 - 10);
}

__device__ __forceinline__ void rfk_cache_clear(rfk_cache& cc) {
    for (unsigned i = threadIdx.x; i < RFK_CACHE_SLOTS; i += RFK_BLOCK) {
        cc.tag[i] = RFK_CACHE_EMPTY;
        cc.val[0][i] = cc.val[1][i] = cc.val[2][i] = cc.val[3][i] = 0.0f;
    }
}

// All threads of the block, between barriers: every claimed slot goes out as
// one red.global.add.v4.f32 and the slot is emptied.
__device__ __forceinline__ void rfk_cache_flush(rfk_cache& cc, float4* __restrict__ bins) {
    for (unsigned i = threadIdx.x; i < RFK_CACHE_SLOTS; i += RFK_BLOCK) {
        const unsigned t = cc.tag[i];
        if (t != RFK_CACHE_EMPTY) {
            rfk_red_v4(bins + t, cc.val[0][i], cc.val[1][i], cc.val[2][i], cc.val[3][i]);
            cc.tag[i] = RFK_CACHE_EMPTY;
            cc.val[0][i] = cc.val[1][i] = cc.val[2][i] = cc.val[3][i] = 0.0f;
        }
    }
}

// Adds one contribution through the block's hot-pixel cache: into the slot of
// `idx` when it holds idx or can be claimed, else straight to the histogram.
__device__ __forceinline__ void rfk_cache_add(rfk_cache& cc, float4* __restrict__ bins, int idx, float4 acc) {
    const unsigned slot = rfk_cache_slot(idx);
    unsigned t = cc.tag[slot];
    if (t == RFK_CACHE_EMPTY) {
        t = atomicCAS(&cc.tag[slot], RFK_CACHE_EMPTY, (unsigned)idx);
        if (t == RFK_CACHE_EMPTY) t = (unsigned)idx;
    }
    if (t == (unsigned)idx) {
        atomicAdd(&cc.val[0][slot], acc.x);
        atomicAdd(&cc.val[1][slot], acc.y);
        atomicAdd(&cc.val[2][slot], acc.z);
        atomicAdd(&cc.val[3][slot], acc.w);
    } else {
        rfk_red_v4(bins + idx, acc.x, acc.y, acc.z, acc.w);
    }
}
#endif

#if RFK_FLUSH == 4
// Per-block table of hot pixels. Flames put a large share of their draws on
// few pixels (the 1080p bench genome: 3.4% on one pixel, 21% on 64), and
// red.global.add on one address serialises in its L2 slice, so those draws
// are summed in shared memory and go out as one red.global.add.v4.f32 per hot
// pixel and check interval; every other draw is one red.v4 after a single
// 16-byte table load, with no warp-wide matching of pixels.
//   discovery  in the first RFK_DISC_PASSES passes of every check interval,
//              the draws of one chain in RFK_CPT (RFK_DISC below) are counted
//              per pixel in a hash table (linear probing, at most
//              RFK_DISC_PROBES places);
//   rebuild    after those passes (all threads, between barriers): the old
//              sums are flushed, and every pixel counted RFK_HOT_MIN times or
//              more becomes hot (at most RFK_HOT_MAX, the first two free ways
//              of its bucket), the counts are cleared;
//   draw       a draw to a hot pixel adds to its sums (RFK_HOT_COPIES copies,
//              picked by lane, so that lanes on one pixel rarely wait on the
//              same shared-memory word), any other draw is one red.v4.
// The sums are also flushed at the end of every check interval, so they
// always go to the histogram of the unit whose draws they hold.
// The sums are fixed point, value * 2^RFK_HOT_SHIFT in one u32 per (slot,
// copy, channel), added with integer shared-memory atomics: on GB300 these
// take 0.87x the time of the chain step with float shared-memory atomics on
// the 1080p bench genome. A copy sums the draws of RFK_BLOCK * RFK_CPT /
// RFK_HOT_COPIES chains over at most RFK_MAX_CHECK passes between flushes,
// each channel at most 1 (a draw with opacity above 1, which only a spline
// overshoot gives, goes out as a red.v4), so the shift below keeps every sum
// under 2^31. One quantum is 2^-17 at the bench's launch shape: 7.6e-6 per
// draw against colour contributions of up to the opacity; an opacity of 1 is
// exact.
#define RFK_HOT_MAX 64
#define RFK_HOT_BUCKETS 128  // two ways each
#define RFK_HOT_COPIES 4
__host__ __device__ constexpr int rfk_log2_ceil(unsigned v) { return v <= 1u ? 0 : 1 + rfk_log2_ceil((v + 1u) / 2u); }
#define RFK_HOT_SHIFT (31 - rfk_log2_ceil((unsigned)(RFK_BLOCK * RFK_CPT / RFK_HOT_COPIES) * RFK_MAX_CHECK))
static_assert(RFK_HOT_SHIFT >= 8, "hot-pixel fixed point needs at least 8 fraction bits");
#define RFK_HOT_MIN 2u
#define RFK_DISC_SLOTS 1024
#define RFK_DISC_PROBES 4
#define RFK_DISC_PASSES 2
#define RFK_HOT_EMPTY 0xFFFFFFFFu
struct rfk_hot {
    uint4 bucket[RFK_HOT_BUCKETS];                       // (pixel, sum slot, pixel, sum slot)
    unsigned acc[4][RFK_HOT_MAX * RFK_HOT_COPIES];       // channel, slot * copies + copy (fixed point)
    unsigned dtag[RFK_DISC_SLOTS];                       // discovery: pixel or empty
    unsigned dcnt[RFK_DISC_SLOTS];                       // discovery: draws counted
    unsigned nhot;
};

__device__ __forceinline__ unsigned rfk_hot_bucket(unsigned idx) {
    return (idx * 2654435761u) >> (32 - 7);  // RFK_HOT_BUCKETS = 2^7
}

__device__ __forceinline__ unsigned rfk_disc_hash(unsigned idx) {
    return (idx * 0x85EBCA77u) >> (32 - 10);  // RFK_DISC_SLOTS = 2^10
}

// All threads of the block: empty table, zero sums, empty discovery.
__device__ __forceinline__ void rfk_hot_clear(rfk_hot& hs) {
    for (unsigned i = threadIdx.x; i < RFK_HOT_BUCKETS; i += RFK_BLOCK)
        hs.bucket[i] = make_uint4(RFK_HOT_EMPTY, 0u, RFK_HOT_EMPTY, 0u);
    for (unsigned i = threadIdx.x; i < RFK_HOT_MAX * RFK_HOT_COPIES; i += RFK_BLOCK)
        hs.acc[0][i] = hs.acc[1][i] = hs.acc[2][i] = hs.acc[3][i] = 0u;
    for (unsigned i = threadIdx.x; i < RFK_DISC_SLOTS; i += RFK_BLOCK) {
        hs.dtag[i] = RFK_HOT_EMPTY;
        hs.dcnt[i] = 0u;
    }
    if (threadIdx.x == 0) hs.nhot = 0u;
}

// All threads of the block, between barriers: the sums of every hot pixel go
// out as one red.v4 each and are zeroed; with `clear` the table is emptied
// too (each thread empties only the ways it flushed).
__device__ __forceinline__ void rfk_hot_flush(rfk_hot& hs, float4* __restrict__ bins, bool clear) {
    for (unsigned b = threadIdx.x; b < RFK_HOT_BUCKETS * 2; b += RFK_BLOCK) {
        unsigned* w = reinterpret_cast<unsigned*>(&hs.bucket[b >> 1]) + 2 * (b & 1u);
        const unsigned idx = w[0], slot = w[1];
        if (idx == RFK_HOT_EMPTY) continue;
        if (clear) w[0] = RFK_HOT_EMPTY;
        float s[4];
#pragma unroll
        for (int ch = 0; ch < 4; ch++) {
            unsigned long long q = 0ull;
#pragma unroll
            for (int c = 0; c < RFK_HOT_COPIES; c++) {
                unsigned& a = hs.acc[ch][slot * RFK_HOT_COPIES + c];
                q += a;
                a = 0u;
            }
            s[ch] = __ull2float_rn(q) * (1.0f / (float)(1u << RFK_HOT_SHIFT));
        }
        if (s[3] != 0.0f || s[0] != 0.0f || s[1] != 0.0f || s[2] != 0.0f) rfk_red_v4(bins + idx, s[0], s[1], s[2], s[3]);
    }
}

// All threads of the block, uniformly, after the discovery passes: flush the
// sums, then make the table from the discovery counts and clear them. Ends
// with a barrier; the caller's draws before it must all be done (the first
// barrier below waits for them).
__device__ __forceinline__ void rfk_hot_rebuild(rfk_hot& hs, float4* __restrict__ bins) {
    __syncthreads();
    rfk_hot_flush(hs, bins, true);
    if (threadIdx.x == 0) hs.nhot = 0u;
    __syncthreads();
    for (unsigned i = threadIdx.x; i < RFK_DISC_SLOTS; i += RFK_BLOCK) {
        const unsigned idx = hs.dtag[i], n = hs.dcnt[i];
        hs.dtag[i] = RFK_HOT_EMPTY;
        hs.dcnt[i] = 0u;
        if (idx == RFK_HOT_EMPTY || n < RFK_HOT_MIN) continue;
        unsigned* w = reinterpret_cast<unsigned*>(&hs.bucket[rfk_hot_bucket(idx)]);
        // claim a way first, then a sum slot: a pixel without a free way stays cold
        int way = -1;
        if (atomicCAS(&w[0], RFK_HOT_EMPTY, RFK_HOT_EMPTY - 1u) == RFK_HOT_EMPTY) way = 0;
        else if (atomicCAS(&w[2], RFK_HOT_EMPTY, RFK_HOT_EMPTY - 1u) == RFK_HOT_EMPTY) way = 2;
        if (way < 0) continue;
        const unsigned slot = atomicAdd(&hs.nhot, 1u);
        if (slot < RFK_HOT_MAX) {
            w[way + 1] = slot;
            w[way] = idx;
        } else {
            w[way] = RFK_HOT_EMPTY;  // table full: the claimed way stays free
        }
    }
    __syncthreads();
}

// Counts one draw of a discovery pass.
__device__ __forceinline__ void rfk_disc_count(rfk_hot& hs, unsigned idx) {
    unsigned h = rfk_disc_hash(idx);
#pragma unroll 1
    for (int p = 0; p < RFK_DISC_PROBES; p++, h = (h + 1u) & (RFK_DISC_SLOTS - 1u)) {
        unsigned t = hs.dtag[h];
        if (t == RFK_HOT_EMPTY) t = atomicCAS(&hs.dtag[h], RFK_HOT_EMPTY, idx);
        if (t == RFK_HOT_EMPTY || t == idx) {
            atomicAdd(&hs.dcnt[h], 1u);
            return;
        }
    }
}
#endif

__device__ __forceinline__ void rfk_flush(float4* __restrict__ bins, int idx, float4 v
#if RFK_FLUSH == 2 || RFK_FLUSH == 3
                                          , rfk_cache& cc
#elif RFK_FLUSH == 4
                                          , rfk_hot& hs, bool disc
#endif
) {
#if RFK_FLUSH == 4
    if (idx < 0) return;
    const uint4 e = hs.bucket[rfk_hot_bucket((unsigned)idx)];
    const unsigned slot = (e.x == (unsigned)idx) ? e.y : (e.z == (unsigned)idx) ? e.w : RFK_HOT_EMPTY;
    if (slot != RFK_HOT_EMPTY && v.w <= 1.0f) {
        const unsigned a = slot * RFK_HOT_COPIES + (threadIdx.x & (RFK_HOT_COPIES - 1));
        const float sc = (float)(1u << RFK_HOT_SHIFT);
        atomicAdd(&hs.acc[0][a], __float2uint_rn(v.x * sc));
        atomicAdd(&hs.acc[1][a], __float2uint_rn(v.y * sc));
        atomicAdd(&hs.acc[2][a], __float2uint_rn(v.z * sc));
        atomicAdd(&hs.acc[3][a], __float2uint_rn(v.w * sc));
    } else {
        rfk_red_v4(bins + idx, v.x, v.y, v.z, v.w);
    }
    if (disc) rfk_disc_count(hs, (unsigned)idx);
#elif RFK_FLUSH == 3
    if (idx >= 0) rfk_cache_add(cc, bins, idx, v);
#elif RFK_FLUSH >= 1
    // lanes that hit the same pixel add their contributions first
    const unsigned active = __activemask();
    const unsigned same = __match_any_sync(active, idx);
    if (idx >= 0) {
        const int leader = __ffs(same) - 1;
        const unsigned lane = threadIdx.x & 31u;
        unsigned rest = same & ~(1u << leader);
        float4 acc = v;
        while (rest) {
            const int src = __ffs(rest) - 1;
            rest &= rest - 1;
            float4 o;
            o.x = __shfl_sync(same, v.x, src);
            o.y = __shfl_sync(same, v.y, src);
            o.z = __shfl_sync(same, v.z, src);
            o.w = __shfl_sync(same, v.w, src);
            acc.x += o.x; acc.y += o.y; acc.z += o.z; acc.w += o.w;
        }
        if ((int)lane == leader) {
#if RFK_FLUSH == 2
            rfk_cache_add(cc, bins, idx, acc);
#else
            rfk_red_v4(bins + idx, acc.x, acc.y, acc.z, acc.w);
#endif
        }
    }
#else
    if (idx >= 0) rfk_red_v4(bins + idx, v.x, v.y, v.z, v.w);
#endif
}

// --------------------------------------------------------------- warmup ----
// Hammersley point idx of `total` (refactor.cu:10-54), in [-1, 1]^2.
__device__ __forceinline__ V2 rfk_hammersley(unsigned idx, unsigned total) {
    unsigned max_val = (total % 2u == 0u) ? total : (1u << (32 - __clz(total - 1u)));
    unsigned radix = 31u - __clz(max_val);
    float inv = 1.0f / (float)max_val;
    unsigned flipped = (radix == 0u) ? 0u : (__brev(idx) >> (32u - radix));
    return fl_vec2((float)idx * inv * 2.0f - 1.0f, (float)flipped * inv * 2.0f - 1.0f);
}

// ------------------------------------------------------------------ bin ----
struct rfk_bin_args {
    const float* samples;
    rfk_chains st;
    float4* bins;
    unsigned w, h;
    unsigned seed, salt;
    unsigned call_id;                   // selects this call's Philox sub-stream
    unsigned check;                     // passes between bailout checks
    unsigned long long quality_target;  // stop when counters->quality >= this (0 = no target)
    unsigned long long max_passes;      // per-chain cap for this call (0 = no cap)
    unsigned long long time_ns;         // time budget per block (0 = none)
    const volatile unsigned* stop;      // host-written stop flag (may be null)
    rfk_counters* counters;
    unsigned tmul;                      // temporal samples per block (rfk_bin_tm)
    unsigned slice;                     // passes per temporal sample before switching (rfk_bin_tm)
};

// Shared memory of a block's passes: the block's chains, the sort counters
// and the hot-pixel cache. Chain slot q of thread t holds (x, y, colour,
// last xform as int bits; 255 = none) at rfk_slot(q): q * RFK_BLOCK + t, or,
// with the warp sort, q * 32 + lane within the warp's region. Keeping the
// chains in shared memory rather than in per-thread register arrays leaves
// only the moving chain in registers (about a third fewer registers per
// thread, more resident warps) and needs no register rotation between slots.
struct rfk_pass_smem {
    float4 chains[RFK_BLOCK * RFK_CPT];
#if RFK_SORT == 1
    unsigned counts[RFK_BLOCK / 32][32];
#elif RFK_SORT == 2
    unsigned counts[2][RFK_NX * (RFK_BLOCK / 32)];  // ping-pong sets, one per pass parity
#endif
#if RFK_FLUSH == 2 || RFK_FLUSH == 3
    rfk_cache cache;
#elif RFK_FLUSH == 4
    rfk_hot hot;
#endif
    unsigned dummy;
};

__device__ __forceinline__ unsigned rfk_slot(int q) {
#if RFK_SORT == 1
    return (threadIdx.x & ~31u) * RFK_CPT + (unsigned)q * 32u + (threadIdx.x & 31u);
#else
    return (unsigned)q * RFK_BLOCK + threadIdx.x;
#endif
}

// All threads of the block, once, before the first pass.
__device__ __forceinline__ void rfk_pass_smem_init(rfk_pass_smem& sm) {
#if RFK_SORT == 2
    for (unsigned i = threadIdx.x; i < 2 * RFK_NX * (RFK_BLOCK / 32); i += RFK_BLOCK) (&sm.counts[0][0])[i] = 0u;
#endif
#if RFK_FLUSH == 2 || RFK_FLUSH == 3
    rfk_cache_clear(sm.cache);
#elif RFK_FLUSH == 4
    rfk_hot_clear(sm.hot);
#endif
}

// This thread's chains chain0 + q * cstride (q < RFK_CPT) from the state
// arrays into its slots, and back. Only the thread's own slots are touched.
__device__ __forceinline__ void rfk_load_chains(rfk_pass_smem& sm, const rfk_chains& st, unsigned chain0,
                                                unsigned cstride) {
#pragma unroll
    for (int q = 0; q < RFK_CPT; q++) {
        const unsigned id = chain0 + (unsigned)q * cstride;
#if RFK_CHAOS
        const unsigned last = st.last[id];
#else
        const unsigned last = 255u;
#endif
        sm.chains[rfk_slot(q)] = make_float4(st.x[id], st.y[id], st.c[id], __int_as_float((int)last));
    }
}

__device__ __forceinline__ void rfk_store_chains(const rfk_pass_smem& sm, const rfk_chains& st, unsigned chain0,
                                                 unsigned cstride) {
#pragma unroll
    for (int q = 0; q < RFK_CPT; q++) {
        const unsigned id = chain0 + (unsigned)q * cstride;
        const float4 v = sm.chains[rfk_slot(q)];
        st.x[id] = v.x;
        st.y[id] = v.y;
        st.c[id] = v.z;
#if RFK_CHAOS
        st.last[id] = (unsigned char)__float_as_int(v.w);
#endif
    }
}

#if RFK_FLUSH == 2 || RFK_FLUSH == 3
#define RFK_CACHE_ARG , sm.cache
#elif RFK_FLUSH == 4
#define RFK_CACHE_ARG , sm.hot, disc
#else
#define RFK_CACHE_ARG
#endif

// Flush 4: the discovery passes of a check interval sample one chain in
// RFK_CPT, spread over the whole sorted chain order (slot q of the threads
// whose index is q modulo RFK_CPT: the sort puts the chains of the first
// xforms in the low slots, so one slot alone would see only those xforms'
// pixels); after the last of them the block rebuilds its hot-pixel table.
// Both depend only on the pass number within the interval (block-uniform).
#if RFK_FLUSH == 4
#define RFK_DISC(it, q) ((it) < RFK_DISC_PASSES && threadIdx.x % RFK_CPT == (unsigned)(q))
#define RFK_HOT_PASS_END(it, bins) \
    if ((it) + 1 == RFK_DISC_PASSES) rfk_hot_rebuild(sm.hot, (bins));
#else
#define RFK_DISC(it, q) false
#define RFK_HOT_PASS_END(it, bins)
#endif

// One pass over this thread's RFK_CPT chains, in two parts with the loop over
// slots in the kernel body:
//   rfk_pick_sort  every thread of the block (the block sort synchronises):
//                  picks of this thread's chains from one Philox stream per
//                  lane (lane_stream, call_id, pass), then the sort by xform,
//                  which leaves each slot's pick in its last-xform field;
//   rfk_move_slot  for q < RFK_CPT: the chain in slot q moves (Philox stream
//                  of the slot's chain id, call_id, pass) and draws unless
//                  `draw` is false (warm-up). Its pointers carry no
//                  __restrict__: with it the compiler kept the flame
//                  parameters in registers across the loop (about 155
//                  registers per thread instead of 60, a quarter of the
//                  occupancy).
// Without sorting (RFK_SORT 0) rfk_pick_sort does nothing and rfk_move_slot
// picks and moves the chain in slot q.
__device__ __forceinline__ void rfk_pick_sort(rfk_pass_smem& sm, const float* P, unsigned lane_stream,
                                              unsigned call_id, unsigned long long pass, unsigned seed,
                                              unsigned salt) {
#if RFK_SORT
    Rng pr;
    pr.start_lazy(lane_stream, call_id, pass, seed, salt ^ 0x9E3779B9u);
#if RFK_SORT == 2
    float3 v3[RFK_CPT];
    unsigned kb[(RFK_CPT + 1) / 2];
#pragma unroll
    for (int q = 0; q < RFK_CPT; q++) {
        // the pick takes the top 24 bits of its word; the low 8 go with the
        // chain to its move (Rng::give_bits)
        const float4 c4 = sm.chains[rfk_slot(q)];
        v3[q] = make_float3(c4.x, c4.y, c4.z);
        const rfk_u32 u = pr.next();
        const unsigned kbq = (unsigned)rfk_pick(rfk_u01f(u), P, (unsigned)__float_as_int(c4.w)) | ((u & 0xFFu) << 8);
        if (q & 1) kb[q >> 1] |= kbq << 16;
        else kb[q >> 1] = kbq;
    }
    rfk_block_sort(sm.chains, v3, kb, sm.counts[pass & 1], sm.counts[(pass + 1) & 1]);
#else
    float4 v[RFK_CPT];
    int kk[RFK_CPT];
    unsigned bits[RFK_CPT];
#pragma unroll
    for (int q = 0; q < RFK_CPT; q++) {
        v[q] = sm.chains[rfk_slot(q)];
        const rfk_u32 u = pr.next();
        kk[q] = rfk_pick(rfk_u01f(u), P, (unsigned)__float_as_int(v[q].w));
        bits[q] = u & 0xFFu;
    }
    rfk_sort_chains(sm.chains + (threadIdx.x & ~31u) * RFK_CPT, v, kk, bits, sm.counts[threadIdx.x >> 5]);
#endif
#else
    (void)sm; (void)P; (void)lane_stream; (void)call_id; (void)pass; (void)seed; (void)salt;
#endif
}

__device__ __forceinline__ void rfk_move_slot(int q, unsigned chain, rfk_pass_smem& sm, const float* P, float4* bins,
                                              unsigned w, unsigned h, unsigned call_id, unsigned long long pass,
                                              unsigned seed, unsigned salt, bool draw, bool disc, unsigned& my_hits,
                                              unsigned& my_draws) {
    (void)disc;
    float4* slot = &sm.chains[rfk_slot(q)];
    const float4 s = *slot;
    float x = s.x, y = s.y, c = s.z;
    unsigned last = (unsigned)__float_as_int(s.w);
    float4 v;
    unsigned hit;
    int idx;
    Rng rng;
#if RFK_SORT
    // the sort left this slot's pick in the last-xform field, with 8 spare
    // random bits of the pick's word above it
    rng.start_lazy(chain, call_id, pass, seed, salt);
    rng.give_bits(last >> 8);
    last &= 0xFFu;
    idx = rfk_move((int)last, x, y, c, rng, P, w, h, v, hit);
#else
    rng.start(chain, call_id, pass, seed, salt);
    idx = rfk_step(x, y, c, last, rng, P, w, h, v, hit);
#endif
    *slot = make_float4(x, y, c, __int_as_float((int)last));
    if (draw) {
        rfk_flush(bins, idx, v RFK_CACHE_ARG);
        my_hits += hit;
        my_draws += (idx >= 0) ? 1u : 0u;
    }
}

// Block totals of the check interval: warp sums, then shared atomics. Ends
// with a barrier after which s_hits / s_draws hold the block's sums and the
// hot-pixel cache is flushed.
__device__ __forceinline__ void rfk_block_totals(unsigned& my_hits, unsigned& my_draws, unsigned long long* s_hits,
                                                 unsigned long long* s_draws, rfk_pass_smem& sm, float4* bins) {
    unsigned wh = __reduce_add_sync(0xffffffffu, my_hits);
    unsigned wd = __reduce_add_sync(0xffffffffu, my_draws);
    my_hits = 0;
    my_draws = 0;
    if ((threadIdx.x & 31u) == 0) {
        atomicAdd(s_hits, (unsigned long long)wh);
        atomicAdd(s_draws, (unsigned long long)wd);
    }
    __syncthreads();
#if RFK_FLUSH == 2 || RFK_FLUSH == 3
    rfk_cache_flush(sm.cache, bins);
#elif RFK_FLUSH == 4
    rfk_hot_flush(sm.hot, bins, false);
#else
    (void)sm;
    (void)bins;
#endif
}

#ifdef RFK_MINB
#define RFK_BIN_BOUNDS __launch_bounds__(RFK_BLOCK, RFK_MINB)
#else
#define RFK_BIN_BOUNDS __launch_bounds__(RFK_BLOCK)
#endif

extern "C" __global__ void RFK_BIN_BOUNDS rfk_bin(rfk_bin_args a) {
    __shared__ __align__(16) float P[RFK_SAMPLE_FLOATS];
    __shared__ unsigned long long s_hits, s_draws;
    __shared__ unsigned s_bail;
    __shared__ unsigned long long s_start;
    __shared__ rfk_pass_smem sm;
    rfk_pass_smem_init(sm);
    const unsigned lane_stream = blockIdx.x * RFK_BLOCK + threadIdx.x;
    const float* src = a.samples + (size_t)blockIdx.x * RFK_SAMPLE_FLOATS;
    rfk_load_params(P, src);
    if (threadIdx.x == 0) {
        s_hits = 0;
        s_draws = 0;
        s_bail = 0;
        s_start = rfk_time();
        atomicMin(&a.counters->start_ns, s_start);
    }
    // chain of slot q: chain0 + q * cstride
    const unsigned chain0 = blockIdx.x * RFK_BLOCK + threadIdx.x, cstride = gridDim.x * RFK_BLOCK;
    rfk_load_chains(sm, a.st, chain0, cstride);
    __syncthreads();

    unsigned long long pass = 0;
    unsigned my_hits = 0, my_draws = 0;
#pragma unroll 1
    for (;;) {
#pragma unroll 1
        for (unsigned it = 0; it < min(a.check, RFK_MAX_CHECK) && (a.max_passes == 0 || pass < a.max_passes); it++) {
            rfk_pick_sort(sm, P, lane_stream, a.call_id, pass, a.seed, a.salt);
#pragma unroll 1
            for (int q = 0; q < RFK_CPT; q++)
                rfk_move_slot(q, chain0 + (unsigned)q * cstride, sm, P, a.bins, a.w, a.h, a.call_id, pass, a.seed,
                              a.salt, true, RFK_DISC(it, q), my_hits, my_draws);
            pass++;
            RFK_HOT_PASS_END(it, a.bins)
        }
        // bailout check: block totals -> global counters -> decision
        rfk_block_totals(my_hits, my_draws, &s_hits, &s_draws, sm, a.bins);
        if (threadIdx.x == 0) {
            unsigned long long q = atomicAdd(&a.counters->quality, s_hits) + s_hits;
            atomicAdd(&a.counters->draws, s_draws);
            s_hits = 0;
            s_draws = 0;
            unsigned bail = 0;
            if (a.quality_target && q >= a.quality_target) bail |= RFK_ST_QUALITY;
            if (a.max_passes && pass >= a.max_passes) bail |= RFK_ST_ITERS;
            if (a.time_ns && rfk_time() - s_start >= a.time_ns) bail |= RFK_ST_TIME;
            if (a.stop && *a.stop) bail |= RFK_ST_STOP;
            if (!bail && a.quality_target) {
                // another block may have met the target already
                unsigned long long gq = *((volatile unsigned long long*)&a.counters->quality);
                if (gq >= a.quality_target) bail |= RFK_ST_QUALITY;
            }
            s_bail = bail;
        }
        __syncthreads();
        if (s_bail) break;
    }
    rfk_store_chains(sm, a.st, chain0, cstride);
    if (threadIdx.x == 0) {
        atomicAdd(&a.counters->passes, pass * (unsigned long long)(RFK_BLOCK * RFK_CPT));
        atomicOr(&a.counters->status, s_bail);
        atomicMax(&a.counters->stop_ns, rfk_time());
    }
}

// --------------------------------------------------------------- warmup ----
// Chain slot k of thread t in block b holds chain (k * gridDim.x + b) *
// RFK_BLOCK + t. Each block owns one temporal sample (sample = block). Start
// points: the Hammersley point of the chain over all chains, mapped to pixel
// space and through the plane-space affine (refactor.cu:301-308), colour
// ~ U(0,1); then warmup_count passes that move the chains without drawing
// (refactor.cu:311-335), on the pass code of rfk_bin (Philox sub-stream
// 0xFFFE, which bin calls never use).
extern "C" __global__ void RFK_BIN_BOUNDS rfk_warmup(const float* __restrict__ samples, rfk_chains st, unsigned w,
                                                     unsigned h, unsigned seed, unsigned salt, unsigned warmup_count) {
    __shared__ __align__(16) float P[RFK_SAMPLE_FLOATS];
    __shared__ rfk_pass_smem sm;
    rfk_pass_smem_init(sm);
    const float* src = samples + (size_t)blockIdx.x * RFK_SAMPLE_FLOATS;
    rfk_load_params(P, src);
    __syncthreads();
    const unsigned total = gridDim.x * RFK_BLOCK * RFK_CPT;
    const unsigned lane_stream = blockIdx.x * RFK_BLOCK + threadIdx.x;
    const unsigned chain0 = blockIdx.x * RFK_BLOCK + threadIdx.x, cstride = gridDim.x * RFK_BLOCK;
#pragma unroll
    for (int q = 0; q < RFK_CPT; q++) {
        const unsigned chain = chain0 + (unsigned)q * cstride;
        Rng rng;
        rng.start(chain, 0xFFFDu, 0ull, seed, salt);
        const V2 pos = rfk_hammersley(chain, total);
        const float px = (pos.x + 1.0f) / 2.0f * (float)w;
        const float py = (pos.y + 1.0f) / 2.0f * (float)h;
        // plane-space affine at P[6..11]
        sm.chains[rfk_slot(q)] = make_float4(fmaf(P[6], px, fmaf(P[8], py, P[10])), fmaf(P[7], px, fmaf(P[9], py, P[11])),
                                             rng.u01(), __int_as_float(255));
    }
    unsigned no_hits = 0, no_draws = 0;
#pragma unroll 1
    for (unsigned pass = 0; pass < warmup_count; pass++) {
        rfk_pick_sort(sm, P, lane_stream, 0xFFFEu, pass, seed, salt);
#pragma unroll 1
        for (int q = 0; q < RFK_CPT; q++) {
            rfk_move_slot(q, chain0 + (unsigned)q * cstride, sm, P, nullptr, w, h, 0xFFFEu, pass, seed, salt, false,
                          false, no_hits, no_draws);
            // without the histogram updates (asm with a memory clobber) the
            // compiler would keep the flame parameters in registers across
            // passes: twice the registers, half the occupancy
            asm volatile("" ::: "memory");
        }
    }
    rfk_store_chains(sm, st, chain0, cstride);
}

// ------------------------------------------------- temporal multiplier ----
// flame_kernel::bin with temporal_multiplier T > 1 (refactor.cu:404-475,
// flamelib.h:203-260): the state holds T x grid temporal samples, each with
// its own parameter block and chains; block b owns samples b + grid * i
// (i < T) and cycles through them, `slice` passes at a time, saving and
// loading the chains in global memory. Each (block, sample) pair stops at an
// equal share of the quality target, so every temporal sample contributes
// alike (the motion-blur average); the block ends when all its samples are
// done or on the pass cap, time budget or stop flag.
#define RFK_MAX_TMUL 32
extern "C" __global__ void RFK_BIN_BOUNDS rfk_bin_tm(rfk_bin_args a) {
    __shared__ __align__(16) float P[RFK_SAMPLE_FLOATS];
    __shared__ unsigned long long s_hits, s_draws, s_start;
    __shared__ unsigned long long s_q[RFK_MAX_TMUL];
    __shared__ unsigned s_bail, s_done;
    __shared__ int s_next;
    __shared__ rfk_pass_smem sm;
    rfk_pass_smem_init(sm);
    const unsigned T = a.tmul;
    const unsigned S = gridDim.x * T;
    const unsigned lane_stream = blockIdx.x * RFK_BLOCK + threadIdx.x;
    const unsigned long long share = a.quality_target ? (a.quality_target + S - 1) / S : 0ull;
    if (threadIdx.x == 0) {
        s_hits = 0;
        s_draws = 0;
        s_bail = 0;
        s_done = 0;
        s_start = rfk_time();
        atomicMin(&a.counters->start_ns, s_start);
    }
    for (unsigned i = threadIdx.x; i < RFK_MAX_TMUL; i += RFK_BLOCK) s_q[i] = 0;
    int cur = 0;
    unsigned smp = blockIdx.x;
    // chain of slot q of temporal sample smp: smp * RFK_BLOCK + t + q * cstride
    const unsigned cstride = S * RFK_BLOCK;
    rfk_load_params(P, a.samples + (size_t)smp * RFK_SAMPLE_FLOATS);
    rfk_load_chains(sm, a.st, smp * RFK_BLOCK + threadIdx.x, cstride);
    __syncthreads();

    unsigned long long pass = 0, total = 0;
    unsigned in_slice = 0;
    unsigned my_hits = 0, my_draws = 0;
#pragma unroll 1
    for (;;) {
        unsigned n = 0;
#pragma unroll 1
        for (; n < min(a.check, RFK_MAX_CHECK) && (a.max_passes == 0 || total < a.max_passes); n++) {
            rfk_pick_sort(sm, P, lane_stream, a.call_id, pass, a.seed, a.salt);
            const unsigned chain0 = smp * RFK_BLOCK + threadIdx.x;
#pragma unroll 1
            for (int q = 0; q < RFK_CPT; q++)
                rfk_move_slot(q, chain0 + (unsigned)q * cstride, sm, P, a.bins, a.w, a.h, a.call_id, pass, a.seed,
                              a.salt, true, RFK_DISC(n, q), my_hits, my_draws);
            pass++;
            total++;
            RFK_HOT_PASS_END(n, a.bins)
        }
        in_slice += n;
        rfk_block_totals(my_hits, my_draws, &s_hits, &s_draws, sm, a.bins);
        if (threadIdx.x == 0) {
            atomicAdd(&a.counters->quality, s_hits);
            atomicAdd(&a.counters->draws, s_draws);
            s_q[cur] += s_hits;
            s_hits = 0;
            s_draws = 0;
            unsigned done = s_done;
            if (share && s_q[cur] >= share) done |= 1u << cur;
            s_done = done;
            unsigned bail = 0;
            if (done == (T >= 32 ? 0xFFFFFFFFu : ((1u << T) - 1u))) bail |= RFK_ST_QUALITY;
            if (a.max_passes && total >= a.max_passes) bail |= RFK_ST_ITERS;
            if (a.time_ns && rfk_time() - s_start >= a.time_ns) bail |= RFK_ST_TIME;
            if (a.stop && *a.stop) bail |= RFK_ST_STOP;
            s_bail = bail;
            int nxt = cur;
            if (!bail && ((done >> cur) & 1u || in_slice >= a.slice)) {
                // next sample not yet done, round robin
                for (unsigned j = 1; j <= T; j++) {
                    const int cand = (int)((cur + j) % T);
                    if (!((done >> cand) & 1u)) {
                        nxt = cand;
                        break;
                    }
                }
            }
            s_next = nxt;
        }
        __syncthreads();
        if (s_bail) break;
        const int nxt = s_next;
        if (nxt != cur) {
            // park this sample's chains, bring in the next sample
            rfk_store_chains(sm, a.st, smp * RFK_BLOCK + threadIdx.x, cstride);
            cur = nxt;
            smp = blockIdx.x + gridDim.x * (unsigned)cur;
            rfk_load_params(P, a.samples + (size_t)smp * RFK_SAMPLE_FLOATS);
            rfk_load_chains(sm, a.st, smp * RFK_BLOCK + threadIdx.x, cstride);
            in_slice = 0;
            __syncthreads();
        } else if (in_slice >= a.slice) {
            in_slice = 0;
        }
    }
    rfk_store_chains(sm, a.st, smp * RFK_BLOCK + threadIdx.x, cstride);
    if (threadIdx.x == 0) {
        atomicAdd(&a.counters->passes, total * (unsigned long long)(RFK_BLOCK * RFK_CPT));
        atomicOr(&a.counters->status, s_bail);
        atomicMax(&a.counters->stop_ns, rfk_time());
    }
}

// ------------------------------------------------------------ batch bin ----
// Many flames or frames (units) of one structure in one persistent launch.
// The work is a queue of items, each `passes_per_item` passes of one block's
// chains on one unit; items are numbered unit after unit. A block takes the
// next item with one atomic, skips it when its unit has reached its quality
// target, loads the unit's parameter block (with a fresh antialiasing jitter
// at the start and at every quality check), and keeps its chains when the item is of the unit it just worked on (new
// chains start uniformly over the image, through the plane-space affine, and
// run `warmup` passes without drawing). A unit's histogram only sees its own
// items; quality (the sum of 255 * opacity over draws) counts per unit.
struct rfk_unit {
    const float* params;                 // prepared parameter block (no jitter)
    float4* bins;                        // w x h histogram, row-major
    unsigned w, h;
    unsigned long long quality_target;   // per-unit target of the quality sum
    unsigned long long first_item;       // first queue item of this unit
    unsigned check;                      // passes between quality checks
    unsigned pad;
};

struct rfk_unit_counters {
    unsigned long long quality;  // sum of (u32)(255 * opacity) over draws
    unsigned long long draws;
    unsigned long long passes;   // chain steps, warm-up included
    unsigned long long items;    // items worked on
};

struct rfk_batch_args {
    const rfk_unit* units;
    rfk_unit_counters* uc;
    unsigned nunits;
    unsigned passes_per_item;
    unsigned long long nitems;
    unsigned long long* next_item;  // queue head, zero at launch
    unsigned warmup;                // warm-up passes for new chains
    unsigned seed, salt;
    const unsigned* call_id;        // device word: Philox sub-stream of this run
    unsigned long long time_ns;     // time budget per block (0 = none)
    const volatile unsigned* stop;  // host-written stop flag (may be null)
    rfk_counters* counters;         // batch totals: passes, start, stop, status
};

// Antialiasing jitter ~ gauss(1/3 px) of the screen affine (as each temporal
// sample of the single-flame path has one), drawn afresh at the start of an
// item and at every quality check, so that a small unit worked on by few
// blocks still averages over many jitters. Philox stream (item, 0xFFFF,
// call_id : block pass), unique per draw.
__device__ __forceinline__ void rfk_batch_jitter(float* P, const float* __restrict__ base, unsigned long long item,
                                                 unsigned call_id, unsigned long long pass, unsigned seed,
                                                 unsigned salt) {
    Rng jr;
    jr.start((unsigned)item, 0xFFFFu, ((unsigned long long)call_id << 32) | (unsigned)pass, seed, salt);
    const V2 j = jr.gauss(1.0f / 3.0f);
    P[4] = base[4] + j.x;
    P[5] = base[5] + j.y;
}

extern "C" __global__ void RFK_BIN_BOUNDS rfk_bin_batch(rfk_batch_args a) {
    __shared__ __align__(16) float P[RFK_SAMPLE_FLOATS];
    __shared__ unsigned long long s_hits, s_draws, s_start, s_item;
    __shared__ int s_unit;
    __shared__ unsigned s_bail;
    __shared__ rfk_pass_smem sm;
    rfk_pass_smem_init(sm);
    const unsigned lane_stream = blockIdx.x * RFK_BLOCK + threadIdx.x;
    const unsigned call_id = *a.call_id;
    if (threadIdx.x == 0) {
        s_hits = 0;
        s_draws = 0;
        s_start = rfk_time();
        atomicMin(&a.counters->start_ns, s_start);
    }
    const unsigned chain0 = blockIdx.x * RFK_BLOCK + threadIdx.x, cstride = gridDim.x * RFK_BLOCK;
    int cur = -1;
    unsigned long long pass = 0;  // the block's running pass count
    unsigned long long total_passes = 0;
    unsigned status = 0;
    unsigned my_hits = 0, my_draws = 0;
#pragma unroll 1
    for (;;) {
        __syncthreads();  // everyone is done with the previous item's parameters
        if (threadIdx.x == 0) {
            int u = -1;
            unsigned long long item = 0;
            unsigned bail = 0;
            if (a.stop && *a.stop) bail |= RFK_ST_STOP;
            if (a.time_ns && rfk_time() - s_start >= a.time_ns) bail |= RFK_ST_TIME;
            while (!bail) {
                item = atomicAdd(a.next_item, 1ull);
                if (item >= a.nitems) break;
                // the unit of the item: the last one whose first item <= item
                int lo = 0, hi = (int)a.nunits - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (a.units[mid].first_item <= item) lo = mid;
                    else hi = mid - 1;
                }
                const unsigned long long q = *((volatile unsigned long long*)&a.uc[lo].quality);
                if (q < a.units[lo].quality_target) {
                    u = lo;
                    break;
                }
            }
            status |= bail;
            s_unit = u;
            s_item = item;
        }
        __syncthreads();
        const int u = s_unit;
        if (u < 0) break;
        const unsigned long long item = s_item;
        const rfk_unit U = a.units[u];
        rfk_load_params(P, U.params);
        __syncthreads();
        if (threadIdx.x == 0) rfk_batch_jitter(P, U.params, item, call_id, pass, a.seed, a.salt);
        __syncthreads();
        unsigned warm = 0;
        if (u != cur) {
#pragma unroll
            for (int q = 0; q < RFK_CPT; q++) {
                Rng r0;
                r0.start(chain0 + (unsigned)q * cstride, 0xFFFDu, ((unsigned long long)call_id << 32) | (unsigned)item,
                         a.seed, a.salt);
                const float px = r0.u01() * (float)U.w, py = r0.u01() * (float)U.h;
                const float cx = fmaf(P[6], px, fmaf(P[8], py, P[10]));
                const float cy = fmaf(P[7], px, fmaf(P[9], py, P[11]));
                sm.chains[rfk_slot(q)] = make_float4(cx, cy, r0.u01(), __int_as_float(255));
            }
            warm = a.warmup;
            cur = u;
        }
        const unsigned total = warm + a.passes_per_item;
        unsigned done = 0;
        unsigned ended = 0;
#pragma unroll 1
        while (done < total) {
            const unsigned n = min(min(U.check, RFK_MAX_CHECK), total - done);
#pragma unroll 1
            for (unsigned it = 0; it < n; it++) {
                const bool draw = done + it >= warm;
                rfk_pick_sort(sm, P, lane_stream, call_id, pass, a.seed, a.salt);
#pragma unroll 1
                for (int q = 0; q < RFK_CPT; q++)
                    rfk_move_slot(q, chain0 + (unsigned)q * cstride, sm, P, U.bins, U.w, U.h, call_id, pass, a.seed,
                                  a.salt, draw, RFK_DISC(it, q), my_hits, my_draws);
                pass++;
                RFK_HOT_PASS_END(it, U.bins)
            }
            done += n;
            rfk_block_totals(my_hits, my_draws, &s_hits, &s_draws, sm, U.bins);
            if (threadIdx.x == 0) {
                const unsigned long long q = atomicAdd(&a.uc[u].quality, s_hits) + s_hits;
                atomicAdd(&a.uc[u].draws, s_draws);
                atomicAdd(&a.uc[u].passes, (unsigned long long)n * (RFK_BLOCK * RFK_CPT));
                s_hits = 0;
                s_draws = 0;
                unsigned bail = 0;
                if (q >= U.quality_target) bail |= RFK_ST_QUALITY;
                if (a.stop && *a.stop) bail |= RFK_ST_STOP;
                if (a.time_ns && rfk_time() - s_start >= a.time_ns) bail |= RFK_ST_TIME;
                s_bail = bail;
                // a new jitter for the next interval: the other threads wait at
                // the barrier below and read P only after it
                if (!bail && done < total) rfk_batch_jitter(P, U.params, item, call_id, pass, a.seed, a.salt);
            }
            __syncthreads();
            ended = s_bail;
            if (ended) break;
        }
        total_passes += done;
        if (threadIdx.x == 0) atomicAdd(&a.uc[u].items, 1ull);
        if (ended & (RFK_ST_STOP | RFK_ST_TIME)) {
            if (threadIdx.x == 0) status |= ended;
            break;
        }
    }
    if (threadIdx.x == 0) {
        atomicAdd(&a.counters->passes, total_passes * (unsigned long long)(RFK_BLOCK * RFK_CPT));
        atomicOr(&a.counters->status, status);
        atomicMax(&a.counters->stop_ns, rfk_time());
    }
}

// ------------------------------------------------------ single application --
// Applies one xform (or the final xform, xform < 0) of one prepared parameter
// block to n points (x, y, colour): the single-map unit of the parity tests.
// Random draws come from Philox stream (point index, sub 0xFFFC).
extern "C" __global__ void __launch_bounds__(256) rfk_apply(const float* __restrict__ params, int xform,
                                                            const float* __restrict__ in, float* __restrict__ out,
                                                            unsigned n, unsigned seed) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Rng rng;
    rng.start(i, 0xFFFCu, 0ull, seed, 0u);
    V2 p = fl_vec2(in[3 * i], in[3 * i + 1]);
    R c = in[3 * i + 2];
    R op = 0.0f;
    if (xform < 0) {
#if RFK_HAS_FINAL
        op = rfk_final(p, c, params, rng);
#endif
    } else {
        op = rfk_dispatch(xform, p, c, params, rng);
    }
    out[4 * i] = p.x;
    out[4 * i + 1] = p.y;
    out[4 * i + 2] = c;
    out[4 * i + 3] = op;
}
