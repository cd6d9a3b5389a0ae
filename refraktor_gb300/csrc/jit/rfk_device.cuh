// rfk device prelude: real type, 2-vector, DSL math library, Philox RNG.
//
// This header is text that the flame compiler prepends to every generated
// chaos-game kernel (NVRTC, sm_103a). The same text also compiles as plain
// C++ (RFK_HOST_TWIN defined) so that the variation code emitted by the DSL
// translator can be evaluated on the CPU in FP64 for parity tests.
//
// Semantics follow the reference device library:
//   flamelib.h:337-404  math overloads (scalar and per-component vec2)
//   flamelib.h:412-450  sincos / cossin / sincospi / cossinpi (vec2 results)
//   flamelib.h:481-489  eps(): exact zero -> 1e-20, other values unchanged
//   flamelib.h:392-408  trunc / rint return int, is_even on int
//   flamelib.h:21       INTERP(a, b, mix) colour blend
//   flamelib.h:25       badvalue(): NaN or |v| > 1e10
// The RNG is replaced: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC 2011), a counter-based generator,
// instead of the per-thread xoroshiro64* state of random.h:39-55.
#pragma once

#ifdef RFK_HOST_TWIN
#include <cmath>
#include <cstdint>
#define RFK_FN inline
#define RFK_RESTRICT __restrict__
typedef uint32_t rfk_u32;
typedef uint64_t rfk_u64;
#else
#define RFK_FN __device__ __forceinline__
#define RFK_RESTRICT __restrict__
typedef unsigned int rfk_u32;
typedef unsigned long long rfk_u64;
#endif

#ifndef RFK_REAL
#define RFK_REAL float
#endif
typedef RFK_REAL R;

#define RFK_PI_D 3.14159265358979323846264338327950288
#define RFK_INV_PI_D 0.318309886183790671537767526745028724
#define RFK_PI R(RFK_PI_D)
#define RFK_INV_PI R(RFK_INV_PI_D)

struct V2 {
    R x, y;
};

RFK_FN V2 fl_vec2(R x, R y) { V2 v; v.x = x; v.y = y; return v; }
RFK_FN V2 operator+(V2 a, V2 b) { return fl_vec2(a.x + b.x, a.y + b.y); }
RFK_FN V2 operator-(V2 a, V2 b) { return fl_vec2(a.x - b.x, a.y - b.y); }
RFK_FN V2 operator-(V2 a) { return fl_vec2(-a.x, -a.y); }
RFK_FN V2 operator*(V2 a, R s) { return fl_vec2(a.x * s, a.y * s); }
RFK_FN V2 operator*(R s, V2 a) { return fl_vec2(s * a.x, s * a.y); }
RFK_FN V2 operator/(V2 a, R s) { return fl_vec2(a.x / s, a.y / s); }
RFK_FN V2& operator+=(V2& a, V2 b) { a.x += b.x; a.y += b.y; return a; }
RFK_FN V2& operator-=(V2& a, V2 b) { a.x -= b.x; a.y -= b.y; return a; }
RFK_FN V2& operator*=(V2& a, R s) { a.x *= s; a.y *= s; return a; }
RFK_FN V2& operator/=(V2& a, R s) { a.x /= s; a.y /= s; return a; }

// ---- scalar math, mapped per real type --------------------------------------
#ifdef RFK_HOST_TWIN
#define RFK_M1(name, expr) \
    RFK_FN R fl_##name(R a) { return (R)(expr); } \
    RFK_FN V2 fl_##name(V2 a) { return fl_vec2(fl_##name(a.x), fl_##name(a.y)); }
RFK_M1(sin, std::sin(a))
RFK_M1(cos, std::cos(a))
RFK_M1(tan, std::tan(a))
RFK_M1(sinh, std::sinh(a))
RFK_M1(cosh, std::cosh(a))
RFK_M1(acos, std::acos(a))
RFK_M1(exp, std::exp(a))
RFK_M1(log, std::log(a))
RFK_M1(log2, std::log2(a))
RFK_M1(log10, std::log10(a))
RFK_M1(sqrt, std::sqrt(a))
RFK_M1(rsqrt, 1.0 / std::sqrt(a))
RFK_M1(abs, std::fabs(a))
RFK_M1(sinpi, std::sin(RFK_PI_D * a))
RFK_M1(cospi, std::cos(RFK_PI_D * a))
RFK_FN R fl_floor(R a) { return std::floor(a); }
RFK_FN int fl_trunc(R a) { return (int)std::trunc(a); }
RFK_FN int fl_rint(R a) { return (int)std::rint(a); }
RFK_FN R fl_pow(R a, R b) { return std::pow(a, b); }
RFK_FN R fl_atan2(R a, R b) { return std::atan2(a, b); }
RFK_FN R fl_hypot(R a, R b) { return std::hypot(a, b); }
RFK_FN R fl_modf(R a, R b) { return std::fmod(a, b); }
RFK_FN R fl_copysign(R a, R b) { return std::copysign(a, b); }
RFK_FN R fl_fma(R a, R b, R c) { return std::fma(a, b, c); }
RFK_FN V2 fl_sincos(R a) { return fl_vec2(std::sin(a), std::cos(a)); }
RFK_FN V2 fl_sincospi(R a) { return fl_vec2(std::sin(RFK_PI_D * a), std::cos(RFK_PI_D * a)); }
#else
#define RFK_M1(name, fexpr, dexpr) \
    RFK_FN float rfk_##name##_f(float a) { return fexpr; } \
    RFK_FN double rfk_##name##_d(double a) { return dexpr; } \
    RFK_FN R fl_##name(R a) { return sizeof(R) == 4 ? (R)rfk_##name##_f((float)a) : (R)rfk_##name##_d((double)a); } \
    RFK_FN V2 fl_##name(V2 a) { return fl_vec2(fl_##name(a.x), fl_##name(a.y)); }
RFK_M1(sin, sinf(a), sin(a))
RFK_M1(cos, cosf(a), cos(a))
RFK_M1(tan, tanf(a), tan(a))
RFK_M1(sinh, sinhf(a), sinh(a))
RFK_M1(cosh, coshf(a), cosh(a))
RFK_M1(acos, acosf(a), acos(a))
RFK_M1(exp, expf(a), exp(a))
RFK_M1(log, logf(a), log(a))
RFK_M1(log2, log2f(a), log2(a))
RFK_M1(log10, log10f(a), log10(a))
RFK_M1(sqrt, sqrtf(a), sqrt(a))
RFK_M1(rsqrt, rsqrtf(a), rsqrt(a))
RFK_M1(abs, fabsf(a), fabs(a))
RFK_M1(sinpi, sinpif(a), sinpi(a))
RFK_M1(cospi, cospif(a), cospi(a))
RFK_FN R fl_floor(R a) { return sizeof(R) == 4 ? (R)floorf((float)a) : (R)floor((double)a); }
RFK_FN int fl_trunc(R a) { return sizeof(R) == 4 ? (int)truncf((float)a) : (int)trunc((double)a); }
RFK_FN int fl_rint(R a) { return sizeof(R) == 4 ? (int)rintf((float)a) : (int)rint((double)a); }
RFK_FN R fl_pow(R a, R b) { return sizeof(R) == 4 ? (R)powf((float)a, (float)b) : (R)pow((double)a, (double)b); }
RFK_FN R fl_atan2(R a, R b) { return sizeof(R) == 4 ? (R)atan2f((float)a, (float)b) : (R)atan2((double)a, (double)b); }
#ifdef RFK_FAST_HYPOT
// fast build: sqrt(a^2 + b^2) without hypot's overflow scaling; chain
// positions beyond 1e10 are reset before they can square to overflow
RFK_FN R fl_hypot(R a, R b) { return sizeof(R) == 4 ? (R)sqrtf(fmaf((float)a, (float)a, (float)b * (float)b)) : (R)hypot((double)a, (double)b); }
#else
RFK_FN R fl_hypot(R a, R b) { return sizeof(R) == 4 ? (R)hypotf((float)a, (float)b) : (R)hypot((double)a, (double)b); }
#endif
RFK_FN R fl_modf(R a, R b) { return sizeof(R) == 4 ? (R)fmodf((float)a, (float)b) : (R)fmod((double)a, (double)b); }
RFK_FN R fl_copysign(R a, R b) { return sizeof(R) == 4 ? (R)copysignf((float)a, (float)b) : (R)copysign((double)a, (double)b); }
RFK_FN R fl_fma(R a, R b, R c) { return sizeof(R) == 4 ? (R)fmaf((float)a, (float)b, (float)c) : (R)fma((double)a, (double)b, (double)c); }
RFK_FN V2 fl_sincos(R a) {
    if (sizeof(R) == 4) { float s, c; sincosf((float)a, &s, &c); return fl_vec2((R)s, (R)c); }
    double s, c; sincos((double)a, &s, &c); return fl_vec2((R)s, (R)c);
}
RFK_FN V2 fl_sincospi(R a) {
    if (sizeof(R) == 4) { float s, c; sincospif((float)a, &s, &c); return fl_vec2((R)s, (R)c); }
    double s, c; sincospi((double)a, &s, &c); return fl_vec2((R)s, (R)c);
}
#endif

RFK_FN V2 fl_cossin(R a) { V2 v = fl_sincos(a); return fl_vec2(v.y, v.x); }
RFK_FN V2 fl_cossinpi(R a) { V2 v = fl_sincospi(a); return fl_vec2(v.y, v.x); }
RFK_FN V2 fl_elmul(V2 a, V2 b) { return fl_vec2(a.x * b.x, a.y * b.y); }
RFK_FN bool fl_is_even(int x) { return !(x & 1); }
RFK_FN R fl_eps(R a) { return (a == R(0)) ? R(1e-20) : a; }
RFK_FN V2 fl_eps(V2 a) { return fl_vec2(fl_eps(a.x), fl_eps(a.y)); }
RFK_FN bool rfk_badvalue(R v) { return (v != v) || (v > R(1e10)) || (v < R(-1e10)); }

// ---- Philox4x32-10 ----------------------------------------------------------
// Round function and key schedule as published by Salmon et al. (SC 2011):
// multipliers 0xD2511F53 / 0xCD9E8D57, Weyl increments 0x9E3779B9 / 0xBB67AE85.
struct rfk_u32x4 { rfk_u32 x, y, z, w; };

RFK_FN rfk_u32 rfk_mulhi(rfk_u32 a, rfk_u32 b) {
#ifdef RFK_HOST_TWIN
    return (rfk_u32)(((rfk_u64)a * (rfk_u64)b) >> 32);
#else
    return __umulhi(a, b);
#endif
}

RFK_FN rfk_u32x4 rfk_philox(rfk_u32x4 c, rfk_u32 k0, rfk_u32 k1) {
#pragma unroll
    for (int i = 0; i < 10; i++) {
        rfk_u32 hi0 = rfk_mulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        rfk_u32 hi1 = rfk_mulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        rfk_u32x4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Uniform in [0, 1): the top 24 bits of a 32-bit draw, exact in FP32.
RFK_FN float rfk_u01f(rfk_u32 u) { return (float)(u >> 8) * 5.9604644775390625e-8f; }

// A chain's random stream for one pass: four words from one Philox block,
// refilled from the next sub-counter when used up. Shifting the words keeps
// every access at a static register index. `pool` holds spare random bits
// handed over by the caller (above a marker bit; 0 or 1 = none), which bit()
// uses before it draws a word: the xform pick of the sorted kernels takes the
// top 24 bits of its word and passes the low 8 on, so a variation's random
// bit (julia) costs no Philox block.
struct Rng {
    rfk_u32 b0, b1, b2, b3;
    rfk_u32 left;
    rfk_u32x4 ctr;
    rfk_u32 k0, k1;
    rfk_u32 pool;

    RFK_FN void start(rfk_u32 stream, rfk_u32 sub, rfk_u64 pass, rfk_u32 key0, rfk_u32 key1) {
        ctr.x = stream; ctr.y = sub; ctr.z = (rfk_u32)pass; ctr.w = (rfk_u32)(pass >> 32);
        k0 = key0; k1 = key1;
        pool = 0u;
        refill();
    }
    // As start(), but the first block is generated on the first draw: a chain
    // step whose variations draw nothing costs no Philox rounds.
    RFK_FN void start_lazy(rfk_u32 stream, rfk_u32 sub, rfk_u64 pass, rfk_u32 key0, rfk_u32 key1) {
        ctr.x = stream; ctr.y = sub; ctr.z = (rfk_u32)pass; ctr.w = (rfk_u32)(pass >> 32);
        k0 = key0; k1 = key1;
        b0 = b1 = b2 = b3 = 0u;
        left = 0;
        pool = 0u;
    }
    // Eight spare random bits for bit().
    RFK_FN void give_bits(rfk_u32 bits8) { pool = (bits8 & 0xFFu) | 0x100u; }
    RFK_FN void refill() {
        rfk_u32x4 r = rfk_philox(ctr, k0, k1);
        b0 = r.x; b1 = r.y; b2 = r.z; b3 = r.w; left = 4;
        ctr.y += 0x10000u;
    }
    RFK_FN rfk_u32 next() {
        if (left == 0) refill();
        rfk_u32 r = b0; b0 = b1; b1 = b2; b2 = b3; left--;
        return r;
    }
    RFK_FN R u01() { return (R)rfk_u01f(next()); }
    RFK_FN R bit() {
        if (pool > 1u) {
            const rfk_u32 r = pool & 1u;
            pool >>= 1;
            return (R)r;
        }
        return (R)((next() >> 24) & 1u);
    }
    // Same distribution as random.h:9-14: angle 2*pi*u, radius sigma * (sum of
    // four uniforms - 2).
    RFK_FN V2 gauss(R sigma) {
        V2 sc = fl_sincospi(u01() * R(2));
        R r = sigma * (u01() + u01() + u01() + u01() - R(2));
        return fl_vec2(r * sc.y, r * sc.x);
    }
};

#define RNG_U01() (rng.u01())
#define RNG_BIT() (rng.bit())
#define RNG_GAUSS() (rng.gauss(R(1)))
