/*
 * FP64 CPU oracle of the flame-rendering hot path. TEST INFRASTRUCTURE ONLY
 * (see oracle.h): the oracle librfk's CUDA kernels are tested against, and the timed CPU
 * baseline. Not part of the library.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

static const double PI = 3.14159265358979323846;

static const char* kNames[ORACLE_NUM_VARIATIONS] = {
    "linear",   "sinusoidal", "spherical", "swirl", "horseshoe", "polar", "handkerchief", "heart", "disc",
    "spiral",   "hyperbolic", "julia",     "exponential", "power", "fisheye", "bubble", "diamond", "ex",
    "bent",     "cylinder",   "exp",       "eyefish", "blur", "gaussian_blur", "cosine"};

const char* oracle_variation_name(int id) { return (id >= 0 && id < ORACLE_NUM_VARIATIONS) ? kNames[id] : NULL; }

int oracle_variation_id(const char* name) {
    for (int i = 0; i < ORACLE_NUM_VARIATIONS; i++)
        if (strcmp(kNames[i], name) == 0) return i;
    return -1;
}

/* ------------------------------------------------------------ Catmull-Rom */
/* catmull.cu:11-28 with tension 0, alpha 0.5 */
static void segment(double p0, double p1, double p2, double p3, double out[4]) {
    const double t01 = pow(hypot(p1 - p0, 1.0), 0.5);
    const double t12 = pow(hypot(p2 - p1, 1.0), 0.5);
    const double t23 = pow(hypot(p3 - p2, 1.0), 0.5);
    const double m1 = p2 - p1 + t12 * ((p1 - p0) / t01 - (p2 - p0) / (t01 + t12));
    const double m2 = p2 - p1 + t12 * ((p3 - p2) / t23 - (p3 - p1) / (t12 + t23));
    out[0] = 2.0 * (p1 - p2) + m1 + m2;
    out[1] = -3.0 * (p1 - p2) - m1 - m1 - m2;
    out[2] = m1;
    out[3] = p1;
}

void oracle_catmull(const double* s, size_t n, size_t nseg, double* coeff) {
    for (size_t g = 0; g < nseg; g++)
        for (size_t r = 0; r < n; r++) {
            const size_t b = g * n + r;
            segment(s[b], s[b + n], s[b + 2 * n], s[b + 3 * n], coeff + 4 * b);
        }
}

/* flame_compiler.cpp:957-1035 */
void oracle_fix_rotation(double* s, size_t n, size_t ss, size_t fs, const size_t* aff, size_t na) {
    const double eps = 1e-10;
    for (size_t a = 0; a < na; a++) {
        const size_t idx = aff[a];
        for (size_t i = 0; i < n; i++) {
            double* o = s + idx + i * ss;
            double ax = atan2(o[1], o[0]), mx = sqrt(o[0] * o[0] + o[1] * o[1]);
            double ay = atan2(o[3], o[2]), my = sqrt(o[2] * o[2] + o[3] * o[3]);
            if (mx == 0.0 && my != 0.0) ax = ay;
            if (my == 0.0 && mx != 0.0) ay = ax;
            o[0] = ax;
            o[1] = ay;
            o[2] = log(mx);
            o[3] = log(my);
        }
        for (size_t i = 1; i < n; i++)
            for (int j = 0; j < 2; j++) {
                double* me = s + idx + i * ss + j;
                const double d = *me - s[idx + (i - 1) * ss + j];
                if (d > PI + eps) *me -= 2 * PI;
                else if (d < -(PI - eps)) *me += 2 * PI;
            }
    }
    for (size_t i = fs; i < ss; i += 3)
        for (size_t j = 1; j < n; j++) {
            double* me = s + i + j * ss;
            const double d = *me - s[i + (j - 1) * ss];
            if (d > 180.0 + eps) *me -= 360.0;
            else if (d < -(180.0 - eps)) *me += 360.0;
        }
}

/* refactor.cu:128-140 */
void oracle_hsv_to_rgb8(double h, double s, double v, double rgb[3]) {
    const double ns[3] = {5.0, 3.0, 1.0};
    for (int j = 0; j < 3; j++) {
        double k = fmod(ns[j] + h / 60.0, 6.0);
        double f = v - v * s * fmax(0.0, fmin(k, fmin(4.0 - k, 1.0)));
        double x = f * 255.0;
        if (x < 0) x = 0;
        if (x > 255) x = 255;
        rgb[j] = (double)(unsigned char)x / 255.0;
    }
}

static double cubic(const double* k, double t) { return ((k[0] * t + k[1]) * t + k[2]) * t + k[3]; }

void oracle_interpolate(const double* coeff, size_t ss, size_t R, size_t seg, double t, const size_t* aff, size_t na,
                        double* params, double* pal) {
    const double* c = coeff + seg * ss * 4;
    for (size_t i = 0; i < R; i++) params[i] = cubic(c + 4 * i, t);
    for (size_t a = 0; a < na; a++) {
        double* o = params + aff[a];
        const double angx = o[0], angy = o[1], magx = exp(o[2]), magy = exp(o[3]);
        o[0] = magx * cos(angx);
        o[1] = magx * sin(angx);
        o[2] = magy * cos(angy);
        o[3] = magy * sin(angy);
    }
    for (int i = 0; i < 256; i++) {
        double hsv[3];
        for (int j = 0; j < 3; j++) hsv[j] = cubic(c + 4 * (R + 3 * i + j), t);
        oracle_hsv_to_rgb8(hsv[0], hsv[1], hsv[2], pal + 3 * i);
    }
}

/* --------------------------------------------------------------- structure */
#define MAX_XF 64
#define MAX_VL 8
#define MAX_VAR 16

typedef struct {
    int n_vlinks;
    size_t base;  /* weight offset */
    size_t aff[MAX_VL];
    int n_vars[MAX_VL];
    int var_id[MAX_VL][MAX_VAR];
    size_t var_off[MAX_VL][MAX_VAR];
} xf_desc;

typedef struct {
    int nx, has_final, chaos;
    xf_desc xf[MAX_XF + 1];
} flame_desc;

static int parse_structure(const int* s, flame_desc* d) {
    int k = 0;
    d->nx = s[k++];
    d->has_final = s[k++];
    d->chaos = s[k++];
    if (d->nx < 1 || d->nx > MAX_XF) return -1;
    size_t off = 13 + (d->chaos ? (size_t)d->nx * (d->nx + 1) : 0);
    for (int x = 0; x < d->nx + d->has_final; x++) {
        xf_desc* xf = &d->xf[x];
        xf->base = off;
        off += 4;
        xf->n_vlinks = s[k++];
        if (xf->n_vlinks < 1 || xf->n_vlinks > MAX_VL) return -1;
        for (int l = 0; l < xf->n_vlinks; l++) {
            xf->aff[l] = off;
            off += 6;
            xf->n_vars[l] = s[k++];
            if (xf->n_vars[l] < 0 || xf->n_vars[l] > MAX_VAR) return -1;
            for (int v = 0; v < xf->n_vars[l]; v++) {
                xf->var_id[l][v] = s[k++];
                xf->var_off[l][v] = off;
                off += 1 + (size_t)s[k++];
            }
        }
    }
    return (int)off;
}

static double eps(double a) { return a == 0.0 ? 1e-20 : a; }

/* config/variations_new.yml formulas, FP64. `u` supplies uniforms. */
static void variation(int id, const double* P, size_t off, double x, double y, double* rx, double* ry, const double* u,
                      int* used) {
    const double w = P[off];
    const double sumsq = x * x + y * y;
    const double sq = hypot(x, y);
    const double rs = 1.0 / sqrt(sumsq);
    const double at = atan2(x, y);
    const double sina = x * rs, cosa = y * rs;
    switch (id) {
    case 0: *rx += w * x; *ry += w * y; break;
    case 1: *rx += w * sin(x); *ry += w * sin(y); break;
    case 2: { double k = w / eps(sumsq); *rx += k * x; *ry += k * y; break; }
    case 3: { double s = sin(sumsq), c = cos(sumsq); *rx += w * (s * x - c * y); *ry += w * (c * x + s * y); break; }
    case 4: { double k = w / eps(sq); *rx += k * (x + y) * (x - y); *ry += k * 2.0 * x * y; break; }
    case 5: *rx += w * at / PI; *ry += w * (sq - 1.0); break;
    case 6: *rx += w * sq * sin(at + sq); *ry += w * sq * cos(at - sq); break;
    case 7: { double a = sq * at, r = w * sq; *rx += r * sin(a); *ry -= r * cos(a); break; }
    case 8: { double k = w * at / PI; *rx += k * sin(PI * sq); *ry += k * cos(PI * sq); break; }
    case 9: { double r = eps(sq); *rx += w / r * (cosa + sin(r)); *ry += w / r * (sina - cos(r)); break; }
    case 10: { double r = eps(sq); *rx += w * sina / r; *ry += w * cosa * r; break; }
    case 11: {
        double bit = (u[(*used)++] < 0.5) ? 0.0 : 1.0;
        double a = 0.5 * at + PI * bit, r = w * sqrt(sq);
        *rx += r * cos(a);
        *ry += r * sin(a);
        break;
    }
    case 12: { double r = w * exp(x - 1.0); *rx += r * cos(PI * y); *ry += r * sin(PI * y); break; }
    case 13: { double r = w * pow(sq, sina); *rx += r * cosa; *ry += r * sina; break; }
    case 14: { double r = 2.0 * w / (sq + 1.0); *rx += r * y; *ry += r * x; break; }
    case 15: { double r = w / (0.25 * sumsq + 1.0); *rx += r * x; *ry += r * y; break; }
    case 16: *rx += w * sina * cos(sq); *ry += w * cosa * sin(sq); break;
    case 17: {
        double n0 = sin(at + sq), n1 = cos(at - sq);
        double m0 = n0 * n0 * n0 * sq, m1 = n1 * n1 * n1 * sq;
        *rx += w * (m0 + m1);
        *ry += w * (m0 - m1);
        break;
    }
    case 18: { double bx = x < 0 ? x * 2 : x, by = y < 0 ? y / 2 : y; *rx += w * bx; *ry += w * by; break; }
    case 19: *rx += w * sin(x); *ry += w * y; break;
    case 20: { double r = w * exp(x); *rx += r * cos(y); *ry += r * sin(y); break; }
    case 21: { double r = 2.0 * w / (sq + 1.0); *rx += r * x; *ry += r * y; break; }
    case 22: {
        double r = w * u[(*used)++], a = u[(*used)++] * 2.0;
        *rx += r * cos(PI * a);
        *ry += r * sin(PI * a);
        break;
    }
    case 23: {
        double a = u[(*used)++] * 2.0;
        double r = u[*used] + u[*used + 1] + u[*used + 2] + u[*used + 3] - 2.0;
        *used += 4;
        *rx += w * r * cos(PI * a);
        *ry += w * r * sin(PI * a);
        break;
    }
    case 24: { double s = sin(PI * x), c = cos(PI * x); *rx += w * c * cosh(y); *ry += w * -s * sinh(y); break; }
    default: break;
    }
}

/* flame.tpl:10-14 (affine), :46-79 (vlink chain), :154 (colour) */
static double apply_xf(const flame_desc* d, const double* P, int xi, double* x, double* y, double* c, const double* u,
                       int* used) {
    const xf_desc* xf = &d->xf[xi];
    double ix = *x, iy = *y;
    for (int l = 0; l < xf->n_vlinks; l++) {
        const double* A = P + xf->aff[l]; /* a d b e c f */
        const double px = A[0] * ix + A[2] * iy + A[4];
        const double py = A[1] * ix + A[3] * iy + A[5];
        double rx = 0.0, ry = 0.0;
        /* a zero-weight variation adds nothing and draws no uniforms (the
           generated kernels skip it the same way) */
        for (int v = 0; v < xf->n_vars[l]; v++)
            if (P[xf->var_off[l][v]] != 0.0) variation(xf->var_id[l][v], P, xf->var_off[l][v], px, py, &rx, &ry, u, used);
        ix = rx;
        iy = ry;
    }
    *x = ix;
    *y = iy;
    const double cs = P[xf->base + 2];
    *c = *c * (1.0 - cs) + P[xf->base + 1] * cs;
    return P[xf->base + 3];
}

double oracle_apply(const int* structure, const double* params, int xf, double* x, double* y, double* c, const double* u,
                    int* used) {
    flame_desc d;
    if (parse_structure(structure, &d) < 0) return NAN;
    int k = 0;
    if (!used) used = &k;
    return apply_xf(&d, params, xf, x, y, c, u, used);
}

void oracle_apply_many(const int* structure, const double* params, int xf, size_t n, const double* in_xyc,
                       double* out_xyco) {
    flame_desc d;
    if (parse_structure(structure, &d) < 0) return;
    const double u[40] = {0};
    for (size_t i = 0; i < n; i++) {
        double x = in_xyc[3 * i], y = in_xyc[3 * i + 1], c = in_xyc[3 * i + 2];
        int used = 0;
        const double op = apply_xf(&d, params, xf, &x, &y, &c, u, &used);
        out_xyco[4 * i] = x;
        out_xyco[4 * i + 1] = y;
        out_xyco[4 * i + 2] = c;
        out_xyco[4 * i + 3] = op;
    }
}

/* -------------------------------------------------------------- RNG (xoshiro256**) */
typedef struct { uint64_t s[4]; } rng_t;

static uint64_t splitmix(uint64_t* x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void rng_seed(rng_t* r, uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; i++) r->s[i] = splitmix(&x);
}

static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t rng_next(rng_t* r) {
    uint64_t* s = r->s;
    const uint64_t res = rotl64(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return res;
}

static double u01(rng_t* r) { return (double)(rng_next(r) >> 11) * 0x1.0p-53; }

/* ------------------------------------------------------------ chaos game */
typedef struct {
    const flame_desc* d;
    const double* P;
    const double* pal;
    uint32_t w, h;
    uint64_t chain_begin, chain_end;
    uint32_t warmup;
    uint64_t passes;
    uint64_t seed;
    const double* jitter; /* n_jitter x 2 */
    int n_jitter;
    uint64_t n_chains;
    int hammersley;
    double* hist;
    uint64_t draws;
    /* pick weights: row 0 the xform weights, row 1 + r (chaos) the chaos row
       of previous xform r times the xform weights (flame.tpl:170-177) */
    double wt[MAX_XF + 1][MAX_XF];
    double wsum[MAX_XF + 1];
    double cum[MAX_XF + 1][MAX_XF];
} job_t;

static int pick(const job_t* j, int row, double u) {
    /* flame.tpl:110-123: first non-zero-weight xform whose running sum reaches
       u * sum, else the last non-zero-weight one (xform 0 when all are zero) */
    const double ratio = u * j->wsum[row];
    int last_nonzero = 0;
    for (int i = 0; i < j->d->nx; i++) {
        if (j->wt[row][i] != 0.0) {
            if (i < j->d->nx - 1 && j->cum[row][i] >= ratio) return i;
            last_nonzero = i;
        }
    }
    return (j->wt[row][j->d->nx - 1] != 0.0) ? j->d->nx - 1 : last_nonzero;
}

static void* render_job(void* arg) {
    job_t* j = (job_t*)arg;
    const flame_desc* d = j->d;
    const double* P = j->P;
    double u[40];
    for (uint64_t ch = j->chain_begin; ch < j->chain_end; ch++) {
        rng_t r;
        rng_seed(&r, j->seed * 0x100000001B3ull + ch);
        /* start: over the image, mapped through the plane-space affine; either
           uniform or the Hammersley point of refactor.cu:39-54, :301-304 */
        double sx0, sy0;
        if (j->hammersley) {
            const uint32_t total = (uint32_t)j->n_chains, idx = (uint32_t)ch;
            uint32_t max_val = total;
            if (total % 2u) {
                max_val = 1;
                while (max_val < total) max_val <<= 1;
            }
            uint32_t radix = 0, v = max_val;
            while (v >>= 1) radix++;
            uint32_t rev = idx;
            rev = (rev << 16) | (rev >> 16);
            rev = ((rev & 0x00ff00ffu) << 8) | ((rev & 0xff00ff00u) >> 8);
            rev = ((rev & 0x0f0f0f0fu) << 4) | ((rev & 0xf0f0f0f0u) >> 4);
            rev = ((rev & 0x33333333u) << 2) | ((rev & 0xccccccccu) >> 2);
            rev = ((rev & 0x55555555u) << 1) | ((rev & 0xaaaaaaaau) >> 1);
            const uint32_t flipped = radix ? rev >> (32 - radix) : 0;
            const double inv = 1.0 / max_val;
            sx0 = ((idx * inv * 2.0 - 1.0) + 1.0) / 2.0 * j->w;
            sy0 = ((flipped * inv * 2.0 - 1.0) + 1.0) / 2.0 * j->h;
        } else {
            sx0 = u01(&r) * j->w;
            sy0 = u01(&r) * j->h;
        }
        double x = P[6] * sx0 + P[8] * sy0 + P[10];
        double y = P[7] * sx0 + P[9] * sy0 + P[11];
        double c = u01(&r);
        const double* jit = j->jitter + 2 * (ch % (uint64_t)j->n_jitter);
        const uint64_t total = (uint64_t)j->warmup + j->passes;
        int last = -1; /* previous xform (chaos); none before the first step */
        for (uint64_t pass = 0; pass < total; pass++) {
            for (int k = 0; k < 40; k++) u[k] = u01(&r);
            int used = 1;
            const int xi = pick(j, d->chaos && last >= 0 ? 1 + last : 0, u[0]);
            last = xi;
            double op = apply_xf(d, P, xi, &x, &y, &c, u, &used);
            /* refactor.cu:195-199 */
            if (isnan(x) || x > 1e10 || x < -1e10 || isnan(y) || y > 1e10 || y < -1e10) {
                x = u[used++] * 2.0 - 1.0;
                y = u[used++] * 2.0 - 1.0;
                op = 0.0;
            }
            if (pass < j->warmup) continue;
            double fx = x, fy = y, fc = c;
            if (d->has_final) apply_xf(d, P, d->nx, &fx, &fy, &fc, u, &used);
            /* refactor.cu:356-383 */
            double px = P[0] * fx + P[2] * fy + (P[4] + jit[0]);
            double py = P[1] * fx + P[3] * fy + (P[5] + jit[1]);
            px = trunc(px);
            py = trunc(py);
            if (px >= 0 && py >= 0 && px < j->w && py < j->h && op > 0.0) {
                double ci = fc < 0 ? 0 : (fc > 1 ? 1 : fc);
                const double idx = ci * 255.0;
                const int lo = (int)floor(idx), hi = (int)ceil(idx);
                const double mix = idx - floor(idx);
                double* b = j->hist + 4 * ((size_t)py * j->w + (size_t)px);
                for (int ch3 = 0; ch3 < 3; ch3++)
                    b[ch3] += ((1.0 - mix) * j->pal[3 * lo + ch3] + mix * j->pal[3 * hi + ch3]) * op;
                b[3] += op;
                j->draws++;
            }
        }
    }
    return NULL;
}

uint64_t oracle_render(const int* structure, const double* params, const double* pal, uint32_t w, uint32_t h,
                       uint64_t n_chains, uint32_t warmup, uint64_t passes, uint64_t seed, int threads, int n_jitter,
                       const double* jitter_in, int hammersley, double* hist) {
    flame_desc* d = (flame_desc*)malloc(sizeof(flame_desc));
    if (!d || parse_structure(structure, d) < 0) {
        free(d);
        return 0;
    }
    if (threads < 1) threads = 1;
    if (n_jitter < 1) n_jitter = 1;
    /* flame.tpl:179-182: screen jitter ~ randgauss(1/3) (random.h:9-14 form) */
    double* jit = (double*)malloc(sizeof(double) * 2 * (size_t)n_jitter);
    rng_t jr;
    rng_seed(&jr, seed ^ 0xA5A5A5A5A5A5ull);
    for (int i = 0; i < n_jitter; i++) {
        if (jitter_in) {
            jit[2 * i] = jitter_in[2 * i];
            jit[2 * i + 1] = jitter_in[2 * i + 1];
            continue;
        }
        const double a = u01(&jr) * 2.0;
        const double r = (1.0 / 3.0) * (u01(&jr) + u01(&jr) + u01(&jr) + u01(&jr) - 2.0);
        jit[2 * i] = r * cos(PI * a);
        jit[2 * i + 1] = r * sin(PI * a);
    }
    job_t* jobs = (job_t*)calloc((size_t)threads, sizeof(job_t));
    pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    const size_t hsz = (size_t)w * h * 4;
    for (int t = 0; t < threads; t++) {
        job_t* j = &jobs[t];
        j->d = d;
        j->P = params;
        j->pal = pal;
        j->w = w;
        j->h = h;
        j->chain_begin = n_chains * (uint64_t)t / (uint64_t)threads;
        j->chain_end = n_chains * (uint64_t)(t + 1) / (uint64_t)threads;
        j->warmup = warmup;
        j->passes = passes;
        j->seed = seed;
        j->jitter = jit;
        j->n_jitter = n_jitter;
        j->n_chains = n_chains;
        j->hammersley = hammersley;
        j->hist = (t == 0) ? hist : (double*)calloc(hsz, sizeof(double));
        const int rows = d->chaos ? 1 + d->nx : 1;
        for (int row = 0; row < rows; row++) {
            double run = 0.0;
            for (int i = 0; i < d->nx; i++) {
                double wv = params[d->xf[i].base];
                if (row > 0) wv *= params[13 + (size_t)(row - 1) * (d->nx + 1) + 1 + i];
                j->wt[row][i] = wv;
                run += wv;
                j->cum[row][i] = run;
            }
            j->wsum[row] = run;
        }
    }
    memset(hist, 0, hsz * sizeof(double));
    for (int t = 1; t < threads; t++) pthread_create(&tid[t], NULL, render_job, &jobs[t]);
    render_job(&jobs[0]);
    uint64_t draws = jobs[0].draws;
    for (int t = 1; t < threads; t++) {
        pthread_join(tid[t], NULL);
        for (size_t i = 0; i < hsz; i++) hist[i] += jobs[t].hist[i];
        draws += jobs[t].draws;
        free(jobs[t].hist);
    }
    free(jobs);
    free(tid);
    free(jit);
    free(d);
    return draws;
}

/* --------------------------------------------------------------- tonemap */
static double sat(double v) { return v < 0 ? 0 : (v > 1 ? 1 : v); }

void oracle_tonemap(const float* bins, size_t n, double quality, double gamma, double brightness, double vibrancy,
                    double highlight_power, double* out) {
    /* tonemapper.cpp:52: the scale constant is computed in single precision */
    const float k2 = powf(10.0f, -log10f((float)quality) - 0.5f);
    const double g = (double)(float)gamma;
    const double inv_gamma = 1.0 / g;
    const double B = (double)(float)brightness, V = (double)(float)vibrancy;
    const double log_div = 4.0 / log(2.0);
    for (size_t i = 0; i < n; i++) {
        const double w_in = bins[4 * i + 3];
        double* o = out + 4 * i;
        if (w_in == 0.0) {
            o[0] = o[1] = o[2] = o[3] = 0.0;
            continue;
        }
        /* log10(1 + x) evaluated as log1p(x) / ln 10 so that tiny densities keep their digits */
        const double f = 0.5 * B * (log1p(w_in * (double)k2) / log(10.0)) / w_in;
        double c[3] = {bins[4 * i] * f, bins[4 * i + 1] * f, bins[4 * i + 2] * f};
        const double wf = w_in * f;
        const double gf = pow(wf, inv_gamma) / wf;
        double lin[3] = {c[0] * gf, c[1] * gf, c[2] * gf};
        if (highlight_power >= 0.0) {
            const double m = fmax(lin[0], fmax(lin[1], lin[2]));
            if (m > 1.0) {
                const double s = 1.0 / m, ratio = pow(s, highlight_power);
                for (int k = 0; k < 3; k++) lin[k] = 1.0 - ratio * (1.0 - lin[k] * s);
            }
        }
        for (int k = 0; k < 3; k++) {
            const double a = pow(c[k], inv_gamma);
            o[k] = sat(a + V * (lin[k] - a));
        }
        o[3] = sat(log(w_in) * log_div / 96.0);
    }
}

/* density_histo.cu:1-42 (float arithmetic as the kernel) */
void oracle_density_histogram(const float* bins, size_t n, uint64_t* hist, uint64_t* max_density) {
    const float log_div = 4.0f / logf(2.0f);
    memset(hist, 0, 97 * sizeof(uint64_t));
    uint64_t mx = 0;
    for (size_t i = 0; i < n; i++) {
        const float v = bins[4 * i + 3];
        if (v >= 1.0f) {
            uint64_t b = (uint64_t)(logf(v) * log_div) + 1;
            if (b > 96) b = 96;
            hist[b]++;
            if ((uint64_t)v > mx) mx = (uint64_t)v;
        } else {
            hist[0]++;
        }
    }
    *max_density = mx;
}

/* ------------------------------------------------------------ DE blur */
#define DE_STEPS 4

void oracle_density_blur(const float* in, uint32_t w, uint32_t h, double max_r, double min_r, double curve, double* out) {
    const int levels = 9 * DE_STEPS + 1;
    double a_tab[9 * DE_STEPS + 1], z_tab[9 * DE_STEPS + 1];
    for (int l = 0; l < levels; l++) {
        const double r = (double)l / DE_STEPS;
        const double a = 1.0 / ((r + 1.0) * (r + 1.0));
        const int rc = (l + DE_STEPS - 1) / DE_STEPS;
        double z = 0.0;
        for (int oy = -rc; oy <= rc; oy++)
            for (int ox = -rc; ox <= rc; ox++) z += fmax(0.0, 1.0 - (double)(ox * ox + oy * oy) * a);
        a_tab[l] = a;
        z_tab[l] = z;
    }
    memset(out, 0, sizeof(double) * 4 * (size_t)w * h);
    for (uint32_t sy = 0; sy < h; sy++)
        for (uint32_t sx = 0; sx < w; sx++) {
            const float* v = in + 4 * ((size_t)sy * w + sx);
            if (!(v[3] > 0.0f)) continue;
            float r = (float)max_r * powf(v[3], -(float)curve);
            r = fminf(fmaxf(r, (float)min_r), (float)max_r);
            const int l = (int)lrintf(r * DE_STEPS);
            const int rc = (l + DE_STEPS - 1) / DE_STEPS;
            for (int dy = -rc; dy <= rc; dy++)
                for (int dx = -rc; dx <= rc; dx++) {
                    const long ty = (long)sy + dy, tx = (long)sx + dx;
                    if (ty < 0 || tx < 0 || ty >= h || tx >= w) continue;
                    const double k = fmax(0.0, 1.0 - (double)(dx * dx + dy * dy) * a_tab[l]);
                    if (k == 0.0) continue;
                    const double wt = k / z_tab[l];
                    double* o = out + 4 * ((size_t)ty * w + tx);
                    for (int c = 0; c < 4; c++) o[c] += v[c] * wt;
                }
        }
}
