/*
 * FP64 CPU oracle of the flame-rendering hot path. TEST INFRASTRUCTURE ONLY:
 * used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference legs as the oracle; never linked into or called by librfk.
 *
 * It restates the reference's formulas independently of the library (no
 * shared source): packed-sample interpolation, the chaos game, the tonemap,
 * the density histogram and the density-estimation blur. Each function cites
 * the reference file:line it follows (paths relative to the reference root).
 *
 * Parity pinning: the reference publishes no test vectors; the oracle is
 * pinned against the reference's own kernels run on the GPU (tonemap,
 * Catmull-Rom, density histogram) and against hand-derived known answers
 * (tests/golden/).
 */
#ifndef RFK_ORACLE_H
#define RFK_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Variation ids understood by oracle_apply (FP64 restatements of
 * config/variations_new.yml of the reference, line numbers there):
 *  0 linear :1   1 sinusoidal :3   2 spherical :5-7   3 swirl :9-12
 *  4 horseshoe :14   5 polar :16-18   6 handkerchief :20   7 heart :22-26
 *  8 disc :28   9 spiral :30-33   10 hyperbolic :35-38   11 julia :53
 *  12 exponential :80   13 power :82   14 fisheye :74   15 bubble :152
 *  16 diamond :40-43   17 ex :45-51   18 bent :55-59   19 cylinder :154-156
 *  20 exp :~ (exp: weight*exp(x)*cossin(y))   21 eyefish :150
 *  22 blur   23 gaussian_blur   24 cosine :84-87 */
#define ORACLE_NUM_VARIATIONS 25
const char* oracle_variation_name(int id);
int oracle_variation_id(const char* name);

/* Structure of a flame, as ints:
 *   [0] NX (standard xforms), [1] has_final, [2] chaos,
 *   then for each of NX + has_final xforms: n_vlinks, and per vlink: n_vars,
 *   then per variation: id, n_params (ordinary + precalc slots).
 * Offsets follow the packed layout of flame_types.h:634-672. */

/* Centripetal Catmull-Rom coefficients (catmull.cu:11-42): samples
 * [nseg+3][sample_size] -> coeff [nseg][sample_size][4]. */
void oracle_catmull(const double* samples, size_t sample_size, size_t nseg, double* coeff);

/* fix_rotation (flame_compiler.cpp:957-1035) over n samples, in place. */
void oracle_fix_rotation(double* samples, size_t n, size_t sample_size, size_t flame_size, const size_t* aff,
                         size_t n_aff);

/* Flame at time t of segment seg (refactor.cu:105-151, :278-294): params
 * [size_reals] with affines converted back from (angle, log magnitude), and
 * the 8-bit palette as RGB in [0,1] [256][3]. */
void oracle_interpolate(const double* coeff, size_t sample_size, size_t size_reals, size_t seg, double t,
                        const size_t* aff, size_t n_aff, double* params, double* palette_rgb);

/* HSV -> 8-bit RGB of refactor.cu:128-140 (values / 255). */
void oracle_hsv_to_rgb8(double h, double s, double v, double rgb[3]);

/* Applies xform `xf` (NX = final) of a flame to (x, y, c); random draws from
 * u[] (uniforms in [0,1), as many as the variations need, at most 32).
 * Returns opacity; writes the new point and colour. flame.tpl:46-79, :146-160. */
double oracle_apply(const int* structure, const double* params, int xf, double* x, double* y, double* c,
                    const double* u, int* used);

/* FP64 chaos game (refactor.cu:176-238, :347-386 semantics with per-chain
 * xform picks): n_chains chains, `warmup` passes without drawing, then
 * `passes` drawing passes, into hist [h][w][4] (doubles, summed). The screen
 * affine of chain i gets offset i % n_jitter of `jitter` (n_jitter x 2), or
 * when `jitter` is NULL, of n_jitter Gaussian(1/3 px) offsets it draws
 * (flame.tpl:179-182). Chains start uniformly over the image, or with
 * `hammersley` at Hammersley point i of n_chains (refactor.cu:39-54,
 * :301-304). Runs on `threads` POSIX threads. Returns the number of draws. */
uint64_t oracle_render(const int* structure, const double* params, const double* palette_rgb, uint32_t w, uint32_t h,
                       uint64_t n_chains, uint32_t warmup, uint64_t passes, uint64_t seed, int threads, int n_jitter,
                       const double* jitter, int hammersley, double* hist);

/* oracle_apply over n points (x, y, c) -> (x, y, c, opacity), with every
 * random draw 0. */
void oracle_apply_many(const int* structure, const double* params, int xf, size_t n, const double* in_xyc,
                       double* out_xyco);

/* tonemap (tonemap.cu:67-104, tonemapper.cpp:52) in FP64: bins [n][4] ->
 * out [n][4] (alpha in the 4th channel). highlight_power < 0 = off. */
void oracle_tonemap(const float* bins, size_t n, double quality, double gamma, double brightness, double vibrancy,
                    double highlight_power, double* out);

/* calculate_histogram<4> (density_histo.cu:1-42): 97 bins + max density. */
void oracle_density_histogram(const float* bins, size_t n, uint64_t* hist, uint64_t* max_density);

/* Density-estimation blur as specified by librfk (rfk.h rfk_density_blur):
 * in/out [h][w][4]. */
void oracle_density_blur(const float* in, uint32_t w, uint32_t h, double max_radius, double min_radius, double curve,
                         double* out);

#ifdef __cplusplus
}
#endif

#endif
