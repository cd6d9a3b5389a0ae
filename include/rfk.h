/*
 * rfk.h - C ABI of the GB300 flame-rendering hot path (librfk.so).
 *
 * Each entry point replaces one call of librefrakt's hot path; the reference
 * interface it stands in for is cited beside it (paths relative to the
 * reference project root). Conventions:
 *   - every call returns an rfk_status (0 = RFK_OK); on failure the message is
 *     available from rfk_last_error() on the calling thread, in place of the
 *     reference's log + exit(1) (src/librefrakt/include/librefrakt/util/cuda.h:16-25);
 *   - opaque handles are released with the matching *_destroy call;
 *   - GPU work is enqueued on the caller's stream (a cudaStream_t passed as
 *     void*, NULL = the legacy default stream); device pointers are CUDA
 *     device addresses on the current device;
 *   - handles are thread-compatible: one state per thread, kernels may be
 *     shared, the compile cache is internally locked.
 */
#ifndef RFK_H
#define RFK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int rfk_status;
#define RFK_OK 0
#define RFK_E_INVALID 1  /* bad argument or size */
#define RFK_E_FORMAT 2   /* genome / database text that does not parse or validate */
#define RFK_E_COMPILE 3  /* NVRTC or module load failure (log returned) */
#define RFK_E_CUDA 4     /* CUDA runtime / driver error */
#define RFK_E_NODEVICE 5 /* no usable sm_100-class device */

typedef struct rfk_db rfk_db;
typedef struct rfk_flame rfk_flame;
typedef struct rfk_kernel rfk_kernel;
typedef struct rfk_state rfk_state;

/* Thread-local text of the last failure on this thread ("" if none). */
const char* rfk_last_error(void);
/* Library version, major * 10000 + minor * 100 + patch. */
int rfk_version(void);

/* ---- variation database ------------------------------------------------
 * rfkt::initialize(flamedb&, config_path)  src/librefrakt/src/flame_info.cpp:60-148
 * Loads <dir>/variations_new.yml and <dir>/common.yml. */
rfk_status rfk_db_load(const char* config_dir, rfk_db** out);
void rfk_db_destroy(rfk_db* db);
/* flamedb::variations() / is_variation  flame_info.h:69-88 */
int rfk_db_variation_count(const rfk_db* db);
rfk_status rfk_db_variation_name(const rfk_db* db, int index, char* buf, size_t cap);
/* flamedb::hash()  flame_info.h:131-133 */
uint64_t rfk_db_hash(const rfk_db* db);
/* flamedb::add_or_update_variation  flame_info.h:94, flame_info.cpp:152-194
 * Adds or replaces every variation of `yaml` (the variations_new.yml format:
 * name: body, or name: {src, precalc, param, tags}), in name order; each is
 * parsed and checked against its parameters and the commons. On the first
 * failure returns RFK_E_FORMAT (message in rfk_last_error) with the earlier
 * entries kept. Changes rfk_db_hash, so kernels compiled afterwards see the
 * new definitions. Not thread-safe against other calls on the same db. */
rfk_status rfk_db_add_variations(rfk_db* db, const char* yaml);
/* flamedb::add_or_update_common  flame_info.h:95: a named common expression. */
rfk_status rfk_db_add_common(rfk_db* db, const char* name, const char* code);
/* flamedb::remove_variation / remove_common  flame_info.h:113-129:
 * 1 removed, 0 not present (or a null argument). */
int rfk_db_remove_variation(rfk_db* db, const char* name);
int rfk_db_remove_common(rfk_db* db, const char* name);
/* flamedb::is_variation / is_parameter / is_common  flame_info.h:69-84: 1 or 0. */
int rfk_db_is_variation(const rfk_db* db, const char* name);
int rfk_db_is_parameter(const rfk_db* db, const char* variation, const char* param);
int rfk_db_is_common(const rfk_db* db, const char* name);
/* Translated device source of one variation (diagnostics, host-twin tests). */
rfk_status rfk_db_variation_source(const rfk_db* db, const char* name, char* buf, size_t cap, size_t* len);

/* ---- genomes -------------------------------------------------------------
 * rfkt::flame::deserialize  src/librefrakt/src/flame_types.cpp:437-485
 * rfkt::import_flam3        src/librefrakt/src/flame_types.cpp:131-239
 * flame::serialize           src/librefrakt/src/flame_types.cpp:399-435 (palette written as [h,s,v] triples) */
rfk_status rfk_flame_from_json(const rfk_db* db, const char* json, rfk_flame** out);
rfk_status rfk_flame_from_flam3(const rfk_db* db, const char* xml, rfk_flame** out);
rfk_status rfk_flame_to_json(const rfk_flame* f, char* buf, size_t cap, size_t* len);
void rfk_flame_destroy(rfk_flame* f);
/* flame::size_reals()  src/librefrakt/include/librefrakt/flame_types.h:602-613 */
size_t rfk_flame_size_reals(const rfk_flame* f);
/* flame::pack_sample(packer, invoker, t, w, h)  flame_types.h:634-672.
 * Writes size_reals + 768 doubles (static genome: every t gives t0 values). */
rfk_status rfk_flame_pack_sample(const rfk_flame* f, int w, int h, double* out, size_t cap);
/* flame::affine_indices()  flame_types.h:674-705 */
rfk_status rfk_flame_affine_indices(const rfk_flame* f, size_t* out, size_t cap, size_t* count);
/* gamma, brightness, vibrancy, highlight_power of the genome (flame_types.h:565-569). */
rfk_status rfk_flame_tonemap_params(const rfk_flame* f, double out[4]);
/* structure hash: equal hashes share a kernel (flame_types.h:578-592) */
uint64_t rfk_flame_structure_hash(const rfk_flame* f);

/* ---- per-flame kernels ---------------------------------------------------
 * flame_compiler::get_flame_kernel(fdb, precision, flame) -> result
 *   src/librefrakt/include/librefrakt/flame_compiler.h:156-182,
 *   src/librefrakt/src/flame_compiler.cpp:601-656
 * One NVRTC (sm_103a) module per (structure, options); changing genome values
 * reuses it. Fields left 0 choose the defaults / the autotuned launch shape. */
typedef struct {
    int precise_math;      /* 0: -use_fast_math as the reference (flame_compiler.cpp:861); 1: full-precision libm */
    int block;             /* threads per block (0 = 256) */
    int chains_per_thread; /* 0 = 4 when sorting, else 1 */
    int flush;             /* histogram update: 0 = red.global.add.v4.f32 per draw, 1 = warp-aggregated,
                              2 = warp-aggregated into a per-block shared-memory cache of hot pixels,
                              3 = the shared-memory cache without warp aggregation, 4 = fixed-point
                              shared-memory sums for the pixels the block's own draws show to be hot,
                              one red per draw elsewhere. 0 and 3 add draws one at a time, so a
                              pixel's FP32 sum stops at 2^24 (adding 1 there rounds back); the
                              autotuner picks among 1, 2 and 4 only */
    int blocks_per_sm;     /* 0 = registers capped so that 1280 / block bin blocks fit per SM, and as
                              many run as fit; n > 0 = registers capped so that n fit, and at most n
                              run per SM (launch bounds) */
    int sort;              /* 1 = sort each warp's chains by xform every pass, 0 or 2 = sort the whole
                              block's chains (both when 2..32 xforms); -1 = never */
} rfk_compile_opts;

typedef struct {
    int grid;               /* persistent blocks = temporal samples */
    int block;
    int chains_per_thread;
    int flush;
    int sort;               /* 1 / 2 when chains are sorted by xform every pass (warp / block) */
    int registers;          /* of the bin kernel */
    int num_xforms;
    int has_final;
    int chaos;
    size_t size_reals;
    size_t sample_floats;   /* floats per prepared parameter block */
    double compile_ms;
    double sfu_per_iter;    /* weighted transcendental calls per chain step */
    double fma_per_iter;    /* weighted affine FMAs per chain step (4 per vlink, + projection) */
} rfk_kernel_info;

rfk_status rfk_compile(const rfk_db* db, const rfk_flame* f, const rfk_compile_opts* opts, rfk_kernel** out,
                       char* log, size_t log_cap);
void rfk_kernel_destroy(rfk_kernel* k);
rfk_status rfk_kernel_get_info(const rfk_kernel* k, rfk_kernel_info* out);
/* Full NVRTC text for a flame (device prelude, generated flame code, kernel
 * bodies); needs no device. */
rfk_status rfk_generate_source(const rfk_db* db, const rfk_flame* f, char* buf, size_t cap, size_t* len);
/* NVRTC-compiles the flame's kernels for `arch` (e.g. "sm_103a") without
 * loading them: a compile check that needs no device. The log holds the
 * compiler's per-kernel resource report (registers, spills, shared memory). */
rfk_status rfk_compile_check(const rfk_db* db, const rfk_flame* f, const rfk_compile_opts* opts, const char* arch, char* log,
                             size_t log_cap);
/* The generated device source (flame_compiler::result::source). */
rfk_status rfk_kernel_source(const rfk_kernel* k, char* buf, size_t cap, size_t* len);

/* ---- render state ----------------------------------------------------------
 * flame_kernel::warmup(stream, samples, dims, seed, count, temporal_multiplier)
 *   flame_compiler.h:99-100, flame_compiler.cpp:1037-1108
 * samples: host array of nsamples x (size_reals + 768) doubles (pack_sample
 * output, nsamples >= 4); the spline segments between samples 1 and
 * nsamples-2 are spread over the persistent blocks as temporal samples. The
 * state owns a cleared w x h float4 histogram (device), chain states and
 * counters. temporal_multiplier T (1..32): T x grid temporal samples, each with
 * its own chains; a persistent block cycles through its T samples during bin
 * (motion blur over the segment with T times the samples at the same chain
 * count), each (block, sample) reaching an equal share of the quality. */
rfk_status rfk_warmup(const rfk_kernel* k, const double* samples, size_t nsamples, uint32_t w, uint32_t h,
                      uint32_t seed, uint32_t warmup_count, int temporal_multiplier, void* stream, rfk_state** out);
/* flame_kernel::warmup(stream, samples, gpu_image<float4>&& bins, seed, count,
 * temporal_multiplier)  flame_compiler.h:100, flame_compiler.cpp:1037-1101
 * As rfk_warmup, but the state accumulates into the caller's w x h float4
 * histogram `bins` (device, 16-byte aligned) as it is, without clearing it
 * (the reference adopts the image it is given; its dims overload clears a new
 * one). The caller keeps ownership: `bins` must outlive the state and is not
 * freed by rfk_state_destroy. */
rfk_status rfk_warmup_adopt(const rfk_kernel* k, const double* samples, size_t nsamples, void* bins, uint32_t w,
                            uint32_t h, uint32_t seed, uint32_t warmup_count, int temporal_multiplier, void* stream,
                            rfk_state** out);
void rfk_state_destroy(rfk_state* s);
/* flame_kernel::warmup into an existing state (no reference counterpart: the
 * reference makes a new saved_state per warmup). For a renderer that draws
 * frame after frame at one size: the state's kernel, size and temporal
 * multiplier stay; its parameter blocks are prepared again from the new host
 * samples, the chains start again from the Hammersley points and run
 * warmup_count passes, the counters and the accumulated quality restart at
 * 0, and the histogram is cleared when `clear` is non-zero (kept otherwise,
 * also an adopted one). Nothing is allocated, so the per-frame cost is the
 * sample upload, the preparation and the warm-up launch. Fails with
 * RFK_E_INVALID while a bin call on the state is pending. */
rfk_status rfk_state_rewarm(rfk_state* s, const double* samples, size_t nsamples, uint32_t seed, uint32_t warmup_count,
                            int clear, void* stream);

/* flame_kernel::bailout_args  flame_compiler.h:92-96 */
typedef struct {
    uint32_t iters;   /* passes per chain cap for this call (0 = none) */
    uint32_t millis;  /* time budget; 0 or above 60000 means 60000 (every call ends) */
    double quality;   /* additional spp to reach (0 = none) */
    uint32_t temporal_slicing; /* passes a block spends on one temporal sample before the next
                                  (temporal_multiplier > 1); 0 = 100, as flame_kernel::bin */
} rfk_bailout;

/* flame_kernel::bin_result  flame_compiler.h:27-35 (+ status bits and draw count) */
typedef struct {
    double quality;           /* spp added by this call: sum(255 * opacity) / (255 * pixels) */
    double elapsed_ms;        /* kernel span from %globaltimer */
    uint64_t total_passes;    /* chain steps */
    uint64_t total_draws;     /* sum(255 * opacity) / 255, as the reference reports */
    uint64_t total_bins;      /* pixels */
    double passes_per_thread;
    double max_density;
    uint64_t draw_count;      /* in-bounds draws with opacity > 0 */
    uint32_t status;          /* 1 quality reached, 2 time, 4 stopped, 8 pass cap */
} rfk_bin_result;

/* flame_kernel::bin(stream, state, bailout, temporal_slicing)
 *   flame_compiler.h:98, flame_compiler.cpp:866-955
 * rfk_bin enqueues and waits; rfk_bin_async enqueues, rfk_bin_wait waits for
 * its result. One call per state at a time: rfk_bin_async fails with
 * RFK_E_INVALID while an earlier call on the state has not been waited for.
 * Repeated calls keep accumulating. */
rfk_status rfk_bin(rfk_state* s, const rfk_bailout* bo, void* stream, rfk_bin_result* out);
rfk_status rfk_bin_async(rfk_state* s, const rfk_bailout* bo, void* stream);
rfk_status rfk_bin_wait(rfk_state* s, rfk_bin_result* out);
/* saved_state::abort_binning()  flame_compiler.h:85-88: safe from any thread.
 * Stops the call enqueued last, whenever it is issued after rfk_bin_async
 * returns (also before the launch starts, while the stream is still busy). */
rfk_status rfk_state_abort(rfk_state* s);
/* Device pointer of the float4 histogram (w * h * 4 floats, row-major). */
float* rfk_state_bins(rfk_state* s);
/* Accumulated spp over all bin calls (saved_state::quality). */
double rfk_state_quality(const rfk_state* s);
/* Chain states copied to the host: x, y, colour (each `count` floats). */
rfk_status rfk_state_chains(rfk_state* s, float* x, float* y, float* c, size_t cap, size_t* count);
/* Prepared per-sample parameter blocks copied to the host (grid x sample_floats floats). */
rfk_status rfk_state_samples(rfk_state* s, float* out, size_t cap, size_t* count);

/* ---- single map application (parity unit) -------------------------------
 * Applies xform `xform` (-1 = final) of one prepared parameter block (host,
 * sample_floats floats) to n points (x, y, colour) -> (x, y, colour, opacity).
 * Uses the xform dispatch of flame.tpl:146-160. Host in, host out. */
rfk_status rfk_apply_xform(const rfk_kernel* k, const float* params, int xform, const float* in_xyc, size_t n,
                           float* out_xyco, uint32_t seed);
/* Prepared parameter blocks for explicit (segment, t) pairs, host in / out:
 * samples as for rfk_warmup; seg[i], t[i] for i < count; out count x sample_floats. */
rfk_status rfk_prepare_samples(const rfk_kernel* k, const double* samples, size_t nsamples, const uint32_t* seg,
                               const float* t, size_t count, uint32_t seed, float* out);

/* Variant of rfk_prepare_samples that allocates no device memory. It has no
 * counterpart in the reference. It is for callers that cannot call cudaMalloc
 * while they run: applications whose device memory belongs to their own pool
 * or that reserve it all at start, and real-time loops that must not stall on
 * the device-wide synchronisation of cudaMalloc / cudaFree. Its device
 * temporaries (FP64 samples, spline segments, schedule, output blocks) live
 * in a fixed 4 MiB array that every device using the library holds until
 * exit; requests that need more fail with RFK_E_INVALID and say how much they
 * need. Every call looks up the array's device address on the current device;
 * the first call on a device also loads the library's module there, so make
 * it before any stream capture. Calls share the array and run on the legacy
 * default stream, blocking until the output is on the host: calls that could
 * overlap on the GPU (from several threads or processes) race on the array.
 * Every region is fully written before it is read, so nothing needs clearing. */
rfk_status rfk_prepare_samples_noalloc(const rfk_kernel* k, const double* samples, size_t nsamples, const uint32_t* seg,
                                       const float* t, size_t count, uint32_t seed, float* out);

/* ---- image steps ----------------------------------------------------------
 * tonemapper::run(bins, out, args, stream)
 *   src/librefrakt/include/librefrakt/image/tonemapper.h:10-22,
 *   src/librefrakt/src/image/tonemapper.cpp:37-56, assets/kernels/tonemap.cu:50-105 */
#define RFK_HALF3 0
#define RFK_HALF4 1
#define RFK_FLOAT3 2
#define RFK_FLOAT4 3
typedef struct {
    double quality;          /* accumulated spp */
    double gamma;
    double brightness;
    double vibrancy;
    double max_density;      /* accepted for interface parity; unused, as in the reference */
    double highlight_power;  /* < 0 = off (reference behaviour); >= 0 flam3-style highlight desaturation */
    int precise;             /* 1 = full-precision log/pow; 0 = the reference kernel's fast intrinsics */
} rfk_tonemap_args;
/* bins: device float4[w*h]; out: device image of the given format.
 * histogram / max_density (device, may be NULL): when given, the density
 * histogram of density_histo.cu:1-42 (97 u64 bins, granularity 4) and the max
 * density are accumulated in the same pass; the caller clears them first. */
rfk_status rfk_tonemap(const float* bins, uint32_t w, uint32_t h, void* out, int format, const rfk_tonemap_args* args,
                       uint64_t* histogram, uint64_t* max_density, void* stream);

/* calculate_histogram<4>  assets/kernels/density_histo.cu:1-42 (launched by
 * flame_kernel::bin, flame_compiler.cpp:928-937). Device pointers; the caller
 * clears histogram[97] and max_density. */
rfk_status rfk_density_histogram(const float* bins, uint32_t count, uint64_t* histogram, uint64_t* max_density,
                                 void* stream);

/* Density-estimation blur (no reference counterpart: the reference README
 * src/librefrakt/README.md:14 replaces it by a denoiser). Device float4 in / out
 * (distinct buffers), radius = clamp(max_radius * density^-curve, min_radius,
 * max_radius), max_radius <= 9. */
typedef struct {
    double max_radius;
    double min_radius;
    double curve;
} rfk_de_args;
rfk_status rfk_density_blur(const float* bins_in, float* bins_out, uint32_t w, uint32_t h, const rfk_de_args* args,
                            void* stream);

/* generate_sample_coefficients  assets/kernels/catmull.cu:33-42: device FP64
 * samples [nseg + 3][sample_size] -> device FP32 segments
 * [nseg][sample_size][4] in Hermite form (p1, p2, m1, m2): the curve is
 * h00(t) p1 + h01(t) p2 + h10(t) m1 + h11(t) m2, the same cubic as the
 * reference's a t^3 + b t^2 + c t + d with m1, m2 its centripetal tangents. */
rfk_status rfk_catmull_coefficients(const double* samples, uint32_t sample_size, uint32_t nseg, float* coeff,
                                    void* stream);

/* ---- output step -----------------------------------------------------------
 * converter convert_to<In, Out>  assets/kernels/convert.cu:70-99: a half3 /
 * half4 tonemapped image (RFK_HALF3 / RFK_HALF4) to RFK_FLOAT3 / RFK_FLOAT4 /
 * RFK_UCHAR3 / RFK_UCHAR4; a byte is min(v * 255, 255) truncated; flip_y
 * writes rows bottom-up, swap_channels exchanges R and B (BGR output), a
 * 4-channel output of a 3-channel input gets alpha 1. Device pointers. */
#define RFK_UCHAR3 4
#define RFK_UCHAR4 5
rfk_status rfk_convert(const void* in, int in_format, void* out, int out_format, uint32_t w, uint32_t h, int flip_y,
                       int swap_channels, void* stream);
/* Headless artefact (no reference counterpart; the reference encodes frames
 * with NVENC / nvJPEG): 8-bit RGB or RGBA host pixels, row-major, to a PNG
 * file. */
rfk_status rfk_write_png(const char* path, const uint8_t* pixels, uint32_t w, uint32_t h, int channels);

/* fix_rotation  src/librefrakt/src/flame_compiler.cpp:957-1035, host, in place. */
rfk_status rfk_fix_rotation(double* samples, size_t nsamples, size_t sample_size, size_t flame_size,
                            const size_t* affine_indices, size_t n_affine);

/* ---- autotuner --------------------------------------------------------------
 * No reference counterpart (the reference picks its launch shape from
 * occupancy alone, flame_compiler.cpp:807-864). Times candidate launch shapes
 * (threads per block, chains per thread) and histogram-flush strategies on
 * this flame at this image size - `passes` passes per chain per candidate -
 * and returns the fastest as compile options. Results are cached per
 * (database, structure, genome values, size); a cached answer reports
 * candidates = 0. */
typedef struct {
    int candidates;
    double best_iters_per_s;
    double worst_iters_per_s;
} rfk_tune_report;
rfk_status rfk_autotune(const rfk_db* db, const rfk_flame* f, const double* samples, size_t nsamples, uint32_t w, uint32_t h,
                        uint32_t passes, rfk_compile_opts* best, rfk_tune_report* report);

/* ---- structure alignment ---------------------------------------------------
 * Gives n genomes one structure (xform count, vlink chains, variation sets,
 * final xform, chaos rows) without changing what each renders, so they pack
 * to one layout: keyframes of different structure can be interpolated, and
 * unrelated flames share one (union-of-variations) kernel in a batch.
 * Replaces the interpolator's rebuild_sides / interp_xforms
 * (src/refraktor/src/refraktor.cpp:117-191) with flamedb::make_padder
 * (src/librefrakt/src/flame_info.cpp:239-320), generalised from two genomes
 * to n. by_weight != 0: each genome gets all genomes' xforms, the foreign ones
 * with weight 0; otherwise xforms align by position and missing vlinks are
 * padded. out receives n new handles (rfk_flame_destroy each). */
rfk_status rfk_flames_align(const rfk_db* db, const rfk_flame* const* flames, size_t n, int by_weight, rfk_flame** out);

/* ---- batched rendering -----------------------------------------------------
 * No reference counterpart: the reference renders one flame per
 * flame_kernel::bin call (flame_compiler.h:92-98). A batch renders many units
 * (flames or animation frames) of the kernel's structure in one persistent
 * launch: each unit's parameter block is the spline of the batch's packed
 * samples at (segment, t), evaluated on the device; every unit iterates into
 * its own histogram until its quality target, then gets its own
 * density-estimation blur and tonemap. rfk_batch_run enqueues the whole
 * pipeline (sample upload, rotation fix-up, spline, prepare, clear, iterate,
 * blur, tonemap, counter read-back) on a stream, directly or as one CUDA
 * graph captured on the first run and replayed afterwards. */
typedef struct rfk_batch rfk_batch;

typedef struct {
    uint32_t width, height;  /* image size */
    double quality;          /* target samples per pixel (as rfk_bailout.quality), > 0 */
    uint32_t segment;        /* spline segment: samples segment .. segment + 3, interpolating
                                between samples segment + 1 and segment + 2 */
    float t;                 /* position in the segment, [0, 1] */
    float gamma, brightness, vibrancy, highlight_power; /* tonemap parameters of this unit */
} rfk_batch_unit;

typedef struct {
    uint32_t passes_per_item; /* passes of one block's chains per queue item; 0 = 256 */
    uint32_t warmup;          /* passes without drawing for chains new to a unit */
    uint32_t seed;
    uint32_t millis;          /* time budget of the iterate launch; 0 or > 60000 = 60000 */
    float de_max_radius;      /* density-estimation blur (as rfk_de_args); 0 = none */
    float de_min_radius;
    float de_curve;
    int out_format;           /* RFK_HALF3 .. RFK_FLOAT4, or -1 = histograms only */
    int precise_tonemap;      /* as rfk_tonemap_args.precise */
    uint32_t item_factor;     /* queue items per unit as a multiple of the least needed at
                                 full efficiency; 0 = 3 (units whose draws fall short of
                                 1 / item_factor of the iterations may end below target) */
} rfk_batch_opts;

typedef struct {
    size_t units;
    uint64_t items;           /* queue length */
    size_t hist_bytes;        /* device bytes of all histograms */
    size_t image_bytes;       /* device bytes of all tonemapped images */
    int launches_per_run;     /* kernel launches of one run (graph nodes that are kernels) */
    int graph;                /* 1 once the pipeline is captured as a CUDA graph */
} rfk_batch_info;

/* nsamples packed samples (n x (size_reals + 768) doubles, the kernel's
 * layout) are given per run by rfk_batch_set_samples. */
rfk_status rfk_batch_create(rfk_kernel* k, const rfk_batch_unit* units, size_t nunits, size_t nsamples,
                            const rfk_batch_opts* opts, rfk_batch** out);
void rfk_batch_destroy(rfk_batch* b);
/* Copies the samples (nsamples x (size_reals + 768) doubles, as given to
 * rfk_batch_create) into the batch's pinned staging; the next run uploads them. */
rfk_status rfk_batch_set_samples(rfk_batch* b, const double* samples);
/* Enqueues one run on `stream` (cudaStream_t). use_graph != 0 captures the
 * pipeline as a CUDA graph on the first such run and replays it later. */
rfk_status rfk_batch_run(rfk_batch* b, int use_graph, void* stream);
/* Waits for the last run; fills the totals and, when per_unit is non-null,
 * one result per unit (quality = accumulated spp of the unit; status has
 * RFK_ST_QUALITY-like bit 1 set when the unit reached its target). */
rfk_status rfk_batch_wait(rfk_batch* b, rfk_bin_result* total, rfk_bin_result* per_unit);
/* Device pointers of unit u: histogram (float4 w x h), tonemapped image (NULL
 * when out_format < 0), prepared parameter block (floats, without jitter). */
void* rfk_batch_bins(rfk_batch* b, size_t unit);
void* rfk_batch_image(rfk_batch* b, size_t unit);
void* rfk_batch_params(rfk_batch* b, size_t unit);
rfk_status rfk_batch_get_info(const rfk_batch* b, rfk_batch_info* info);

/* ---- measurement helpers -------------------------------------------------- */
/* red.global.add.v4.f32 operations per second into a device buffer of
 * `bytes` (random slots): the L2-atomic roofline. */
rfk_status rfk_probe_red_v4(size_t bytes, uint32_t iters_per_thread, double* ops_per_s);
/* Issue rate of one arithmetic pipe, in lane operations per second: pipe 0 =
 * FP32 FMA, pipe 1 = special-function unit (sin.approx / rsqrt.approx). */
rfk_status rfk_probe_pipe(int pipe, uint32_t iters_per_thread, double* ops_per_s);
/* Number of SMs of the current device. */
int rfk_device_sm_count(void);

#ifdef __cplusplus
}
#endif

#endif /* RFK_H */
