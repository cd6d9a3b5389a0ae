/*
 * rfk_cpp.h - header-only C++20 shim over rfk.h / rfk_denoise.h with the class
 * and method names of librefrakt's render path, so that code written against
 * the reference compiles against librfk with few edits.
 *
 *   rfkt::initialize(flamedb&, path)   src/librefrakt/src/flame_info.cpp:60-148
 *   rfkt::flamedb                      src/librefrakt/include/librefrakt/flame_info.h:18-157
 *   rfkt::flame, import_flam3,         src/librefrakt/include/librefrakt/flame_types.h:552-807,
 *   flame::deserialize / serialize     src/librefrakt/src/flame_types.cpp:131-239, :399-485
 *   rfkt::flame_compiler               src/librefrakt/include/librefrakt/flame_compiler.h:153-229
 *   rfkt::flame_kernel, saved_state,   flame_compiler.h:22-149
 *   bailout_args, bin_result
 *   rfkt::tonemapper                   src/librefrakt/include/librefrakt/image/tonemapper.h:6-35
 *   rfkt::denoiser (make / denoise)    src/librefrakt/include/librefrakt/interface/denoiser.h:21-39
 *
 * Differences from the reference: streams are cudaStream_t values passed as
 * void* (nullptr = the legacy default stream); images are device pointers
 * with their dimensions; the variation database is edited with text in the
 * variations_new.yml format; CUDA failures throw rfkt::gb300_error (the
 * reference logs and exits) and compile failures come back as an empty
 * kernel with the NVRTC log, as flame_compiler::result does. The library
 * computes the chain step in FP32; precision::f64 is rejected.
 */
#ifndef RFK_CPP_H
#define RFK_CPP_H

#include <cstdint>
#include <future>
#include <memory>
#include <optional>
#include <span>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "rfk.h"
#include "rfk_denoise.h"

namespace rfkt {

struct gb300_error : std::runtime_error {
    rfk_status status;
    gb300_error(rfk_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

namespace detail {
inline void check(rfk_status s, const char* call) {
    if (s != RFK_OK) throw gb300_error(s, std::string(call) + ": " + rfk_last_error());
}
template <class F>
std::string text(F&& f) {
    size_t len = 0;
    check(f(nullptr, 0, &len), "text size");
    std::string out(len + 1, '\0');
    check(f(out.data(), out.size(), &len), "text");
    out.resize(len);
    return out;
}
}  // namespace detail

class flamedb {
public:
    flamedb() = default;
    flamedb(const flamedb&) = delete;
    flamedb& operator=(const flamedb&) = delete;
    flamedb(flamedb&& o) noexcept : db_(std::exchange(o.db_, nullptr)) {}
    flamedb& operator=(flamedb&& o) noexcept {
        std::swap(db_, o.db_);
        return *this;
    }
    ~flamedb() {
        if (db_) rfk_db_destroy(db_);
    }

    /* flamedb::add_or_update_variation: every entry of a variations_new.yml
     * document; false (message in rfk_last_error) on the first invalid one. */
    bool add_or_update_variation(const std::string& yaml) { return rfk_db_add_variations(db_, yaml.c_str()) == RFK_OK; }
    bool add_or_update_common(const std::string& name, const std::string& code) {
        return rfk_db_add_common(db_, name.c_str(), code.c_str()) == RFK_OK;
    }
    bool remove_variation(const std::string& name) { return rfk_db_remove_variation(db_, name.c_str()) == 1; }
    bool remove_common(const std::string& name) { return rfk_db_remove_common(db_, name.c_str()) == 1; }
    bool is_variation(const std::string& name) const { return rfk_db_is_variation(db_, name.c_str()) == 1; }
    bool is_parameter(const std::string& variation, const std::string& param) const {
        return rfk_db_is_parameter(db_, variation.c_str(), param.c_str()) == 1;
    }
    bool is_common(const std::string& name) const { return rfk_db_is_common(db_, name.c_str()) == 1; }
    std::uint64_t hash() const { return rfk_db_hash(db_); }
    std::vector<std::string> variations() const {
        std::vector<std::string> out;
        char buf[256];
        for (int i = 0, n = rfk_db_variation_count(db_); i < n; i++) {
            detail::check(rfk_db_variation_name(db_, i, buf, sizeof buf), "rfk_db_variation_name");
            out.emplace_back(buf);
        }
        return out;
    }

    rfk_db* handle() const { return db_; }

private:
    friend bool initialize(flamedb&, const std::string&);
    rfk_db* db_ = nullptr;
};

/* rfkt::initialize: loads <config_path>/variations_new.yml and common.yml. */
inline bool initialize(flamedb& fdb, const std::string& config_path) {
    rfk_db* db = nullptr;
    if (rfk_db_load(config_path.c_str(), &db) != RFK_OK) return false;
    if (fdb.db_) rfk_db_destroy(fdb.db_);
    fdb.db_ = db;
    return true;
}

class flame {
public:
    flame(const flame&) = delete;
    flame& operator=(const flame&) = delete;
    flame(flame&& o) noexcept : f_(std::exchange(o.f_, nullptr)) {}
    flame& operator=(flame&& o) noexcept {
        std::swap(f_, o.f_);
        return *this;
    }
    ~flame() {
        if (f_) rfk_flame_destroy(f_);
    }

    /* flame::deserialize(json, fdb): nullopt when the text does not parse or
     * names a variation the database does not hold. */
    static std::optional<flame> deserialize(const std::string& json, const flamedb& fdb) {
        rfk_flame* f = nullptr;
        if (rfk_flame_from_json(fdb.handle(), json.c_str(), &f) != RFK_OK) return std::nullopt;
        return flame(f);
    }
    std::string serialize() const {
        return detail::text([&](char* b, size_t c, size_t* l) { return rfk_flame_to_json(f_, b, c, l); });
    }
    std::size_t size_reals() const { return rfk_flame_size_reals(f_); }
    /* pack_sample(packer, invoker, t, w, h) of a static genome: size_reals + 768 doubles. */
    std::vector<double> pack_sample(int w, int h) const {
        std::vector<double> out(size_reals() + 768);
        detail::check(rfk_flame_pack_sample(f_, w, h, out.data(), out.size()), "rfk_flame_pack_sample");
        return out;
    }
    /* count copies of pack_sample, as a renderer of a still frame passes them. */
    std::vector<double> pack_samples(int count, int w, int h) const {
        const std::vector<double> one = pack_sample(w, h);
        std::vector<double> out;
        out.reserve(one.size() * count);
        for (int i = 0; i < count; i++) out.insert(out.end(), one.begin(), one.end());
        return out;
    }
    std::vector<std::size_t> affine_indices() const {
        size_t n = 0;
        detail::check(rfk_flame_affine_indices(f_, nullptr, 0, &n), "rfk_flame_affine_indices");
        std::vector<std::size_t> out(n);
        detail::check(rfk_flame_affine_indices(f_, out.data(), n, &n), "rfk_flame_affine_indices");
        return out;
    }
    std::uint64_t hash() const { return rfk_flame_structure_hash(f_); }

    rfk_flame* handle() const { return f_; }

private:
    friend std::optional<flame> import_flam3(const flamedb&, const std::string&);
    explicit flame(rfk_flame* f) : f_(f) {}
    rfk_flame* f_ = nullptr;
};

/* rfkt::import_flam3(fdb, xml): the first <flame> of a flam3 document. */
inline std::optional<flame> import_flam3(const flamedb& fdb, const std::string& xml) {
    rfk_flame* f = nullptr;
    if (rfk_flame_from_flam3(fdb.handle(), xml.c_str(), &f) != RFK_OK) return std::nullopt;
    return flame(f);
}

struct bailout_args {
    std::uint32_t iters = 4'000'000'000u;  // reference default; any value above a pass cap is no cap
    std::uint32_t millis = 1000;
    double quality = 128.0;
};

struct bin_result {
    double quality = 0;
    double elapsed_ms = 0;
    std::size_t total_passes = 0;
    std::size_t total_draws = 0;
    std::size_t total_bins = 0;
    double passes_per_thread = 0;
    double max_density = 0;
    std::uint32_t status = 0;  // 1 quality, 2 time, 4 aborted, 8 pass cap
};

class flame_kernel;

/* flame_kernel::saved_state: the histogram, chains and counters of one render. */
class saved_state {
public:
    saved_state(const saved_state&) = delete;
    saved_state& operator=(const saved_state&) = delete;
    saved_state(saved_state&& o) noexcept : s_(std::exchange(o.s_, nullptr)), w_(o.w_), h_(o.h_) {}
    saved_state& operator=(saved_state&& o) noexcept {
        std::swap(s_, o.s_);
        std::swap(w_, o.w_);
        std::swap(h_, o.h_);
        return *this;
    }
    ~saved_state() {
        if (s_) rfk_state_destroy(s_);
    }
    /* Safe from any thread: stops the bin call running on this state. */
    void abort_binning() { rfk_state_abort(s_); }
    /* Device float4 histogram, w x h, row-major. */
    float* bins() const { return rfk_state_bins(s_); }
    std::uint32_t width() const { return w_; }
    std::uint32_t height() const { return h_; }
    double quality() const { return rfk_state_quality(s_); }

    rfk_state* handle() const { return s_; }

private:
    friend class flame_kernel;
    saved_state(rfk_state* s, std::uint32_t w, std::uint32_t h) : s_(s), w_(w), h_(h) {}
    rfk_state* s_ = nullptr;
    std::uint32_t w_ = 0, h_ = 0;
};

class flame_kernel {
public:
    flame_kernel(const flame_kernel&) = delete;
    flame_kernel& operator=(const flame_kernel&) = delete;
    flame_kernel(flame_kernel&& o) noexcept : k_(std::exchange(o.k_, nullptr)) {}
    flame_kernel& operator=(flame_kernel&& o) noexcept {
        std::swap(k_, o.k_);
        return *this;
    }
    ~flame_kernel() {
        if (k_) rfk_kernel_destroy(k_);
    }

    /* warmup(stream, samples, dims, seed, count, temporal_multiplier): a new
     * state with a cleared histogram of dims.x x dims.y (Dims: CUDA's uint2
     * or any type with x and y). */
    template <class Dims>
    saved_state warmup(void* stream, std::span<const double> samples, const Dims& dims, std::uint32_t seed,
                       std::uint32_t count, int temporal_multiplier = 1) const {
        rfk_state* s = nullptr;
        detail::check(rfk_warmup(k_, samples.data(), samples.size() / sample_size(), dims.x, dims.y, seed, count,
                                 temporal_multiplier, stream, &s),
                      "rfk_warmup");
        return saved_state(s, dims.x, dims.y);
    }
    /* warmup(stream, samples, gpu_image<float4>&& bins, ...): draws on top of
     * the caller's w x h float4 image, which must outlive the state. */
    saved_state warmup(void* stream, std::span<const double> samples, float* bins, std::uint32_t w, std::uint32_t h,
                       std::uint32_t seed, std::uint32_t count, int temporal_multiplier = 1) const {
        rfk_state* s = nullptr;
        detail::check(rfk_warmup_adopt(k_, samples.data(), samples.size() / sample_size(), bins, w, h, seed, count,
                                       temporal_multiplier, stream, &s),
                      "rfk_warmup_adopt");
        return saved_state(s, w, h);
    }
    /* bin(stream, state, bailout, temporal_slicing): enqueued now, the result
     * through the future. The state must outlive the future's get(). */
    std::future<bin_result> bin(void* stream, saved_state& state, const bailout_args& bo,
                                int temporal_slicing = 100) const {
        rfk_bailout b{bo.iters, bo.millis, bo.quality, (std::uint32_t)temporal_slicing};
        detail::check(rfk_bin_async(state.handle(), &b, stream), "rfk_bin_async");
        rfk_state* s = state.handle();
        return std::async(std::launch::async, [s] {
            rfk_bin_result r{};
            detail::check(rfk_bin_wait(s, &r), "rfk_bin_wait");
            bin_result out;
            out.quality = r.quality;
            out.elapsed_ms = r.elapsed_ms;
            out.total_passes = r.total_passes;
            out.total_draws = r.total_draws;
            out.total_bins = r.total_bins;
            out.passes_per_thread = r.passes_per_thread;
            out.max_density = r.max_density;
            out.status = r.status;
            return out;
        });
    }
    rfk_kernel_info info() const {
        rfk_kernel_info i{};
        detail::check(rfk_kernel_get_info(k_, &i), "rfk_kernel_get_info");
        return i;
    }
    std::size_t sample_size() const { return info().size_reals + 768; }

    rfk_kernel* handle() const { return k_; }

private:
    friend class flame_compiler;
    explicit flame_kernel(rfk_kernel* k) : k_(k) {}
    rfk_kernel* k_ = nullptr;
};

enum class precision { f32, f64 };

class flame_compiler {
public:
    struct result {
        std::optional<flame_kernel> kernel;
        std::string source;
        std::string log;
        double compile_ms = 0;
    };
    /* get_flame_kernel(fdb, precision, flame): one kernel per flame structure
     * (cached inside the library); `opts` carries the launch shape, e.g. from
     * autotune(). An empty kernel and the NVRTC log on failure. */
    result get_flame_kernel(const flamedb& fdb, precision prec, const flame& f, const rfk_compile_opts* opts = nullptr) {
        result r;
        if (prec != precision::f32) {
            r.log = "librfk computes the chain step in FP32 only";
            return r;
        }
        rfk_compile_opts o{};
        if (opts) o = *opts;
        std::vector<char> log(1 << 16, '\0');
        rfk_kernel* k = nullptr;
        if (rfk_compile(fdb.handle(), f.handle(), &o, &k, log.data(), log.size()) != RFK_OK) {
            r.log = std::string(log.data()) + rfk_last_error();
            return r;
        }
        r.log = log.data();
        flame_kernel fk(k);
        r.compile_ms = fk.info().compile_ms;
        r.source = detail::text([&](char* b, size_t c, size_t* l) { return rfk_kernel_source(k, b, c, l); });
        r.kernel.emplace(std::move(fk));
        return r;
    }
    /* The library's autotuner (no reference counterpart): launch shape and
     * flush strategy timed on this flame at this size. */
    static rfk_compile_opts autotune(const flamedb& fdb, const flame& f, std::span<const double> samples, std::uint32_t w,
                                     std::uint32_t h, std::uint32_t passes = 256) {
        rfk_compile_opts o{};
        rfk_tune_report rep{};
        detail::check(rfk_autotune(fdb.handle(), f.handle(), samples.data(), samples.size() / (f.size_reals() + 768), w, h,
                                   passes, &o, &rep),
                      "rfk_autotune");
        return o;
    }
};

class tonemapper {
public:
    struct args_t {
        double quality;
        double gamma;
        double brightness;
        double vibrancy;
        double max_density = 0.0;
    };
    enum class format { half3 = RFK_HALF3, half4 = RFK_HALF4, float3 = RFK_FLOAT3, float4 = RFK_FLOAT4 };
    /* run(bins, out, args, stream): device float4 histogram in, device image out. */
    void run(const float* bins, void* out, format fmt, std::uint32_t w, std::uint32_t h, const args_t& a,
             void* stream) const {
        rfk_tonemap_args t{a.quality, a.gamma, a.brightness, a.vibrancy, a.max_density, -1.0, 1};
        detail::check(rfk_tonemap(bins, w, h, out, (int)fmt, &t, nullptr, nullptr, stream), "rfk_tonemap");
    }
};

class denoiser {
public:
    denoiser(const denoiser&) = delete;
    denoiser& operator=(const denoiser&) = delete;
    ~denoiser() {
        if (d_) rfk_denoiser_destroy(d_);
    }
    /* denoiser::make(name, ...): nullptr for a name that is not registered.
     * weights_path: an .npz weight file, or empty for seeded initial weights. */
    static std::unique_ptr<denoiser> make(const std::string& name, const std::string& weights_path = "") {
        rfk_denoiser* d = nullptr;
        if (rfk_denoiser_make(name.c_str(), weights_path.empty() ? nullptr : weights_path.c_str(), &d) != RFK_OK)
            return nullptr;
        return std::unique_ptr<denoiser>(new denoiser(d));
    }
    /* denoise: the low-spp histogram and its tonemapped float4 image in, the
     * denoised image out (w, h multiples of 8). */
    void denoise(const float* bins, const float* base, std::uint32_t w, std::uint32_t h, double spp, void* out,
                 tonemapper::format fmt, void* stream) const {
        detail::check(rfk_denoise(d_, bins, base, w, h, spp, out, (int)fmt, stream), "rfk_denoise");
    }

private:
    explicit denoiser(rfk_denoiser* d) : d_(d) {}
    rfk_denoiser* d_ = nullptr;
};

}  // namespace rfkt

#endif /* RFK_CPP_H */
