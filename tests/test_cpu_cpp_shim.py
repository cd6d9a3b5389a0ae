"""The header-only C++ shim include/rfk_cpp.h (the reference's rfkt:: class and
method names over the C ABI) compiles against rfk.h with g++ -std=c++20 and
links against librfk. Without a GPU the program exercises the database,
genome and factory parts; tests/test_gpu_cpp_shim.py runs the same program's
render path on the GPU."""
import json
import shutil
import subprocess
from pathlib import Path

import pytest

from refraktor_gb300 import build
from refraktor_gb300 import synthetic as syn

ROOT = Path(__file__).resolve().parent.parent
CUDA = Path("/usr/local/cuda")

PROGRAM = r"""
#include "rfk_cpp.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>

#ifdef SHIM_GPU
#include <cuda_runtime.h>
#endif

static std::string read_file(const char* path) {
    std::ifstream f(path);
    std::stringstream s;
    s << f.rdbuf();
    return s.str();
}

#define REQUIRE(c)                                                \
    do {                                                          \
        if (!(c)) {                                               \
            std::printf("FAILED %s at line %d\n", #c, __LINE__); \
            return 1;                                             \
        }                                                         \
    } while (0)

struct dims_t {
    std::uint32_t x, y;
};

int main(int argc, char** argv) {
    // argv: config dir, genome json file, flam3 file, expected size_reals
    rfkt::flamedb fdb;
    REQUIRE(!rfkt::initialize(fdb, "/nonexistent-config-dir"));
    REQUIRE(rfkt::initialize(fdb, argv[1]));
    REQUIRE(fdb.is_variation("julia") && !fdb.is_variation("no_such_variation"));
    REQUIRE(fdb.is_common("sqrt"));
    const auto h0 = fdb.hash();
    REQUIRE(fdb.add_or_update_variation("shim_probe: result += weight * p;\n"));
    REQUIRE(fdb.is_variation("shim_probe") && fdb.hash() != h0);
    REQUIRE(fdb.remove_variation("shim_probe") && !fdb.is_variation("shim_probe"));
    REQUIRE(!fdb.add_or_update_variation("shim_bad: result += weight * param.missing * p;\n"));
    REQUIRE(fdb.variations().size() > 40);

    auto f = rfkt::flame::deserialize(read_file(argv[2]), fdb);
    REQUIRE(f.has_value());
    REQUIRE(!rfkt::flame::deserialize("{ not json", fdb).has_value());
    REQUIRE(f->size_reals() == (std::size_t)std::atol(argv[4]));
    const auto samples = f->pack_samples(4, 128, 128);
    REQUIRE(samples.size() == 4 * (f->size_reals() + 768));
    REQUIRE(!f->affine_indices().empty());
    auto again = rfkt::flame::deserialize(f->serialize(), fdb);
    REQUIRE(again.has_value() && again->hash() == f->hash());
    auto sheep = rfkt::import_flam3(fdb, read_file(argv[3]));
    REQUIRE(sheep.has_value() && sheep->size_reals() > 0);
    REQUIRE(!rfkt::import_flam3(fdb, "<flames></flames>").has_value());
    REQUIRE(rfkt::denoiser::make("rfkt::no_such_denoiser") == nullptr);
    std::printf("shim cpu ok: %zu reals\n", f->size_reals());

#ifdef SHIM_GPU
    rfkt::flame_compiler fc;
    auto bad = fc.get_flame_kernel(fdb, rfkt::precision::f64, *f);
    REQUIRE(!bad.kernel.has_value() && !bad.log.empty());
    auto res = fc.get_flame_kernel(fdb, rfkt::precision::f32, *f);
    REQUIRE(res.kernel.has_value() && !res.source.empty());
    const rfkt::flame_kernel& k = *res.kernel;
    cudaStream_t stream;
    REQUIRE(cudaStreamCreate(&stream) == cudaSuccess);
    auto st = k.warmup(stream, samples, dims_t{128, 128}, 7, 20);
    auto fut = k.bin(stream, st, rfkt::bailout_args{0, 0, 4.0});
    const rfkt::bin_result r = fut.get();
    REQUIRE((r.status & 1) && r.quality >= 4.0 && r.total_bins == 128u * 128u);
    REQUIRE(std::fabs(st.quality() - r.quality) < 1e-9);
    float* img = nullptr;
    REQUIRE(cudaMalloc(&img, 128 * 128 * 16) == cudaSuccess);
    rfkt::tonemapper tm;
    tm.run(st.bins(), img, rfkt::tonemapper::format::float4, 128, 128, {st.quality(), 2.2, 4.0, 1.0}, stream);
    std::vector<float> host(128 * 128 * 4);
    REQUIRE(cudaMemcpy(host.data(), img, host.size() * 4, cudaMemcpyDeviceToHost) == cudaSuccess);
    int lit = 0;
    for (std::size_t i = 0; i < host.size(); i++) {
        REQUIRE(std::isfinite(host[i]) && host[i] >= 0.0f && host[i] <= 1.0f);
        if (i % 4 == 3 && host[i] > 0.0f) lit++;
    }
    REQUIRE(lit > 100);
    // adopted histogram: draws go on top of the caller's image
    auto st2 = k.warmup(stream, samples, st.bins(), 128, 128, 8, 20);
    const rfkt::bin_result r2 = k.bin(stream, st2, rfkt::bailout_args{0, 0, 1.0}).get();
    REQUIRE(r2.status & 1);
    auto dn = rfkt::denoiser::make("rfkt::gb300_unet_denoiser");
    REQUIRE(dn != nullptr);
    cudaFree(img);
    cudaStreamDestroy(stream);
    std::printf("shim gpu ok: %.2f spp, %zu passes, %d lit pixels\n", r.quality, r.total_passes, lit);
#endif
    return 0;
}
"""

SHEEP = """<flames><flame name="t" size="640 480" center="0.1 -0.2" scale="120" rotate="10" brightness="3"
  gamma="2.5" vibrancy="0.8">
  <xform weight="0.7" color="0.2" spherical="0.5" julia="0.5" coefs="0.5 0.1 -0.1 0.5 0.2 0.3" post="1 0 0 1 0.5 0"/>
  <xform weight="0.3" color="0.9" linear="1" coefs="0.3 0 0 0.3 0 0"/>
  <palette count="256" format="RGB">""" + "FF0000" * 128 + "00FF00" * 128 + """</palette>
  </flame></flames>"""


def build_shim(tmp: Path, gpu: bool) -> tuple[Path, list[str]]:
    """Compiles the shim program; returns the executable and its arguments."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    lib = build.build()
    (tmp / "shim.cpp").write_text(PROGRAM)
    exe = tmp / ("shim_gpu" if gpu else "shim")
    cmd = [cxx, "-std=c++20", "-O1", "-Wall", f"-I{ROOT / 'include'}", str(tmp / "shim.cpp"), "-o", str(exe),
           f"-L{lib.parent}", "-lrfk", f"-Wl,-rpath,{lib.parent}"]
    if gpu:
        cmd += ["-DSHIM_GPU", f"-I{CUDA / 'include'}", f"-L{CUDA / 'lib64'}", "-lcudart", f"-Wl,-rpath,{CUDA / 'lib64'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    from refraktor_gb300 import librefrakt as lr

    g = syn.plain_flame(0)
    (tmp / "genome.json").write_text(json.dumps(g))
    (tmp / "sheep.flam3").write_text(SHEEP)
    reals = lr.flame.from_json(lr.flamedb(), g).size_reals()
    return exe, [str(build.PKG / "config"), str(tmp / "genome.json"), str(tmp / "sheep.flam3"), str(reals)]


def test_cpp_shim_compiles_and_runs_without_a_gpu(tmp_path):
    exe, args = build_shim(tmp_path, gpu=False)
    r = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "shim cpu ok" in r.stdout
