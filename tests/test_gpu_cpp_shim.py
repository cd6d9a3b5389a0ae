"""The render path of the C++ shim include/rfk_cpp.h on the GPU:
flame_compiler::get_flame_kernel (f32, and the f64 request refused with a
log), flame_kernel::warmup + bin (the future), saved_state, tonemapper::run,
the adopting warm-up and denoiser::make - the program of
tests/test_cpu_cpp_shim.py built with its GPU part."""
import subprocess

import pytest

from tests.test_cpu_cpp_shim import build_shim

pytestmark = pytest.mark.gpu


def test_cpp_shim_renders_on_the_gpu(tmp_path):
    exe, args = build_shim(tmp_path, gpu=True)
    r = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "shim cpu ok" in r.stdout and "shim gpu ok" in r.stdout
