"""Philox4x32-10 of the kernel prelude on the GPU: the prelude text
(csrc/jit/rfk_device.cuh, which the flame compiler prepends to every
chaos-game kernel) NVRTC-compiled for sm_103a with a one-line kernel around
rfk_philox, against the Random123 known-answer vectors and the Python
restatement of the published round function."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle.build_ref import compile_module
from refraktor_gb300 import build
from oracle import refkernels
from tests.test_cpu_philox import KAT, philox_py, random_cases

pytestmark = pytest.mark.gpu

KERNEL = r"""
extern "C" __global__ void philox_kat(const unsigned* in, unsigned* out, unsigned n) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    rfk_u32x4 c;
    c.x = in[6 * i]; c.y = in[6 * i + 1]; c.z = in[6 * i + 2]; c.w = in[6 * i + 3];
    const rfk_u32x4 r = rfk_philox(c, in[6 * i + 4], in[6 * i + 5]);
    out[4 * i] = r.x; out[4 * i + 1] = r.y; out[4 * i + 2] = r.z; out[4 * i + 3] = r.w;
}
"""


def test_device_philox_matches_the_vectors():
    src = (build.CSRC / "jit" / "rfk_device.cuh").read_text() + KERNEL
    cubin, names = compile_module(src, "philox_kat", ["philox_kat"], ["-use_fast_math"])
    rt = refkernels._rt()
    buf = C.create_string_buffer(cubin, len(cubin))
    lib, k = C.c_void_p(), C.c_void_p()
    assert rt.cudaLibraryLoadData(C.byref(lib), buf, None, None, 0, None, None, 0) == 0
    assert rt.cudaLibraryGetKernel(C.byref(k), lib, names["philox_kat"].encode()) == 0
    cases = [(c, key) for c, key, _ in KAT] + random_cases(256)
    inp = torch.tensor(np.array([[*c, *key] for c, key in cases], dtype=np.uint64).astype(np.uint32).view(np.int32),
                       device="cuda")
    out = torch.zeros((len(cases), 4), dtype=torch.int32, device="cuda")
    refkernels.launch(k, (len(cases) + 127) // 128, 128,
                      [C.c_void_p(inp.data_ptr()), C.c_void_p(out.data_ptr()), C.c_uint(len(cases))])
    got = out.cpu().numpy().view(np.uint32)
    for (c, key), row in zip(cases, got):
        assert tuple(int(v) for v in row) == philox_py(c, key)
    for (c, key, want), row in zip(KAT, got):
        assert tuple(int(v) for v in row) == want
    rt.cudaLibraryUnload(lib)
