"""Tensor-core kernels of the denoiser against a plain PyTorch fp32 reference
of the same op on the same bf16-rounded inputs: the 3x3 convolution (forward,
input gradient through transposed/flipped weights, channel slices, bias,
ReLU, mask, accumulate) and the weight gradient."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
F = torch.nn.functional

from refraktor_gb300 import _lib

pytestmark = pytest.mark.gpu


def _L():
    L = _lib.lib()
    L.rfk_unet_conv3x3.restype = C.c_int
    L.rfk_unet_conv3x3.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                   C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                   C.c_int, C.c_void_p, C.c_void_p]
    L.rfk_unet_wgrad3x3.restype = C.c_int
    L.rfk_unet_wgrad3x3.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return L


def _bf16_close(got, ref, scale):
    """Within one bf16 rounding of the fp32 reference (plus fp32 summation-order
    noise relative to the output scale)."""
    got = got.float()
    ulp = torch.where(ref.abs() > 0, 2.0 ** (torch.floor(torch.log2(ref.abs())) - 7), torch.zeros_like(ref))
    err = (got - ref).abs()
    bound = 1.01 * ulp + 1e-5 * scale
    assert bool((err <= bound).all()), float((err - bound).max())


def _conv(L, x, cin_off, cin, w_nkc, cout, bias=None, relu=0, out=None, out_coff=0, mask=None, mask_coff=0, acc=0):
    n, h, wd, cst = x.shape
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.rfk_unet_conv3x3(x.data_ptr(), n, h, wd, cst, cin_off, cin, w_nkc.data_ptr(), cout,
                            None if bias is None else bias.data_ptr(), relu, out.data_ptr(), out.shape[3], out_coff,
                            None if mask is None else mask.data_ptr(), 0 if mask is None else mask.shape[3], mask_coff, acc,
                            err.data_ptr(), None)
    assert rc == 0, rc
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return out


def _ref_conv(x_nhwc, w_nkc, bias):
    """fp32 reference: NHWC input slice, weights [cout][9][cin]."""
    cout, _, cin = w_nkc.shape
    wt = w_nkc.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    y = F.conv2d(x_nhwc.float().permute(0, 3, 1, 2), wt, None if bias is None else bias.float(), padding=1)
    return y.permute(0, 2, 3, 1)


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 5, 200, 64, 128), (1, 4, 64, 32, 32), (2, 3, 130, 96, 64),
                                            (1, 3, 256, 384, 256), (1, 2, 128, 256, 32), (3, 6, 70, 128, 64),
                                            (2, 9, 260, 96, 32)])
def test_conv3x3_matches_fp32_reference(n, h, w, cin, cout):
    L = _L()
    g = torch.Generator(device="cuda").manual_seed(n * 1000 + cin + cout)
    x = torch.randn(n, h, w, cin, device="cuda", generator=g).to(torch.bfloat16)
    wt = (torch.randn(cout, 9, cin, device="cuda", generator=g) / np.sqrt(9 * cin)).to(torch.bfloat16)
    b = torch.randn(cout, device="cuda", generator=g)
    out = torch.empty(n, h, w, cout, dtype=torch.bfloat16, device="cuda")
    _conv(L, x, 0, cin, wt, cout, bias=b, relu=1, out=out)
    ref = torch.relu(_ref_conv(x, wt, b))
    _bf16_close(out, ref, float(ref.abs().max()))


def test_conv3x3_slices_mask_and_accumulate():
    """Input channel slice of a wider tensor, output into a slice of another,
    multiplication by (mask > 0), accumulation into what the output holds:
    the input-gradient path of the U-Net's concatenations."""
    L = _L()
    g = torch.Generator(device="cuda").manual_seed(7)
    n, h, w, cin, cout = 2, 7, 150, 64, 32
    big = torch.randn(n, h, w, 160, device="cuda", generator=g).to(torch.bfloat16)
    wt = (torch.randn(cout, 9, cin, device="cuda", generator=g) / 24).to(torch.bfloat16)
    mask = torch.randn(n, h, w, 96, device="cuda", generator=g).to(torch.bfloat16)
    out = torch.randn(n, h, w, 128, device="cuda", generator=g).to(torch.bfloat16)
    before = out.clone()
    _conv(L, big, 64, cin, wt, cout, out=out, out_coff=64, mask=mask, mask_coff=32, acc=1)
    ref = _ref_conv(big[..., 64:128], wt, None)
    ref = torch.where(mask[..., 32:64].float() > 0, ref, torch.zeros_like(ref)) + before[..., 64:96].float()
    _bf16_close(out[..., 64:96], ref, float(ref.abs().max()))
    # channels outside the written slice are untouched
    assert torch.equal(out[..., :64], before[..., :64]) and torch.equal(out[..., 96:], before[..., 96:])


@pytest.mark.parametrize("cin,cout", [(256, 256), (128, 128), (64, 64)])
def test_conv3x3_fused_upsample_store(cin, cout):
    """RFK_UNET_UP2: the epilogue stores each output pixel at its 2x2 pixels
    of a (2h, 2w) output, in a channel slice of a wider tensor (the decoder's
    concatenation): the same values as the convolution followed by nearest
    upsampling, and the other channels untouched."""
    L = _L()
    g = torch.Generator(device="cuda").manual_seed(cin + 3)
    n, h, w = 2, 6, 68
    x = torch.randn(n, h, w, cin, device="cuda", generator=g).to(torch.bfloat16)
    wt = (torch.randn(cout, 9, cin, device="cuda", generator=g) / np.sqrt(9 * cin)).to(torch.bfloat16)
    b = torch.randn(cout, device="cuda", generator=g)
    wide = cout + cout // 2
    out = torch.randn(n, 2 * h, 2 * w, wide, device="cuda", generator=g).to(torch.bfloat16)
    before = out.clone()
    _conv(L, x, 0, cin, wt, cout, bias=b, relu=1 | 4, out=out, out_coff=0)
    ref = torch.relu(_ref_conv(x, wt, b))
    ref_up = ref.repeat_interleave(2, dim=1).repeat_interleave(2, dim=2)
    _bf16_close(out[..., :cout], ref_up, float(ref.abs().max()))
    assert torch.equal(out[..., cout:], before[..., cout:])
    # f32 or accumulating outputs are not combined with the upsampling store
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.rfk_unet_conv3x3(x.data_ptr(), n, h, w, cin, 0, cin, wt.data_ptr(), cout, b.data_ptr(), 1 | 2 | 4,
                            out.data_ptr(), wide, 0, None, 0, 0, 0, err.data_ptr(), None)
    assert rc != 0


def test_conv3x3_input_gradient_with_flipped_weights():
    """dX of y = conv(x, W) is conv(dY, W'), W'[c][8 - t][n] = W[n][t][c]."""
    L = _L()
    g = torch.Generator(device="cuda").manual_seed(11)
    n, h, w, cin, cout = 2, 9, 128, 64, 128
    x = torch.randn(n, cin, h, w, device="cuda", generator=g).to(torch.bfloat16).float().requires_grad_(True)
    wt = (torch.randn(cout, 9, cin, device="cuda", generator=g) / 24).to(torch.bfloat16)
    y = F.conv2d(x, wt.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2), padding=1)
    dy = torch.randn_like(y).to(torch.bfloat16)
    y.backward(dy.float())
    wflip = wt.flip(1).permute(2, 1, 0).contiguous()  # [cin][9][cout]
    dx = torch.empty(n, h, w, cin, dtype=torch.bfloat16, device="cuda")
    _conv(L, dy.permute(0, 2, 3, 1).contiguous(), 0, cout, wflip, cin, out=dx)
    ref = x.grad.permute(0, 2, 3, 1)
    _bf16_close(dx, ref, float(ref.abs().max()))


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 3, 128, 32, 32), (1, 4, 64, 64, 128), (2, 2, 192, 128, 256),
                                            (1, 3, 128, 96, 64), (3, 5, 192, 96, 32)])
def test_wgrad3x3_matches_fp32_reference(n, h, w, cin, cout):
    L = _L()
    g = torch.Generator(device="cuda").manual_seed(cin * 7 + cout)
    x = torch.randn(n, h, w, cin, device="cuda", generator=g).to(torch.bfloat16)
    dy = torch.randn(n, h, w, cout, device="cuda", generator=g).to(torch.bfloat16)
    dw = torch.zeros(cout, 9, cin, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    # X read in place: a channel slice of a wider NHWC tensor
    wide = torch.randn(n, h, w, cin + 64, device="cuda", generator=g).to(torch.bfloat16)
    wide[..., 32:32 + cin] = x
    assert L.rfk_unet_wgrad3x3(dy.data_ptr(), wide.data_ptr(), cin + 64, 32, n, h, w, cout, cin, dw.data_ptr(),
                               err.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = torch.nn.grad.conv2d_weight(x.float().permute(0, 3, 1, 2), (cout, cin, 3, 3), dy.float().permute(0, 3, 1, 2),
                                      padding=1)
    ref = ref.permute(0, 2, 3, 1).reshape(cout, 9, cin)
    torch.testing.assert_close(dw, ref, rtol=1e-4, atol=1e-4 * float(ref.abs().max()))
