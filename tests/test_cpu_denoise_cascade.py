"""Host-side accounting of the denoised path's cascade
(refraktor_gb300/workloads/train_denoiser.py: cascade_time) on hand-made
evaluation rows: each stage's render, tonemap and U-Net are paid, a stage is
skipped once the plain image reached 40 dB, and the plain render finishes
frames that no stage brought to 40 dB."""
import pytest

from refraktor_gb300.workloads import train_denoiser as td

CK = td.FALLBACK_CHECKPOINTS
STAGES = (32, 64, 128)


def _row(den, s40, tb40, warm=1.0, tm=0.1, unet=2.0):
    # bin time to checkpoint c: c / 10 (a flame that renders 10 spp per time unit)
    t_bin = [c / 10.0 for c in CK]
    return {"spp": [float(c) for c in CK], "t_bin": t_bin, "t_tonemap": tm, "t_warmup": warm,
            "spp_to_40db": s40, "tb40": tb40, "t_unet_at": {str(s): unet for s in STAGES},
            "psnr_denoised_at": {str(s): d for s, d in zip(STAGES, den)}}


def test_first_stage_reaches_40db():
    r = _row([41.0, 45.0, 47.0], s40=300.0, tb40=30.0)
    assert td.cascade_time(r, STAGES) == pytest.approx(1.0 + 3.2 + 0.1 + 2.0)


def test_second_stage_pays_the_render_to_64_spp_and_a_second_unet():
    r = _row([39.0, 40.5, 47.0], s40=300.0, tb40=30.0)
    assert td.cascade_time(r, STAGES) == pytest.approx(1.0 + 3.2 + 0.1 + 2.0 + (6.4 - 3.2) + 0.1 + 2.0)


def test_plain_image_done_before_a_stage_skips_its_unet():
    # the plain render reaches 40 dB at 50 spp: after the failed 32-spp stage
    # the render continues to that spp and stops there
    r = _row([39.0, 45.0, 47.0], s40=50.0, tb40=5.0)
    assert td.cascade_time(r, STAGES) == pytest.approx(1.0 + 3.2 + 0.1 + 2.0 + (5.0 - 3.2) + 0.1)


def test_default_cascade_starts_at_32_spp():
    assert td.CASCADE_SPP[0] == 32 and list(td.CASCADE_SPP) == sorted(td.CASCADE_SPP)
    assert all(s in CK for s in td.CASCADE_SPP)


def test_every_stage_failing_falls_back_to_the_plain_render():
    r = _row([35.0, 37.0, 39.0], s40=400.0, tb40=40.0)
    staged = 1.0 + 3.2 + 0.1 + 2.0 + (6.4 - 3.2) + 0.1 + 2.0 + (12.8 - 6.4) + 0.1 + 2.0
    assert td.cascade_time(r, STAGES) == pytest.approx(staged + (40.0 - 12.8) + 0.1)
    # the single attempt: one U-Net at 32 spp, then the plain render
    assert td.cascade_time(r, STAGES[:1]) == pytest.approx(1.0 + 3.2 + 0.1 + 2.0 + (40.0 - 3.2) + 0.1)
