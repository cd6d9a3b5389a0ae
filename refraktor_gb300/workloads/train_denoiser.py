"""Trains the learned denoiser on renders of this library and evaluates it
against the plain path (the learned-denoiser workload):

  training     `--train` seeded flames of the 1080p workload's distribution
               (8 xforms, Dirichlet(1) weights, final xform, 1-3 variations
               each from the 14-variation set), visibility-rejected and framed
               at 512 x 512; input: the 32-spp histogram and its tonemapped
               image, and in turn the 64-spp ones (--input-spp; the network's
               log-spp channel tells them apart), target: the tonemapped
               4096-spp render; Adam, lr 1e-3 (cosine decay), batch 16,
               random mirroring
  evaluation   `--eval` held-out seeded flames at 1920 x 1080: the plain path
               renders to 32, 64, ..., 4096 spp (one progressive render), the
               denoised path denoises its 32-spp histogram; both are scored by
               PSNR against an independent 4096-spp render, and the spp the
               plain path needs for 40 dB is interpolated on log2(spp)

Writes the weights (denoiser_weights.npz) and the evaluation record
(denoiser_eval.json) next to this file, or under --out.
Run: python -m refraktor_gb300.workloads.train_denoiser [--train N] [--eval N] [--steps N]
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
TRAIN_SEED0, EVAL_SEED0 = 100_000, 900_000
LOW_SPP, HIGH_SPP = 32.0, 4096.0
CHECKPOINTS = [32, 64, 128, 256, 512, 1024, 2048, 4096]


def log(*a):
    print(time.strftime("%H:%M:%S"), *a, flush=True)


def dataset(db, n: int, seed0: int, w: int, h: int):
    from refraktor_gb300 import denoise as dn
    from refraktor_gb300 import synthetic as syn

    return dn.visible_set(db, syn.hd_flame, list(range(seed0, seed0 + int(n * 3.5) + 16)), n, w, h)


def spp_for(psnrs: list[float], target: float = 40.0) -> float:
    """log2-linear interpolation of the spp where the PSNR curve crosses target
    (inf when it never does within the checkpoints)."""
    for i, p in enumerate(psnrs):
        if p >= target:
            if i == 0:
                return float(CHECKPOINTS[0])
            a, b = psnrs[i - 1], p
            f = (target - a) / (b - a) if b > a else 1.0
            return float(2 ** (np.log2(CHECKPOINTS[i - 1]) + f))
    return float("inf")


def evaluate(db, net, genomes, w: int, h: int, seed: int = 7) -> dict:
    import torch

    from refraktor_gb300 import denoise as dn
    from refraktor_gb300 import librefrakt as lr

    fs = [lr.flame.from_json(db, g) for g in genomes]
    # one union kernel for the set (the genomes share their structure), with
    # the launch shape the autotuner picks on the first flame
    opts, _ = lr.autotune(db, fs[0], fs[0].pack_samples(4, w, h), (w, h))
    k = lr.flame_compiler().get_flame_kernel(db, fs[0], **opts)
    tm = lr.tonemapper()
    img = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    ref = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    den = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    rows = []
    render_ms_per_spp = []
    den_ms = []
    for i, f in enumerate(fs):
        tp = f.tonemap_params()
        samples = f.pack_samples(4, w, h)
        # independent reference
        st_ref = k.warmup(samples, (w, h), seed=seed + 2 * i + 1, count=20)
        k.bin(st_ref, lr.bailout_args(iters=0, millis=0, quality=HIGH_SPP))
        tm.run(st_ref.bins(), ref, (w, h), st_ref.quality, tp["gamma"], tp["brightness"], tp["vibrancy"], fmt=lr.FLOAT4)
        del st_ref
        # progressive plain render
        st = k.warmup(samples, (w, h), seed=seed + 2 * i, count=20)
        psnrs, done, spent = [], 0.0, 0.0
        for c in CHECKPOINTS:
            r = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=c - done))
            done = st.quality
            spent += r.elapsed_ms
            tm.run(st.bins(), img, (w, h), st.quality, tp["gamma"], tp["brightness"], tp["vibrancy"], fmt=lr.FLOAT4)
            psnrs.append(dn.psnr(img, ref))
            if c == CHECKPOINTS[0]:
                bins32 = st.bins().clone()
                base32 = img.clone()
                q32 = st.quality
                t32 = spent
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                net.denoise(bins32, base32, den, q32)
                e1.record()
                torch.cuda.synchronize()
                den_ms.append(e0.elapsed_time(e1))
                p_den = dn.psnr(den, ref)
        render_ms_per_spp.append(spent / st.quality)
        rows.append({"psnr_plain": psnrs, "psnr_denoised": p_den, "spp_to_40db": spp_for(psnrs), "ms_32spp": t32})
        del st
    ms_spp = float(np.median(render_ms_per_spp))
    den_t = float(np.median(den_ms))
    spp40 = np.array([r["spp_to_40db"] for r in rows])
    pden = np.array([r["psnr_denoised"] for r in rows])
    reached = np.isfinite(spp40)
    plain_ms = ms_spp * spp40[reached]
    den_total = ms_spp * LOW_SPP + den_t
    out = {
        "flames": len(rows), "width": w, "height": h,
        "plain_ms_per_spp": ms_spp, "denoise_ms": den_t,
        "psnr_plain_mean": {str(c): float(np.mean([r["psnr_plain"][j] for r in rows])) for j, c in enumerate(CHECKPOINTS)},
        "psnr_denoised_32spp_mean": float(pden.mean()),
        "psnr_denoised_32spp_median": float(np.median(pden)),
        "denoised_reaches_40db": float((pden >= 40.0).mean()),
        "plain_reaches_40db_within_4096": float(reached.mean()),
        "plain_spp_to_40db_median": float(np.median(spp40)) if reached.any() else None,
        "plain_s_per_frame_to_40db_median": float(np.median(plain_ms) / 1e3) if reached.any() else None,
        "denoised_s_per_frame": den_total / 1e3,
        "per_flame": rows,
    }
    both = reached & (pden >= 40.0)
    if both.any():
        out["speedup_where_both_reach_40db_median"] = float(np.median(ms_spp * spp40[both] / den_total))
    return out


FALLBACK_CHECKPOINTS = [32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096]


def evaluate_with_fallback(db, net, genomes, w: int, h: int, seed: int = 7, kernel=None) -> dict:
    """Seconds per frame to 40 dB PSNR, denoised path against plain path, with
    the plain path as the denoised path's fallback. Per flame (device time
    with CUDA events on the render stream):
      plain     warm-up + bin to the spp where the PSNR against an independent
                4096-spp render first reaches 40 dB (interpolated on log2 spp
                between checkpoints, the bin time likewise) + one tonemap;
      denoised  a cascade, each stage paid in full: warm-up + bin to 32 spp
                + tonemap + U-Net; a frame still below 40 dB continues its
                render to 64 spp and tonemaps (done if the plain image reached
                40 dB by 64 spp), else runs the U-Net again on the 64-spp
                histogram; a frame below 40 dB after that continues the plain
                render to the plain path's 40 dB spp and tonemaps again.
      32 only   the same without the 64-spp stage (keys *_32_only).
    Flames whose plain render stays below 40 dB at 4096 spp have no plain time
    and are left out of both means (counted in `plain_never_reaches`)."""
    import torch

    from refraktor_gb300 import denoise as dn
    from refraktor_gb300 import librefrakt as lr

    fs = [lr.flame.from_json(db, g) for g in genomes]
    if kernel is None:
        opts, _ = lr.autotune(db, fs[0], fs[0].pack_samples(4, w, h), (w, h))
        kernel = lr.flame_compiler().get_flame_kernel(db, fs[0], **opts)
    k = kernel
    tm = lr.tonemapper()
    stream = torch.cuda.Stream()
    img = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    ref = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    den = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return out, e0.elapsed_time(e1) / 1e3

    rows = []
    for i, f in enumerate(fs):
        tp = f.tonemap_params()
        tmargs = (tp["gamma"], tp["brightness"], tp["vibrancy"])
        samples = f.pack_samples(4, w, h)
        st_ref = k.warmup(samples, (w, h), seed=seed + 2 * i + 1, count=20, stream=stream)
        k.bin(st_ref, lr.bailout_args(iters=0, millis=0, quality=HIGH_SPP), stream=stream)
        tm.run(st_ref.bins(), ref, (w, h), st_ref.quality, *tmargs, fmt=lr.FLOAT4, stream=stream)
        stream.synchronize()
        del st_ref
        st, t_warm = timed(lambda: k.warmup(samples, (w, h), seed=seed + 2 * i, count=20, stream=stream))
        _, t_tm = timed(lambda: tm.run(st.bins(), img, (w, h), 1.0, *tmargs, fmt=lr.FLOAT4, stream=stream))
        spp, t_bin, psnrs, den_db, t_den, den64_db, den_vs_plain = [0.0], [0.0], [], None, None, None, None
        t_den64 = None
        for c in FALLBACK_CHECKPOINTS:
            _, dt = timed(lambda: k.bin(st, lr.bailout_args(iters=0, millis=0, quality=c - st.quality), stream=stream))
            spp.append(st.quality)
            t_bin.append(t_bin[-1] + dt)
            tm.run(st.bins(), img, (w, h), st.quality, *tmargs, fmt=lr.FLOAT4, stream=stream)
            stream.synchronize()
            psnrs.append(dn.psnr(img, ref))
            if c == FALLBACK_CHECKPOINTS[0]:
                _, t_den = timed(lambda: net.denoise(st.bins(), img, den, st.quality, stream=stream))
                den_db = dn.psnr(den, ref)
                # no-reference: how far the U-Net moved the plain image
                den_vs_plain = dn.psnr(den, img)
            if c == 64:
                _, t_den64 = timed(lambda: net.denoise(st.bins(), img, den, st.quality, stream=stream))
                den64_db = dn.psnr(den, ref)
            if psnrs[-1] >= 40.0 and c >= 64:
                break
        row = {"psnr_denoised": den_db, "psnr_plain": psnrs, "spp": spp[1:], "t_warmup": t_warm, "t_tonemap": t_tm,
               "t_unet": t_den, "t_bin_32": t_bin[1], "psnr_denoised_64": den64_db,
               "psnr_denoised_vs_plain_32": den_vs_plain, "t_bin": t_bin[1:]}
        if max(psnrs) >= 40.0:
            # the first checkpoint at or above 40 dB
            j = next(i for i, v in enumerate(psnrs) if v >= 40.0)
            if j == 0:
                s40, tb40 = spp[1], t_bin[1]
            else:
                a, b = psnrs[j - 1], psnrs[j]
                fr = (40.0 - a) / (b - a) if b > a else 1.0
                s40 = float(2 ** (np.log2(spp[j]) + fr * (np.log2(spp[j + 1]) - np.log2(spp[j]))))
                tb40 = t_bin[j] + fr * (t_bin[j + 1] - t_bin[j])
            plain = t_warm + tb40 + t_tm
            dpath = t_warm + t_bin[1] + t_tm + t_den
            casc = dpath
            if den_db < 40.0:
                dpath += max(tb40 - t_bin[1], 0.0) + t_tm
                # cascade: at 64 spp the plain image is done if it reached 40
                # dB by then, else the U-Net runs again; then the plain render
                i64 = FALLBACK_CHECKPOINTS.index(64) + 1
                if s40 <= 64.0:
                    casc += max(tb40 - t_bin[1], 0.0) + t_tm
                else:
                    casc += t_bin[i64] - t_bin[1] + t_tm + t_den64
                    if den64_db < 40.0:
                        casc += max(tb40 - t_bin[i64], 0.0) + t_tm
            row.update(spp_to_40db=s40, plain_s=plain, denoised_s=dpath, cascade_s=casc)
        rows.append(row)
        del st
    ok = [r for r in rows if "plain_s" in r]
    plain = np.array([r["plain_s"] for r in ok])
    dpath = np.array([r["denoised_s"] for r in ok])
    casc = np.array([r["cascade_s"] for r in ok])
    pden = np.array([r["psnr_denoised"] for r in rows])
    pden64 = np.array([r["psnr_denoised_64"] for r in rows])
    out = {
        "flames": len(rows), "width": w, "height": h, "plain_never_reaches": len(rows) - len(ok),
        "s_per_frame_to_40db_plain": float(plain.mean()) if ok else None,
        "s_per_frame_to_40db_denoised": float(casc.mean()) if ok else None,
        "speedup": float(plain.mean() / casc.mean()) if ok else None,
        "speedup_per_flame_median": float(np.median(plain / casc)) if ok else None,
        "s_per_frame_to_40db_denoised_32_only": float(dpath.mean()) if ok else None,
        "speedup_32_only": float(plain.mean() / dpath.mean()) if ok else None,
        "denoised_reaches_40db": float((pden >= 40.0).mean()),
        "denoised_64_reaches_40db": float((pden64 >= 40.0).mean()),
        "cascade_reaches_40db_by_64spp": float(np.mean([(a >= 40.0) or (b >= 40.0) or r.get("spp_to_40db", 1e9) <= 64.0
                                                        for a, b, r in zip(pden, pden64, rows)])),
        "denoised_psnr_db_mean": float(pden.mean()), "denoised_psnr_db_median": float(np.median(pden)),
        "plain_psnr_db_32spp_mean": float(np.mean([r["psnr_plain"][0] for r in rows])),
        "plain_spp_to_40db_median": float(np.median([r["spp_to_40db"] for r in ok])) if ok else None,
        "unet_ms_median": 1e3 * float(np.median([r["t_unet"] for r in rows])),
        "render_32spp_ms_median": 1e3 * float(np.median([r["t_bin_32"] + r["t_warmup"] + r["t_tonemap"] for r in rows])),
        "per_flame": rows,
    }
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2000)
    ap.add_argument("--eval", type=int, default=200)
    ap.add_argument("--steps", type=int, default=1500)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--input-spp", default="32,64",
                    help="input sample counts of the training pairs, comma separated; the steps take them in turn")
    ap.add_argument("--out", default=str(HERE))
    ap.add_argument("--eval-only", default=None,
                    help="evaluate these weights (keeping the training record of the eval file in --out)")
    args = ap.parse_args()
    import torch

    from refraktor_gb300 import build
    from refraktor_gb300 import denoise as dn
    from refraktor_gb300 import librefrakt as lr

    build.build()
    db = lr.flamedb()
    out = Path(args.out)
    if args.eval_only:
        net = dn.denoiser.load(args.eval_only)
        prev = out / "denoiser_eval.json"
        training = json.loads(prev.read_text()).get("training") if prev.exists() else None
        eval_g = dataset(db, args.eval, EVAL_SEED0, 1920, 1080)
        log("evaluation genomes", len(eval_g))
        ev = evaluate(db, net, eval_g, 1920, 1080)
        if training:
            ev["training"] = training
        prev.write_text(json.dumps(ev, indent=1))
        log(json.dumps({k: v for k, v in ev.items() if k != "per_flame"}))
        return
    t0 = time.perf_counter()
    train_g = dataset(db, args.train, TRAIN_SEED0, 512, 512)
    log("training genomes", len(train_g), f"{time.perf_counter() - t0:.1f}s")
    t1 = time.perf_counter()
    in_spp = [float(x) for x in args.input_spp.split(",")]
    sets = [dn.render_set(db, train_g, 512, 512, sp, seed=1 + 10 * i, both=True) for i, sp in enumerate(in_spp)]
    tgt = dn.render_set(db, train_g, 512, 512, HIGH_SPP, seed=2, tonemap=True)
    torch.cuda.synchronize()
    render_s = time.perf_counter() - t1
    log("rendered training pairs", f"{render_s:.1f}s")
    nval = max(1, len(train_g) // 20)
    net = dn.denoiser(seed=1)
    base = sets[0][1]
    val_plain = float(torch.mean((base[:nval, ..., :3] - tgt[:nval, ..., :3]) ** 2).item())
    log(f"validation MSE of the plain {in_spp[0]:g}-spp images", val_plain)
    rep = dn.train(net, [b[nval:] for b, _ in sets], [i[nval:] for _, i in sets], tgt[nval:], in_spp, args.steps,
                   batch=args.batch, val=([b[:nval] for b, _ in sets], [i[:nval] for _, i in sets], tgt[:nval]),
                   log=log)
    log("trained", rep)
    net.save(out / "denoiser_weights.npz")
    del sets, base, tgt
    torch.cuda.empty_cache()
    eval_g = dataset(db, args.eval, EVAL_SEED0, 1920, 1080)
    log("evaluation genomes", len(eval_g))
    ev = evaluate(db, net, eval_g, 1920, 1080)
    ev["training"] = {"flames": len(train_g), "validation_flames": nval, "steps": rep.steps, "batch": args.batch,
                      "input_spp": in_spp,
                      "seconds": rep.seconds, "ms_per_step": rep.ms_per_step, "first_loss": rep.first_loss,
                      "last_loss": rep.last_loss, "val_loss": rep.val_loss, "val_loss_plain_32spp": val_plain,
                      "render_seconds": render_s}
    (out / "denoiser_eval.json").write_text(json.dumps(ev, indent=1))
    summary = {k: v for k, v in ev.items() if k != "per_flame"}
    log(json.dumps(summary))


if __name__ == "__main__":
    main()
