"""Trains the learned denoiser on renders of this library and evaluates it
against the plain path (the learned-denoiser workload):

  training     `--train` seeded flames of the 1080p workload's distribution
               (8 xforms, Dirichlet(1) weights, final xform, 1-3 variations
               each from the 14-variation set), visibility-rejected and framed
               at 512 x 512; input: the 32-spp histogram and its tonemapped
               image, and in turn the 64- and 128-spp ones (--input-spp; the
               network's log-spp channel tells them apart), target: the tonemapped
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
# spp at which the denoised path runs the U-Net, in turn, before it falls back
# to the plain render. Chosen among the subsets of {48, 64, 96, 128} after 32
# by the mean time to 40 dB on 200 tuning flames (seeds 500000 on, disjoint
# from the training and evaluation seeds): (32, 64, 96, 128) 2.77x, (32, 64,
# 128) 2.72x, (32, 48, 96, 128) 2.70x against the plain path.
CASCADE_SPP = (32, 64, 96, 128)


def cascade_time(row: dict, stages=CASCADE_SPP) -> float:
    """Device time of one frame on the denoised path (cascade), from one
    evaluation row: warm-up + bin to stages[0] + tonemap + U-Net; while the
    frame is below 40 dB, continue the render to the next stage and tonemap -
    done if the plain image reached 40 dB by then (the render stops at the
    plain path's interpolated 40 dB spp, as the plain path's own time does) -
    else run the U-Net again; below 40 dB after the last stage, continue the
    plain render to its 40 dB spp and tonemap. Every stage is paid."""
    spp, t_bin, t_tm, s40, tb40 = row["spp"], row["t_bin"], row["t_tonemap"], row["spp_to_40db"], row["tb40"]

    def tb(sp):  # bin time to the checkpoint of sp spp
        return t_bin[FALLBACK_CHECKPOINTS.index(sp)]

    t = row["t_warmup"] + tb(stages[0]) + t_tm + row["t_unet_at"][str(stages[0])]
    if row["psnr_denoised_at"][str(stages[0])] >= 40.0:
        return t
    prev = stages[0]
    for sp in stages[1:]:
        if s40 <= sp:
            return t + max(tb40 - tb(prev), 0.0) + t_tm
        t += tb(sp) - tb(prev) + t_tm + row["t_unet_at"][str(sp)]
        if row["psnr_denoised_at"][str(sp)] >= 40.0:
            return t
        prev = sp
    return t + max(tb40 - tb(prev), 0.0) + t_tm


def evaluate_with_fallback(db, net, genomes, w: int, h: int, seed: int = 7, kernel=None,
                           stages=CASCADE_SPP) -> dict:
    """Seconds per frame to 40 dB PSNR, denoised path against plain path, with
    the plain path as the denoised path's fallback. Per flame (device time
    with CUDA events on the render stream; one render state re-warmed per
    frame, as a renderer drawing frame after frame keeps it):
      plain     warm-up + bin to the spp where the PSNR against an independent
                4096-spp render first reaches 40 dB (interpolated on log2 spp
                between checkpoints, the bin time likewise) + one tonemap;
      denoised  the cascade of cascade_time over `stages` (U-Net at 32, 64,
                96, 128 spp in turn, then the plain render);
      32 only   U-Net at 32 spp, then the plain render (keys *_32_only).
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
    first = fs[0].pack_samples(4, w, h)
    st = k.warmup(first, (w, h), seed=seed, count=20, stream=stream)
    st_ref = k.warmup(first, (w, h), seed=seed + 1, count=20, stream=stream)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return out, e0.elapsed_time(e1) / 1e3

    last = max(stages)
    rows = []
    for i, f in enumerate(fs):
        tp = f.tonemap_params()
        tmargs = (tp["gamma"], tp["brightness"], tp["vibrancy"])
        samples = f.pack_samples(4, w, h)
        st_ref.rewarm(samples, seed=seed + 2 * i + 1, count=20, stream=stream)
        k.bin(st_ref, lr.bailout_args(iters=0, millis=0, quality=HIGH_SPP), stream=stream)
        tm.run(st_ref.bins(), ref, (w, h), st_ref.quality, *tmargs, fmt=lr.FLOAT4, stream=stream)
        stream.synchronize()
        _, t_warm = timed(lambda: st.rewarm(samples, seed=seed + 2 * i, count=20, stream=stream))
        _, t_tm = timed(lambda: tm.run(st.bins(), img, (w, h), 1.0, *tmargs, fmt=lr.FLOAT4, stream=stream))
        spp, t_bin, psnrs, den_at, t_unet_at, den_vs_plain = [], [], [], {}, {}, None
        for c in FALLBACK_CHECKPOINTS:
            _, dt = timed(lambda: k.bin(st, lr.bailout_args(iters=0, millis=0, quality=c - st.quality), stream=stream))
            spp.append(st.quality)
            t_bin.append((t_bin[-1] if t_bin else 0.0) + dt)
            tm.run(st.bins(), img, (w, h), st.quality, *tmargs, fmt=lr.FLOAT4, stream=stream)
            stream.synchronize()
            psnrs.append(dn.psnr(img, ref))
            if c in stages:
                _, t_unet_at[str(c)] = timed(lambda: net.denoise(st.bins(), img, den, st.quality, stream=stream))
                den_at[str(c)] = dn.psnr(den, ref)
                if c == stages[0]:
                    # no-reference: how far the U-Net moved the plain image
                    den_vs_plain = dn.psnr(den, img)
            if psnrs[-1] >= 40.0 and c >= last:
                break
        row = {"psnr_denoised": den_at[str(stages[0])], "psnr_denoised_at": den_at, "t_unet_at": t_unet_at,
               "psnr_plain": psnrs, "spp": spp, "t_warmup": t_warm, "t_tonemap": t_tm,
               "t_unet": t_unet_at[str(stages[0])], "t_bin_first": t_bin[0], "t_bin": t_bin,
               "psnr_denoised_vs_plain_first": den_vs_plain}
        if max(psnrs) >= 40.0:
            # the first checkpoint at or above 40 dB
            j = next(i for i, v in enumerate(psnrs) if v >= 40.0)
            if j == 0:
                s40, tb40 = spp[0], t_bin[0]
            else:
                a, b = psnrs[j - 1], psnrs[j]
                fr = (40.0 - a) / (b - a) if b > a else 1.0
                s40 = float(2 ** (np.log2(spp[j - 1]) + fr * (np.log2(spp[j]) - np.log2(spp[j - 1]))))
                tb40 = t_bin[j - 1] + fr * (t_bin[j] - t_bin[j - 1])
            row.update(spp_to_40db=s40, tb40=tb40, plain_s=t_warm + tb40 + t_tm)
            row["denoised_s"] = cascade_time(row, stages[:1])
            row["cascade_s"] = cascade_time(row, stages)
        rows.append(row)
    del st, st_ref
    ok = [r for r in rows if "plain_s" in r]
    plain = np.array([r["plain_s"] for r in ok])
    dpath = np.array([r["denoised_s"] for r in ok])
    casc = np.array([r["cascade_s"] for r in ok])
    out = {
        "flames": len(rows), "width": w, "height": h, "plain_never_reaches": len(rows) - len(ok),
        "cascade_spp": list(stages),
        "s_per_frame_to_40db_plain": float(plain.mean()) if ok else None,
        "s_per_frame_to_40db_denoised": float(casc.mean()) if ok else None,
        "speedup": float(plain.mean() / casc.mean()) if ok else None,
        "speedup_per_flame_median": float(np.median(plain / casc)) if ok else None,
        "s_per_frame_to_40db_denoised_32_only": float(dpath.mean()) if ok else None,
        "speedup_32_only": float(plain.mean() / dpath.mean()) if ok else None,
        "plain_psnr_db_32spp_mean": float(np.mean([r["psnr_plain"][0] for r in rows])),
        "plain_spp_to_40db_median": float(np.median([r["spp_to_40db"] for r in ok])) if ok else None,
        "unet_ms_median": 1e3 * float(np.median([r["t_unet"] for r in rows])),
        "warmup_ms_median": 1e3 * float(np.median([r["t_warmup"] for r in rows])),
        "render_first_stage_ms_median": 1e3 * float(np.median([r["t_bin_first"] + r["t_warmup"] + r["t_tonemap"]
                                                               for r in rows])),
        "per_flame": rows,
    }
    for sp in stages:
        pd = np.array([r["psnr_denoised_at"][str(sp)] for r in rows])
        out[f"denoised_{sp}spp_reaches_40db"] = float((pd >= 40.0).mean())
        out[f"denoised_{sp}spp_psnr_db_mean"] = float(pd.mean())
    # frames done by the end of each stage (denoised or plain image at 40 dB)
    for n in range(1, len(stages) + 1):
        out[f"cascade_done_by_{stages[n - 1]}spp"] = float(np.mean([
            any(r["psnr_denoised_at"][str(sp)] >= 40.0 for sp in stages[:n]) or r.get("spp_to_40db", 1e9) <= stages[n - 1]
            for r in rows]))
    out["denoised_reaches_40db"] = out[f"denoised_{stages[0]}spp_reaches_40db"]
    out["denoised_psnr_db_mean"] = out[f"denoised_{stages[0]}spp_psnr_db_mean"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2000)
    ap.add_argument("--eval", type=int, default=200)
    ap.add_argument("--steps", type=int, default=1500)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--input-spp", default="32,64,128",
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
