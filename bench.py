"""Benchmark of the flame-rendering hot path.

Workload: the plain 1080p single flame - 1920x1080, 1024 spp, 8 xforms with
Dirichlet(1) weights plus a final xform, 1-3 variations each from the
14-variation set, density-estimation blur (radius 0-9 px ~ 1/sqrt(density)),
tonemap. The genome is the committed seeded synthetic workload
refraktor_gb300/workloads/hd_1080p.json (the reference publishes no benchmark
genomes); the launch shape and histogram-flush strategy come from the
library's autotuner.

One step = one frame: bin to 1024 spp on a warmed state (value), or the full
public-API path from host genome samples to a host image (e2e).
  value  iterations/s (chain steps per second), device-timed with CUDA events
         around the bin calls on their stream, histogram already resident
  e2e    the same metric through rfk_warmup + rfk_bin + rfk_density_blur +
         rfk_tonemap with host samples in and the host image out
Between timed steps a 512 MiB buffer is written to flush L2 (129 MB).

--impl reference times the reference path on the CPU: the reference has no
CPU implementation, so this is the FP64 oracle port (oracle/), on all host
cores, over a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

W, H, SPP = 1920, 1080, 1024.0
WARMUP_PASSES = 20
METRIC = "iterations/s"
DATA = "synthetic (seeded genome refraktor_gb300/workloads/hd_1080p.json)"
WORKLOAD = "plain 1080p single flame: 1920x1080, 1024 spp, 8 xforms + final xform, 14-variation set, DE blur, tonemap"


# dram__bytes_read.sum + dram__bytes_write.sum of one 1024-spp rfk_bin launch of
# this workload at the bench's launch shape (608 x 256, 8 chains per thread,
# flush 4 with fixed-point hot-pixel sums, block sort, 4 blocks per SM; one ncu
# pass over the --ncu-case launch at 1024 spp)
BIN_DRAM_BYTES_PER_LAUNCH = 46690816 + 1081344
# smsp__inst_executed.sum / chain steps of the same 1024-spp launch: 21.736 G
# warp instructions for 2.168 G chain steps; each SM sub-partition issues one
# warp instruction per clock
BIN_WARP_INST_PER_ITER = 21736283626 / 2168258560
# dram__bytes_read.sum + dram__bytes_write.sum of one rfk_bin_batch launch of
# each batched workload (ncu, one pass over the bench's first launch at the
# chosen queue-item length, flush 4 at 608 x 256, 8 chains per thread)
BATCH_DRAM_BYTES_PER_RUN: dict = {"anim": 1005712640 + 1424995072, "hetero": 769470464 + 1991087360}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def _free_port() -> int:
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_ranks(n: int, argv: list[str]) -> int:
    """`bench.py --gpus N` started outside torchrun: runs this script again
    under torch.distributed.run with N ranks on this node (one process per
    GPU, rendezvous on 127.0.0.1) and returns its exit code. Under torchrun
    (WORLD_SIZE set) the ranks already exist and nothing is launched."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), str(Path(__file__).resolve()), *argv]
    return subprocess.call(cmd)


def _init_dist(ws: int, backend: str = "nccl") -> None:
    """One process per GPU under torchrun: the process group for the barrier
    and the rank totals (no data-path collective: ranks are replicas)."""
    if ws > 1:
        import torch.distributed as dist

        if not dist.is_initialized():
            dist.init_process_group(backend)


def _barrier(ws: int) -> None:
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def merge_ranks(seconds: float, counts: list, device: str = "cuda") -> tuple:
    """Whole-job totals of a replicas-only run: the slowest rank's time (all
    ranks start together after a barrier, so the job ends with it) and the
    sum of every rank's counts. One process per GPU; a no-op for one rank."""
    import torch

    if not torch.distributed.is_available() or not torch.distributed.is_initialized():
        return seconds, list(counts)
    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    c = torch.tensor([float(x) for x in counts], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(c)
    return float(t.item()), [int(x) for x in c.tolist()]


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    def __init__(self, gpu: int = 0):
        self.gpu = gpu
        self.rows: list[list[str]] = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                           "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except FileNotFoundError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *exc):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self) -> dict:
        rows = [r for r in self.rows if len(r) >= 7]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[3:7]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": float(rows[0][1]) if rows else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def _flush_l2(buf):
    buf.fill_(1.0)


def load_workload(name: str = "hd_1080p.json") -> dict:
    return json.loads((ROOT / "refraktor_gb300" / "workloads" / name).read_text())


def run_gpu(args) -> dict:
    import torch

    from refraktor_gb300 import build
    from refraktor_gb300 import librefrakt as lr
    from refraktor_gb300 import synthetic as syn

    ws, rank = _dist()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    _init_dist(ws)
    build.build()
    db = lr.flamedb()
    genome = load_workload()
    f = lr.flame.from_json(db, genome)
    tp = f.tonemap_params()
    comp = lr.flame_compiler()
    samples = f.pack_samples(4, W, H)
    tuned, tune_report = lr.autotune(db, f, samples, (W, H))
    k = comp.get_flame_kernel(db, f, **tuned)
    stream = torch.cuda.Stream()
    flush = torch.empty(512 << 20 >> 2, dtype=torch.float32, device="cuda")

    # ---- value: bin to 1024 spp on a warmed state, device-timed ------------
    st = k.warmup(samples, (W, H), seed=rank + 1, count=WARMUP_PASSES, stream=stream)
    bo = lr.bailout_args(iters=0, millis=0, quality=SPP)
    for _ in range(args.warmup):
        k.bin(st, bo, stream=stream)
    times, passes, draws, elapsed_kernel = [], 0, 0, 0.0
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        for _ in range(args.steps):
            _flush_l2(flush)
            torch.cuda.synchronize()
            if ws > 1:
                torch.distributed.barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            k.bin_async(st, bo, stream=stream)
            e1.record(stream)
            r = st.wait()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            passes += r.total_passes
            draws += r.draw_count
            elapsed_kernel += r.elapsed_ms / 1e3
    t_total = sum(times)
    t_total, (passes, draws) = merge_ranks(t_total, [passes, draws])
    value = passes / t_total
    bin_launch_s = t_total / args.steps

    # roofline: draws are red.global.add.v4.f32 (16 B payload) into the L2-resident histogram
    peak_ops = lr.probe_red_v4(W * H * 16, 512)
    achieved_ops = draws / max(elapsed_kernel, 1e-9) if ws == 1 else draws / t_total
    info = k.info
    # the chain step's arithmetic pipes: measured SFU and FP32 FMA issue rates
    # against the translator's per-step counts (weighted by xform weights)
    per_rank = value / ws
    pipes = {}
    for name, pipe, iters, per_iter in (("sfu", 1, 4096, info["sfu_per_iter"]), ("fma", 0, 16384, info["fma_per_iter"])):
        peak = lr.probe_pipe(pipe, iters)
        pipes[name] = {"per_iter": per_iter, "achieved_ops": per_rank * per_iter, "peak_ops": peak,
                       "frac": per_rank * per_iter / peak}
    pipes["issue"] = {"per_iter": BIN_WARP_INST_PER_ITER}
    pipes["note"] = ("sfu: transcendental calls of the generated variation code per chain step (a call such as "
                     "atan2 issues several instructions) vs sin.approx/rsqrt.approx lane ops/s; fma: affine FMAs "
                     "per chain step (4 per vlink + projection) vs FP32 FMA lane ops/s; both peaks measured live; "
                     "issue: warp instructions per chain step (ncu) vs one per sub-partition per clock")

    # issue slots: warp instructions per chain step (ncu) x iterations/s vs
    # 4 sub-partitions x SMs x the median SM clock sampled during the timed steps
    csum = clocks.summary()
    mhz = csum.get("sm_mhz") or csum.get("sm_max_mhz") or 2070.0
    iss = pipes["issue"]
    iss["achieved_ops"] = per_rank * BIN_WARP_INST_PER_ITER
    iss["peak_ops"] = 4.0 * lr.sm_count() * mhz * 1e6
    iss["frac"] = iss["achieved_ops"] / iss["peak_ops"]

    # ---- e2e: public API, host samples in, host image out ------------------
    # The render state and the image buffers are kept, as a renderer drawing
    # frame after frame at one size keeps them; every frame runs
    # rfk_state_rewarm (the host samples uploaded, prepared, chains warmed up
    # again, histogram cleared), bin, blur, tonemap and the image read-back.
    # The state is the one the device-timed steps used: the bin's speed
    # depends by a few % on where its histogram was allocated (which L2
    # slices the hot pixels' lines fall on), so both figures measure one
    # allocation.
    out_host = torch.empty((H, W, 4), dtype=torch.float16, pin_memory=True)
    blurred = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    img = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    tmap = lr.tonemapper()
    e2e_times = []
    e2e_passes = 0
    e2e_bin_s = 0.0
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as e2e_clocks:
        for i in range(args.warmup + args.steps):
            _flush_l2(flush)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st.rewarm(samples, seed=100 + i, count=WARMUP_PASSES, stream=stream)
            r = k.bin(st, bo, stream=stream)
            with torch.cuda.stream(stream):
                lr.density_blur(st.bins(), blurred, (W, H), 9.0, 0.0, 0.5, stream=stream)
                tmap.run(blurred, img, (W, H), st.quality, tp["gamma"], tp["brightness"], tp["vibrancy"],
                         fmt=lr.HALF4, stream=stream)
                out_host.copy_(img, non_blocking=True)
            stream.synchronize()
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                e2e_times.append(dt)
                e2e_passes += r.total_passes  # bin iterations only; the warm-up passes count as time
                e2e_bin_s += r.elapsed_ms / 1e3
    e2e_t = sum(e2e_times)
    e2e_t, (e2e_passes,) = merge_ranks(e2e_t, [e2e_passes])

    line = {
        "metric": METRIC,
        "value": value,
        "unit": "iterations/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_total / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": DATA,
        "config": {"workload": WORKLOAD, "genome": genome.get("name"), "width": W, "height": H, "spp": SPP, "xforms": 8,
                   "final_xform": True, "grid": info["grid"], "block": info["block"],
                   "chains_per_thread": info["chains_per_thread"], "flush": info["flush"], "sort": info["sort"],
                   "autotune": tune_report, "l2": "512 MiB buffer written between timed steps",
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": e2e_passes / e2e_t, "unit": "iterations/s", "s_per_frame": e2e_t / args.steps,
                "h2d_bytes_per_step": int(samples.nbytes), "d2h_bytes_per_step": int(W * H * 4 * 2),
                "bin_kernel_ms_per_frame": 1e3 * e2e_bin_s / args.steps, "clocks": e2e_clocks.summary()},
        "roofline": {"bound": "l2_atomic", "achieved": achieved_ops * 16 / 1e9, "peak": peak_ops * 16 / 1e9,
                     "unit": "GB/s", "frac": achieved_ops / peak_ops, "traffic": BIN_DRAM_BYTES_PER_LAUNCH,
                     "achieved_ops": achieved_ops, "peak_ops": peak_ops,
                     "note": "red.global.add.v4.f32 payload (16 B per draw); peak = measured random red.v4 rate into a "
                             "buffer of the histogram's size; traffic = DRAM bytes of one 1024-spp rfk_bin "
                             "launch from an ncu capture (the histogram stays in L2)",
                     "pipes": pipes},
        "gpu_launches": args.steps * 3,
        "clocks": csum,
        "draws_per_s": draws / t_total,
        "bin_ms": 1e3 * bin_launch_s,
        "bin_kernel_ms": 1e3 * elapsed_kernel / args.steps,
        "registers": info["registers"],
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(genome, seconds=args.cpu_seconds)
    if rank == 0 and args.denoise_flames > 0:
        line["denoise"] = denoise_leg(db, args.denoise_flames)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return line if rank == 0 else {}


def denoise_leg(db, flames: int) -> dict:
    """The second half of the metric: s/frame to 40 dB PSNR at 1920x1080,
    denoised path (render + U-Net) against the plain path, on `flames`
    held-out seeded flames of the 1080p workload's distribution: the denoised
    path is a cascade (U-Net at 32, 64, 96, 128 spp in turn, then the plain render
    as the fallback of every frame still below 40 dB), with the single-attempt
    figures beside it (refraktor_gb300/workloads/train_denoiser.py:
    evaluate_with_fallback). Device time per frame; rank 0 only."""
    from refraktor_gb300 import denoise as dn
    from refraktor_gb300.workloads import train_denoiser as td

    t0 = time.perf_counter()
    net = dn.denoiser.load(ROOT / "refraktor_gb300" / "workloads" / "denoiser_weights.npz")
    gs = td.dataset(db, flames, td.EVAL_SEED0, 1920, 1080)
    ev = td.evaluate_with_fallback(db, net, gs, 1920, 1080)
    ev.pop("per_flame")
    ev["metric"] = "s/frame to 40 dB PSNR at 1080p (denoised low-spp vs plain, plain fallback)"
    ev["unit"] = "s/frame"
    ev["input_spp"] = td.LOW_SPP
    ev["reference_spp"] = td.HIGH_SPP
    ev["wall_s"] = time.perf_counter() - t0
    return ev


def cpu_baseline(genome: dict, seconds: float = 12.0, threads: int | None = None) -> dict:
    """The FP64 oracle chaos game on the host cores, bounded sample of the workload."""
    from oracle import oracle as orc

    threads = threads or os.cpu_count() or 1
    chains = 64 * threads
    params, pal = orc.prepared(genome, W, H)
    # calibrate passes for about `seconds` of work: grow a probe to >= 0.5 s
    probe = 200
    while True:
        t0 = time.perf_counter()
        orc.render(genome, W, H, chains, probe, warmup=WARMUP_PASSES, threads=threads, params=params, palette=pal)
        dt = time.perf_counter() - t0
        if dt >= 0.5 or probe > 1 << 26:
            break
        probe *= 4
    passes = max(probe, int(probe * seconds / dt))
    t0 = time.perf_counter()
    _, draws = orc.render(genome, W, H, chains, passes, warmup=WARMUP_PASSES, threads=threads, params=params,
                          palette=pal)
    dt = time.perf_counter() - t0
    iters = chains * (passes + WARMUP_PASSES)
    return {"value": iters / dt, "unit": "iterations/s", "cores": threads, "kind": "port",
            "sample": f"{chains} chains x {passes + WARMUP_PASSES} passes of the same 1920x1080 flame "
                      f"({iters / 1e9:.2f} G iterations, {draws / 1e9:.2f} G draws, {dt:.1f} s)",
            "draws_per_s": draws / dt, "seconds": dt, "iterations": iters}


ANIM_WORKLOAD = ("batched animation: 120 frames 1280x720, 256 spp, Catmull-Rom over 4 keyframes (6 xforms, "
                 "shared variation sets), one persistent launch, DE blur + tonemap, one CUDA graph")
HETERO_WORKLOAD = ("heterogeneous batch: 64 flames, sizes 256^2..2048x1152, 2-12 xforms, 64/256/1024 spp, "
                   "union-of-variations kernel, one persistent launch, DE blur + tonemap, one CUDA graph")


def batch_workload(lr, db, name: str):
    """(kernel genome, packed samples, units, workload text, tune genome + size)."""
    units, samples = [], []
    if name == "anim":
        wl = load_workload("anim_720p.json")
        w, h, n, spp = wl["width"], wl["height"], wl["frames"], float(wl["spp"])
        keys = lr.align_flames(db, [lr.flame.from_json(db, g) for g in wl["keyframes"]])
        ks = [f.pack_sample(w, h) for f in keys]
        samples = np.stack([ks[0], ks[0], ks[1], ks[2], ks[3], ks[3]])
        tp = keys[0].tonemap_params()
        for i in range(n):
            x = 3.0 * i / (n - 1)
            seg = min(int(x), 2)
            units.append(lr.batch_unit(w, h, spp, segment=seg, t=float(x - seg), gamma=tp["gamma"],
                                       brightness=tp["brightness"], vibrancy=tp["vibrancy"]))
        return keys[0], samples, units, ANIM_WORKLOAD, (keys[0], np.stack([ks[0]] * 4), (w, h))
    wl = load_workload("hetero_64.json")
    fl = wl["flames"]
    al = lr.align_flames(db, [lr.flame.from_json(db, e["genome"]) for e in fl])
    for i, (f, e) in enumerate(zip(al, fl)):
        tp = f.tonemap_params()
        units.append(lr.batch_unit(e["width"], e["height"], float(e["spp"]), segment=4 * i, t=0.0, gamma=tp["gamma"],
                                   brightness=tp["brightness"], vibrancy=tp["vibrancy"]))
        samples.append(f.pack_samples(4, e["width"], e["height"]).reshape(4, -1))
    big = max(range(len(fl)), key=lambda i: fl[i]["width"] * fl[i]["height"] * fl[i]["spp"])
    tune = (al[big], samples[big], (fl[big]["width"], fl[big]["height"]))
    return al[0], np.concatenate(samples), units, HETERO_WORKLOAD, tune


def batch_working_set(units, grid: int, chains_per_block: int, passes_per_item: int) -> int:
    """Histogram bytes the persistent batch launch keeps under atomic traffic
    at once, averaged over its draws: the queue hands items out unit after
    unit, so while unit u is drawn the `grid` resident blocks work on about
    grid / N_u + 1 units, N_u = the items u needs at one draw per chain step
    (quality * pixels / (chains per block * passes per item)); each of those
    holds a histogram of about u's size (16 B per pixel)."""
    per_item = float(chains_per_block * passes_per_item)
    num = den = 0.0
    for U in units:
        px = U.width * U.height
        draws = U.quality * px
        n_u = max(draws / per_item, 1.0)
        active = min(float(len(units)), grid / n_u + 1.0)
        num += draws * active * px * 16
        den += draws
    return int(max(num / max(den, 1.0), 4 << 20))


def run_batch(args) -> dict:
    """Batched workloads (animation frames / heterogeneous flames): one batch
    run = prepare + one persistent iterate launch + blur + tonemap per unit,
    replayed as a CUDA graph; `value` times the graph on the device, `e2e`
    adds the host sample copy and the read-back of every tonemapped image."""
    import torch

    from refraktor_gb300 import build
    from refraktor_gb300 import librefrakt as lr

    ws, rank = _dist()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    _init_dist(ws)
    build.build()
    db = lr.flamedb()
    kf, samples, units, text, (tf, tsamples, tdims) = batch_workload(lr, db, args.workload)
    tuned, tune_report = lr.autotune(db, tf, tsamples, tdims)
    k = lr.flame_compiler().get_flame_kernel(db, kf, **tuned)
    stream = torch.cuda.Stream()
    flush = torch.empty(512 << 20 >> 2, dtype=torch.float32, device="cuda")
    nsamples = samples.shape[0]
    de = (9.0, 0.0, 0.5)

    # schedule: queue-item length, one timed graph run each
    sched = {}
    for ppi in (128, 256, 512):
        b = lr.batch(k, units, nsamples, passes_per_item=ppi, warmup=WARMUP_PASSES, de=de, out_format=lr.HALF4)
        b.set_samples(samples)
        b.run(use_graph=True, stream=stream)
        b.wait()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(use_graph=True, stream=stream)
        e1.record(stream)
        tot, _ = b.wait()
        sched[ppi] = tot.total_passes / (e0.elapsed_time(e1) / 1e3)
        del b
    ppi = max(sched, key=sched.get)
    b = lr.batch(k, units, nsamples, passes_per_item=ppi, warmup=WARMUP_PASSES, de=de, out_format=lr.HALF4)
    b.set_samples(samples)
    info = b.info()

    for _ in range(args.warmup):
        b.run(use_graph=True, stream=stream)
        b.wait()
    times, passes, draws, kern_ms, reached = [], 0, 0, 0.0, True
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        for _ in range(args.steps):
            _flush_l2(flush)
            torch.cuda.synchronize()
            _barrier(ws)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            b.run(use_graph=True, stream=stream)
            e1.record(stream)
            tot, per = b.wait()
            times.append(e0.elapsed_time(e1) / 1e3)
            passes += tot.total_passes
            draws += tot.draw_count
            kern_ms += tot.elapsed_ms
            reached = reached and bool(tot.status & 1)
    t_total, (passes, draws) = merge_ranks(sum(times), [passes, draws])
    info = b.info()

    # e2e: host samples in, every tonemapped image out (pinned)
    img_host = torch.empty(info["image_bytes"], dtype=torch.uint8, pin_memory=True)
    img_dev = lr._device_view(lr.lib().rfk_batch_image(b._h, 0), (info["image_bytes"],), "|u1")
    e2e_times, e2e_passes = [], 0
    for i in range(args.warmup + args.steps):
        _flush_l2(flush)
        torch.cuda.synchronize()
        _barrier(ws)
        t0 = time.perf_counter()
        b.set_samples(samples)
        b.run(use_graph=True, stream=stream)
        with torch.cuda.stream(stream):
            img_host.copy_(img_dev, non_blocking=True)
        tot, _ = b.wait()
        stream.synchronize()
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
            e2e_passes += tot.total_passes
    e2e_t, (e2e_passes,) = merge_ranks(sum(e2e_times), [e2e_passes])
    ws_bytes = batch_working_set(units, k.info["grid"], k.info["block"] * k.info["chains_per_thread"], ppi)
    peak_ops = lr.probe_red_v4(ws_bytes, 512)
    achieved_ops = draws / max(kern_ms / 1e3, 1e-9)
    if rank != 0:
        return {}
    return {
        "metric": METRIC, "value": passes / t_total, "unit": "iterations/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded genomes refraktor_gb300/workloads/)",
        "config": {"workload": text, "units": len(units), "pixels": int(sum(u.width * u.height for u in units)),
                   "grid": k.info["grid"], "block": k.info["block"], "chains_per_thread": k.info["chains_per_thread"],
                   "flush": k.info["flush"], "sort": k.info["sort"], "autotune": tune_report,
                   "passes_per_item": ppi, "schedule_iters_per_s": sched, "queue_items": info["items"],
                   "l2": "512 MiB buffer written between timed steps", "all_units_reached_target": reached},
        "e2e": {"value": e2e_passes / e2e_t, "unit": "iterations/s", "s_per_run": e2e_t / args.steps,
                "s_per_unit": e2e_t / args.steps / len(units), "h2d_bytes_per_step": int(samples.nbytes),
                "d2h_bytes_per_step": int(info["image_bytes"])},
        "roofline": {"bound": "l2_atomic", "achieved": achieved_ops * 16 / 1e9, "peak": peak_ops * 16 / 1e9, "unit": "GB/s",
                     "frac": achieved_ops / peak_ops, "traffic": BATCH_DRAM_BYTES_PER_RUN.get(args.workload),
                     "achieved_ops": achieved_ops, "peak_ops": peak_ops, "peak_buffer_bytes": ws_bytes,
                     "note": "red.global.add.v4.f32 payload (16 B per draw); peak = measured random red.v4 rate "
                             "into a buffer of the launch's histogram working set (peak_buffer_bytes: the units "
                             "drawn at once, weighted by draws); traffic = DRAM bytes of one rfk_bin_batch launch "
                             "(ncu)"},
        "gpu_launches": info["launches_per_run"] * args.steps,
        "clocks": clocks.summary(),
        "draws_per_s": draws / t_total,
    }


DENOISE_WORKLOAD = ("learned denoiser at 1920x1080: 32-spp render + U-Net (trained weights "
                    "refraktor_gb300/workloads/denoiser_weights.npz), then below 40 dB 64-, 96- and 128-spp "
                    "renders + U-Net, then the plain render as the fallback, vs the plain path's time to 40 dB PSNR "
                    "against an independent 4096-spp render, seeded held-out flames")


def run_denoise(args) -> dict:
    """s/frame to 40 dB PSNR at 1080p on `--flames` held-out flames: the plain
    path renders progressively until its PSNR against an independent 4096-spp
    render crosses 40 dB (spp and time interpolated on log2 spp); the denoised
    path renders 32 spp and runs the U-Net, a frame left below 40 dB continues
    to 64, 96, then 128 spp and runs the U-Net again at each (unless its plain
    image reached 40 dB), and a frame still below 40 dB continues the plain
    render to the plain path's 40 dB spp; every stage is paid. `value` is the denoised path's mean
    device time per frame with that cascade; the plain path's is beside it,
    and the single-attempt figures (U-Net at 32 spp, then the plain render)
    are the *_32_only keys."""
    import torch

    from refraktor_gb300 import build
    from refraktor_gb300 import denoise as dn
    from refraktor_gb300 import librefrakt as lr
    from refraktor_gb300.workloads import train_denoiser as td

    ws, rank = _dist()
    if rank != 0:
        # a fixed evaluation set, not sharded: the other ranks have no work
        return {}
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    build.build()
    db = lr.flamedb()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        ev = denoise_leg(db, args.flames)
    net = dn.denoiser.load(ROOT / "refraktor_gb300" / "workloads" / "denoiser_weights.npz")
    gs = td.dataset(db, min(args.flames, 8), td.EVAL_SEED0, 1920, 1080)
    e2e_s, h2d, d2h = _denoise_e2e(db, net, gs, td, args)
    den_s = ev["s_per_frame_to_40db_denoised"]
    return {
        "metric": ev["metric"], "value": den_s, "unit": "s/frame",
        "n_gpus": 1, "steps": ev["flames"], "warmup": 0, "ms_per_step": 1e3 * den_s, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic (seeded held-out flames)",
        "config": {"workload": DENOISE_WORKLOAD, "flames": ev["flames"]},
        **{k: v for k, v in ev.items() if k not in ("metric", "unit")},
        "e2e": {"value": e2e_s, "unit": "s/frame", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "host genome samples -> warm-up + bin to 32 spp -> tonemap -> U-Net -> half4 image on the "
                        "host, wall clock per frame (no fallback)"},
        "clocks": clocks.summary(),
    }


def _denoise_e2e(db, net, gs, td, args, w: int = 1920, h: int = 1080) -> tuple[float, int, int]:
    """The denoised path through the public API, frame by frame: packed host
    samples in (H2D inside the timed region), warm-up + bin to the low spp,
    tonemap, U-Net, the half4 image read back into pinned host memory. The
    median wall-clock time per frame over the first flames (one untimed frame
    first)."""
    import torch

    from refraktor_gb300 import librefrakt as lr

    fs = [lr.flame.from_json(db, g) for g in gs]
    opts, _ = lr.autotune(db, fs[0], fs[0].pack_samples(4, w, h), (w, h))
    k = lr.flame_compiler().get_flame_kernel(db, fs[0], **opts)
    tm = lr.tonemapper()
    base = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    out = torch.empty((h, w, 4), dtype=torch.float16, device="cuda")
    host = torch.empty((h, w, 4), dtype=torch.float16, pin_memory=True)
    times, h2d = [], 0
    n = min(len(fs), max(args.steps, 3))
    # the flames share one structure: one render state, warmed up again per frame
    st = k.warmup(fs[0].pack_samples(4, w, h), (w, h), seed=999, count=20)
    for i in range(n + 1):
        f = fs[i % len(fs)]
        tp = f.tonemap_params()
        samples = f.pack_samples(4, w, h)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st.rewarm(samples, seed=1000 + i, count=20)
        k.bin(st, lr.bailout_args(iters=0, millis=0, quality=td.LOW_SPP))
        tm.run(st.bins(), base, (w, h), st.quality, tp["gamma"], tp["brightness"], tp["vibrancy"], fmt=lr.FLOAT4)
        net.denoise(st.bins(), base, out, st.quality, fmt=lr.HALF4)
        host.copy_(out, non_blocking=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if i > 0:
            times.append(dt)
            h2d = int(np.asarray(samples).nbytes)
    return float(np.median(times)), h2d, int(out.numel() * out.element_size())


def reference_cuda(spp: float = SPP) -> dict:
    """The reference's own chaos-game kernel on this GPU: assets/kernels/refactor.cu
    specialised for the bench genome (oracle/ref_flame.py, oracle/build_ref.py)
    and run as flame_kernel::warmup + bin drive it (oracle/ref_run.py), at the
    bench's size and spp; chain steps per second of its bin launch (CUDA
    events), and the fraction of its draws its histogram kept, as written
    (non-atomic update) and with that update made atomic."""
    try:
        import torch
    except ImportError:
        return {"unavailable": "no torch"}
    if not torch.cuda.is_available():
        return {"unavailable": "no GPU"}
    from oracle import ref_run, refkernels

    if not (refkernels.available("refactor_bench") and refkernels.available("catmull")):
        return {"unavailable": "the reference's kernels were not built (oracle/build_ref.py needs the reference sources)"}
    out = {"workload": WORKLOAD, "spp": spp}
    for key, mod in (("as_written", "refactor_bench"), ("atomic_update", "refactor_bench_atomic")):
        ref_run.reference_render(mod, 1, 16.0)  # load the module, warm up
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        _, info = ref_run.reference_render(mod, 2, spp, timing=(e0, e1))
        ms = e0.elapsed_time(e1)
        out[key] = {"iterations_per_s": info["passes"] / (ms * 1e-3), "bin_ms": ms, "kept": 1.0 - info["lost"],
                    "quality": info["quality"]}
    return out


def run_reference(args) -> dict:
    """CPU reference leg: the FP64 oracle port on all host cores; beside it,
    the reference's own CUDA kernel timed on this GPU (`reference_cuda`)."""
    ws, rank = _dist()
    if rank != 0:
        return {}
    genome = load_workload()
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(genome, seconds=2.0)
    for _ in range(args.steps):
        vals.append(cpu_baseline(genome, seconds=args.cpu_seconds / max(args.steps, 1)))
    total_s = sum(x["seconds"] for x in vals)
    v = sum(x["iterations"] for x in vals) / total_s
    return {
        "metric": METRIC, "value": v, "unit": "iterations/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_s / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": DATA,
        "config": {"workload": WORKLOAD, "genome": genome.get("name"), "width": W, "height": H, "spp": SPP,
                   "xforms": 8, "final_xform": True, "parallelism": f"rank 0 of {ws}"},
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": "iterations/s", "cores": vals[0]["cores"], "kind": "port",
                         "sample": vals[0]["sample"]},
        "e2e": {"value": v, "unit": "iterations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_cuda": reference_cuda() if args.reference_cuda else {"unavailable": "not requested"},
    }


def run_ncu_case(args) -> None:
    """Small case for ncu captures of rfk_bin: the 1080p workload genome,
    warm-up, then `--ncu-launches` bin launches to `--ncu-spp` spp each
    (16 spp: ~0.5 ms; 1024 spp is the bench step), with
    the autotuned options unless --flush/--cpt/--block/--sort/--minb are given."""
    from refraktor_gb300 import build
    from refraktor_gb300 import librefrakt as lr

    build.build()
    db = lr.flamedb()
    f = lr.flame.from_json(db, load_workload())
    samples = f.pack_samples(4, W, H)
    if args.flush is None:
        opts, _ = lr.autotune(db, f, samples, (W, H))
    else:
        opts = dict(flush=args.flush, chains_per_thread=args.cpt, block=args.block, sort=args.sort,
                    blocks_per_sm=args.minb)
    k = lr.flame_compiler().get_flame_kernel(db, f, **opts)
    st = k.warmup(samples, (W, H), 1, WARMUP_PASSES)
    for _ in range(args.ncu_launches):
        r = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=float(args.ncu_spp)))
    print(json.dumps({"ncu_case": k.info, "opts": opts, "passes": r.total_passes, "ms": r.elapsed_ms}))


def run_ncu_batch(args) -> None:
    """Small case for ncu captures of rfk_bin_batch: the first 8 flames of the
    heterogeneous workload (one union-of-variations kernel, the autotuner's
    launch shape for the workload) at 32 spp each, one batch run (a few tens
    of MB on the device)."""
    import dataclasses

    from refraktor_gb300 import build
    from refraktor_gb300 import librefrakt as lr

    build.build()
    db = lr.flamedb()
    kf, samples, units, _, (tf, tsamples, tdims) = batch_workload(lr, db, "hetero")
    opts, _ = lr.autotune(db, tf, tsamples, tdims)
    k = lr.flame_compiler().get_flame_kernel(db, kf, **opts)
    ss = kf.sample_size()
    units = [dataclasses.replace(u, quality=32.0) for u in units[:8]]
    smp = np.asarray(samples, dtype=np.float64).reshape(-1, ss)[:4 * len(units)]
    b = lr.batch(k, units, smp.shape[0], passes_per_item=128, warmup=WARMUP_PASSES, out_format=-1)
    b.set_samples(smp)
    b.run()
    tot, _ = b.wait()
    print(json.dumps({"ncu_batch": k.info, "opts": opts, "units": [(u.width, u.height) for u in units],
                      "passes": tot.total_passes, "ms": tot.elapsed_ms}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ncu-case", action="store_true")
    ap.add_argument("--ncu-batch", action="store_true",
                    help="small case for profiler captures of rfk_bin_batch (8 heterogeneous flames, 32 spp)")
    ap.add_argument("--ncu-launches", type=int, default=2)
    ap.add_argument("--ncu-spp", type=int, default=16)
    ap.add_argument("--flush", type=int, default=None)
    ap.add_argument("--cpt", type=int, default=4)
    ap.add_argument("--block", type=int, default=256)
    ap.add_argument("--sort", type=int, default=2)
    ap.add_argument("--minb", type=int, default=0, help="blocks_per_sm of the --ncu-case kernel (0 = library default)")
    ap.add_argument("--gpus", type=int, default=1,
                    help="GPUs (ranks) of this node; outside torchrun, N > 1 relaunches under torch.distributed.run")
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-cuda", type=int, default=1,
                    help="--impl reference: also time the reference's own CUDA kernel on the GPU (1) or not (0)")
    ap.add_argument("--workload", default="hd", choices=["hd", "anim", "hetero", "denoise"],
                    help="hd: the 1080p single-flame bench (default); anim / hetero: the batched workloads; "
                         "denoise: the learned denoiser's s/frame to 40 dB")
    ap.add_argument("--flames", type=int, default=200, help="evaluation flames of --workload denoise")
    ap.add_argument("--denoise-flames", type=int, default=200,
                    help="held-out 1080p flames of the denoise key of the default run (0 = leave it out)")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args.gpus, sys.argv[1:]))
    ws, _ = _dist()
    if ws != args.gpus and "WORLD_SIZE" in os.environ:
        print(f"bench.py: --gpus {args.gpus} under a launcher with WORLD_SIZE {ws}; the ranks present run",
              file=sys.stderr)
    if args.ncu_case:
        run_ncu_case(args)
        return
    if args.ncu_batch:
        run_ncu_batch(args)
        return
    if args.impl == "reference":
        line = run_reference(args)
    elif args.workload == "denoise":
        line = run_denoise(args)
    elif args.workload != "hd":
        line = run_batch(args)
    else:
        line = run_gpu(args)
    if line:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
