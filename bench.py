#!/usr/bin/env python3
"""Benchmark of the GB300 Lienard-Wiechert field integration.

Metric: particle x step x pixel evaluations per second of the FP32-split
kernel (every step of every particle against every pixel counts, in window
or not), on the 1e5-particle coherent-emission screen: 200 x 200 pixels over
0.4 x 0.4 m at z = 20 m, 4096 x 2 fs traces, gamma = 300 bunch in a
lambda_u = 0.3 m, 20-period, K = 3 undulator at 100 steps per period.
One step integrates one batch of particles of that bunch onto the whole
screen; every step uses a different batch.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  Under torchrun each rank integrates its own
batches of the bunch onto the whole screen (weak scaling, no exchange).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle·step·pixel evals/s: FP32 split vs FP64 GPU at ≤1e-5 rel L2 vs FP64"
UNIT = "evals/s"
# algorithmic flops per in-window (pixel, particle, step) and per extra bin
# of a multi-bin step (one LW field evaluation 89 + single-bin deposit 21)
FLOPS_PER_STEP = 110.0
FLOPS_PER_EXTRA_BIN = 14.0
# DRAM bytes (read + write) per in-window (pixel, particle, step) of the pair
# kernel, from an ncu capture of one launch on 1250 of the 40000 pixels (the
# bench's 1024 particles, 4096 samples and 9 slots): 23.46e9 B / 3.101e9
# in-window steps.  Nothing of the partial traces is reused from L2 at either
# size, so the per-step figure carries over to the full launch.
DRAM_BYTES_PER_INWINDOW_STEP = 7.57


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=1024, help="particles per step")
    ap.add_argument("--pixels", type=int, default=0,
                    help="integrate an evenly spaced subset of about this many pixels (0 = all)")
    ap.add_argument("--slots", type=int, default=0,
                    help="particle-range slots per launch (0 = library default)")
    ap.add_argument("--nots", type=int, default=0,
                    help="trace samples (0 = the workload's 4096); only for small profiling runs")
    ap.add_argument("--variant", type=int, default=0,
                    help="FP32 kernel variant (teufel_options.kernel_variant; 0 = automatic)")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner (the automatic variant then uses its default)")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched-observer measurement")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the FP32-vs-FP64 comparison on the other workloads")
    ap.add_argument("--fp64-full", action="store_true",
                    help="instead of the bench line: FP32 split against FP64 GPU on the full "
                         "single-electron, 1e4-particle and gamma = 2000 workloads (~10 min)")
    ap.add_argument("--full-configs", action="store_true",
                    help="instead of the bench line: the 1e5-particle screen as ONE integration "
                         "call (multi-pass slots) and the 16 batched screens at a quarter of "
                         "their particle draws (~5 min, ~220 GB of device memory)")
    return ap.parse_args()


def workload_config(batch, n_pix, nots, npts, extra=None):
    c = {"workload": "config4: 1e5-particle 200 pC bunch (sigma_z 100 um, sigma_xy 1 mm, "
                     "gamma 300 +- 0.05%) in a lambda_u=0.3 m, 20-period, K=3 undulator at "
                     "100 steps/period; 200x200-pixel screen over 0.4x0.4 m at z=20 m; "
                     "4096 x 2 fs E/B traces; one step = one batch of the bunch onto the "
                     "whole screen",
         "particles_per_step": batch, "points_per_particle": npts, "pixels": n_pix,
         "samples": nots, "bunch_particles": 100000,
         "l2": "no flush: every step reads a new trajectory batch (~"
               f"{batch * npts * 160 / 1e6:.0f} MB) and writes {n_pix * nots * 48 / 1e9:.1f} GB "
               "of FP64 traces, both larger than the 129 MB L2"}
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [ln.strip().split(",") for ln in self.f.read().splitlines() if ln.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for k, n in enumerate(names):
                    if r[5 + k].strip().lower() in ("active", "1"):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------
def make_batches(n_batches, batch, nthreads=0, rank=0, world=1):
    """The batches of the 1e5-particle bunch that rank `rank` of `world`
    integrates (disjoint across ranks while they fit in the bunch)."""
    from teufel_gb300 import harness as H
    from teufel_gb300.sharding import rank_batches
    return [H.config4(first=first, count=batch, nthreads=nthreads)
            for first in rank_batches(rank, world, n_batches, batch, 100000)]


KERNEL_NAMES = {0: "lw_fp32_pair_kernel<128>", 1: "lw_fp32_warp_kernel<2>",
                2: "lw_fp32_lanes_kernel", 3: "lw_fp32_warp_kernel<3>",
                4: "lw_fp32_pair_kernel<128>", 5: "lw_fp32_pair_kernel<160>",
                6: "lw_fp32_pair_kernel<136>", 7: "lw_fp32_pair_kernel<144>",
                8: "lw_fp32_pair_kernel<128, multi-bin>",
                9: "lw_fp32_pair_kernel<128, FP64 arrival times>",
                10: "lw_fp32_pair_kernel<128, chunks of 8>",
                11: "lw_fp32_pair_kernel<128, chunks of 32>"}


def batch_measure(dev, reps=2, scale=64):
    """The batched uneven observers (16 seeded screens of the batched-observer
    configuration, each screen's particle draw divided by `scale`) as one
    teufel_cuda_batch: evaluations per second of one graph replay."""
    import torch
    from teufel_gb300 import abi, harness as H
    sets, bufs, obs = [], [], []
    evals = 0
    for spec in H.config3_specs():
        w = H.config3_screen(spec, count=max(4, spec["n_particles"] // scale))
        ts = abi.TrajSet(w.traj)
        pos = torch.from_numpy(np.ascontiguousarray(w.pix_pos)).to(dev)
        t0 = torch.from_numpy(np.ascontiguousarray(w.pix_t0)).to(dev)
        out = torch.zeros((w.n_pix, w.nots, 6), dtype=torch.float64, device=dev)
        sets.append(ts)
        bufs.append((pos, t0, out))
        obs.append((ts, pos.data_ptr(), t0.data_ptr(), w.dt, w.nots, w.n_pix, out.data_ptr()))
        evals += w.n_pix * int(np.sum(w.traj.n_points - 1))
    b = abi.Batch(obs)
    b.run()
    st, items, _, _ = b.status()
    abi.check(st, "batch")
    best = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record()
        b.run(torch.cuda.current_stream(dev).cuda_stream)
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    st, items, inwin, kms = b.status()
    abi.check(st, "batch")
    b.close()
    for ts in sets:
        ts.free()
    return {"value": evals / (best / 1e3), "unit": UNIT, "observers": len(obs),
            "work_items": items, "evals": evals, "ms": best,
            "launches": "one persistent integration kernel + one reduction, replayed as a CUDA graph",
            "workload": f"16 seeded screens of the batched uneven-observer configuration "
                        f"(meshes 16^2..128^2, 512..8192 samples, 2e3..2e4 steps), each with "
                        f"its particle draw / {scale} (min 4)"}


def other_workloads():
    """FP32-split against FP64-GPU throughput and accuracy on the other
    workloads (untimed by the driver; FP64 once and FP32 best of three, after a
    warm-up call each; the FP32 path tuned for the workload first, as
    teufel_cuda_autotune does for any caller):
    the single electron on the 21x21 screen in full, a 128-particle draw of
    the 1e4-particle bunch on its 64x64 screen, and a 64-particle draw of the
    gamma = 2000 bunch (multi-bin steps) on every 4th pixel of its 100x100
    screen."""
    from teufel_gb300 import abi, harness as H
    cases = [("single_electron_21x21_2048x5fs", H.config1(), None),
             ("bunch_1e4_100pC_64x64_2048x5fs_128_particles", H.config2(count=128), None),
             ("gamma2000_bunch_1e3_100x100_8192x1as_64_particles_every_4th_pixel",
              H.config5(count=64), 4)]
    out = {}
    for name, w, every in cases:
        if every:
            w = w.pixel_subset(np.arange(0, w.n_pix, every))
        evals = w.n_pix * int(np.sum(np.maximum(w.traj.n_points.astype(np.int64) - 1, 0)))
        res = {}
        with abi.TrajSet(w.traj) as ts:
            tv, _, _ = ts.autotune(w.pix_pos, w.pix_t0, w.dt, w.nots)
            # after a warm-up call: the FP64 path once (seconds), the FP32 path
            # best of three (tens of milliseconds, so single runs are noisy)
            # where the automatic choice is the FP64-time kernel, the chained
            # FP32 kernel (multi-bin deposits) is timed beside it
            runs = [(abi.PREC_FP64, 0, "fp64", 1), (abi.PREC_FP32_SPLIT, 0, "fp32", 3)]
            if tv == 9:
                runs.append((abi.PREC_FP32_SPLIT, 8, "fp32_chained", 3))
            for prec, variant, key, reps in runs:
                ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, precision=prec,
                                    variant=variant)
                best = None
                for _ in range(reps):
                    tt = time.perf_counter()
                    r = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, precision=prec,
                                            variant=variant)
                    el = time.perf_counter() - tt
                    best = el if best is None else min(best, el)
                res[key] = (r, best)
        ref = res["fp64"][0]
        out[name] = {"evals": evals, "pixels": w.n_pix, "particles": w.traj.n_particles,
                     "fp32_kernel": KERNEL_NAMES.get(tv, "?"),
                     "fp32_split_evals_per_s": evals / res["fp32"][1],
                     "fp64_gpu_evals_per_s": evals / res["fp64"][1],
                     "speedup_fp32_split_over_fp64": res["fp64"][1] / res["fp32"][1],
                     "rel_l2_fp32_split_vs_fp64":
                         float(np.linalg.norm(res["fp32"][0] - ref) / np.linalg.norm(ref))}
        if "fp32_chained" in res:
            out[name]["chained_fp32_times"] = {
                "kernel": KERNEL_NAMES[8],
                "evals_per_s": evals / res["fp32_chained"][1],
                "speedup_over_fp64": res["fp64"][1] / res["fp32_chained"][1],
                "rel_l2_vs_fp64": float(np.linalg.norm(res["fp32_chained"][0] - ref) /
                                        np.linalg.norm(ref))}
    return out


def full_comparison():
    """FP32 split against the FP64 GPU path on three workloads in full: the
    single electron on its 21x21 screen, the 1e4-particle 100 pC bunch on its
    64x64 screen and the 1e3-particle gamma = 2000 bunch on its 100x100 screen
    (8192 x 1 as).  Host buffers through integrate_screen, as a caller uses
    it.  The FP64 path runs once (minutes) after a warm-up call on one pixel;
    the FP32 path is tuned for the workload, then runs once as a warm-up and
    best of three."""
    from teufel_gb300 import abi, harness as H
    out = {}
    for name, make in (("single_electron_21x21_2048x5fs", H.config1),
                       ("bunch_1e4_100pC_64x64_2048x5fs", H.config2),
                       ("gamma2000_bunch_1e3_100x100_8192x1as", H.config5)):
        tt = time.perf_counter()
        w = make()
        t_track = time.perf_counter() - tt
        evals = w.n_pix * int(np.sum(np.maximum(w.traj.n_points.astype(np.int64) - 1, 0)))
        with abi.TrajSet(w.traj) as ts:
            ts.integrate_screen(w.pix_pos[:1], w.pix_t0[:1], w.dt, w.nots,
                                precision=abi.PREC_FP64)
            tt = time.perf_counter()
            r64 = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, precision=abi.PREC_FP64)
            t64 = time.perf_counter() - tt
            tv, _, _ = ts.autotune(w.pix_pos, w.pix_t0, w.dt, w.nots)
            ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots)
            t32 = None
            for _ in range(3):
                tt = time.perf_counter()
                r32 = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots)
                el = time.perf_counter() - tt
                t32 = el if t32 is None else min(t32, el)
            inwin, fallbacks, st = ts.last_inwindow()
            chained = None
            if tv == 9:
                # the chained FP32 arrival times (multi-bin deposits) beside it
                ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=8)
                tc = None
                for _ in range(2):
                    tt = time.perf_counter()
                    rc8 = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=8)
                    el = time.perf_counter() - tt
                    tc = el if tc is None else min(tc, el)
                chained = {"kernel": KERNEL_NAMES[8], "s": tc, "evals_per_s": evals / tc,
                           "speedup_over_fp64": t64 / tc,
                           "rel_l2_vs_fp64": float(np.linalg.norm(rc8 - r64) / np.linalg.norm(r64))}
                del rc8
        diff = r32 - r64
        out[name] = {"evals": evals, "pixels": w.n_pix, "particles": w.traj.n_particles,
                     "samples": w.nots, "dt": w.dt, "in_window_fraction": inwin / evals,
                     "exact_fallback_points": fallbacks, "status": st,
                     "fp32_kernel": KERNEL_NAMES.get(tv, "?"),
                     "fp32_split_s": t32, "fp64_gpu_s": t64,
                     "fp32_split_evals_per_s": evals / t32, "fp64_gpu_evals_per_s": evals / t64,
                     "speedup_fp32_split_over_fp64": t64 / t32,
                     "rel_l2_fp32_split_vs_fp64":
                         float(np.linalg.norm(diff) / np.linalg.norm(r64)),
                     "peak_sample_rel_err": float(np.abs(diff).max() / np.abs(r64).max()),
                     "tracking_s": t_track}
        if chained:
            out[name]["chained_fp32_times"] = chained
        del r32, r64, diff
    return out


def full_configs():
    """The workloads at (or near) their stated sizes through the public API:
    the 1e5-particle coherent-emission screen integrated by ONE
    teufel_cuda_integrate_screen call with host buffers (its 49+ FP32 slots
    run as successive passes of the partial-trace budget), checked against
    the FP64 GPU path on every 400th pixel; and the 16 batched uneven screens
    at a quarter of each screen's particle draw (the full draw's trajectories
    alone need ~630 GB) as one persistent launch."""
    import torch
    from teufel_gb300 import abi, harness as H
    out = {}
    # ---- the 1e5-particle bunch, one call ----
    tt = time.perf_counter()
    w = H.config4()
    t_track = time.perf_counter() - tt
    npts = int(w.traj.n_points[0])
    evals = w.n_pix * w.traj.n_particles * (npts - 1)
    with abi.TrajSet(w.traj) as ts:
        tv = 0  # the automatic kernel choice (one tuning trial here would take minutes)
        res = np.zeros((w.n_pix, w.nots, 6))
        tt = time.perf_counter()
        ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, out=res)
        t32 = time.perf_counter() - tt
        _, _, launches, _, _ = ts.last_timing()
        inwin, fallbacks, st = ts.last_inwindow()
        sub = np.arange(0, w.n_pix, 400)
        tt = time.perf_counter()
        r64 = ts.integrate_screen(w.pix_pos[sub], w.pix_t0[sub], w.dt, w.nots,
                                  precision=abi.PREC_FP64)
        t64 = time.perf_counter() - tt
        tt = time.perf_counter()
        r32s = ts.integrate_screen(w.pix_pos[sub], w.pix_t0[sub], w.dt, w.nots)
        t32s = time.perf_counter() - tt
    diff = res[sub] - r64
    out["bunch_1e5_200x200_4096x2fs_one_call"] = {
        "particles": w.traj.n_particles, "points_per_particle": npts, "pixels": w.n_pix,
        "samples": w.nots, "evals": evals, "in_window_fraction": inwin / evals,
        "fp32_kernel": KERNEL_NAMES.get(tv, "?"), "launches": launches,
        "passes": launches // 2, "status": st, "seconds": t32,
        "evals_per_s": evals / t32, "tracking_s": t_track,
        "fp64_check": {"pixels": len(sub), "rel_l2_fp32_split_vs_fp64":
                       float(np.linalg.norm(diff) / np.linalg.norm(r64)),
                       "peak_sample_rel_err": float(np.abs(diff).max() / np.abs(r64).max()),
                       "fp64_gpu_s": t64, "fp32_split_s_same_pixels": t32s,
                       "speedup_fp32_split_over_fp64": t64 / t32s}}
    del res, r64, r32s, diff, w
    # ---- the batched uneven screens at a quarter of their draws ----
    dev = torch.device("cuda", 0)
    torch.cuda.empty_cache()
    b = batch_measure(dev, reps=2, scale=4)
    out["batched_16_screens_quarter_draw"] = b
    return out


# ---------------------------------------------------------------------------
# CPU baseline / reference arm
# ---------------------------------------------------------------------------
def cpu_rate(w, target_s, nthreads):
    """Time the CPU oracle on a pixel x particle sample of workload w; the
    sample grows until one run takes at least target_s seconds."""
    from oracle import lw
    from teufel_gb300 import harness as H
    rng = np.random.default_rng(11)
    npts = int(w.traj.n_points[0])
    n_pix, n_part = max(nthreads, 4), 4
    while True:
        pix = np.sort(rng.choice(w.n_pix, min(n_pix, w.n_pix), replace=False))
        sub = w.traj.subset(list(range(min(n_part, w.traj.n_particles))))
        t = time.perf_counter()
        _, rc = lw.integrate_screen(sub, w.pix_pos[pix], w.pix_t0[pix], w.dt, w.nots,
                                    nthreads=nthreads)
        el = time.perf_counter() - t
        evals = len(pix) * sub.n_particles * (npts - 1)
        if el >= target_s or (n_part >= w.traj.n_particles and n_pix >= w.n_pix):
            return evals / el, f"{len(pix)} random pixels x {sub.n_particles} particles x " \
                               f"{npts - 1} steps ({evals:.3g} evals, {el:.1f} s)", el
        grow = max(2.0, min(8.0, 1.5 * target_s / max(el, 1e-3)))
        if n_part < w.traj.n_particles:
            n_part = min(w.traj.n_particles, int(math.ceil(n_part * grow)))
        else:
            n_pix = min(w.n_pix, int(math.ceil(n_pix * grow)))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import lw
    lw.build(with_reference=False)
    nthreads = os.cpu_count() or 1
    w = make_batches(1, args.batch)[0]
    npts = int(w.traj.n_points[0])
    budget = max(2.0, 150.0 / (args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_rate(w, min(1.0, budget), nthreads)
    rates, times, sample = [], [], ""
    for _ in range(args.steps):
        r, sample, el = cpu_rate(w, budget, nthreads)
        rates.append(r)
        times.append(el)
    value = statistics.median(rates)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.median(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.batch, w.n_pix, w.nots, npts),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": sample + " per step; the oracle's C restatement of "
                             "ChargedParticle::integrateFieldTrace with an OpenMP pixel loop "
                             "(the reference's own build needs its source tree, absent here)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------
def run_gb300(args):
    import torch
    from teufel_gb300 import abi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def barrier_sync():
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()

    K, W = args.steps, max(args.warmup, 0)
    n_batches = min(K + W, 64)
    batches = make_batches(n_batches, args.batch, rank=rank, world=world)
    if args.pixels:
        stride = max(1, batches[0].n_pix // args.pixels)
        batches = [b.pixel_subset(np.arange(0, b.n_pix, stride)) for b in batches]
    w0 = batches[0]
    npts = int(w0.traj.n_points[0])
    # every rank integrates its own batches onto the whole screen (weak scaling)
    lo, hi = 0, w0.n_pix
    n_pix = hi - lo
    nots = args.nots or w0.nots
    pos = torch.from_numpy(np.ascontiguousarray(w0.pix_pos[lo:hi])).to(dev)
    t0 = torch.from_numpy(np.ascontiguousarray(w0.pix_t0[lo:hi])).to(dev)
    out = torch.zeros((n_pix, nots, 6), dtype=torch.float64, device=dev)
    sets = [abi.TrajSet(b.traj) for b in batches]
    evals_step = n_pix * args.batch * (npts - 1)

    # the autotuner times the kernel configurations on the first batch; the
    # automatic variant (0) then uses its choice for this shape
    tuned = None
    if args.variant == 0 and not args.no_tune:
        tv, tslots, tms = sets[0].autotune(pos.data_ptr(), t0.data_ptr(), w0.dt, nots,
                                           n_pix=n_pix, device=True)
        tuned = {"kernel_variant": tv, "n_slots": tslots, "ms": tms}
        torch.cuda.synchronize(dev)

    def step(j, timing):
        sets[j % n_batches].integrate_screen_device(pos.data_ptr(), t0.data_ptr(), w0.dt, nots,
                                                    n_pix, out.data_ptr(), stream=sptr,
                                                    timing=timing, n_slots=args.slots,
                                                    variant=args.variant)

    peak32, peak32x2, peak64 = abi.probe_peaks()
    peak_fp32 = max(peak32, peak32x2)
    for j in range(W):
        step(j, False)
    barrier_sync()
    clocks = Clocks(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    kernel_ms, reduce_ms, launches = 0.0, 0.0, 0
    deposits, inwin, fallbacks, evaluations = 0, 0, 0, 0
    barrier_sync()
    e0.record(stream)
    for j in range(W, W + K):
        step(j, True)
        d, ne, nl, km, rm = sets[j % n_batches].last_timing()
        iw, fb, st = sets[j % n_batches].last_inwindow()
        abi.check(st, "integration")
        kernel_ms += km
        reduce_ms += rm
        launches += nl
        deposits += d
        evaluations += ne
        inwin += iw
        fallbacks += fb
    e1.record(stream)
    barrier_sync()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    ms_all = torch.tensor([ms], dtype=torch.float64, device=dev)
    if dist:
        dist.all_reduce(ms_all, op=dist.ReduceOp.MAX)
    ms_max = float(ms_all.item())
    value = evals_step * world * K / (ms_max / 1e3)
    flops = FLOPS_PER_STEP * inwin + FLOPS_PER_EXTRA_BIN * max(deposits - inwin, 0)
    achieved = flops / (kernel_ms / 1e3) / 1e12 if kernel_ms > 0 else 0.0

    # FP64 device path and accuracy on a pixel subset of the first batch
    sub = np.arange(lo, hi, 16)
    ws = w0.pixel_subset(sub)
    comp = {}
    with abi.TrajSet(ws.traj) as ts:
        for prec, name in ((abi.PREC_FP64, "fp64"), (abi.PREC_FP32_SPLIT, "fp32")):
            ts.integrate_screen(ws.pix_pos, ws.pix_t0, ws.dt, ws.nots, precision=prec)
            torch.cuda.synchronize(dev)
            reps = 2
            tt = time.perf_counter()
            for _ in range(reps):
                res = ts.integrate_screen(ws.pix_pos, ws.pix_t0, ws.dt, ws.nots, precision=prec)
            el = (time.perf_counter() - tt) / reps
            comp[name] = (res, el)
    ev_sub = len(sub) * args.batch * (npts - 1)
    fp64_rate = ev_sub / comp["fp64"][1]
    fp32_rate_sub = ev_sub / comp["fp32"][1]
    ref64 = comp["fp64"][0]
    rel = float(np.linalg.norm(comp["fp32"][0] - ref64) / np.linalg.norm(ref64))
    peak_err = float(np.abs(comp["fp32"][0] - ref64).max() / np.abs(ref64).max())

    # end to end through the C-ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        out_h = torch.zeros((n_pix, nots, 6), dtype=torch.float64).pin_memory().numpy()
        pos_h = torch.from_numpy(np.ascontiguousarray(w0.pix_pos[lo:hi])).pin_memory().numpy()
        t0_h = torch.from_numpy(np.ascontiguousarray(w0.pix_t0[lo:hi])).pin_memory().numpy()
        pinned = []
        for b in batches[:min(n_batches, K)]:
            tr = b.traj
            pinned.append(tuple(torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
                                for a in (tr.n_points.astype(np.int32), tr.charge, tr.t, tr.x,
                                          tr.p, tr.a)))
        h2d = 0
        d2h = n_pix * nots * 48
        def e2e_loop(overwrite):
            h2d = 0
            barrier_sync()
            tt = time.perf_counter()
            for j in range(K):
                npnt, ch, t, x, p, a = pinned[j % len(pinned)]
                with abi.TrajSet.from_arrays(npnt, ch, t, x, p, a) as ts:
                    ts.integrate_screen(pos_h, t0_h, w0.dt, nots, out=out_h,
                                        overwrite_out=overwrite)
                if j == 0:
                    h2d = sum(v.nbytes for v in (npnt, ch, t, x, p, a)) + pos_h.nbytes + \
                        t0_h.nbytes + (0 if overwrite else out_h.nbytes)
            barrier_sync()
            el = time.perf_counter() - tt
            el_all = torch.tensor([el], dtype=torch.float64, device=dev)
            if dist:
                dist.all_reduce(el_all, op=dist.ReduceOp.MAX)
            return float(el_all.item()), h2d

        # each step's traces added into the caller's buffer (FieldTrace::add)
        el, h2d = e2e_loop(False)
        e2e = {"value": evals_step * world * K / el, "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": 1e3 * el / K}
        # the call an observer makes right after zero(): the traces are
        # stored (overwrite_out), so the buffer is not uploaded
        el, h2d = e2e_loop(True)
        e2e["overwrite_out"] = {"value": evals_step * world * K / el,
                                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                                "ms_per_step": 1e3 * el / K}

    batch = None
    if rank == 0 and world == 1 and not args.no_batch:
        # the trajectory sets of the timed loop are released first
        for ts in sets:
            ts.free()
        sets = []
        out = None
        torch.cuda.empty_cache()
        batch = batch_measure(dev)

    others = None
    if rank == 0 and world == 1 and not args.no_configs:
        others = other_workloads()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        rate, sample, _ = cpu_rate(w0, 12.0, nthreads)
        rate1, sample1, _ = cpu_rate(w0, 5.0, 1)
        cpu = {"value": rate, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": sample + "; the oracle's C restatement of the reference's "
                         "integrateFieldTrace, OpenMP over pixels",
               "value_1_thread": rate1, "sample_1_thread": sample1}

    if rank == 0:
        frac_in = inwin / (evals_step * K) if K else 0.0
        # the metric's own qualifiers (accuracy against the FP64 GPU path and
        # the speed-up over it) go into config, whose keys the line keeps
        headline = {
            "rel_l2_fp32_split_vs_fp64": rel, "peak_sample_rel_err_vs_fp64": peak_err,
            "fp64_gpu_evals_per_s": fp64_rate, "fp32_split_evals_per_s_same_sample": fp32_rate_sub,
            "speedup_fp32_split_over_fp64": fp32_rate_sub / fp64_rate,
            "accuracy_sample": f"{len(sub)} pixels (every 16th) x {args.batch} particles",
        }
        if others:
            headline["other_workloads"] = {
                k.split("_")[0] + "_" + k.split("_")[1]: {
                    "speedup_fp32_split_over_fp64": v["speedup_fp32_split_over_fp64"],
                    "rel_l2_fp32_split_vs_fp64": v["rel_l2_fp32_split_vs_fp64"],
                    "fp32_split_evals_per_s": v["fp32_split_evals_per_s"]}
                for k, v in others.items()}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms_max / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args.batch, w0.n_pix, nots, npts,
                                      {"parallelism": f"particle batches x{world}: every rank integrates "
                                                      "its own batches of the bunch onto the whole "
                                                      "screen, no exchange",
                                       "in_window_fraction": frac_in,
                                       "point_evaluations_per_in_window_step":
                                           evaluations / inwin if inwin else None,
                                       "exact_fallback_points": fallbacks,
                                       "fp32_vs_fp64": headline}),
            "fp64_gpu": {"value": fp64_rate, "unit": UNIT,
                         "sample": f"{len(sub)} pixels (every 16th) x {args.batch} particles",
                         "fp32_split_same_sample": fp32_rate_sub,
                         "speedup_fp32_split_over_fp64": fp32_rate_sub / fp64_rate},
            "accuracy": {"rel_l2_fp32_split_vs_fp64": rel, "peak_sample_rel_err": peak_err,
                         "sample": f"{len(sub)} pixels x {args.batch} particles"},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_fp32,
                         "unit": "TFLOP/s", "frac": achieved / peak_fp32 if peak_fp32 else None,
                         "traffic": DRAM_BYTES_PER_INWINDOW_STEP * inwin / max(K, 1),
                         "traffic_note": f"DRAM bytes per launch: "
                                         f"{DRAM_BYTES_PER_INWINDOW_STEP} B per in-window step "
                                         "(dram__bytes_read.sum + write.sum of one launch on "
                                         "1250 of the 40000 pixels, 1024 particles, 9 slots) "
                                         "times the in-window steps of one full launch",
                         "kernel": KERNEL_NAMES.get(tuned["kernel_variant"] if tuned
                                                    else args.variant, "?"),
                         "peak_source": "the larger of the FFMA and packed-FFMA2 throughput "
                                        "probes run by bench.py on this GPU "
                                        "(MEASURED_PEAKS.json has no FP32 figure)",
                         "ffma_probe_tflops": peak32, "ffma2_probe_tflops": peak32x2,
                         "algorithmic_flops": flops, "kernel_ms": kernel_ms,
                         "reduce_ms": reduce_ms, "fp64_probe_tflops": peak64},
            "autotune": tuned,
            "batched_observers": batch,
            "gpu_launches": launches,
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        # the full comparison on the other workloads on a line of its own
        # (stderr), so that it cannot push the bench line out of a log's tail
        if others:
            print(json.dumps({"other_workloads": others}), file=sys.stderr)
        print(json.dumps(line))
    for s in sets:
        s.free()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.fp64_full:
        print(json.dumps({"fp32_split_vs_fp64_gpu_full_workloads": full_comparison()}))
        return 0
    if args.full_configs:
        print(json.dumps({"full_configs": full_configs()}))
        return 0
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
