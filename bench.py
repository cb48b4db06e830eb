#!/usr/bin/env python
"""Benchmark of the sightline-interpolation path (`_Particle_Interpolate`) on GB300.

One step = one full call for the Ly-a line over every sightline of the
workload: the sightline-particle search and the tau deposit, inputs resident
in HBM (device API).  `value` is Ly-a tau pixels/s of the tuned FP32 form
(sightlines x pixels per call / call time), whole job over all ranks.

Beside it, on the same workload:
  fp64_plain   the plain FP64 form (on a stated sightline subset when the full
               set would take minutes: FP64 runs at 1/64 of the FP32 rate here);
  accuracy     max|dF|, relative tau error and column-density error of the FP32
               form against the FP64 form on those sightlines;
  e2e          the same metric through the host-pointer C ABI call
               (fsg_particle_interpolate), with the host<->device copies timed,
               and through the Python drop-in (a new output array per call);
  roofline     the deposit kernel against the FP32 FMA-pipe peak measured by
               the library's own microbenchmark, from exact work counts;
  cpu_baseline the CPU oracle (C restatement of the reference, OpenMP, all
               host cores) on a stated sample of sightlines.

`--impl reference` times the CPU implementation alone (the oracle; the
reference sources are not on the GPU machine) on the same workload.
Multi-GPU: independent replicas (the path is not sharded), weak scaling.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HEADLINE_METRIC = ("Ly-α tau pixels/s, tuned FP32 vs plain FP64 GPU at max|ΔF|≤1e-4; "
                   "fwd+bwd ms")

# Algorithmic work unit of the roofline: one profile evaluation of the
# reference's 7-node line-of-sight sum under its window rule, counted exactly by
# the counting variant of the deposit kernel, at a frozen F_EVAL flops per
# evaluation: the cheapest complete FP32 evaluation (asymptotic branch, 15 FMA
# + 1 reciprocal, and the weighted add of the node sum; FMA = 2 flops).
F_EVAL = 32
# Flops executed per evaluation by each branch, counted once from the source
# (fsg_voigt.cuh, fsg_deposit.cu), for the executed-flop figure beside it.  Wing
# evaluations summed by the far-wing multipole form cost 20 flops per pixel
# (7 evaluations): 20/7 each.
FLOPS_FP32 = {"core": 69, "wing": 32, "other": 214, "multipole": 20.0 / 7.0}
# DRAM traffic of the FP32 deposit from one ncu capture of the 512^3 workload's
# recipe at 192^3 particles and 2048 sightlines (dram__bytes_read.sum +
# dram__bytes_write.sum, kept with the profile summaries): 2.751220 GB read for
# 5038719 pairs, 0.245783040 GB written for 2048 x 11152 pixels; scaled to a
# launch by pairs (reads) and output pixels (writes).
TRAFFIC_READ_PER_PAIR = 2.751220e9 / 5038719
TRAFFIC_WRITE_PER_PIXEL = 0.245783040e9 / (2048 * 11152)
FLOPS_FP64 = {"core": 214, "wing": 144, "other": 20}


FALLBACK_HBM_GBS = 6800.0   # one earlier STREAM-style copy measurement on a GB300


def measured_hbm_gbs():
    """(GB/s, source): the measured copy bandwidth of MEASURED_PEAKS.json, else
    the fallback figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f).get("hbm_gbs")), "measured (MEASURED_PEAKS.json)"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback (no MEASURED_PEAKS.json)"


def search_roofline(npart, npairs, nlos, ms):
    """HBM view of the sightline search (particle sort + count + emit): the
    algorithmic bytes are the particle stream and the pair lists.  Sort: read
    pos (12 B), write the cell key (4 B), read the key and write the order
    (8 B); count and emit: read the order (4 B), pos (12 B) and h (4 B) each;
    emit: write 12 B per pair; offsets 8 B per sightline."""
    algo = npart * (12 + 4 + 8 + 2 * (4 + 12 + 4)) + npairs * 12 + nlos * 8
    hbm, src = measured_hbm_gbs()
    achieved = algo / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "peak_source": src,
            "unit": "GB/s", "frac": achieved / hbm, "bytes": algo,
            "note": "the search is limited by the cell walk (latency of the dependent cell "
                    "and sightline loads), not by HBM (16 B of particle data per particle "
                    "per pass); the FP64 predicate runs only on the thin shell the float "
                    "tests cannot decide"}


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="fsg", choices=["fsg", "reference"])
    p.add_argument("--config", type=int, default=3, choices=[1, 2, 3, 4])
    p.add_argument("--nside", type=int, default=0, help="particles per side (0 = the config's)")
    p.add_argument("--nlos", type=int, default=0, help="sightlines (0 = the config's)")
    p.add_argument("--fp64-lines", type=int, default=512,
                   help="sightlines timed in the plain FP64 form (0 = all)")
    p.add_argument("--cpu-per-stratum", type=int, default=11,
                   help="sightlines per stratum in the CPU baseline sample")
    p.add_argument("--no-config2", action="store_true",
                   help="skip the per-line 256^3 three-line report against the oracle")
    p.add_argument("--no-tophat", action="store_true",
                   help="skip the 256^3 cubic-spline / top-hat section")
    p.add_argument("--sweep", action="store_true",
                   help="time every launch candidate on the full call (autotuner evidence)")
    p.add_argument("--launch", default="",
                   help="threads,chunk,persistent[,records] of the FP32 deposit instead of the "
                        "autotuner's choice (no tuning run; for profiling a fixed launch)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--no-bwd", action="store_true")
    p.add_argument("--no-extra", action="store_true",
                   help="skip the multi-channel column density and flux statistics sections")
    p.add_argument("--flux-only", type=int, default=0, metavar="NSPEC",
                   help="time only the flux statistics on a seeded synthetic tau of NSPEC x "
                        "11152 pixels (a small case for profiling their kernels)")
    return p.parse_args()


def flux_only(args):
    """The flux statistics alone on a seeded lognormal tau of nspec x 11152
    pixels (saturated and empty pixels included), resident on the device."""
    import torch
    from fake_spectra_gb300 import build
    from fake_spectra_gb300 import fluxstatistics as fstat
    build.build()
    g = torch.Generator(device="cuda")
    g.manual_seed(2024)
    nspec, npix = args.flux_only, 11152
    tau = torch.exp(2.0 * torch.randn((nspec, npix), generator=g, device="cuda",
                                      dtype=torch.float64))
    u = torch.rand((nspec, npix), generator=g, device="cuda", dtype=torch.float64)
    tau[u < 0.01] = 0.0
    tau[u > 0.99] = 1e4
    torch.cuda.synchronize()
    calls = {"mean_flux": lambda: fstat.mean_flux(tau, 0.7),
             "flux_pdf": lambda: fstat.flux_pdf(tau, 20, None),
             "flux_power": lambda: fstat.flux_power(tau, npix * 1.0, 8, 0.7, False)}
    res = {}
    for name, fn in calls.items():
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fn()
        torch.cuda.synchronize()
        res[name + "_ms"] = (time.perf_counter() - t0) * 1e3 / max(args.steps, 1)
        res[name + "_kernels_ms"] = fstat._context().stats()["ms_flux"]
    print(json.dumps({"flux_only": {"nspec": nspec, "npix": npix, "steps": args.steps,
                                    "warmup": args.warmup, **res,
                                    "note": "kernels_ms is the device time of the last "
                                            "call's kernels"}}))


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return self
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        smax = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(self.rows)}


def make_workload(args, device):
    from fake_spectra_gb300 import synth
    return synth.generate_torch(args.config, device=device, nside=args.nside or None,
                                nlos=args.nlos or None)


def subset_lines(nlos, k, seed=12345):
    if k <= 0 or k >= nlos:
        return np.arange(nlos)
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(nlos, size=k, replace=False))


# Port/reference speed factor: the C restatement against the reference's own
# build on the same inputs (32^3 workload, 64 sightlines, 8 threads, x86 host):
# 1.61 s against 1.33 s.  The reference build cannot run on the GPU machine.
PORT_OVER_REFERENCE_TIME = 1.61 / 1.33


def strata_of(w):
    """Strata of the CPU sample: sightline axis x placement (through a clump
    centre or not, where the workload records it)."""
    cls = w.line_class if w.line_class is not None else np.zeros(w.nlos, np.int8)
    keys = sorted(set(zip(w.axis.tolist(), cls.tolist())))
    return {k: np.nonzero((w.axis == k[0]) & (cls == k[1]))[0] for k in keys}


def stratified_picks(strata, per_stratum, seed):
    rng = np.random.default_rng(seed)
    return {k: np.sort(rng.choice(v, size=min(per_stratum, len(v)), replace=False))
            for k, v in strata.items()}


class CpuEstimate:
    """Whole-workload CPU time of the oracle from a stratified sightline sample.

    T = T_search(all sightlines) + sum over strata N_s x (mean thread-seconds per
    sampled sightline of stratum s) / cores: the oracle's deposit is an OpenMP
    loop over sightlines (part_int.cpp:25-27), so with N >> cores the threads
    stay busy and the wall time is the thread time over the cores."""

    def __init__(self, w, strata, cores):
        self.w, self.strata, self.cores = w, strata, cores
        self.sec = {k: [] for k in strata}
        self.t_search_full = None
        self.npairs_full = None

    def add(self, keys, line_sec):
        for k, t in zip(keys, line_sec):
            self.sec[k].append(float(t))

    def seconds(self):
        dep = sum(len(self.strata[k]) * float(np.mean(v)) / self.cores
                  for k, v in self.sec.items() if v)
        return (self.t_search_full or 0.0) + dep, dep

    def value(self):
        return self.w.nlos * self.w.nbins / self.seconds()[0]

    def describe(self, seed, extra=""):
        t, dep = self.seconds()
        per = {"axis%d_%s" % (k[0], "clump" if k[1] else "field"):
               {"sightlines": int(len(self.strata[k])), "sampled": len(v),
                "thread_s_per_line": float(np.mean(v)) if v else None}
               for k, v in self.sec.items()}
        return {"strata": per, "seed": seed, "search_all_s": self.t_search_full,
                "deposit_all_s_est": dep, "total_s_est": t,
                "port_over_reference_time": PORT_OVER_REFERENCE_TIME,
                "note": "extrapolated: search timed on all %d sightlines; deposit from "
                        "per-sightline thread seconds of a stratified sample (axis x "
                        "clump-centred or not), weighted by stratum size, over %d cores. The "
                        "C restatement runs %.2fx the reference build's time on the same "
                        "inputs (measured on an x86 host; the reference build cannot run on "
                        "this machine), so the reference's own CPU rate would be about that "
                        "factor higher.%s" % (self.w.nlos, self.cores,
                                             PORT_OVER_REFERENCE_TIME, extra)}


def oracle_lines(port, wh, transition, ct, lines, timed=False):
    """The oracle on the given sightlines (all particles).  timed: also the search
    seconds and per-sightline thread seconds."""
    a = list(wh.call_args(transition, ct))
    a[16], a[17] = wh.axis[lines], wh.cofm[lines]
    if timed:
        return port.particle_interpolate_timed(*a)
    return port.particle_interpolate(*a)


def accuracy_stats(got, want, ct):
    """max|dF|, tau relative error (tau >= 1e-3) or column-density relative error."""
    if ct:
        dF = np.abs(np.exp(-got) - np.exp(-want))
        big = want >= 1e-3
        rel = np.abs(got - want)[big] / want[big] if big.any() else np.zeros(1)
        return {"max_abs_dF": float(dF.max()), "tau_rel_err_max": float(rel.max()),
                "tau_rel_err_median": float(np.median(rel))}
    nz = want != 0
    rel = np.abs(got - want)[nz] / np.abs(want[nz]) if nz.any() else np.zeros(1)
    return {"colden_rel_err_max": float(rel.max())}


def run_reference(args):
    rank, world, local = dist_setup()
    if rank != 0:
        return
    import torch
    import oracle
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    w = make_workload(args, dev).to_host()
    threads = os.cpu_count() or 1
    port = oracle.port()
    port.set_threads(threads)
    strata = strata_of(w)
    keys = sorted(strata)
    picks = stratified_picks(strata, args.cpu_per_stratum, seed=12345)
    est = CpuEstimate(w, strata, threads)
    est.t_search_full, est.npairs_full = port.search_seconds(w.pos, w.hh, w.axis, w.cofm, w.box)
    rounds = max(len(v) for v in picks.values())

    def one_round(r):
        lines = np.array([picks[k][r % len(picks[k])] for k in keys])
        t0 = time.perf_counter()
        _, _, sec = oracle_lines(port, w, synth_lya(), 1, lines, timed=True)
        return time.perf_counter() - t0, sec

    for r in range(args.warmup):
        one_round(rounds - 1 - r % rounds)
    walls = []
    for step in range(args.steps):
        dt, sec = one_round(step % rounds)
        walls.append(dt)
        est.add(keys, sec)
    value = est.value()
    sample = ("CPU oracle (C restatement of the reference path, OpenMP, %d threads); each step "
              "one sightline from each of the %d strata (axis x clump-centred or not) with all "
              "%d particles" % (threads, len(keys), w.npart))
    print(json.dumps({
        "impl": "reference", "metric": HEADLINE_METRIC, "value": value, "unit": "pixels/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(walls) / len(walls), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w.name, "particles": w.npart, "sightlines": w.nlos,
                   "nbins": w.nbins, "line": "Ly-a 1215.67 A", "kernel": "cubic spline"},
        "cpu_baseline": {"value": value, "unit": "pixels/s", "cores": threads, "kind": "port",
                         "sample": sample, "estimate": est.describe(12345)},
        "e2e": {"value": value, "unit": "pixels/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }))


def synth_lya():
    from fake_spectra_gb300 import synth
    return synth.LYA


def config2_report(ctx, interp, synth):
    """Ly-a, Ly-b and CIV 1548 on the 256^3 three-line workload: the batched FP32
    call over all 3600 sightlines and FP64 calls on a sightline sample, each
    against the oracle on that sample (the 6 sightlines with the most pairs and
    18 random ones), per line, for tau and column density."""
    import torch
    import oracle
    port = oracle.port()
    port.set_threads(os.cpu_count() or 1)
    w2 = synth.generate_torch(2, device="cuda")
    npairs = interp.build_pairs(ctx, w2.box, w2.pos, w2.hh, w2.axis, w2.cofm)
    off, _, _ = interp.copy_pairs(ctx, w2.nlos, npairs, sorted=False)
    cnt = np.diff(off)
    top = np.argsort(-cnt, kind="stable")[:6]
    rng = np.random.default_rng(2024)
    lines = np.sort(np.concatenate([top, rng.choice(np.setdiff1d(np.arange(w2.nlos), top),
                                                    size=18, replace=False)]))
    wh = w2.to_host()
    _, ppart, _ = port.near_particles(wh.pos, wh.hh, w2.axis[lines], w2.cofm[lines], w2.box)
    sub = np.unique(ppart)
    blines = [(t, w2.dens[t.species], True, True) for t in w2.transitions]

    def batch():
        return interp.spectra_batch_device(ctx, w2.nbins, w2.kernel, w2.box, w2.velfac,
                                           w2.atime, w2.tautail, w2.pos, w2.vel, w2.temp, w2.hh,
                                           w2.axis, w2.cofm, blines, precision="fp32")
    outs = batch()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    outs = batch()
    torch.cuda.synchronize()
    ms_batch = (time.perf_counter() - t0) * 1e3
    rows = torch.from_numpy(lines).cuda()
    per_line = {}
    for (t, _, _, _), (tau_t, col_t) in zip(blines, outs):
        r = {}
        for ct, full in ((1, tau_t), (0, col_t)):
            a = list(w2.call_args(t, ct))
            a[16], a[17] = w2.axis[lines], w2.cofm[lines]
            g64 = interp.particle_interpolate_device(ctx, *a, precision="fp64").cpu().numpy()
            ha = list(wh.call_args(t, ct))
            for k in range(11, 16):
                ha[k] = ha[k][sub]
            ha[16], ha[17] = wh.axis[lines], wh.cofm[lines]
            want = port.particle_interpolate(*ha)
            g32 = full[rows].cpu().numpy()
            for form, got in (("fp32", g32), ("fp64", g64)):
                r.setdefault(form, {}).update(accuracy_stats(got, want, ct))
        per_line[t.name] = r
    del outs
    return {"workload": w2.name, "particles": w2.npart, "sightlines_total": w2.nlos,
            "nbins": w2.nbins, "sightlines_compared": int(len(lines)),
            "sample": "the 6 sightlines with the most pairs and 18 random ones (seed 2024)",
            "fp32": "one batched call over all sightlines (search + one CUDA graph of 3 tau + "
                    "3 column-density deposits): %.1f ms" % ms_batch,
            "fp64": "one call per line and quantity on the sampled sightlines",
            "against": "CPU oracle (FP64 C restatement, pinned to the reference build)",
            "lines": per_line}


def config1_kernels(ctx, interp, synth, stream, with_cpu=True):
    """The 256^3 workload (3600 sightlines x 6691 pixels, Ly-a) with the cubic
    spline and the top-hat kernel: FP32 over all sightlines, FP64 on a 600-line
    subset, the CPU oracle's estimate for the whole workload from 8 sampled
    sightlines, and both GPU forms against the oracle on those 8."""
    import torch
    w1 = synth.generate_torch(1, device="cuda")
    lya = synth.LYA
    wh = w1.to_host() if with_cpu else None
    sub = subset_lines(w1.nlos, 600, seed=31)
    samp = subset_lines(w1.nlos, 8, seed=32)
    pixels = w1.nlos * w1.nbins
    out = {"workload": w1.name, "particles": w1.npart, "sightlines": w1.nlos,
           "nbins": w1.nbins}
    if with_cpu:
        import oracle
        port = oracle.port()
        threads = os.cpu_count() or 1
        port.set_threads(threads)
        t_search, _ = port.search_seconds(wh.pos, wh.hh, wh.axis, wh.cofm, wh.box)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for kernel, name in ((1, "cubic_spline"), (0, "top_hat")):
        a = list(w1.call_args(lya, 1, kernel=kernel))
        o = torch.empty((w1.nlos, w1.nbins), dtype=torch.float64, device="cuda")
        interp.particle_interpolate_device(ctx, *a, out=o, precision="fp32", tune=1)
        tuned = ctx.stats()
        dflt = []
        for _ in range(2):
            interp.particle_interpolate_device(ctx, *a, out=o, precision="fp32", tune=-1)
            dflt.append(ctx.stats()["ms_deposit"])
        torch.cuda.synchronize()
        e0.record(stream)
        dep = []
        for _ in range(3):
            interp.particle_interpolate_device(ctx, *a, out=o, precision="fp32")
            dep.append(ctx.stats()["ms_deposit"])
        e1.record(stream)
        torch.cuda.synchronize()
        ms32 = e0.elapsed_time(e1) / 3
        a64 = list(a)
        a64[16], a64[17] = w1.axis[sub], w1.cofm[sub]
        o64 = torch.empty((len(sub), w1.nbins), dtype=torch.float64, device="cuda")
        e0.record(stream)
        interp.particle_interpolate_device(ctx, *a64, out=o64, precision="fp64")
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        r = {"fp32": {"value": pixels / (ms32 * 1e-3), "unit": "pixels/s", "ms_per_call": ms32,
                      "sightlines": w1.nlos,
                      "autotune": {"chosen": tuned["launch"], "sample": tuned["tune"],
                                   "deposit_ms_default_launch": min(dflt),
                                   "deposit_ms_tuned": min(dep),
                                   "gain": min(dflt) / min(dep)}},
             "fp64": {"value": len(sub) * w1.nbins / (ms64 * 1e-3), "unit": "pixels/s",
                      "ms_per_call": ms64, "sightlines": int(len(sub))}}
        if with_cpu:
            ha = list(wh.call_args(lya, 1, kernel=kernel))
            ha[16], ha[17] = wh.axis[samp], wh.cofm[samp]
            want, _, sec = port.particle_interpolate_timed(*ha)
            t_all = t_search + w1.nlos * float(np.mean(sec)) / threads
            r["cpu"] = {"value": pixels / t_all, "unit": "pixels/s", "cores": threads,
                        "kind": "port", "estimate_s": t_all,
                        "sample": "search timed on all sightlines (%.1f s); deposit from the "
                                  "thread seconds of 8 random sightlines" % t_search}
            g32 = o[torch.from_numpy(samp).cuda()].cpu().numpy()
            a64[16], a64[17] = w1.axis[samp], w1.cofm[samp]
            g64 = interp.particle_interpolate_device(ctx, *a64, precision="fp64").cpu().numpy()
            r["fp32"].update(accuracy_stats(g32, want, 1))
            r["fp64"].update(accuracy_stats(g64, want, 1))
            r["compared_sightlines"] = 8
        out[name] = r
        del o, o64
    return out


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.flux_only:
        flux_only(args)
        return
    rank, world, local = dist_setup()
    import torch
    torch.cuda.set_device(local)
    from fake_spectra_gb300 import build, synth, interp, _lib
    build.build()
    w = make_workload(args, "cuda")
    torch.cuda.synchronize()
    ctx = _lib.Context(local)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    lya = synth.LYA
    targs = w.call_args(lya, 1)
    pixels = w.nlos * w.nbins
    out = torch.empty((w.nlos, w.nbins), dtype=torch.float64, device="cuda")

    def step(precision, o=out, lines=None, count=False, **kw):
        a = list(targs)
        if lines is not None:
            a[16] = w.axis[lines]
            a[17] = w.cofm[lines]
        return interp.particle_interpolate_device(ctx, *a, out=o, precision=precision,
                                                  count_work=count, **kw)

    # ---- the autotuner picks the FP32 deposit's launch (timed on a sample of the
    # call's sightlines), untimed; the calls below use its cached choice
    fixed = {}
    if args.launch:
        v = [int(x) for x in args.launch.split(",")]
        fixed = dict(threads=v[0], chunk=v[1], persistent=v[2],
                     records=v[3] if len(v) > 3 else 0)
    else:
        step("fp32", tune=1)
    tuned = ctx.stats()
    # ---- tuned FP32 form: the timed region
    for _ in range(args.warmup):
        step("fp32", **fixed)
    stream = torch.cuda.current_stream()
    launches0 = ctx.stats()["gpu_launches"]
    clocks = ClockSampler(local).start()
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    dep_ms, search_ms = [], []
    for _ in range(args.steps):
        step("fp32", **fixed)
        st = ctx.stats()
        dep_ms.append(st["ms_deposit"])
        search_ms.append(st["ms_search"])
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    launches = ctx.stats()["gpu_launches"] - launches0
    ms_step = allreduce_max(ev0.elapsed_time(ev1) / args.steps, world)
    value = world * pixels / (ms_step * 1e-3)
    tau32 = out.clone()
    npairs = ctx.stats()["npairs"]

    # ---- work counts for the roofline (untimed counting variant)
    step("fp32", o=torch.empty_like(out), count=True)
    cnt = ctx.stats()
    mp = cnt["evals_wing_multipole"]
    evals = cnt["evals_core"] + cnt["evals_wing"] + cnt["evals_other"]
    executed = (cnt["evals_core"] * FLOPS_FP32["core"]
                + (cnt["evals_wing"] - mp) * FLOPS_FP32["wing"]
                + cnt["evals_other"] * FLOPS_FP32["other"] + mp * FLOPS_FP32["multipole"])
    dep_mean = sum(dep_ms) / len(dep_ms)
    peak32 = _lib.fma_peak_tflops("fp32")
    achieved = evals * F_EVAL / (dep_mean * 1e-3) / 1e12
    achieved_exec = executed / (dep_mean * 1e-3) / 1e12
    peak64 = _lib.fma_peak_tflops("fp64")
    res = {
        "metric": HEADLINE_METRIC, "value": value, "unit": "pixels/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded torch generator (clumpy particles, lognormal fields, "
                "sightline grid or random sightlines with a quarter through clump centres)",
        "config": {"workload": w.name, "particles": w.npart, "sightlines": w.nlos,
                   "nbins": w.nbins, "pairs": npairs, "line": "Ly-a 1215.67 A",
                   "kernel": "cubic spline", "form": "FP32 tuned (persistent sightline queue)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (%.2f GB of particle arrays)" % (w.npart * 36 / 1e9)},
        "gpu_launches": launches,
        "clocks": clk,
        "phases_ms": {"search": sum(search_ms) / len(search_ms), "deposit": dep_mean},
        "search_roofline": search_roofline(w.npart, npairs, w.nlos,
                                           sum(search_ms) / len(search_ms)),
        "roofline": {"bound": "fp32-pipe", "kernel": "deposit_kernel<tau, FP32>",
                     "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                     "frac": achieved / peak32,
                     "peak_source": "measured: libfsg FMA-chain microbenchmark (MEASURED_PEAKS.json "
                                    "has no FP32 figure)",
                     "work": {"unit": "reference profile evaluations (7 per pixel sample)",
                              "evals": evals, "flops_per_eval": F_EVAL,
                              "evals_core": cnt["evals_core"], "evals_wing": cnt["evals_wing"],
                              "evals_wing_multipole": mp,
                              "samples_by_path": {"multipole": mp // 7,
                                                  "wing": cnt["samples_wing_path"],
                                                  "core": cnt["samples_core_path"],
                                                  "mixed": cnt["samples_mixed_path"]},
                              "evals_other": cnt["evals_other"], "pixels": cnt["pixels"],
                              "launches_timed": 1,
                              "deposit_ms_per_launch": dep_mean},
                     "executed": {"flops_per_eval_by_branch": FLOPS_FP32,
                                  "achieved": achieved_exec, "frac": achieved_exec / peak32,
                                  "note": "flops of the pixel-by-pixel walk over the same "
                                          "windows; far-field tiles execute fewer (10 node "
                                          "evaluations per 64 far pixels), so this is an upper "
                                          "bound of the executed rate"},
                     "peak_fp64": peak64,
                     "traffic": npairs * TRAFFIC_READ_PER_PAIR + pixels * TRAFFIC_WRITE_PER_PIXEL,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the "
                                       "192^3 x 2048-sightline capture, scaled by pairs and "
                                       "output pixels"},
    }

    # ---- the tuner's gain on the full call: the library's default launch, same work
    dflt = []
    for _ in range(2):
        step("fp32", tune=-1)
        dflt.append(ctx.stats()["ms_deposit"])
    res["autotune"] = {
        "chosen": tuned["launch"], "sample": tuned["tune"],
        "deposit_ms_default_launch": min(dflt), "deposit_ms_tuned": dep_mean,
        "gain": min(dflt) / dep_mean,
        "note": "candidates (threads per block in builds of 512/768/1024, pairs staged per "
                "warp, queue mode) timed on every k-th sightline of the descending pair-count "
                "order, about four per resident block; all give the same output bits"}
    if args.sweep:
        sweep = {}
        for th, ch, pm, rc in ((512, 8, 1, 0), (512, 16, 1, 0), (768, 8, 1, 0), (1024, 8, 1, 0),
                               (1024, 4, 1, 0), (1024, 8, 0, 0), (1024, 8, 1, 1),
                               (768, 8, 1, 1)):
            ms = []
            for _ in range(2):
                step("fp32", threads=th, chunk=ch, persistent=pm, records=rc)
                ms.append(ctx.stats()["ms_deposit"])
            sweep["%d_%d_%d%s" % (th, ch, pm, "_records" if rc else "")] = min(ms)
        res["autotune"]["full_call_sweep_ms"] = sweep

    # ---- end to end through the host-pointer C ABI (copies inside the timed region),
    # right after the device-resident measurement, under the same conditions
    if not args.no_e2e:
        import ctypes
        from fake_spectra_gb300._spectra_priv import _Particle_Interpolate, _ptr
        pin = lambda t: t.cpu().pin_memory().numpy()
        h = [pin(x) for x in (w.pos, w.vel, w.dens["HI"], w.temp, w.hh)]
        hargs = list(targs[:11]) + h + [w.axis, w.cofm]
        ke = max(1, min(args.steps, 3))
        # (a) the C ABI call a host program makes: its own output array,
        # allocated once; every call copies the inputs in and the spectra out
        L = _lib.load()
        opt = _lib.make_options("fp32")
        eb = _lib.errbuf()
        tau_h = np.zeros((w.nlos, w.nbins))
        axis_h, cofm_h = np.ascontiguousarray(w.axis), np.ascontiguousarray(w.cofm)

        def c_call():
            rc = L.fsg_particle_interpolate(
                1, w.nbins, int(targs[2]), *[float(x) for x in targs[3:11]],
                *[_ptr(x) for x in h], w.npart, _ptr(axis_h), _ptr(cofm_h), w.nlos, _ptr(tau_h),
                ctypes.byref(opt), eb, 512)
            _lib.raise_for(rc, eb.value.decode(errors="replace"))

        c_call()
        barrier(world)
        ck = ClockSampler(local).start()
        t0 = time.perf_counter()
        for _ in range(ke):
            c_call()
        dt = allreduce_max((time.perf_counter() - t0) / ke, world)
        dst = _lib.default_context_stats() or {}
        # (b) the Python drop-in: a new zeroed array per call, as the reference
        # returns, so each call also pays the first touch and the release of
        # 2.9 GB of host pages
        _Particle_Interpolate(*hargs, precision="fp32")
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(ke):
            tau_d = _Particle_Interpolate(*hargs, precision="fp32")
        dt_d = allreduce_max((time.perf_counter() - t0) / ke, world)
        e2e_clk = ck.stop()
        dst_d = _lib.default_context_stats() or {}
        same = bool(np.array_equal(tau_d, tau_h))
        del tau_d
        res["e2e"] = {"value": world * pixels / dt, "unit": "pixels/s",
                      "h2d_bytes_per_step": int(sum(x.nbytes for x in h)),
                      "d2h_bytes_per_step": int(tau_h.nbytes),
                      "ms_per_step": dt * 1e3,
                      "phases_ms_last_call": {k: dst.get(k) for k in ("ms_h2d", "ms_search",
                                                                      "ms_deposit", "ms_d2h")},
                      "api": "fsg_particle_interpolate (host pointers; inputs pinned, output a "
                             "pageable array the caller allocated once)",
                      "dropin": {"value": world * pixels / dt_d, "ms_per_step": dt_d * 1e3,
                                 "phases_ms_last_call": {
                                     k: dst_d.get(k) for k in ("ms_h2d", "ms_search",
                                                               "ms_deposit", "ms_d2h")},
                                 "api": "_spectra_priv._Particle_Interpolate (new output "
                                        "array per call)",
                                 "same_result": same},
                      "clocks": e2e_clk}

    # ---- plain FP64 form on a sightline subset, and the accuracy of FP32 against it
    if not args.no_fp64:
        lines = subset_lines(w.nlos, args.fp64_lines)
        o64 = torch.empty((len(lines), w.nbins), dtype=torch.float64, device="cuda")
        step("fp64", o=o64, lines=lines)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step("fp64", o=o64, lines=lines)
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        v64 = len(lines) * w.nbins / (ms64 * 1e-3)
        # FP32 on the same subset (same call shape) for a like-for-like ratio
        o32 = torch.empty_like(o64)
        step("fp32", o=o32, lines=lines)
        torch.cuda.synchronize()
        e0.record(stream)
        step("fp32", o=o32, lines=lines)
        e1.record(stream)
        torch.cuda.synchronize()
        ms32s = e0.elapsed_time(e1)
        t64 = o64.cpu().numpy()
        t32 = tau32[torch.from_numpy(lines).cuda()].cpu().numpy()
        dF = np.abs(np.exp(-t32) - np.exp(-t64))
        big = t64 >= 1e-3
        rel = np.abs(t32 - t64)[big] / t64[big] if big.any() else np.zeros(1)
        # column density, both forms
        cargs = list(w.call_args(lya, 0))
        cargs[16], cargs[17] = w.axis[lines], w.cofm[lines]
        c64 = interp.particle_interpolate_device(ctx, *cargs, precision="fp64").cpu().numpy()
        c32 = interp.particle_interpolate_device(ctx, *cargs, precision="fp32").cpu().numpy()
        nz = c64 != 0
        crel = np.abs(c32 - c64)[nz] / np.abs(c64[nz]) if nz.any() else np.zeros(1)
        res["fp64_plain"] = {"value": v64, "unit": "pixels/s", "ms_per_call": ms64,
                             "sightlines": int(len(lines)),
                             "fp32_same_subset": {"value": len(lines) * w.nbins / (ms32s * 1e-3),
                                                  "ms_per_call": ms32s},
                             "fp32_over_fp64": (len(lines) * w.nbins / (ms32s * 1e-3)) / v64}
        res["accuracy"] = {"max_abs_dF": float(dF.max()), "tau_rel_err_max": float(rel.max()),
                           "tau_rel_err_median": float(np.median(rel)),
                           "colden_rel_err_max": float(crel.max()),
                           "against": "plain FP64 form on the same %d sightlines" % len(lines)}

    # ---- batched form: every line of the workload (tau) plus the column densities, one call
    if not args.no_batch and len(w.transitions) > 1:
        blines = [(t, w.dens[t.species], True, t.name != "lyb") for t in w.transitions]

        def batch():
            return interp.spectra_batch_device(ctx, w.nbins, w.kernel, w.box, w.velfac, w.atime,
                                               w.tautail, w.pos, w.vel, w.temp, w.hh, w.axis,
                                               w.cofm, blines, precision="fp32")
        outs = batch()
        del outs
        torch.cuda.synchronize()
        nb = max(1, min(args.steps, 2))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(nb):
            outs = batch()
        e1.record(stream)
        torch.cuda.synchronize()
        msb = e0.elapsed_time(e1) / nb
        ntau = sum(1 for b in blines if b[2])
        ncol = sum(1 for b in blines if b[3])
        res["batched"] = {"ms_per_call": msb, "lines": [t.name for t in w.transitions],
                          "tau_arrays": ntau, "colden_arrays": ncol,
                          "tau_pixels_per_s": ntau * pixels / (msb * 1e-3),
                          "graph": "one CUDA graph of all deposits after one sightline search"}
        del outs

    # ---- weighted column densities: 5 channels fused against 5 single calls (FP32)
    if not args.no_extra:
        d = w.dens["HI"]
        chans = [d, d * w.vel[:, 0], d * w.vel[:, 1], d * w.vel[:, 2], d * w.temp]
        cargs = list(w.call_args(lya, 0))

        def fused():
            return interp.colden_channels_device(ctx, w.nbins, w.kernel, w.box, w.velfac, w.pos,
                                                 w.hh, w.axis, w.cofm, chans, precision="fp32")

        def singles():
            r = []
            for dc in chans:
                cargs[13] = dc
                r.append(interp.particle_interpolate_device(ctx, *cargs, precision="fp32"))
            return r
        timings = {}
        for name, fn in (("fused", fused), ("single_calls", singles)):
            outs = fn()
            del outs
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            outs = fn()
            e1.record(stream)
            torch.cuda.synchronize()
            timings[name] = e0.elapsed_time(e1)
            del outs
        del chans
        res["colden_channels"] = {"channels": 5, "ms_fused": timings["fused"],
                                  "ms_single_calls": timings["single_calls"],
                                  "weights": "dens x {1, v_x, v_y, v_z, T}",
                                  "form": "FP32, one search + one kernel vs 5 calls"}

        # ---- flux statistics of the FP32 tau still in HBM (HBM-bound reductions)
        from fake_spectra_gb300 import fluxstatistics as fstat
        hbm, hbm_src = measured_hbm_gbs()
        ntau = tau32.numel()

        def timed(fn):
            fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = fn()
            torch.cuda.synchronize()
            return r, (time.perf_counter() - t0) * 1e3
        fstat._context()
        scale, ms_mf = timed(lambda: fstat.mean_flux(tau32, 0.7))
        _, ms_pdf = timed(lambda: fstat.flux_pdf(tau32, 20, None))
        pdf_kernel_ms = fstat._context().stats()["ms_flux"]
        _, ms_pow = timed(lambda: fstat.flux_power(tau32, w.nbins * 1.0, 8, None, False))
        power_kernels_ms = fstat._context().stats()["ms_flux"]
        nspec, npix = tau32.shape
        # the usual flop count of a complex transform of length n, 5 n log2 n,
        # per pair of sightlines
        fft_flops = 5.0 * npix * math.log2(npix) * ((nspec + 1) // 2)
        res["flux_statistics"] = {
            "tau_pixels": ntau, "mean_flux_ms": ms_mf, "scale": scale,
            "flux_pdf_ms": ms_pdf, "flux_power_ms": ms_pow,
            "pdf_kernel_ms": pdf_kernel_ms,
            "pdf_kernel_hbm_frac": (ntau * 8 / (pdf_kernel_ms * 1e-3) / 1e9) / hbm,
            "power_kernels_ms": power_kernels_ms,
            "power_fft_gflops": fft_flops / (power_kernels_ms * 1e-3) / 1e9,
            "hbm_peak_gbs": hbm, "hbm_peak_source": hbm_src,
            "note": "wall time of each call (host API, tau resident in HBM); pdf_kernel_ms is "
                    "the histogram kernel's device time (8 B of tau per pixel, read once); "
                    "power_kernels_ms the device time of the power's own kernels (pack with "
                    "the FP64 exponentials, transform passes, ordered power sums), without "
                    "the mean-flux pass that flux_power_ms includes; power_fft_gflops counts "
                    "5 n log2 n flops per complex transform of a sightline pair"}

    # ---- differentiation form: forward and forward+backward on the 128^3 workload
    if not args.no_bwd:
        from fake_spectra_gb300.autograd import particle_tau
        w4 = synth.generate_torch(4, device="cuda")
        w4t = synth.generate_torch(4, seed=5, device="cuda")
        t4 = synth.LYA
        a4 = lambda wk: (wk.nbins, wk.kernel, wk.box, wk.velfac, wk.atime, t4.lambda_cm,
                         t4.gamma, t4.fosc, t4.amumass, wk.tautail)
        ftarget = torch.exp(-interp.particle_interpolate_device(
            ctx, *w4t.call_args(t4, 1)[:11], w4t.pos, w4t.vel, w4t.dens["HI"], w4t.temp,
            w4t.hh, w4t.axis, w4t.cofm, precision="fp32"))
        dens4 = w4.dens["HI"].clone().requires_grad_(True)
        temp4 = w4.temp.clone().requires_grad_(True)
        vel4 = w4.vel.clone().requires_grad_(True)

        def fwd():
            return particle_tau(ctx, *a4(w4), w4.pos, vel4, dens4, temp4, w4.hh, w4.axis,
                                w4.cofm)

        def fwd_bwd():
            tau = fwd()
            loss = ((torch.exp(-tau) - ftarget) ** 2).sum()
            loss.backward()
            return loss

        for _ in range(2):
            fwd_bwd()
        nr = max(3, args.steps)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.no_grad():
            e0.record(stream)
            for _ in range(nr):
                fwd()
            e1.record(stream)
        torch.cuda.synchronize()
        msf = e0.elapsed_time(e1) / nr
        e0.record(stream)
        for _ in range(nr):
            fwd_bwd()
        e1.record(stream)
        torch.cuda.synchronize()
        msfb = e0.elapsed_time(e1) / nr
        res["fwd_bwd"] = {"workload": w4.name, "particles": w4.npart, "sightlines": w4.nlos,
                          "nbins": w4.nbins, "fwd_ms": msf, "fwd_bwd_ms": msfb,
                          "ratio": msfb / msf,
                          "loss": "sum (exp(-tau) - F_target)^2, F_target from seed 5",
                          "grads": "dens, temp, v_los (FP32 backward kernel)"}
        del w4, w4t, dens4, temp4, vel4, ftarget

    # ---- CPU baseline: the oracle on a stratified sample of the same workload, and
    # the accuracy of both GPU forms against the oracle's output on those sightlines
    if not args.no_cpu and rank == 0 and world == 1:
        import oracle
        wh = w.to_host()
        threads = os.cpu_count() or 1
        port = oracle.port()
        port.set_threads(threads)
        strata = strata_of(w)
        keys = sorted(strata)
        picks = stratified_picks(strata, args.cpu_per_stratum, seed=777)
        lines = np.concatenate([picks[k] for k in keys])
        est = CpuEstimate(w, strata, threads)
        est.t_search_full, est.npairs_full = port.search_seconds(wh.pos, wh.hh, wh.axis,
                                                                 wh.cofm, wh.box)
        t0 = time.perf_counter()
        want, t_s, sec = oracle_lines(port, wh, lya, 1, lines, timed=True)
        wall = time.perf_counter() - t0
        est.add([k for k in keys for _ in picks[k]], sec)
        v = est.value()
        res["cpu_baseline"] = {
            "value": v, "unit": "pixels/s", "cores": threads, "kind": "port",
            "sample": "CPU oracle (C restatement, OpenMP, %d threads) on a stratified sample of "
                      "%d of %d sightlines (%d per stratum of axis x clump-centred or not, seed "
                      "777) with all %d particles: %.1f s wall (%.3g px/s on the sample itself); "
                      "the search over all sightlines %.1f s" % (
                          threads, len(lines), w.nlos, args.cpu_per_stratum, w.npart, wall,
                          len(lines) * w.nbins / wall, est.t_search_full),
            "estimate": est.describe(777)}
        # accuracy of the GPU forms against the oracle on the sampled sightlines
        rows = torch.from_numpy(lines).cuda()
        g32 = tau32[rows].cpu().numpy()
        o64 = torch.empty((len(lines), w.nbins), dtype=torch.float64, device="cuda")
        g64 = step("fp64", o=o64, lines=lines).cpu().numpy()
        want_c = oracle_lines(port, wh, lya, 0, lines)
        cargs = list(w.call_args(lya, 0))
        cargs[16], cargs[17] = w.axis[lines], w.cofm[lines]
        c32 = interp.particle_interpolate_device(ctx, *cargs, precision="fp32").cpu().numpy()
        c64 = interp.particle_interpolate_device(ctx, *cargs, precision="fp64").cpu().numpy()
        res.setdefault("accuracy", {})["vs_oracle"] = {
            "sightlines": int(len(lines)),
            "sample": "the CPU baseline's stratified sample (seed 777)",
            "fp32": {**accuracy_stats(g32, want, 1), **accuracy_stats(c32, want_c, 0),
                     "from": "the timed full-size FP32 call (all sightlines)"},
            "fp64": {**accuracy_stats(g64, want, 1), **accuracy_stats(c64, want_c, 0),
                     "from": "an FP64 call on the sampled sightlines"}}
        del o64, rows

    # ---- 256^3 workload with three lines: per line, both GPU forms against the oracle
    if not args.no_config2 and not args.no_cpu and rank == 0 and world == 1:
        res["config2_per_line"] = config2_report(ctx, interp, synth)

    # ---- 256^3 workload (60 x 60 grid along axis 3): cubic spline and top hat
    if not args.no_tophat and rank == 0 and world == 1:
        res["config1_kernels"] = config1_kernels(ctx, interp, synth, stream,
                                                 with_cpu=not args.no_cpu)
    if rank == 0:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
