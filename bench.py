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
# dram__bytes_write.sum, kept with the profile summaries): 2.372797 GB read for
# 5038719 pairs, 0.174416896 GB written for 2048 x 11152 pixels; scaled to a
# launch by pairs (reads) and output pixels (writes).
TRAFFIC_READ_PER_PAIR = 2.372797e9 / 5038719
TRAFFIC_WRITE_PER_PIXEL = 0.174416896e9 / (2048 * 11152)
FLOPS_FP64 = {"core": 214, "wing": 144, "other": 20}


def measured_hbm_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f).get("hbm_gbs"))
    except Exception:
        return None


def search_roofline(npart, npairs, nlos, ms):
    """HBM view of the sightline search (particle sort + count + emit): the
    algorithmic bytes are the particle stream and the pair lists.  Sort: read
    pos (12 B), write the cell key (4 B), read the key and write the order
    (8 B); count and emit: read the order (4 B), pos (12 B) and h (4 B) each;
    emit: write 12 B per pair; offsets 8 B per sightline."""
    algo = npart * (12 + 4 + 8 + 2 * (4 + 12 + 4)) + npairs * 12 + nlos * 8
    hbm = measured_hbm_gbs()
    achieved = algo / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm if hbm else None, "bytes": algo,
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
    p.add_argument("--cpu-lines", type=int, default=16,
                   help="sightlines in the CPU baseline sample")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--no-bwd", action="store_true")
    p.add_argument("--no-extra", action="store_true",
                   help="skip the multi-channel column density and flux statistics sections")
    return p.parse_args()


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


def cpu_sample(w_host, lines, threads):
    """Time the CPU oracle on a subset of sightlines; returns (pixels/s, seconds)."""
    import oracle
    port = oracle.port()
    port.set_threads(threads)
    from fake_spectra_gb300 import synth
    args = list(w_host.call_args(synth.LYA, 1))
    args[16] = w_host.axis[lines]
    args[17] = w_host.cofm[lines]
    t0 = time.perf_counter()
    port.particle_interpolate(*args)
    dt = time.perf_counter() - t0
    return len(lines) * w_host.nbins / dt, dt


def run_reference(args):
    rank, world, local = dist_setup()
    if rank != 0:
        return
    import torch
    from fake_spectra_gb300 import synth  # noqa: F401
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    w = make_workload(args, dev).to_host()
    threads = os.cpu_count() or 1
    lines = subset_lines(w.nlos, args.cpu_lines)
    for _ in range(args.warmup):
        cpu_sample(w, lines[:max(1, len(lines) // 4)], threads)
    vals, secs = [], []
    for _ in range(args.steps):
        v, s = cpu_sample(w, lines, threads)
        vals.append(v)
        secs.append(s)
    value = len(lines) * w.nbins * len(secs) / sum(secs)
    sample = ("CPU oracle (C restatement of the reference path, OpenMP) on %d of %d sightlines "
              "with all %d particles, per step" % (len(lines), w.nlos, w.npart))
    print(json.dumps({
        "impl": "reference", "metric": HEADLINE_METRIC, "value": value, "unit": "pixels/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(secs) / len(secs), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w.name, "particles": w.npart, "sightlines": w.nlos,
                   "nbins": w.nbins, "line": "Ly-a 1215.67 A", "kernel": "cubic spline"},
        "cpu_baseline": {"value": value, "unit": "pixels/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "pixels/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }))


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
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

    def step(precision, o=out, lines=None, count=False):
        a = list(targs)
        if lines is not None:
            a[16] = w.axis[lines]
            a[17] = w.cofm[lines]
        return interp.particle_interpolate_device(ctx, *a, out=o, precision=precision,
                                                  count_work=count)

    # ---- tuned FP32 form: the timed region
    for _ in range(args.warmup):
        step("fp32")
    stream = torch.cuda.current_stream()
    launches0 = ctx.stats()["gpu_launches"]
    clocks = ClockSampler(local).start()
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    dep_ms, search_ms = [], []
    for _ in range(args.steps):
        step("fp32")
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
        same = bool(np.array_equal(tau_d, tau_h))
        del tau_d
        res["e2e"] = {"value": world * pixels / dt, "unit": "pixels/s",
                      "h2d_bytes_per_step": int(sum(x.nbytes for x in h)),
                      "d2h_bytes_per_step": int(tau_h.nbytes),
                      "ms_per_step": dt * 1e3,
                      "api": "fsg_particle_interpolate (host pointers; inputs pinned, output a "
                             "pageable array the caller allocated once)",
                      "dropin": {"value": world * pixels / dt_d, "ms_per_step": dt_d * 1e3,
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
        hbm = measured_hbm_gbs()
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
        _, ms_pow = timed(lambda: fstat.flux_power(tau32, w.nbins * 1.0, 8, None, False))
        res["flux_statistics"] = {
            "tau_pixels": ntau, "mean_flux_ms": ms_mf, "scale": scale,
            "flux_pdf_ms": ms_pdf, "flux_power_ms": ms_pow,
            "pdf_hbm_frac": (ntau * 8 / (ms_pdf * 1e-3) / 1e9) / hbm if hbm else None,
            "note": "wall time of each call (host API, tau resident in HBM); the PDF pass reads "
                    "8 B per pixel once, against the measured HBM copy bandwidth"}

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

    # ---- CPU baseline: the oracle on a bounded sample of the same workload
    if not args.no_cpu and rank == 0 and world == 1:
        wh = w.to_host()
        threads = os.cpu_count() or 1
        lines = subset_lines(w.nlos, args.cpu_lines, seed=777)
        v, s = cpu_sample(wh, lines, threads)
        res["cpu_baseline"] = {"value": v, "unit": "pixels/s", "cores": threads, "kind": "port",
                               "sample": "CPU oracle (C restatement, OpenMP) on %d random of %d "
                                         "sightlines with all %d particles: %.1f s"
                                         % (len(lines), w.nlos, w.npart, s)}
    if rank == 0:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
