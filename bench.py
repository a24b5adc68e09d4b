#!/usr/bin/env python3
"""Benchmark: batched odd-even Kalman smoothing on GB300 (smoothed steps/s).

Workload: 4,096 independent constant-velocity tracks (n=6 [pos; vel], m=3,
dt=0.1, process noise diag(1e-2), observation noise diag(1e-1), prior N(0, I)
folded into a square step-0 observation), lengths floor(exp(U[ln 100,
ln 20000])) from a fixed seed -- 15.1 million steps, 23.3 GB of FP64
equations (larger than the 126 MB L2, so nothing is re-read from cache
between timed steps).  Data is synthetic (seeded NumPy).

One "step" of the benchmark = one odd-even smoothing of every track through
the library's C ABI.  The headline is the precision form: FP32 factorization
with FP64-residual refinement of the smoothed states (KALMAN_GPU_FP32_REFINE),
whose error against the plain FP64 path is measured in the same run and must
be <= 1e-9; the plain FP64 path (states, and states + covariances) is timed
beside it.
  value -- inputs resident in HBM, kalman_gpu_smooth_oddeven_packed on device
           arrays (CUDA events on the launching stream, synchronized);
  e2e   -- the same call handed page-locked HOST arrays: host->device copy of
           the equations, smoothing, device->host copy of the states inside
           the timed region.
Other keys: per-kernel roofline, p50/p99 per-smoothing latency, the CPU
baseline (the oracle's C restatement of the reference smoother, states only as
the headline computes, on all host cores, a bounded sample of the same
tracks), clocks.

--impl reference: times the CPU restatement of the reference's odd-even
smoother (oracle/kalman_oracle.c, OpenMP over tracks, FP64, states only) on a
bounded sample of the same workload, per step, with all host threads.

Multi-GPU (torchrun): every rank smooths its own 4,096 tracks (different
seed); no collective on the data path (replicas); value = all ranks' steps /
max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "smoothed steps/s (batched odd-even), FP32 factorization + FP64-residual refinement vs plain FP64, at <=1e-9 rel err"
UNIT = "steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--tracks", type=int, default=4096)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the library's default tuning")
    ap.add_argument("--no-large", action="store_true", help="skip the n=128 large-state line")
    ap.add_argument("--fp32-only", action="store_true",
                    help="time the precision form only (no plain FP64 pass, probes, e2e or CPU leg): profiling runs")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--sweeps", type=int, default=1,
                    help="refinement sweeps (one meets the 1e-9 bar with margin; 0: the library default, two)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(tracks, rank):
    from ultimate_kalman_gb300 import problem as pb
    lengths = pb.batched_lengths(tracks, 100, 20000, seed=0)
    return pb.constant_velocity(lengths, seed=1000 + rank)


def config_dict(P, tracks, world):
    return {"workload": "batched constant-velocity tracks, odd-even smoother, smoothed states",
            "tracks_per_gpu": tracks, "steps_per_gpu": int(P.nsteps), "n": 6, "m": 3,
            "track_lengths": "floor(exp(U[ln 100, ln 20000]))",
            "precision": "FP32 factorization + FP64-residual refinement (plain FP64 timed beside it)",
            "l2": "inputs (23 GB/GPU) exceed L2; no flush needed", "parallelism": f"replicas x{world}"}


class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_sample(P, seconds, threads=0, algorithm="oddeven", covariance=False):
    """Times the oracle's restatement on the first tracks of P, grown until the
    sample takes about `seconds`; returns (steps/s, steps, tracks, threads,
    seconds, states of the sample)."""
    import oracle
    nt = threads or oracle.max_threads()
    ntr = 8
    while True:
        S = P.select_tracks(range(min(ntr, P.ntracks)))
        t0 = time.perf_counter()
        _, X, _ = oracle.smooth(S, algorithm, covariance=covariance, threads=nt)
        dt = time.perf_counter() - t0
        if dt >= seconds * 0.6 or ntr >= P.ntracks:
            return S.nsteps / dt, S.nsteps, S.ntracks, nt, dt, X
        ntr = min(P.ntracks, max(ntr * 2, int(ntr * seconds / max(dt, 1e-3))))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build()
    P = workload(args.tracks, 0)
    budget = max(1.0, 150.0 / max(1, args.steps + args.warmup))
    # choose the sample once, then time each step on it
    _, _, ntr, nt, _, _ = cpu_sample(P, budget)
    S = P.select_tracks(range(ntr))
    for _ in range(args.warmup):
        oracle.smooth(S, "oddeven", covariance=False, threads=nt)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.smooth(S, "oddeven", covariance=False, threads=nt)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.mean(times))
    v = S.nsteps / (ms * 1e-3)
    sample = f"first {ntr} of {P.ntracks} tracks ({S.nsteps} steps) per step, FP64 odd-even, states only"
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(P, args.tracks, world),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nt, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_smooths(D, steps, stream, **kw):
    """Times `steps` smoothings, each bracketed by CUDA events on `stream`;
    returns (mean ms, per-smoothing ms list)."""
    import torch
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    torch.cuda.synchronize()
    evs[0].record(stream)
    for i in range(steps):
        D.smooth("oddeven", stream=stream, **kw)
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    per = [evs[i].elapsed_time(evs[i + 1]) for i in range(steps)]
    return evs[0].elapsed_time(evs[-1]) / steps, per


def time_plan(plan, steps, stream):
    """Times `steps` replays of a plan's CUDA graph, each bracketed by CUDA
    events on `stream`; returns (mean ms, per-replay ms list)."""
    import torch
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    torch.cuda.synchronize()
    evs[0].record(stream)
    for i in range(steps):
        plan.execute(stream)
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    per = [evs[i].elapsed_time(evs[i + 1]) for i in range(steps)]
    return evs[0].elapsed_time(evs[-1]) / steps, per


def roofline_for(prof, fl, steps, fp64_peak, fp32_peak, hbm_peak, compulsory_in, traffic_model):
    """Roofline of the kernel category with the largest time.

    Algorithmic bytes are the problem's compulsory bytes (every step's
    equations read once at their real sizes, flops.compulsory_bytes): they are
    credited to the kernel that reads the caller's equations (the weighing
    kernel); the other kernels move only intermediates, whose modelled bytes
    are reported as traffic, not as algorithmic work, and are placed against
    their pipe with the flops of the model (flops.py: FP32 kernels against the
    FP32 FMA peak, FP64 kernels against the FP64 one).  A kernel goes against
    whichever of HBM and its pipe it is nearer to."""
    top = max(prof, key=lambda k: prof[k][0])
    kms, kl = prof[top]
    secs = kms * 1e-3 / steps
    flops = fl.get(top, 0.0)
    is32 = top.startswith("fp32") or top.startswith("refine") or top not in fl
    peak_f = fp32_peak if is32 else fp64_peak
    ach_f = flops / secs / 1e12
    alg = compulsory_in if top == "weigh_kernel" else 0.0
    ach_b = alg / secs / 1e9
    frac_f, frac_b = ach_f / peak_f, ach_b / hbm_peak
    if frac_b >= frac_f:
        r = {"bound": "hbm", "achieved": ach_b, "peak": hbm_peak, "unit": "GB/s", "frac": frac_b,
             "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
             "algorithmic_bytes_per_launch": alg / max(1.0, kl / steps)}
    else:
        r = {"bound": "fp32" if is32 else "fp64", "achieved": ach_f, "peak": peak_f, "unit": "TFLOP/s",
             "frac": frac_f, "peak_source": "FMA-chain probe kernel timed in this run (of measured)"}
    r.update({"kernel": top, "traffic": None, "ms_per_step": kms / steps, "launches_per_step": kl / steps,
              "fp_tflops": ach_f, "fp_frac": frac_f, "modelled_traffic_bytes": traffic_model.get(top),
              "flops_model": "ultimate_kalman_gb300/flops.py (FMA = 2 flops)",
              "bytes_model": "flops.compulsory_bytes: F, H, K, c, G, o, C at real sizes in; states out"})
    return r


def whole_step(compulsory, ms, hbm_peak):
    """The whole smoothing against HBM: compulsory bytes in + out over the
    time of one smoothing."""
    b = compulsory[0] + compulsory[1]
    gbs = b / (ms * 1e-3) / 1e9
    return {"algorithmic_bytes": b, "ms": ms, "achieved_gbs": gbs, "frac": gbs / hbm_peak,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}


def rel_states(X, Xref):
    """max over steps of ||x - xref||_inf / ||xref||_inf (torch or numpy)."""
    if hasattr(X, "abs"):
        num = (X - Xref).abs().reshape(len(X), -1).amax(dim=1)
        den = Xref.abs().reshape(len(X), -1).amax(dim=1)
        return float((num / den).max().item())
    num = np.abs(X - Xref).reshape(len(X), -1).max(axis=1)
    den = np.abs(Xref).reshape(len(X), -1).max(axis=1)
    return float((num / den).max())


def time_call(fn, reps, stream):
    """Mean ms of `reps` calls of fn() bracketed by CUDA events on `stream`."""
    import torch
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record(stream)
    for _ in range(reps):
        fn()
    e.record(stream)
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def run_gpu(args):
    import torch
    from ultimate_kalman_gb300 import autotune, build, flops, native
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build()
    native.load()
    P = workload(args.tracks, rank)
    D = native.DeviceProblem(P, covariance=True)
    fp32 = dict(covariance=False, fp32_refine=True, sweeps=args.sweeps)
    stream = torch.cuda.current_stream()
    # the autotuner picks the work mapping and block shapes for this class (about a second here)
    tuned = autotune.tune(D, fp32_refine=True, covariance=False, sweeps=args.sweeps, reps=3, stream=stream,
                          save=False) if not args.no_tune else None
    # kernels and per-kernel times of one smoothing by direct calls (also the warm-up)
    for _ in range(args.warmup):
        D.smooth("oddeven", **fp32)
    prof_steps = max(3, args.steps // 2)
    native.profile_enable(True)
    launches0 = native.launch_count()
    ms_direct, _ = time_smooths(D, prof_steps, stream, **fp32)
    launches_per = (native.launch_count() - launches0) / prof_steps
    prof = native.profile_read()
    native.profile_enable(False)
    # the timed steps: the smoothing captured once into a CUDA graph (kalman_gpu_plan_*) and replayed
    plan = D.plan("oddeven", **fp32)
    for _ in range(args.warmup):
        plan.execute(stream)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    sampler = ClockSampler(local)
    time.sleep(0.5)  # let the sampler start before the timed region
    barrier()
    ms, per = time_plan(plan, args.steps, stream)
    barrier()
    clocks = sampler.stop()
    if plan.status() != 0:
        raise RuntimeError("the plan's smoothing reported %s" % (native.last_error(),))
    plan.close()
    del plan
    launches = int(round(launches_per * args.steps))
    X32 = D.state.clone()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    total_steps = P.nsteps * world
    value = total_steps / (ms * 1e-3)
    if args.fp32_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": ms, "note": "--fp32-only profiling run",
                              "config": config_dict(P, args.tracks, world), "gpu_launches": int(launches)}), flush=True)
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # the plain FP64 path (states + covariances, and states only) and the precision form with
    # covariances (double-float), each under its own tuning
    k2 = max(2, args.steps // 2)
    tunings = {"fp32_refine_states": tuned}
    for name, kw in (("fp64_states_and_covariances", dict(covariance=True)),
                     ("fp64_states", dict(covariance=False)),
                     ("fp32_refine_states_and_covariances", dict(covariance=True, fp32_refine=True))):
        tunings[name] = autotune.tune(D, reps=2, stream=stream, save=False, **kw) if not args.no_tune else None
        D.smooth("oddeven", **kw)
        if name == "fp64_states_and_covariances":
            native.profile_enable(True)
            ms64c, _ = time_smooths(D, k2, stream, **kw)
            prof64 = native.profile_read()
            native.profile_enable(False)
            S64 = D.cov.clone()
            X64c = D.state.clone()
        elif name == "fp64_states":
            ms64, _ = time_smooths(D, k2, stream, **kw)
        else:
            native.profile_enable(True)
            msdd, _ = time_smooths(D, k2, stream, **kw)
            profdd = native.profile_read()
            native.profile_enable(False)
            err_dd = {"states": rel_states(D.state, X64c), "covariances": rel_states(D.cov, S64)}
            del S64
    native.set_tuning(default=True)
    X64 = X64c
    err = float(((X32 - X64).abs().amax(dim=1) / X64.abs().amax(dim=1)).max().item())

    peak64 = native.measure_fp64_tflops(32)
    peak32 = native.measure_fp32_tflops()
    peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(REPO, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
    # FP32 kernels against the FP32 FMA peak by the model's flops; the weighing (double-float
    # arithmetic on the FP32 pipe, reading the caller's equations) against HBM by the compulsory bytes
    fl32 = flops.plan_flops_fast_fp32(P.track_lengths(), 6, 3, sweeps=args.sweeps or 2)
    fl32.pop("weigh_kernel")
    fl64 = flops.plan_flops_fast(P.track_lengths(), 6, 3, covariance=True)
    by32 = flops.plan_bytes_fast(P.track_lengths(), 6, 3, fp32=True, sweeps=args.sweeps or 2)
    by64 = flops.plan_bytes_fast(P.track_lengths(), 6, 3, fp32=False)
    comp = flops.compulsory_bytes(P.track_lengths(), 6, 3, covariance=False)
    comp_cov = flops.compulsory_bytes(P.track_lengths(), 6, 3, covariance=True)
    roof = roofline_for(prof, fl32, prof_steps, peak64, peak32, peaks["hbm_gbs"], comp[0], by32)
    # the weighing kernel, which reads the caller's equations, against the compulsory bytes
    # (the same object as `roofline` when the weighing is the longest kernel)
    roof_w = roofline_for({k: v for k, v in prof.items() if k == "weigh_kernel"}, fl32, prof_steps, peak64, peak32,
                          peaks["hbm_gbs"], comp[0], by32) if "weigh_kernel" in prof else None
    tfile = os.path.join(REPO, "profiles", "traffic_per_launch.json")
    if os.path.exists(tfile):
        traffic = json.load(open(tfile))
        roof["traffic"] = traffic.get(roof["kernel"])
        if roof_w:
            roof_w["traffic"] = traffic.get("weigh_kernel")
    roof["per_kernel"] = {k: {"ms_per_step": v[0] / prof_steps, "launches_per_step": v[1] / prof_steps,
                              "share": v[0] / sum(x[0] for x in prof.values())} for k, v in prof.items()}
    roof64 = roofline_for(prof64, fl64, k2, peak64, peak32, peaks["hbm_gbs"], comp_cov[0], by64)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 factorization + double-float (f32 pair, ~47-bit) residual refinement; f64 in and out", "data": "synthetic",
            "config": config_dict(P, args.tracks, world), "gpu_launches": int(launches),
            "latency_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99)),
                           "what": "one smoothing of all 4,096 tracks"},
            "rel_err_vs_fp64": err, "roofline": roof, "roofline_weighing": roof_w,
            "whole_step": whole_step(comp, ms, peaks["hbm_gbs"]),
            "clocks": clocks,
            "plain_fp64": {"states_and_covariances": total_steps / (ms64c * 1e-3),
                           "states_only": total_steps / (ms64 * 1e-3), "unit": UNIT,
                           "speedup_fp32_refine_vs_fp64_states_only": ms64 / ms, "roofline": roof64},
            "precision_form_with_covariances": {
                "value": total_steps / (msdd * 1e-3), "unit": UNIT, "ms_per_step": msdd,
                "form": "double-float (FP32 pairs, ~47 bits) factorization and covariance recurrence",
                "rel_err_vs_fp64": err_dd, "speedup_vs_fp64_states_and_covariances": ms64c / msdd,
                "per_kernel_ms": {k: v[0] / k2 for k, v in profdd.items()}},
            "execution": {"timed": "kalman_gpu_plan_execute: the smoothing captured once into a CUDA graph",
                          "plan_graph_ms": ms, "direct_call_ms": ms_direct,
                          "kernels_per_smoothing": launches_per},
            "tuning": {k: ({"tuning": v["tuning"], "ms": v["ms"], "default_ms": v["default_ms"],
                            "trials": len(v["table"])} if v else None) for k, v in tunings.items()},
            "peaks": {"fp64_tflops": peak64, "fp32_tflops": peak32, "hbm_gbs": peaks["hbm_gbs"]}}

    # filtered estimates of the same tracks (the sequential filter, tracks in parallel)
    if rank == 0 and world == 1 and not args.no_large:
        line["filter"] = filter_line(D, P, stream)

    # end to end through the C ABI with page-locked host buffers
    if not args.no_e2e:
        del D
        torch.cuda.empty_cache()
        (pin, st_h), pin_node = numa_local(lambda: (
            {f: torch.from_numpy(np.ascontiguousarray(getattr(P, f))).pin_memory() for f in native._FIELDS},
            torch.empty((P.nsteps, 6), dtype=torch.float64).pin_memory()))
        s = native.host_struct_from_tensors(P, pin, st_h, None)
        native.smooth_struct("oddeven", s, **fp32)  # warm-up (device staging allocated)
        times = []
        for _ in range(args.e2e_steps):
            barrier()
            t0 = time.perf_counter()
            native.smooth_struct("oddeven", s, **fp32)
            times.append(time.perf_counter() - t0)
        e2e_ms = 1e3 * float(np.median(times))
        h2d = sum(t.numel() * t.element_size() for t in pin.values())
        link = h2d_probe()
        padded = {"value": total_steps / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                       "d2h_bytes_per_step": int(st_h.numel() * 8), "ms_per_step": e2e_ms,
                       "path": "kalman_gpu_smooth_oddeven_packed, KALMAN_GPU_HOST arrays (every step stored with the "
                               "first step's 6 observation rows), FP32 + refinement",
                       "host_link": link, "h2d_share_at_probe_bandwidth": h2d / (link["h2d_gbs"] * 1e9) / (e2e_ms * 1e-3),
                       "pinned_buffers_numa_node": pin_node,
                       "all_times_ms": [1e3 * t for t in times]}
        del pin, st_h, s
        line["e2e"] = first_obs_e2e(P, X32, fp32, args.e2e_steps, barrier)
        line["e2e"]["packed_layout"] = padded
        if rank == 0 and world == 1:
            line["e2e"]["reference_api"] = secondary(lambda: struct_e2e(P, X32, fp32, args.e2e_steps))

    if rank == 0 and world == 1 and not args.no_cpu:
        v, nsteps, ntr, nt, dt, Xo = cpu_sample(P, args.cpu_seconds)
        Xg = X32[:nsteps].cpu().numpy()
        err_o = float((np.abs(Xg - Xo).max(axis=1) / np.abs(Xo).max(axis=1)).max())
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nt, "kind": "port",
                                "sample": f"first {ntr} of {P.ntracks} tracks ({nsteps} steps), {dt:.1f} s, "
                                          f"oracle/kalman_oracle.c odd-even, FP64, states only, OpenMP over tracks",
                                "rel_err_of_gpu_states_on_sample": err_o}
    if rank == 0 and world == 1 and not args.no_large:
        torch.cuda.empty_cache()
        for key, fn in (("large_state", lambda: large_state(stream)), ("builder", builder_line),
                        ("config0", lambda: config0_line(stream, not args.no_cpu)),
                        ("config1", lambda: config1_line(stream, not args.no_cpu)), ("serving", serving_line)):
            native.release()
            line[key] = secondary(fn)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def first_obs_e2e(P, X32, kw, reps, barrier):
    """End to end with host arrays through kalman_gpu_smooth_oddeven_first_obs:
    the same equations with every step stored at its own observation rows and
    each track's first observation (the folded prior, 6 rows) in per-track
    arrays -- no padding crosses the host link; the library pads on the
    device.  Page-locked host arrays, host wall clock per call, copies in and
    states out inside the timed region."""
    import ctypes
    import torch
    from ultimate_kalman_gb300 import native, problem as pb
    Pc, F0 = pb.split_first_obs(P)
    (pin, f0p, st_h), node = numa_local(lambda: (
        {f: torch.from_numpy(np.ascontiguousarray(getattr(Pc, f))).pin_memory() for f in native._FIELDS},
        {k: torch.from_numpy(np.ascontiguousarray(F0[k])).pin_memory() for k in native.FIRST_OBS_FIELDS},
        torch.empty((P.nsteps, P.n), dtype=torch.float64).pin_memory()))
    s = native.host_struct_from_tensors(Pc, pin, st_h, None)
    f = native.first_obs_struct(F0, f0p)
    L = native.load()
    opts = native.options_for("oddeven", **kw)
    call = lambda: native._check(L.kalman_gpu_smooth_oddeven_first_obs(opts, ctypes.byref(s), ctypes.byref(f), None))
    call()  # warm-up: device staging allocated
    times = []
    for _ in range(reps):
        barrier()
        t0 = time.perf_counter()
        call()
        times.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.median(times))
    h2d = sum(t.numel() * t.element_size() for t in pin.values()) + sum(t.numel() * t.element_size()
                                                                        for t in f0p.values())
    err = rel_states(st_h.numpy(), X32.cpu().numpy())
    link = h2d_probe()
    out = {"value": P.nsteps / (ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(st_h.numel() * 8), "ms_per_step": ms, "all_times_ms": [1e3 * t for t in times],
           "path": "kalman_gpu_smooth_oddeven_first_obs, KALMAN_GPU_HOST arrays: steps at their own 3 observation "
                   "rows, each track's folded-prior first observation apart; FP32 + refinement",
           "rel_err_vs_device_path": err, "host_link": link, "pinned_buffers_numa_node": node,
           "h2d_share_at_probe_bandwidth": h2d / (link["h2d_gbs"] * 1e9) / (ms * 1e-3)}
    del pin, f0p, st_h, s
    native.release()
    return out


def struct_e2e(P, X32, kw, reps):
    """End to end through the reference's own calling convention: one
    kalman_step_equations_t per step, its matrices pointing at the caller's
    host data, smoothed by the batched form of kalman_smooth_oddeven
    (kalman_gpu_smooth_tracks): the library packs the structs into page-locked
    staging, copies, smooths, copies back and gives every step its own state
    matrix (the reference's result contract).  Host wall clock per call."""
    from ultimate_kalman_gb300 import native
    t0 = time.perf_counter()
    V = native.EquationsView(P)
    build_s = time.perf_counter() - t0
    st = V.smooth_tracks("oddeven", **kw)  # warm-up: page-locked staging allocated
    if st != 0:
        raise RuntimeError(str(native.last_error()))
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        st = V.smooth_tracks("oddeven", **kw)
        times.append(time.perf_counter() - t0)
        if st != 0:
            raise RuntimeError(str(native.last_error()))
    ms = 1e3 * float(np.median(times))
    sample = np.linspace(0, P.nsteps - 1, 2000).astype(np.int64)
    err = rel_states(V.states(sample), X32[sample].cpu().numpy())
    native.release()  # the page-locked staging of this thread
    return {"value": P.nsteps / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "all_times_ms": [1e3 * t for t in times],
            "path": "kalman_gpu_smooth_tracks on one kalman_step_equations_t per step (host matrices, results "
                    "returned as one state matrix per step), FP32 + refinement",
            "structs_built_s": build_s, "rel_err_vs_device_path_on_2000_steps": err}


def filter_line(D, P, stream):
    """Filtered estimates x_{s|s} of every step of the workload's tracks
    (kalman_gpu_filter_packed), states only, one timed call after a warm-up."""
    import torch
    D.filter(covariance=False, stream=stream)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    D.filter(covariance=False, stream=stream)
    e.record(stream)
    torch.cuda.synchronize()
    ms = s.elapsed_time(e)
    return {"what": "filtered estimates of every step of the same tracks (sequential filter per track, tracks "
                    "in parallel), states, FP64", "ms": ms, "steps_per_s": P.nsteps / (ms * 1e-3)}


def builder_line():
    """The device-side equation builder on one time-invariant n=24, m=12 track
    of 200,000 steps (4.7 GB of packed equations written), 10 timed builds."""
    import torch
    from ultimate_kalman_gb300 import shapes
    D, build = shapes.device_track(200000, 24, 12, covariance=False, with_builder=True)
    for _ in range(3):
        build()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(10):
        build()
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / 10
    out = {"what": "kalman_gpu_expand_invariant, n=24, m=12, k=200000 (packed per-step arrays written)",
           "ms": ms, "written_gb": D.input_bytes() / 1e9, "write_gbs": D.input_bytes() / (ms * 1e-3) / 1e9}
    del D, build
    torch.cuda.empty_cache()
    return out


def large_state(stream):
    """The large-state shape beside the headline: one n=128, m=64, k=20,000
    track (F = 0.995 Q, G ~ N(0, 1/m), noise covariance eigenvalues
    log-uniform in [1e-3, 1], 5 % of steps unobserved), odd-even smoother,
    states: the precision form (FP32 blocked QR + one FP64-residual sweep)
    and plain FP64."""
    import torch
    from ultimate_kalman_gb300 import native, shapes
    P = shapes.synthetic_track(20000, 128, 64, rho=0.995, lo=1e-3, log_cov=True)
    D = native.DeviceProblem(P, covariance=False)
    kw32 = dict(covariance=False, fp32_refine=True, sweeps=1)
    D.smooth("oddeven", **kw32)
    ms32, _ = time_smooths(D, 3, stream, **kw32)
    X32 = D.state.clone()
    D.smooth("oddeven", covariance=False)
    ms64, _ = time_smooths(D, 2, stream, covariance=False)
    X64 = D.state
    rel = lambda X: float(((X - X64).abs().amax(dim=1) / X64.abs().amax(dim=1)).max().item())
    out = {"what": "single track n=128, m=64, k=20000, odd-even, states; F = 0.995 Q, G ~ N(0, 1/m), noise "
                   "covariance eigenvalues log-uniform in [1e-3, 1], 5 % of steps unobserved; synthetic",
           "fp32_refine": {"ms": ms32, "steps_per_s": P.nsteps / (ms32 * 1e-3), "rel_err_vs_fp64": rel(X32),
                           "form": "FP32 blocked QR (FMA updates) + 1 FP64-residual sweep"},
           "plain_fp64": {"ms": ms64, "steps_per_s": P.nsteps / (ms64 * 1e-3)},
           "speedup_fp32_refine_vs_fp64": ms64 / ms32}
    del D
    torch.cuda.empty_cache()
    return out


def secondary(fn):
    """Runs one secondary leg of the bench; a failure is reported in its key
    (with the library's message) instead of ending the run."""
    import torch
    try:
        return fn()
    except Exception as e:  # the headline line must still be printed
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        return {"error": f"{type(e).__name__}: {e}"}


def gpu_numa_cpus():
    """(NUMA node of the current GPU, the host CPUs of that node) from sysfs,
    or (None, None)."""
    import torch
    try:
        pr = torch.cuda.get_device_properties(torch.cuda.current_device())
        bus = f"{pr.pci_domain_id:04x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0"
        with open(f"/sys/bus/pci/devices/{bus}/numa_node") as f:
            node = int(f.read().strip())
        if node < 0:
            return None, None
        cpus = set()
        with open(f"/sys/devices/system/node/node{node}/cpulist") as f:
            for part in f.read().strip().split(","):
                a, _, b = part.partition("-")
                cpus.update(range(int(a), int(b or a) + 1))
        return node, cpus
    except Exception:
        return None, None


def numa_local(fn):
    """Runs fn() with this thread restricted to the host CPUs of the GPU's
    NUMA node (when that is known and allowed), so that page-locked buffers
    fn allocates are placed in memory local to the GPU's host link; restores
    the affinity afterwards.  Returns (fn(), node used or None)."""
    node, cpus = gpu_numa_cpus()
    old = os.sched_getaffinity(0)
    use = (old & cpus) if cpus else set()
    if not use:
        return fn(), None
    os.sched_setaffinity(0, use)
    try:
        return fn(), node
    finally:
        os.sched_setaffinity(0, old)


def h2d_probe(gb=4.0):
    """Host-to-device bandwidth of this machine: one copy of a `gb` GB page-locked
    buffer into device memory (cudaMemcpyAsync), CUDA events, best of 3; and
    the host NUMA node of the GPU where sysfs says."""
    import torch
    n = int(gb * 1e9) // 8
    h, _ = numa_local(lambda: torch.empty(n, dtype=torch.float64).pin_memory())
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    best = None
    for _ in range(3):
        ms = time_call(lambda: d.copy_(h, non_blocking=True), 1, torch.cuda.current_stream())
        best = ms if best is None else min(best, ms)
    out = {"h2d_gbs": n * 8 / (best * 1e-3) / 1e9, "probe_gb": n * 8 / 1e9}
    try:
        pr = torch.cuda.get_device_properties(0)
        bus = f"{pr.pci_domain_id:04x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0"
        with open(f"/sys/bus/pci/devices/{bus}/numa_node") as f:
            out["gpu_numa_node"] = int(f.read().strip())
    except Exception:
        pass
    del h, d
    torch.cuda.empty_cache()
    return out


def serving_line():
    """The serving form: a seeded Poisson stream of requests with state
    dimensions drawn from {4, 6, 12, 24} (m = n/2), F = 0.98 Q, SPD noise
    covariances, lengths log-uniform in [64, 1,000,000], shipped compactly
    (model + observations) and expanded on the device at admission; HBM
    budget 90 GiB; two lanes.  Per precision (FP64, and FP32 + refinement):
    the capacity served back to back, then 48 requests at each of the offered
    loads 0.3, 0.6 and 0.9 of it, with p50/p99 latency and throughput."""
    from ultimate_kalman_gb300 import serve
    out = {"what": "Poisson request stream, n in {4,6,12,24}, m=n/2, lengths log-uniform [64, 1e6], compact "
                   "requests expanded on the device, HBM budget 90 GiB, 2 lanes, states; synthetic, seeded"}
    for name, f32 in (("fp64", False), ("fp32_refine", True)):
        out[name] = serve.run_loads(requests=48, loads=(0.3, 0.6, 0.9), max_len=1000000, budget_gb=90.0,
                                    fp32_refine=f32, compact=True, calibration=24, lanes=2)
    return out


def config0_line(stream, with_cpu):
    """Single constant-velocity track, n=6, m=3, dt=0.1, k=100,000 (prior
    folded into a square step-0 observation): the odd-even smoother in plain
    FP64 with covariances and states only, the precision form (states), and
    the associative smoother in FP64 with covariances.  Errors of every GPU
    result against the plain FP64 odd-even path are measured here; with
    with_cpu the oracle's restatement of the reference smoother is timed on
    the same track (its CPU baseline) and the GPU results are checked
    against it."""
    import torch
    from ultimate_kalman_gb300 import native, problem as pb
    P = pb.constant_velocity([100000], seed=7)
    D = native.DeviceProblem(P, covariance=True)
    runs = {"fp64_states_and_covariances": dict(covariance=True),
            "fp64_states": dict(covariance=False),
            "fp32_refine_states": dict(covariance=False, fp32_refine=True, sweeps=1)}
    out = {"what": "one constant-velocity track, n=6, m=3, k=100000, odd-even smoother (and the associative "
                   "smoother, FP64 with covariances); synthetic, seeded", "steps": int(P.nsteps)}
    res = {}
    for name, kw in runs.items():
        D.smooth("oddeven", **kw)
        ms = time_call(lambda: D.smooth("oddeven", stream=stream, **kw), 5, stream)
        res[name] = (D.state.clone(), D.cov.clone() if kw["covariance"] else None)
        out[name] = {"ms": ms, "steps_per_s": P.nsteps / (ms * 1e-3)}
    D.smooth("associative", covariance=True)
    ms = time_call(lambda: D.smooth("associative", stream=stream, covariance=True), 5, stream)
    res["assoc"] = (D.state.clone(), D.cov.clone())
    out["associative_fp64_states_and_covariances"] = {"ms": ms, "steps_per_s": P.nsteps / (ms * 1e-3)}
    X64, S64 = res["fp64_states_and_covariances"]
    out["fp32_refine_states"]["rel_err_vs_fp64"] = rel_states(res["fp32_refine_states"][0], X64)
    out["associative_fp64_states_and_covariances"]["rel_err_vs_fp64_oddeven"] = {
        "states": rel_states(res["assoc"][0], X64), "covariances": rel_states(res["assoc"][1], S64)}
    out["speedup_fp32_refine_vs_fp64_states"] = out["fp64_states"]["ms"] / out["fp32_refine_states"]["ms"]
    if with_cpu:
        import oracle
        nt = oracle.max_threads()
        t0 = time.perf_counter()
        st, Xo, So = oracle.smooth(P, "oddeven", covariance=True, threads=nt)
        dt = time.perf_counter() - t0
        t0 = time.perf_counter()
        sta, Xa, Sa = oracle.smooth(P, "associative", covariance=True, threads=nt)
        dta = time.perf_counter() - t0
        cov_t = lambda S: np.ascontiguousarray(S.cpu().numpy().transpose(0, 2, 1))
        out["cpu_baseline"] = {
            "kind": "port", "cores": 1, "unit": UNIT,
            "oddeven_states_and_covariances": P.nsteps / dt, "associative_states_and_covariances": P.nsteps / dta,
            "sample": "the whole track; oracle/kalman_oracle.c (one track runs on one thread)",
            "rel_err_vs_oracle": {
                "fp64_states": rel_states(X64.cpu().numpy(), Xo), "fp64_covariances": rel_states(cov_t(S64), So),
                "fp32_refine_states": rel_states(res["fp32_refine_states"][0].cpu().numpy(), Xo),
                "associative_states": rel_states(res["assoc"][0].cpu().numpy(), Xa),
                "associative_covariances": rel_states(cov_t(res["assoc"][1]), Sa)}}
    del D, res
    torch.cuda.empty_cache()
    return out


def config1_line(stream, with_cpu):
    """Single track, n=48, m=24, k=1,000,000, F = 0.99 Q, G ~ N(0, 1/m), SPD
    noise covariances with eigenvalues in [0.1, 1], 5 % of steps unobserved;
    its 93 GB of per-step equations are written on the device by the
    equation builder.  The associative smoother (FP64, states and
    covariances), the odd-even smoother (FP64 with covariances) and the
    precision form (states), each timed once after a warm-up; errors against
    the FP64 odd-even result.  With with_cpu the oracle runs on a 3,000-step
    track of the same shape and the GPU smoothers are checked against it."""
    import torch
    from ultimate_kalman_gb300 import native, shapes
    k = 1000000
    D = shapes.device_track(k, 48, 24, missing=0.05, covariance=True)
    out = {"what": "one track n=48, m=24, k=1000000, F = 0.99 Q, G ~ N(0, 1/m), noise covariance eigenvalues "
                   "U[0.1, 1], 5 % unobserved; equations built on the device; synthetic, seeded",
           "input_gb": D.input_bytes() / 1e9}
    runs = [("oddeven_fp64_states_and_covariances", "oddeven", dict(covariance=True)),
            ("associative_fp64_states_and_covariances", "associative", dict(covariance=True)),
            ("oddeven_fp32_refine_states", "oddeven", dict(covariance=False, fp32_refine=True, sweeps=1))]
    ref = None  # the FP64 odd-even states and every 50th covariance block (HBM: 93 GB inputs + workspace)
    for name, alg, kw in runs:
        D.smooth(alg, **kw)
        ms = time_call(lambda: D.smooth(alg, stream=stream, **kw), 1, stream)
        out[name] = {"ms": ms, "steps_per_s": k / (ms * 1e-3)}
        if ref is None:
            ref = (D.state.clone(), D.cov[::50].clone())
        elif kw["covariance"]:
            out[name]["rel_err_vs_fp64_oddeven"] = {"states": rel_states(D.state, ref[0]),
                                                    "covariances_every_50th_step": rel_states(D.cov[::50], ref[1])}
        else:
            out[name]["rel_err_vs_fp64"] = rel_states(D.state, ref[0])
        native.release()
        torch.cuda.empty_cache()
    del D, ref
    torch.cuda.empty_cache()
    if with_cpu:
        import oracle
        ks = 3000
        P = shapes.synthetic_track(ks, 48, 24, missing=0.05)
        Ds = native.DeviceProblem(P, covariance=True)
        got = {}
        for alg, kw in (("associative", dict(covariance=True)), ("oddeven", dict(covariance=True)),
                        ("fp32", dict(covariance=False, fp32_refine=True, sweeps=1))):
            Ds.smooth("oddeven" if alg == "fp32" else alg, **kw)
            X, S = Ds.results()
            got[alg] = (X, S if kw["covariance"] else None)
        t0 = time.perf_counter()
        _, Xoe, Soe = oracle.smooth(P, "oddeven", covariance=True)
        dto = time.perf_counter() - t0
        t0 = time.perf_counter()
        _, Xas, Sas = oracle.smooth(P, "associative", covariance=True)
        dta = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "kind": "port", "cores": 1, "unit": UNIT, "oddeven_states_and_covariances": ks / dto,
            "associative_states_and_covariances": ks / dta,
            "sample": f"a {ks}-step track of the same shape and distribution; oracle/kalman_oracle.c, one thread",
            "rel_err_vs_oracle": {
                "oddeven_fp64_states": rel_states(got["oddeven"][0], Xoe),
                "oddeven_fp64_covariances": rel_states(got["oddeven"][1], Soe),
                "associative_fp64_states": rel_states(got["associative"][0], Xas),
                "associative_fp64_covariances": rel_states(got["associative"][1], Sas),
                "fp32_refine_states": rel_states(got["fp32"][0], Xoe)}}
        del Ds
        torch.cuda.empty_cache()
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
