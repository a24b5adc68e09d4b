#!/usr/bin/env python3
"""Benchmark: batched odd-even Kalman smoothing on GB300 (smoothed steps/s).

Workload (default, "batched"): 4,096 independent constant-velocity tracks
(n=6 [pos; vel], m=3, dt=0.1, process noise diag(1e-2), observation noise
diag(1e-1), prior N(0, I) folded into a square step-0 observation), lengths
floor(exp(U[ln 100, ln 20000])) from a fixed seed -- 15.1 million steps,
23.3 GB of FP64 equations (larger than the 126 MB L2, so nothing is re-read
from cache between timed steps).  Data is synthetic (seeded NumPy).

One "step" of the benchmark = one full odd-even smoothing (states and
covariances, FP64) of every track, through the library's C ABI:
  value -- inputs resident in HBM, kalman_gpu_smooth_oddeven_packed on device
           arrays (CUDA events on the launching stream, synchronized);
  e2e   -- the same call handed page-locked HOST arrays: host->device copy of
           the equations, smoothing, device->host copy of states and
           covariances all inside the timed region.
Other keys: per-kernel roofline (FP64 pipe: the kernels are arithmetic-bound),
CPU baseline (the oracle's C restatement of the reference
smoother on all host cores, a bounded sample of the same tracks), clocks.

--impl reference: times the CPU restatement of the reference's odd-even
smoother (oracle/kalman_oracle.c, OpenMP over tracks) on a bounded sample of
the same workload, per step, with all host threads.

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

METRIC = "smoothed steps/s (batched odd-even, FP64)"
UNIT = "steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--tracks", type=int, default=4096)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
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
    return {"workload": "batched constant-velocity tracks, odd-even smoother (states + covariances)",
            "tracks_per_gpu": tracks, "steps_per_gpu": int(P.nsteps), "n": 6, "m": 3,
            "track_lengths": "floor(exp(U[ln 100, ln 20000]))", "precision": "FP64",
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
                                          "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
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


def cpu_sample(P, seconds, threads=0, algorithm="oddeven"):
    """Times the oracle's restatement on the first tracks of P, grown until the
    sample takes about `seconds`; returns (steps/s, steps, tracks, threads)."""
    import oracle
    nt = threads or oracle.max_threads()
    ntr = 8
    while True:
        S = P.select_tracks(range(min(ntr, P.ntracks)))
        t0 = time.perf_counter()
        oracle.smooth(S, algorithm, covariance=True, threads=nt)
        dt = time.perf_counter() - t0
        if dt >= seconds * 0.6 or ntr >= P.ntracks:
            return S.nsteps / dt, S.nsteps, S.ntracks, nt, dt
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
    _, _, ntr, nt, _ = cpu_sample(P, budget)
    S = P.select_tracks(range(ntr))
    for _ in range(args.warmup):
        oracle.smooth(S, "oddeven", threads=nt)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.smooth(S, "oddeven", threads=nt)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.mean(times))
    v = S.nsteps / (ms * 1e-3)
    sample = f"first {ntr} of {P.ntracks} tracks ({S.nsteps} steps) per step"
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(P, args.tracks, world),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nt, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    from ultimate_kalman_gb300 import build, flops, native
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build()
    native.load()
    P = workload(args.tracks, rank)
    D = native.DeviceProblem(P, covariance=True)
    for _ in range(args.warmup):
        D.smooth("oddeven", covariance=True)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    sampler = ClockSampler(local)
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    native.profile_enable(True)
    launches0 = native.launch_count()
    barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        D.smooth("oddeven", covariance=True, stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = native.launch_count() - launches0
    prof = native.profile_read()
    native.profile_enable(False)
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    total_steps = P.nsteps * world
    value = total_steps / (ms * 1e-3)

    # states-only throughput (KALMAN_NO_COVARIANCE), for reference
    ev0.record(stream)
    for _ in range(max(1, args.steps // 2)):
        D.smooth("oddeven", covariance=False, stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms_nocov = ev0.elapsed_time(ev1) / max(1, args.steps // 2)

    # roofline of the dominant kernel: FP64 pipe
    fl = flops.plan_flops_fast(P.track_lengths(), 6, 3, covariance=True)
    top = max(prof, key=lambda k: prof[k][0])
    kms, kl = prof[top]
    achieved = fl[top] * args.steps / (kms * 1e-3) / 1e12
    peak = native.measure_fp64_tflops(32)
    total_tf = sum(fl.values()) / (ms * 1e-3) / 1e12
    per_kernel = {k: {"ms_per_step": v[0] / args.steps, "launches_per_step": v[1] / args.steps,
                      "share": v[0] / sum(x[0] for x in prof.values()),
                      "tflops": fl.get(k, 0.0) * args.steps / (v[0] * 1e-3) / 1e12} for k, v in prof.items()}
    traffic = None
    tfile = os.path.join(REPO, "profiles", "traffic_per_launch.json")
    if os.path.exists(tfile):
        traffic = json.load(open(tfile)).get(top)
    roofline = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": top,
                "peak_source": "FP64 FMA-chain probe kernel timed in this run (MEASURED_PEAKS.json has no FP64 figure)",
                "flops_model": "ultimate_kalman_gb300/flops.py (FMA = 2 flops)",
                "whole_smoother_tflops": total_tf, "per_kernel": per_kernel}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config_dict(P, args.tracks, world),
            "gpu_launches": int(launches), "roofline": roofline, "clocks": clocks,
            "states_only": {"value": total_steps / (ms_nocov * 1e-3), "unit": UNIT, "ms_per_step": ms_nocov}}

    # end to end through the C ABI with page-locked host buffers
    if not args.no_e2e:
        del D
        torch.cuda.empty_cache()
        pin = {f: torch.from_numpy(np.ascontiguousarray(getattr(P, f))).pin_memory() for f in native._FIELDS}
        st_h = torch.empty((P.nsteps, 6), dtype=torch.float64).pin_memory()
        cov_h = torch.empty((P.nsteps, 6, 6), dtype=torch.float64).pin_memory()
        s = native.host_struct_from_tensors(P, pin, st_h, cov_h)
        native.smooth_struct("oddeven", s, covariance=True)  # warm-up (device staging allocated)
        times = []
        for _ in range(args.e2e_steps):
            barrier()
            t0 = time.perf_counter()
            native.smooth_struct("oddeven", s, covariance=True)
            times.append(time.perf_counter() - t0)
        e2e_ms = 1e3 * max(times) if world == 1 else 1e3 * float(np.mean(times))
        h2d = sum(t.numel() * t.element_size() for t in pin.values())
        d2h = st_h.numel() * 8 + cov_h.numel() * 8
        line["e2e"] = {"value": total_steps / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                       "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
                       "path": "kalman_gpu_smooth_oddeven_packed with KALMAN_GPU_HOST arrays"}

    if rank == 0 and world == 1 and not args.no_cpu:
        v, nsteps, ntr, nt, dt = cpu_sample(P, args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nt, "kind": "port",
                                "sample": f"first {ntr} of {P.ntracks} tracks ({nsteps} steps), {dt:.1f} s, "
                                          f"oracle/kalman_oracle.c odd-even, OpenMP over tracks"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
