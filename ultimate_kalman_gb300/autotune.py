"""Autotuner for the odd-even smoother's work mapping and block shapes.

The library exposes its launch choices as kalman_gpu_tuning_t
(include/kalman_gpu.h): whether a work item (step pair, tail, even step) goes
to one thread or to one thread block (cta_min_n), how many blocks per SM the
block-per-item kernels' persistent grid keeps (ctas_per_sm), and the block
sizes of the precision form's register-tile pair kernel (pair_block) and
double-float weighing kernel (weigh_block).  Which choice is fastest depends
on the problem class -- state dimension, observation rows, precision, whether
covariances are wanted, and how much parallel work the tracks offer -- so
this module measures them on the GPU and keeps the winners.

A problem class is keyed by (n, mmax, precision, covariances, mean track
length rounded to a power of two, track count rounded to a power of two).
tune() times the candidates by coordinate descent (every value of one knob
with the others fixed at the best so far, knobs in turn, until a full pass
changes nothing), each candidate as the mean of `reps` smoothings after a
warm-up, with CUDA events on the launching stream; knobs that cannot affect
the class (the FP32 block sizes in FP64, the grid in the thread mapping) are
not searched.  The result and the whole table go into a JSON cache
(tuning_gb300.json beside this file), which apply() reads.  The reference's
only tuning knob is the TBB grain (c/parallel_tbb.cpp:31,39-43, set through
parallel_set_blocksize, c/parallel.h:31-32).

    python -m ultimate_kalman_gb300.autotune --workload batched
"""
from __future__ import annotations

import argparse
import datetime
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(HERE, "tuning_gb300.json")

SPACE = {"cta_min_n": None,  # per class: the thread mapping (n + 1) or the block mapping (n)
         "ctas_per_sm": [1, 2, 3, 4, 6, 8],
         "pair_block": [32, 64, 128],
         "weigh_block": [64, 128, 256]}


def class_key(n, mmax, track_lengths, fp32_refine, covariance):
    lens = np.asarray(track_lengths, dtype=np.int64)
    lb = int(round(math.log2(max(1.0, float(lens.mean())))))
    tb = int(round(math.log2(max(1, len(lens)))))
    prec = "dd" if (fp32_refine and covariance) else "fp32" if fp32_refine else "fp64"
    return f"oddeven|n{n}|m{mmax}|{prec}|{'cov' if covariance else 'states'}|L2^{lb}|T2^{tb}"


def candidates(knob, n, mmax, fp32_refine, covariance, current):
    """Values of `knob` that can change the launches for this class."""
    thread_ok = n <= 8 and max(n, mmax) <= 8
    blocks = current["cta_min_n"] <= n or not thread_ok
    if knob == "cta_min_n":
        return [n + 1, n] if thread_ok else [current["cta_min_n"]]
    if knob == "ctas_per_sm":
        return SPACE[knob] if blocks else [current[knob]]
    fp32_thread = fp32_refine and not covariance and not blocks and n == max(n, mmax) and n in (4, 6)
    return SPACE[knob] if fp32_thread else [current[knob]]


def _time(D, kw, reps, stream):
    import torch
    D.smooth("oddeven", stream=stream, **kw)  # warm-up (workspace, first launches)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record(stream)
    for _ in range(reps):
        D.smooth("oddeven", stream=stream, **kw)
    e.record(stream)
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def tune(D, fp32_refine=False, covariance=False, sweeps=0, reps=3, stream=None, save=True, cache=CACHE):
    """Tunes the class of device problem D (a native.DeviceProblem); returns
    the cache entry {"key", "tuning", "ms", "default_ms", "table"} and, with
    save, records it in the cache.  Leaves the best tuning in force."""
    import torch
    from . import native
    stream = stream or torch.cuda.current_stream()
    s = D.struct
    n, mmax = s.n, s.mmax
    lens = np.diff(D.track_start)
    key = class_key(n, mmax, lens, fp32_refine, covariance)
    kw = dict(covariance=covariance, fp32_refine=fp32_refine, sweeps=sweeps)
    best = native.set_tuning(default=True)
    table = []

    def trial(t):
        native.set_tuning(**t)
        ms = _time(D, kw, reps, stream)
        table.append({**t, "ms": ms})
        return ms

    best_ms = default_ms = trial(best)
    changed = True
    while changed:
        changed = False
        for knob in SPACE:
            for v in candidates(knob, n, mmax, fp32_refine, covariance, best):
                if v == best[knob]:
                    continue
                t = dict(best, **{knob: v})
                ms = trial(t)
                if ms < best_ms * 0.99:  # a change must win by more than the timing noise
                    best, best_ms, changed = t, ms, True
    native.set_tuning(**best)
    entry = {"key": key, "tuning": best, "ms": best_ms, "default_ms": default_ms, "table": table,
             "device": torch.cuda.get_device_name(), "reps": reps,
             "when": datetime.datetime.now(datetime.timezone.utc).strftime("%Y-%m-%dT%H:%M:%SZ")}
    if save:
        record(entry, cache)
    return entry


def load_cache(cache=CACHE):
    if not os.path.exists(cache):
        return {}
    with open(cache) as f:
        return json.load(f)


def record(entry, cache=CACHE):
    data = load_cache(cache)
    data[entry["key"]] = entry
    tmp = cache + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, cache)


def lookup(n, mmax, track_lengths, fp32_refine, covariance, cache=CACHE):
    """The cached tuning of this class, or None."""
    e = load_cache(cache).get(class_key(n, mmax, track_lengths, fp32_refine, covariance))
    return e["tuning"] if e else None


def apply(n, mmax, track_lengths, fp32_refine, covariance, cache=CACHE):
    """Puts the cached tuning of the class in force (the defaults when the
    class was never tuned); returns (tuning, whether it came from the cache)."""
    from . import native
    t = lookup(n, mmax, track_lengths, fp32_refine, covariance, cache)
    if t is None:
        return native.set_tuning(default=True), False
    native.set_tuning(default=True)
    return native.set_tuning(**t), True


def main():
    import torch
    from . import native, problem as pb
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", default="batched", choices=["batched", "single"],
                    help="batched: 4,096 constant-velocity tracks (n=6, m=3, lengths log-uniform in [100, 20000]); "
                         "single: one 100,000-step constant-velocity track")
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    native.load()
    if args.workload == "batched":
        P = pb.constant_velocity(pb.batched_lengths(4096, 100, 20000, seed=0), seed=1000)
    else:
        P = pb.constant_velocity([100000], seed=7)
    D = native.DeviceProblem(P, covariance=True)
    for f32, cov in ((True, False), (True, True), (False, False), (False, True)):
        e = tune(D, fp32_refine=f32, covariance=cov, sweeps=1 if (f32 and not cov) else 0, reps=args.reps)
        print(json.dumps({k: e[k] for k in ("key", "tuning", "ms", "default_ms")}), flush=True)
    native.set_tuning(default=True)
    torch.cuda.synchronize()


if __name__ == "__main__":
    main()
