"""Serving form: a stream of smoothing requests on one GPU.

Requests (one track each, of any length and state dimension) arrive over time.
The server admits a waiting request once its device footprint fits the HBM
budget, uploading its equations so they stay resident on the device until it
is answered.  Whenever the GPU is free it runs one batch: every admitted
request of the shape class (n, mmax, options) whose oldest request arrived
first, up to a step limit, gathered into one packed problem and smoothed with
one call of the batched entry point (kalman_gpu_smooth_oddeven_packed on
device arrays: tracks are independent, so a request's result does not depend
on its batch).  Results go back to the host and the request's device memory is
released.  Latency = completion - arrival.

This is host-side scheduling around the library's C ABI; torch provides the
device allocations and copies.  `Server` takes its executor and clock as
arguments so that the scheduling rules are testable without a GPU.

    python -m ultimate_kalman_gb300.serve --requests 300 --loads 0.3,0.6,0.9
"""
from __future__ import annotations

import argparse
import collections
import dataclasses
import json
import time

import numpy as np

from . import problem as pb

FIELDS = ("H", "F", "c", "K", "K_type", "G", "o", "C", "C_type", "obs_rows")


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float            # seconds after the start of the stream
    problem: pb.PackedProblem  # one track
    covariance: bool = False
    fp32_refine: bool = False
    device: dict = None        # resident device arrays once admitted
    admitted: float = None
    completed: float = None
    state: np.ndarray = None
    cov: np.ndarray = None

    @property
    def steps(self):
        return int(self.problem.nsteps)

    def key(self):
        return (self.problem.n, self.problem.mmax, self.covariance, self.fp32_refine)


def footprint(req: Request) -> int:
    """Device bytes a request holds while admitted: its equations, its outputs
    and its share of the smoother's workspace (level equations and records,
    about twice the equations' size in FP64)."""
    P = req.problem
    eq = P.nbytes()
    out = P.nsteps * P.n * 8 * (1 + (P.n if req.covariance else 0))
    return int(eq + out + 2 * eq)


def serving_track(k, n, m, rng):
    """One request of the serving form: F = 0.98 Q (Q random orthogonal: spectral
    radius 0.98), H = I, c = 0, SPD process and observation covariances with
    eigenvalues in [0.1, 1], G i.i.d. N(0, 1/m), a square identity-weighted
    step-0 observation, observations drawn at random (valid least-squares
    problems; their values do not change the work)."""
    P = pb.empty_problem(n, n, [k])
    Fm = 0.98 * pb.random_orthogonal(rng, n)
    Gm = rng.standard_normal((m, n)) / np.sqrt(m)
    Kc = pb.random_spd(rng, n)
    Cc = pb.random_spd(rng, m)
    P.H[1:] = np.eye(n)
    P.F[1:] = Fm.T
    P.K[1:] = Kc.T
    P.G[0, :, :] = np.eye(n)  # column-major blocks: G[s] holds G^T
    P.C[0] = np.eye(n)
    P.o[0] = rng.standard_normal(n)
    P.obs_rows[0] = n
    Gt = np.zeros((n, n))
    Gt[:, :m] = Gm.T
    Ct = np.zeros((n, n))
    Ct[:m, :m] = Cc.T
    P.G[1:] = Gt
    P.C[1:] = Ct
    P.o[1:, :m] = rng.standard_normal((k - 1, m))
    P.obs_rows[1:] = m
    return P


def request_stream(nreq, rate, seed=0, dims=(4, 6, 12, 24), min_len=64, max_len=20000, covariance=False,
                   fp32_refine=False):
    """Poisson arrivals at `rate` requests/s; state dimension uniform over `dims`
    (m = n/2); lengths log-uniform in [min_len, max_len]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(nreq):
        t += rng.exponential(1.0 / rate)
        n = int(rng.choice(dims))
        k = int(np.floor(np.exp(rng.uniform(np.log(min_len), np.log(max_len)))))
        out.append(Request(i, t, serving_track(k, n, n // 2, rng), covariance, fp32_refine))
    return out


class GpuExecutor:
    """Uploads admitted requests and runs batches through the C ABI."""

    def __init__(self, device="cuda"):
        import torch
        from . import native
        self.torch, self.native, self.device = torch, native, device
        native.load()

    def upload(self, req: Request):
        torch = self.torch
        req.device = {f: torch.from_numpy(np.ascontiguousarray(getattr(req.problem, f))).to(self.device,
                                                                                          non_blocking=True)
                      for f in FIELDS}

    def release(self, req: Request):
        req.device = None

    def run(self, batch):
        """Smooths the batch as one packed problem; fills state (and cov)."""
        import ctypes
        torch, native = self.torch, self.native
        n, mmax, cov, f32 = batch[0].key()
        arrays = {f: torch.cat([r.device[f] for r in batch]) for f in FIELDS}
        lens = np.array([r.steps for r in batch], dtype=np.int64)
        ts = np.zeros(len(batch) + 1, dtype=np.int64)
        ts[1:] = np.cumsum(lens)
        N = int(ts[-1])
        state = torch.empty((N, n), dtype=torch.float64, device=self.device)
        covs = torch.empty((N, n, n), dtype=torch.float64, device=self.device) if cov else None
        s = native.ProblemStruct()
        s.n, s.mmax, s.ntracks, s.location = n, mmax, len(batch), native.KALMAN_GPU_DEVICE
        s.nsteps = N
        s.track_start = ts.ctypes.data
        for f in FIELDS:
            setattr(s, f, arrays[f].data_ptr())
        s.state = state.data_ptr()
        s.covariance = covs.data_ptr() if cov else None
        native.smooth_struct("oddeven", s, covariance=cov, fp32_refine=f32,
                             stream=torch.cuda.current_stream())
        X = state.cpu().numpy()
        S = covs.cpu().numpy() if cov else None
        for i, r in enumerate(batch):
            r.state = X[ts[i]:ts[i + 1]]
            if cov:
                r.cov = np.ascontiguousarray(S[ts[i]:ts[i + 1]].transpose(0, 2, 1))


class Server:
    """Continuous batching with HBM-budget admission (see the module docstring).

    executor: upload(req), release(req), run(batch)
    clock: returns seconds since the stream started (wall clock by default);
    wait(dt) lets time pass while idle."""

    def __init__(self, executor, hbm_budget=16 << 30, max_batch_steps=1 << 25, clock=None, wait=None):
        self.ex = executor
        self.budget = int(hbm_budget)
        self.max_batch_steps = int(max_batch_steps)
        self.in_use = 0
        self.peak_in_use = 0
        self.batches = []
        self._t0 = None
        self.clock = clock or self._wall
        self.wait = wait or (lambda dt: time.sleep(max(0.0, min(dt, 0.01))))

    def _wall(self):
        if self._t0 is None:
            self._t0 = time.perf_counter()
        return time.perf_counter() - self._t0

    def serve(self, requests):
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        queue = collections.deque()                 # arrived, not yet admitted (FIFO)
        admitted = collections.OrderedDict()        # class -> list of resident requests
        done = []
        while pending or queue or any(admitted.values()):
            now = self.clock()
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            while queue:
                r = queue[0]
                f = footprint(r)
                if f > self.budget:
                    raise ValueError(f"request {r.rid} needs {f} bytes, above the HBM budget {self.budget}")
                if self.in_use + f > self.budget:
                    break
                queue.popleft()
                self.ex.upload(r)
                r.admitted = self.clock()
                self.in_use += f
                self.peak_in_use = max(self.peak_in_use, self.in_use)
                admitted.setdefault(r.key(), []).append(r)
            live = [k for k, v in admitted.items() if v]
            if not live:
                if pending:
                    self.wait(pending[0].arrival - now)
                continue
            key = min(live, key=lambda k: admitted[k][0].arrival)
            batch, steps = [], 0
            for r in admitted[key]:
                if batch and steps + r.steps > self.max_batch_steps:
                    break
                batch.append(r)
                steps += r.steps
            admitted[key] = admitted[key][len(batch):]
            self.ex.run(batch)
            t = self.clock()
            for r in batch:
                r.completed = t
                self.ex.release(r)
                self.in_use -= footprint(r)
                done.append(r)
            self.batches.append((key, len(batch), steps))
        return done


def summarize(done, makespan=None):
    lat = np.array([r.completed - r.arrival for r in done])
    steps = sum(r.steps for r in done)
    span = makespan if makespan is not None else max(r.completed for r in done) - min(r.arrival for r in done)
    return {"requests": len(done), "steps": int(steps), "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
            "throughput_steps_per_s": float(steps / span) if span > 0 else None}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--requests", type=int, default=300)
    ap.add_argument("--loads", default="0.3,0.6,0.9", help="offered loads as fractions of the measured capacity")
    ap.add_argument("--max-len", type=int, default=20000)
    ap.add_argument("--budget-gb", type=float, default=16.0)
    ap.add_argument("--fp32-refine", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    ex = GpuExecutor()
    # capacity: steps/s of one batch of a calibration stream served back to back
    cal = request_stream(min(args.requests, 64), 1e9, seed=args.seed + 99, max_len=args.max_len,
                         fp32_refine=args.fp32_refine)
    for r in cal:
        r.arrival = 0.0
    srv = Server(ex, hbm_budget=args.budget_gb * 2 ** 30)
    srv.serve(cal[:8])  # warm-up
    t0 = time.perf_counter()
    done = Server(ex, hbm_budget=args.budget_gb * 2 ** 30).serve(cal)
    cap_steps = sum(r.steps for r in done) / (time.perf_counter() - t0)
    mean_steps = np.mean([r.steps for r in cal])
    cap_rate = cap_steps / mean_steps
    out = {"capacity_steps_per_s": cap_steps, "capacity_requests_per_s": cap_rate, "loads": []}
    for load in [float(x) for x in args.loads.split(",")]:
        reqs = request_stream(args.requests, load * cap_rate, seed=args.seed, max_len=args.max_len,
                              fp32_refine=args.fp32_refine)
        srv = Server(ex, hbm_budget=args.budget_gb * 2 ** 30)
        done = srv.serve(reqs)
        s = summarize(done)
        s.update({"offered_load": load, "arrival_rate_per_s": load * cap_rate,
                  "batches": len(srv.batches), "mean_batch_requests": float(np.mean([b[1] for b in srv.batches])),
                  "peak_hbm_gb": srv.peak_in_use / 2 ** 30})
        out["loads"].append(s)
        print(json.dumps(s), flush=True)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
