"""Serving form: a stream of smoothing requests on one GPU, continuously batched.

Requests (one track each, of any length and state dimension) arrive over time.
The server admits a waiting request once its device footprint fits the HBM
budget, uploading its equations on a copy stream so they stay resident on the
device until it is answered.  Batches run on lanes: each lane is a host thread
with its own CUDA stream and its own library workspace, so while one batch is
on the GPU the loop keeps admitting arrivals and starts the next batch on a
free lane, and the batches' kernels overlap on the device.  A batch is every
admitted, not yet running request of one shape class (n, mmax, options) --
the class whose oldest request arrived first -- up to a step limit, gathered
into one packed problem and smoothed with one call of the batched entry point
(kalman_gpu_smooth_oddeven_packed on device arrays: tracks are independent, so
a request's result does not depend on its batch or on what runs beside it).
Results go back to the host and the request's device memory is released.
Latency = completion - arrival.

HBM accounting uses the library's own figures: a request holds its equations,
its outputs, its share of the batch's gathered copy and the workspace the
library reports for it (kalman_gpu_oddeven_workspace_bytes).

This is host-side scheduling around the library's C ABI; torch provides the
device allocations and copies.  `Server` takes its executor and clock as
arguments so that the scheduling rules are testable without a GPU.

    python -m ultimate_kalman_gb300.serve --requests 300 --loads 0.3,0.6,0.9
"""
from __future__ import annotations

import argparse
import collections
import concurrent.futures as cf
import dataclasses
import json
import threading
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
    ready: object = None       # CUDA event: the upload has completed
    workspace: int = 0         # library workspace bytes for the request alone
    track_id: object = None    # a track the server keeps on the device (None: a one-off track)
    keep: bool = False         # keep the (extended) track resident after answering
    prior_steps: int = 0       # steps of the resident track this request extends (set at admission)
    admitted: float = None
    started: float = None
    completed: float = None
    state: np.ndarray = None
    cov: np.ndarray = None

    @property
    def steps(self):
        """Steps smoothed for this request: the resident track's and its own."""
        return int(self.prior_steps + self.problem.nsteps)

    def key(self):
        return (self.problem.n, self.problem.mmax, self.covariance, self.fp32_refine)


def footprint(req: Request) -> int:
    """Device bytes a request holds while admitted: its equations, its share of
    the batch's gathered copy of them, its outputs and the workspace the
    library reports for it (req.workspace, set by the executor at admission;
    the library's workspace for a batch is the sum over its requests up to
    per-track table entries)."""
    P = req.problem
    eq = P.nbytes() * req.steps // max(1, P.nsteps)  # the whole (extended) track on the device
    out = req.steps * P.n * 8 * (1 + (P.n if req.covariance else 0))
    return int(eq + eq + out + req.workspace)


def track_bytes(req: Request) -> int:
    """Device bytes of the request's whole track's equations (what stays
    resident when the request keeps its track)."""
    return int(req.problem.nbytes() * req.steps // max(1, req.problem.nsteps))


@dataclasses.dataclass
class TrackSpec:
    """One request of the serving form in compact form: a time-invariant track
    ships its matrices once and its observations per step, and is expanded into
    the packed per-step arrays on the device when admitted (a tracking service
    receives a model and a measurement stream, not k copies of the model).
    to_packed() gives the same arrays on the host."""
    n: int
    m: int
    k: int
    F: np.ndarray         # n x n
    G: np.ndarray         # m x n
    K: np.ndarray         # n x n process noise covariance
    C: np.ndarray         # m x m observation noise covariance
    o0: np.ndarray        # n: the square identity-weighted step-0 observation
    o: np.ndarray         # (k-1) x m
    ntracks: int = 1

    @property
    def nsteps(self):
        return self.k

    @property
    def mmax(self):
        return self.n

    def nbytes(self):
        """Bytes of the packed per-step arrays it expands into."""
        n, k = self.n, self.k
        return k * (8 * (4 * n * n + 2 * n + n * n) + 2 + 4)

    def to_packed(self) -> pb.PackedProblem:
        n, m, k = self.n, self.m, self.k
        P = pb.empty_problem(n, n, [k])
        P.H[1:] = np.eye(n)
        P.F[1:] = self.F.T  # column-major blocks: block s holds M^T
        P.K[1:] = self.K.T
        P.G[0] = np.eye(n)
        P.C[0] = np.eye(n)
        P.o[0] = self.o0
        P.obs_rows[0] = n
        P.G[1:, :, :m] = self.G.T
        P.C[1:, :m, :m] = self.C.T
        P.o[1:, :m] = self.o
        P.obs_rows[1:] = m
        return P

    def materialize(self, torch, device, stream=None):
        """The packed arrays of to_packed(), built on the device by the
        library's equation builder (kalman_gpu_expand_invariant): only the
        model and the observations cross the host link."""
        from . import native
        n, m, k = self.n, self.m, self.k
        f64 = dict(dtype=torch.float64, device=device)
        arrays = {"H": torch.empty((k, n, n), **f64), "F": torch.empty((k, n, n), **f64),
                  "c": torch.empty((k, n), **f64), "K": torch.empty((k, n, n), **f64),
                  "K_type": torch.empty(k, dtype=torch.uint8, device=device), "G": torch.empty((k, n, n), **f64),
                  "o": torch.empty((k, n), **f64), "C": torch.empty((k, n, n), **f64),
                  "C_type": torch.empty(k, dtype=torch.uint8, device=device),
                  "obs_rows": torch.empty(k, dtype=torch.int32, device=device)}
        s = native.ProblemStruct()
        s.n, s.mmax, s.ntracks, s.location, s.nsteps = n, n, 1, native.KALMAN_GPU_DEVICE, k
        for f, a in arrays.items():
            setattr(s, f, a.data_ptr())
        dev = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(device)
        eye = dev(np.eye(n))
        # column-major device copies: the row-major memory of M^T
        F, K, G, C, c = dev(self.F.T), dev(self.K.T), dev(self.G.T), dev(self.C.T), dev(np.zeros(n))
        o0, o = dev(self.o0), dev(self.o if k > 1 else np.zeros((1, m)))
        md = native.InvariantModel(m0=n, m=m, H=eye.data_ptr(), F=F.data_ptr(), c=c.data_ptr(), K=K.data_ptr(),
                                   K_type=b"C", G0=eye.data_ptr(), o0=o0.data_ptr(), C0=eye.data_ptr(), C0_type=b"C",
                                   G=G.data_ptr(), C=C.data_ptr(), C_type=b"C")
        native.expand_invariant(s, 0, k, md, o.data_ptr(), m, None, stream or torch.cuda.current_stream())
        return arrays


def serving_spec(k, n, m, rng) -> TrackSpec:
    """One request of the serving form: F = 0.98 Q (Q random orthogonal: spectral
    radius 0.98), H = I, c = 0, SPD process and observation covariances with
    eigenvalues in [0.1, 1], G i.i.d. N(0, 1/m), a square identity-weighted
    step-0 observation, observations drawn at random (valid least-squares
    problems; their values do not change the work)."""
    Fm = 0.98 * pb.random_orthogonal(rng, n)
    Gm = rng.standard_normal((m, n)) / np.sqrt(m)
    Kc = pb.random_spd(rng, n)
    Cc = pb.random_spd(rng, m)
    o0 = rng.standard_normal(n)
    o = rng.standard_normal((k - 1, m))
    return TrackSpec(n, m, k, Fm, Gm, Kc, Cc, o0, o)


def serving_track(k, n, m, rng) -> pb.PackedProblem:
    """serving_spec's track as host packed arrays."""
    return serving_spec(k, n, m, rng).to_packed()


def request_stream(nreq, rate, seed=0, dims=(4, 6, 12, 24), min_len=64, max_len=20000, covariance=False,
                   fp32_refine=False, compact=False):
    """Poisson arrivals at `rate` requests/s; state dimension uniform over `dims`
    (m = n/2); lengths log-uniform in [min_len, max_len].  compact=True ships
    each request as a TrackSpec (expanded on the device at admission)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(nreq):
        t += rng.exponential(1.0 / rate)
        n = int(rng.choice(dims))
        k = int(np.floor(np.exp(rng.uniform(np.log(min_len), np.log(max_len)))))
        spec = serving_spec(k, n, n // 2, rng)
        out.append(Request(i, t, spec if compact else spec.to_packed(), covariance, fp32_refine))
    return out


class GpuExecutor:
    """Uploads admitted requests on a copy stream and runs batches on lanes
    through the C ABI.  A lane is a host thread with its own CUDA stream (the
    library keeps one workspace per host thread), so batches on different
    lanes overlap on the device; ctypes releases the GIL during each call."""

    def __init__(self, device="cuda", lanes=2):
        import torch
        from . import native
        self.torch, self.native, self.device = torch, native, device
        native.load()
        self.lanes = int(lanes)
        self.copy_stream = torch.cuda.Stream(device)
        self.streams = [torch.cuda.Stream(device) for _ in range(self.lanes)]
        self.pool = cf.ThreadPoolExecutor(self.lanes)
        self.t0 = torch.cuda.Event(enable_timing=True)
        self.t0.record()
        self.intervals = []  # (lane, device ms at start, device ms at end, requests) per finished batch
        self.held = {}       # lane -> device bytes its thread's library workspace holds
        self.resident = {}   # track id -> (device arrays of the track's equations, steps)
        self.uploaded_bytes = 0
        self._lock = threading.Lock()

    def _struct(self, n, mmax, ts, arrays, state, covs):
        native = self.native
        s = native.ProblemStruct()
        s.n, s.mmax, s.ntracks, s.location = n, mmax, len(ts) - 1, native.KALMAN_GPU_DEVICE
        s.nsteps = int(ts[-1])
        s.track_start = ts.ctypes.data
        for f in FIELDS:
            setattr(s, f, arrays[f].data_ptr() if arrays is not None else 0)
        s.state = state.data_ptr() if state is not None else 0
        s.covariance = covs.data_ptr() if covs is not None else None
        return s

    def workspace_bytes(self, req: Request) -> int:
        """The library's workspace figure for the request smoothed alone."""
        n, mmax, cov, f32 = req.key()
        ts = np.array([0, req.steps], dtype=np.int64)
        s = self._struct(n, mmax, ts, None, None, None)
        s.covariance = 1 if cov else None  # only its presence matters
        return int(self.native.oddeven_workspace_bytes(s, covariance=cov, fp32_refine=f32))

    def resident_steps(self, track_id):
        return self.resident[track_id][1] if track_id in self.resident else 0

    def upload(self, req: Request):
        """Puts the request's equations on the device.  A request extending a
        resident track uploads only its own steps; the track is assembled on
        the device (its first step carries the evolution from the track's last
        resident step)."""
        torch = self.torch
        with torch.cuda.stream(self.copy_stream):
            if isinstance(req.problem, TrackSpec):
                if req.prior_steps:
                    raise ValueError("a compact request cannot extend a resident track (send packed steps)")
                mine = req.problem.materialize(torch, self.device, self.copy_stream)
            else:
                mine = {f: torch.from_numpy(np.ascontiguousarray(getattr(req.problem, f))).to(
                    self.device, non_blocking=True) for f in FIELDS}
                self.uploaded_bytes += req.problem.nbytes()
            if req.prior_steps:
                old = self.resident[req.track_id][0]
                req.device = {f: torch.cat([old[f], mine[f]]) for f in FIELDS}
            else:
                req.device = mine
            req.ready = torch.cuda.Event()
            req.ready.record(self.copy_stream)

    def release(self, req: Request):
        """Frees the request's device arrays, or keeps them as its track's
        resident equations (req.keep)."""
        if req.track_id is not None:
            if req.keep:
                self.resident[req.track_id] = (req.device, req.steps)
            else:
                self.resident.pop(req.track_id, None)
        req.device = None
        req.ready = None

    def launch(self, batch, lane):
        """Starts the batch on a lane; returns a concurrent.futures.Future."""
        return self.pool.submit(self._run_checked, batch, lane)

    def _run_checked(self, batch, lane):
        try:
            return self._run(batch, lane)
        except Exception as e:
            n, mmax, cov, f32 = batch[0].key()
            raise RuntimeError(f"batch of {len(batch)} requests (n={n}, mmax={mmax}, covariance={cov}, "
                               f"fp32_refine={f32}, steps={sum(r.steps for r in batch)}) on lane {lane}: {e}") from e

    def _run(self, batch, lane):
        torch, native = self.torch, self.native
        st = self.streams[lane]
        n, mmax, cov, f32 = batch[0].key()
        with torch.cuda.stream(st):
            for r in batch:
                st.wait_event(r.ready)
            arrays = {f: (batch[0].device[f] if len(batch) == 1 else torch.cat([r.device[f] for r in batch]))
                      for f in FIELDS}
            lens = np.array([r.steps for r in batch], dtype=np.int64)
            ts = np.zeros(len(batch) + 1, dtype=np.int64)
            ts[1:] = np.cumsum(lens)
            N = int(ts[-1])
            state = torch.empty((N, n), dtype=torch.float64, device=self.device)
            covs = torch.empty((N, n, n), dtype=torch.float64, device=self.device) if cov else None
            s = self._struct(n, mmax, ts, arrays, state, covs)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            native.smooth_struct("oddeven", s, covariance=cov, fp32_refine=f32, stream=st)
            e1.record(st)
            X = state.cpu().numpy()
            S = covs.cpu().numpy() if cov else None
        e1.synchronize()
        held = native.workspace_held()
        with self._lock:
            self.intervals.append((lane, self.t0.elapsed_time(e0), self.t0.elapsed_time(e1), [r.rid for r in batch]))
            self.held[lane] = held
        for i, r in enumerate(batch):
            r.state = X[ts[i]:ts[i + 1]]
            if cov:
                r.cov = np.ascontiguousarray(S[ts[i]:ts[i + 1]].transpose(0, 2, 1))
        return len(batch)

    def close(self):
        self.pool.shutdown(wait=True)


class Server:
    """Continuous batching with HBM-budget admission (see the module docstring).

    executor: lanes, upload(req), release(req), launch(batch, lane) -> a
    future (done(), result(); an optional eta() -- seconds until done -- lets
    a simulated clock jump to the completion)
    clock: returns seconds since the stream started (wall clock by default);
    wait(dt) lets time pass while there is nothing to do."""

    def __init__(self, executor, hbm_budget=16 << 30, max_batch_steps=1 << 25, clock=None, wait=None):
        self.ex = executor
        self.lanes = int(getattr(executor, "lanes", 1))
        self.budget = int(hbm_budget)
        self.max_batch_steps = int(max_batch_steps)
        self.in_use = 0
        self.peak_in_use = 0
        self.batches = []
        self.max_running = 0
        self.resident = {}  # track id -> device bytes of its resident equations (part of in_use)
        self._t0 = None
        self.clock = clock or self._wall
        self.wait = wait or (lambda dt: time.sleep(max(0.0, min(dt, 0.0005))))

    def _wall(self):
        if self._t0 is None:
            self._t0 = time.perf_counter()
        return time.perf_counter() - self._t0

    def serve(self, requests):
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        queue = collections.deque()                 # arrived, not yet admitted (FIFO)
        admitted = collections.OrderedDict()        # class -> resident requests not yet running
        running = []                                # (future, lane, batch)
        free = list(range(self.lanes))
        done = []
        busy_tracks = set()  # tracks with a request admitted or running: the next one waits for it
        while pending or queue or any(admitted.values()) or running:
            now = self.clock()
            progressed = False
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            while queue:
                r = queue[0]
                if r.track_id is not None:
                    if r.track_id in busy_tracks:
                        break  # requests of one track are answered in order, each extending the last
                    r.prior_steps = self.ex.resident_steps(r.track_id) if hasattr(self.ex, "resident_steps") else 0
                if hasattr(self.ex, "workspace_bytes") and not r.workspace:
                    r.workspace = self.ex.workspace_bytes(r)
                f = footprint(r)
                if f > self.budget:
                    raise ValueError(f"request {r.rid} needs {f} bytes, above the HBM budget {self.budget}")
                if self.in_use + f > self.budget:
                    break
                queue.popleft()
                self.ex.upload(r)
                if r.track_id is not None:
                    busy_tracks.add(r.track_id)
                r.admitted = self.clock()
                self.in_use += f
                self.peak_in_use = max(self.peak_in_use, self.in_use)
                admitted.setdefault(r.key(), []).append(r)
                progressed = True
            for item in list(running):
                fut, lane, batch = item
                if not fut.done():
                    continue
                fut.result()  # re-raises a failure of the batch
                running.remove(item)
                free.append(lane)
                t = self.clock()
                for r in batch:
                    r.completed = t
                    self.ex.release(r)
                    self.in_use -= footprint(r)
                    if r.track_id is not None:
                        busy_tracks.discard(r.track_id)
                        self.in_use -= self.resident.pop(r.track_id, 0)
                        if r.keep:
                            self.resident[r.track_id] = track_bytes(r)
                            self.in_use += self.resident[r.track_id]
                    done.append(r)
                progressed = True
            while free:
                live = [k for k, v in admitted.items() if v]
                if not live:
                    break
                key = min(live, key=lambda k: admitted[k][0].arrival)
                batch, steps = [], 0
                for r in admitted[key]:
                    if batch and steps + r.steps > self.max_batch_steps:
                        break
                    batch.append(r)
                    steps += r.steps
                admitted[key] = admitted[key][len(batch):]
                lane = free.pop(0)
                t = self.clock()
                for r in batch:
                    r.started = t
                running.append((self.ex.launch(batch, lane), lane, batch))
                self.max_running = max(self.max_running, len(running))
                self.batches.append((key, len(batch), steps, lane))
                progressed = True
            if progressed:
                continue
            # nothing to do now: let time pass until the next arrival or completion
            waits = [pending[0].arrival - now] if pending else []
            waits += [f.eta() for f, _, _ in running if hasattr(f, "eta")]
            self.wait(max(0.0, min(waits)) if waits else 0.0005)
        return done


def summarize(done, makespan=None):
    lat = np.array([r.completed - r.arrival for r in done])
    steps = sum(r.steps for r in done)
    span = makespan if makespan is not None else max(r.completed for r in done) - min(r.arrival for r in done)
    return {"requests": len(done), "steps": int(steps), "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
            "throughput_steps_per_s": float(steps / span) if span > 0 else None}


def device_overlap(intervals):
    """(sum of batch durations) / (length of their union) on the device
    timeline: 1.0 when batches ran one after another, above 1 when they
    overlapped."""
    if not intervals:
        return None
    iv = sorted((a, b) for _, a, b, _ in intervals)
    busy, cur_a, cur_b = 0.0, iv[0][0], iv[0][1]
    for a, b in iv[1:]:
        if a > cur_b:
            busy += cur_b - cur_a
            cur_a, cur_b = a, b
        else:
            cur_b = max(cur_b, b)
    busy += cur_b - cur_a
    return float(sum(b - a for a, b in iv) / busy) if busy > 0 else None


def run_loads(requests=300, loads=(0.3, 0.6, 0.9), min_len=64, max_len=20000, budget_gb=16.0, fp32_refine=False,
              compact=False, calibration=64, seed=0, lanes=2, echo=False):
    """Capacity calibration, then one served stream per offered load; returns
    the summary dict (capacity, and per load p50/p99 latency, throughput,
    batches, device overlap, HBM held by the model and measured)."""
    import torch
    ex = GpuExecutor(lanes=lanes)
    stream = lambda nreq, rate, sd: request_stream(nreq, rate, seed=sd, min_len=min_len, max_len=max_len,
                                                   fp32_refine=fp32_refine, compact=compact)
    budget = budget_gb * 2 ** 30
    # capacity: steps/s of a calibration stream served back to back
    cal = stream(min(requests, calibration), 1e9, seed + 99)
    for r in cal:
        r.arrival = 0.0
    Server(ex, hbm_budget=budget).serve(cal[:8])  # warm-up
    t0 = time.perf_counter()
    done = Server(ex, hbm_budget=budget).serve(cal)
    cap_steps = sum(r.steps for r in done) / (time.perf_counter() - t0)
    # request rate at capacity, from the length distribution's mean (log-uniform:
    # (max - min) / ln(max / min)), so that a load is a fraction of capacity in steps/s
    mean_steps = (max_len - min_len) / np.log(max_len / min_len)
    cap_rate = cap_steps / mean_steps
    out = {"capacity_steps_per_s": cap_steps, "capacity_requests_per_s": cap_rate, "lanes": lanes,
           "lengths": [min_len, max_len], "compact": compact, "budget_gb": budget_gb,
           "precision": "FP32 + refinement" if fp32_refine else "FP64", "requests_per_load": requests, "loads": []}
    for load in loads:
        reqs = stream(requests, load * cap_rate, seed)
        ex.intervals.clear()
        torch.cuda.reset_peak_memory_stats()
        srv = Server(ex, hbm_budget=budget)
        done = srv.serve(reqs)
        s = summarize(done)
        span = max(r.arrival for r in reqs) - min(r.arrival for r in reqs)
        s.update({"offered_load": load, "arrival_rate_per_s": load * cap_rate,
                  "realized_load": float(sum(r.steps for r in reqs) / span / cap_steps) if span > 0 else None,
                  "batches": len(srv.batches), "mean_batch_requests": float(np.mean([b[1] for b in srv.batches])),
                  "max_batches_in_flight": srv.max_running, "device_overlap": device_overlap(ex.intervals),
                  "peak_hbm_gb_model": srv.peak_in_use / 2 ** 30,
                  "peak_hbm_gb_measured": (torch.cuda.max_memory_allocated() + sum(ex.held.values())) / 2 ** 30})
        out["loads"].append(s)
        if echo:
            print(json.dumps(s), flush=True)
    ex.close()
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--requests", type=int, default=300)
    ap.add_argument("--loads", default="0.3,0.6,0.9", help="offered loads as fractions of the measured capacity")
    ap.add_argument("--min-len", type=int, default=64)
    ap.add_argument("--max-len", type=int, default=20000)
    ap.add_argument("--budget-gb", type=float, default=16.0)
    ap.add_argument("--fp32-refine", action="store_true")
    ap.add_argument("--compact", action="store_true",
                    help="ship requests as time-invariant models + observation streams, expanded on the device")
    ap.add_argument("--calibration", type=int, default=64, help="requests of the capacity calibration")
    ap.add_argument("--lanes", type=int, default=2, help="batches that may run on the GPU at once")
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    out = run_loads(args.requests, [float(x) for x in args.loads.split(",")], args.min_len, args.max_len,
                    args.budget_gb, args.fp32_refine, args.compact, args.calibration, args.seed, args.lanes, echo=True)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
