"""The serving loop (ultimate_kalman_gb300/serve.py): scheduling rules on a
simulated clock (CPU), and on the GPU, results of requests served in mixed
batches -- with batches of other requests running beside them on other lanes
-- equal the same requests smoothed alone (bit-equal: tracks are independent,
so neither a batch nor what overlaps it changes a track's arithmetic)."""
import numpy as np
import pytest

from ultimate_kalman_gb300 import serve


class FakeFuture:
    def __init__(self, clock, finish):
        self.clock, self.finish = clock, finish

    def done(self):
        return self.clock.t >= self.finish

    def result(self):
        return None

    def eta(self):
        return max(0.0, self.finish - self.clock.t)


class FakeExecutor:
    """Records uploads and batches; a batch finishes after its steps / rate
    on the simulated clock, and `lanes` batches may run at once."""

    def __init__(self, clock, rate=1e6, lanes=1):
        self.clock, self.rate, self.lanes = clock, rate, lanes
        self.resident = set()
        self.tracks = {}   # track id -> steps kept resident
        self.batches = []
        self.running = []  # (start, finish) of every batch

    def resident_steps(self, tid):
        return self.tracks.get(tid, 0)

    def upload(self, r):
        self.resident.add(r.rid)

    def release(self, r):
        self.resident.discard(r.rid)
        if r.track_id is not None:
            if r.keep:
                self.tracks[r.track_id] = r.steps
            else:
                self.tracks.pop(r.track_id, None)

    def launch(self, batch, lane):
        assert all(r.rid in self.resident for r in batch)
        self.batches.append([r.rid for r in batch])
        finish = self.clock.t + sum(r.steps for r in batch) / self.rate
        self.running.append((self.clock.t, finish))
        for r in batch:
            r.state = np.zeros((r.steps, r.problem.n))
        return FakeFuture(self.clock, finish)


class Clock:
    t = 0.0

    def __call__(self):
        return self.t

    def wait(self, dt):
        self.t += max(dt, 1e-6)


def make_stream(nreq=40, rate=200.0, seed=3):
    return serve.request_stream(nreq, rate, seed=seed, dims=(4, 6, 12), min_len=64, max_len=600)


def test_admission_respects_the_budget_and_every_request_completes():
    clock = Clock()
    reqs = make_stream()
    budget = 3 * max(serve.footprint(r) for r in reqs)
    ex = FakeExecutor(clock)
    srv = serve.Server(ex, hbm_budget=budget, clock=clock, wait=clock.wait)
    done = srv.serve(reqs)
    assert sorted(r.rid for r in done) == list(range(len(reqs)))
    assert srv.peak_in_use <= budget
    assert srv.in_use == 0 and not ex.resident
    for r in done:
        assert r.admitted >= r.arrival and r.completed >= r.admitted


def test_batches_are_one_shape_class_in_arrival_order():
    clock = Clock()
    reqs = make_stream(nreq=60, rate=2000.0)
    by_id = {r.rid: r for r in reqs}
    ex = FakeExecutor(clock, rate=2e5)
    srv = serve.Server(ex, hbm_budget=1 << 40, clock=clock, wait=clock.wait)
    srv.serve(reqs)
    for b in ex.batches:
        keys = {by_id[i].key() for i in b}
        assert len(keys) == 1
        arr = [by_id[i].arrival for i in b]
        assert arr == sorted(arr)
    assert max(len(b) for b in ex.batches) > 1  # requests were batched


def test_batch_step_limit():
    clock = Clock()
    reqs = make_stream(nreq=30, rate=1e5)
    ex = FakeExecutor(clock)
    limit = 1500
    srv = serve.Server(ex, hbm_budget=1 << 40, max_batch_steps=limit, clock=clock, wait=clock.wait)
    srv.serve(reqs)
    by_id = {r.rid: r for r in reqs}
    for b in ex.batches:
        steps = sum(by_id[i].steps for i in b)
        assert steps <= limit or len(b) == 1


def test_request_larger_than_the_budget_is_refused():
    clock = Clock()
    reqs = make_stream(nreq=3)
    srv = serve.Server(FakeExecutor(clock), hbm_budget=16, clock=clock, wait=clock.wait)
    with pytest.raises(ValueError):
        srv.serve(reqs)


def test_lanes_admit_and_start_batches_while_others_run():
    """With two lanes a second batch starts before the first one finishes, and
    requests that arrive meanwhile are admitted (not held until the GPU is
    idle)."""
    clock = Clock()
    reqs = make_stream(nreq=40, rate=400.0, seed=4)
    ex = FakeExecutor(clock, rate=5e4, lanes=2)
    srv = serve.Server(ex, hbm_budget=1 << 40, clock=clock, wait=clock.wait)
    done = srv.serve(reqs)
    assert len(done) == len(reqs)
    assert srv.max_running == 2
    iv = sorted(ex.running)
    assert any(b[0] < a[1] for a, b in zip(iv, iv[1:]))  # some batches overlapped
    admitted_while_busy = [r for r in done if any(a < r.admitted < b for a, b in iv)]
    assert admitted_while_busy


def test_footprint_counts_the_library_workspace():
    r = make_stream(nreq=1)[0]
    base = serve.footprint(r)
    r.workspace = 12345
    assert serve.footprint(r) == base + 12345


def test_device_overlap_measure():
    assert serve.device_overlap([(0, 0.0, 1.0, []), (1, 1.0, 2.0, [])]) == 1.0
    assert serve.device_overlap([(0, 0.0, 2.0, []), (1, 0.0, 2.0, [])]) == 2.0
    assert serve.device_overlap([(0, 0.0, 2.0, []), (1, 1.0, 3.0, [])]) == pytest.approx(4.0 / 3.0)


@pytest.mark.gpu
@pytest.mark.parametrize("fp32", [False, True])
def test_served_results_equal_results_alone(fp32):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from ultimate_kalman_gb300 import native
    reqs = serve.request_stream(24, 1e6, seed=11, dims=(4, 6, 12), min_len=64, max_len=3000, fp32_refine=fp32)
    ex = serve.GpuExecutor(lanes=2)
    srv = serve.Server(ex, hbm_budget=1 << 32)
    done = srv.serve(reqs)
    ex.close()
    assert len(srv.batches) < len(reqs)  # some requests shared a batch
    for r in done:
        X, _ = native.smooth(r.problem, covariance=False, fp32_refine=fp32)
        np.testing.assert_array_equal(r.state, X)


@pytest.mark.gpu
def test_two_batches_in_flight_overlap_on_the_device_and_match_alone():
    """Requests of two shape classes arrive together; with two lanes both
    batches are on the GPU at once (their device intervals intersect) and every
    result equals the request smoothed alone, bit for bit.  Each batch holds one
    request (max_batch_steps below two requests' steps), so a batch needs no
    device-side concatenation before its start is recorded: the interval
    starts when the lane's stream reaches the smoothing, not when a copy
    kernel queued behind the other lane's kernels gets an SM."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from ultimate_kalman_gb300 import native
    rng = np.random.default_rng(21)
    problems = [serve.serving_track(40000 if n == 12 else 60000, n, n // 2, rng) for n in [12, 6, 12, 6, 12, 6]]
    ex = serve.GpuExecutor(lanes=2)
    for _ in range(2):  # the first pass warms the lanes (workspaces, kernel loading), the second is checked
        reqs = [serve.Request(i, 0.0, P, covariance=(P.n == 6)) for i, P in enumerate(problems)]
        ex.intervals.clear()
        srv = serve.Server(ex, hbm_budget=1 << 36, max_batch_steps=60000)
        done = srv.serve(reqs)
    ex.close()
    assert srv.max_running == 2
    iv = sorted((a, b) for _, a, b, _ in ex.intervals)
    assert any(b[0] < a[1] for a, b in zip(iv, iv[1:])), iv
    assert serve.device_overlap(ex.intervals) > 1.0
    for r in done:
        X, S = native.smooth(r.problem, covariance=r.covariance)
        np.testing.assert_array_equal(r.state, X)
        if r.covariance:
            np.testing.assert_array_equal(r.cov, S)


@pytest.mark.gpu
def test_library_workspace_figure_is_what_a_call_holds():
    """kalman_gpu_oddeven_workspace_bytes equals the workspace a fresh host
    thread holds after smoothing the problem (per-thread and CTA kernels, FP64
    and the precision form)."""
    import threading
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from ultimate_kalman_gb300 import native, problem as pb
    cases = [(pb.constant_velocity([300, 41], seed=1), dict(covariance=True)),
             (pb.constant_velocity([300, 41], seed=1), dict(covariance=False, fp32_refine=True)),
             (pb.random_dynamics([200, 33], 12, 6, seed=2), dict(covariance=True)),
             (pb.random_dynamics([200, 33], 12, 6, seed=2), dict(covariance=False, fp32_refine=True))]
    for P, kw in cases:
        D = native.DeviceProblem(P, covariance=kw["covariance"])
        got = {}

        def work():
            torch.cuda.set_device(0)
            D.smooth("oddeven", **kw)
            torch.cuda.synchronize()
            got["held"] = native.workspace_held()
            native.release()

        th = threading.Thread(target=work)
        th.start()
        th.join()
        want = native.oddeven_workspace_bytes(D.struct, **kw)
        assert want > 0 and got["held"] == want, (P.n, kw, got, want)


def test_compact_requests_expand_to_the_packed_track():
    """A TrackSpec's packed arrays (host) have the bytes footprint() counts and
    the layout of serving_track's problems."""
    rng = np.random.default_rng(5)
    spec = serve.serving_spec(50, 6, 3, rng)
    P = spec.to_packed()
    assert P.nsteps == 50 and P.n == 6 and P.mmax == 6
    assert spec.nbytes() == P.nbytes()
    assert (P.obs_rows[1:] == 3).all() and P.obs_rows[0] == 6
    np.testing.assert_array_equal(P.F[7], spec.F.T)
    np.testing.assert_array_equal(P.G[7][:, :3], spec.G.T)
    r = serve.request_stream(3, 10.0, seed=2, dims=(4,), max_len=100, compact=True)
    assert all(isinstance(x.problem, serve.TrackSpec) for x in r)
    assert serve.footprint(r[0]) == serve.footprint(serve.Request(0, 0.0, r[0].problem.to_packed()))


@pytest.mark.gpu
def test_compact_requests_served_equal_packed_alone():
    """Compact requests, expanded on the device at admission, give the results
    of their packed tracks smoothed alone (bit-equal)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from ultimate_kalman_gb300 import native
    reqs = serve.request_stream(12, 1e6, seed=13, dims=(4, 6, 12), min_len=64, max_len=3000, compact=True)
    ex = serve.GpuExecutor()
    srv = serve.Server(ex, hbm_budget=1 << 32)
    done = srv.serve(reqs)
    ex.close()
    for r in done:
        X, _ = native.smooth(r.problem.to_packed(), covariance=False)
        np.testing.assert_array_equal(r.state, X)


def test_resident_tracks_are_extended_in_order_and_accounted():
    """Requests of one track are admitted one at a time, each extending the
    steps kept from the last; HBM held afterwards is exactly the kept tracks'
    equations."""
    clock = Clock()
    rng = np.random.default_rng(8)
    full = serve.serving_track(900, 4, 2, rng)
    pieces = [full.step_range(0, 300), full.step_range(300, 700), full.step_range(700, 900)]
    reqs = [serve.Request(i, 0.001 * i, P, track_id="t", keep=(i < 2)) for i, P in enumerate(pieces)]
    other = make_stream(nreq=10, rate=5000.0, seed=9)
    for j, r in enumerate(other):
        r.rid = 100 + j
    ex = FakeExecutor(clock, rate=1e5, lanes=2)
    srv = serve.Server(ex, hbm_budget=1 << 40, clock=clock, wait=clock.wait)
    done = srv.serve(reqs + other)
    by = {r.rid: r for r in done}
    assert [by[i].steps for i in range(3)] == [300, 700, 900]
    assert by[0].completed <= by[1].admitted and by[1].completed <= by[2].admitted
    assert srv.in_use == 0 and not srv.resident and not ex.tracks  # the last request did not keep it
    srv2 = serve.Server(ex, hbm_budget=1 << 40, clock=clock, wait=clock.wait)
    kept = [serve.Request(0, clock.t, pieces[0], track_id="u", keep=True)]
    srv2.serve(kept)
    assert srv2.in_use == serve.track_bytes(kept[0]) == srv2.resident["u"]


@pytest.mark.gpu
def test_resident_track_extensions_equal_the_whole_track_alone():
    """A track served in three requests -- the first keeps it on the device,
    the next two append their steps -- gives, for every request, the smoothing
    of the track so far, bit for bit; only each request's new steps are
    uploaded."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from ultimate_kalman_gb300 import native
    rng = np.random.default_rng(17)
    full = serve.serving_track(6000, 6, 3, rng)
    cuts = [0, 3000, 5000, 6000]
    pieces = [full.step_range(a, b) for a, b in zip(cuts, cuts[1:])]
    reqs = [serve.Request(i, 0.0, P, track_id=42, keep=(i < 2)) for i, P in enumerate(pieces)]
    others = serve.request_stream(6, 1e6, seed=19, dims=(6,), min_len=64, max_len=2000)
    for j, r in enumerate(others):
        r.rid = 10 + j
    ex = serve.GpuExecutor(lanes=2)
    srv = serve.Server(ex, hbm_budget=1 << 34)
    done = srv.serve(reqs + others)
    ex.close()
    by = {r.rid: r for r in done}
    for i in range(3):
        X, _ = native.smooth(full.step_range(0, cuts[i + 1]), covariance=False)
        np.testing.assert_array_equal(by[i].state, X)
    assert ex.uploaded_bytes == sum(P.nbytes() for P in pieces) + sum(r.problem.nbytes() for r in others)
    assert not ex.resident and srv.in_use == 0
