"""The allocation-free odd-even entry point, kalman_gpu_smooth_oddeven_noalloc.

Some callers cannot allocate device memory while they run: real-time tracking
loops that forbid it (cudaMalloc/cudaFree may synchronize the device and take
unbounded time), and plugins whose host program owns every device allocation.
For them the library keeps a fixed scratch array on each device; the caller
allocates only the inputs and outputs.  These tests call the entry point
through the C ABI and check it against the ordinary entry point on two calls
in a row (the second one finds the first one's leftovers in the shared array),
and check that problems larger than the array are refused.  This file is
collected last so that a run that stops at the first failure has run every
other test first."""
import ctypes

import numpy as np
import pytest

import oracle
from ultimate_kalman_gb300 import native, problem as pb

pytestmark = pytest.mark.gpu
TOL = 1e-11  # the same relative-error bar as the other FP64 parity tests


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return native.load()


def run_noalloc(L, D, covariance=True, opts=None):
    """Calls the allocation-free entry point on the device arrays of D, writing
    into freshly allocated output buffers of the caller."""
    import torch
    state = torch.full_like(D.state, float("nan"))
    cov = torch.full_like(D.cov, float("nan")) if covariance else None
    s = native.ProblemStruct.from_buffer_copy(D.struct)
    s.state = state.data_ptr()
    s.covariance = cov.data_ptr() if covariance else None
    if opts is None:
        opts = native.options_for("oddeven", covariance)
    st = torch.cuda.current_stream()
    status = L.kalman_gpu_smooth_oddeven_noalloc(opts, ctypes.byref(s), ctypes.c_void_p(st.cuda_stream))
    X = state.cpu().numpy()
    S = np.ascontiguousarray(cov.cpu().numpy().transpose(0, 2, 1)) if covariance else None
    return status, X, S


def rel(a, b):
    num = np.abs(a - b).reshape(len(a), -1).max(axis=1)
    den = np.abs(b).reshape(len(b), -1).max(axis=1)
    return float((num / den).max())


def test_matches_ordinary_entry_point_on_consecutive_calls(lib):
    problems = [pb.constant_velocity([700, 33, 1], seed=1),
                pb.random_dynamics([150, 9, 64], 5, 3, seed=2, per_step=True, missing=0.2, K_type="w", C_type="F")]
    for P in problems:
        D = native.DeviceProblem(P, covariance=True)
        D.smooth("oddeven", covariance=True)
        Xr, Sr = D.results()
        status, X, S = run_noalloc(lib, D)
        assert status == 0, native.last_error()
        assert rel(X, Xr) < TOL
        assert rel(S, Sr) < TOL
        status, X2, _ = run_noalloc(lib, D, covariance=False)
        assert status == 0
        assert rel(X2, Xr) < TOL


# Shapes at which the ordinary entry point runs CTA kernels (n >= 9 or more
# than 8 observation rows) while this entry point keeps the per-thread ones.
LARGE_SHAPES = [(12, 6, [900, 77, 2]), (24, 12, [300, 41]), (6, 12, [800, 65])]


@pytest.mark.parametrize("n,m,lengths", LARGE_SHAPES, ids=[f"n{n}_m{m}" for n, m, _ in LARGE_SHAPES])
def test_larger_shapes_match_ordinary_entry_point_and_oracle(lib, n, m, lengths):
    P = pb.random_dynamics(lengths, n, m, seed=n + m, per_step=False, missing=0.1)
    D = native.DeviceProblem(P, covariance=True)
    D.smooth("oddeven", covariance=True)
    Xr, Sr = D.results()
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert st == 0
    for call in range(2):  # the second call finds the first one's contents in the array
        status, X, S = run_noalloc(lib, D)
        assert status == 0, native.last_error()
        assert rel(X, Xr) < TOL and rel(S, Sr) < TOL, (call, rel(X, Xr), rel(S, Sr))
        assert rel(X, Xo) < TOL and rel(S, So) < TOL, (call, rel(X, Xo), rel(S, So))


def test_refuses_the_precision_form(lib):
    P = pb.constant_velocity([50], seed=6)
    D = native.DeviceProblem(P, covariance=False)
    opts = native.options_for("oddeven", False) | native.KALMAN_GPU_FP32_REFINE
    status, X, _ = run_noalloc(lib, D, covariance=False, opts=opts)
    assert status == 1
    assert "plain FP64" in native.last_error()[1]


def test_refuses_problems_beyond_the_scratch_array(lib):
    P = pb.constant_velocity([120000], seed=3)
    D = native.DeviceProblem(P, covariance=True)
    status, X, _ = run_noalloc(lib, D)
    assert status == 1
    st, msg = native.last_error()
    assert "bytes of scratch" in msg and str(64 << 20) in msg


def test_refuses_host_arrays(lib):
    P = pb.constant_velocity([10], seed=4)
    s = native.ProblemStruct()
    s.n, s.mmax, s.ntracks, s.location = P.n, P.mmax, P.ntracks, native.KALMAN_GPU_HOST
    s.nsteps = P.nsteps
    ts = np.ascontiguousarray(P.track_start)
    s.track_start = ts.ctypes.data
    arrs = {f: np.ascontiguousarray(getattr(P, f)) for f in native._FIELDS}
    for f in native._FIELDS:
        setattr(s, f, arrs[f].ctypes.data)
    out = np.zeros((P.nsteps, P.n))
    s.state = out.ctypes.data
    assert lib.kalman_gpu_smooth_oddeven_noalloc(native.KALMAN_NO_COVARIANCE | 4, ctypes.byref(s), None) == 1
