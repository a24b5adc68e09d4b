"""Prepared plans replayed as CUDA graphs (kalman_gpu_plan_*): each execution
smooths the current contents of the plan's device arrays and equals the
ordinary packed entry point on the same data.

Tolerance: bit-equal states (the same kernels run in the same order)."""
import numpy as np
import pytest

from ultimate_kalman_gb300 import native, problem as pb

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    native.load()


@pytest.mark.parametrize("shape,fp32,cov", [((6, 3), False, True), ((6, 3), True, False), ((12, 6), False, True)])
def test_plan_replays_match_direct_calls(shape, fp32, cov):
    import torch
    n, m = shape
    if n == 6:
        P = pb.constant_velocity([300, 77, 1, 2], seed=3)
    else:
        P = pb.random_dynamics([120, 33, 2], n, m, seed=3, per_step=True, missing=0.1)
    D = native.DeviceProblem(P, covariance=cov)
    plan = D.plan(covariance=cov, fp32_refine=fp32)
    rng = np.random.default_rng(0)
    for rep in range(3):
        if rep:  # new observations in place: the plan sees the arrays' current contents
            o = D.arrays["o"]
            o.add_(torch.from_numpy(0.1 * rng.standard_normal(o.shape)).to(o.device))
        plan.execute()
        assert plan.status() == 0
        Xp = D.state.clone()
        Sp = D.cov.clone() if cov else None
        D.smooth(covariance=cov, fp32_refine=fp32)
        torch.cuda.synchronize()
        assert torch.equal(Xp, D.state)
        if cov:
            assert torch.equal(Sp, D.cov)
    plan.close()


def test_plan_refuses_host_arrays():
    P = pb.constant_velocity([10], seed=1)
    L = native.load()
    s = native.ProblemStruct()
    s.n, s.mmax, s.ntracks, s.location = P.n, P.mmax, P.ntracks, native.KALMAN_GPU_HOST
    s.nsteps = P.nsteps
    ts = np.ascontiguousarray(P.track_start, dtype=np.int64)
    s.track_start = ts.ctypes.data
    arrs = {f: np.ascontiguousarray(getattr(P, f)) for f in native._FIELDS}
    for f in native._FIELDS:
        setattr(s, f, arrs[f].ctypes.data)
    state = np.zeros((P.nsteps, P.n))
    s.state = state.ctypes.data
    import ctypes
    assert not L.kalman_gpu_plan_create(native.options_for("oddeven", False), ctypes.byref(s))
    assert L.kalman_gpu_last_status() == 1
