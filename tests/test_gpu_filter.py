"""Filtered estimates on the device (kalman_gpu_filter_packed, the sequential
UltimateKalman filter of c/kalman_ultimate.c run per track): the estimate and
covariance of step s equal the oracle's smoothed estimate and covariance of
the last step of the track cut after s (the filtered estimate is the smoothed
one of the prefix problem).  Tolerance 1e-10 relative (states and
covariances): different elimination orders of the same FP64 least-squares
problems."""
import numpy as np
import pytest

import oracle
from ultimate_kalman_gb300 import native
from ultimate_kalman_gb300 import problem as pb

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return torch


def prefixes(P):
    """Every prefix of every track as its own track; returns the packed
    problem and, per original step, the index of its prefix's last step."""
    idx, lens, last = [], [], []
    for t in range(P.ntracks):
        a, b = int(P.track_start[t]), int(P.track_start[t + 1])
        for L in range(1, b - a + 1):
            idx.extend(range(a, a + L))
            lens.append(L)
            last.append(len(idx) - 1)
    idx = np.array(idx)
    ts = np.zeros(len(lens) + 1, dtype=np.int64)
    ts[1:] = np.cumsum(lens)
    Q = pb.PackedProblem(n=P.n, mmax=P.mmax, track_start=ts, **{f: getattr(P, f)[idx] for f in (
        "H", "F", "c", "K", "K_type", "G", "o", "C", "C_type", "obs_rows")})
    return Q, np.array(last)


@pytest.mark.parametrize("n,m,kt,ct", [(6, 3, "C", "C"), (4, 2, "W", "w"), (12, 6, "C", "W"), (9, 4, "F", "C")])
def test_filtered_estimates_equal_prefix_smoothing(n, m, kt, ct):
    _cuda()
    P = pb.random_dynamics([23, 1, 9, 14], n, m, seed=40 + n, per_step=True, missing=0.15, K_type=kt, C_type=ct)
    D = native.DeviceProblem(P, covariance=True)
    D.filter()
    X, S = D.results()
    Q, last = prefixes(P)
    st, Xo, So = oracle.smooth(Q, "oddeven", covariance=True)
    assert st == 0
    assert oracle.rel_err_states(X, Xo[last]) < TOL
    assert oracle.rel_err_covs(S, So[last]) < TOL


def test_last_filtered_estimate_is_the_smoothed_one():
    """At a track's last step filtering and smoothing use the same equations."""
    _cuda()
    P = pb.random_dynamics([300, 77], 8, 4, seed=5, missing=0.1)
    D = native.DeviceProblem(P, covariance=True)
    D.filter()
    Xf, Sf = D.results()
    D.smooth("oddeven")
    Xs, Ss = D.results()
    ends = P.track_start[1:] - 1
    assert oracle.rel_err_states(Xf[ends], Xs[ends]) < TOL
    assert oracle.rel_err_covs(Sf[ends], Ss[ends]) < TOL


def test_states_only_and_undetermined_steps():
    """Without covariances only states are written; steps whose state is not
    yet determined (step 0 unobserved, then 2 observation rows a step for 4
    states) are NaN and the call reports it."""
    torch = _cuda()
    P = pb.random_dynamics([12], 4, 2, seed=8)
    P.obs_rows[0] = 0
    P.obs_rows[1:] = 2
    D = native.DeviceProblem(P, covariance=False)
    status = D.filter(covariance=False, check=False)
    assert status == native.KALMAN_GPU_ESINGULAR
    X = D.state.cpu().numpy()
    assert np.isnan(X[:2]).all()
    assert np.isfinite(X[2:]).all()
