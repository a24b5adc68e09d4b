"""The precision form of the odd-even smoother (KALMAN_GPU_FP32_REFINE).

States only: FP32 factorization, FP64 residuals of the weighted
least-squares system and refinement sweeps with the FP32 factors.  With
covariances: the factorization and the covariance recurrence run in
double-float arithmetic (pairs of FP32 numbers, about 47 bits, on the FP32
pipe), because covariances from FP32 factors cannot get below about 1e-6.

Bar: states and covariances within 1e-9 relative error of the FP64 oracle
(the target of this form)."""
import numpy as np
import pytest

import oracle
from ultimate_kalman_gb300 import native, problem as pb

pytestmark = pytest.mark.gpu
TOL_STATE = 1e-9
TOL_COV = 1e-9


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    native.load()


def run(P, cov=False):
    return native.smooth(P, "oddeven", covariance=cov, fp32_refine=True)


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 7, 8, 16, 17, 33, 100, 257])
def test_lengths(k):
    P = pb.constant_velocity([k], seed=k)
    X, _ = run(P)
    st, Xo, _ = oracle.smooth(P, "oddeven", covariance=False)
    assert oracle.rel_err_states(X, Xo) < TOL_STATE


@pytest.mark.parametrize("n,m,cov", [(2, 1, "C"), (4, 2, "W"), (5, 3, "w"), (6, 3, "F"), (8, 4, "C")])
def test_shapes_missing(n, m, cov):
    P = pb.random_dynamics([14, 6, 1, 9, 2], n, m, seed=n + 10 * m, K_type=cov, C_type=cov, missing=0.25,
                           per_step=True)
    X, S = run(P, cov=True)
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert oracle.rel_err_states(X, Xo) < TOL_STATE
    assert oracle.rel_err_covs(S, So) < TOL_COV


def test_batched_and_full_size():
    lens = pb.batched_lengths(200, 50, 3000, seed=8)
    P = pb.constant_velocity(lens, seed=9, missing=0.05)
    X, _ = run(P)
    st, Xo, _ = oracle.smooth(P, "oddeven", covariance=False)
    assert oracle.rel_err_states(X, Xo) < TOL_STATE
    P = pb.constant_velocity([100000], seed=10)
    X, _ = run(P)
    st, Xo, _ = oracle.smooth(P, "oddeven", covariance=False)
    assert oracle.rel_err_states(X, Xo) < TOL_STATE


@pytest.mark.parametrize("n,k", [(9, 60), (12, 200), (24, 90), (48, 40)])
def test_precision_form_larger_states(n, k):
    """FP32 CTA factorization + FP64 refinement for state dimensions past 8:
    states within 1e-9 of the oracle."""
    P = pb.random_dynamics([k, 37, 1, 2], n, n // 2, seed=30 + n, per_step=True, missing=0.1)
    X, _ = native.smooth(P, covariance=False, fp32_refine=True)
    st, Xo, _ = oracle.smooth(P, "oddeven", covariance=False)
    assert st == 0
    assert oracle.rel_err_states(X, Xo) < 1e-9


@pytest.mark.parametrize("n,k", [(64, 41), (96, 23), (128, 17)])
def test_precision_form_blocked_qr(n, k):
    """64 <= n <= 128: the FP32 blocked QR (panels of 16 reflectors, trailing
    updates from their Gram matrix); after the FP64 refinement the states are
    within 1e-9 of the oracle."""
    P = pb.random_dynamics([k, 5, 2], n, n // 2, seed=70 + n, per_step=True, missing=0.1)
    X32, _ = native.smooth(P, covariance=False, fp32_refine=True)
    st, Xo, _ = oracle.smooth(P, "oddeven", covariance=False)
    assert st == 0
    assert oracle.rel_err_states(X32, Xo) < 1e-9


@pytest.mark.parametrize("k", [1, 2, 3, 5, 8, 17, 33, 257, 1000])
def test_covariances_lengths(k):
    """Every parity pattern of the recursion, with covariances: double-float
    kernels, states and covariances within 1e-9 of the oracle."""
    P = pb.constant_velocity([k, 3, 1], seed=k + 3)
    X, S = run(P, cov=True)
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert st == 0
    assert oracle.rel_err_states(X, Xo) < TOL_STATE
    assert oracle.rel_err_covs(S, So) < TOL_COV


def test_covariances_batched_and_full_size():
    """The batched workload's shape (n=6, m=3, uneven tracks, 5 % missing) and
    one 100,000-step track, with covariances."""
    lens = pb.batched_lengths(100, 50, 3000, seed=18)
    P = pb.constant_velocity(lens, seed=19, missing=0.05)
    X, S = run(P, cov=True)
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert oracle.rel_err_states(X, Xo) < TOL_STATE
    assert oracle.rel_err_covs(S, So) < TOL_COV
    P = pb.constant_velocity([100000], seed=20)
    X, S = run(P, cov=True)
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert oracle.rel_err_states(X, Xo) < TOL_STATE
    assert oracle.rel_err_covs(S, So) < TOL_COV


@pytest.mark.parametrize("n,k", [(9, 60), (12, 200), (24, 90), (48, 40), (128, 9)])
def test_covariances_larger_states(n, k):
    """CTA kernels in double-float for state dimensions past 8, with
    covariances, missing observations and a one-step track."""
    P = pb.random_dynamics([k, 37, 1, 2], n, n // 2, seed=50 + n, per_step=True, missing=0.1)
    X, S = run(P, cov=True)
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert st == 0
    assert oracle.rel_err_states(X, Xo) < TOL_STATE
    assert oracle.rel_err_covs(S, So) < TOL_COV


def test_covariances_plan_replay_equals_direct_call():
    """A CUDA-graph plan of the double-float form gives the direct call's
    results bit for bit."""
    import torch
    P = pb.constant_velocity([500, 77, 3], seed=23)
    D = native.DeviceProblem(P, covariance=True)
    D.smooth("oddeven", covariance=True, fp32_refine=True)
    X, S = D.results()
    plan = D.plan("oddeven", covariance=True, fp32_refine=True)
    D.state.zero_()
    D.cov.zero_()
    plan.execute()
    assert plan.status() == 0
    torch.cuda.synchronize()
    X2, S2 = D.results()
    plan.close()
    np.testing.assert_array_equal(X2, X)
    np.testing.assert_array_equal(S2, S)
