"""Parity of the CUDA associative-scan smoother (through the C ABI) with the
oracle's restatement, the reference's own outputs and the dense solution.

Tolerance: 1e-9 relative error.  The associative smoother forms explicit
inverses (like the reference), so it loses a few digits against the QR-based
odd-even smoother; the reference's own associative smoother differs from the
dense solution by up to ~4e-11 on these shapes."""
import numpy as np
import pytest

import oracle
from ultimate_kalman_gb300 import native, problem as pb

pytestmark = pytest.mark.gpu
TOL = 1e-9


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    native.load()


def check(P, X, S, tol=TOL):
    st, Xo, So = oracle.smooth(P, "associative")
    assert st == 0
    assert oracle.rel_err_states(X, Xo) < tol
    assert oracle.rel_err_covs(S, So) < tol
    st, Xe, Se = oracle.smooth(P, "oddeven")
    assert oracle.rel_err_states(X, Xe) < tol
    assert oracle.rel_err_covs(S, Se) < tol


def test_golden_against_reference(golden):
    P, d = golden
    if "X_associative" not in d:
        pytest.skip("the reference associative smoother does not accept this input")
    X, S = native.smooth(P, "associative")
    Sr = d["S_associative"]
    ok = np.all(np.isfinite(Sr), axis=(1, 2))  # the reference's last covariance is NaN
    assert oracle.rel_err_states(X, d["X_associative"]) < TOL
    assert oracle.rel_err_covs(S[ok], Sr[ok]) < TOL
    assert oracle.rel_err_covs(S[-1:], d["S_ultimate"][-1:]) < TOL
    check(P, X, S)


@pytest.mark.parametrize("k", list(range(1, 12)) + [16, 17, 31, 33, 64, 100, 129])
def test_lengths(k):
    P = pb.constant_velocity([k], seed=k)
    X, S = native.smooth(P, "associative")
    check(P, X, S)


@pytest.mark.parametrize("n,m", [(2, 1), (3, 5), (4, 2), (6, 3), (8, 4)])
@pytest.mark.parametrize("cov", ["C", "W", "w", "F"])
def test_shapes_cov_types_missing(n, m, cov):
    P = pb.random_dynamics([12, 5, 1, 9, 2], n, m, seed=n * 7 + m, K_type=cov, C_type=cov, missing=0.3,
                           per_step=True)
    X, S = native.smooth(P, "associative")
    check(P, X, S)


def test_batched_uneven_tracks():
    lens = pb.batched_lengths(200, 1, 800, seed=5)
    P = pb.constant_velocity(lens, seed=6, missing=0.05)
    X, S = native.smooth(P, "associative")
    check(P, X, S)


def test_full_size_single_track():
    P = pb.constant_velocity([100000], seed=12)
    X, S = native.smooth(P, "associative")
    check(P, X, S)


def test_reference_entry_point_with_step_structs():
    P = pb.random_dynamics([15, 3], 4, 2, seed=9, per_step=True, K_type="W", C_type="w")
    Xp, Sp = native.smooth(P, "associative")
    X1, S1, st = native.smooth_equations(P, "associative", covariance=False)
    assert st == 0 and S1 is not None  # like the reference, it always returns covariances
    np.testing.assert_array_equal(X1, Xp)
    np.testing.assert_array_equal(S1, Sp)


def test_non_square_first_observation_is_rejected():
    P = pb.constant_velocity([5], seed=2, fold=False)  # step 0 observed by 3 rows of 6
    with pytest.raises(native.KalmanError) as e:
        native.smooth(P, "associative")
    assert e.value.status == 1


@pytest.mark.parametrize("n,k", [(9, 41), (12, 200), (24, 80), (48, 30)])
def test_larger_states_cta_path(n, k):
    """State dimensions past 8 run one thread block per element or combine:
    parity with the oracle, with missing observations and short tracks."""
    P = pb.random_dynamics([k, 37, 2], n, n // 2, seed=5 + n, per_step=True, missing=0.1)
    X, S = native.smooth(P, algorithm="associative")
    st, Xo, So = oracle.smooth(P, "associative", covariance=True)
    assert st == 0
    assert oracle.rel_err_states(X, Xo) < TOL
    assert oracle.rel_err_covs(S, So) < TOL


def test_n48_m24_covariance_types():
    """n = 48, m = 24 (the associative benchmark shape) with the 'W' and 'w'
    covariance forms."""
    P = pb.random_dynamics([33, 4], 48, 24, seed=77, per_step=True, K_type="W", C_type="w", missing=0.05)
    X, S = native.smooth(P, algorithm="associative")
    st, Xo, So = oracle.smooth(P, "associative", covariance=True)
    assert st == 0
    assert oracle.rel_err_states(X, Xo) < TOL
    assert oracle.rel_err_covs(S, So) < TOL
