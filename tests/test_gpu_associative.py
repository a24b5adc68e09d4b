"""Parity of the CUDA associative-scan smoother (through the C ABI) with the
oracle's restatement, the reference's own outputs and the dense solution.

Tolerance: 1e-11 relative error (normwise per step, states and covariances),
against the oracle's associative and odd-even smoothers and the reference's
outputs.  The kernels solve the combines' systems by QR, and reach about
5e-15 on states and 3e-14 on covariances on these cases (the achieved
errors are recorded through the parity_log fixture)."""
import numpy as np
import pytest

import oracle
from ultimate_kalman_gb300 import native, problem as pb

pytestmark = pytest.mark.gpu
TOL = 1e-11


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    native.load()


def check(P, X, S, log, case, tol=TOL):
    st, Xo, So = oracle.smooth(P, "associative")
    assert st == 0
    st, Xe, Se = oracle.smooth(P, "oddeven")
    e = dict(states_vs_oracle_assoc=oracle.rel_err_states(X, Xo), covs_vs_oracle_assoc=oracle.rel_err_covs(S, So),
             states_vs_oracle_oddeven=oracle.rel_err_states(X, Xe), covs_vs_oracle_oddeven=oracle.rel_err_covs(S, Se))
    log("associative " + case, **e)
    assert max(e.values()) < tol, e


def test_golden_against_reference(golden, parity_log):
    P, d = golden
    if "X_associative" not in d:
        pytest.skip("the reference associative smoother does not accept this input")
    X, S = native.smooth(P, "associative")
    Sr = d["S_associative"]
    ok = np.all(np.isfinite(Sr), axis=(1, 2))  # the reference's last covariance is NaN
    e = dict(states_vs_reference=oracle.rel_err_states(X, d["X_associative"]),
             covs_vs_reference=oracle.rel_err_covs(S[ok], Sr[ok]))
    parity_log("associative golden", **e)
    assert max(e.values()) < TOL, e
    assert oracle.rel_err_covs(S[-1:], d["S_ultimate"][-1:]) < TOL
    check(P, X, S, parity_log, "golden")


@pytest.mark.parametrize("k", list(range(1, 12)) + [16, 17, 31, 33, 64, 100, 129])
def test_lengths(k, parity_log):
    P = pb.constant_velocity([k], seed=k)
    X, S = native.smooth(P, "associative")
    check(P, X, S, parity_log, f"k={k}")


@pytest.mark.parametrize("n,m", [(2, 1), (3, 5), (4, 2), (6, 3), (8, 4)])
@pytest.mark.parametrize("cov", ["C", "W", "w", "F"])
def test_shapes_cov_types_missing(n, m, cov, parity_log):
    P = pb.random_dynamics([12, 5, 1, 9, 2], n, m, seed=n * 7 + m, K_type=cov, C_type=cov, missing=0.3,
                           per_step=True)
    X, S = native.smooth(P, "associative")
    check(P, X, S, parity_log, f"n={n} m={m} {cov}")


def test_batched_uneven_tracks(parity_log):
    lens = pb.batched_lengths(200, 1, 800, seed=5)
    P = pb.constant_velocity(lens, seed=6, missing=0.05)
    X, S = native.smooth(P, "associative")
    check(P, X, S, parity_log, "200 uneven tracks")


def test_full_size_single_track(parity_log):
    P = pb.constant_velocity([100000], seed=12)
    X, S = native.smooth(P, "associative")
    check(P, X, S, parity_log, "k=100000")


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
def test_larger_states_cta_path(n, k, parity_log):
    """State dimensions past 8 run one thread block per element or combine:
    parity with the oracle, with missing observations and short tracks."""
    P = pb.random_dynamics([k, 37, 2], n, n // 2, seed=5 + n, per_step=True, missing=0.1)
    X, S = native.smooth(P, algorithm="associative")
    check(P, X, S, parity_log, f"CTA n={n}")


def test_n48_m24_covariance_types(parity_log):
    """n = 48, m = 24 (the associative benchmark shape) with the 'W' and 'w'
    covariance forms."""
    P = pb.random_dynamics([33, 4], 48, 24, seed=77, per_step=True, K_type="W", C_type="w", missing=0.05)
    X, S = native.smooth(P, algorithm="associative")
    check(P, X, S, parity_log, "n=48 W/w")


def test_n48_m24_long_track_with_missing_observations(parity_log):
    """The associative benchmark's model (n = 48, m = 24, F = 0.99 Q, G ~ N(0,
    1/m), SPD noise with eigenvalues in [0.1, 1]) on a 2,000-step track with 5 %
    of steps unobserved (the reference smoother rejects missing observations;
    the oracle restates the fix of treating them as e = 0, J = 0)."""
    from ultimate_kalman_gb300 import shapes
    P = shapes.synthetic_track(2000, 48, 24, missing=0.05, seed=3)
    assert (P.obs_rows[1:] == 0).sum() > 50
    X, S = native.smooth(P, algorithm="associative")
    check(P, X, S, parity_log, "n=48 k=2000 5% missing")
