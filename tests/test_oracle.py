"""The oracle (oracle/kalman_oracle.c) against the reference's own outputs
(tests/golden, produced by the compiled reference C library) and against the
dense least-squares solution.  CPU only."""
import numpy as np
import pytest

import oracle
from ultimate_kalman_gb300 import problem as pb

TOL = 1e-11  # relative error bar for FP64 smoothed states and covariances


def finite_rows(S):
    return np.all(np.isfinite(S), axis=(1, 2))


def test_oracle_oddeven_matches_reference(golden):
    P, d = golden
    st, X, S = oracle.smooth(P, "oddeven")
    assert st == 0
    for alg in ("oddeven", "ultimate"):
        if f"X_{alg}" not in d:
            continue
        assert oracle.rel_err_states(X, d[f"X_{alg}"]) < TOL
        assert oracle.rel_err_covs(S, d[f"S_{alg}"]) < TOL


def test_oracle_associative_matches_reference(golden):
    P, d = golden
    if "X_associative" not in d:
        pytest.skip("the reference associative smoother does not accept this input")
    st, X, S = oracle.smooth(P, "associative")
    assert st == 0
    Sr = d["S_associative"]
    ok = finite_rows(Sr)
    # the reference leaves the last step's covariance NaN (it copies an unset field)
    assert not ok[-1] and ok[:-1].all()
    assert oracle.rel_err_states(X, d["X_associative"]) < TOL
    assert oracle.rel_err_covs(S[ok], Sr[ok]) < TOL
    # the last covariance is the filtered one, which the ultimate smoother agrees with
    assert oracle.rel_err_covs(S[-1:], d["S_ultimate"][-1:]) < TOL


def test_oracle_dense(golden):
    P, d = golden
    Xd, Sd = oracle.dense_smooth(P)
    st, X, S = oracle.smooth(P, "oddeven")
    assert oracle.rel_err_states(X, Xd) < TOL
    assert oracle.rel_err_covs(S, Sd) < TOL


@pytest.mark.parametrize("n,m", [(4, 2), (3, 6), (5, 3), (2, 1)])
@pytest.mark.parametrize("cov", ["C", "W", "w", "F"])
@pytest.mark.parametrize("k", [1, 2, 3, 6, 7, 13])
def test_oracle_shapes_against_dense(n, m, cov, k):
    """Every covariance form, tall and flat G, odd and even lengths, several
    tracks, missing observations (including consecutive and trailing ones,
    which the reference's odd-even rejects)."""
    P = pb.random_dynamics([k, k + 2, 1], n, m, seed=31 * k + n, K_type=cov, C_type=cov, missing=0.35,
                           per_step=True)
    Xd, Sd = oracle.dense_smooth(P)
    st, X, S = oracle.smooth(P, "oddeven")
    assert st == 0
    assert oracle.rel_err_states(X, Xd) < TOL
    assert oracle.rel_err_covs(S, Sd) < TOL
    st, X, S = oracle.smooth(P, "associative")
    assert st == 0
    assert oracle.rel_err_states(X, Xd) < 1e-9
    assert oracle.rel_err_covs(S, Sd) < 1e-9


def test_oracle_threads_agree():
    P = pb.constant_velocity([257], seed=3)
    _, X1, S1 = oracle.smooth(P, "oddeven", threads=1)
    _, X4, S4 = oracle.smooth(P, "oddeven", threads=4)
    np.testing.assert_array_equal(X1, X4)
    np.testing.assert_array_equal(S1, S4)


def test_oracle_unobservable_reports_singular():
    P = pb.constant_velocity([1], seed=1)
    P.obs_rows[0] = 3  # a 3x6 observation of a single step cannot determine it
    st, X, S = oracle.smooth(P, "oddeven")
    assert st == 4 and np.isnan(X).all()
