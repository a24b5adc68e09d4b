"""A seeded sweep of random problems against the oracle: state dimensions
1..12 (and 9..40 for the thread-block kernels), observation rows 1..2n, every covariance representation of the
reference ('C', 'W', 'w', 'F', 'U') for evolution and observation noise,
missing observations, several uneven tracks per call.  Bars: 1e-10 for FP64
(odd-even and associative, states and covariances), 1e-9 for the precision
form (states, and double-float covariances).  The achieved errors are recorded
in the parity log."""
import numpy as np
import pytest

import oracle
from ultimate_kalman_gb300 import native, problem as pb

pytestmark = pytest.mark.gpu
TYPES = ["C", "W", "w", "F", "U"]


def random_case(seed):
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(1, 13))
    m = int(rng.integers(1, 2 * n + 1))
    lengths = [int(x) for x in rng.integers(1, 400, size=int(rng.integers(1, 6)))]
    kt, ct = TYPES[int(rng.integers(0, 5))], TYPES[int(rng.integers(0, 5))]
    missing = float(rng.uniform(0.0, 0.4))
    P = pb.random_dynamics(lengths, n, m, seed=seed, K_type=kt, C_type=ct, missing=missing, per_step=True)
    return P, dict(n=n, m=m, lengths=lengths, K_type=kt, C_type=ct, missing=round(missing, 2))


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    native.load()


@pytest.mark.parametrize("seed", range(48))
def test_random_problem(seed, parity_log):
    P, desc = random_case(seed)
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert st == 0, desc
    e = {}
    X, S = native.smooth(P, "oddeven")
    e["oddeven_states"], e["oddeven_covs"] = oracle.rel_err_states(X, Xo), oracle.rel_err_covs(S, So)
    X, S = native.smooth(P, "associative")
    e["assoc_states"], e["assoc_covs"] = oracle.rel_err_states(X, Xo), oracle.rel_err_covs(S, So)
    X, _ = native.smooth(P, covariance=False, fp32_refine=True)
    e["precision_states"] = oracle.rel_err_states(X, Xo)
    X, S = native.smooth(P, covariance=True, fp32_refine=True)
    e["precision_dd_states"], e["precision_dd_covs"] = oracle.rel_err_states(X, Xo), oracle.rel_err_covs(S, So)
    parity_log(f"random {desc}", **e)
    for k, v in e.items():
        assert v < (1e-9 if k.startswith("precision") else 1e-10), (k, v, desc)


def random_large_case(seed):
    """Sizes of the thread-block kernels (n from 9 to 40), shorter tracks."""
    rng = np.random.default_rng(5000 + seed)
    n = int(rng.integers(9, 41))
    m = int(rng.integers(1, 2 * n + 1))
    lengths = [int(x) for x in rng.integers(1, 120, size=int(rng.integers(1, 4)))]
    kt, ct = TYPES[int(rng.integers(0, 5))], TYPES[int(rng.integers(0, 5))]
    missing = float(rng.uniform(0.0, 0.3))
    P = pb.random_dynamics(lengths, n, m, seed=seed, K_type=kt, C_type=ct, missing=missing, per_step=True)
    return P, dict(n=n, m=m, lengths=lengths, K_type=kt, C_type=ct, missing=round(missing, 2))


@pytest.mark.parametrize("seed", range(8))
def test_random_problem_large_states(seed, parity_log):
    P, desc = random_large_case(seed)
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert st == 0, desc
    e = {}
    X, S = native.smooth(P, "oddeven")
    e["oddeven_states"], e["oddeven_covs"] = oracle.rel_err_states(X, Xo), oracle.rel_err_covs(S, So)
    X, S = native.smooth(P, "associative")
    e["assoc_states"], e["assoc_covs"] = oracle.rel_err_states(X, Xo), oracle.rel_err_covs(S, So)
    X, _ = native.smooth(P, covariance=False, fp32_refine=True)
    e["precision_states"] = oracle.rel_err_states(X, Xo)
    X, S = native.smooth(P, covariance=True, fp32_refine=True)
    e["precision_dd_states"], e["precision_dd_covs"] = oracle.rel_err_states(X, Xo), oracle.rel_err_covs(S, So)
    parity_log(f"random large {desc}", **e)
    for k, v in e.items():
        assert v < (1e-9 if k.startswith("precision") else 1e-10), (k, v, desc)
