"""The explicit representation (kalman_create / evolve / observe / forget /
rollback / smooth / estimate / covariance, c/kalman_explicit_representation.c:
164-267) on the GPU after forget and rollback, the 'U' covariance type, and the
precision form on an ill-conditioned problem.  Parity against the oracle: 1e-11
for FP64, 1e-9 for the precision form."""
import ctypes

import numpy as np
import pytest

import oracle
from ultimate_kalman_gb300 import native, problem as pb

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    L = native.load()
    M = ctypes.POINTER(native.Matrix)
    L.kalman_create_options.restype = ctypes.c_void_p
    L.kalman_create_options.argtypes = [ctypes.c_uint32]
    L.kalman_evolve.argtypes = [ctypes.c_void_p, ctypes.c_int32, M, M, M, M, ctypes.c_char]
    L.kalman_observe.argtypes = [ctypes.c_void_p, M, M, M, ctypes.c_char]
    L.kalman_smooth.argtypes = [ctypes.c_void_p]
    L.kalman_forget.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_rollback.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_estimate.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_estimate.restype = M
    L.kalman_covariance.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_covariance.restype = M
    L.kalman_free.argtypes = [ctypes.c_void_p]
    return L


def step_matrices(P, s, keep):
    """The reference-API matrices of packed step s (one-track problem)."""
    n = P.n
    ev = None
    if s > 0:
        kt = chr(P.K_type[s])
        K = P.K[s].reshape(-1)[:n] if kt == "w" else P.K[s].T
        ev = (native._matrix(P.H[s].T, keep), native._matrix(P.F[s].T, keep), native._matrix(P.c[s], keep),
              native._matrix(K, keep), kt.encode())
    m = int(P.obs_rows[s])
    ob = None
    if m > 0:
        ct = chr(P.C_type[s])
        C = P.C[s].reshape(-1)[:m] if ct == "w" else P.C[s].T[:m, :m]
        ob = (native._matrix(P.G[s].T[:m], keep), native._matrix(P.o[s][:m], keep), native._matrix(C, keep),
              ct.encode())
    return ev, ob


def feed(L, kf, P, s, keep, observe=True):
    ev, ob = step_matrices(P, s, keep)
    if ev is None:
        L.kalman_evolve(kf, P.n, None, None, None, None, b"C")
    else:
        L.kalman_evolve(kf, P.n, *ev)
    if observe:
        if ob is None:
            L.kalman_observe(kf, None, None, None, b"C")
        else:
            L.kalman_observe(kf, *ob)


def results(L, kf, steps, n):
    X, S = [], []
    for s in steps:
        x, c = L.kalman_estimate(kf, s), L.kalman_covariance(kf, s)
        X.append(native._read_matrix(x)[:, 0])
        S.append(native._read_matrix(c))
        L.matrix_free(x)
        L.matrix_free(c)
    return np.array(X), np.array(S)


def algorithm_option(alg):
    return native.KALMAN_ALGORITHM_ODDEVEN if alg == "oddeven" else native.KALMAN_ALGORITHM_ASSOCIATIVE


# every step observed by 4 rows of 4 states: the pieces left by forget and
# rollback begin with a square observation, which the associative smoother needs
def square_problem(seed):
    return pb.random_dynamics([60], 4, 4, seed=seed, K_type="w", C_type="F", per_step=True)


@pytest.mark.parametrize("alg", ["oddeven", "associative"])
def test_forget_then_smooth(L, alg):
    """After kalman_forget(19) the held steps are 20..59; smoothing them
    equals the oracle on that piece (its first step's evolution unused)."""
    P = square_problem(61)
    keep = []
    kf = L.kalman_create_options(algorithm_option(alg))
    for s in range(60):
        feed(L, kf, P, s, keep)
    L.kalman_forget(kf, 19)
    L.kalman_smooth(kf)
    assert L.kalman_gpu_last_status() == 0, native.last_error()
    X, S = results(L, kf, range(20, 60), P.n)
    st, Xo, So = oracle.smooth(P.step_range(20, 60), alg)
    assert st == 0
    assert oracle.rel_err_states(X, Xo) < 1e-11 and oracle.rel_err_covs(S, So) < 1e-11
    L.kalman_free(kf)


@pytest.mark.parametrize("alg", ["oddeven", "associative"])
def test_rollback_and_observe_again_then_smooth(L, alg):
    """kalman_rollback(39) returns step 39 to "just evolved"; observing it
    again and smoothing gives the oracle's smoothing of steps 0..39."""
    P = square_problem(62)
    keep = []
    kf = L.kalman_create_options(algorithm_option(alg))
    for s in range(60):
        feed(L, kf, P, s, keep)
    L.kalman_rollback(kf, 39)
    _, ob = step_matrices(P, 39, keep)
    L.kalman_observe(kf, *ob)
    L.kalman_smooth(kf)
    assert L.kalman_gpu_last_status() == 0, native.last_error()
    X, S = results(L, kf, range(0, 40), P.n)
    st, Xo, So = oracle.smooth(P.step_range(0, 40), alg)
    assert st == 0
    assert oracle.rel_err_states(X, Xo) < 1e-11 and oracle.rel_err_covs(S, So) < 1e-11
    L.kalman_free(kf)


@pytest.mark.parametrize("alg", ["oddeven", "associative"])
def test_U_covariance_type(L, alg):
    P = pb.random_dynamics([40, 9, 2], 5, 3, seed=63, K_type="U", C_type="U", missing=0.1, per_step=True)
    X, S = native.smooth(P, alg)
    st, Xo, So = oracle.smooth(P, alg)
    assert st == 0
    assert oracle.rel_err_states(X, Xo) < 1e-11 and oracle.rel_err_covs(S, So) < 1e-11


@pytest.mark.parametrize("n,m", [(6, 3), (12, 6)])
def test_precision_form_ill_conditioned(L, n, m, parity_log):
    """Noise covariances with eigenvalues log-uniform in [1e-4, 1] (condition
    1e4, the weighed system's condition about 1e2 times the model's): the
    library's default two refinement sweeps meet 1e-9 on the states, and the
    double-float form 1e-9 on the covariances."""
    P = pb.random_dynamics([500, 77, 3], n, m, seed=64 + n, cov_lo=1e-4, log_cov=True, missing=0.05, per_step=True)
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert st == 0
    X, _ = native.smooth(P, covariance=False, fp32_refine=True)
    X2, S2 = native.smooth(P, covariance=True, fp32_refine=True)
    e = dict(states=oracle.rel_err_states(X, Xo), dd_states=oracle.rel_err_states(X2, Xo),
             dd_covs=oracle.rel_err_covs(S2, So))
    parity_log(f"precision form, covariance eigenvalues in [1e-4, 1], n={n}", **e)
    assert max(e.values()) < 1e-9, e
