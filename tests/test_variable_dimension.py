"""Steps with different state dimensions, through the reference entry points.

The reference's step structure carries a dimension per step and an evolution
with l_i rows (H_i is l_i x n_i, F_i is l_i x n_{i-1}; c/kalman.h:56-75), and
its test catalogue grows the state along a track
(matlab/examples/kalmanTest.m:93-94).  The library pads such problems to the
largest dimension with dummy components that no real equation touches, so the
results must equal the dense least-squares solution of the caller's own
problem.  The dense solution here is written for variable dimensions (the
oracle's packed problems have one dimension); the bar is the odd-even parity
bar, 1e-11."""
import ctypes

import numpy as np
import pytest

from ultimate_kalman_gb300 import native

# (n_i, l_i, m_i) per step; l_0 is unused.  The reference catalogue's two
# growing-state cases, and longer tracks that grow and shrink.
CASES = {
    "grow_2": [(1, 1, 1), (1, 1, 2)],
    "grow_7": [(1, 1, 1), (1, 1, 1), (2, 1, 2), (3, 2, 3), (3, 3, 0), (3, 2, 3), (4, 2, 3)],
    "grow_shrink_40": [(2 + (i % 7) // 2 if i < 20 else 5 - (i % 5) // 2, None, 2 + (i % 3)) for i in range(40)],
}


def make_case(spec, seed, square=False):
    """Random equations for a list of (n, l, m); l None means l = n.  With
    square, every evolution has l = n and H = I (the associative smoother's
    model)."""
    rng = np.random.default_rng(seed)
    steps = []
    for i, (n, l, m) in enumerate(spec):
        l = n if (l is None or square) else l
        st = {"n": n, "m": m}
        if i > 0:
            npv = steps[-1]["n"]
            st["H"] = np.eye(n) if square else rng.standard_normal((l, n))
            st["F"] = 0.9 * rng.standard_normal((l, npv)) / np.sqrt(npv)
            st["c"] = rng.standard_normal(l)
            A = rng.standard_normal((l, l))
            st["K"] = A @ A.T / l + 0.5 * np.eye(l)
        if m > 0:
            st["G"] = rng.standard_normal((m, n))
            st["o"] = rng.standard_normal(m)
            B = rng.standard_normal((m, m))
            st["C"] = B @ B.T / m + 0.5 * np.eye(m)
        steps.append(st)
    return steps


def dense(steps):
    """Dense weighted least squares of the whole track: (states, covariance blocks)."""
    off = np.cumsum([0] + [s["n"] for s in steps])
    N = off[-1]
    rows, rhs = [], []
    for i, s in enumerate(steps):
        if i > 0:
            W = np.linalg.inv(np.linalg.cholesky(s["K"]))
            r = np.zeros((len(s["c"]), N))
            r[:, off[i]:off[i + 1]] = s["H"]
            r[:, off[i - 1]:off[i]] = -s["F"]
            rows.append(W @ r)
            rhs.append(W @ s["c"])
        if s["m"] > 0:
            W = np.linalg.inv(np.linalg.cholesky(s["C"]))
            r = np.zeros((s["m"], N))
            r[:, off[i]:off[i + 1]] = s["G"]
            rows.append(W @ r)
            rhs.append(W @ s["o"])
    A, b = np.vstack(rows), np.concatenate(rhs)
    assert np.linalg.matrix_rank(A) == N, "the test problem must be full rank"
    x = np.linalg.lstsq(A, b, rcond=None)[0]
    S = np.linalg.inv(A.T @ A)
    return [x[off[i]:off[i + 1]] for i in range(len(steps))], [S[off[i]:off[i + 1], off[i]:off[i + 1]]
                                                               for i in range(len(steps))]


def equations(steps, keep):
    arr = (ctypes.POINTER(native.StepEquations) * len(steps))()
    for i, s in enumerate(steps):
        e = native.StepEquations()
        e.step, e.dimension = i, s["n"]
        if i > 0:
            e.H, e.F = native._matrix(s["H"], keep), native._matrix(s["F"], keep)
            e.c, e.K = native._matrix(s["c"], keep), native._matrix(s["K"], keep)
            e.K_type = b"C"
        if s["m"] > 0:
            e.G, e.o, e.C = native._matrix(s["G"], keep), native._matrix(s["o"], keep), native._matrix(s["C"], keep)
            e.C_type = b"C"
        keep.append(e)
        arr[i] = ctypes.pointer(e)
    return arr


def smooth(steps, algorithm):
    L = native.load()
    keep = []
    arr = equations(steps, keep)
    f = L.kalman_smooth_oddeven if algorithm == "oddeven" else L.kalman_smooth_associative
    f(native.KALMAN_ALGORITHM_ODDEVEN if algorithm == "oddeven" else native.KALMAN_ALGORITHM_ASSOCIATIVE, arr,
      len(steps))
    status = L.kalman_gpu_last_status()
    X, S = [], []
    for i in range(len(steps)):
        e = arr[i].contents
        X.append(native._read_matrix(e.state)[:, 0] if e.state else None)
        S.append(native._read_matrix(e.covariance) if e.covariance else None)
        if e.state:
            L.matrix_free(e.state)
        if e.covariance:
            L.matrix_free(e.covariance)
    return status, X, S


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_associative_refuses_non_square_evolution():
    """The associative smoother takes H as the identity, so evolutions with
    fewer rows than states are refused (on any machine: it is checked before
    the device is used)."""
    status, X, _ = smooth(make_case(CASES["grow_7"], 1), "associative")
    assert status == native.KALMAN_GPU_EINVAL
    assert "evolution rows" in native.last_error()[1]
    assert all(np.isnan(x).all() for x in X)


def test_inconsistent_shapes_are_refused():
    steps = make_case(CASES["grow_2"], 2)
    steps[1]["F"] = np.ones((1, 2))  # the previous step has one state
    status, _, _ = smooth(steps, "oddeven")
    assert status == native.KALMAN_GPU_EINVAL


def _gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(CASES))
def test_oddeven_matches_dense_solution(case):
    _gpu()
    steps = make_case(CASES[case], 7)
    Xd, Sd = dense(steps)
    status, X, S = smooth(steps, "oddeven")
    assert status == 0, native.last_error()
    for i in range(len(steps)):
        assert X[i].shape == (steps[i]["n"],) and S[i].shape == (steps[i]["n"],) * 2
        assert rel(X[i], Xd[i]) < 1e-11 and rel(S[i], Sd[i]) < 1e-11, i


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["grow_7", "grow_shrink_40"])
def test_associative_matches_dense_solution_with_square_evolution(case):
    _gpu()
    spec = [(n, n, max(m, n) if i == 0 else m) for i, (n, _, m) in enumerate(CASES[case])]  # square first step
    steps = make_case(spec, 8, square=True)
    Xd, Sd = dense(steps)
    status, X, S = smooth(steps, "associative")
    assert status == 0, native.last_error()
    for i in range(len(steps)):
        assert rel(X[i], Xd[i]) < 1e-11 and rel(S[i], Sd[i]) < 1e-11, i


@pytest.mark.gpu
def test_explicit_representation_with_growing_state():
    """kalman_create / evolve / observe / smooth / estimate / covariance on the
    reference catalogue's growing case."""
    _gpu()
    L = native.load()
    steps = make_case(CASES["grow_7"], 9)
    Xd, Sd = dense(steps)
    L.kalman_create_options.restype = ctypes.c_void_p
    L.kalman_create_options.argtypes = [ctypes.c_uint32]
    M = ctypes.POINTER(native.Matrix)
    L.kalman_evolve.argtypes = [ctypes.c_void_p, ctypes.c_int32, M, M, M, M, ctypes.c_char]
    L.kalman_observe.argtypes = [ctypes.c_void_p, M, M, M, ctypes.c_char]
    L.kalman_smooth.argtypes = [ctypes.c_void_p]
    L.kalman_estimate.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_estimate.restype = M
    L.kalman_covariance.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_covariance.restype = M
    L.kalman_free.argtypes = [ctypes.c_void_p]
    kf = L.kalman_create_options(native.KALMAN_ALGORITHM_ODDEVEN)
    keep = []
    for i, s in enumerate(steps):
        if i == 0:
            L.kalman_evolve(kf, s["n"], None, None, None, None, b"C")
        else:
            L.kalman_evolve(kf, s["n"], native._matrix(s["H"], keep), native._matrix(s["F"], keep),
                            native._matrix(s["c"], keep), native._matrix(s["K"], keep), b"C")
        if s["m"] > 0:
            L.kalman_observe(kf, native._matrix(s["G"], keep), native._matrix(s["o"], keep),
                             native._matrix(s["C"], keep), b"C")
        else:
            L.kalman_observe(kf, None, None, None, b"C")
    L.kalman_smooth(kf)
    assert L.kalman_gpu_last_status() == 0, native.last_error()
    for i in range(len(steps)):
        x, S = L.kalman_estimate(kf, i), L.kalman_covariance(kf, i)
        assert rel(native._read_matrix(x)[:, 0], Xd[i]) < 1e-11
        assert rel(native._read_matrix(S), Sd[i]) < 1e-11
        L.matrix_free(x)
        L.matrix_free(S)
    L.kalman_free(kf)
