"""The C-ABI library without a GPU: it loads, exports every function the
headers declare, and its host-side logic (explicit representation, matrix
helpers, error reporting) behaves like the reference's.  CPU only."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from ultimate_kalman_gb300 import build, native, problem as pb

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return native.load()


def header_functions():
    names = set()
    for h in ("kalman.h", "matrix_ops.h", "kalman_gpu.h", "parallel.h"):
        path = os.path.join(REPO, "include", h)
        if not os.path.exists(path):
            continue
        src = open(path).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"^\s*#.*$", "", src, flags=re.M)
        for m in re.finditer(r"([A-Za-z_]\w*)\s*\(([^;{}()]*(?:\([^()]*\)[^;{}()]*)*)\)\s*;", src):
            name = m.group(1)
            if name in ("if", "while", "sizeof", "return"):
                continue
            names.add(name)
    return names


def exported_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True, text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_every_declared_function_is_exported(lib):
    declared = header_functions()
    assert "kalman_smooth_oddeven" in declared and "matrix_create_mutate_qr" in declared
    missing = declared - exported_symbols()
    assert not missing, missing
    assert set(native.EXPORTED) <= exported_symbols() | {"kalman_nan"}
    ctypes.c_double.in_dll(lib, "kalman_nan")


def test_no_device_is_reported_not_fatal(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ultimate_kalman_gb300 import problem
    P = problem.constant_velocity([5], seed=1)
    with pytest.raises(native.KalmanError) as e:
        native.smooth(P, location="host")
    assert e.value.status == 5
    X, S, status = native.smooth_equations(P)
    assert status == 5 and np.isnan(X).all() and np.isnan(S).all()
    assert lib.kalman_gpu_check_bounded_wait(None) == native.KALMAN_GPU_ENODEV


def _mat(lib, A, keep):
    return native._matrix(A, keep)


def test_explicit_representation_bookkeeping(lib):
    """kalman_create / evolve / observe / estimate / forget / rollback follow
    c/kalman_base.c:298-460 and c/kalman_explicit_representation.c:164-244."""
    L = lib
    L.kalman_create_options.restype = ctypes.c_void_p
    L.kalman_create_options.argtypes = [ctypes.c_uint32]
    L.kalman_evolve.argtypes = [ctypes.c_void_p, ctypes.c_int32] + [ctypes.POINTER(native.Matrix)] * 4 + [ctypes.c_char]
    L.kalman_observe.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(native.Matrix)] * 3 + [ctypes.c_char]
    for f in ("kalman_earliest", "kalman_latest"):
        getattr(L, f).argtypes = [ctypes.c_void_p]
        getattr(L, f).restype = ctypes.c_int32
    L.kalman_estimate.restype = ctypes.POINTER(native.Matrix)
    L.kalman_estimate.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_covariance.restype = ctypes.POINTER(native.Matrix)
    L.kalman_covariance.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_covariance_type.restype = ctypes.c_char
    L.kalman_covariance_type.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_forget.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_rollback.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.kalman_free.argtypes = [ctypes.c_void_p]
    assert L.kalman_create_options(1) is None  # ULTIMATE is not provided
    assert b"ODDEVEN" in L.kalman_gpu_last_error()
    k = L.kalman_create_options(native.KALMAN_ALGORITHM_ODDEVEN)
    assert L.kalman_earliest(k) == -1 and L.kalman_latest(k) == -1
    keep = []
    I2 = np.eye(2)
    for i in range(6):
        if i == 0:
            L.kalman_evolve(k, 2, None, None, None, None, b"C")
        else:
            L.kalman_evolve(k, 2, _mat(L, I2, keep), _mat(L, I2, keep), _mat(L, np.zeros(2), keep),
                            _mat(L, I2, keep), b"C")
        L.kalman_observe(k, _mat(L, I2, keep), _mat(L, np.ones(2) * i, keep), _mat(L, I2, keep), b"C")
    assert L.kalman_earliest(k) == 0 and L.kalman_latest(k) == 5
    e = L.kalman_estimate(k, 3)  # not smoothed yet: NaN of the step's dimension
    assert e.contents.row_dim == 2 and np.isnan(e.contents.elements[0])
    L.matrix_free(e)
    assert L.kalman_covariance_type(k, -1) == b"C"
    L.kalman_forget(k, 1)
    assert L.kalman_earliest(k) == 2
    L.kalman_forget(k, -1)  # everything but the last step
    assert L.kalman_earliest(k) == 5 and L.kalman_latest(k) == 5
    L.kalman_rollback(k, 5)  # back to just after evolve of step 5: observe re-appends it
    assert L.kalman_latest(k) == -1
    L.kalman_observe(k, _mat(L, I2, keep), _mat(L, np.ones(2), keep), _mat(L, I2, keep), b"C")
    assert L.kalman_latest(k) == 5
    L.kalman_free(k)


def test_matrix_helpers_match_numpy(lib):
    L = lib
    R = native.Matrix
    L.matrix_create_mutate_qr.restype = ctypes.POINTER(R)
    L.matrix_create_mutate_qr.argtypes = [ctypes.POINTER(R)]
    L.matrix_mutate_apply_qt.argtypes = [ctypes.POINTER(R)] * 3
    L.matrix_create_mldivide.restype = ctypes.POINTER(R)
    L.matrix_create_mldivide.argtypes = [ctypes.POINTER(R)] * 2
    L.kalman_covariance_matrix_explicit.restype = ctypes.POINTER(R)
    L.kalman_covariance_matrix_explicit.argtypes = [ctypes.POINTER(R), ctypes.c_char]
    L.kalman_covariance_matrix_weigh.restype = ctypes.POINTER(R)
    L.kalman_covariance_matrix_weigh.argtypes = [ctypes.POINTER(R), ctypes.c_char, ctypes.POINTER(R)]
    rng = np.random.default_rng(0)
    A = rng.standard_normal((7, 4))
    keep = []
    m = _mat(L, A, keep)
    tau = L.matrix_create_mutate_qr(m)
    B = rng.standard_normal((7, 2))
    mb = _mat(L, B, keep)
    L.matrix_mutate_apply_qt(m, tau, mb)
    Rr = np.triu(native._read_matrix(m)[:4])
    QtB = native._read_matrix(mb)
    Q, Rn = np.linalg.qr(A, mode="complete")
    # R unique up to row signs; Q^T B likewise
    sgn = np.sign(np.diag(Rr)) * np.sign(np.diag(Rn[:4]))
    np.testing.assert_allclose(Rr, sgn[:, None] * Rn[:4], atol=1e-12)
    np.testing.assert_allclose(QtB[:4], sgn[:, None] * (Q.T @ B)[:4], atol=1e-12)
    S = rng.standard_normal((5, 5))
    X = native._read_matrix(L.matrix_create_mldivide(_mat(L, S, keep), _mat(L, B[:5], keep)))
    np.testing.assert_allclose(X, np.linalg.solve(S, B[:5]), rtol=1e-10)
    C = S @ S.T + np.eye(5)
    Wa = native._read_matrix(L.kalman_covariance_matrix_weigh(_mat(L, C, keep), b"C", _mat(L, B[:5], keep)))
    np.testing.assert_allclose(Wa, np.linalg.solve(np.linalg.cholesky(C), B[:5]), rtol=1e-10)
    W = np.linalg.inv(np.linalg.cholesky(C))
    Ce = native._read_matrix(L.kalman_covariance_matrix_explicit(_mat(L, W, keep), b"W"))
    np.testing.assert_allclose(Ce, C, rtol=1e-9)


def test_builder_and_filter_refuse_bad_arguments_without_touching_a_device(lib):
    """kalman_gpu_expand_invariant and kalman_gpu_filter_packed check their
    arguments on the host first: host-array problems, step ranges outside the
    problem, observation rows above mmax and unknown covariance types are
    refused with EINVAL before any CUDA call."""
    from ultimate_kalman_gb300 import problem
    P = problem.constant_velocity([5], seed=1)
    keep = []
    s = native.ProblemStruct()
    s.n, s.mmax, s.ntracks, s.location, s.nsteps = P.n, P.mmax, 1, native.KALMAN_GPU_HOST, P.nsteps
    ts = np.ascontiguousarray(P.track_start, dtype=np.int64)
    s.track_start = ts.ctypes.data
    arrs = {f: np.ascontiguousarray(getattr(P, f)) for f in native._FIELDS}
    for f, a in arrs.items():
        setattr(s, f, a.ctypes.data)
    state = np.zeros((P.nsteps, P.n))
    s.state = state.ctypes.data
    assert lib.kalman_gpu_filter_packed(native.KALMAN_NO_COVARIANCE, ctypes.byref(s), None) == native.KALMAN_GPU_EINVAL
    assert "device arrays" in native.last_error()[1]
    md = native.InvariantModel(m0=P.n, m=3, K_type=b"C", C0_type=b"W", C_type=b"C")
    assert lib.kalman_gpu_expand_invariant(ctypes.byref(s), 0, 5, ctypes.byref(md), None, 3, None, None) == \
        native.KALMAN_GPU_EINVAL  # host arrays
    s.location = native.KALMAN_GPU_DEVICE
    assert lib.kalman_gpu_expand_invariant(ctypes.byref(s), 3, 5, ctypes.byref(md), None, 3, None, None) == \
        native.KALMAN_GPU_EINVAL  # steps 3..7 of a 5-step problem
    bad = native.InvariantModel(m0=P.mmax + 1, m=3, K_type=b"C", C0_type=b"W", C_type=b"C")
    assert lib.kalman_gpu_expand_invariant(ctypes.byref(s), 0, 5, ctypes.byref(bad), None, 3, None, None) == \
        native.KALMAN_GPU_EINVAL
    bad = native.InvariantModel(m0=P.n, m=3, K_type=b"Q", C0_type=b"W", C_type=b"C")
    assert lib.kalman_gpu_expand_invariant(ctypes.byref(s), 0, 5, ctypes.byref(bad), None, 3, None, None) == \
        native.KALMAN_GPU_EINVAL
    assert "covariance types" in native.last_error()[1]


def test_bulk_equation_structs_equal_the_per_step_builder():
    """native.EquationsView (numpy-built kalman_step_equations_t arrays that
    point into the packed arrays) describes exactly the matrices that the
    per-step ctypes builder copies out: shapes, leading dimensions, values,
    missing observations and 'w' covariances."""
    import ctypes
    P = pb.random_dynamics([40, 3, 17], 4, 3, seed=3, missing=0.2, K_type="w", C_type="w")
    V = native.EquationsView(P)
    _, _, structs = native.build_equations(P)

    def mat(p):
        if not p:
            return None
        M = p.contents
        a = np.ctypeslib.as_array(M.elements, shape=(M.col_dim * M.ld,)).reshape(M.col_dim, M.ld)
        return a[:, :M.row_dim].T.copy()

    for s in range(P.nsteps):
        ev = native.StepEquations.from_address(int(V.ptrs[s]))
        e = structs[s]
        assert ev.dimension == e.dimension == P.n
        for f in ("H", "F", "K", "c", "G", "o", "C"):
            a, b = mat(getattr(ev, f)), mat(getattr(e, f))
            assert (a is None) == (b is None), (s, f)
            if a is not None:
                np.testing.assert_array_equal(a, b)
        if e.K:
            assert ev.K_type == e.K_type
        if e.o:
            assert ev.C_type == e.C_type
    assert ctypes.sizeof(native.StepEquations) == V.eq.dtype.itemsize
