"""Invalid arguments at the drop-in boundary are refused with KALMAN_GPU_EINVAL
and a message -- never a crash, never a silent success.  The checks run before
the device is touched, so this runs on any machine.  (The reference asserts or
dereferences bad pointers on such input; a library loaded into a caller's
process must not.)"""
import ctypes

import numpy as np
import pytest

from ultimate_kalman_gb300 import native, problem as pb

EINVAL = native.KALMAN_GPU_EINVAL


@pytest.fixture(scope="module")
def lib():
    return native.load()


def packed_struct(P, keep, location=native.KALMAN_GPU_HOST):
    s = native.ProblemStruct()
    s.n, s.mmax, s.ntracks, s.location, s.nsteps = P.n, P.mmax, P.ntracks, location, P.nsteps
    ts = np.ascontiguousarray(P.track_start, dtype=np.int64)
    keep.append(ts)
    s.track_start = ts.ctypes.data
    for f in native._FIELDS:
        a = np.ascontiguousarray(getattr(P, f))
        keep.append(a)
        setattr(s, f, a.ctypes.data)
    st = np.zeros((P.nsteps, P.n))
    cv = np.zeros((P.nsteps, P.n, P.n))
    keep += [st, cv]
    s.state, s.covariance = st.ctypes.data, cv.ctypes.data
    return s


PACKED_CASES = {
    "state dimension 0": lambda s, ts: setattr(s, "n", 0),
    "negative mmax": lambda s, ts: setattr(s, "mmax", -1),
    "no tracks": lambda s, ts: setattr(s, "ntracks", 0),
    "unknown location": lambda s, ts: setattr(s, "location", 7),
    "track_start[0] != 0": lambda s, ts: ts.__setitem__(0, 1),
    "decreasing track_start": lambda s, ts: ts.__setitem__(1, ts[2] + 1),
    "steps not the sum of the tracks": lambda s, ts: setattr(s, "nsteps", int(ts[-1]) + 1),
    "NULL evolution block": lambda s, ts: setattr(s, "H", None),
    "NULL observation block": lambda s, ts: setattr(s, "G", None),
    "NULL state output": lambda s, ts: setattr(s, "state", None),
}


@pytest.mark.parametrize("case", list(PACKED_CASES))
@pytest.mark.parametrize("entry", ["kalman_gpu_smooth_oddeven_packed", "kalman_gpu_smooth_associative_packed"])
def test_packed_problem_refused(lib, case, entry):
    P = pb.constant_velocity([5, 7, 3], seed=1)
    keep = []
    s = packed_struct(P, keep)
    ts = keep[0]
    PACKED_CASES[case](s, ts)
    assert getattr(lib, entry)(0, ctypes.byref(s), None) == EINVAL, case
    assert native.last_error()[0] == EINVAL and native.last_error()[1]


def test_null_problem_refused(lib):
    assert lib.kalman_gpu_smooth_oddeven_packed(0, None, None) == EINVAL
    assert lib.kalman_gpu_smooth_oddeven_noalloc(0, None, None) == EINVAL


def step_structs(P, keep):
    """(kalman_step_equations_t* array, the structs it points to)"""
    arr, held, structs = native.build_equations(P)
    keep += [arr, held, structs]
    return arr, structs


def mutate(structs, s, **fields):
    for k, v in fields.items():
        setattr(structs[s], k, v)


def bad_matrix(rows, cols, ld, keep, elements=True):
    A = np.zeros(max(1, ld * cols))
    keep.append(A)
    m = native.Matrix(rows, cols, ld, A.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if elements else None)
    keep.append(m)
    return ctypes.pointer(m)


STRUCT_CASES = {
    "state dimension 0": lambda st, k: mutate(st, 3, dimension=0),
    "H of the wrong width": lambda st, k: mutate(st, 3, H=bad_matrix(6, 5, 6, k)),
    "F of the wrong height": lambda st, k: mutate(st, 3, F=bad_matrix(5, 6, 5, k)),
    "c missing": lambda st, k: mutate(st, 3, c=None),
    "H without elements": lambda st, k: mutate(st, 3, H=bad_matrix(6, 6, 6, k, elements=False)),
    "H with ld below its rows": lambda st, k: mutate(st, 3, H=bad_matrix(6, 6, 2, k)),
    "unknown evolution covariance type": lambda st, k: mutate(st, 3, K_type=b"Q"),
    "evolution covariance of the wrong size": lambda st, k: mutate(st, 3, K=bad_matrix(5, 5, 5, k)),
    "G of the wrong width": lambda st, k: mutate(st, 4, G=bad_matrix(3, 5, 3, k)),
    "o with two columns": lambda st, k: mutate(st, 4, o=bad_matrix(3, 2, 3, k)),
    "observation covariance without elements": lambda st, k: mutate(st, 4, C=bad_matrix(3, 3, 3, k, False)),
    "unknown observation covariance type": lambda st, k: mutate(st, 4, C_type=b"x"),
}


@pytest.mark.parametrize("case", list(STRUCT_CASES))
def test_step_structs_refused(lib, case):
    P = pb.constant_velocity([9], seed=2)
    keep = []
    arr, structs = step_structs(P, keep)
    STRUCT_CASES[case](structs, keep)
    lib.kalman_smooth_oddeven(native.KALMAN_ALGORITHM_ODDEVEN, arr, P.nsteps)
    assert lib.kalman_gpu_last_status() == EINVAL, case
    # every step's outputs are NaN-filled matrices, as the reference fills missing
    # estimates (a step declared with no state gets none)
    for e in structs:
        if e.dimension < 1:
            assert not e.state
            continue
        assert e.state and np.isnan(native._read_matrix(e.state)).all()
        lib.matrix_free(e.state)
        e.state = None
        if e.covariance:
            lib.matrix_free(e.covariance)
            e.covariance = None


def test_null_equations_and_null_steps_refused(lib):
    lib.kalman_smooth_oddeven(native.KALMAN_ALGORITHM_ODDEVEN, None, 5)
    assert lib.kalman_gpu_last_status() == EINVAL
    P = pb.constant_velocity([4], seed=3)
    keep = []
    arr, _ = step_structs(P, keep)
    arr[2] = None
    lib.kalman_smooth_associative(native.KALMAN_ALGORITHM_ASSOCIATIVE, arr, P.nsteps)
    assert lib.kalman_gpu_last_status() == EINVAL


@pytest.mark.parametrize("lengths", [[5, -5], [-1], [3, 2, -1, 1]])
def test_batched_structs_with_negative_lengths_refused(lib, lengths):
    P = pb.constant_velocity([5], seed=4)
    keep = []
    arr, _ = step_structs(P, keep)
    L = (ctypes.c_int32 * len(lengths))(*lengths)
    assert lib.kalman_gpu_smooth_tracks(native.KALMAN_ALGORITHM_ODDEVEN, arr, L, len(lengths)) == EINVAL


def test_explicit_representation_misuse(lib):
    lib.kalman_create_options.restype = ctypes.c_void_p
    lib.kalman_create_options.argtypes = [ctypes.c_uint32]
    assert not lib.kalman_create_options(1)  # KALMAN_ALGORITHM_ULTIMATE is not provided
    assert lib.kalman_gpu_last_status() == EINVAL
    M = ctypes.POINTER(native.Matrix)
    lib.kalman_observe.argtypes = [ctypes.c_void_p, M, M, M, ctypes.c_char]
    lib.kalman_evolve.argtypes = [ctypes.c_void_p, ctypes.c_int32, M, M, M, M, ctypes.c_char]
    lib.kalman_free.argtypes = [ctypes.c_void_p]
    kf = lib.kalman_create_options(native.KALMAN_ALGORITHM_ODDEVEN)
    keep = []
    lib.kalman_observe(kf, bad_matrix(2, 2, 2, keep), bad_matrix(2, 1, 2, keep), bad_matrix(2, 2, 2, keep), b"C")
    assert lib.kalman_gpu_last_status() == EINVAL  # observe before any evolve
    # blocks that cannot be read are not copied; calls on NULL handles are ignored
    lib.kalman_evolve(kf, 2, None, None, None, None, b"C")
    lib.kalman_observe(kf, bad_matrix(2, 2, 1, keep), bad_matrix(2, 1, 2, keep), bad_matrix(-1, 2, 2, keep), b"C")
    lib.kalman_evolve(None, 2, None, None, None, None, b"C")
    lib.kalman_free(None)
    lib.kalman_free(kf)
