"""ctypes binding of libukgpu.so, the C-ABI library (include/kalman.h,
include/kalman_gpu.h).

The library is the product; this module only loads it and passes pointers.
It provides

  * ``smooth(P, ...)`` -- the packed entry points on a ``PackedProblem``, with
    the arrays either copied to the GPU first (device-resident run, the way a
    caller keeps data in HBM) or passed as host memory (the library stages them);
  * ``DeviceProblem`` -- a packed problem held in GPU memory for repeated runs;
  * ``smooth_equations(P, ...)`` -- the reference entry points
    ``kalman_smooth_oddeven`` / ``kalman_smooth_associative`` fed with
    ``kalman_step_equations_t`` structs, exactly as a C client of
    UltimateKalman's kalman.h would call them.

There is no fallback: if the library or a CUDA device is missing, calls fail.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libukgpu.so")

KALMAN_ALGORITHM_ODDEVEN = 1 << 2
KALMAN_ALGORITHM_ASSOCIATIVE = 1 << 3
KALMAN_NO_COVARIANCE = 1 << 16
KALMAN_GPU_FP32_REFINE = 1 << 20
KALMAN_GPU_DEVICE, KALMAN_GPU_HOST = 0, 1
KALMAN_GPU_OK, KALMAN_GPU_EINVAL, KALMAN_GPU_ECUDA, KALMAN_GPU_ENOMEM, KALMAN_GPU_ESINGULAR, KALMAN_GPU_ENODEV = range(6)

STATUS = {0: "OK", 1: "EINVAL", 2: "ECUDA", 3: "ENOMEM", 4: "ESINGULAR", 5: "ENODEV"}


class KalmanError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Matrix(ctypes.Structure):
    _fields_ = [("row_dim", ctypes.c_int32), ("col_dim", ctypes.c_int32), ("ld", ctypes.c_int32),
                ("elements", ctypes.POINTER(ctypes.c_double))]


class StepEquations(ctypes.Structure):
    """kalman_step_equations_t (c/kalman.h:56-75), int32 step index."""
    _fields_ = [("step", ctypes.c_int32), ("dimension", ctypes.c_int32), ("C_type", ctypes.c_char),
                ("K_type", ctypes.c_char),
                ("H", ctypes.POINTER(Matrix)), ("F", ctypes.POINTER(Matrix)), ("K", ctypes.POINTER(Matrix)),
                ("c", ctypes.POINTER(Matrix)), ("G", ctypes.POINTER(Matrix)), ("o", ctypes.POINTER(Matrix)),
                ("C", ctypes.POINTER(Matrix)), ("state", ctypes.POINTER(Matrix)),
                ("covariance", ctypes.POINTER(Matrix)), ("covariance_type", ctypes.c_char)]


class ProblemStruct(ctypes.Structure):
    """kalman_gpu_problem_t (include/kalman_gpu.h)."""
    _fields_ = [
        ("n", ctypes.c_int32), ("mmax", ctypes.c_int32), ("ntracks", ctypes.c_int32), ("location", ctypes.c_int32),
        ("nsteps", ctypes.c_int64), ("track_start", ctypes.c_void_p),
        ("H", ctypes.c_void_p), ("F", ctypes.c_void_p), ("c", ctypes.c_void_p), ("K", ctypes.c_void_p),
        ("K_type", ctypes.c_void_p), ("G", ctypes.c_void_p), ("o", ctypes.c_void_p), ("C", ctypes.c_void_p),
        ("C_type", ctypes.c_void_p), ("obs_rows", ctypes.c_void_p),
        ("state", ctypes.c_void_p), ("covariance", ctypes.c_void_p),
    ]


class FirstObs(ctypes.Structure):
    """kalman_gpu_first_obs_t (include/kalman_gpu.h)."""
    _fields_ = [("m0max", ctypes.c_int32), ("G0", ctypes.c_void_p), ("o0", ctypes.c_void_p), ("C0", ctypes.c_void_p),
                ("C0_type", ctypes.c_void_p), ("obs_rows0", ctypes.c_void_p)]


class Tuning(ctypes.Structure):
    """kalman_gpu_tuning_t (include/kalman_gpu.h)."""
    _fields_ = [("cta_min_n", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("pair_block", ctypes.c_int32),
                ("weigh_block", ctypes.c_int32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class InvariantModel(ctypes.Structure):
    """kalman_gpu_invariant_model_t (include/kalman_gpu.h): device pointers to
    column-major model matrices."""
    _fields_ = [
        ("m0", ctypes.c_int32), ("m", ctypes.c_int32),
        ("H", ctypes.c_void_p), ("F", ctypes.c_void_p), ("c", ctypes.c_void_p), ("K", ctypes.c_void_p),
        ("K_type", ctypes.c_char),
        ("G0", ctypes.c_void_p), ("o0", ctypes.c_void_p), ("C0", ctypes.c_void_p), ("C0_type", ctypes.c_char),
        ("G", ctypes.c_void_p), ("C", ctypes.c_void_p), ("C_type", ctypes.c_char),
    ]


# every symbol include/*.h declares (checked by tests/test_abi.py)
EXPORTED = [
    "kalman_covariance_matrix_weigh", "kalman_covariance_matrix_explicit", "kalman_create", "kalman_create_options",
    "kalman_free", "kalman_earliest", "kalman_latest", "kalman_evolve", "kalman_observe", "kalman_smooth",
    "kalman_estimate", "kalman_covariance", "kalman_covariance_type", "kalman_forget", "kalman_rollback",
    "kalman_perftest", "kalman_smooth_oddeven", "kalman_smooth_associative", "kalman_nan",
    "matrix_set", "matrix_get", "matrix_create", "matrix_create_constant", "matrix_create_copy",
    "matrix_create_sub", "matrix_mutate_copy_sub", "matrix_free", "matrix_rows", "matrix_cols", "matrix_ld",
    "matrix_create_identity", "matrix_create_from_rowwise", "matrix_print", "matrix_mutate_gemm",
    "matrix_mutate_scale", "matrix_mutate_triu", "matrix_mutate_chop", "matrix_mutate_copy",
    "matrix_mutate_trisolve", "matrix_mutate_chol", "matrix_create_mutate_qr", "matrix_mutate_apply_qt",
    "matrix_create_trisolve", "matrix_create_chol", "matrix_create_vconcat", "matrix_create_inverse",
    "matrix_create_transpose", "matrix_create_mldivide", "matrix_create_multiply", "matrix_create_subtract",
    "matrix_create_add", "parallel_set_thread_limit", "parallel_set_blocksize",
    "kalman_gpu_last_status", "kalman_gpu_last_error", "kalman_gpu_clear_error",
    "kalman_gpu_smooth_oddeven_packed", "kalman_gpu_smooth_associative_packed", "kalman_gpu_smooth_tracks",
    "kalman_gpu_release", "kalman_gpu_profile_enable", "kalman_gpu_profile_read", "kalman_gpu_launch_count",
    "kalman_gpu_measure_fp64_tflops", "kalman_gpu_measure_fp32_tflops", "kalman_gpu_smooth_oddeven_noalloc",
    "kalman_gpu_plan_create", "kalman_gpu_plan_execute", "kalman_gpu_plan_status", "kalman_gpu_plan_destroy",
    "kalman_gpu_expand_invariant", "kalman_gpu_filter_packed", "kalman_gpu_oddeven_workspace_bytes",
    "kalman_gpu_workspace_held", "kalman_gpu_set_tuning", "kalman_gpu_get_tuning",
    "kalman_gpu_smooth_oddeven_first_obs", "kalman_gpu_check_bounded_wait",
]

_lib = None


def load(path=LIB_PATH):
    """Loads libukgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run ultimate_kalman_gb300/build.py (or __graft_entry__.build())")
    L = ctypes.CDLL(path)
    P = ctypes.POINTER(ProblemStruct)
    for f in ("kalman_gpu_smooth_oddeven_packed", "kalman_gpu_smooth_associative_packed",
              "kalman_gpu_smooth_oddeven_noalloc", "kalman_gpu_filter_packed"):
        getattr(L, f).argtypes = [ctypes.c_uint32, P, ctypes.c_void_p]
        getattr(L, f).restype = ctypes.c_int
    L.kalman_gpu_last_error.restype = ctypes.c_char_p
    L.kalman_gpu_last_status.restype = ctypes.c_int
    SE = ctypes.POINTER(ctypes.POINTER(StepEquations))
    L.kalman_smooth_oddeven.argtypes = [ctypes.c_uint32, SE, ctypes.c_int32]
    L.kalman_smooth_associative.argtypes = [ctypes.c_uint32, SE, ctypes.c_int32]
    L.kalman_gpu_smooth_tracks.argtypes = [ctypes.c_uint32, SE, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32]
    L.kalman_gpu_smooth_tracks.restype = ctypes.c_int
    L.matrix_free.argtypes = [ctypes.POINTER(Matrix)]
    L.kalman_gpu_profile_enable.argtypes = [ctypes.c_int]
    L.kalman_gpu_profile_read.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                          ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]
    L.kalman_gpu_profile_read.restype = ctypes.c_int
    L.kalman_gpu_launch_count.restype = ctypes.c_int64
    L.kalman_gpu_measure_fp64_tflops.argtypes = [ctypes.c_int]
    L.kalman_gpu_measure_fp64_tflops.restype = ctypes.c_double
    L.kalman_gpu_measure_fp32_tflops.restype = ctypes.c_double
    L.kalman_gpu_check_bounded_wait.argtypes = [ctypes.c_void_p]
    L.kalman_gpu_check_bounded_wait.restype = ctypes.c_int
    L.kalman_gpu_plan_create.argtypes = [ctypes.c_uint32, P]
    L.kalman_gpu_plan_create.restype = ctypes.c_void_p
    L.kalman_gpu_plan_execute.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.kalman_gpu_plan_execute.restype = ctypes.c_int
    L.kalman_gpu_plan_status.argtypes = [ctypes.c_void_p]
    L.kalman_gpu_plan_status.restype = ctypes.c_int
    L.kalman_gpu_plan_destroy.argtypes = [ctypes.c_void_p]
    L.kalman_gpu_expand_invariant.argtypes = [P, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(InvariantModel),
                                              ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    L.kalman_gpu_expand_invariant.restype = ctypes.c_int
    L.kalman_gpu_oddeven_workspace_bytes.argtypes = [ctypes.c_uint32, P]
    L.kalman_gpu_oddeven_workspace_bytes.restype = ctypes.c_int64
    L.kalman_gpu_workspace_held.restype = ctypes.c_int64
    L.kalman_gpu_smooth_oddeven_first_obs.argtypes = [ctypes.c_uint32, P, ctypes.POINTER(FirstObs), ctypes.c_void_p]
    L.kalman_gpu_smooth_oddeven_first_obs.restype = ctypes.c_int
    L.kalman_gpu_set_tuning.argtypes = [ctypes.POINTER(Tuning)]
    L.kalman_gpu_set_tuning.restype = ctypes.c_int
    L.kalman_gpu_get_tuning.argtypes = [ctypes.POINTER(Tuning)]
    _lib = L
    return L


def last_error():
    L = load()
    return L.kalman_gpu_last_status(), L.kalman_gpu_last_error().decode()


def _check(status):
    if status not in (0,):
        st, msg = last_error()
        raise KalmanError(status, msg)


def profile_enable(on=True):
    load().kalman_gpu_profile_enable(1 if on else 0)


def profile_read():
    """{kernel name: (total ms, launches)} since profile_enable()."""
    L = load()
    names = (ctypes.c_char_p * 32)()
    ms = (ctypes.c_double * 32)()
    cnt = (ctypes.c_int64 * 32)()
    k = L.kalman_gpu_profile_read(32, names, ms, cnt)
    return {names[i].decode(): (ms[i], cnt[i]) for i in range(k)}


def launch_count():
    return load().kalman_gpu_launch_count()


def measure_fp64_tflops(active_lanes=32):
    return load().kalman_gpu_measure_fp64_tflops(active_lanes)


def measure_fp32_tflops():
    return load().kalman_gpu_measure_fp32_tflops()


def oddeven_workspace_bytes(s, **kw):
    """kalman_gpu_oddeven_workspace_bytes for a ProblemStruct and the options
    that options_for(**kw) gives."""
    return load().kalman_gpu_oddeven_workspace_bytes(options_for("oddeven", **kw), ctypes.byref(s))


def workspace_held():
    """kalman_gpu_workspace_held: device bytes the calling thread's library
    state holds."""
    return load().kalman_gpu_workspace_held()


def set_tuning(**knobs):
    """kalman_gpu_set_tuning with the current values overridden by `knobs`
    (cta_min_n, ctas_per_sm, pair_block, weigh_block); set_tuning(default=True)
    restores the library's defaults.  Returns the setting now in force."""
    L = load()
    if knobs.pop("default", False):
        _check(L.kalman_gpu_set_tuning(None))
    t = get_tuning()
    for k, v in knobs.items():
        if k not in t:
            raise KeyError(k)
        t[k] = int(v)
    if knobs:
        _check(L.kalman_gpu_set_tuning(ctypes.byref(Tuning(**t))))
    return get_tuning()


def get_tuning():
    """kalman_gpu_get_tuning as a dict."""
    t = Tuning()
    load().kalman_gpu_get_tuning(ctypes.byref(t))
    return t.as_dict()


FIRST_OBS_FIELDS = ("G0", "o0", "C0", "C0_type", "obs_rows0")


def first_obs_struct(F0, arrays):
    """kalman_gpu_first_obs_t over the arrays (numpy or torch, host or
    device) of a problem.split_first_obs dictionary."""
    f = FirstObs()
    f.m0max = int(F0["m0max"])
    for k in FIRST_OBS_FIELDS:
        a = arrays[k]
        setattr(f, k, a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data)
    return f


def smooth_first_obs(Pc, F0, covariance=True, fp32_refine=False, location="device", sweeps=0):
    """kalman_gpu_smooth_oddeven_first_obs on a problem in first-step-
    observation form (problem.split_first_obs); returns (states, covs or
    None) like smooth()."""
    import torch
    L = load()
    N, n = Pc.nsteps, Pc.n
    opts = options_for("oddeven", covariance, fp32_refine, sweeps)
    if location == "device":
        D = DeviceProblem(Pc, covariance)
        f0a = {k: torch.from_numpy(np.ascontiguousarray(F0[k])).cuda() for k in FIRST_OBS_FIELDS}
        f = first_obs_struct(F0, f0a)
        st = torch.cuda.current_stream()
        _check(L.kalman_gpu_smooth_oddeven_first_obs(opts, ctypes.byref(D.struct), ctypes.byref(f),
                                                     ctypes.c_void_p(st.cuda_stream)))
        torch.cuda.synchronize()
        return D.results() if covariance else (D.state.cpu().numpy(), None)
    state = np.full((N, n), np.nan)
    cov = np.full((N, n, n), np.nan) if covariance else None
    arrs = {f_: np.ascontiguousarray(getattr(Pc, f_)) for f_ in _FIELDS}
    s = ProblemStruct()
    s.n, s.mmax, s.ntracks, s.location, s.nsteps = Pc.n, Pc.mmax, Pc.ntracks, KALMAN_GPU_HOST, N
    ts = np.ascontiguousarray(Pc.track_start, dtype=np.int64)
    s.track_start = ts.ctypes.data
    for f_ in _FIELDS:
        setattr(s, f_, arrs[f_].ctypes.data)
    s.state = state.ctypes.data
    s.covariance = cov.ctypes.data if cov is not None else None
    f0a = {k: np.ascontiguousarray(F0[k]) for k in FIRST_OBS_FIELDS}
    f = first_obs_struct(F0, f0a)
    _check(L.kalman_gpu_smooth_oddeven_first_obs(opts, ctypes.byref(s), ctypes.byref(f), None))
    if cov is not None:
        cov = np.ascontiguousarray(cov.transpose(0, 2, 1))
    return state, cov


def release():
    """kalman_gpu_release: frees the library's cached device workspace and
    staging buffers of the calling thread."""
    load().kalman_gpu_release()


def options_for(algorithm, covariance=True, fp32_refine=False, sweeps=0):
    o = KALMAN_ALGORITHM_ODDEVEN if algorithm == "oddeven" else KALMAN_ALGORITHM_ASSOCIATIVE
    if not covariance:
        o |= KALMAN_NO_COVARIANCE
    if fp32_refine:
        o |= KALMAN_GPU_FP32_REFINE | ((sweeps & 3) << 21)
    return o


# ---------------------------------------------------------------------------
# packed problems
# ---------------------------------------------------------------------------

_FIELDS = ("H", "F", "c", "K", "K_type", "G", "o", "C", "C_type", "obs_rows")


class DeviceProblem:
    """A PackedProblem copied into GPU memory (torch tensors as allocations),
    with device output buffers, ready for repeated smoothing calls."""

    def __init__(self, P, covariance=True, device="cuda"):
        import torch
        arrays = {f: torch.from_numpy(np.ascontiguousarray(getattr(P, f))).to(device) for f in _FIELDS}
        self._setup(P.n, P.mmax, P.track_start, arrays, covariance, device)

    @classmethod
    def from_arrays(cls, n, mmax, track_start, arrays, covariance=True, device="cuda"):
        """A device problem over packed arrays already in GPU memory (torch
        tensors, e.g. written by expand_invariant)."""
        self = cls.__new__(cls)
        self._setup(n, mmax, track_start, arrays, covariance, device)
        return self

    def _setup(self, n, mmax, track_start, arrays, covariance, device):
        import torch
        self.torch = torch
        self.arrays = arrays
        self.track_start = np.ascontiguousarray(track_start, dtype=np.int64)
        nsteps = int(self.track_start[-1])
        self.state = torch.empty((nsteps, n), dtype=torch.float64, device=device)
        self.cov = torch.empty((nsteps, n, n), dtype=torch.float64, device=device) if covariance else None
        s = ProblemStruct()
        s.n, s.mmax, s.ntracks, s.location = n, mmax, len(self.track_start) - 1, KALMAN_GPU_DEVICE
        s.nsteps = nsteps
        s.track_start = self.track_start.ctypes.data
        for f in _FIELDS:
            setattr(s, f, self.arrays[f].data_ptr())
        s.state = self.state.data_ptr()
        s.covariance = self.cov.data_ptr() if covariance else None
        self.struct = s

    def input_bytes(self):
        return sum(a.numel() * a.element_size() for a in self.arrays.values())

    def smooth(self, algorithm="oddeven", covariance=True, fp32_refine=False, stream=None, check=True, sweeps=0):
        L = load()
        torch = self.torch
        st = stream if stream is not None else torch.cuda.current_stream()
        opts = options_for(algorithm, covariance and self.cov is not None, fp32_refine, sweeps)
        f = L.kalman_gpu_smooth_oddeven_packed if algorithm == "oddeven" else L.kalman_gpu_smooth_associative_packed
        status = f(opts, ctypes.byref(self.struct), ctypes.c_void_p(st.cuda_stream))
        if check:
            _check(status)
        return status

    def filter(self, covariance=True, stream=None, check=True):
        """Filtered estimates x_{s|s} (and P_{s|s}) of every step into
        self.state / self.cov: kalman_gpu_filter_packed."""
        L = load()
        st = stream if stream is not None else self.torch.cuda.current_stream()
        opts = 0 if (covariance and self.cov is not None) else KALMAN_NO_COVARIANCE
        status = L.kalman_gpu_filter_packed(opts, ctypes.byref(self.struct), ctypes.c_void_p(st.cuda_stream))
        if check:
            _check(status)
        return status

    def plan(self, algorithm="oddeven", covariance=True, fp32_refine=False, sweeps=0):
        """A CUDA-graph plan over these device arrays (odd-even only): see
        kalman_gpu_plan_create.  Returns a Plan; refill the arrays in place
        between executions."""
        if algorithm != "oddeven":
            raise ValueError("plans cover the odd-even smoother")
        L = load()
        opts = options_for(algorithm, covariance and self.cov is not None, fp32_refine, sweeps)
        h = L.kalman_gpu_plan_create(opts, ctypes.byref(self.struct))
        if not h:
            _check(L.kalman_gpu_last_status())
        return Plan(h, self)

    def results(self):
        X = self.state.cpu().numpy()
        S = None
        if self.cov is not None:
            S = np.ascontiguousarray(self.cov.cpu().numpy().transpose(0, 2, 1))
        return X, S


class Plan:
    """A prepared odd-even plan replayed as a CUDA graph (kalman_gpu_plan_*)."""

    def __init__(self, handle, owner):
        self.h = handle
        self.owner = owner  # keeps the device arrays alive

    def execute(self, stream=None):
        L = load()
        import torch
        st = stream if stream is not None else torch.cuda.current_stream()
        _check(L.kalman_gpu_plan_execute(self.h, ctypes.c_void_p(st.cuda_stream)))

    def status(self):
        return load().kalman_gpu_plan_status(self.h)

    def close(self):
        if self.h:
            load().kalman_gpu_plan_destroy(self.h)
            self.h = None
        self.owner = None  # the device arrays may be freed now

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def smooth(P, algorithm="oddeven", covariance=True, fp32_refine=False, location="device", sweeps=0):
    """Smooths a PackedProblem on the GPU; returns (states [N,n], covs [N,n,n] or None).
    location="device": inputs are copied to GPU memory first and the device
    entry point runs on them; "host": the library is handed host arrays."""
    if location == "device":
        D = DeviceProblem(P, covariance)
        D.smooth(algorithm, covariance, fp32_refine, sweeps=sweeps)
        return D.results()
    L = load()
    N, n = P.nsteps, P.n
    state = np.full((N, n), np.nan)
    cov = np.full((N, n, n), np.nan) if covariance else None
    s = ProblemStruct()
    s.n, s.mmax, s.ntracks, s.location = P.n, P.mmax, P.ntracks, KALMAN_GPU_HOST
    s.nsteps = N
    ts = np.ascontiguousarray(P.track_start, dtype=np.int64)
    s.track_start = ts.ctypes.data
    arrs = {f: np.ascontiguousarray(getattr(P, f)) for f in _FIELDS}
    for f in _FIELDS:
        setattr(s, f, arrs[f].ctypes.data)
    s.state = state.ctypes.data
    s.covariance = cov.ctypes.data if cov is not None else None
    opts = options_for(algorithm, covariance, fp32_refine, sweeps)
    f = L.kalman_gpu_smooth_oddeven_packed if algorithm == "oddeven" else L.kalman_gpu_smooth_associative_packed
    _check(f(opts, ctypes.byref(s), None))
    if cov is not None:
        cov = np.ascontiguousarray(cov.transpose(0, 2, 1))
    return state, cov


# ---------------------------------------------------------------------------
# the reference entry points, fed with kalman_step_equations_t structs
# ---------------------------------------------------------------------------

def _matrix(A, keep):
    A = np.asfortranarray(np.asarray(A, dtype=np.float64))
    if A.ndim == 1:
        A = A.reshape(-1, 1, order="F")
    keep.append(A)
    m = Matrix(A.shape[0], A.shape[1], A.shape[0], A.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    keep.append(m)
    return ctypes.pointer(m)


def build_equations(P):
    """kalman_step_equations_t* array for every step of P (tracks back to back).
    Returns (array, keepalive list, structs)."""
    keep = []
    structs = []
    firsts = set(int(s) for s in P.track_start[:-1])
    for s in range(P.nsteps):
        e = StepEquations()
        e.step = 0 if s in firsts else 1
        e.dimension = P.n
        if s not in firsts:
            e.H = _matrix(P.H[s].T, keep)
            e.F = _matrix(P.F[s].T, keep)
            e.c = _matrix(P.c[s], keep)
            kt = chr(P.K_type[s])
            e.K = _matrix(P.K[s].reshape(-1)[:P.n] if kt == "w" else P.K[s].T, keep)
            e.K_type = kt.encode()
        m = int(P.obs_rows[s])
        if m > 0:
            ct = chr(P.C_type[s])
            e.G = _matrix(P.G[s].T[:m], keep)
            e.o = _matrix(P.o[s][:m], keep)
            e.C = _matrix(P.C[s].reshape(-1)[:m] if ct == "w" else P.C[s].T[:m, :m], keep)
            e.C_type = ct.encode()
        structs.append(e)
    arr = (ctypes.POINTER(StepEquations) * P.nsteps)(*[ctypes.pointer(e) for e in structs])
    return arr, keep, structs


class EquationsView:
    """kalman_step_equations_t structs for every step of a PackedProblem,
    built with numpy in bulk (the matrices point into the problem's packed
    arrays: blocks are column-major with ld = n, or ld = mmax for G, o, C),
    for driving the reference entry points on millions of steps.  Keeps the
    problem alive; results are written into the structs by the library.

    ptrs: the kalman_step_equations_t* array; lengths: the track lengths."""

    def __init__(self, P):
        fields = {f: np.ascontiguousarray(getattr(P, f)) for f in _FIELDS}
        self.keep = fields
        N, n, mm = int(P.nsteps), int(P.n), int(P.mmax)
        mat = np.dtype({"names": ["rows", "cols", "ld", "elements"], "formats": ["<i4", "<i4", "<i4", "<u8"],
                        "offsets": [0, 4, 8, 16], "itemsize": ctypes.sizeof(Matrix)})
        kinds = ["H", "F", "K", "c", "G", "o", "C"]
        self.mats = np.zeros((len(kinds), N), dtype=mat)
        first = np.zeros(N, dtype=bool)
        first[np.asarray(P.track_start[:-1])[np.diff(P.track_start) > 0]] = True
        m = fields["obs_rows"].astype(np.int32)
        steps = np.arange(N, dtype=np.uint64)
        kt, ct = fields["K_type"], fields["C_type"]
        spec = {"H": (n, n, n, n * n), "F": (n, n, n, n * n), "c": (n, 1, n, n), "G": (m, n, mm, mm * n),
                "o": (m, 1, mm, mm), "C": (m, np.where(ct == ord("w"), 1, m), mm, mm * mm),
                "K": (n, np.where(kt == ord("w"), 1, n), n, n * n)}
        for i, k in enumerate(kinds):
            rows, cols, ld, per = spec[k]
            a = self.mats[i]
            a["rows"], a["cols"], a["ld"] = rows, cols, ld
            a["elements"] = np.uint64(fields[k].ctypes.data) + steps * np.uint64(per * 8)
        eqd = np.dtype({"names": [f for f, _ in StepEquations._fields_],
                        "formats": ["<i4", "<i4", "S1", "S1"] + ["<u8"] * 9 + ["S1"],
                        "offsets": [getattr(StepEquations, f).offset for f, _ in StepEquations._fields_],
                        "itemsize": ctypes.sizeof(StepEquations)})
        self.eq = np.zeros(N, dtype=eqd)
        self.eq["step"] = np.where(first, 0, 1)
        self.eq["dimension"] = n
        self.eq["K_type"] = kt.view("S1")
        self.eq["C_type"] = ct.view("S1")
        self.eq["covariance_type"] = b"C"
        base = np.uint64(self.mats.ctypes.data)
        sz = np.uint64(ctypes.sizeof(Matrix))
        for i, k in enumerate(kinds):
            ptr = base + (np.uint64(i * N) + steps) * sz
            if k in ("H", "F", "K", "c"):
                ptr = np.where(first, np.uint64(0), ptr)
            else:
                ptr = np.where(m > 0, ptr, np.uint64(0))
            self.eq[k] = ptr
        self.ptrs = np.uint64(self.eq.ctypes.data) + steps * np.uint64(ctypes.sizeof(StepEquations))
        self.lengths = np.ascontiguousarray(np.diff(P.track_start), dtype=np.int32)
        self.n = n

    def smooth_tracks(self, algorithm="oddeven", covariance=False, fp32_refine=False, sweeps=0):
        """kalman_gpu_smooth_tracks over every track; returns the status.  The
        library frees the previous call's result matrices before writing."""
        L = load()
        opts = options_for(algorithm, covariance, fp32_refine, sweeps)
        arr = self.ptrs.ctypes.data_as(ctypes.POINTER(ctypes.POINTER(StepEquations)))
        lens = self.lengths.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        return L.kalman_gpu_smooth_tracks(opts, arr, lens, len(self.lengths))

    def states(self, steps):
        """The smoothed states of the given step indices (from the structs)."""
        out = np.full((len(steps), self.n), np.nan)
        for j, s in enumerate(steps):
            p = int(self.eq["state"][s])
            if p:
                M = Matrix.from_address(p)
                out[j] = np.ctypeslib.as_array(M.elements, shape=(self.n,))
        return out


def _read_matrix(mp):
    if not mp:
        return None
    m = mp.contents
    out = np.ctypeslib.as_array(m.elements, shape=(m.col_dim * m.ld,)).reshape(m.col_dim, m.ld)[:, :m.row_dim]
    return np.array(out.T)


def smooth_equations(P, algorithm="oddeven", covariance=True, batched=False):
    """Runs kalman_smooth_oddeven / kalman_smooth_associative on the equations of
    P (one call per track), or kalman_gpu_smooth_tracks on all of them when
    batched=True; returns (states, covs or None, last status)."""
    L = load()
    arr, keep, structs = build_equations(P)
    opts = options_for(algorithm, covariance)
    if batched:
        lens = (ctypes.c_int32 * P.ntracks)(*[int(x) for x in P.track_lengths()])
        status = L.kalman_gpu_smooth_tracks(opts, arr, lens, P.ntracks)
    else:
        status = 0
        f = L.kalman_smooth_oddeven if algorithm == "oddeven" else L.kalman_smooth_associative
        for t in range(P.ntracks):
            s0, s1 = int(P.track_start[t]), int(P.track_start[t + 1])
            sub = ctypes.cast(ctypes.byref(arr, s0 * ctypes.sizeof(ctypes.c_void_p)),
                              ctypes.POINTER(ctypes.POINTER(StepEquations)))
            f(opts, sub, s1 - s0)
            status = status or L.kalman_gpu_last_status()
    X = np.full((P.nsteps, P.n), np.nan)
    S = np.full((P.nsteps, P.n, P.n), np.nan)
    have_cov = False
    for s, e in enumerate(structs):
        x = _read_matrix(e.state)
        if x is not None:
            X[s] = x[:, 0]
        c = _read_matrix(e.covariance)
        if c is not None:
            S[s] = c
            have_cov = True
        if e.state:
            L.matrix_free(e.state)
        if e.covariance:
            L.matrix_free(e.covariance)
    return X, (S if have_cov else None), status


def host_struct_from_tensors(P, arrays, state, cov):
    """kalman_gpu_problem_t over (page-locked) host torch tensors, for the
    end-to-end path in which the library copies inputs in and results out."""
    s = ProblemStruct()
    s.n, s.mmax, s.ntracks, s.location = P.n, P.mmax, P.ntracks, KALMAN_GPU_HOST
    s.nsteps = P.nsteps
    s._track_start = np.ascontiguousarray(P.track_start, dtype=np.int64)
    s.track_start = s._track_start.ctypes.data
    for f in _FIELDS:
        setattr(s, f, arrays[f].data_ptr())
    s.state = state.data_ptr()
    s.covariance = cov.data_ptr() if cov is not None else None
    return s


def smooth_struct(algorithm, s, covariance=True, fp32_refine=False, stream=None, sweeps=0):
    """Runs a packed entry point on a prepared ProblemStruct."""
    L = load()
    opts = options_for(algorithm, covariance, fp32_refine, sweeps)
    f = L.kalman_gpu_smooth_oddeven_packed if algorithm == "oddeven" else L.kalman_gpu_smooth_associative_packed
    _check(f(opts, ctypes.byref(s), ctypes.c_void_p(stream.cuda_stream) if stream is not None else None))


def expand_invariant(s, first, k, model, o, ldo, obs_rows=None, stream=None):
    """kalman_gpu_expand_invariant on the device arrays of ProblemStruct s:
    steps first .. first+k-1 from the InvariantModel and the observation
    stream o (a device pointer, ldo doubles per step).  Raises on failure."""
    L = load()
    st = stream.cuda_stream if stream is not None and hasattr(stream, "cuda_stream") else stream
    _check(L.kalman_gpu_expand_invariant(ctypes.byref(s), int(first), int(k), ctypes.byref(model),
                                         ctypes.c_void_p(o), int(ldo), ctypes.c_void_p(obs_rows), ctypes.c_void_p(st)))
