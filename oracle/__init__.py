"""TEST INFRASTRUCTURE -- the oracle for the GB300 Kalman smoothers.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker or the timed CPU reference; the library never
imports it.

  * ``kalman_oracle.c`` -- a plain-C FP64 restatement of UltimateKalman's
    odd-even and associative smoothers (c/kalman_oddeven_smoother.c,
    c/kalman_associative_smoother.c), compiled here into liboracle.so and
    called through ctypes.  It is pinned against outputs of the reference C
    library itself (tests/golden/, made by tests/golden/make_golden.py) and
    against the dense least-squares solution below.
  * ``dense_smooth`` -- the dense FP64 least-squares solution of the whole
    weighted block-bidiagonal system with covariance blocks from (R^T R)^{-1},
    restating the gold standard of the reference's test suite
    (matlab/KalmanSparse.m:97-306, smooth at 263-306).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "liboracle.so")

KALMAN_NO_COVARIANCE = 1 << 16


class ProblemStruct(ctypes.Structure):
    """ctypes image of kalman_gpu_problem_t (include/kalman_gpu.h)."""
    _fields_ = [
        ("n", ctypes.c_int32), ("mmax", ctypes.c_int32), ("ntracks", ctypes.c_int32), ("location", ctypes.c_int32),
        ("nsteps", ctypes.c_int64), ("track_start", ctypes.c_void_p),
        ("H", ctypes.c_void_p), ("F", ctypes.c_void_p), ("c", ctypes.c_void_p), ("K", ctypes.c_void_p),
        ("K_type", ctypes.c_void_p), ("G", ctypes.c_void_p), ("o", ctypes.c_void_p), ("C", ctypes.c_void_p),
        ("C_type", ctypes.c_void_p), ("obs_rows", ctypes.c_void_p),
        ("state", ctypes.c_void_p), ("covariance", ctypes.c_void_p),
    ]


def _ptr(a):
    return None if a is None else a.ctypes.data


def host_struct(P, state, cov):
    """kalman_gpu_problem_t over the host arrays of a PackedProblem."""
    for f in ("H", "F", "c", "K", "G", "o", "C"):
        a = getattr(P, f)
        assert a.dtype == np.float64 and a.flags.c_contiguous, f
    s = ProblemStruct()
    s.n, s.mmax, s.ntracks, s.location = P.n, P.mmax, P.ntracks, 1
    s.nsteps = P.nsteps
    s.track_start = _ptr(P.track_start)
    s.H, s.F, s.c, s.K = _ptr(P.H), _ptr(P.F), _ptr(P.c), _ptr(P.K)
    s.K_type, s.G, s.o, s.C = _ptr(P.K_type), _ptr(P.G), _ptr(P.o), _ptr(P.C)
    s.C_type, s.obs_rows = _ptr(P.C_type), _ptr(P.obs_rows)
    s.state, s.covariance = _ptr(state), _ptr(cov)
    return s


def build(force=False, quiet=True):
    """Compiles liboracle.so (gcc, OpenMP).  Cheap; safe to call repeatedly."""
    src = os.path.join(HERE, "kalman_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c11", "-Wall", "-Wno-unused-variable",
           "-Wno-unused-but-set-variable", "-o", LIB_PATH + ".tmp", src, "-lm"]
    subprocess.run(cmd, check=True, capture_output=quiet)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        for name in ("oracle_smooth_oddeven", "oracle_smooth_associative"):
            f = getattr(L, name)
            f.argtypes = [ctypes.c_uint32, ctypes.POINTER(ProblemStruct), ctypes.c_int]
            f.restype = ctypes.c_int
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def max_threads():
    return lib().oracle_max_threads()


def smooth(P, algorithm="oddeven", covariance=True, threads=0):
    """Runs the oracle smoother; returns (status, states [N,n], covs [N,n,n] or None).
    Covariance blocks come back as arr[s] = S_s^T (column-major), which for the
    symmetric S_s is S_s up to rounding."""
    N, n = P.nsteps, P.n
    state = np.full((N, n), np.nan)
    cov = np.full((N, n, n), np.nan) if covariance else None
    s = host_struct(P, state, cov)
    opts = 0 if covariance else KALMAN_NO_COVARIANCE
    f = lib().oracle_smooth_oddeven if algorithm == "oddeven" else lib().oracle_smooth_associative
    status = f(opts, ctypes.byref(s), threads)
    if cov is not None:
        cov = np.ascontiguousarray(cov.transpose(0, 2, 1))
    return status, state, cov


# --------------------------------------------------------------------------
# dense least-squares oracle (KalmanSparse restated)
# --------------------------------------------------------------------------

def _weigh(cov_block, kind, rows, A):
    """W A for the covariance factor of the given kind (c/kalman_base.c:61-175)."""
    kind = chr(kind) if not isinstance(kind, str) else kind
    if kind == "W":
        W = cov_block[:rows, :rows]
        return W @ A
    if kind == "w":
        w = cov_block.T.reshape(-1)[:rows]
        return w[:, None] * A
    if kind == "C":
        L = np.linalg.cholesky(cov_block[:rows, :rows])
        return np.linalg.solve(L, A)
    if kind in ("U", "F"):
        L = np.tril(cov_block[:rows, :rows])
        return np.linalg.solve(L, A)
    raise ValueError(kind)


def dense_system(P, t):
    """Weighted block-bidiagonal system (A, b) of track t."""
    n = P.n
    s0, s1 = int(P.track_start[t]), int(P.track_start[t + 1])
    k = s1 - s0
    rows, rhs = [], []
    for i in range(k):
        s = s0 + i
        if i > 0:
            H = P.H[s].T
            F = P.F[s].T
            c = P.c[s]
            Kb = P.K[s].T
            blk = np.zeros((n, k * n))
            blk[:, (i - 1) * n:i * n] = -_weigh(Kb, P.K_type[s], n, F)
            blk[:, i * n:(i + 1) * n] = _weigh(Kb, P.K_type[s], n, H)
            rows.append(blk)
            rhs.append(_weigh(Kb, P.K_type[s], n, c[:, None])[:, 0])
        m = int(P.obs_rows[s])
        if m > 0:
            G = P.G[s].T[:m]
            o = P.o[s][:m]
            Cb = P.C[s].T
            blk = np.zeros((m, k * n))
            blk[:, i * n:(i + 1) * n] = _weigh(Cb, P.C_type[s], m, G)
            rows.append(blk)
            rhs.append(_weigh(Cb, P.C_type[s], m, o[:, None])[:, 0])
    return np.vstack(rows), np.concatenate(rhs)


def dense_smooth(P, covariance=True):
    """Dense FP64 least-squares smoothing of every track (small problems only).
    Returns (states [N,n], covs [N,n,n] or None)."""
    n, N = P.n, P.nsteps
    X = np.zeros((N, n))
    S = np.zeros((N, n, n)) if covariance else None
    for t in range(P.ntracks):
        A, b = dense_system(P, t)
        s0, s1 = int(P.track_start[t]), int(P.track_start[t + 1])
        k = s1 - s0
        Q, R = np.linalg.qr(A)
        u = np.linalg.solve(R, Q.T @ b)
        X[s0:s1] = u.reshape(k, n)
        if covariance:
            Ri = np.linalg.solve(R, np.eye(k * n))
            for i in range(k):
                blk = Ri[i * n:(i + 1) * n]
                S[s0 + i] = blk @ blk.T
    return X, S


def rel_err_states(X, Xref, track_start=None):
    """max over steps of ||x_i - xref_i||_inf / ||xref_i||_inf"""
    num = np.abs(X - Xref).max(axis=1)
    den = np.abs(Xref).max(axis=1)
    return float(np.max(num / np.maximum(den, np.finfo(float).tiny)))


def rel_err_covs(S, Sref):
    """max over steps of ||P_i - Pref_i||_max / ||Pref_i||_max"""
    num = np.abs(S - Sref).reshape(len(S), -1).max(axis=1)
    den = np.abs(Sref).reshape(len(S), -1).max(axis=1)
    return float(np.max(num / np.maximum(den, np.finfo(float).tiny)))
