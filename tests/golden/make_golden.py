"""Generates the golden fixtures in tests/golden/ from the REFERENCE C library.

Run here (the only machine that has the reference sources):
    python oracle/build_ref.py && python tests/golden/make_golden.py

Every case is a single track.  It is fed to the reference through its own
public API -- kalman_create_options / kalman_evolve / kalman_observe /
kalman_smooth / kalman_estimate / kalman_covariance (c/kalman.h:117-131) -- with
each of the reference's smoothers that accepts it: ODDEVEN, ASSOCIATIVE
(square step 0, no missing observation) and ULTIMATE (sequential, used as a
third opinion).  Each run happens in a child process because the reference
aborts (assert) on inputs it does not support; such runs are recorded as
missing.  The fixture stores the packed inputs and the reference outputs.

Inputs:
  * rotation   -- c/rotation.c: the rotating-point example with its MATLAB
                  rng(5) noise tables (parsed from that file), 16 steps.
  * perf6/48   -- c/performance.c: the MATLAB rng(1) tables F6/G6/o6 and
                  F48/G48/o48 with identity 'W' covariances, as the reference's
                  timing driver sets them up (performance.c:328-340).
  * cv_*, rand_* -- seeded synthetic tracks of the benchmark configurations'
                  shapes (n=6/m=3 constant velocity; random n, m dynamics).
"""
from __future__ import annotations

import ctypes
import multiprocessing as mp
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from ultimate_kalman_gb300 import problem as pb  # noqa: E402

REF_LIB = os.path.join(REPO, "oracle", "_ref", "libukref.so")
# the reference C sources: UKG_REFERENCE_C, else where the build machine keeps them
REF_C = os.environ.get("UKG_REFERENCE_C", "/root/reference/c")

ALG = {"ultimate": 1, "oddeven": 4, "associative": 8}


class Mat(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int32), ("cols", ctypes.c_int32), ("ld", ctypes.c_int32),
                ("elements", ctypes.POINTER(ctypes.c_double))]


def _mat(A, keep):
    A = np.asfortranarray(np.asarray(A, dtype=np.float64))
    if A.ndim == 1:
        A = A.reshape(-1, 1, order="F")
    keep.append(A)
    return ctypes.pointer(Mat(A.shape[0], A.shape[1], A.shape[0],
                              A.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))


def _read(m):
    r, c, ld = m.contents.rows, m.contents.cols, m.contents.ld
    out = np.zeros((r, c))
    for j in range(c):
        for i in range(r):
            out[i, j] = m.contents.elements[j * ld + i]
    return out


def _cov_arg(block, kind, dim):
    """Reference-API argument for a stored covariance factor."""
    if kind == "w":
        return block.reshape(-1)[:dim].copy()  # the column sits in the first entries
    return block.T[:dim, :dim].copy()


def _run_reference(args):
    path, alg, q = args
    try:
        lib = ctypes.CDLL(REF_LIB)
        lib.kalman_create_options.restype = ctypes.c_void_p
        lib.kalman_create_options.argtypes = [ctypes.c_uint32]
        lib.kalman_evolve.argtypes = [ctypes.c_void_p, ctypes.c_int32] + [ctypes.POINTER(Mat)] * 4 + [ctypes.c_char]
        lib.kalman_observe.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(Mat)] * 3 + [ctypes.c_char]
        lib.kalman_smooth.argtypes = [ctypes.c_void_p]
        lib.kalman_estimate.restype = ctypes.POINTER(Mat)
        lib.kalman_estimate.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        lib.kalman_covariance.restype = ctypes.POINTER(Mat)
        lib.kalman_covariance.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        lib.kalman_covariance_type.restype = ctypes.c_char
        lib.kalman_covariance_type.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        lib.kalman_covariance_matrix_explicit.restype = ctypes.POINTER(Mat)
        lib.kalman_covariance_matrix_explicit.argtypes = [ctypes.POINTER(Mat), ctypes.c_char]
        lib.matrix_free.argtypes = [ctypes.POINTER(Mat)]
        d = np.load(path)
        n, k = int(d["n"]), int(d["track_start"][-1])
        devnull = os.open(os.devnull, os.O_WRONLY)
        os.dup2(devnull, 1)
        kal = lib.kalman_create_options(ALG[alg])
        keep = []
        for i in range(k):
            if i == 0:
                lib.kalman_evolve(kal, n, None, None, None, None, b"C")
            else:
                kt = chr(d["K_type"][i])
                lib.kalman_evolve(kal, n, _mat(d["H"][i].T, keep), _mat(d["F"][i].T, keep), _mat(d["c"][i], keep),
                                  _mat(_cov_arg(d["K"][i], kt, n), keep), kt.encode())
            m = int(d["obs_rows"][i])
            if m == 0:
                lib.kalman_observe(kal, None, None, None, b"C")
            else:
                ct = chr(d["C_type"][i])
                lib.kalman_observe(kal, _mat(d["G"][i].T[:m], keep), _mat(d["o"][i][:m], keep),
                                   _mat(_cov_arg(d["C"][i], ct, m), keep), ct.encode())
        lib.kalman_smooth(kal)
        X = np.zeros((k, n))
        S = np.zeros((k, n, n))
        for i in range(k):
            e = lib.kalman_estimate(kal, i)
            X[i] = _read(e)[:, 0]
            lib.matrix_free(e)
            c = lib.kalman_covariance(kal, i)
            t = lib.kalman_covariance_type(kal, i)
            ce = lib.kalman_covariance_matrix_explicit(c, t) if t != b"C" else c
            S[i] = _read(ce)
            if ce is not c:
                lib.matrix_free(ce)
            lib.matrix_free(c)
        q.put((True, X, S))
    except Exception as ex:  # pragma: no cover - generation-time only
        q.put((False, repr(ex), None))


def run_reference(path, alg):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_run_reference, args=((path, alg, q),))
    p.start()
    res = None
    while res is None and (p.is_alive() or not q.empty()):
        try:
            res = q.get(timeout=1.0)  # read before join: large results fill the pipe
        except Exception:
            pass
    p.join(30)
    if p.is_alive():
        p.kill()
    if res is None or not res[0]:
        return None
    return res[1], res[2]


def _parse_table(src, name, rows, cols):
    m = re.search(r"double\s+" + name + r"\s*\[\]\s*=\s*\{(.*?)\};", src, re.S)
    vals = [float(v) for v in re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?", m.group(1))]
    assert len(vals) == rows * cols, (name, len(vals))
    return np.array(vals).reshape(rows, cols)


def case_rotation():
    src = open(os.path.join(REF_C, "rotation.c")).read()
    ev = _parse_table(src, "evolErrs_rowwise", 2, 15)
    ob = _parse_table(src, "obsErrs_rowwise", 2, 16)
    a = 2 * np.pi / 16
    F = np.array([[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]])
    G = np.eye(2)
    k, es, os_ = 16, 1e-3, 1e-1
    x = np.zeros((k, 2))
    x[0] = [1.0, 0.0]
    for i in range(1, k):
        x[i] = F @ x[i - 1] + es * ev[:, i - 1]
    P = pb.empty_problem(2, 2, [k])
    for i in range(k):
        if i > 0:
            P.H[i] = np.eye(2)
            P.F[i] = F.T
            P.K[i] = (np.eye(2) / es).T
            P.K_type[i] = ord("W")
        P.G[i] = G.T
        P.o[i] = G @ x[i] + os_ * ob[:, i]
        P.C[i] = (np.eye(2) / os_).T
        P.C_type[i] = ord("W")
        P.obs_rows[i] = 2
    return P


def case_perf(n, k):
    src = open(os.path.join(REF_C, "performance.c")).read()
    F = _parse_table(src, f"F{n}", n, n)
    G = _parse_table(src, f"G{n}", n, n)
    o = _parse_table(src, f"o{n}", n, 1)[:, 0]
    P = pb.empty_problem(n, n, [k])
    for i in range(k):
        if i > 0:
            P.H[i] = np.eye(n)
            P.F[i] = F.T
            P.K[i] = np.eye(n)
            P.K_type[i] = ord("W")
        P.G[i] = G.T
        P.o[i] = o
        P.C[i] = np.eye(n)
        P.C_type[i] = ord("W")
        P.obs_rows[i] = n
    return P


def cases():
    yield "rotation", case_rotation()
    yield "perf6_k7", case_perf(6, 7)
    yield "perf6_k100", case_perf(6, 100)
    yield "perf48_k5", case_perf(48, 5)
    for k in (1, 2, 3, 17, 64):
        yield f"cv_k{k}", pb.constant_velocity([k], seed=100 + k)
    yield "cv_w_k33", pb.constant_velocity([33], seed=7, K_type="w", C_type="w")
    yield "cv_F_k20", pb.constant_velocity([20], seed=8, K_type="F", C_type="F")
    yield "cv_W_k19", pb.constant_velocity([19], seed=9, K_type="W", C_type="W")
    yield "rand_n5m3_k21", pb.random_dynamics([21], 5, 3, seed=11, per_step=True)
    yield "rand_n4m6_k13_W", pb.random_dynamics([13], 4, 6, seed=12, per_step=True, K_type="W", C_type="W")
    yield "rand_n48m24_k5", pb.random_dynamics([5], 48, 24, seed=13)
    # isolated missing observations (odd-even and ultimate only)
    P = pb.random_dynamics([24], 4, 3, seed=14, per_step=True)
    for s in (2, 7, 12, 19):
        P.obs_rows[s] = 0
    yield "rand_miss_k24", P
    P = pb.constant_velocity([40], seed=15)
    for s in (5, 10, 21, 30):
        P.obs_rows[s] = 0
    yield "cv_miss_k40", P


def save_problem(path, P, **extra):
    np.savez_compressed(path, n=P.n, mmax=P.mmax, track_start=P.track_start, H=P.H, F=P.F, c=P.c, K=P.K,
                        K_type=P.K_type, G=P.G, o=P.o, C=P.C, C_type=P.C_type, obs_rows=P.obs_rows, **extra)


def main():
    for name, P in cases():
        path = os.path.join(HERE, f"{name}.npz")
        save_problem(path, P)
        out = {}
        for alg in ("oddeven", "associative", "ultimate"):
            r = run_reference(path, alg)
            if r is not None:
                out[f"X_{alg}"], out[f"S_{alg}"] = r
        save_problem(path, P, **out)
        print(name, sorted(k for k in out if k.startswith("X_")))


if __name__ == "__main__":
    main()
