"""A compiled C client of the drop-in boundary (tests/c_client/smooth_client.c):
built with gcc against include/ only, linked with -lukgpu, and driving the
reference API (kalman_create_options / evolve / observe / smooth / estimate /
covariance).  On a machine without a GPU the program must still build, link
and run, and report KALMAN_GPU_ENODEV with NaN estimates; on the GPU its
estimates and covariances equal the reference's outputs of the golden cases
(c/rotation.c's example, a tall/flat case with 'W'/'w' weights and missing
observations) within 1e-11."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import REPO, load_golden

SRC = os.path.join(REPO, "tests", "c_client", "smooth_client.c")
LIBDIR = os.path.join(REPO, "ultimate_kalman_gb300")


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    if not os.path.exists(os.path.join(LIBDIR, "libukgpu.so")):
        pytest.skip("libukgpu.so not built")
    exe = str(tmp_path_factory.mktemp("cclient") / "smooth_client")
    r = subprocess.run([gcc, "-std=c11", "-O1", "-Wall", "-Werror", "-I", os.path.join(REPO, "include"), SRC,
                        "-L", LIBDIR, "-lukgpu", "-Wl,-rpath," + LIBDIR, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def write_input(P, path):
    """The client's input format: one track of a packed problem."""
    n, k = int(P.n), int(P.nsteps)
    with open(path, "wb") as f:
        f.write(struct.pack("ii", n, k))
        col = lambda A: np.asarray(A, dtype=np.float64).T.tobytes()  # packed blocks hold M^T row-major = M column-major
        for s in range(k):
            if s > 0:
                f.write(P.H[s].tobytes() + P.F[s].tobytes() + P.c[s].tobytes())
                kt = chr(P.K_type[s])
                f.write(kt.encode())
                f.write(P.K[s].reshape(-1)[:n].tobytes() if kt == "w" else P.K[s].tobytes())
            m = int(P.obs_rows[s])
            f.write(struct.pack("i", m))
            if m > 0:
                G = P.G[s].T[:m, :]  # (m x n)
                f.write(col(G))
                f.write(P.o[s][:m].tobytes())
                ct = chr(P.C_type[s])
                f.write(ct.encode())
                f.write(P.C[s].reshape(-1)[:m].tobytes() if ct == "w" else col(P.C[s].T[:m, :m]))


def run_client(exe, P, alg, tmp_path):
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(P, fin)
    r = subprocess.run([exe, fin, fout, alg], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = open(fout, "rb").read()
    status = struct.unpack("i", raw[:4])[0]
    n, k = P.n, P.nsteps
    vals = np.frombuffer(raw[4:], dtype=np.float64).reshape(k, n + n * n)
    X = vals[:, :n]
    S = vals[:, n:].reshape(k, n, n).transpose(0, 2, 1)  # column-major blocks
    return status, X, S, r.stdout


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_client_builds_links_and_reports_no_device(client, tmp_path):
    if gpu_available():
        pytest.skip("this machine has a GPU (the GPU test runs the client)")
    P, _ = load_golden(os.path.join(REPO, "tests", "golden", "rotation.npz"))
    status, X, S, out = run_client(client, P, "oddeven", tmp_path)
    assert status == 5, out  # KALMAN_GPU_ENODEV
    assert np.isnan(X).all() and np.isnan(S).all()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["rotation", "rand_n4m6_k13_W", "cv_w_k33", "cv_miss_k40"])
@pytest.mark.parametrize("alg", ["oddeven", "associative"])
def test_client_matches_reference_outputs(client, tmp_path, case, alg):
    if not gpu_available():
        pytest.skip("needs a CUDA device")
    P, d = load_golden(os.path.join(REPO, "tests", "golden", case + ".npz"))
    if f"X_{alg}" not in d:
        pytest.skip("the reference smoother does not accept this input")
    status, X, S, out = run_client(client, P, alg, tmp_path)
    assert status == 0, out
    Xr, Sr = d[f"X_{alg}"], d[f"S_{alg}"]
    ok = np.all(np.isfinite(Sr), axis=(1, 2))  # the reference associative's last covariance is NaN
    rel = lambda A, B: float((np.abs(A - B).reshape(len(A), -1).max(1) / np.abs(B).reshape(len(B), -1).max(1)).max())
    assert rel(X, Xr) < 1e-11
    assert rel(S[ok], Sr[ok]) < 1e-11
