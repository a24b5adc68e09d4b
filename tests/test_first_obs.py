"""kalman_gpu_smooth_oddeven_first_obs: tracks whose first-step observation
is kept apart from the packed rows (a prior folded into a square first
observation has n rows, the other steps m), so that the steps are stored and
copied without padding.  The results must equal the padded problem's from
kalman_gpu_smooth_oddeven_packed bit for bit (the library pads on the device
and runs the same kernels), for device and host arrays, FP64 with
covariances and the precision form, one and several host staging chunks."""
import numpy as np
import pytest

from ultimate_kalman_gb300 import native, problem as pb


def unsplit(Pc, F0, mmax):
    """The padded packed problem a first-observation problem stands for."""
    n, N = Pc.n, Pc.nsteps
    P = pb.empty_problem(n, mmax, np.diff(Pc.track_start))
    for f in ("H", "F", "c", "K", "K_type", "C_type", "obs_rows"):
        getattr(P, f)[:] = getattr(Pc, f)
    mc, m0 = Pc.mmax, F0["m0max"]
    P.G[:, :, :mc] = Pc.G.reshape(N, n, mc)
    P.o[:, :mc] = Pc.o
    P.C[:, :mc, :mc] = Pc.C.reshape(N, mc, mc)
    ts = Pc.track_start
    for t in range(Pc.ntracks):
        if ts[t + 1] > ts[t]:
            s = ts[t]
            P.G[s] = 0.0
            P.o[s] = 0.0
            P.C[s] = 0.0
            P.G[s][:, :m0] = F0["G0"][t]
            P.o[s][:m0] = F0["o0"][t]
            P.C[s][:m0, :m0] = F0["C0"][t]
            P.C_type[s] = F0["C0_type"][t]
            P.obs_rows[s] = F0["obs_rows0"][t]
    return P


def test_split_keeps_the_equations_and_drops_the_padding():
    P = pb.constant_velocity([50, 7, 1, 3], seed=2, missing=0.2, C_type="w")
    Pc, F0 = pb.split_first_obs(P)
    assert (P.mmax, Pc.mmax, F0["m0max"]) == (6, 3, 6)
    assert Pc.nbytes() < 0.8 * P.nbytes()
    Q = unsplit(Pc, F0, P.mmax)
    for f in ("H", "F", "c", "K", "K_type", "G", "o", "C", "C_type", "obs_rows"):
        np.testing.assert_array_equal(getattr(Q, f), getattr(P, f), err_msg=f)


def test_incomplete_first_observations_are_refused():
    import ctypes
    L = native.load()
    P = pb.constant_velocity([20], seed=3)
    Pc, F0 = pb.split_first_obs(P)
    s = native.ProblemStruct()
    s.n, s.mmax, s.ntracks, s.location, s.nsteps = Pc.n, Pc.mmax, 1, native.KALMAN_GPU_HOST, Pc.nsteps
    f = native.FirstObs()
    f.m0max = 0
    assert L.kalman_gpu_smooth_oddeven_first_obs(0, ctypes.byref(s), ctypes.byref(f), None) == native.KALMAN_GPU_EINVAL


def _gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")


@pytest.mark.gpu
@pytest.mark.parametrize("location", ["device", "host"])
@pytest.mark.parametrize("form", ["fp64", "fp32_refine"])
def test_equals_the_padded_problem(location, form):
    _gpu()
    P = pb.random_dynamics([300, 17, 1, 2, 129], 5, 2, seed=4, missing=0.15, K_type="w", C_type="F")
    Pc, F0 = pb.split_first_obs(P)
    assert Pc.mmax == 2 and F0["m0max"] == 5
    kw = dict(covariance=(form == "fp64"), fp32_refine=(form == "fp32_refine"))
    X, S = native.smooth(P, location=location, **kw)
    Xc, Sc = native.smooth_first_obs(Pc, F0, location=location, **kw)
    np.testing.assert_array_equal(Xc, X)
    if S is not None:
        np.testing.assert_array_equal(Sc, S)


@pytest.mark.gpu
def test_host_arrays_in_several_staging_chunks():
    """2.6 M steps: the host path stages them in chunks of whole tracks (about
    half a million steps each), each chunk with its own tracks' first
    observations."""
    _gpu()
    P = pb.constant_velocity(pb.batched_lengths(260, 5000, 15000, seed=5), seed=6)
    assert P.nsteps > 2 * (1 << 20)
    Pc, F0 = pb.split_first_obs(P)
    X, _ = native.smooth(P, location="host", covariance=False, fp32_refine=True, sweeps=1)
    Xc, _ = native.smooth_first_obs(Pc, F0, location="host", covariance=False, fp32_refine=True, sweeps=1)
    np.testing.assert_array_equal(Xc, X)
