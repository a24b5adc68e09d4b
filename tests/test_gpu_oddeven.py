"""Parity of the CUDA odd-even smoother (through the C ABI) with the oracle,
the reference's own outputs and the dense least-squares solution.

Tolerance: 1e-11 relative error (normwise per step) for FP64 states and
covariances, against the oracle and the reference."""
import numpy as np
import pytest

import oracle
from ultimate_kalman_gb300 import native, problem as pb

pytestmark = pytest.mark.gpu
TOL = 1e-11


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    native.load()


def check(P, X, S, tol=TOL, cov=True):
    st, Xo, So = oracle.smooth(P, "oddeven", covariance=cov)
    assert st == 0
    assert oracle.rel_err_states(X, Xo) < tol
    if cov:
        assert oracle.rel_err_covs(S, So) < tol


def test_golden_against_reference(golden):
    P, d = golden
    X, S = native.smooth(P, "oddeven")
    ref = "oddeven" if "X_oddeven" in d else "ultimate"
    assert oracle.rel_err_states(X, d[f"X_{ref}"]) < TOL
    assert oracle.rel_err_covs(S, d[f"S_{ref}"]) < TOL
    check(P, X, S)


@pytest.mark.parametrize("k", list(range(1, 18)) + [31, 32, 33, 63, 64, 65, 100, 257])
def test_lengths_every_parity_pattern(k):
    P = pb.constant_velocity([k], seed=k)
    X, S = native.smooth(P)
    check(P, X, S)


@pytest.mark.parametrize("n,m", [(1, 1), (2, 1), (3, 6), (4, 2), (5, 3), (6, 3), (8, 4), (12, 6)])
@pytest.mark.parametrize("cov", ["C", "W", "w", "F"])
def test_shapes_cov_types_missing(n, m, cov):
    """Tall and flat G, every covariance form, 35% missing observations
    (including the consecutive and trailing ones the reference rejects)."""
    P = pb.random_dynamics([13, 6, 1, 9, 2], n, m, seed=n * 10 + m, K_type=cov, C_type=cov, missing=0.35,
                           per_step=True)
    X, S = native.smooth(P)
    check(P, X, S)
    Xd, Sd = oracle.dense_smooth(P)
    assert oracle.rel_err_states(X, Xd) < TOL
    assert oracle.rel_err_covs(S, Sd) < TOL


def test_batched_uneven_tracks():
    lens = pb.batched_lengths(300, 1, 600, seed=3)
    P = pb.constant_velocity(lens, seed=4, missing=0.05)
    X, S = native.smooth(P)
    check(P, X, S)


def test_full_size_single_track_100k():
    """The plain single-track workload (n=6, m=3, k=100,000) at full size."""
    P = pb.constant_velocity([100000], seed=11)
    X, S = native.smooth(P)
    check(P, X, S)


def test_host_and_device_locations_agree():
    P = pb.random_dynamics([40, 17], 5, 3, seed=2, per_step=True)
    Xd, Sd = native.smooth(P, location="device")
    Xh, Sh = native.smooth(P, location="host")
    np.testing.assert_array_equal(Xd, Xh)
    np.testing.assert_array_equal(Sd, Sh)


@pytest.mark.parametrize("fp32", [False, True])
def test_host_location_in_pipelined_chunks(fp32):
    """Host arrays of more than 2^19 steps are staged in chunks of whole tracks
    (copies overlapped with smoothing); the results equal the device path's."""
    P = pb.constant_velocity([600000, 600000, 100000, 37], seed=9)
    cov = not fp32
    Xd, Sd = native.smooth(P, covariance=cov, fp32_refine=fp32, location="device")
    Xh, Sh = native.smooth(P, covariance=cov, fp32_refine=fp32, location="host")
    np.testing.assert_array_equal(Xd, Xh)
    if cov:
        np.testing.assert_array_equal(Sd, Sh)


def test_no_covariance_gives_same_states():
    P = pb.constant_velocity([77, 5], seed=6)
    X1, S1 = native.smooth(P, covariance=True)
    X2, S2 = native.smooth(P, covariance=False)
    assert S2 is None
    np.testing.assert_array_equal(X1, X2)


def test_reference_entry_points_with_step_structs():
    """kalman_smooth_oddeven on kalman_step_equations_t structs, per track and
    through the batched entry, equals the packed path."""
    P = pb.random_dynamics([19, 4, 1], 4, 2, seed=8, per_step=True, missing=0.2, K_type="w", C_type="F")
    Xp, Sp = native.smooth(P)
    X1, S1, st1 = native.smooth_equations(P, "oddeven")
    X2, S2, st2 = native.smooth_equations(P, "oddeven", batched=True)
    assert st1 == 0 and st2 == 0
    np.testing.assert_array_equal(X1, Xp)
    np.testing.assert_array_equal(S1, Sp)
    np.testing.assert_array_equal(X2, Xp)
    X3, S3, st3 = native.smooth_equations(P, "oddeven", covariance=False)
    assert S3 is None and st3 == 0
    np.testing.assert_array_equal(X3, Xp)


def test_unobservable_reports_singular():
    P = pb.constant_velocity([1, 5], seed=1)
    P.obs_rows[0] = 3  # one step observed by 3 rows of 6 unknowns
    with pytest.raises(native.KalmanError) as e:
        native.smooth(P)
    assert e.value.status == 4


def test_bounded_wait_gives_up_and_the_context_stays_usable():
    """The device side of a bounded wait that runs out (an mbarrier armed for
    a transfer nothing delivers): the kernel gives up after its bound, the host
    reads the error flag and reports ECUDA, and the next smoothing on the same
    context is correct."""
    import time
    L = native.load()
    t0 = time.perf_counter()
    assert L.kalman_gpu_check_bounded_wait(None) == native.KALMAN_GPU_ECUDA
    assert "did not complete in time" in native.last_error()[1]
    assert time.perf_counter() - t0 < 30.0
    P = pb.constant_velocity([300, 7], seed=8)
    X, S = native.smooth(P)
    check(P, X, S)


@pytest.mark.parametrize("location", ["device", "host"])
@pytest.mark.parametrize("fp32_refine", [False, True])
def test_malformed_observation_rows(location, fp32_refine):
    """Observation rows outside [0, mmax] are reported as malformed input by
    the kernels that read them, for device and host arrays."""
    P = pb.constant_velocity([6, 40], seed=1)
    P.obs_rows[2] = P.mmax + 3
    P.obs_rows[20] = -1
    with pytest.raises(native.KalmanError) as e:
        native.smooth(P, location=location, covariance=not fp32_refine, fp32_refine=fp32_refine)
    assert e.value.status == 1
    assert "malformed input" in native.last_error()[1]


@pytest.mark.parametrize("n,k", [(9, 41), (12, 300), (24, 120), (48, 40)])
def test_larger_states_cta_path(n, k):
    """State dimensions past 8 run one thread block per item: parity with the
    oracle (states and covariances), with missing observations and tracks of
    length 1 and 2."""
    P = pb.random_dynamics([k, 37, 1, 2], n, n // 2, seed=4 + n, per_step=True, missing=0.1)
    X, S = native.smooth(P)
    check(P, X, S)


def test_n128_m64_log_uniform_covariances():
    """n = 128, m = 64 (the largest shape this build accepts), all covariance
    types of the reference in one problem."""
    P = pb.random_dynamics([23, 6], 128, 64, seed=21, per_step=True, K_type="W", C_type="F")
    X, S = native.smooth(P)
    check(P, X, S)
    X2, _ = native.smooth(P, covariance=False, fp32_refine=True)
    assert oracle.rel_err_states(X2, X) < 1e-11


@pytest.mark.parametrize("fp32", [False, True])
def test_cta_path_every_length_1_to_17(fp32):
    """The CTA kernels over every track length 1..17 (every parity of every
    level, odd-length fix-ups, one-step base cases) in one batch, n = 10."""
    P = pb.random_dynamics(list(range(1, 18)), 10, 5, seed=12, per_step=True, missing=0.15)
    if fp32:
        X, _ = native.smooth(P, covariance=False, fp32_refine=True)
        st, Xo, _ = oracle.smooth(P, "oddeven", covariance=False)
        assert st == 0 and oracle.rel_err_states(X, Xo) < 1e-9
    else:
        X, S = native.smooth(P)
        check(P, X, S)


def test_concurrent_host_threads_with_different_shapes():
    """Host threads smoothing problems of different state dimensions at the
    same time, each on its own stream (the serving lanes): every call
    succeeds and equals the same problem smoothed alone, bit for bit.  The
    FP64 kernels shared between shapes need different amounts of dynamic
    shared memory, so a per-call kernel attribute would race here."""
    import threading
    import torch
    probs = {4: pb.random_dynamics([3000, 17], 4, 2, seed=41), 6: pb.constant_velocity([2500, 33], seed=42),
             5: pb.random_dynamics([2000, 9], 5, 3, seed=43)}
    alone = {n: native.smooth(P, "oddeven", covariance=True) for n, P in probs.items()}
    errors, results = [], {}

    def work(n):
        try:
            torch.cuda.set_device(0)
            st = torch.cuda.Stream()
            D = native.DeviceProblem(probs[n], covariance=True)
            for _ in range(20):
                with torch.cuda.stream(st):
                    D.smooth("oddeven", covariance=True, stream=st)
            torch.cuda.synchronize()
            results[n] = D.results()
        except Exception as e:  # reported below
            errors.append(f"n={n}: {e}")

    threads = [threading.Thread(target=work, args=(n,)) for n in probs]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for n, (X, S) in results.items():
        np.testing.assert_array_equal(X, alone[n][0])
        np.testing.assert_array_equal(S, alone[n][1])


def test_bulk_structs_through_the_batched_reference_entry_equal_the_packed_path():
    """kalman_gpu_smooth_tracks on numpy-built step structs (the bench's
    struct-API end-to-end leg) gives the packed entry point's states bit for
    bit, FP64 and precision form, on repeated calls (each frees the previous
    call's result matrices)."""
    P = pb.random_dynamics([700, 3, 129, 1], 5, 3, seed=31, missing=0.1, K_type="w", C_type="F")
    V = native.EquationsView(P)
    for f32 in (False, True):
        Xp, _ = native.smooth(P, "oddeven", covariance=False, fp32_refine=f32)
        for _ in range(2):
            assert V.smooth_tracks("oddeven", fp32_refine=f32) == 0, native.last_error()
            np.testing.assert_array_equal(V.states(np.arange(P.nsteps)), Xp)


@pytest.mark.parametrize("n,m", [(4, 2), (6, 3), (6, 6)])
def test_register_tiled_covariance_solve_at_every_level(n, m, parity_log):
    """n = 4 and 6 run the covariance back-substitution register-tiled
    (solve_cov_reg_kernel): FP64 and double-float against the oracle at
    every recursion parity pattern, with missing observations."""
    lens = [1, 2, 3, 5, 8, 17, 33, 64, 129, 700]
    P = (pb.constant_velocity(lens, seed=51, missing=0.1) if (n, m) == (6, 3)
         else pb.random_dynamics(lens, n, m, seed=52 + n + m, missing=0.1))
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert st == 0
    for f32 in (False, True):
        X, S = native.smooth(P, "oddeven", covariance=True, fp32_refine=f32)
        ex, es = oracle.rel_err_states(X, Xo), oracle.rel_err_covs(S, So)
        parity_log(f"register-tiled covariance n={n} m={m} {'double-float' if f32 else 'FP64'}", states=ex, covs=es)
        assert ex < (1e-9 if f32 else 1e-11) and es < (1e-9 if f32 else 1e-11), (f32, ex, es)
