"""The device-side equation builder (kalman_gpu_expand_invariant): the packed
arrays it writes equal, bit for bit, the host-built arrays of the same
time-invariant tracks, including step ranges inside a multi-track problem,
missing observations and diagonal ('w') covariances."""
import numpy as np
import pytest

from ultimate_kalman_gb300 import native, serve
from ultimate_kalman_gb300 import problem as pb

pytestmark = pytest.mark.gpu

FIELDS = ("H", "F", "c", "K", "K_type", "G", "o", "C", "C_type", "obs_rows")


def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return torch


def _struct(arrays, n, mmax, nsteps):
    s = native.ProblemStruct()
    s.n, s.mmax, s.ntracks, s.location, s.nsteps = n, mmax, 1, native.KALMAN_GPU_DEVICE, nsteps
    for f, a in arrays.items():
        setattr(s, f, a.data_ptr())
    return s


def test_compact_track_expands_to_its_packed_arrays():
    torch = _cuda()
    spec = serve.serving_spec(257, 12, 6, np.random.default_rng(4))
    got = spec.materialize(torch, "cuda")
    P = spec.to_packed()
    for f in FIELDS:
        np.testing.assert_array_equal(got[f].cpu().numpy(), getattr(P, f), err_msg=f)


@pytest.mark.parametrize("ktype", ["C", "w"])
def test_step_ranges_missing_observations_and_diagonal_covariances(ktype):
    torch = _cuda()
    rng = np.random.default_rng(9)
    n, m, mmax, k1, k2 = 6, 3, 8, 40, 33
    N = k1 + k2
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    arrays = {f: torch.full(s, 7, dtype=d, device="cuda") for f, s, d in (
        ("H", (N, n, n), torch.float64), ("F", (N, n, n), torch.float64), ("c", (N, n), torch.float64),
        ("K", (N, n, n), torch.float64), ("K_type", (N,), torch.uint8), ("G", (N, n, mmax), torch.float64),
        ("o", (N, mmax), torch.float64), ("C", (N, mmax, mmax), torch.float64), ("C_type", (N,), torch.uint8),
        ("obs_rows", (N,), torch.int32))}
    s = _struct(arrays, n, mmax, N)
    H, F, c = rng.standard_normal((n, n)), rng.standard_normal((n, n)), rng.standard_normal(n)
    K = pb.random_spd(rng, n) if ktype == "C" else rng.uniform(1, 2, (n, 1))
    G, C = rng.standard_normal((m, n)), pb.random_spd(rng, m)
    G0, C0, o0 = rng.standard_normal((n + 1, n)), pb.random_spd(rng, n + 1), rng.standard_normal(n + 1)
    obs = rng.standard_normal((k2 - 1, m + 2))  # ldo = m + 2
    rows = np.where(rng.random(k2 - 1) < 0.3, 0, m).astype(np.int32)
    keep = {"H": dev(H.T), "F": dev(F.T), "c": dev(c), "K": dev(K.T), "G": dev(G.T), "C": dev(C.T),
            "G0": dev(G0.T), "C0": dev(C0.T), "o0": dev(o0), "o": dev(obs)}
    rows_d = torch.as_tensor(rows).cuda()
    md = native.InvariantModel(m0=n + 1, m=m, H=keep["H"].data_ptr(), F=keep["F"].data_ptr(), c=keep["c"].data_ptr(),
                               K=keep["K"].data_ptr(), K_type=ktype.encode(), G0=keep["G0"].data_ptr(),
                               o0=keep["o0"].data_ptr(), C0=keep["C0"].data_ptr(), C0_type=b"C",
                               G=keep["G"].data_ptr(), C=keep["C"].data_ptr(), C_type=b"W")
    native.expand_invariant(s, k1, k2, md, keep["o"].data_ptr(), m + 2, rows_d.data_ptr())
    torch.cuda.synchronize()
    got = {f: a.cpu().numpy() for f, a in arrays.items()}
    # the first track's steps are untouched
    for f in FIELDS:
        assert (got[f][:k1] == 7).all(), f
    t = slice(k1, N)
    assert (got["H"][t][0] == 0).all() and (got["F"][t][0] == 0).all() and (got["K"][t][0] == 0).all()
    for i in range(1, k2):
        s_ = k1 + i
        np.testing.assert_array_equal(got["H"][s_], H.T)
        np.testing.assert_array_equal(got["F"][s_], F.T)
        np.testing.assert_array_equal(got["c"][s_], c)
        if ktype == "C":
            np.testing.assert_array_equal(got["K"][s_], K.T)
        else:
            np.testing.assert_array_equal(got["K"][s_][0], K[:, 0])
            assert (got["K"][s_][1:] == 0).all()
        np.testing.assert_array_equal(got["G"][s_][:, :m], G.T)
        assert (got["G"][s_][:, m:] == 0).all()
        np.testing.assert_array_equal(got["C"][s_][:m, :m], C.T)
        assert (got["C"][s_][m:] == 0).all() and (got["C"][s_][:, m:] == 0).all()
        np.testing.assert_array_equal(got["o"][s_][:m], obs[i - 1, :m])
        assert (got["o"][s_][m:] == 0).all()
        assert got["obs_rows"][s_] == rows[i - 1]
        assert chr(got["K_type"][s_]) == ktype and chr(got["C_type"][s_]) == "W"
    np.testing.assert_array_equal(got["G"][k1][:, :n + 1], G0.T)
    np.testing.assert_array_equal(got["C"][k1][:n + 1, :n + 1], C0.T)
    np.testing.assert_array_equal(got["o"][k1][:n + 1], o0)
    assert got["obs_rows"][k1] == n + 1 and chr(got["K_type"][k1]) == "C" and chr(got["C_type"][k1]) == "C"


def test_bad_ranges_are_refused():
    torch = _cuda()
    arrays = {f: torch.zeros(4, dtype=torch.float64, device="cuda") for f in FIELDS}
    s = _struct(arrays, 2, 2, 10)
    md = native.InvariantModel(m0=3, m=1)  # m0 above mmax
    with pytest.raises(native.KalmanError):
        native.expand_invariant(s, 0, 5, md, 0, 1)
    md = native.InvariantModel(m0=0, m=0, K_type=b"C", C0_type=b"C", C_type=b"C")
    with pytest.raises(native.KalmanError):
        native.expand_invariant(s, 8, 5, md, 0, 1)  # past the problem's steps


def test_device_built_track_equals_the_host_built_track():
    """shapes.device_track (the builder) and shapes.synthetic_track (host
    numpy) give the same packed arrays for the same seed."""
    torch = _cuda()
    from ultimate_kalman_gb300 import shapes
    P = shapes.synthetic_track(300, 10, 5, seed=3)
    D = shapes.device_track(300, 10, 5, seed=3)
    for f in FIELDS:
        np.testing.assert_array_equal(D.arrays[f].cpu().numpy(), getattr(P, f), err_msg=f)
