"""The launch tuning (kalman_gpu_set_tuning) and the autotuner
(ultimate_kalman_gb300/autotune.py).

CPU: problem-class keys, the search space per class, the JSON cache, and the
library's validation of a tuning.  GPU: every tuning choice -- thread or thread
block per work item at small state dimensions, the persistent grid, the FP32
and double-float block sizes -- gives results within the parity bars of the
oracle, and block sizes do not change a result at all (the per-item
arithmetic is the same)."""
import numpy as np
import pytest

from ultimate_kalman_gb300 import autotune, native, problem as pb


@pytest.fixture(autouse=True)
def _defaults():
    native.load()
    native.set_tuning(default=True)
    yield
    native.set_tuning(default=True)


def test_class_key_buckets_lengths_and_tracks():
    k = autotune.class_key(6, 6, [100, 300, 900, 3000], True, False)
    assert k == "oddeven|n6|m6|fp32|states|L2^10|T2^2"
    assert autotune.class_key(6, 6, [5000] * 4096, True, True).split("|")[3:5] == ["dd", "cov"]
    assert autotune.class_key(48, 24, [1000000], False, True).startswith("oddeven|n48|m24|fp64|cov")


def test_candidates_follow_the_mapping():
    d = {"cta_min_n": 9, "ctas_per_sm": 4, "pair_block": 64, "weigh_block": 128}
    assert autotune.candidates("cta_min_n", 6, 6, True, False, d) == [7, 6]
    assert autotune.candidates("ctas_per_sm", 6, 6, True, False, d) == [4]  # thread mapping: no grid to tune
    assert autotune.candidates("pair_block", 6, 6, True, False, d) == [32, 64, 128]
    assert autotune.candidates("pair_block", 6, 6, False, False, d) == [64]  # FP64: not this kernel
    assert autotune.candidates("pair_block", 6, 6, True, True, d) == [64]   # double-float: not this kernel
    blocks = dict(d, cta_min_n=6)
    assert autotune.candidates("ctas_per_sm", 6, 6, True, False, blocks) == autotune.SPACE["ctas_per_sm"]
    assert autotune.candidates("weigh_block", 6, 6, True, False, blocks) == [128]
    assert autotune.candidates("cta_min_n", 12, 6, False, True, d) == [9]  # past 8 states: blocks only


def test_cache_round_trip(tmp_path):
    cache = str(tmp_path / "t.json")
    e = {"key": autotune.class_key(4, 4, [64] * 8, True, False), "tuning": {"cta_min_n": 5, "ctas_per_sm": 4,
                                                                           "pair_block": 32, "weigh_block": 256},
         "ms": 1.0, "default_ms": 1.2, "table": []}
    autotune.record(e, cache)
    assert autotune.lookup(4, 4, [64] * 8, True, False, cache) == e["tuning"]
    assert autotune.lookup(4, 4, [64] * 8, False, False, cache) is None
    t, hit = autotune.apply(4, 4, [64] * 8, True, False, cache)
    assert hit and t == e["tuning"] and native.get_tuning() == e["tuning"]


def test_library_refuses_out_of_range_tuning():
    before = native.get_tuning()
    for bad in (dict(cta_min_n=0), dict(ctas_per_sm=17), dict(pair_block=48), dict(weigh_block=512)):
        with pytest.raises(native.KalmanError) as e:
            native.set_tuning(**bad)
        assert e.value.status == native.KALMAN_GPU_EINVAL
        assert native.get_tuning() == before


def _gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")


@pytest.mark.gpu
@pytest.mark.parametrize("n,m", [(2, 1), (4, 2), (5, 3), (6, 3), (8, 4)])
def test_block_per_item_mapping_at_small_state_dimensions(n, m):
    """cta_min_n = 1 sends even 2..8-state problems to the thread-block
    kernels: FP64 (1e-11), the precision form's states (1e-9) and its
    double-float covariances (1e-9) against the oracle."""
    _gpu()
    import oracle
    P = pb.random_dynamics([300, 17, 1, 2], n, m, seed=90 + n, missing=0.1)
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert st == 0
    native.set_tuning(cta_min_n=1, ctas_per_sm=2)
    X, S = native.smooth(P, covariance=True)
    assert oracle.rel_err_states(X, Xo) < 1e-11 and oracle.rel_err_covs(S, So) < 1e-11
    X, _ = native.smooth(P, covariance=False, fp32_refine=True)
    assert oracle.rel_err_states(X, Xo) < 1e-9
    X, S = native.smooth(P, covariance=True, fp32_refine=True)
    assert oracle.rel_err_states(X, Xo) < 1e-9 and oracle.rel_err_covs(S, So) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("n", [4, 6])
def test_block_sizes_do_not_change_results(n):
    _gpu()
    P = pb.constant_velocity([2000, 333, 5], seed=3) if n == 6 else pb.random_dynamics([1500, 41], 4, 4, seed=4)
    ref, _ = native.smooth(P, covariance=False, fp32_refine=True)
    for pb_ in (32, 64, 128):
        for wb in (64, 128, 256):
            native.set_tuning(pair_block=pb_, weigh_block=wb)
            X, _ = native.smooth(P, covariance=False, fp32_refine=True)
            np.testing.assert_array_equal(X, ref)


@pytest.mark.gpu
def test_grid_size_does_not_change_results():
    _gpu()
    P = pb.random_dynamics([400, 77], 12, 6, seed=5, missing=0.1)
    ref, Sref = native.smooth(P, covariance=True)
    for c in (1, 3, 8):
        native.set_tuning(ctas_per_sm=c)
        X, S = native.smooth(P, covariance=True)
        np.testing.assert_array_equal(X, ref)
        np.testing.assert_array_equal(S, Sref)


@pytest.mark.gpu
def test_tuner_picks_a_measured_choice(tmp_path):
    _gpu()
    P = pb.constant_velocity(pb.batched_lengths(64, 50, 2000, seed=6), seed=7)
    D = native.DeviceProblem(P, covariance=False)
    cache = str(tmp_path / "t.json")
    e = autotune.tune(D, fp32_refine=True, covariance=False, sweeps=1, reps=1, cache=cache)
    assert e["ms"] <= e["default_ms"]
    assert any(all(r[k] == v for k, v in e["tuning"].items()) for r in e["table"])
    assert native.get_tuning() == e["tuning"]
    assert autotune.lookup(6, 6, np.diff(D.track_start), True, False, cache) == e["tuning"]
