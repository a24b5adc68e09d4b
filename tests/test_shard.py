"""Sharding the batched smoother across processes by track
(ultimate_kalman_gb300/shard.py): the step-balanced split, the cut of a packed
problem, and the merge of per-rank results on rank 0 through
torch.distributed -- with two gloo ranks on the CPU -- and, on a GPU, that
smoothing the shards one after another gives the whole batch's results bit for
bit (tracks are independent)."""
import os
import socket

import numpy as np
import pytest

from ultimate_kalman_gb300 import problem as pb
from ultimate_kalman_gb300 import shard


def test_split_balances_steps_by_whole_tracks():
    rng = np.random.default_rng(3)
    lengths = rng.integers(1, 5000, size=257)
    for world in (1, 2, 3, 8):
        b = shard.split_tracks(lengths, world)
        assert b[0] == 0 and b[-1] == len(lengths) and (np.diff(b) >= 0).all()
        steps = np.array([lengths[b[r]:b[r + 1]].sum() for r in range(world)])
        assert steps.sum() == lengths.sum()
        assert np.abs(steps - lengths.sum() / world).max() <= lengths.max()


def test_more_ranks_than_tracks_leaves_ranks_empty():
    b = shard.split_tracks([5, 3], 4)
    assert b[0] == 0 and b[-1] == 2 and (np.diff(b) >= 0).all()
    P = pb.constant_velocity([5, 3], seed=1)
    parts = [shard.shard(P, r, 4) for r in range(4)]
    assert sum(q.nsteps for q, _ in parts if q is not None) == P.nsteps
    assert any(q is None for q, _ in parts)


def test_shards_put_together_are_the_problem():
    P = pb.random_dynamics([40, 7, 1, 300, 2, 19], 4, 2, seed=5, missing=0.1)
    parts = [q for q in (shard.shard(P, r, 3)[0] for r in range(3)) if q is not None]
    assert [q.ntracks for q in parts] == [3, 1, 2]  # the 300-step track on its own
    for f in ("H", "F", "c", "K", "K_type", "G", "o", "C", "C_type", "obs_rows"):
        np.testing.assert_array_equal(np.concatenate([getattr(q, f) for q in parts]), getattr(P, f), err_msg=f)


def stand_in_results(P):
    """Per-step arrays that depend only on each step's own data (the states
    and covariance shapes of a smoothing), for the merge plumbing."""
    X = P.c + P.o[:, :P.n].sum(axis=1, keepdims=True)
    S = P.K * (1.0 + np.abs(P.o).sum(axis=1))[:, None, None]
    return X, S


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        for lengths in ([40, 7, 1, 300, 2, 19, 64], [33]):  # the second leaves rank 1 without tracks
            P = pb.constant_velocity(lengths, seed=9)
            mine, _ = shard.shard(P, rank, world)
            if mine is None:
                X = np.zeros((0, P.n))
                S = np.zeros((0, P.n, P.n))
            else:
                X, S = stand_in_results(mine)
            Xa, Sa = shard.merge(X, rank, world), shard.merge(S, rank, world)
            if rank == 0:
                Xw, Sw = stand_in_results(P)
                np.testing.assert_array_equal(Xa, Xw)
                np.testing.assert_array_equal(Sa, Sw)
            else:
                assert Xa is None and Sa is None
        dist.barrier()
        if rank == 0:
            open(out, "w").write("ok")
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_merge_results_in_track_order(tmp_path):
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "rank0.txt")
    mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
    assert open(out).read() == "ok"


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "fp32_refine"])
def test_shards_smoothed_apart_equal_the_whole_batch(form):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from ultimate_kalman_gb300 import native
    P = pb.constant_velocity(pb.batched_lengths(64, 50, 3000, seed=4), seed=5)
    kw = dict(covariance=(form == "fp64"), fp32_refine=(form == "fp32_refine"))
    X, S = native.smooth(P, **kw)
    for world in (2, 3):
        parts = [native.smooth(q, **kw) for q in (shard.shard(P, r, world)[0] for r in range(world))]
        np.testing.assert_array_equal(np.concatenate([x for x, _ in parts]), X)
        if S is not None:
            np.testing.assert_array_equal(np.concatenate([s for _, s in parts]), S)
