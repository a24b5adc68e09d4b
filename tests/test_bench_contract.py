"""The bench's host-side pieces, on any machine: the roofline of the dominant
kernel is never a silent zero whichever kernel dominates (the weighing against
HBM by the compulsory bytes, an FP32 kernel against the FP32 FMA peak by the
modelled flops), the whole-step figure, the per-rank workloads, and the
reference arm's JSON line (run on a small sample with the oracle's C port)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import REPO

sys.path.insert(0, REPO)
import bench  # noqa: E402
from ultimate_kalman_gb300 import flops, problem as pb  # noqa: E402


@pytest.fixture(scope="module")
def model():
    lens = pb.batched_lengths(4096, 100, 20000, seed=0)
    fl32 = flops.plan_flops_fast_fp32(lens, 6, 3, sweeps=1)
    fl32.pop("weigh_kernel")
    return lens, fl32, flops.compulsory_bytes(lens, 6, 3), flops.plan_bytes_fast(lens, 6, 3, fp32=True, sweeps=1)


@pytest.mark.parametrize("weigh_ms,pair_ms", [(8.6, 8.9), (9.0, 8.9)])
def test_roofline_of_the_dominant_kernel_is_never_zero(model, weigh_ms, pair_ms):
    lens, fl32, comp, by32 = model
    steps = 5
    prof = {"weigh_kernel": (weigh_ms * steps, steps), "fp32_pair_kernel": (pair_ms * steps, 14 * steps),
            "refine_residual_kernel": (4.3 * steps, steps), "tail_kernel": (0.5 * steps, 15 * steps)}
    r = bench.roofline_for(prof, fl32, steps, 1.26, 74.0, 6697.8, comp[0], by32)
    assert r["kernel"] == ("weigh_kernel" if weigh_ms > pair_ms else "fp32_pair_kernel")
    assert 0.0 < r["frac"] < 1.5 and r["achieved"] > 0
    if r["kernel"] == "weigh_kernel":
        assert (r["bound"], r["unit"]) == ("hbm", "GB/s")
        assert r["achieved"] == pytest.approx(comp[0] / (weigh_ms * 1e-3) / 1e9)
    else:
        assert (r["bound"], r["unit"]) == ("fp32", "TFLOP/s")
    w = bench.roofline_for({"weigh_kernel": prof["weigh_kernel"]}, fl32, steps, 1.26, 74.0, 6697.8, comp[0], by32)
    assert w["bound"] == "hbm" and 0.2 < w["frac"] < 0.4


def test_whole_step_and_compulsory_bytes(model):
    lens, _, comp, _ = model
    N = int(np.sum(lens))
    assert comp == (N * 1152.0, N * 48.0)  # n=6, m=3: F, H, K, c, G, o, C in; states out
    ws = bench.whole_step(comp, 27.6, 6697.8)
    assert ws["frac"] == pytest.approx((comp[0] + comp[1]) / 27.6e-3 / 1e9 / 6697.8)


def test_ranks_get_their_own_seeded_tracks():
    a, b = bench.workload(8, 0), bench.workload(8, 1)
    np.testing.assert_array_equal(a.track_start, b.track_start)  # same lengths: weak scaling
    assert not np.array_equal(a.o, b.o)                          # different data per rank


def test_reference_arm_prints_one_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--tracks", "16"], cwd=REPO, capture_output=True, text=True, timeout=600,
                       env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([x for x in r.stdout.splitlines() if x.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "steps/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
