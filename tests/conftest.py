"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; the rest run on
CPU.  The oracle package (test infrastructure) is importable from here."""
import glob
import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from ultimate_kalman_gb300 import problem as pb  # noqa: E402

GOLDEN = sorted(glob.glob(os.path.join(REPO, "tests", "golden", "*.npz")))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


def load_golden(path):
    d = np.load(path)
    P = pb.PackedProblem(int(d["n"]), int(d["mmax"]), d["track_start"],
                         *[d[f] for f in ("H", "F", "c", "K", "K_type", "G", "o", "C", "C_type", "obs_rows")])
    return P, d


@pytest.fixture(params=GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def golden(request):
    return load_golden(request.param)


_PARITY = []


@pytest.fixture(scope="session")
def parity_log():
    """record(case, **errors): keeps the achieved relative errors of a parity
    test; at the end of the session they are printed and, when the
    environment names a file in UKG_PARITY_LOG, written there as JSON."""
    def record(case, **errors):
        _PARITY.append({"case": case, **{k: float(v) for k, v in errors.items()}})
    yield record
    if _PARITY:
        worst = {}
        for r in _PARITY:
            for k, v in r.items():
                if k != "case":
                    worst[k] = max(worst.get(k, 0.0), v)
        print("\nachieved relative errors (max over cases):", json.dumps(worst))
        path = os.environ.get("UKG_PARITY_LOG")
        if path:
            with open(path, "w") as f:
                json.dump({"worst": worst, "cases": _PARITY}, f, indent=1)
