"""The level-0 weighing stages the caller's blocks into shared memory with
bulk asynchronous copies when the arrays are 16-byte aligned, and reads them
directly otherwise; both give the same results.  Problem sizes cover full and
partial 128-step blocks and block sizes that are and are not multiples of 16
bytes (odd state dimension)."""
import numpy as np
import pytest
import torch

import oracle
from ultimate_kalman_gb300 import native, problem as pb

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    native.load()


@pytest.mark.parametrize("n,m,lens", [(6, 3, [127, 1, 300]), (5, 3, [257, 11]), (3, 2, [129, 128]),
                                      (4, 4, [128, 128, 128])])
def test_aligned_and_misaligned_inputs_agree(n, m, lens):
    P = pb.random_dynamics(lens, n, m, seed=n * m, per_step=True, missing=0.1)
    D = native.DeviceProblem(P, covariance=True)
    D.smooth("oddeven")
    Xa, Sa = D.results()
    # the same arrays at an address 8 bytes past a 16-byte boundary
    shifted = {}
    for f in ("H", "F", "c", "K", "G", "o", "C"):
        a = D.arrays[f]
        buf = torch.empty(a.numel() + 1, dtype=a.dtype, device=a.device)
        view = buf[1:].view(a.shape)
        view.copy_(a)
        shifted[f] = (buf, view)
        setattr(D.struct, f, view.data_ptr())
    D.smooth("oddeven")
    Xb, Sb = D.results()
    np.testing.assert_array_equal(Xa, Xb)
    np.testing.assert_array_equal(Sa, Sb)
    st, Xo, So = oracle.smooth(P, "oddeven")
    assert oracle.rel_err_states(Xa, Xo) < 1e-11
    assert oracle.rel_err_covs(Sa, So) < 1e-11
