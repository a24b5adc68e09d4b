"""Times one smoothing of a single synthetic track of a given shape on the GPU
(the larger-state workloads: n=48/m=24 for the associative smoother,
n=128/m=64 for the odd-even smoother, n in {4, 6, 12, 24} for serving).

The track follows the large-state workloads' recipe: F = rho Q (Q random orthogonal),
H = I, G i.i.d. N(0, 1/m), SPD noise covariances with eigenvalues in [lo, hi]
(log-uniform with --log-cov), a square step-0 observation, a fraction of
steps without observation.  Matrices are shared along the track (the work does
not depend on their values), so large k is cheap to build.

    python -m ultimate_kalman_gb300.shapes --n 48 --m 24 --k 100000 --algorithm associative
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import problem as pb


def synthetic_track(k, n, m, rho=0.99, lo=0.1, hi=1.0, log_cov=False, missing=0.05, seed=0):
    rng = np.random.default_rng(seed)
    P = pb.empty_problem(n, max(n, m), [k])
    mx = max(n, m)
    Fm = rho * pb.random_orthogonal(rng, n)
    Gm = rng.standard_normal((m, n)) / np.sqrt(m)
    Kc = pb.random_spd(rng, n, lo, hi, log_cov)
    Cc = pb.random_spd(rng, m, lo, hi, log_cov)
    P.H[1:] = np.eye(n)
    P.F[1:] = Fm.T
    P.K[1:] = Kc.T
    Gt = np.zeros((n, mx))
    Gt[:, :m] = Gm.T
    Ct = np.zeros((mx, mx))
    Ct[:m, :m] = Cc.T
    P.G[1:] = Gt
    P.C[1:] = Ct
    P.o[1:, :m] = rng.standard_normal((k - 1, m))
    P.obs_rows[1:] = m
    if missing > 0:
        P.obs_rows[1:][rng.random(k - 1) < missing] = 0
    G0 = np.zeros((n, mx))
    G0[:, :n] = np.eye(n)
    C0 = np.zeros((mx, mx))
    C0[:n, :n] = np.eye(n)
    P.G[0], P.C[0] = G0, C0
    P.o[0, :n] = rng.standard_normal(n)
    P.obs_rows[0] = n
    return P


def device_track(k, n, m, rho=0.99, lo=0.1, hi=1.0, log_cov=False, missing=0.05, seed=0, covariance=True,
                 with_builder=False):
    """synthetic_track's track built on the GPU by the library's equation
    builder (kalman_gpu_expand_invariant): only the model, the observations
    and the step row counts cross the host link, so tracks of 10^6 steps with
    48 states (92 GB of per-step equations) need no host copy of them.
    Returns a native.DeviceProblem."""
    import torch
    from . import native
    rng = np.random.default_rng(seed)
    mx = max(n, m)
    Fm = rho * pb.random_orthogonal(rng, n)
    Gm = rng.standard_normal((m, n)) / np.sqrt(m)
    Kc = pb.random_spd(rng, n, lo, hi, log_cov)
    Cc = pb.random_spd(rng, m, lo, hi, log_cov)
    o = rng.standard_normal((k - 1, m))
    rows = np.full(k - 1, m, dtype=np.int32)
    if missing > 0:
        rows[rng.random(k - 1) < missing] = 0
    o0 = rng.standard_normal(n)
    f64 = dict(dtype=torch.float64, device="cuda")
    arrays = {"H": torch.empty((k, n, n), **f64), "F": torch.empty((k, n, n), **f64), "c": torch.empty((k, n), **f64),
              "K": torch.empty((k, n, n), **f64), "K_type": torch.empty(k, dtype=torch.uint8, device="cuda"),
              "G": torch.empty((k, n, mx), **f64), "o": torch.empty((k, mx), **f64),
              "C": torch.empty((k, mx, mx), **f64), "C_type": torch.empty(k, dtype=torch.uint8, device="cuda"),
              "obs_rows": torch.empty(k, dtype=torch.int32, device="cuda")}
    D = native.DeviceProblem.from_arrays(n, mx, [0, k], arrays, covariance)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a)).cuda()
    eye = dev(np.eye(n))
    keep = [eye, dev(Fm.T), dev(np.zeros(n)), dev(Kc.T), dev(o0), dev(Gm.T), dev(Cc.T), dev(o), dev(rows)]
    md = native.InvariantModel(m0=n, m=m, H=eye.data_ptr(), F=keep[1].data_ptr(), c=keep[2].data_ptr(),
                               K=keep[3].data_ptr(), K_type=b"C", G0=eye.data_ptr(), o0=keep[4].data_ptr(),
                               C0=eye.data_ptr(), C0_type=b"C", G=keep[5].data_ptr(), C=keep[6].data_ptr(),
                               C_type=b"C")
    def build():
        native.expand_invariant(D.struct, 0, k, md, keep[7].data_ptr(), m, keep[8].data_ptr(),
                                torch.cuda.current_stream())

    build()
    torch.cuda.synchronize()
    return (D, build) if with_builder else D


def main():
    import torch
    from . import native
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--n", type=int, default=48)
    ap.add_argument("--m", type=int, default=24)
    ap.add_argument("--k", type=int, default=100000)
    ap.add_argument("--algorithm", default="associative", choices=["oddeven", "associative"])
    ap.add_argument("--no-covariance", action="store_true")
    ap.add_argument("--fp32-refine", action="store_true", help="the precision form (odd-even; states)")
    ap.add_argument("--sweeps", type=int, default=0)
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--log-cov", action="store_true", help="covariance eigenvalues log-uniform in [1e-3, 1]")
    ap.add_argument("--device-build", action="store_true",
                    help="build the track on the GPU with the equation builder (no host copy of the equations)")
    ap.add_argument("--batched", type=int, default=0, metavar="TRACKS",
                    help="instead of one track: the first TRACKS of the batched workload (constant-velocity, n=6, "
                         "m=3, lengths log-uniform in [100, 20000]); a small case of the same kernels for profiling")
    ap.add_argument("--time-build", action="store_true",
                    help="time the equation builder on the track (CUDA events) instead of smoothing it")
    args = ap.parse_args()
    if args.time_build:
        D, build = device_track(args.k, args.n, args.m, covariance=False, with_builder=True)
        for _ in range(3):
            build()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(args.repeats):
            build()
        e.record()
        torch.cuda.synchronize()
        ms = s.elapsed_time(e) / args.repeats
        written = D.input_bytes()
        print(json.dumps({"n": args.n, "m": args.m, "k": args.k, "build_ms": ms, "written_gb": written / 1e9,
                          "write_gbs": written / (ms * 1e-3) / 1e9}))
        return
    lo = 1e-3 if args.log_cov else 0.1
    rho = 0.995 if args.n >= 128 else 0.99
    cov = not args.no_covariance and not (args.fp32_refine and args.batched == 0)
    if args.batched:
        P = pb.constant_velocity(pb.batched_lengths(4096, 100, 20000, seed=0)[:args.batched], seed=1000)
        D = native.DeviceProblem(P, covariance=True)
        args.k, args.n, args.m = int(P.nsteps), 6, 3
    elif args.device_build:
        D = device_track(args.k, args.n, args.m, rho=rho, lo=lo, log_cov=args.log_cov, covariance=cov)
    else:
        P = synthetic_track(args.k, args.n, args.m, lo=lo, log_cov=args.log_cov, rho=rho)
        D = native.DeviceProblem(P, covariance=True)
    kw = dict(covariance=cov, fp32_refine=args.fp32_refine, sweeps=args.sweeps)
    D.smooth(args.algorithm, **kw)
    torch.cuda.synchronize()
    native.profile_enable(True)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(args.repeats):
        D.smooth(args.algorithm, **kw)
    e.record()
    torch.cuda.synchronize()
    prof = native.profile_read()
    native.profile_enable(False)
    ms = s.elapsed_time(e) / args.repeats
    rel_err = None
    if args.fp32_refine:  # against the plain FP64 smoothing of the same track
        X32 = D.state.clone()
        D.smooth(args.algorithm, covariance=False)
        X64 = D.state
        rel_err = float(((X32 - X64).abs().amax(dim=1) / X64.abs().amax(dim=1)).max().item())
    print(json.dumps({"algorithm": args.algorithm, "n": args.n, "m": args.m, "k": args.k, "covariance": cov,
                      "fp32_refine": args.fp32_refine, "rel_err_vs_fp64": rel_err,
                      "ms": ms, "steps_per_s": args.k / (ms * 1e-3),
                      "per_kernel_ms": {k2: v[0] / args.repeats for k2, v in prof.items()},
                      "input_gb": D.input_bytes() / 1e9}))


if __name__ == "__main__":
    main()
