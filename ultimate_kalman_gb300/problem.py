"""Packed smoothing problems and the synthetic workloads they are benchmarked on.

A ``PackedProblem`` is the host-side image of ``kalman_gpu_problem_t``
(include/kalman_gpu.h): the steps of several independent tracks concatenated,
every block stored column-major.  Arrays are shaped so that ``arr[s]`` is the
TRANSPOSE of step s's matrix (so that memory is column-major):

    H[s].T, F[s].T, K[s].T      n x n          (K 'w': K[s].reshape(-1)[:n])
    c[s]                        n
    G[s].T[:m_s]                m_s x n, leading dimension mmax
    o[s][:m_s]                  m_s
    C[s].T[:m_s, :m_s]          m_s x m_s      (C 'w': C[s].reshape(-1)[:m_s])

The equations are those of UltimateKalman (c/kalman.h:56-75):
    H_i x_i = F_i x_{i-1} + c_i + e_i,   cov(e_i) given by (K_i, K_type_i)
    G_i x_i = o_i + d_i,                 cov(d_i) given by (C_i, C_type_i)
Step 0 of each track has no evolution equation.

The workload generators follow the synthetic configurations of the smoothers'
benchmark (constant-velocity tracks; random orthogonal dynamics) with seeded
NumPy generators.  They run on the host and are not part of the smoothing path.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class PackedProblem:
    n: int
    mmax: int
    track_start: np.ndarray  # int64 [ntracks+1]
    H: np.ndarray
    F: np.ndarray
    c: np.ndarray
    K: np.ndarray
    K_type: np.ndarray  # uint8 [nsteps]
    G: np.ndarray
    o: np.ndarray
    C: np.ndarray
    C_type: np.ndarray  # uint8 [nsteps]
    obs_rows: np.ndarray  # int32 [nsteps]

    @property
    def nsteps(self) -> int:
        return int(self.track_start[-1])

    @property
    def ntracks(self) -> int:
        return len(self.track_start) - 1

    def track_lengths(self) -> np.ndarray:
        return np.diff(self.track_start)

    def nbytes(self) -> int:
        return sum(getattr(self, f).nbytes for f in ("H", "F", "c", "K", "K_type", "G", "o", "C", "C_type", "obs_rows"))

    def select_tracks(self, tracks) -> "PackedProblem":
        """A new problem holding only the given tracks (in that order)."""
        idx = np.concatenate([np.arange(self.track_start[t], self.track_start[t + 1]) for t in tracks])
        lens = np.array([self.track_start[t + 1] - self.track_start[t] for t in tracks], dtype=np.int64)
        ts = np.zeros(len(tracks) + 1, dtype=np.int64)
        ts[1:] = np.cumsum(lens)
        kw = {f: np.ascontiguousarray(getattr(self, f)[idx]) for f in
              ("H", "F", "c", "K", "K_type", "G", "o", "C", "C_type", "obs_rows")}
        return PackedProblem(self.n, self.mmax, ts, **kw)


    def step_range(self, a, b) -> "PackedProblem":
        """Steps a .. b-1 of a one-track problem as a one-track problem.  The
        first of them keeps its evolution arrays: ignored when the piece is
        smoothed on its own (a track's first step has no evolution), used when
        it is appended to the steps before it (a resident track extended)."""
        assert self.ntracks == 1 and 0 <= a < b <= self.nsteps
        kw = {f: np.ascontiguousarray(getattr(self, f)[a:b]) for f in
              ("H", "F", "c", "K", "K_type", "G", "o", "C", "C_type", "obs_rows")}
        return PackedProblem(self.n, self.mmax, np.array([0, b - a], dtype=np.int64), **kw)


def split_first_obs(P: PackedProblem):
    """The first-step-observation form of a packed problem
    (kalman_gpu_smooth_oddeven_first_obs): (Pc, F0) where Pc stores every
    step's observation with as many rows as the other steps need (the tracks'
    first steps' slots zero) and F0 holds each track's first observation with
    ld m0max = the largest first-step row count.  Same equations, fewer bytes
    when the first steps carry more rows (a folded square prior)."""
    ts = np.asarray(P.track_start)
    T, n = P.ntracks, P.n
    firsts = ts[:-1][np.diff(ts) > 0]
    rest = np.ones(P.nsteps, dtype=bool)
    rest[firsts] = False
    mc = max(1, int(P.obs_rows[rest].max()) if rest.any() else 1)
    m0 = max(1, int(P.obs_rows[firsts].max()) if len(firsts) else 1)
    mx = P.mmax
    Pc = PackedProblem(n, mc, ts.copy(), P.H, P.F, P.c, P.K, P.K_type,
                       np.ascontiguousarray(P.G.reshape(-1, n, mx)[:, :, :mc]),
                       np.ascontiguousarray(P.o[:, :mc]),
                       np.ascontiguousarray(P.C.reshape(-1, mx, mx)[:, :mc, :mc]),
                       P.C_type.copy(), P.obs_rows.copy())
    # first steps: their packed slots are ignored; keep them zero
    Pc.G[firsts], Pc.o[firsts], Pc.C[firsts], Pc.obs_rows[firsts] = 0.0, 0.0, 0.0, 0
    F0 = {"m0max": m0, "G0": np.zeros((T, n, m0)), "o0": np.zeros((T, m0)), "C0": np.zeros((T, m0, m0)),
          "C0_type": np.full(T, ord("C"), dtype=np.uint8), "obs_rows0": np.zeros(T, dtype=np.int32)}
    for t in range(T):
        if ts[t + 1] > ts[t]:
            s0 = ts[t]
            F0["G0"][t] = P.G[s0][:, :m0]
            F0["o0"][t] = P.o[s0][:m0]
            F0["C0"][t] = P.C[s0][:m0, :m0]
            F0["C0_type"][t] = P.C_type[s0]
            F0["obs_rows0"][t] = P.obs_rows[s0]
    return Pc, F0


def empty_problem(n: int, mmax: int, lengths) -> PackedProblem:
    lengths = np.asarray(lengths, dtype=np.int64)
    ts = np.zeros(len(lengths) + 1, dtype=np.int64)
    ts[1:] = np.cumsum(lengths)
    N = int(ts[-1])
    return PackedProblem(
        n=n, mmax=mmax, track_start=ts,
        H=np.zeros((N, n, n)), F=np.zeros((N, n, n)), c=np.zeros((N, n)),
        K=np.zeros((N, n, n)), K_type=np.full(N, ord("C"), dtype=np.uint8),
        G=np.zeros((N, n, mmax)), o=np.zeros((N, mmax)), C=np.zeros((N, mmax, mmax)),
        C_type=np.full(N, ord("C"), dtype=np.uint8), obs_rows=np.zeros(N, dtype=np.int32),
    )


def _fold_prior(G0, y0, Wobs, x0_mean, prior_w):
    """Square step-0 observation equivalent, in least squares, to the prior
    x0 ~ N(mean, (W0^T W0)^{-1}) plus the first measurement: QR of the weighted
    stack [W0; Wobs G0] with right-hand side [W0 mean; Wobs y0]."""
    A = np.vstack([prior_w, Wobs @ G0])
    b = np.concatenate([prior_w @ x0_mean, Wobs @ y0])
    Q, R = np.linalg.qr(A)
    return R, Q.T @ b


def constant_velocity(lengths, seed=0, K_type="C", C_type="C", missing=0.0, fold=True):
    """3-D constant-velocity tracks: n=6 [pos; vel], dt=0.1, F=[[I, dt I],[0, I]],
    H=I, process noise cov diag(1e-2), observation G=[I 0] (m=3) with noise cov
    diag(1e-1), initial state N(0, I).  With fold=True the prior and the first
    measurement become a square 6x6 step-0 observation with identity 'W'
    weights (the form all three reference smoothers accept).  Every step
    carries its own copy of the matrices, as the reference's evolve/observe
    store them."""
    rng = np.random.default_rng(seed)
    lengths = np.asarray(lengths, dtype=np.int64)
    n, m, dt = 6, 3, 0.1
    F = np.eye(n)
    F[:3, 3:] = dt * np.eye(3)
    G = np.zeros((m, n))
    G[:, :3] = np.eye(3)
    q, r = 1e-2, 1e-1
    P = empty_problem(n, n, lengths)
    N = P.nsteps
    T = len(lengths)
    ts = P.track_start
    firsts = ts[:-1][lengths > 0]
    P.H[:] = np.eye(n)
    P.F[:] = F.T
    allsteps = np.arange(N)
    _set_cov(P.K, P.K_type, allsteps, n, q * np.eye(n), K_type)
    P.G[:, :, :m] = G.T
    _set_cov(P.C, P.C_type, allsteps, m, r * np.eye(m), C_type)
    P.obs_rows[:] = m
    # trajectories and observations, vectorised over tracks
    kmax = int(lengths.max()) if T else 0
    x = rng.standard_normal((T, n))
    Y = np.zeros((N, m))
    for i in range(kmax):
        tr = np.nonzero(lengths > i)[0]
        if i > 0:
            x[tr] = x[tr] @ F.T + np.sqrt(q) * rng.standard_normal((len(tr), n))
        Y[ts[tr] + i] = x[tr] @ G.T + np.sqrt(r) * rng.standard_normal((len(tr), m))
    P.o[:, :m] = Y
    if missing > 0:
        drop = rng.random(N) < missing
        drop[firsts] = False
        P.obs_rows[drop] = 0
    if fold:
        Wobs = np.eye(m) / np.sqrt(r)
        for s in firsts:
            R0, o0 = _fold_prior(G, Y[s], Wobs, np.zeros(n), np.eye(n))
            P.G[s] = 0.0
            P.G[s, :, :n] = R0.T
            P.o[s] = 0.0
            P.o[s, :n] = o0
            P.C[s] = 0.0
            P.C[s, :n, :n] = np.eye(n)
            P.C_type[s] = ord("W")
            P.obs_rows[s] = n
    return P


def _set_cov(arr, types, s, dim, cov, kind):
    """Stores the covariance `cov` (dim x dim) for steps s in the factor form
    `kind` ('C' explicit, 'W' inverse square-root factor, 'w' inverse std
    column, 'F' and 'U' lower Cholesky factor -- the reference weighs both
    kinds with the lower triangle, c/kalman_base.c)."""
    if len(s) == 0:
        return
    if kind == "C":
        arr[s, :dim, :dim] = cov.T
    elif kind in ("F", "U"):
        arr[s, :dim, :dim] = np.linalg.cholesky(cov).T
    elif kind == "W":
        w, V = np.linalg.eigh(cov)
        W = (V / np.sqrt(w)).T  # W^T W = cov^{-1}
        arr[s, :dim, :dim] = W.T
    elif kind == "w":
        d = np.diag(cov)
        flat = np.zeros(arr.shape[1] * arr.shape[2])
        flat[:dim] = 1.0 / np.sqrt(d)
        arr[s] = flat.reshape(arr.shape[1], arr.shape[2])
    else:
        raise ValueError(kind)
    types[s] = ord(kind)


def random_orthogonal(rng, n):
    Q, R = np.linalg.qr(rng.standard_normal((n, n)))
    return Q * np.sign(np.diag(R))


def random_spd(rng, n, lo=0.1, hi=1.0, log=False):
    U = random_orthogonal(rng, n)
    lam = np.exp(rng.uniform(np.log(lo), np.log(hi), n)) if log else rng.uniform(lo, hi, n)
    return (U * lam) @ U.T


def random_dynamics(lengths, n, m, seed=0, rho=0.99, missing=0.0, cov_lo=0.1, cov_hi=1.0, log_cov=False,
                    K_type="C", C_type="C", fold=True, per_step=False):
    """Tracks with F = rho * Q (Q random orthogonal), G i.i.d. N(0, 1/m), process
    and observation noise covariances U diag(lambda) U^T with lambda uniform in
    [cov_lo, cov_hi] (log-uniform if log_cov), H = I, c = 0, a fraction
    `missing` of steps unobserved (never step 0), initial state N(0, I).
    per_step=True draws fresh F, G and covariances at every step (used by the
    parity tests); otherwise each track shares them."""
    rng = np.random.default_rng(seed)
    lengths = np.asarray(lengths, dtype=np.int64)
    P = empty_problem(n, max(n, m), lengths)
    for t, L in enumerate(lengths):
        base = P.track_start[t]
        Fm = rho * random_orthogonal(rng, n)
        Gm = rng.standard_normal((m, n)) / np.sqrt(m)
        Kc = random_spd(rng, n, cov_lo, cov_hi, log_cov)
        Cc = random_spd(rng, m, cov_lo, cov_hi, log_cov)
        x = rng.standard_normal(n)
        for i in range(int(L)):
            s = base + i
            if per_step and i > 0:
                Fm = rho * random_orthogonal(rng, n)
                Gm = rng.standard_normal((m, n)) / np.sqrt(m)
                Kc = random_spd(rng, n, cov_lo, cov_hi, log_cov)
                Cc = random_spd(rng, m, cov_lo, cov_hi, log_cov)
            if i > 0:
                x = Fm @ x + np.linalg.cholesky(Kc) @ rng.standard_normal(n)
                P.H[s] = np.eye(n)
                P.F[s] = Fm.T
                _set_cov(P.K, P.K_type, np.array([s]), n, Kc, K_type)
            y = Gm @ x + np.linalg.cholesky(Cc) @ rng.standard_normal(m)
            if i == 0 and fold:
                Lc = np.linalg.cholesky(Cc)
                Wobs = np.linalg.inv(Lc)
                R0, o0 = _fold_prior(Gm, y, Wobs, np.zeros(n), np.eye(n))
                P.G[s, :, :n] = R0.T
                P.o[s, :n] = o0
                P.C[s, :n, :n] = np.eye(n)
                P.C_type[s] = ord("W")
                P.obs_rows[s] = n
                continue
            if i > 0 and missing > 0 and rng.random() < missing:
                continue
            P.G[s, :, :m] = Gm.T
            P.o[s, :m] = y
            _set_cov(P.C, P.C_type, np.array([s]), m, Cc, C_type)
            P.obs_rows[s] = m
    return P


def batched_lengths(ntracks=4096, lo=100, hi=20000, seed=0):
    """Track lengths floor(exp(U[ln lo, ln hi])), seeded."""
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), ntracks))).astype(np.int64)
