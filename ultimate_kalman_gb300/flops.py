"""FP64 operation counts of the odd-even kernels (oddeven.cu), for rooflines.

The counts mirror the kernels' loops: a fused multiply-add counts 2 flops, a
multiply, add, divide or square root 1.  They are the algorithmic flops of the
Householder formulation the kernels implement -- the same reflectors LAPACK's
dgeqrf/dormqr would apply -- not extra work, so achieved FLOP/s = these counts
divided by measured kernel time.

``plan_flops(track_lengths, obs_rows_level0, n, covariance)`` walks the level
structure of the odd-even recursion (lengths halve, observation rows of odd
steps become min(m_j + m_{j+1}, n)) and returns flops per kernel class.
"""
from __future__ import annotations

import numpy as np


def hh_flops(r, p, w):
    """householder(rows r, pivots p, columns w); r may be an array."""
    r = np.asarray(r, dtype=np.float64)
    tot = np.zeros_like(r)
    for k in range(p):
        t = np.maximum(r - k - 1, 0)
        active = (k < r) & (t > 0)
        per = 2 * t + 5 + t + (w - k - 1) * (4 * t + 2)
        tot += np.where(active, per, 0)
    return tot


def apply_flops(r, p):
    """apply_qt of p reflectors of a block with r rows to one column."""
    r = np.asarray(r, dtype=np.float64)
    tot = np.zeros_like(r)
    for k in range(p):
        t = np.maximum(r - k - 1, 0)
        tot += np.where((k < r) & (t > 0), 4 * t + 2, 0)
    return tot


def pair_flops(n, mj, mj1, first):
    """one item of pair_kernel"""
    mj = np.asarray(mj, dtype=np.float64)
    mj1 = np.asarray(mj1, dtype=np.float64)
    a = hh_flops(mj + n, n, n + 1) + n * apply_flops(mj + n, n)
    c = hh_flops(mj + mj1, n, n + 1)
    b = hh_flops(np.full_like(mj, 2 * n), n, n + 1) + 2 * n * apply_flops(np.full_like(mj, 2 * n), n)
    return a + c + np.where(first, 0, b)


def trsv_flops(n):
    return n + n * (n - 1)  # divides + fused updates


def solve_flops(n, hp, hn, covariance):
    hp = np.asarray(hp, dtype=np.float64)
    hn = np.asarray(hn, dtype=np.float64)
    f = (hp + hn) * 2 * n * n + trsv_flops(n)
    if covariance:
        cols = (hp + hn) * n
        per_col = (hp + hn) * 2 * n * n + 2 * n * n + trsv_flops(n)
        f = f + cols * per_col + n + 2 * n * trsv_flops(n)
    return f


def weigh_flops(n, m, first, cov_type="C"):
    """one item of weigh_kernel with 'C' (Cholesky) covariance factors"""
    m = np.asarray(m, dtype=np.float64)
    chol = lambda d: d ** 3 / 3 + d * d  # noqa: E731
    evol = np.where(first, 0, chol(n) + (2 * n + 1) * trsv_flops(n))
    obs = np.where(m > 0, chol(m) + (n + 1) * (m + m * (m - 1)), 0)
    return evol + obs


def _segments(counts):
    """(segment id, index within segment) for segments of the given sizes"""
    counts = np.asarray(counts, dtype=np.int64)
    seg = np.repeat(np.arange(len(counts)), counts)
    first = np.zeros(len(counts) + 1, dtype=np.int64)
    first[1:] = np.cumsum(counts)
    return seg, np.arange(int(first[-1])) - first[seg], first


def _grouped(fn, *cols):
    """sum of fn over rows, evaluating fn once per distinct row (entries are
    small non-negative integers)"""
    if len(cols[0]) == 0:
        return 0.0
    key = np.zeros(len(cols[0]), dtype=np.int64)
    for c in cols:
        key = key * 65536 + np.asarray(c, dtype=np.int64)
    uniq, counts = np.unique(key, return_counts=True)
    parts = []
    for _ in cols:
        parts.append(uniq % 65536)
        uniq = uniq // 65536
    vals = fn(*parts[::-1])
    return float((np.asarray(vals, dtype=np.float64) * counts).sum())


def plan_flops(track_lengths, obs_rows, track_start, n, covariance=True):
    """Flops per kernel class for one odd-even smoothing of a packed problem,
    vectorised over tracks and pairs level by level."""
    L = np.asarray(track_lengths, dtype=np.int64).copy()
    ts = np.asarray(track_start, dtype=np.int64)
    out = {"weigh_kernel": 0.0, "pair_kernel": 0.0, "tail_kernel": 0.0, "solve_kernel": 0.0}
    firsts = np.zeros(int(ts[-1]), dtype=bool)
    firsts[ts[:-1][L > 0]] = True
    out["weigh_kernel"] = _grouped(lambda a, b: weigh_flops(n, a, b.astype(bool)), obs_rows, firsts)
    m = np.asarray(obs_rows, dtype=np.int64)
    starts = ts[:-1].copy()
    while (L >= 2).any():
        p = np.where(L >= 2, L // 2, 0)
        seg, q, _ = _segments(p)
        base = starts[seg] + 2 * q
        mj, mj1 = m[base], m[base + 1]
        out["pair_kernel"] += _grouped(lambda a, b, c: pair_flops(n, a, b, c.astype(bool)), mj, mj1, q == 0)
        nm = np.minimum(mj + mj1, n)
        # odd lengths: the last pair also folds in the single last step
        odd = (L >= 3) & (L % 2 == 1)
        _, _, first = _segments(p)
        last_pair = first[1:][odd] - 1
        mt = np.minimum(m[starts[odd] + L[odd] - 1], n)
        nm[last_pair] = np.minimum(nm[last_pair] + mt, n)
        e = np.where(L >= 2, (L + 1) // 2, 0)
        seg_e, qe, _ = _segments(e)
        hp = qe > 0
        hn = 2 * qe + 1 < L[seg_e]
        out["solve_kernel"] += _grouped(lambda a, b: solve_flops(n, a, b, covariance), hp, hn)
        newL = L // 2
        new_starts = np.zeros_like(starts)
        new_starts[1:] = np.cumsum(p)[:-1]
        m, L, starts = nm, newL, new_starts
    return out


def plan_flops_fast(track_lengths, n, m0, covariance=True):
    """plan_flops for tracks whose first step has n observation rows and every
    other step m0 (the constant-velocity workload)."""
    lengths = np.asarray(track_lengths, dtype=np.int64)
    ts = np.zeros(len(lengths) + 1, dtype=np.int64)
    ts[1:] = np.cumsum(lengths)
    obs = np.full(int(ts[-1]), m0, dtype=np.int64)
    obs[ts[:-1][lengths > 0]] = n
    return plan_flops(lengths, obs, ts, n, covariance)


def refine_flops(track_lengths, n, m, sweeps=2):
    """One or more refinement sweeps: FP64 residual and A^T r per step (the
    evolution rows of the step and of the next step, its observation rows),
    then R^T y = z and R d = y over the levels in FP32."""
    lengths = np.asarray(track_lengths, dtype=np.int64)
    N = float(lengths.sum())
    per_step = 2.0 * (6 * n * n + 2 * m * n)
    evens = 0.0
    L = lengths.copy()
    while (L >= 2).any():
        evens += float(np.where(L >= 2, (L + 1) // 2, 0).sum())
        L = L // 2
    per_even = 2.0 * (n * n / 2 + 2 * n * n + 2 * n * n + n * n / 2)
    return sweeps * (N * per_step + evens * per_even)


def plan_flops_fast_fp32(track_lengths, n, m0, sweeps=2):
    """Kernel classes of the precision form (states only): FP64 weighing, FP32
    factorization and back-substitution, refinement sweeps."""
    f = plan_flops_fast(track_lengths, n, m0, covariance=False)
    return {"weigh_kernel": f["weigh_kernel"], "fp32_pair_kernel": f["pair_kernel"], "tail_kernel": f["tail_kernel"],
            "fp32_solve_kernel": f["solve_kernel"], "refine_kernel": refine_flops(track_lengths, n, m0, sweeps)}


def compulsory_bytes(track_lengths, n, m, covariance=False):
    """The smoothing problem's compulsory DRAM bytes (FP64): every step's
    equations read once at their real sizes -- F, H, K (n x n), c (n), G
    (m x n), o (m), C (m x m) -- and the smoothed state (n), plus its
    covariance (n x n), written once.  Returns (bytes in, bytes out); for
    n=6, m=3: 1,152 B in and 48 B (states) or 336 B (with covariances) out per
    step.  Everything else a kernel moves (padding of the packed layout,
    weighed equations, level equations, records) is traffic above this."""
    N = float(np.asarray(track_lengths, dtype=np.int64).sum())
    per_in = (3 * n * n + n + m * n + m + m * m) * 8
    per_out = (n + (n * n if covariance else 0)) * 8
    return N * per_in, N * per_out


def plan_bytes_fast(track_lengths, n, m, fp32=False, sweeps=1):
    """Modelled DRAM traffic per kernel category (not the algorithmic bytes:
    those are compulsory_bytes) for one states-only smoothing
    of tracks with n states and m observation rows per step: every input block
    read once, every output and intermediate written once and read once.

    Level 0 (weigh_kernel): the raw FP64 equations K, H, F, c, C, G, o in and
    the weighed level-0 equations out -- FP64 in the plain path, FP32 high
    plus FP32 low parts (8 bytes an entry) in the precision form.  Levels
    l >= 1 carry g_l = min(m 2^l, n) observation rows.  The precision form's
    levels and records are FP32 (4 bytes an entry), the plain path's FP64."""
    lengths = np.asarray(track_lengths, dtype=np.int64)
    N = float(lengths.sum())
    t = 4.0 if fp32 else 8.0

    def eq_rows(g):
        return 2 * n * n + n + g * n + g

    raw = (3 * n * n + n + m * n + m + m * m) * 8 + 2 + 4  # + covariance types, observation rows
    out = {"weigh_kernel": N * (raw + eq_rows(m) * 8 + 4)}
    rec = 3 * n * n + n
    pair = solve = rt = 0.0
    L = lengths.copy()
    level = 0
    while (L >= 2).any():
        pairs = float(np.where(L >= 2, L // 2, 0).sum())
        evens = float(np.where(L >= 2, (L + 1) // 2, 0).sum())
        g, g1 = min(m << level, n), min(m << (level + 1), n)
        pair += pairs * (2 * eq_rows(g) * t + rec * t + eq_rows(g1) * t)
        solve += evens * ((n * (n + 1) // 2 + 2 * n * n + n) * t + 3 * n * 8)
        rt += evens * ((n * (n + 1) // 2 + 2 * n) * 4) + pairs * ((2 * n * n + 4 * n) * 4)
        L = L // 2
        level += 1
    if fp32:
        out["fp32_pair_kernel"] = pair
        out["fp32_solve_kernel"] = solve
        out["refine_residual_kernel"] = sweeps * N * (eq_rows(m) * 8 + n * 8 + n * 4)
        out["refine_rt_kernel"] = sweeps * rt
        out["refine_solve_kernel"] = sweeps * solve
        out["refine_kernel"] = sweeps * N * n * 24
    else:
        out["pair_kernel"] = pair
        out["solve_kernel"] = solve
    return out
