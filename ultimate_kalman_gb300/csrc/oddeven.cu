/*
 * oddeven.cu -- the odd-even (Gargir-Toledo) parallel Kalman smoother on the
 * GPU, FP64.  Restates, as CUDA kernels, c/kalman_oddeven_smoother.c of
 * UltimateKalman 2.1.0:
 *
 *   weigh_kernel     steps_weigh 1620-1659 + kalman_covariance_matrix_weigh
 *                    (c/kalman_base.c:61-175): V H, -V F, V c, W G, W o
 *   pair_kernel      one thread per step pair (j, j+1) of a level:
 *                      stage A  G_F_to_R_tilde 379-457      QR of [G_j; F_{j+1}]
 *                      stage C  H_tilde_G_to_G_tilde 526-560 QR of [H~_{j+1}; G_{j+1}]
 *                      stage B  H_R_tilde_to_R 460-523      QR of [H_j; R~_j]
 *                      renaming Variables_Renaming 563-597 (writes the next level)
 *   tail_kernel      one thread per odd-length track of a level: the single last
 *                    step (stage A on G alone, stage B) and the fix-up that folds
 *                    its leftover rows into the last odd step (smooth_recursive
 *                    1452-1476); or, for a one-step level, the base case
 *                    (smooth_recursive 1360-1423)
 *   solve_kernel     one thread per even step: back-substitution and the
 *                    covariance recurrence (Solve_Estimates 614-975)
 *
 * Every "QR, then apply Q^T" of the reference is a Householder triangularization
 * of the pivot block whose reflectors are then streamed over the other columns
 * one column at a time (LAPACK dlarfg sign convention, so R equals LAPACK's up to
 * rounding).  Each thread keeps its pivot block, reflector scalars and one
 * streamed column in shared memory, interleaved across the threads of the block
 * (element e of thread t at smem[e*blockDim + t]) so that accesses never
 * conflict.  Intermediate blocks travel through global memory in the record and
 * next-level arrays they end up in.
 *
 * Layout in HBM (all FP64, "slot" = a step of a level, every track's slots start
 * at an even slot so pairs never straddle tracks):
 *   level equations  F, H [n*n][S], c [n][S], G [mx*n][S], o [mx][S], m [S]
 *                    -- element-major ("SoA"): consecutive threads read
 *                    consecutive slots, so every load and store is coalesced
 *   records          R, Ft, Y [n*n][E], cr [n][E]: R x_j + Ft x_{j-1} + Y x_{j+1} = cr
 *   off-diagonals    U [n*n][S]: U[q] = cov(x_{q-1}, x_q) of the level
 *   outputs          state [nsteps][n], covariance [nsteps][n*n] (caller's layout)
 * Level l slot q of track t is original step track_start[t] + ((q+1) << l) - 1.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "profiling.h"
#include "ukgpu_internal.h"

namespace {

/* ---------------------------------------------------------------------------
 * per-thread views into interleaved shared memory
 * ------------------------------------------------------------------------ */
struct PV {
  double* p;
  int s;
  __device__ __forceinline__ double& operator[](int i) const { return p[i * s]; }
  __device__ __forceinline__ PV operator+(int off) const { return PV{p + off * s, s}; }
};

/* Householder triangularization of the rows x cols block W (leading dimension
 * ld) using the first npiv columns as pivots; reflector scalars go to tau
 * (tau[k] = 0 for an identity reflector).                                    */
__device__ void householder(PV W, int ld, int rows, int npiv, int cols, PV tau)
{
  const int nref = rows < npiv ? rows : npiv;
  for (int k = 0; k < nref; ++k) {
    PV v = W + k * ld;
    const double alpha = v[k];
    double tail = 0.0;
    for (int i = k + 1; i < rows; ++i) tail = fma(v[i], v[i], tail);
    double t = 0.0;
    if (tail != 0.0) {
      const double beta = -copysign(sqrt(fma(alpha, alpha, tail)), alpha);
      t = (beta - alpha) / beta;
      const double scale = 1.0 / (alpha - beta);
      for (int i = k + 1; i < rows; ++i) v[i] *= scale;
      v[k] = beta;
      for (int j = k + 1; j < cols; ++j) {
        PV a = W + j * ld;
        double d = a[k];
        for (int i = k + 1; i < rows; ++i) d = fma(v[i], a[i], d);
        d *= t;
        a[k] -= d;
        for (int i = k + 1; i < rows; ++i) a[i] = fma(-d, v[i], a[i]);
      }
    }
    tau[k] = t;
  }
  for (int k = nref; k < npiv; ++k) tau[k] = 0.0;
}

/* col <- Q^T col for the reflectors stored in W / tau by householder().      */
__device__ void apply_qt(PV W, int ld, int rows, int npiv, PV tau, PV col)
{
  const int nref = rows < npiv ? rows : npiv;
  for (int k = 0; k < nref; ++k) {
    const double t = tau[k];
    if (t == 0.0) continue;
    PV v = W + k * ld;
    double d = col[k];
    for (int i = k + 1; i < rows; ++i) d = fma(v[i], col[i], d);
    d *= t;
    col[k] -= d;
    for (int i = k + 1; i < rows; ++i) col[i] = fma(-d, v[i], col[i]);
  }
}

/* x <- U^{-1} x, U upper triangular n x n given by an element accessor.       */
template <class UA, class XA>
__device__ bool solve_upper(const UA& U, int n, XA& x)
{
  bool bad = false;
  for (int j = n - 1; j >= 0; --j) {
    const double d = U(j, j);
    bad |= (d == 0.0);
    const double xj = x(j) / d;
    x(j) = xj;
    for (int i = 0; i < j; ++i) x(i) = fma(-xj, U(i, j), x(i));
  }
  return bad;
}

/* element-major (SoA) array: element e of slot s at p[e*stride + s]           */
struct Soa {
  double* p;
  int64_t stride;
  __device__ __forceinline__ double& at(int e, int64_t s) const { return p[(int64_t)e * stride + s]; }
};

struct LevelDev {
  Soa F, H, c, G, o;
  int32_t* m;
  Soa R, Ft, Y, cr;
  Soa U;
  const int64_t* L;      /* [T] steps of each track at this level            */
  const int64_t* slot;   /* [T] first slot                                   */
  const int64_t* pair;   /* [T+1] prefix of floor(L/2) (tracks with L >= 2)  */
  const int64_t* solve;  /* [T+1] prefix of ceil(L/2) (tracks with L >= 2)   */
  const int64_t* tail;   /* tracks with odd L                                */
  int64_t npairs, nsolve, ntail;
};

struct Args {
  LevelDev cur, nxt;
  int n, mx, level, ntracks;
  const int64_t* track_start; /* device copy, [T+1] */
  double* state;
  double* cov;
  int* flag;
};

/* last t with base[t] <= i (base has T+1 nondecreasing entries, i < base[T]) */
__device__ __forceinline__ int find_track(const int64_t* base, int T, int64_t i)
{
  int lo = 0, hi = T; /* invariant: base[lo] <= i < base[hi] */
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (base[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int64_t orig_step(const Args& a, int t, int64_t q)
{
  return a.track_start[t] + ((q + 1) << a.level) - 1;
}

/* ---------------------------------------------------------------------------
 * level 0: weigh the raw equations into the SoA level arrays
 * ------------------------------------------------------------------------ */
struct RawDev {
  const double *H, *F, *c, *K, *G, *o, *C;
  const char *K_type, *C_type;
  const int32_t* obs_rows;
  int mmax;
};

/* Weighs column `col` (rows entries) in place by the covariance factor
 * (cov, type, ld): 'W' cov*col, 'w' diag(cov)*col, 'C' chol(cov)^{-1} col,
 * 'U'/'F' tril(cov)^{-1} col.  L holds the prepared factor for 'C' (rows x rows
 * in shared memory, ld rows).  tmp has `rows` entries.                       */
__device__ void weigh_column(char type, const double* cov, int ldc, int rows, PV L, PV col, PV tmp)
{
  if (type == 'W') {
    for (int i = 0; i < rows; ++i) {
      double s = 0.0;
      for (int j = 0; j < rows; ++j) s = fma(cov[(int64_t)j * ldc + i], col[j], s);
      tmp[i] = s;
    }
    for (int i = 0; i < rows; ++i) col[i] = tmp[i];
  } else if (type == 'w') {
    for (int i = 0; i < rows; ++i) col[i] *= cov[i];
  } else { /* forward substitution with a lower-triangular factor */
    const bool c = (type == 'C');
    for (int j = 0; j < rows; ++j) {
      const double d = c ? L[j * rows + j] : cov[(int64_t)j * ldc + j];
      const double xj = col[j] / d;
      col[j] = xj;
      for (int i = j + 1; i < rows; ++i) col[i] = fma(-xj, c ? L[j * rows + i] : cov[(int64_t)j * ldc + i], col[i]);
    }
  }
}

__device__ __forceinline__ bool valid_type(char c)
{
  return c == 'W' || c == 'w' || c == 'C' || c == 'U' || c == 'F';
}

/* lower Cholesky factor of cov (rows x rows) into L; false if not SPD        */
__device__ bool cholesky(const double* cov, int ldc, int rows, PV L)
{
  for (int j = 0; j < rows; ++j) {
    double d = cov[(int64_t)j * ldc + j];
    for (int k = 0; k < j; ++k) d = fma(-L[k * rows + j], L[k * rows + j], d);
    if (!(d > 0.0)) return false;
    d = sqrt(d);
    L[j * rows + j] = d;
    for (int i = j + 1; i < rows; ++i) {
      double s = cov[(int64_t)j * ldc + i];
      for (int k = 0; k < j; ++k) s = fma(-L[k * rows + i], L[k * rows + j], s);
      L[j * rows + i] = s / d;
    }
  }
  return true;
}

__global__ void weigh_kernel(Args a, RawDev raw, int64_t nsteps)
{
  extern __shared__ double smem[];
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nsteps) return;
  const int n = a.n, mx = a.mx, mm = raw.mmax;
  PV ws{smem + threadIdx.x, (int)blockDim.x};
  PV L = ws, col = ws + mx * mx, tmp = ws + mx * mx + mx;
  const int t = find_track(a.track_start, a.ntracks, g);
  const int64_t i = g - a.track_start[t];
  const int64_t q = a.cur.slot[t] + i;
  const int64_t nn = (int64_t)n * n;
  bool bad = false;
  if (i > 0) {
    const char kt = raw.K_type[g];
    if (!valid_type(kt)) atomicOr(a.flag, 4);
    const double* K = raw.K + g * nn;
    if (kt == 'C') bad |= !cholesky(K, n, n, L);
    for (int part = 0; part <= 2 * n; ++part) { /* n columns of H, n of F, then c */
      const double* src = part < n ? raw.H + g * nn + (int64_t)part * n
                        : part < 2 * n ? raw.F + g * nn + (int64_t)(part - n) * n : raw.c + g * n;
      const double sgn = (part >= n && part < 2 * n) ? -1.0 : 1.0;
      for (int r = 0; r < n; ++r) col[r] = sgn * src[r];
      weigh_column(kt, K, n, n, L, col, tmp);
      for (int r = 0; r < n; ++r) {
        if (part < n) a.cur.H.at(part * n + r, q) = col[r];
        else if (part < 2 * n) a.cur.F.at((part - n) * n + r, q) = col[r];
        else a.cur.c.at(r, q) = col[r];
      }
    }
  }
  int m = raw.obs_rows[g];
  if (m < 0 || m > mm) { /* malformed input: no observation, and report it */
    m = 0;
    atomicOr(a.flag, 4);
  }
  a.cur.m[q] = m;
  if (m > 0) {
    const char ct = raw.C_type[g];
    if (!valid_type(ct)) atomicOr(a.flag, 4);
    const double* C = raw.C + g * (int64_t)mm * mm;
    if (ct == 'C') bad |= !cholesky(C, mm, m, L);
    for (int part = 0; part <= n; ++part) { /* n columns of G, then o */
      const double* src = part < n ? raw.G + g * (int64_t)mm * n + (int64_t)part * mm : raw.o + g * mm;
      for (int r = 0; r < m; ++r) col[r] = src[r];
      weigh_column(ct, C, mm, m, L, col, tmp);
      for (int r = 0; r < m; ++r) {
        if (part < n) a.cur.G.at(part * mx + r, q) = col[r];
        else a.cur.o.at(r, q) = col[r];
      }
    }
  }
  if (bad) atomicOr(a.flag, 1);
}

/* ---------------------------------------------------------------------------
 * forward elimination of one pair of a level
 * ------------------------------------------------------------------------ */
__global__ void pair_kernel(Args a, int rmax)
{
  extern __shared__ double smem[];
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.cur.npairs) return;
  const int n = a.n, mx = a.mx;
  PV ws{smem + threadIdx.x, (int)blockDim.x};
  PV W = ws, tau = ws + rmax * (n + 1), col = tau + n;

  const LevelDev& C = a.cur;
  const LevelDev& N = a.nxt;
  const int t = find_track(C.pair, a.ntracks, item);
  const int64_t p = item - C.pair[t];
  const int64_t sj = C.slot[t] + 2 * p, sj1 = sj + 1;
  const int64_t sn = N.slot[t] + p;
  const int64_t se = C.solve[t] + p;
  const int mj = C.m[sj], mj1 = C.m[sj1];

  /* stage A: pivot [G_j; F_{j+1}], rhs [o_j; c_{j+1}] */
  {
    const int rA = mj + n, ld = rA;
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < mj; ++i) W[q * ld + i] = C.G.at(q * mx + i, sj);
      for (int i = 0; i < n; ++i) W[q * ld + mj + i] = C.F.at(q * n + i, sj1);
    }
    for (int i = 0; i < mj; ++i) W[n * ld + i] = C.o.at(i, sj);
    for (int i = 0; i < n; ++i) W[n * ld + mj + i] = C.c.at(i, sj1);
    householder(W, ld, rA, n, n + 1, tau);
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < n; ++i) C.R.at(q * n + i, se) = (i <= q) ? W[q * ld + i] : 0.0;
    for (int i = 0; i < n; ++i) C.cr.at(i, se) = W[n * ld + i];
    for (int i = 0; i < mj; ++i) N.o.at(i, sn) = W[n * ld + n + i]; /* c'_{j+1} */
    /* stream [0; H_{j+1}]: X_j -> record Y (temporarily), H~_{j+1} -> next G */
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < mj; ++i) col[i] = 0.0;
      for (int i = 0; i < n; ++i) col[mj + i] = C.H.at(q * n + i, sj1);
      apply_qt(W, ld, rA, n, tau, col);
      for (int i = 0; i < n; ++i) C.Y.at(q * n + i, se) = col[i];
      for (int i = 0; i < mj; ++i) N.G.at(q * mx + i, sn) = col[n + i];
    }
  }

  /* stage C: pivot [H~_{j+1}; G_{j+1}], rhs [c'_{j+1}; o_{j+1}] -> next observation */
  {
    const int rC = mj + mj1, ld = rC > 0 ? rC : 1;
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < mj; ++i) W[q * ld + i] = N.G.at(q * mx + i, sn);
      for (int i = 0; i < mj1; ++i) W[q * ld + mj + i] = C.G.at(q * mx + i, sj1);
    }
    for (int i = 0; i < mj; ++i) W[n * ld + i] = N.o.at(i, sn);
    for (int i = 0; i < mj1; ++i) W[n * ld + mj + i] = C.o.at(i, sj1);
    householder(W, ld, rC, n, n + 1, tau);
    const int g = rC < n ? rC : n;
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < g; ++i) N.G.at(q * mx + i, sn) = (i <= q) ? W[q * ld + i] : 0.0;
    for (int i = 0; i < g; ++i) N.o.at(i, sn) = W[n * ld + i];
    N.m[sn] = g;
  }

  /* stage B */
  if (p == 0) {
    for (int e = 0; e < n * n; ++e) C.Ft.at(e, se) = 0.0;
    return;
  }
  {
    const int ld = 2 * n;
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < n; ++i) W[q * ld + i] = C.H.at(q * n + i, sj);
      for (int i = 0; i < n; ++i) W[q * ld + n + i] = C.R.at(q * n + i, se);
    }
    for (int i = 0; i < n; ++i) W[n * ld + i] = C.c.at(i, sj);
    for (int i = 0; i < n; ++i) W[n * ld + n + i] = C.cr.at(i, se);
    householder(W, ld, 2 * n, n, n + 1, tau);
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < n; ++i) C.R.at(q * n + i, se) = (i <= q) ? W[q * ld + i] : 0.0;
    for (int i = 0; i < n; ++i) C.cr.at(i, se) = W[n * ld + i];
    for (int i = 0; i < n; ++i) N.c.at(i, sn) = W[n * ld + n + i];
    /* stream [F_j; 0] -> F~_j (record) and Z_j (next F) */
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < n; ++i) col[i] = C.F.at(q * n + i, sj);
      for (int i = 0; i < n; ++i) col[n + i] = 0.0;
      apply_qt(W, ld, 2 * n, n, tau, col);
      for (int i = 0; i < n; ++i) C.Ft.at(q * n + i, se) = col[i];
      for (int i = 0; i < n; ++i) N.F.at(q * n + i, sn) = col[n + i];
    }
    /* stream [0; X_j] -> Y_j (record) and X~_j (next H) */
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < n; ++i) col[i] = 0.0;
      for (int i = 0; i < n; ++i) col[n + i] = C.Y.at(q * n + i, se);
      apply_qt(W, ld, 2 * n, n, tau, col);
      for (int i = 0; i < n; ++i) C.Y.at(q * n + i, se) = col[i];
      for (int i = 0; i < n; ++i) N.H.at(q * n + i, sn) = col[n + i];
    }
  }
}

/* ---------------------------------------------------------------------------
 * odd-length tracks: single last step + fix-up, or the one-step base case
 * ------------------------------------------------------------------------ */
__global__ void tail_kernel(Args a)
{
  extern __shared__ double smem[];
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.cur.ntail) return;
  const int n = a.n, mx = a.mx;
  const LevelDev& C = a.cur;
  const LevelDev& N = a.nxt;
  PV ws{smem + threadIdx.x, (int)blockDim.x};
  const int t = (int)C.tail[item];
  const int64_t L = C.L[t];
  const int64_t sb = C.slot[t];

  if (L == 1) { /* base case: x = R^{-1} Q^T o, S = R^{-1} R^{-T} */
    const int m0 = C.m[sb];
    const int64_t os = orig_step(a, t, 0);
    double* x = a.state + os * n;
    double* S = a.cov ? a.cov + os * (int64_t)n * n : nullptr;
    if (m0 < n) {
      for (int i = 0; i < n; ++i) x[i] = NAN;
      if (S) for (int e = 0; e < n * n; ++e) S[e] = NAN;
      atomicOr(a.flag, 2);
      return;
    }
    const int ld = m0;
    PV W = ws, tau = ws + mx * (n + 1), Ri = tau + n;
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < m0; ++i) W[q * ld + i] = C.G.at(q * mx + i, sb);
    for (int i = 0; i < m0; ++i) W[n * ld + i] = C.o.at(i, sb);
    householder(W, ld, m0, n, n + 1, tau);
    auto Ru = [&](int i, int j) -> double { return W[j * ld + i]; };
    auto xv = [&](int i) -> double& { return W[n * ld + i]; };
    bool bad = solve_upper(Ru, n, xv);
    for (int i = 0; i < n; ++i) x[i] = W[n * ld + i];
    if (S) {
      for (int q = 0; q < n; ++q) {
        for (int i = 0; i < n; ++i) Ri[q * n + i] = (i == q) ? 1.0 : 0.0;
        auto rc = [&](int i) -> double& { return Ri[q * n + i]; };
        solve_upper(Ru, n, rc);
      }
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double s = 0.0;
          for (int k = (i > j ? i : j); k < n; ++k) s = fma(Ri[k * n + i], Ri[k * n + j], s);
          S[(int64_t)j * n + i] = s;
        }
    }
    if (bad) atomicOr(a.flag, 2);
    return;
  }

  /* single last step s = L-1 of an odd-length level (L >= 3) */
  const int64_t s = sb + L - 1;
  const int64_t es = C.solve[t] + (L - 1) / 2;
  const int64_t sn = N.slot[t] + L / 2 - 1;
  const int ms = C.m[s], mt = ms < n ? ms : n;
  const int ldS = ms > 0 ? ms : 1, ldT = n + mt;
  PV WS = ws, WT = ws + mx * (n + 1), WF = WT + 2 * n * (2 * n + 1), tau = WF + 2 * n * (n + 1);
  /* stage A on [G_s | o_s] */
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < ms; ++i) WS[q * ldS + i] = C.G.at(q * mx + i, s);
  for (int i = 0; i < ms; ++i) WS[n * ldS + i] = C.o.at(i, s);
  householder(WS, ldS, ms, n, n + 1, tau);
  /* stage B on [H_s F_s c_s; R~_s 0 o'_s] */
  for (int q = 0; q < n; ++q) {
    for (int i = 0; i < n; ++i) WT[q * ldT + i] = C.H.at(q * n + i, s);
    for (int i = 0; i < mt; ++i) WT[q * ldT + n + i] = (i <= q) ? WS[q * ldS + i] : 0.0;
    for (int i = 0; i < n; ++i) WT[(n + q) * ldT + i] = C.F.at(q * n + i, s);
    for (int i = 0; i < mt; ++i) WT[(n + q) * ldT + n + i] = 0.0;
  }
  for (int i = 0; i < n; ++i) WT[2 * n * ldT + i] = C.c.at(i, s);
  for (int i = 0; i < mt; ++i) WT[2 * n * ldT + n + i] = WS[n * ldS + i];
  householder(WT, ldT, n + mt, n, 2 * n + 1, tau);
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < n; ++i) {
      C.R.at(q * n + i, es) = (i <= q) ? WT[q * ldT + i] : 0.0;
      C.Ft.at(q * n + i, es) = WT[(n + q) * ldT + i];
      C.Y.at(q * n + i, es) = 0.0;
    }
  for (int i = 0; i < n; ++i) C.cr.at(i, es) = WT[2 * n * ldT + i];
  /* fix-up: QR of [G~_{L-2} o; Z_s o''_s] becomes the next observation */
  const int gp = N.m[sn], rF = gp + mt, ldF = rF > 0 ? rF : 1;
  for (int q = 0; q < n; ++q) {
    for (int i = 0; i < gp; ++i) WF[q * ldF + i] = N.G.at(q * mx + i, sn);
    for (int i = 0; i < mt; ++i) WF[q * ldF + gp + i] = WT[(n + q) * ldT + n + i];
  }
  for (int i = 0; i < gp; ++i) WF[n * ldF + i] = N.o.at(i, sn);
  for (int i = 0; i < mt; ++i) WF[n * ldF + gp + i] = WT[2 * n * ldT + n + i];
  householder(WF, ldF, rF, n, n + 1, tau);
  const int g2 = rF < n ? rF : n;
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < g2; ++i) N.G.at(q * mx + i, sn) = (i <= q) ? WF[q * ldF + i] : 0.0;
  for (int i = 0; i < g2; ++i) N.o.at(i, sn) = WF[n * ldF + i];
  N.m[sn] = g2;
}

/* ---------------------------------------------------------------------------
 * back-substitution and covariance recurrence for the even steps of a level
 *
 * With B = [Ft Y] and Sigma = [[Smm Smp]; [Smp^T Spp]] the joint covariance of
 * the odd neighbours (x_{j-1}, x_{j+1}):
 *   x_j            = R^{-1} (cr - Ft x_{j-1} - Y x_{j+1})
 *   S_j            = R^{-1} (I + B Sigma B^T) R^{-T}
 *   cov(x_j, x_{j-1}) = -R^{-1} (B Sigma)[:, 0:n]
 *   cov(x_j, x_{j+1}) = -R^{-1} (B Sigma)[:, n:2n]
 * (the reference's formulas, Solve_Estimates 703-903, grouped by columns of
 * B Sigma, which are streamed one at a time).
 * ------------------------------------------------------------------------ */
__global__ void solve_kernel(Args a, int want_cov)
{
  extern __shared__ double smem[];
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.cur.nsolve) return;
  const int n = a.n;
  const int64_t nn = (int64_t)n * n;
  const LevelDev& C = a.cur;
  const LevelDev& N = a.nxt;
  const int t = find_track(C.solve, a.ntracks, item);
  const int64_t e = item - C.solve[t];
  const int64_t j = 2 * e, L = C.L[t];
  const bool hp = j > 0, hn = j + 1 < L;
  const int64_t se = item; /* records are indexed by the solve prefix */
  const int64_t oj = orig_step(a, t, j), om = hp ? orig_step(a, t, j - 1) : 0, op = hn ? orig_step(a, t, j + 1) : 0;

  PV ws{smem + threadIdx.x, (int)blockDim.x};
  PV Rs = ws, Fs = ws + n * n, Ys = ws + 2 * n * n, M = ws + 3 * n * n, sg = ws + 4 * n * n, pv = sg + 2 * n;
  for (int k = 0; k < n * n; ++k) {
    Rs[k] = C.R.at(k, se);
    Fs[k] = hp ? C.Ft.at(k, se) : 0.0;
    Ys[k] = hn ? C.Y.at(k, se) : 0.0;
  }
  auto Ru = [&](int i, int jj) -> double { return Rs[jj * n + i]; };

  /* state */
  for (int i = 0; i < n; ++i) pv[i] = C.cr.at(i, se);
  if (hp) {
    const double* xm = a.state + om * n;
    for (int k = 0; k < n; ++k) {
      const double xk = xm[k];
      for (int i = 0; i < n; ++i) pv[i] = fma(-Fs[k * n + i], xk, pv[i]);
    }
  }
  if (hn) {
    const double* xp = a.state + op * n;
    for (int k = 0; k < n; ++k) {
      const double xk = xp[k];
      for (int i = 0; i < n; ++i) pv[i] = fma(-Ys[k * n + i], xk, pv[i]);
    }
  }
  auto pvr = [&](int i) -> double& { return pv[i]; };
  bool bad = solve_upper(Ru, n, pvr);
  double* xo = a.state + oj * n;
  for (int i = 0; i < n; ++i) xo[i] = pv[i];
  if (!want_cov) {
    if (bad) atomicOr(a.flag, 2);
    return;
  }

  const double* Smm = hp ? a.cov + om * nn : nullptr;
  const double* Spp = hn ? a.cov + op * nn : nullptr;
  const int64_t smp = (hp && hn) ? N.slot[t] + (j + 1) / 2 : 0; /* U of the next level */
  for (int k = 0; k < n * n; ++k) M[k] = 0.0;
  const int q0 = hp ? 0 : n, q1 = hn ? 2 * n : n;
  for (int q = q0; q < q1; ++q) {
    /* column q of Sigma */
    if (q < n) {
      for (int i = 0; i < n; ++i) sg[i] = Smm[(int64_t)q * n + i];
      for (int i = 0; i < n; ++i) sg[n + i] = hn ? N.U.at(i * n + q, smp) : 0.0; /* Smp^T[:, q] = Smp[q, :] */
    } else {
      const int qq = q - n;
      for (int i = 0; i < n; ++i) sg[i] = hp ? N.U.at(qq * n + i, smp) : 0.0;
      for (int i = 0; i < n; ++i) sg[n + i] = Spp[(int64_t)qq * n + i];
    }
    /* pv = B sigma */
    for (int i = 0; i < n; ++i) pv[i] = 0.0;
    if (hp)
      for (int k = 0; k < n; ++k) {
        const double sk = sg[k];
        for (int i = 0; i < n; ++i) pv[i] = fma(Fs[k * n + i], sk, pv[i]);
      }
    if (hn)
      for (int k = 0; k < n; ++k) {
        const double sk = sg[n + k];
        for (int i = 0; i < n; ++i) pv[i] = fma(Ys[k * n + i], sk, pv[i]);
      }
    /* M += pv b_q^T, b_q = column q of B */
    PV bq = q < n ? Fs + q * n : Ys + (q - n) * n;
    for (int c = 0; c < n; ++c) {
      const double bc = bq[c];
      for (int i = 0; i < n; ++i) M[c * n + i] = fma(pv[i], bc, M[c * n + i]);
    }
    /* off-diagonal block column: -R^{-1} pv */
    solve_upper(Ru, n, pvr);
    if (a.level == 0) continue; /* level 0's off-diagonal blocks are not needed */
    if (q < n) { /* cov(x_{j-1}, x_j) = cov(x_j, x_{j-1})^T: row q */
      const int64_t sU = C.slot[t] + j;
      for (int i = 0; i < n; ++i) C.U.at(i * n + q, sU) = -pv[i];
    } else {
      const int64_t sU = C.slot[t] + j + 1;
      for (int i = 0; i < n; ++i) C.U.at((q - n) * n + i, sU) = -pv[i];
    }
  }
  for (int i = 0; i < n; ++i) M[i * n + i] += 1.0;
  /* S = R^{-1} M R^{-T}: solve the columns, transpose, solve again, transpose */
  for (int c = 0; c < n; ++c) {
    auto mc = [&](int i) -> double& { return M[c * n + i]; };
    solve_upper(Ru, n, mc);
  }
  for (int c = 0; c < n; ++c)
    for (int i = c + 1; i < n; ++i) {
      const double tmp = M[c * n + i];
      M[c * n + i] = M[i * n + c];
      M[i * n + c] = tmp;
    }
  for (int c = 0; c < n; ++c) {
    auto mc = [&](int i) -> double& { return M[c * n + i]; };
    solve_upper(Ru, n, mc);
  }
  double* So = a.cov + oj * nn;
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < n; ++i) So[(int64_t)c * n + i] = M[i * n + c];
  if (bad) atomicOr(a.flag, 2);
}

/* ---------------------------------------------------------------------------
 * host side: plan, workspace, launches
 * ------------------------------------------------------------------------ */
constexpr int kMaxLevels = 64;

struct LevelPlan {
  int64_t S = 0, E = 0, npairs = 0, nsolve = 0, ntail = 0;
  size_t off_L = 0, off_slot = 0, off_pair = 0, off_solve = 0, off_tail = 0; /* in int64 entries */
};

/* Everything the launches need besides the arrays: per-level track tables
 * (host copy, uploaded into the workspace) and the workspace layout.        */
struct Plan {
  int nlev = 0;
  LevelPlan lp[kMaxLevels];
  size_t tab_entries = 0, off_ts = 0;
  size_t o_tab = 0, o_flag = 0, o_eq[2] = {0, 0}, o_m[2] = {0, 0}, o_rec[kMaxLevels] = {0}, o_U[kMaxLevels] = {0};
  size_t bytes = 0;
  int64_t S0 = 0, S1 = 0;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

/* Builds the plan.  Track t has k_t >> l steps at level l.  When tab is not
 * NULL the tables are written into it (tab_cap entries).  Returns the number
 * of table entries needed, or 0 if the recursion is deeper than kMaxLevels. */
size_t build_plan(const kalman_gpu_problem_t* p, bool want_cov, Plan& P, int64_t* tab, size_t tab_cap)
{
  const int n = p->n, T = p->ntracks;
  const int mx = p->mmax > n ? p->mmax : n;
  const int64_t nn = (int64_t)n * n;
  int64_t kmax = 0;
  for (int t = 0; t < T; ++t) kmax = std::max<int64_t>(kmax, p->track_start[t + 1] - p->track_start[t]);
  P.nlev = 1;
  for (int64_t L = kmax; L > 1; L /= 2) ++P.nlev;
  if (P.nlev > kMaxLevels) return 0;
  size_t pos = 0;
  auto put = [&](int64_t v) {
    if (tab && pos < tab_cap) tab[pos] = v;
    ++pos;
  };
  auto len = [&](int t, int l) { return (p->track_start[t + 1] - p->track_start[t]) >> l; };
  for (int l = 0; l < P.nlev; ++l) {
    LevelPlan& L = P.lp[l];
    L = LevelPlan();
    L.off_L = pos;
    for (int t = 0; t < T; ++t) put(len(t, l));
    L.off_slot = pos;
    int64_t s = 0;
    for (int t = 0; t < T; ++t) { put(s); s += (len(t, l) + 1) & ~int64_t(1); }
    L.S = s;
    L.off_pair = pos;
    int64_t acc = 0;
    for (int t = 0; t < T; ++t) { put(acc); const int64_t k = len(t, l); acc += k >= 2 ? k / 2 : 0; }
    put(acc);
    L.npairs = acc;
    L.off_solve = pos;
    acc = 0;
    for (int t = 0; t < T; ++t) { put(acc); const int64_t k = len(t, l); acc += k >= 2 ? (k + 1) / 2 : 0; }
    put(acc);
    L.nsolve = L.E = acc;
    L.off_tail = pos;
    for (int t = 0; t < T; ++t)
      if (len(t, l) & 1) { put(t); ++L.ntail; }
  }
  P.off_ts = pos;
  for (int t = 0; t <= T; ++t) put(p->track_start[t]);
  P.tab_entries = pos;

  /* workspace layout; level equations ping-pong between two regions sized
     for levels 0 and 1, records and off-diagonal blocks per level           */
  size_t bytes = 0;
  auto take = [&](size_t b) { size_t o = bytes; bytes = align_up(bytes + b, 256); return o; };
  P.o_tab = take(pos * sizeof(int64_t));
  P.o_flag = take(sizeof(int));
  const int64_t eq_doubles_per_slot = 2 * nn + n + (int64_t)mx * n + mx;
  P.S0 = P.lp[0].S;
  P.S1 = P.nlev > 1 ? P.lp[1].S : 0;
  P.o_eq[0] = take((size_t)std::max<int64_t>(P.S0, 1) * eq_doubles_per_slot * sizeof(double));
  P.o_m[0] = take((size_t)std::max<int64_t>(P.S0, 1) * sizeof(int32_t));
  P.o_eq[1] = take((size_t)std::max<int64_t>(P.S1, 1) * eq_doubles_per_slot * sizeof(double));
  P.o_m[1] = take((size_t)std::max<int64_t>(P.S1, 1) * sizeof(int32_t));
  for (int l = 0; l < P.nlev; ++l) {
    P.o_rec[l] = take((size_t)std::max<int64_t>(P.lp[l].E, 1) * (3 * nn + n) * sizeof(double));
    P.o_U[l] = (want_cov && l > 0) ? take((size_t)std::max<int64_t>(P.lp[l].S, 1) * nn * sizeof(double)) : 0;
  }
  P.bytes = bytes;
  return pos;
}

int pick_block(size_t per_thread_bytes, int preferred, int* block)
{
  int dev = 0;
  cudaGetDevice(&dev);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  /* large state dimensions get small blocks (down to one thread): correct,
     though a warp-cooperative kernel would use the SM far better there     */
  int bs = preferred;
  while (bs > 32 && (size_t)bs * per_thread_bytes > (size_t)optin / 2) bs /= 2;
  while (bs > 1 && (size_t)bs * per_thread_bytes > (size_t)optin) bs /= 2;
  if ((size_t)bs * per_thread_bytes > (size_t)optin) return -1;
  *block = bs;
  return 0;
}

/* Uploads the tables, runs every kernel of the smoother on stream st using
 * the device workspace at B (at least P.bytes), waits, reports the flags.   */
int run_plan(uint32_t options, const kalman_gpu_problem_t* p, cudaStream_t st, const Plan& P, const int64_t* tab,
             char* B)
{
  const int n = p->n, T = p->ntracks, nlev = P.nlev;
  const int mx = p->mmax > n ? p->mmax : n;
  const bool want_cov = !(options & KALMAN_NO_COVARIANCE) && p->covariance;
  const int64_t nn = (int64_t)n * n;
  const LevelPlan* lp = P.lp;
  int64_t* dtab = (int64_t*)(B + P.o_tab);
  int* dflag = (int*)(B + P.o_flag);
  cudaMemcpyAsync(dtab, tab, P.tab_entries * sizeof(int64_t), cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(dflag, 0, sizeof(int), st);

  auto level_dev = [&](int l) {
    LevelDev d;
    memset(&d, 0, sizeof(d));
    if (l >= nlev) return d;
    const LevelPlan& L = lp[l];
    const int64_t Sr = (l & 1) ? std::max<int64_t>(P.S1, 1) : std::max<int64_t>(P.S0, 1); /* region stride */
    double* eq = (double*)(B + P.o_eq[l & 1]);
    d.F = Soa{eq, Sr};
    d.H = Soa{eq + nn * Sr, Sr};
    d.c = Soa{eq + 2 * nn * Sr, Sr};
    d.G = Soa{eq + (2 * nn + n) * Sr, Sr};
    d.o = Soa{eq + (2 * nn + n + (int64_t)mx * n) * Sr, Sr};
    d.m = (int32_t*)(B + P.o_m[l & 1]);
    const int64_t E = std::max<int64_t>(L.E, 1);
    double* rec = (double*)(B + P.o_rec[l]);
    d.R = Soa{rec, E};
    d.Ft = Soa{rec + nn * E, E};
    d.Y = Soa{rec + 2 * nn * E, E};
    d.cr = Soa{rec + 3 * nn * E, E};
    d.U = (want_cov && l > 0) ? Soa{(double*)(B + P.o_U[l]), std::max<int64_t>(L.S, 1)} : Soa{nullptr, 0};
    d.L = dtab + L.off_L;
    d.slot = dtab + L.off_slot;
    d.pair = dtab + L.off_pair;
    d.solve = dtab + L.off_solve;
    d.tail = dtab + L.off_tail;
    d.npairs = L.npairs;
    d.nsolve = L.nsolve;
    d.ntail = L.ntail;
    return d;
  };

  Args a;
  memset(&a, 0, sizeof(a));
  a.n = n;
  a.mx = mx;
  a.ntracks = T;
  a.track_start = dtab + P.off_ts;
  a.state = p->state;
  a.cov = want_cov ? p->covariance : nullptr;
  a.flag = dflag;

  /* ---- launch configuration ---- */
  const int rmax = 2 * mx;
  const size_t pt_weigh = (size_t)(mx * mx + 2 * mx) * sizeof(double);
  const size_t pt_pair = (size_t)(rmax * (n + 1) + n + rmax) * sizeof(double);
  const size_t pt_tail = (size_t)(mx * (n + 1) + 2 * n * (2 * n + 1) + 2 * n * (n + 1) + n + nn) * sizeof(double);
  const size_t pt_solve = (size_t)(4 * nn + 3 * n) * sizeof(double);
  int bw, bp, bt, bs;
  if (pick_block(pt_weigh, 128, &bw) || pick_block(pt_pair, 128, &bp) || pick_block(pt_tail, 32, &bt) ||
      pick_block(pt_solve, 64, &bs))
    return ukg_set_error(KALMAN_GPU_EINVAL, "state dimension %d (observation rows %d) needs more shared memory per "
                         "thread than this build's odd-even kernels use", n, mx);
  cudaFuncSetAttribute(weigh_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(bw * pt_weigh));
  cudaFuncSetAttribute(pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(bp * pt_pair));
  cudaFuncSetAttribute(tail_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(bt * pt_tail));
  cudaFuncSetAttribute(solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(bs * pt_solve));

  auto grid = [](int64_t items, int block) { return (unsigned)((items + block - 1) / block); };

  /* ---- level 0: weighing ---- */
  {
    a.level = 0;
    a.cur = level_dev(0);
    RawDev raw{p->H, p->F, p->c, p->K, p->G, p->o, p->C, p->K_type, p->C_type, p->obs_rows, p->mmax};
    UKG_LAUNCH(UKG_K_WEIGH, st, (weigh_kernel<<<grid(p->nsteps, bw), bw, bw * pt_weigh, st>>>(a, raw, p->nsteps)));
  }
  /* ---- forward elimination ---- */
  for (int l = 0; l < nlev; ++l) {
    a.level = l;
    a.cur = level_dev(l);
    a.nxt = level_dev(l + 1);
    if (lp[l].npairs > 0)
      UKG_LAUNCH(UKG_K_PAIR, st, (pair_kernel<<<grid(lp[l].npairs, bp), bp, bp * pt_pair, st>>>(a, rmax)));
    if (lp[l].ntail > 0) UKG_LAUNCH(UKG_K_TAIL, st, (tail_kernel<<<grid(lp[l].ntail, bt), bt, bt * pt_tail, st>>>(a)));
  }
  /* ---- back-substitution ---- */
  for (int l = nlev - 2; l >= 0; --l) {
    a.level = l;
    a.cur = level_dev(l);
    a.nxt = level_dev(l + 1);
    if (lp[l].nsolve > 0)
      UKG_LAUNCH(UKG_K_SOLVE, st,
                 (solve_kernel<<<grid(lp[l].nsolve, bs), bs, bs * pt_solve, st>>>(a, want_cov ? 1 : 0)));
  }
  int hflag = 0;
  cudaMemcpyAsync(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return ukg_set_error(KALMAN_GPU_ECUDA, "odd-even smoother: %s", cudaGetErrorString(e));
  ukg_prof_collect();
  if (hflag & 4) return ukg_set_error(KALMAN_GPU_EINVAL, "malformed input: observation rows outside [0, mmax] or an "
                                     "unknown covariance type");
  if (hflag & 1) return ukg_set_error(KALMAN_GPU_ESINGULAR, "a covariance factor is not positive definite");
  if (hflag & 2) return ukg_set_error(KALMAN_GPU_ESINGULAR, "zero pivot: the smoothing problem is not observable");
  return 0;
}

/* cached device workspace and plan tables of the ordinary entry point */
struct Workspace {
  int device = -1;
  void* dev = nullptr;
  size_t dev_bytes = 0;
};
thread_local Workspace tl_ws; /* one cached device arena per host thread */
thread_local std::vector<int64_t> tl_tab;

int ensure_workspace(size_t bytes, void** out)
{
  int dev = 0;
  cudaGetDevice(&dev);
  Workspace& w = tl_ws;
  if (w.dev && (w.dev_bytes < bytes || w.device != dev)) {
    cudaFree(w.dev);
    w.dev = nullptr;
    w.dev_bytes = 0;
  }
  if (!w.dev) {
    size_t want = bytes + (bytes >> 3);
    cudaError_t e = cudaMalloc(&w.dev, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return ukg_set_error(KALMAN_GPU_ENOMEM, "cudaMalloc of %zu bytes of workspace failed: %s", want,
                           cudaGetErrorString(e));
    }
    w.dev_bytes = want;
    w.device = dev;
  }
  *out = w.dev;
  return 0;
}

}  // namespace

extern "C" void ukg_release_oddeven_workspace(void)
{
  if (tl_ws.dev) cudaFree(tl_ws.dev);
  tl_ws = Workspace();
}

extern "C" int ukg_oddeven_device(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream)
{
  if (p->nsteps == 0) return 0;
  const bool want_cov = !(options & KALMAN_NO_COVARIANCE) && p->covariance;
  Plan P;
  const size_t need = build_plan(p, want_cov, P, nullptr, 0);
  if (need == 0) return ukg_set_error(KALMAN_GPU_EINVAL, "tracks longer than 2^%d steps", kMaxLevels - 1);
  tl_tab.resize(need);
  build_plan(p, want_cov, P, tl_tab.data(), need);
  void* base = nullptr;
  if (int e = ensure_workspace(P.bytes, &base)) return e;
  return run_plan(options, p, (cudaStream_t)cuda_stream, P, tl_tab.data(), (char*)base);
}

/* ---------------------------------------------------------------------------
 * Allocation-free entry point (kalman_gpu_smooth_oddeven_noalloc).
 *
 * For callers that must not allocate device memory once they are running --
 * real-time tracking loops with a no-allocation rule (cudaMalloc and cudaFree
 * can synchronize the device and take unbounded time) and plugins whose host
 * program owns all device memory through its own allocator -- this variant of
 * the odd-even smoother takes its scratch (track tables, flags, level
 * equations, back-substitution records, off-diagonal covariance blocks) from
 * the fixed array below instead of from cudaMalloc.  The caller still owns and
 * passes the input and output arrays.
 *
 * The array is KALMAN_GPU_NOALLOC_SCRATCH_BYTES (64 MiB) on every device that
 * loads the library, for the life of the process.  In host code its name is
 * only a host-side stand-in, so its device address is looked up with
 * cudaGetSymbolAddress, once per device, by the first call made with that
 * device current; that first call should come before any stream capture.
 * Every call shares the array and finds the previous call's contents in it;
 * everything the kernels read is written first in the same call, except the
 * status flag, which is cleared.  Host-side bookkeeping uses a fixed static
 * table and a mutex, and each call waits for its kernels before returning, so
 * calls through this entry point do not overlap; work that did overlap on the
 * GPU with a call would race on the array.
 * ------------------------------------------------------------------------ */
static __device__ __align__(256) unsigned char g_noalloc_scratch[KALMAN_GPU_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr size_t kNoallocTabEntries = size_t(1) << 16; /* host plan tables, int64 entries */
int64_t g_noalloc_tab[kNoallocTabEntries];
std::mutex g_noalloc_mutex;
constexpr int kNoallocDevices = 64;
void* g_noalloc_addr[kNoallocDevices] = {nullptr};
}  // namespace

extern "C" int kalman_gpu_smooth_oddeven_noalloc(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream)
{
  ukg_clear_error();
  if (int e = ukg_validate_problem(p, 0)) return e;
  if (p->location != KALMAN_GPU_DEVICE)
    return ukg_set_error(KALMAN_GPU_EINVAL, "the allocation-free entry point takes device arrays only "
                         "(host arrays would need a device copy)");
  if (p->nsteps == 0) return 0;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    return ukg_set_error(KALMAN_GPU_ENODEV, "no CUDA device: %s", cudaGetErrorString(ce));
  }
  if (dev < 0 || dev >= kNoallocDevices) return ukg_set_error(KALMAN_GPU_EINVAL, "device index %d too large", dev);
  if (!g_noalloc_addr[dev]) { /* set-up, once per device, with that device current */
    void* ptr = nullptr;
    ce = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (ce != cudaSuccess || !ptr) {
      cudaGetLastError();
      return ukg_set_error(KALMAN_GPU_ECUDA, "cudaGetSymbolAddress of the scratch array failed: %s",
                           cudaGetErrorString(ce));
    }
    g_noalloc_addr[dev] = ptr;
  }
  const bool want_cov = !(options & KALMAN_NO_COVARIANCE) && p->covariance;
  Plan P;
  const size_t need = build_plan(p, want_cov, P, nullptr, 0);
  if (need == 0 || need > kNoallocTabEntries)
    return ukg_set_error(KALMAN_GPU_EINVAL, "the allocation-free entry point plans at most %zu table entries "
                         "(this problem needs %zu: too many tracks)", kNoallocTabEntries, need);
  build_plan(p, want_cov, P, g_noalloc_tab, kNoallocTabEntries);
  if (P.bytes > (size_t)KALMAN_GPU_NOALLOC_SCRATCH_BYTES)
    return ukg_set_error(KALMAN_GPU_EINVAL, "this problem needs %zu bytes of scratch; the allocation-free entry "
                         "point has %zu (use kalman_gpu_smooth_oddeven_packed)", P.bytes,
                         (size_t)KALMAN_GPU_NOALLOC_SCRATCH_BYTES);
  const int prof = ukg_prof_pause(); /* profiling would create CUDA events */
  const int status = run_plan(options, p, (cudaStream_t)cuda_stream, P, g_noalloc_tab, (char*)g_noalloc_addr[dev]);
  ukg_prof_resume(prof);
  return status;
}
