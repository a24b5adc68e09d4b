/*
 * oddeven_cta.cuh -- the odd-even smoother for larger state dimensions, one
 * thread block (CTA) per work item.  Included by oddeven.cu (it uses that
 * file's Tables, find_track and orig_step).
 *
 * The per-thread kernels of oddeven.cu give a whole step pair to one thread;
 * past n = 8 a pair's panels (up to 2n x (3n+1) entries) no longer fit one
 * thread's share of shared memory.  Here the CTA's threads share each item:
 * every panel is a row-major matrix in a per-CTA region of global scratch
 * (L1/L2 resident), each Householder reflector is built from a block-wide
 * reduction and applied with one thread per column (consecutive threads touch
 * consecutive addresses), triangular solves run one thread per right-hand
 * side, and the grid is persistent (CTAs loop over the items).  Same algorithm
 * and arithmetic as the per-thread kernels (c/kalman_oddeven_smoother.c):
 *   weigh_cta  steps_weigh 1620-1659 + kalman_covariance_matrix_weigh
 *   pair_cta   stages A (379-457), C (526-560), B (460-523) and renaming
 *   tail_cta   the odd-length fix-up (1452-1476) and the base case (1360-1423)
 *   solve_cta  Solve_Estimates 614-975 (states and the covariance recurrence)
 * Level arrays are slot-major here (all entries of a slot contiguous).  FP64.
 */
#pragma once
#include "cta_linalg.cuh"

namespace ctak {
using namespace ::cta;

template <typename T>
struct EqA {
  Aos<T> F, H, c, G, o;
  int32_t* m;
};
template <typename T>
struct RecA {
  Aos<T> R, Ft, Y, rhs, U;
};

/* T: the arithmetic type of the levels and records (FP64, or FP32 in the
 * precision form); states and covariances are FP64 */
template <typename T>
struct CArgs {
  Tables ct, nt;
  EqA<T> ce, ne;
  RecA<T> cr, nr;
  int n, mx, level, ntracks;
  const int64_t* track_start;
  double* state;   /* x, or the correction d in a refinement sweep */
  double* cov;
  int* flag;
  T* scratch;      /* per CTA: scratch + blockIdx.x * scratch_per_cta */
  int64_t scratch_per_cta;
  Soa<T> baseR;    /* refinement: base-case R per track (p may be null) */
  Soa<T> yrhs;     /* refinement: right-hand side of the even steps (p may be null) */
};

struct RawA {
  const double *H, *F, *c, *K, *G, *o, *C;
  const char *K_type, *C_type;
  const int32_t* obs_rows;
  int mmax;
};

/* ---------------------------------------------------------------------------
 * level 0: weighing.  Per step: panel [H | -F | c] (n x (2n+1)) weighed by K's
 * factor, panel [G | o] (m x (n+1)) by C's; written slot-major to level 0.
 * Scratch: n^2 (L) + n (2n+1) (panel) + rows x NT (the 'W' product).
 * ------------------------------------------------------------------------ */
template <typename T>
struct Narrow {
  __device__ __forceinline__ T operator()(double v) const { return ukg_df::narrow<T>(v); }
};
template <typename T>
struct NegNarrow {
  __device__ __forceinline__ T operator()(double v) const { return -ukg_df::narrow<T>(v); }
};

template <typename T>
__global__ void __launch_bounds__(NT) weigh_cta(CArgs<T> a, RawA raw, int64_t nsteps)
{
  __shared__ T red[33];
  __shared__ Tile<T> tl;
  const int n = a.n, mx = a.mx, mm = raw.mmax, tid = threadIdx.x;
  const int rmax = n > mm ? n : mm;
  T* L = a.scratch + (int64_t)blockIdx.x * a.scratch_per_cta;
  T* B = L + (int64_t)rmax * rmax;
  T* tmp = B + (int64_t)rmax * (2 * n + 1);
  const int64_t nn = (int64_t)n * n;
  for (int64_t g = blockIdx.x; g < nsteps; g += gridDim.x) {
    const int t = find_track(a.track_start, a.ntracks, g);
    const int64_t i = g - a.track_start[t], q = a.ct.slot[t] + i;
    bool bad = false;
    if (i > 0) {
      const int ld = 2 * n + 1;
      cm_to_rm(raw.H + g * nn, n, n, n, B, ld, Narrow<T>(), tl);
      cm_to_rm(raw.F + g * nn, n, n, n, B + n, ld, NegNarrow<T>(), tl);
      for (int r = tid; r < n; r += NT) B[(int64_t)r * ld + 2 * n] = ukg_df::narrow<T>(raw.c[g * n + r]);
      __syncthreads();
      const char kt = raw.K_type[g];
      if (tid == 0 && !valid_cov_type(kt)) atomicOr(a.flag, 4);
      bad |= !weigh_panel(kt, raw.K + g * nn, n, n, B, ld, ld, L, red, tmp);
      rm_to_cm(B, ld, n, n, &a.ce.H.at(0, q), n, tl);
      rm_to_cm(B + n, ld, n, n, &a.ce.F.at(0, q), n, tl);
      for (int r = tid; r < n; r += NT) a.ce.c.at(r, q) = B[(int64_t)r * ld + 2 * n];
      __syncthreads();
    }
    int m = raw.obs_rows[g];
    if (m < 0 || m > mm) {
      m = 0;
      if (tid == 0) atomicOr(a.flag, 4);
    }
    if (tid == 0) a.ce.m[q] = m;
    if (m > 0) {
      const int ld = n + 1;
      cm_to_rm(raw.G + g * (int64_t)mm * n, mm, m, n, B, ld, Narrow<T>(), tl);
      for (int r = tid; r < m; r += NT) B[(int64_t)r * ld + n] = ukg_df::narrow<T>(raw.o[g * mm + r]);
      __syncthreads();
      const char ct = raw.C_type[g];
      if (tid == 0 && !valid_cov_type(ct)) atomicOr(a.flag, 4);
      bad |= !weigh_panel(ct, raw.C + g * (int64_t)mm * mm, mm, m, B, ld, ld, L, red, tmp);
      rm_to_cm(B, ld, m, n, &a.ce.G.at(0, q), mx, tl);
      for (int r = tid; r < m; r += NT) a.ce.o.at(r, q) = B[(int64_t)r * ld + n];
      __syncthreads();
    }
    if (bad && tid == 0) atomicOr(a.flag, 1);
  }
}

/* ---------------------------------------------------------------------------
 * forward elimination of one pair per CTA: stages A, C, B
 * Scratch: the largest panel, 2n x (3n+1).
 * ------------------------------------------------------------------------ */
template <typename T, bool kBlocked>
__global__ void __launch_bounds__(NT, 4) pair_cta(CArgs<T> a)
{
  __shared__ T red[33];
  __shared__ __align__(16) T sh[kBlocked ? kWyShared : 1]; /* the blocked QR's panel */
  const int n = a.n, mx = a.mx, tid = threadIdx.x;
  T* A = a.scratch + (int64_t)blockIdx.x * a.scratch_per_cta;
  const EqA<T>& C = a.ce;
  const EqA<T>& Nx = a.ne;
  const RecA<T>& Rr = a.cr;
  for (int64_t item = blockIdx.x; item < a.ct.npairs; item += gridDim.x) {
    const int t = find_track(a.ct.pair, a.ntracks, item);
    const int64_t p = item - a.ct.pair[t];
    const int64_t sj = a.ct.slot[t] + 2 * p, sj1 = sj + 1;
    const int64_t sn = a.nt.slot[t] + p, se = a.ct.solve[t] + p;
    const int mj = C.m[sj], mj1 = C.m[sj1];

    /* stage A: [G_j | o_j | 0; F_{j+1} | c_{j+1} | H_{j+1}], n pivots */
    {
      const int rows = mj + n, ld = 2 * n + 1;
      for (int e = tid; e < rows * ld; e += NT) {
        const int r = e / ld, c = e - r * ld;
        T v;
        if (r < mj) v = c < n ? C.G.at(c * mx + r, sj) : c == n ? C.o.at(r, sj) : T(0);
        else {
          const int rr = r - mj;
          v = c < n ? C.F.at(c * n + rr, sj1) : c == n ? C.c.at(rr, sj1) : C.H.at((c - n - 1) * n + rr, sj1);
        }
        A[e] = v;
      }
      __syncthreads();
      ::cta::panel_qr<kBlocked>(A, ld, rows, n, ld, red, sh);
      for (int e = tid; e < n * n; e += NT) {
        const int r = e / n, c = e - r * n; /* R~ (r, c), Y~ (r, c) */
        Rr.R.at(c * n + r, se) = r <= c ? A[(int64_t)r * ld + c] : T(0);
        Rr.Y.at(c * n + r, se) = A[(int64_t)r * ld + n + 1 + c];
      }
      for (int r = tid; r < n; r += NT) Rr.rhs.at(r, se) = A[(int64_t)r * ld + n];
      for (int e = tid; e < mj * n; e += NT) { /* H~ and o~: the next level's first observation rows */
        const int r = e / n, c = e - r * n;
        Nx.G.at(c * mx + r, sn) = A[(int64_t)(n + r) * ld + n + 1 + c];
      }
      for (int r = tid; r < mj; r += NT) Nx.o.at(r, sn) = A[(int64_t)(n + r) * ld + n];
      __syncthreads();
    }
    /* stage C: [H~ | o~; G_{j+1} | o_{j+1}] */
    if (mj + mj1 == 0) {
      if (tid == 0) Nx.m[sn] = 0;
    } else {
      const int rows = mj + mj1, ld = n + 1;
      for (int e = tid; e < rows * ld; e += NT) {
        const int r = e / ld, c = e - r * ld;
        A[e] = r < mj ? (c < n ? Nx.G.at(c * mx + r, sn) : Nx.o.at(r, sn))
                      : (c < n ? C.G.at(c * mx + (r - mj), sj1) : C.o.at(r - mj, sj1));
      }
      __syncthreads();
      ::cta::panel_qr<kBlocked>(A, ld, rows, n, ld, red, sh);
      const int g2 = rows < n ? rows : n;
      for (int e = tid; e < g2 * n; e += NT) {
        const int r = e / n, c = e - r * n;
        Nx.G.at(c * mx + r, sn) = r <= c ? A[(int64_t)r * ld + c] : T(0);
      }
      for (int r = tid; r < g2; r += NT) Nx.o.at(r, sn) = A[(int64_t)r * ld + n];
      if (tid == 0) Nx.m[sn] = g2;
      __syncthreads();
    }
    /* stage B: [H_j | F_j | c_j | 0; R~ | 0 | rhs~ | Y~] */
    if (p == 0) {
      for (int e = tid; e < n * n; e += NT) Rr.Ft.at(e, se) = T(0);
      __syncthreads();
      continue;
    }
    {
      const int rows = 2 * n, ld = 3 * n + 1;
      for (int e = tid; e < rows * ld; e += NT) {
        const int r = e / ld, c = e - r * ld;
        T v;
        if (r < n) {
          v = c < n ? C.H.at(c * n + r, sj) : c < 2 * n ? C.F.at((c - n) * n + r, sj) : c == 2 * n ? C.c.at(r, sj) : T(0);
        } else {
          const int rr = r - n;
          v = c < n ? (rr <= c ? Rr.R.at(c * n + rr, se) : T(0))
              : c < 2 * n ? T(0) : c == 2 * n ? Rr.rhs.at(rr, se) : Rr.Y.at((c - 2 * n - 1) * n + rr, se);
        }
        A[e] = v;
      }
      __syncthreads();
      ::cta::panel_qr<kBlocked>(A, ld, rows, n, ld, red, sh);
      for (int e = tid; e < n * n; e += NT) {
        const int r = e / n, c = e - r * n;
        Rr.R.at(c * n + r, se) = r <= c ? A[(int64_t)r * ld + c] : T(0);
        Rr.Ft.at(c * n + r, se) = A[(int64_t)r * ld + n + c];
        Nx.F.at(c * n + r, sn) = A[(int64_t)(n + r) * ld + n + c];
        Rr.Y.at(c * n + r, se) = A[(int64_t)r * ld + 2 * n + 1 + c];
        Nx.H.at(c * n + r, sn) = A[(int64_t)(n + r) * ld + 2 * n + 1 + c];
      }
      for (int r = tid; r < n; r += NT) {
        Rr.rhs.at(r, se) = A[(int64_t)r * ld + 2 * n];
        Nx.c.at(r, sn) = A[(int64_t)(n + r) * ld + 2 * n];
      }
      __syncthreads();
    }
  }
}

/* ---------------------------------------------------------------------------
 * odd-length tracks: the single last step and its fix-up, or the base case.
 * Scratch: the (n+m) x (2n+1) panel, an n x n inverse, an n-vector.
 * ------------------------------------------------------------------------ */
template <typename T, bool kBlocked>
__global__ void __launch_bounds__(NT) tail_cta(CArgs<T> a)
{
  __shared__ T red[33];
  __shared__ __align__(16) T sh[kBlocked ? kWyShared : 1]; /* the blocked QR's panel */
  const int n = a.n, mx = a.mx, tid = threadIdx.x;
  T* A = a.scratch + (int64_t)blockIdx.x * a.scratch_per_cta;
  const EqA<T>& C = a.ce;
  const EqA<T>& Nx = a.ne;
  const RecA<T>& Rr = a.cr;
  for (int64_t item = blockIdx.x; item < a.ct.ntail; item += gridDim.x) {
    const int t = (int)a.ct.tail[item];
    const int64_t L = a.ct.L[t], sb = a.ct.slot[t];
    if (L == 1) { /* base case: x = R^{-1} Q^T o, S = R^{-1} R^{-T} */
      const int m0 = C.m[sb];
      const int64_t os = orig_step(a.track_start, a.level, t, 0);
      double* x = a.state + os * n;
      double* S = a.cov ? a.cov + os * (int64_t)n * n : nullptr;
      if (m0 < n) {
        for (int i = tid; i < n; i += NT) x[i] = NAN;
        if (S)
          for (int e = tid; e < n * n; e += NT) S[e] = NAN;
        if (tid == 0) atomicOr(a.flag, 2);
        __syncthreads();
        continue;
      }
      const int ld = n + 1;
      for (int e = tid; e < m0 * ld; e += NT) {
        const int r = e / ld, c = e - r * ld;
        A[e] = c < n ? C.G.at(c * mx + r, sb) : C.o.at(r, sb);
      }
      __syncthreads();
      ::cta::panel_qr<kBlocked>(A, ld, m0, n, ld, red, sh);
      if (tid == 0)
        for (int i = 0; i < n; ++i)
          if (A[(int64_t)i * ld + i] == T(0)) atomicOr(a.flag, 2);
      if (a.baseR.p) /* the base factor, for the refinement's transpose solve */
        for (int e = tid; e < n * n; e += NT) {
          const int r = e % n, c = e / n;
          a.baseR.at(c * n + r, t) = r <= c ? A[(int64_t)r * ld + c] : T(0);
        }
      T* v = A + (int64_t)m0 * ld; /* the right-hand side, then x */
      for (int i = tid; i < n; i += NT) v[i] = A[(int64_t)i * ld + n];
      __syncthreads();
      solve_upper_vec(A, ld, n, v);
      for (int i = tid; i < n; i += NT) x[i] = ukg_df::widen(v[i]);
      if (S) {
        T* Ri = v + n; /* R^{-1}, row-major n x n */
        for (int e = tid; e < n * n; e += NT) Ri[e] = (e / n == e % n) ? T(1) : T(0);
        __syncthreads();
        solve_upper_cols(A, ld, n, Ri, n, 0, n);
        for (int e = tid; e < n * n; e += NT) { /* S(r, c) = sum_k Ri(r, k) Ri(c, k) */
          const int r = e / n, c = e - r * n;
          T s = T(0);
          for (int k = (r > c ? r : c); k < n; ++k) s = fma(Ri[(int64_t)r * n + k], Ri[(int64_t)c * n + k], s);
          S[(int64_t)c * n + r] = ukg_df::to_f64(s);
        }
      }
      __syncthreads();
      continue;
    }
    /* single last step s = L-1 of an odd-length level */
    const int64_t s = sb + L - 1;
    const int64_t es = a.ct.solve[t] + (L - 1) / 2;
    const int64_t sn = a.nt.slot[t] + L / 2 - 1;
    const int ms = C.m[s], mt = ms < n ? ms : n;
    /* stage A on [G_s | o_s]: its R~ and o' go into the lower rows of the
       stage-B panel, built in the same scratch below it */
    const int ldA = n + 1, ldT = 2 * n + 1, rowsT = n + mt;
    T* WS = A;
    T* WT = A + (int64_t)(ms > 0 ? ms : 1) * ldA;
    if (ms > 0) {
      for (int e = tid; e < ms * ldA; e += NT) {
        const int r = e / ldA, c = e - r * ldA;
        WS[e] = c < n ? C.G.at(c * mx + r, s) : C.o.at(r, s);
      }
      __syncthreads();
      ::cta::panel_qr<kBlocked>(WS, ldA, ms, n, ldA, red, sh);
    }
    for (int e = tid; e < rowsT * ldT; e += NT) {
      const int r = e / ldT, c = e - r * ldT;
      T v;
      if (r < n) v = c < n ? C.H.at(c * n + r, s) : c < 2 * n ? C.F.at((c - n) * n + r, s) : C.c.at(r, s);
      else {
        const int rr = r - n;
        v = c < n ? (rr <= c ? WS[(int64_t)rr * ldA + c] : T(0)) : c < 2 * n ? T(0) : WS[(int64_t)rr * ldA + n];
      }
      WT[e] = v;
    }
    __syncthreads();
    ::cta::panel_qr<kBlocked>(WT, ldT, rowsT, n, ldT, red, sh);
    for (int e = tid; e < n * n; e += NT) {
      const int r = e / n, c = e - r * n;
      Rr.R.at(c * n + r, es) = r <= c ? WT[(int64_t)r * ldT + c] : T(0);
      Rr.Ft.at(c * n + r, es) = WT[(int64_t)r * ldT + n + c];
      Rr.Y.at(c * n + r, es) = T(0);
    }
    for (int r = tid; r < n; r += NT) Rr.rhs.at(r, es) = WT[(int64_t)r * ldT + 2 * n];
    __syncthreads();
    /* fix-up: QR of [G~ o (gp rows of the next level's slot); Z o''] */
    const int gp = Nx.m[sn], rF = gp + mt;
    if (rF == 0) {
      if (tid == 0) Nx.m[sn] = 0;
      __syncthreads();
      continue;
    }
    T* WF = WT + (int64_t)rowsT * ldT;
    const int ldF = n + 1;
    for (int e = tid; e < rF * ldF; e += NT) {
      const int r = e / ldF, c = e - r * ldF;
      WF[e] = r < gp ? (c < n ? Nx.G.at(c * mx + r, sn) : Nx.o.at(r, sn))
                     : (c < n ? WT[(int64_t)(n + r - gp) * ldT + n + c] : WT[(int64_t)(n + r - gp) * ldT + 2 * n]);
    }
    __syncthreads();
    ::cta::panel_qr<kBlocked>(WF, ldF, rF, n, ldF, red, sh);
    const int g2 = rF < n ? rF : n;
    for (int e = tid; e < g2 * n; e += NT) {
      const int r = e / n, c = e - r * n;
      Nx.G.at(c * mx + r, sn) = r <= c ? WF[(int64_t)r * ldF + c] : T(0);
    }
    for (int r = tid; r < g2; r += NT) Nx.o.at(r, sn) = WF[(int64_t)r * ldF + n];
    if (tid == 0) Nx.m[sn] = g2;
    __syncthreads();
  }
}

/* ---------------------------------------------------------------------------
 * back-substitution and covariance recurrence of one even step per CTA:
 *   x_j = R^{-1}(rhs - Ft x_{j-1} - Y x_{j+1})
 *   W = B Sigma (B = [Ft Y], Sigma the joint covariance of x_{j-1}, x_{j+1})
 *   cov(x_j, x_{j-1}) = -R^{-1} W[:, 0:n], cov(x_j, x_{j+1}) = -R^{-1} W[:, n:2n]
 *   S_j = R^{-1} (I + W B^T) R^{-T}
 * Scratch (row-major): R, B (n x 2n), W (n x 2n), M, X (n x n each), x.
 * ------------------------------------------------------------------------ */
constexpr int kSigmaCols = 16; /* columns of Sigma staged in shared memory at a time */

template <typename T>
__global__ void __launch_bounds__(NT) solve_cta(CArgs<T> a, int want_cov)
{
  __shared__ T Sq[kSigmaCols][2 * kMaxCov]; /* Sigma(:, q0 .. q0 + 15), column by column */
  const int n = a.n, tid = threadIdx.x;
  const int64_t nn = (int64_t)n * n;
  T* R = a.scratch + (int64_t)blockIdx.x * a.scratch_per_cta;
  T* Bt = R + nn;       /* B^T = [F~ | Y]^T, 2n x n: Bt[k * n + r] = B(r, k) */
  T* W = Bt + 2 * nn;   /* n x 2n, row-major */
  T* M = W + 2 * nn;    /* n x n */
  T* X = M + nn;        /* n x n */
  T* xv = X + nn;       /* n */
  const RecA<T>& Rr = a.cr;
  for (int64_t item = blockIdx.x; item < a.ct.nsolve; item += gridDim.x) {
    const int t = find_track(a.ct.solve, a.ntracks, item);
    const int64_t j = 2 * (item - a.ct.solve[t]), L = a.ct.L[t];
    const bool hp = j > 0, hn = j + 1 < L;
    const int64_t oj = orig_step(a.track_start, a.level, t, j);
    const int64_t om = hp ? orig_step(a.track_start, a.level, t, j - 1) : 0;
    const int64_t op = hn ? orig_step(a.track_start, a.level, t, j + 1) : 0;
    for (int e = tid; e < n * n; e += NT) { /* records are column-major: contiguous copies */
      const int r = e / n, c = e - r * n;
      R[e] = Rr.R.at(c * n + r, item);
      Bt[e] = hp ? Rr.Ft.at(e, item) : T(0);
      Bt[nn + e] = hn ? Rr.Y.at(e, item) : T(0);
    }
    __syncthreads();
    /* state */
    for (int r = tid; r < n; r += NT) {
      T s = a.yrhs.p ? a.yrhs.at(r, item) : Rr.rhs.at(r, item);
      if (hp)
        for (int k = 0; k < n; ++k) s = fma(-Bt[(int64_t)k * n + r], ukg_df::narrow<T>(a.state[om * n + k]), s);
      if (hn)
        for (int k = 0; k < n; ++k) s = fma(-Bt[nn + (int64_t)k * n + r], ukg_df::narrow<T>(a.state[op * n + k]), s);
      xv[r] = s;
    }
    __syncthreads();
    solve_upper_vec(R, n, n, xv);
    for (int r = tid; r < n; r += NT) a.state[oj * n + r] = ukg_df::widen(xv[r]);
    if (tid == 0)
      for (int i = 0; i < n; ++i)
        if (R[(int64_t)i * n + i] == T(0)) atomicOr(a.flag, 2);
    if (!want_cov) {
      __syncthreads();
      continue;
    }
    /* W = B Sigma over the neighbours' covariance blocks, Sigma staged in
       shared memory kSigmaCols columns at a time (read along its columns),
       outputs one per thread with consecutive threads on consecutive rows */
    const double* Smm = hp ? a.cov + om * nn : nullptr;
    const double* Spp = hn ? a.cov + op * nn : nullptr;
    const int64_t smp = (hp && hn) ? a.nt.slot[t] + (j + 1) / 2 : 0;
    auto sigma = [&](int k, int q) -> T { /* Sigma(k, q), 0 <= k, q < 2n */
      if (k < n) {
        if (q < n) return hp ? T(Smm[(int64_t)q * n + k]) : T(0);
        return (hp && hn) ? a.nr.U.at((q - n) * n + k, smp) : T(0); /* Smp(k, q-n) */
      }
      if (q < n) return (hp && hn) ? a.nr.U.at((k - n) * n + q, smp) : T(0); /* Smp(q, k-n) */
      return hn ? T(Spp[(int64_t)(q - n) * n + (k - n)]) : T(0);
    };
    const int k0 = hp ? 0 : n, k1 = hn ? 2 * n : n, kw = k1 - k0;
    for (int q0 = k0; q0 < k1; q0 += kSigmaCols) {
      const int qn = k1 - q0 < kSigmaCols ? k1 - q0 : kSigmaCols;
      for (int e = tid; e < qn * kw; e += NT) {
        const int qi = e / kw, k = k0 + (e - qi * kw);
        Sq[qi][k] = sigma(k, q0 + qi);
      }
      __syncthreads();
      for (int e = tid; e < qn * n; e += NT) {
        const int qi = e / n, r = e - qi * n;
        T s0 = T(0), s1 = T(0);
        int k = k0;
        for (; k + 1 < k1; k += 2) {
          s0 = fma(Bt[(int64_t)k * n + r], Sq[qi][k], s0);
          s1 = fma(Bt[(int64_t)(k + 1) * n + r], Sq[qi][k + 1], s1);
        }
        if (k < k1) s0 = fma(Bt[(int64_t)k * n + r], Sq[qi][k], s0);
        W[(int64_t)r * 2 * n + q0 + qi] = s0 + s1;
      }
      __syncthreads();
    }
    for (int r = tid; r < n; r += NT)
      for (int q = 0; q < 2 * n; ++q)
        if (q < k0 || q >= k1) W[(int64_t)r * 2 * n + q] = T(0);
    __syncthreads();
    /* M = I + W B^T */
    for (int e = tid; e < n * n; e += NT) {
      const int r = e / n, c = e - r * n;
      T s0 = r == c ? T(1) : T(0), s1 = T(0);
      int q = k0;
      for (; q + 1 < k1; q += 2) {
        s0 = fma(W[(int64_t)r * 2 * n + q], Bt[(int64_t)q * n + c], s0);
        s1 = fma(W[(int64_t)r * 2 * n + q + 1], Bt[(int64_t)(q + 1) * n + c], s1);
      }
      if (q < k1) s0 = fma(W[(int64_t)r * 2 * n + q], Bt[(int64_t)q * n + c], s0);
      M[e] = s0 + s1;
    }
    __syncthreads();
    if (a.level > 0) { /* off-diagonal blocks: -R^{-1} W */
      solve_upper_cols(R, n, n, W, 2 * n, k0, k1);
      for (int e = tid; e < n * 2 * n; e += NT) {
        const int r = e / (2 * n), q = e - r * 2 * n;
        if (q < k0 || q >= k1) continue;
        if (q < n) Rr.U.at(r * n + q, a.ct.slot[t] + j) = -W[e];          /* cov(x_{j-1}, x_j)(q, r) */
        else Rr.U.at((q - n) * n + r, a.ct.slot[t] + j + 1) = -W[e];      /* cov(x_j, x_{j+1})(r, q-n) */
      }
      __syncthreads();
    }
    /* S = R^{-1} M R^{-T}: X = R^{-1} M, then S^T = R^{-1} X^T */
    solve_upper_cols(R, n, n, M, n, 0, n);
    for (int e = tid; e < n * n; e += NT) {
      const int r = e / n, c = e - r * n;
      X[(int64_t)c * n + r] = M[e];
    }
    __syncthreads();
    solve_upper_cols(R, n, n, X, n, 0, n);
    double* So = a.cov + oj * nn;
    for (int e = tid; e < n * n; e += NT) { /* X now holds S^T = S; column-major out */
      const int r = e / n, c = e - r * n;
      So[(int64_t)c * n + r] = ukg_df::to_f64(X[e]);
    }
    __syncthreads();
  }
}

/* ---------------------------------------------------------------------------
 * refinement right-hand side, first part, one step per CTA (FP64, from the
 * raw equations; as residual_kernel): with r = c + F x_{i-1} - H x_i and
 * s = o - G x_i,  wE = K^{-1} r,  zp = H^T wE + G^T C^{-1} s.  Scratch: a
 * factor (rmax^2) and four vectors of rmax.
 * ------------------------------------------------------------------------ */
/* w <- Cov^{-1} w for the covariance factor (cov column-major, ld ldc, rows
 * x rows): 'C' L^{-T} L^{-1} (L = chol), 'U'/'F' the same with L = tril(cov),
 * 'W' W^T W, 'w' diag(cov)^2.  w and tmp are vectors shared by the CTA. */
__device__ void apply_precision_cta(char type, const double* cov, int ldc, int rows, double* L, double* w, double* tmp)
{
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (type == 'w') {
    for (int i = tid; i < rows; i += NT) w[i] *= cov[i] * cov[i];
    __syncthreads();
    return;
  }
  if (type == 'W') {
    for (int i = tid; i < rows; i += NT) {
      double sm = 0.0;
      for (int j = 0; j < rows; ++j) sm = fma(cov[(int64_t)j * ldc + i], w[j], sm);
      tmp[i] = sm;
    }
    __syncthreads();
    for (int j = warp; j < rows; j += NT / 32) { /* w_j = sum_i W(i, j) tmp_i: column j along the lanes */
      double sm = 0.0;
      for (int i = lane; i < rows; i += 32) sm = fma(cov[(int64_t)j * ldc + i], tmp[i], sm);
      for (int off = 16; off > 0; off >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, off);
      if (lane == 0) w[j] = sm;
    }
    __syncthreads();
    return;
  }
  if (type != 'C' && type != 'U' && type != 'F') return;
  for (int j = warp; j < rows; j += NT / 32)
    for (int i = lane; i < rows; i += 32) L[(int64_t)j * rows + i] = i >= j ? cov[(int64_t)j * ldc + i] : 0.0;
  __syncthreads();
  if (type == 'C') cholesky_cm(L, rows); /* the weighing reports a bad factor */
  tri_solve_vec_cm(L, rows, w, true);
  tri_solve_vec_cm(L, rows, w, false);
}

__global__ void __launch_bounds__(NT) residual_cta(CArgs<float> a, RawA raw, Soa<double> wE, Soa<double> zp,
                                                   double* scratch, int64_t per_cta, int64_t nsteps)
{
  const int n = a.n, mm = raw.mmax, tid = threadIdx.x;
  const int rmax = n > mm ? n : mm;
  const int64_t nn = (int64_t)n * n;
  double* L = scratch + (int64_t)blockIdx.x * per_cta;
  double* w = L + (int64_t)rmax * rmax;
  double* tmp = w + rmax;
  double* z = tmp + rmax;
  for (int64_t g = blockIdx.x; g < nsteps; g += gridDim.x) {
    const int t = find_track(a.track_start, a.ntracks, g);
    const int64_t i = g - a.track_start[t], q = a.ct.slot[t] + i;
    const double* x = a.state + g * n;
    for (int c = tid; c < n; c += NT) z[c] = 0.0;
    if (i > 0) {
      const double* xm = x - n;
      const double* H = raw.H + g * nn;
      const double* F = raw.F + g * nn;
      for (int r = tid; r < n; r += NT) {
        double sm = raw.c[g * n + r];
        for (int c = 0; c < n; ++c) sm = fma(F[(int64_t)c * n + r], xm[c], fma(-H[(int64_t)c * n + r], x[c], sm));
        w[r] = sm;
      }
      __syncthreads();
      apply_precision_cta(raw.K_type[g], raw.K + g * nn, n, n, L, w, tmp);
      for (int r = tid; r < n; r += NT) wE.at(r, q) = w[r];
      for (int c = tid >> 5; c < n; c += NT / 32) { /* z = H^T w, column c of H along the lanes */
        double sm = 0.0;
        for (int r = tid & 31; r < n; r += 32) sm = fma(H[(int64_t)c * n + r], w[r], sm);
        for (int off = 16; off > 0; off >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, off);
        if ((tid & 31) == 0) z[c] = sm;
      }
      __syncthreads();
    }
    const int m = a.ce.m[q];
    if (m > 0) {
      const double* G = raw.G + g * (int64_t)mm * n;
      for (int r = tid; r < m; r += NT) {
        double sm = raw.o[g * mm + r];
        for (int c = 0; c < n; ++c) sm = fma(-G[(int64_t)c * mm + r], x[c], sm);
        w[r] = sm;
      }
      __syncthreads();
      apply_precision_cta(raw.C_type[g], raw.C + g * (int64_t)mm * mm, mm, m, L, w, tmp);
      for (int c = tid >> 5; c < n; c += NT / 32) {
        double sm = 0.0;
        for (int r = tid & 31; r < m; r += 32) sm = fma(G[(int64_t)c * mm + r], w[r], sm);
        for (int off = 16; off > 0; off >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, off);
        if ((tid & 31) == 0) z[c] += sm;
      }
      __syncthreads();
    }
    for (int c = tid; c < n; c += NT) zp.at(c, q) = z[c];
    __syncthreads();
  }
}

/* refinement transpose solves over slot-major FP32 records, one warp per
 * item (as rt_even_kernel / rt_odd_kernel), state entries k = lane + 32 q
 * (q < 4: n <= 128) held in registers, record columns read along the lanes:
 *   even steps  y_j = R_j^{-T} z_j
 *   odd steps   z' = z_{2p+1} - Y_{2p}^T y_{2p} - Ft_{2p+2}^T y_{2p+2}      */
constexpr int kRtQ = 4;

static __device__ __forceinline__ float warp_sum(float v)
{
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

__global__ void rt_even_aos(CArgs<float> a, Soa<float> zc, Soa<float> yc)
{
  const int64_t item = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (item >= a.ct.nsolve) return; /* uniform over the warp */
  const int lane = threadIdx.x & 31, n = a.n;
  const int t = find_track(a.ct.solve, a.ntracks, item);
  const int64_t sz = a.ct.slot[t] + 2 * (item - a.ct.solve[t]);
  const float* Rp = &a.cr.R.at(0, item); /* column i of R (entries k < i) at Rp[i * n + k] */
  float yr[kRtQ];
#pragma unroll
  for (int q = 0; q < kRtQ; ++q) yr[q] = 0.f;
  for (int i = 0; i < n; ++i) {
    float d = 0.f;
#pragma unroll
    for (int q = 0; q < kRtQ; ++q) {
      const int k = lane + 32 * q;
      if (k < i) d = fmaf(Rp[(int64_t)i * n + k], yr[q], d);
    }
    d = warp_sum(d);
    const float yi = (zc.at(i, sz) - d) / Rp[(int64_t)i * n + i];
#pragma unroll
    for (int q = 0; q < kRtQ; ++q)
      if (i == lane + 32 * q) yr[q] = yi;
  }
#pragma unroll
  for (int q = 0; q < kRtQ; ++q)
    if (lane + 32 * q < n) yc.at(lane + 32 * q, item) = yr[q];
}

__global__ void rt_odd_aos(CArgs<float> a, Soa<float> zc, Soa<float> yc, Soa<float> zn)
{
  const int64_t item = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (item >= a.ct.npairs) return; /* uniform over the warp */
  const int lane = threadIdx.x & 31, n = a.n;
  const int t = find_track(a.ct.pair, a.ntracks, item);
  const int64_t p = item - a.ct.pair[t], L = a.ct.L[t];
  const int64_t so = a.ct.slot[t] + 2 * p + 1, sn = a.nt.slot[t] + p;
  const int64_t e0 = a.ct.solve[t] + p, e1 = e0 + 1;
  const bool right = 2 * p + 2 <= L - 1;
  const float* Yp = &a.cr.Y.at(0, e0);
  const float* Fp = &a.cr.Ft.at(0, right ? e1 : e0);
  float y0[kRtQ], y1[kRtQ];
#pragma unroll
  for (int q = 0; q < kRtQ; ++q) {
    const int r = lane + 32 * q;
    y0[q] = r < n ? yc.at(r, e0) : 0.f;
    y1[q] = r < n && right ? yc.at(r, e1) : 0.f;
  }
  for (int c = 0; c < n; ++c) {
    float d = 0.f;
#pragma unroll
    for (int q = 0; q < kRtQ; ++q) {
      const int r = lane + 32 * q;
      if (r < n) {
        d = fmaf(Yp[(int64_t)c * n + r], y0[q], d);
        if (right) d = fmaf(Fp[(int64_t)c * n + r], y1[q], d);
      }
    }
    d = warp_sum(d);
    if (lane == 0) zn.at(c, sn) = zc.at(c, so) - d;
  }
}

}  // namespace ctak
