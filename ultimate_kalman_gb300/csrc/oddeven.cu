/*
 * oddeven.cu -- the odd-even (Gargir-Toledo) parallel Kalman smoother on the
 * GPU.  Restates, as CUDA kernels, c/kalman_oddeven_smoother.c of
 * UltimateKalman 2.1.0:
 *
 *   weigh_kernel     steps_weigh 1620-1659 + kalman_covariance_matrix_weigh
 *                    (c/kalman_base.c:61-175): V H, -V F, V c, W G, W o (FP64)
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
 * next-level arrays they end up in.  Divisions are by reciprocals computed once
 * per pivot: FP64 division and square root are multi-instruction sequences on
 * the FP64 pipe, the resource these kernels are bound by.
 *
 * Precision.  The kernels are templates over the arithmetic type T.  FP64 is
 * the plain path.  With KALMAN_GPU_FP32_REFINE the factorization (levels,
 * records) is FP32; the states are then refined with corrected semi-normal
 * equations: the residual r = b - A x of the weighted block-bidiagonal
 * least-squares system and z = A^T r in extended precision, R^T y = z level by
 * level and R d = y with the FP32 R factors, x += d in FP64 -- one or two
 * sweeps.  For the common shapes (n = 4, 6) the level-0 weighing and the
 * residual run in double-float arithmetic on the FP32 pipe (weigh_df_kernel
 * stores the weighed equations as FP32 high + low parts, residual_df_kernel
 * reads them; df64.cuh); other shapes weigh in FP32 and form the residual in
 * FP64 from the raw equations (residual_kernel, atr_kernel).
 *
 * Layout in HBM ("slot" = a step of a level, every track's slots start at an
 * even slot so pairs never straddle tracks):
 *   level equations  F, H [n*n][S], c [n][S], G [mx*n][S], o [mx][S], m [S]
 *                    -- element-major ("SoA"): consecutive threads read
 *                    consecutive slots, so every load and store is coalesced
 *   records          R, Ft, Y [n*n][E], rhs [n][E]: R x_j + Ft x_{j-1} + Y x_{j+1} = rhs
 *   off-diagonals    U [n*n][S]: U[q] = cov(x_{q-1}, x_q) of the level
 *   base factors     baseR [n*n][tracks] (refinement only)
 *   outputs          state [nsteps][n], covariance [nsteps][n*n] (caller's layout)
 * Level l slot q of track t is original step track_start[t] + ((q+1) << l) - 1.
 */
#include <cuda_runtime.h>

#include "df64.cuh"
#include "cta_linalg.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "profiling.h"
#include "ukgpu_internal.h"

namespace {

/* ---------------------------------------------------------------------------
 * per-thread views into interleaved shared memory
 * ------------------------------------------------------------------------ */
template <typename T>
struct PV {
  T* p;
  int s;
  __device__ __forceinline__ T& operator[](int i) const { return p[i * s]; }
  __device__ __forceinline__ PV operator+(int off) const { return PV{p + off * s, s}; }
};

/* The same view with the stride (the block size) known at compile time, so
 * that every shared-memory address is a base plus an immediate offset.       */
template <typename T, int BS>
struct PVc {
  T* p;
  __device__ __forceinline__ T& operator[](int i) const { return p[i * BS]; }
  __device__ __forceinline__ PVc operator+(int off) const { return PVc{p + off * BS}; }
};

template <typename T, int BS>
struct ViewOf {
  using type = PVc<T, BS>;
  static __device__ __forceinline__ type make(T* smem) { return type{smem + threadIdx.x}; }
};
template <typename T>
struct ViewOf<T, 0> {
  using type = PV<T>;
  static __device__ __forceinline__ type make(T* smem) { return type{smem + threadIdx.x, (int)blockDim.x}; }
};

/* Householder triangularization of the rows x cols block W (leading dimension
 * ld) using the first npiv columns as pivots; reflector scalars go to tau
 * (tau[k] = 0 for an identity reflector).  One division per reflector: with
 * inv = 1/(beta (alpha - beta)), 1/(alpha - beta) = beta inv and
 * tau = (beta - alpha)/beta = -(alpha - beta)^2 inv.                        */
template <typename T, class V>
__device__ void householder(V W, int ld, int rows, int npiv, int cols, V tau)
{
  const int nref = rows < npiv ? rows : npiv;
  for (int k = 0; k < nref; ++k) {
    V v = W + k * ld;
    const T alpha = v[k];
    T tail = T(0);
    for (int i = k + 1; i < rows; ++i) tail = fma(v[i], v[i], tail);
    T t = T(0);
    if (tail != T(0)) {
      const T beta = -copysign(sqrt(fma(alpha, alpha, tail)), alpha);
      const T amb = alpha - beta;
      const T inv = T(1) / (beta * amb);
      t = -(amb * amb) * inv;
      const T scale = beta * inv;
      for (int i = k + 1; i < rows; ++i) v[i] *= scale;
      v[k] = beta;
      for (int j = k + 1; j < cols; ++j) {
        V a = W + j * ld;
        T d = a[k];
        for (int i = k + 1; i < rows; ++i) d = fma(v[i], a[i], d);
        d *= t;
        a[k] -= d;
        for (int i = k + 1; i < rows; ++i) a[i] = fma(-d, v[i], a[i]);
      }
    }
    tau[k] = t;
  }
  for (int k = nref; k < npiv; ++k) tau[k] = T(0);
}

/* col <- Q^T col for the reflectors stored in W / tau by householder().      */
template <typename T, class V>
__device__ void apply_qt(V W, int ld, int rows, int npiv, V tau, V col)
{
  const int nref = rows < npiv ? rows : npiv;
  for (int k = 0; k < nref; ++k) {
    const T t = tau[k];
    if (t == T(0)) continue;
    V v = W + k * ld;
    T d = col[k];
    for (int i = k + 1; i < rows; ++i) d = fma(v[i], col[i], d);
    d *= t;
    col[k] -= d;
    for (int i = k + 1; i < rows; ++i) col[i] = fma(-d, v[i], col[i]);
  }
}

/* x <- U^{-1} x for the upper triangle of U (n x n) with precomputed
 * reciprocals dinv of its diagonal.                                          */
template <class UA, class DA, class XA>
__device__ void solve_upper(const UA& U, const DA& dinv, int n, XA& x)
{
  for (int j = n - 1; j >= 0; --j) {
    const auto xj = x(j) * dinv(j);
    x(j) = xj;
    for (int i = 0; i < j; ++i) x(i) = fma(-xj, U(i, j), x(i));
  }
}

/* x <- U^{-T} x (forward substitution with the transpose of the upper U)     */
template <class UA, class DA, class XA>
__device__ void solve_upper_t(const UA& U, const DA& dinv, int n, XA& x)
{
  for (int i = 0; i < n; ++i) {
    auto s = x(i);
    for (int k = 0; k < i; ++k) s = fma(-U(k, i), x(k), s);
    x(i) = s * dinv(i);
  }
}

/* element-major (SoA) array: element e of slot s at p[e*stride + s]           */
template <typename T>
struct Soa {
  T* p;
  int64_t stride;
  __device__ __forceinline__ T& at(int e, int64_t s) const { return p[(int64_t)e * stride + s]; }
};

struct Tables {
  const int64_t* L;      /* [T] steps of each track at this level            */
  const int64_t* slot;   /* [T] first slot                                   */
  const int64_t* pair;   /* [T+1] prefix of floor(L/2) (tracks with L >= 2)  */
  const int64_t* solve;  /* [T+1] prefix of ceil(L/2) (tracks with L >= 2)   */
  const int64_t* tail;   /* tracks with odd L                                */
  int64_t npairs, nsolve, ntail;
};

template <typename T>
struct Eq {
  Soa<T> F, H, c, G, o;
  int32_t* m;
};

template <typename T>
struct Rec {
  Soa<T> R, Ft, Y, rhs, U;
};

template <typename T, typename TI>
struct Args {
  Tables ct, nt;   /* current and next level                                  */
  Eq<TI> ce;       /* equations of the current level                           */
  Eq<T> ne;        /* equations of the next level                              */
  Rec<T> cr, nr;   /* records and off-diagonal blocks, current / next level   */
  int n, mx, level, ntracks;
  const int64_t* track_start; /* device copy, [T+1] */
  double* state;   /* x, or the correction d in a refinement sweep            */
  double* cov;
  int* flag;
  Soa<T> baseR;    /* base-case R per track (refinement), p may be null      */
  Soa<T> yrhs;     /* refinement: right-hand side of the even steps          */
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

__device__ __forceinline__ int64_t orig_step(const int64_t* track_start, int level, int t, int64_t q)
{
  return track_start[t] + ((q + 1) << level) - 1;
}

/* ---------------------------------------------------------------------------
 * level 0: weigh the raw equations into the SoA level arrays (FP64)
 * ------------------------------------------------------------------------ */
struct RawDev {
  const double *H, *F, *c, *K, *G, *o, *C;
  const char *K_type, *C_type;
  const int32_t* obs_rows;
  int mmax;
};

/* Weighs column `col` (rows entries) in place by the covariance factor
 * (cov, type, ld): 'W' cov*col, 'w' diag(cov)*col, 'C' chol(cov)^{-1} col,
 * 'U'/'F' tril(cov)^{-1} col.  L holds the lower factor for 'C' and 'U'/'F'
 * (rows x rows, ld rows) and dinv the reciprocals of its diagonal; tmp has
 * `rows` entries.  Arithmetic in T; the factors are read as FP64.             */
template <typename T>
__device__ void weigh_column(char type, const double* cov, int ldc, int rows, PV<T> L, PV<T> dinv, PV<T> col,
                             PV<T> tmp)
{
  if (type == 'W') {
    for (int i = 0; i < rows; ++i) {
      T s = T(0);
      for (int j = 0; j < rows; ++j) s = fma(ukg_df::narrow<T>(cov[(int64_t)j * ldc + i]), col[j], s);
      tmp[i] = s;
    }
    for (int i = 0; i < rows; ++i) col[i] = tmp[i];
  } else if (type == 'w') {
    for (int i = 0; i < rows; ++i) col[i] *= ukg_df::narrow<T>(cov[i]);
  } else { /* forward substitution with the lower-triangular factor */
    for (int j = 0; j < rows; ++j) {
      const T xj = col[j] * dinv[j];
      col[j] = xj;
      for (int i = j + 1; i < rows; ++i) col[i] = fma(-xj, L[j * rows + i], col[i]);
    }
  }
}

__device__ __forceinline__ bool valid_type(char c)
{
  return c == 'W' || c == 'w' || c == 'C' || c == 'U' || c == 'F';
}

/* the lower factor used by weigh_column: Cholesky of cov for 'C', the lower
 * triangle of cov for 'U'/'F'; false if not positive definite / singular    */
template <typename T>
__device__ bool lower_factor(char type, const double* cov, int ldc, int rows, PV<T> L, PV<T> dinv)
{
  if (type == 'U' || type == 'F') {
    bool ok = true;
    for (int j = 0; j < rows; ++j) {
      for (int i = j; i < rows; ++i) L[j * rows + i] = ukg_df::narrow<T>(cov[(int64_t)j * ldc + i]);
      const T d = L[j * rows + j];
      ok &= (d != T(0));
      dinv[j] = T(1) / d;
    }
    return ok;
  }
  if (type != 'C') return true;
  for (int j = 0; j < rows; ++j) {
    T d = ukg_df::narrow<T>(cov[(int64_t)j * ldc + j]);
    for (int k = 0; k < j; ++k) d = fma(-L[k * rows + j], L[k * rows + j], d);
    if (!(d > T(0))) return false;
    d = sqrt(d);
    const T r = T(1) / d;
    L[j * rows + j] = d;
    dinv[j] = r;
    for (int i = j + 1; i < rows; ++i) {
      T s = ukg_df::narrow<T>(cov[(int64_t)j * ldc + i]);
      for (int k = 0; k < j; ++k) s = fma(-L[k * rows + i], L[k * rows + j], s);
      L[j * rows + i] = s * r;
    }
  }
  return true;
}

template <typename T>
__global__ void weigh_kernel(Args<T, T> a, RawDev raw, int64_t nsteps)
{
  extern __shared__ unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nsteps) return;
  const int n = a.n, mx = a.mx, mm = raw.mmax;
  PV<T> ws{smem + threadIdx.x, (int)blockDim.x};
  PV<T> L = ws, dinv = ws + mx * mx, col = dinv + mx, tmp = col + mx;
  const int t = find_track(a.track_start, a.ntracks, g);
  const int64_t i = g - a.track_start[t];
  const int64_t q = a.ct.slot[t] + i;
  const int64_t nn = (int64_t)n * n;
  bool bad = false;
  if (i > 0) {
    const char kt = raw.K_type[g];
    if (!valid_type(kt)) atomicOr(a.flag, 4);
    const double* K = raw.K + g * nn;
    bad |= !lower_factor(kt, K, n, n, L, dinv);
    for (int part = 0; part <= 2 * n; ++part) { /* n columns of H, n of F, then c */
      const double* src = part < n ? raw.H + g * nn + (int64_t)part * n
                        : part < 2 * n ? raw.F + g * nn + (int64_t)(part - n) * n : raw.c + g * n;
      const T sgn = (part >= n && part < 2 * n) ? T(-1) : T(1);
      for (int r = 0; r < n; ++r) col[r] = sgn * ukg_df::narrow<T>(src[r]);
      weigh_column(kt, K, n, n, L, dinv, col, tmp);
      for (int r = 0; r < n; ++r) {
        if (part < n) a.ce.H.at(part * n + r, q) = col[r];
        else if (part < 2 * n) a.ce.F.at((part - n) * n + r, q) = col[r];
        else a.ce.c.at(r, q) = col[r];
      }
    }
  }
  int m = raw.obs_rows[g];
  if (m < 0 || m > mm) { /* malformed input: no observation, and report it */
    m = 0;
    atomicOr(a.flag, 4);
  }
  a.ce.m[q] = m;
  if (m > 0) {
    const char ct = raw.C_type[g];
    if (!valid_type(ct)) atomicOr(a.flag, 4);
    const double* C = raw.C + g * (int64_t)mm * mm;
    bad |= !lower_factor(ct, C, mm, m, L, dinv);
    for (int part = 0; part <= n; ++part) { /* n columns of G, then o */
      const double* src = part < n ? raw.G + g * (int64_t)mm * n + (int64_t)part * mm : raw.o + g * mm;
      for (int r = 0; r < m; ++r) col[r] = ukg_df::narrow<T>(src[r]);
      weigh_column(ct, C, mm, m, L, dinv, col, tmp);
      for (int r = 0; r < m; ++r) {
        if (part < n) a.ce.G.at(part * mx + r, q) = col[r];
        else a.ce.o.at(r, q) = col[r];
      }
    }
  }
  if (bad) atomicOr(a.flag, 1);
}

/* ---------------------------------------------------------------------------
 * level 0, bulk-staged: the caller's blocks of 128 consecutive steps are
 * contiguous, so each kind of matrix (K, H, F, c, C, G, o) is brought into
 * shared memory by one bulk asynchronous copy (cp.async.bulk, the TMA engine)
 * completing on an mbarrier, then every thread weighs its own step from there.
 * Waits are bounded: a copy that does not complete sets flag bit 8.
 * ------------------------------------------------------------------------ */
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

/* one potentially blocking wait on the phase: the thread may be suspended in
 * hardware until the phase completes or a time limit of the implementation
 * passes, instead of spending issue slots on polls                          */
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity)
{
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

/* waits for the phase with a bound of one second of wall time */
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
{
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try(bar, parity)) return true;
    if (global_ns() - t0 > 1000000000ull) return false;
  }
}

/* the failure path of mbar_wait (kalman_gpu_check_bounded_wait): an mbarrier
 * armed for 16 bytes that no copy delivers never completes its phase; the
 * bounded wait gives up and the block reports flag bit 8, as the weighing
 * kernels do.  No copy is issued, so none is in flight when the block exits. */
__global__ void bounded_wait_check_kernel(int* flag)
{
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&bar)), "r"(16u) : "memory");
    if (!mbar_wait(&bar, 0)) atomicOr(flag, 8);
  }
}

/* prepared weighing of one covariance factor in per-thread shared memory:
 * 'C' Cholesky factor, 'U'/'F' lower triangle (L and reciprocal diagonal),
 * 'W' the matrix itself (in L), 'w' the column (in dinv)                     */
template <typename T, class V>
__device__ bool prepare_weights(char type, const double* cov, int ldc, int rows, V L, V dinv)
{
  if (type == 'W') {
    for (int j = 0; j < rows; ++j)
      for (int i = 0; i < rows; ++i) L[j * rows + i] = ukg_df::narrow<T>(cov[j * ldc + i]);
    return true;
  }
  if (type == 'w') {
    for (int i = 0; i < rows; ++i) dinv[i] = ukg_df::narrow<T>(cov[i]);
    return true;
  }
  if (type == 'U' || type == 'F') {
    bool ok = true;
    for (int j = 0; j < rows; ++j) {
      for (int i = j; i < rows; ++i) L[j * rows + i] = ukg_df::narrow<T>(cov[j * ldc + i]);
      ok &= (L[j * rows + j] != T(0));
      dinv[j] = T(1) / L[j * rows + j];
    }
    return ok;
  }
  for (int j = 0; j < rows; ++j) { /* 'C' */
    T d = ukg_df::narrow<T>(cov[j * ldc + j]);
    for (int k = 0; k < j; ++k) d = fma(-L[k * rows + j], L[k * rows + j], d);
    if (!(d > T(0))) return false;
    d = sqrt(d);
    const T r = T(1) / d;
    L[j * rows + j] = d;
    dinv[j] = r;
    for (int i = j + 1; i < rows; ++i) {
      T sum = ukg_df::narrow<T>(cov[j * ldc + i]);
      for (int k = 0; k < j; ++k) sum = fma(-L[k * rows + i], L[k * rows + j], sum);
      L[j * rows + i] = sum * r;
    }
  }
  return true;
}

template <typename T, class V>
__device__ void apply_weights(char type, int rows, V L, V dinv, V col, V tmp)
{
  if (type == 'W') {
    for (int i = 0; i < rows; ++i) {
      T sum = T(0);
      for (int j = 0; j < rows; ++j) sum = fma(L[j * rows + i], col[j], sum);
      tmp[i] = sum;
    }
    for (int i = 0; i < rows; ++i) col[i] = tmp[i];
  } else if (type == 'w') {
    for (int i = 0; i < rows; ++i) col[i] *= dinv[i];
  } else {
    for (int j = 0; j < rows; ++j) {
      const T xj = col[j] * dinv[j];
      col[j] = xj;
      for (int i = j + 1; i < rows; ++i) col[i] = fma(-xj, L[j * rows + i], col[i]);
    }
  }
}

constexpr int kWeighBS = 128;

template <typename T>
__global__ void __launch_bounds__(kWeighBS) weigh_staged_kernel(Args<T, T> a, RawDev raw, int64_t nsteps, int blk)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  double* buf = reinterpret_cast<double*>(smem_raw + 16);
  T* wsb = reinterpret_cast<T*>(smem_raw + 16 + (size_t)kWeighBS * blk * sizeof(double));
  const int tid = threadIdx.x;
  const int64_t g0 = (int64_t)blockIdx.x * kWeighBS, g = g0 + tid;
  const int cnt = (int)((nsteps - g0) < kWeighBS ? (nsteps - g0) : kWeighBS);
  const bool active = tid < cnt;
  const int n = a.n, mx = a.mx, mm = raw.mmax;
  PVc<T, kWeighBS> ws{wsb + tid};
  PVc<T, kWeighBS> L = ws, dinv = ws + mx * mx, col = dinv + mx, tmp = col + mx;
  if (tid == 0) mbar_init(bar);
  __syncthreads();

  int64_t q = 0, i = 0;
  bool evol = false;
  int m = 0;
  char kt = 'C', ct = 'C';
  if (active) {
    const int t = find_track(a.track_start, a.ntracks, g);
    i = g - a.track_start[t];
    q = a.ct.slot[t] + i;
    evol = i > 0;
    kt = raw.K_type[g];
    m = raw.obs_rows[g];
    if (m < 0 || m > mm) {
      m = 0;
      atomicOr(a.flag, 4);
    }
    ct = raw.C_type[g];
    if (evol && !valid_type(kt)) atomicOr(a.flag, 4);
    if (m > 0 && !valid_type(ct)) atomicOr(a.flag, 4);
    a.ce.m[q] = m;
  }
  bool bad = false;
  uint32_t phase = 0;
  /* parts: 0 K, 1 H, 2 F, 3 c, 4 C, 5 G, 6 o */
  for (int part = 0; part < 7; ++part) {
    const double* src;
    int per;
    switch (part) {
      case 0: src = raw.K; per = n * n; break;
      case 1: src = raw.H; per = n * n; break;
      case 2: src = raw.F; per = n * n; break;
      case 3: src = raw.c; per = n; break;
      case 4: src = raw.C; per = mm * mm; break;
      case 5: src = raw.G; per = mm * n; break;
      default: src = raw.o; per = mm; break;
    }
    if (per == 0) continue;
    const uint32_t bytes = (uint32_t)cnt * per * sizeof(double);
    if (bytes % 16 == 0) { /* one bulk copy; both addresses are 16-byte aligned (g0 is a multiple of 128) */
      if (tid == 0) bulk_load(buf, src + g0 * per, bytes, bar);
      const bool ok = mbar_wait(bar, phase);
      if (!__syncthreads_and(ok)) { /* the same decision in every thread */
        if (tid == 0) atomicOr(a.flag, 8);
        mbar_wait(bar, phase); /* give a late copy one more bounded chance before leaving */
        return;
      }
      phase ^= 1;
    } else {
      for (int e = tid; e < cnt * per; e += kWeighBS) buf[e] = src[g0 * per + e];
      __syncthreads();
    }
    if (active) {
      const double* mine = buf + (size_t)tid * per;
      if (part == 0 && evol) bad |= !prepare_weights<T>(kt, mine, n, n, L, dinv);
      if ((part == 1 || part == 2 || part == 3) && evol) {
        const int ncols = part == 3 ? 1 : n;
        const T sgn = part == 2 ? T(-1) : T(1);
        for (int cc = 0; cc < ncols; ++cc) {
          for (int r = 0; r < n; ++r) col[r] = sgn * ukg_df::narrow<T>(mine[cc * n + r]);
          apply_weights<T>(kt, n, L, dinv, col, tmp);
          for (int r = 0; r < n; ++r) {
            if (part == 1) a.ce.H.at(cc * n + r, q) = col[r];
            else if (part == 2) a.ce.F.at(cc * n + r, q) = col[r];
            else a.ce.c.at(r, q) = col[r];
          }
        }
      }
      if (part == 4 && m > 0) bad |= !prepare_weights<T>(ct, mine, mm, m, L, dinv);
      if ((part == 5 || part == 6) && m > 0) {
        const int ncols = part == 6 ? 1 : n;
        for (int cc = 0; cc < ncols; ++cc) {
          for (int r = 0; r < m; ++r) col[r] = ukg_df::narrow<T>(mine[cc * mm + r]);
          apply_weights<T>(ct, m, L, dinv, col, tmp);
          for (int r = 0; r < m; ++r) {
            if (part == 5) a.ce.G.at(cc * mx + r, q) = col[r];
            else a.ce.o.at(r, q) = col[r];
          }
        }
      }
    }
    __syncthreads(); /* the buffer is refilled by the next part */
  }
  if (bad) atomicOr(a.flag, 1);
}

/* ---------------------------------------------------------------------------
 * Level-0 weighing in double-float arithmetic (FP32 factors with refinement).
 * The same weighing as weigh_kernel, each weighed entry computed to about 47
 * bits and stored as its FP32 high part (the level-0 arrays the FP32
 * factorization reads) and FP32 low part (`lo`, read by the refinement
 * residual).  Parts are staged as in weigh_staged_kernel; the covariance
 * factor of a part lives in registers (compile-time N and MX).
 * ------------------------------------------------------------------------ */
template <int R>
struct DfWeights {
  /* 'W': the matrix W (column-major: (i, j) at v[j * R + i]); 'C', 'U', 'F':
   * the lower factor L below the diagonal and 1/L_jj on it; 'w' (and an
   * unknown type, reported by the caller): the weights on the diagonal */
  ukg_df::df v[R * R];
  int mode; /* 0: W col, 1: diagonal, 2: L^{-1} col */
  int rows;

  /* the weighing for the covariance factor (cov: entry (i, j) at
   * cov[j * ld + i], the first nrows rows and columns): 'W' col <- W col,
   * 'w' col <- diag(cov) col, 'C' col <- chol(cov)^{-1} col, 'U'/'F'
   * col <- tril(cov)^{-1} col.  False: not positive definite or a zero pivot. */
  __device__ __forceinline__ bool prepare(char t, const double* cov, int ld, int nrows)
  {
    using namespace ukg_df;
    rows = nrows;
    mode = t == 'W' ? 0 : (t == 'C' || t == 'U' || t == 'F') ? 2 : 1;
    if (mode == 0) {
#pragma unroll
      for (int j = 0; j < R; ++j)
#pragma unroll
        for (int i = 0; i < R; ++i)
          if (i < rows && j < rows) v[j * R + i] = split(cov[j * ld + i]);
      return true;
    }
    if (mode == 1) {
#pragma unroll
      for (int i = 0; i < R; ++i)
        if (i < rows) v[i * R + i] = t == 'w' ? split(cov[i]) : make(1.0f);
      return true;
    }
    bool ok = true;
#pragma unroll
    for (int j = 0; j < R; ++j) {
      if (j >= rows) break;
#pragma unroll
      for (int i = j; i < R; ++i)
        if (i < rows) v[j * R + i] = split(cov[j * ld + i]);
    }
    if (t == 'C') { /* lower Cholesky factor in place, reciprocal diagonal */
#pragma unroll
      for (int j = 0; j < R; ++j) {
        if (j >= rows) break;
        acc da = start(v[j * R + j]);
#pragma unroll
        for (int k = 0; k < j; ++k) add_prod(da, neg(v[k * R + j]), v[k * R + j]);
        df d = finish(da);
        if (!(d.hi > 0.0f)) {
          ok = false;
          d = make(1.0f);
        }
        const df r = rcp(ukg_df::sqrt(d));
        v[j * R + j] = r;
#pragma unroll
        for (int i = j + 1; i < R; ++i) {
          if (i >= rows) break;
          acc sm = start(v[j * R + i]);
#pragma unroll
          for (int k = 0; k < j; ++k) add_prod(sm, neg(v[k * R + i]), v[k * R + j]);
          v[j * R + i] = mul(finish(sm), r);
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < R; ++j) {
        if (j >= rows) break;
        ok &= v[j * R + j].hi != 0.0f;
        v[j * R + j] = rcp(v[j * R + j]);
      }
    }
    return ok;
  }

  /* col <- V col on the first `rows` entries */
  __device__ __forceinline__ void apply(ukg_df::df (&col)[R]) const
  {
    using namespace ukg_df;
    if (mode == 2) { /* forward substitution, each entry one compensated dot product */
#pragma unroll
      for (int i = 0; i < R; ++i) {
        if (i >= rows) break;
        acc sm = start(col[i]);
#pragma unroll
        for (int j = 0; j < i; ++j) add_prod(sm, neg(v[j * R + i]), col[j]);
        col[i] = mul(finish(sm), v[i * R + i]);
      }
    } else if (mode == 1) {
#pragma unroll
      for (int i = 0; i < R; ++i)
        if (i < rows) col[i] = mul(col[i], v[i * R + i]);
    } else {
      df t[R];
#pragma unroll
      for (int i = 0; i < R; ++i) {
        acc sm = start(make(0.0f));
#pragma unroll
        for (int j = 0; j < R; ++j)
          if (i < rows && j < rows) add_prod(sm, v[j * R + i], col[j]);
        t[i] = finish(sm);
      }
#pragma unroll
      for (int i = 0; i < R; ++i) col[i] = t[i];
    }
  }
};

/* BS: threads (steps) per block, a tuning choice (64, 128 or 256); the
 * register budget per thread is that of four 128-thread blocks per SM.
 * (Staging the next part while weighing this one, in two buffers, was slower:
 * the doubled shared memory halves the resident blocks.)                     */
template <int N, int MX, int BS = kWeighBS>
__global__ void __launch_bounds__(BS, 512 / BS) weigh_df_kernel(Args<float, float> a, Eq<float> lo, RawDev raw,
                                                               int64_t nsteps, int bulk)
{
  using namespace ukg_df;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  double* buf = reinterpret_cast<double*>(smem_raw + 16);
  const int tid = threadIdx.x;
  const int64_t g0 = (int64_t)blockIdx.x * BS, g = g0 + tid;
  const int cnt = (int)((nsteps - g0) < BS ? (nsteps - g0) : BS);
  const bool active = tid < cnt;
  const int mm = raw.mmax;
  if (tid == 0) mbar_init(bar);
  __syncthreads();

  int64_t q = 0, i = 0;
  bool evol = false;
  int m = 0;
  char kt = 'C', ct = 'C';
  if (active) {
    const int t = find_track(a.track_start, a.ntracks, g);
    i = g - a.track_start[t];
    q = a.ct.slot[t] + i;
    evol = i > 0;
    kt = raw.K_type[g];
    m = raw.obs_rows[g];
    if (m < 0 || m > mm) {
      m = 0;
      atomicOr(a.flag, 4);
    }
    ct = raw.C_type[g];
    if (evol && !valid_type(kt)) atomicOr(a.flag, 4);
    if (m > 0 && !valid_type(ct)) atomicOr(a.flag, 4);
    a.ce.m[q] = m;
  }
  bool bad = false;
  uint32_t phase = 0;
  DfWeights<MX> V;
  /* parts: 0 K, 1 H, 2 F, 3 c, 4 C, 5 G, 6 o */
  for (int part = 0; part < 7; ++part) {
    const double* src;
    int per;
    switch (part) {
      case 0: src = raw.K; per = N * N; break;
      case 1: src = raw.H; per = N * N; break;
      case 2: src = raw.F; per = N * N; break;
      case 3: src = raw.c; per = N; break;
      case 4: src = raw.C; per = mm * mm; break;
      case 5: src = raw.G; per = mm * N; break;
      default: src = raw.o; per = mm; break;
    }
    if (per == 0) continue;
    const uint32_t bytes = (uint32_t)cnt * per * sizeof(double);
    if (bulk && bytes % 16 == 0) { /* one bulk copy; both addresses are 16-byte aligned (g0 is a multiple of 64) */
      if (tid == 0) bulk_load(buf, src + g0 * per, bytes, bar);
      const bool ok = mbar_wait(bar, phase);
      if (!__syncthreads_and(ok)) { /* the same decision in every thread */
        if (tid == 0) atomicOr(a.flag, 8);
        mbar_wait(bar, phase); /* give a late copy one more bounded chance before leaving */
        return;
      }
      phase ^= 1;
    } else {
      for (int e = tid; e < cnt * per; e += BS) buf[e] = src[g0 * per + e];
      __syncthreads();
    }
    if (active) {
      const double* mine = buf + (size_t)tid * per;
      const bool evpart = part <= 3;
      const int rows = evpart ? N : m, ld = evpart ? N : mm;
      if ((evpart ? evol : m > 0)) {
        if (part == 0 || part == 4) {
          bad |= !V.prepare(part == 0 ? kt : ct, mine, ld, rows);
        } else {
          const int ncols = (part == 3 || part == 6) ? 1 : N;
          Soa<float> hi, lw;
          int stride; /* element index of (row r, column cc): cc * stride + r */
          switch (part) {
            case 1: hi = a.ce.H, lw = lo.H, stride = N; break;
            case 2: hi = a.ce.F, lw = lo.F, stride = N; break;
            case 3: hi = a.ce.c, lw = lo.c, stride = 0; break;
            case 5: hi = a.ce.G, lw = lo.G, stride = MX; break;
            default: hi = a.ce.o, lw = lo.o, stride = 0; break;
          }
          const bool negate = part == 2;
          /* with an even leading dimension and block size every column starts on
           * 16 bytes: read the staged column two entries at a time (half the
           * shared-memory wavefronts of 8-byte loads at this thread stride).  The
           * second entry of a pair past `rows` still lies in the step's block. */
          const bool pairs = (MX % 2 == 0) && ((ld | per) & 1) == 0;
          for (int cc = 0; cc < ncols; ++cc) {
            df col[MX];
            if (pairs) {
              const double2* m2 = reinterpret_cast<const double2*>(mine + cc * ld);
#pragma unroll
              for (int r = 0; r < MX; r += 2) {
                double2 w = make_double2(0.0, 0.0);
                if (r < rows) w = m2[r / 2];
                col[r] = r < rows ? split(w.x) : make(0.0f);
                if (r + 1 < MX) col[r + 1] = r + 1 < rows ? split(w.y) : make(0.0f);
              }
            } else {
#pragma unroll
              for (int r = 0; r < MX; ++r) {
                col[r] = make(0.0f);
                if (r < rows) col[r] = split(mine[cc * ld + r]);
              }
            }
            if (negate)
#pragma unroll
              for (int r = 0; r < MX; ++r) col[r] = neg(col[r]);
            V.apply(col);
#pragma unroll
            for (int r = 0; r < MX; ++r) {
              if (r >= rows) continue;
              hi.at(cc * stride + r, q) = col[r].hi;
              lw.at(cc * stride + r, q) = col[r].lo;
            }
          }
        }
      }
    }
    __syncthreads(); /* the buffer is refilled by the next part */
  }
  if (bad) atomicOr(a.flag, 1);
}

/* ---------------------------------------------------------------------------
 * forward elimination of one pair of a level
 * ------------------------------------------------------------------------ */
/* NT, MT: compile-time n and mx (0: taken from the arguments); BS: the
 * compile-time block size (0: runtime)                                      */
template <typename T, typename TI, int NT = 0, int MT = 0, int BS = 0>
__global__ void __launch_bounds__(BS ? BS : 1024) pair_kernel(Args<T, TI> a, int rmax_rt)
{
  extern __shared__ unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.ct.npairs) return;
  const int n = NT ? NT : a.n, mx = MT ? MT : a.mx, rmax = MT ? 2 * MT : rmax_rt;
  using View = typename ViewOf<T, BS>::type;
  View ws = ViewOf<T, BS>::make(smem);
  View W = ws, tau = ws + rmax * (n + 1), col = tau + n;

  const Eq<TI>& C = a.ce;
  const Eq<T>& N = a.ne;
  const Rec<T>& Rr = a.cr;
  const int t = find_track(a.ct.pair, a.ntracks, item);
  const int64_t p = item - a.ct.pair[t];
  const int64_t sj = a.ct.slot[t] + 2 * p, sj1 = sj + 1;
  const int64_t sn = a.nt.slot[t] + p;
  const int64_t se = a.ct.solve[t] + p;
  const int mj = C.m[sj], mj1 = C.m[sj1];

  /* stage A: pivot [G_j; F_{j+1}], rhs [o_j; c_{j+1}] */
  {
    const int rA = mj + n, ld = rA;
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < mj; ++i) W[q * ld + i] = (T)C.G.at(q * mx + i, sj);
      for (int i = 0; i < n; ++i) W[q * ld + mj + i] = (T)C.F.at(q * n + i, sj1);
    }
    for (int i = 0; i < mj; ++i) W[n * ld + i] = (T)C.o.at(i, sj);
    for (int i = 0; i < n; ++i) W[n * ld + mj + i] = (T)C.c.at(i, sj1);
    householder<T>(W, ld, rA, n, n + 1, tau);
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < n; ++i) Rr.R.at(q * n + i, se) = (i <= q) ? W[q * ld + i] : T(0);
    for (int i = 0; i < n; ++i) Rr.rhs.at(i, se) = W[n * ld + i];
    for (int i = 0; i < mj; ++i) N.o.at(i, sn) = W[n * ld + n + i]; /* c'_{j+1} */
    /* stream [0; H_{j+1}]: X_j -> record Y (temporarily), H~_{j+1} -> next G */
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < mj; ++i) col[i] = T(0);
      for (int i = 0; i < n; ++i) col[mj + i] = (T)C.H.at(q * n + i, sj1);
      apply_qt<T>(W, ld, rA, n, tau, col);
      for (int i = 0; i < n; ++i) Rr.Y.at(q * n + i, se) = col[i];
      for (int i = 0; i < mj; ++i) N.G.at(q * mx + i, sn) = col[n + i];
    }
  }

  /* stage C: pivot [H~_{j+1}; G_{j+1}], rhs [c'_{j+1}; o_{j+1}] -> next observation */
  {
    const int rC = mj + mj1, ld = rC > 0 ? rC : 1;
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < mj; ++i) W[q * ld + i] = N.G.at(q * mx + i, sn);
      for (int i = 0; i < mj1; ++i) W[q * ld + mj + i] = (T)C.G.at(q * mx + i, sj1);
    }
    for (int i = 0; i < mj; ++i) W[n * ld + i] = N.o.at(i, sn);
    for (int i = 0; i < mj1; ++i) W[n * ld + mj + i] = (T)C.o.at(i, sj1);
    householder<T>(W, ld, rC, n, n + 1, tau);
    const int g = rC < n ? rC : n;
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < g; ++i) N.G.at(q * mx + i, sn) = (i <= q) ? W[q * ld + i] : T(0);
    for (int i = 0; i < g; ++i) N.o.at(i, sn) = W[n * ld + i];
    N.m[sn] = g;
  }

  /* stage B */
  if (p == 0) {
    for (int e = 0; e < n * n; ++e) Rr.Ft.at(e, se) = T(0);
    return;
  }
  {
    const int ld = 2 * n;
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < n; ++i) W[q * ld + i] = (T)C.H.at(q * n + i, sj);
      for (int i = 0; i < n; ++i) W[q * ld + n + i] = Rr.R.at(q * n + i, se);
    }
    for (int i = 0; i < n; ++i) W[n * ld + i] = (T)C.c.at(i, sj);
    for (int i = 0; i < n; ++i) W[n * ld + n + i] = Rr.rhs.at(i, se);
    householder<T>(W, ld, 2 * n, n, n + 1, tau);
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < n; ++i) Rr.R.at(q * n + i, se) = (i <= q) ? W[q * ld + i] : T(0);
    for (int i = 0; i < n; ++i) Rr.rhs.at(i, se) = W[n * ld + i];
    for (int i = 0; i < n; ++i) N.c.at(i, sn) = W[n * ld + n + i];
    /* stream [F_j; 0] -> F~_j (record) and Z_j (next F) */
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < n; ++i) col[i] = (T)C.F.at(q * n + i, sj);
      for (int i = 0; i < n; ++i) col[n + i] = T(0);
      apply_qt<T>(W, ld, 2 * n, n, tau, col);
      for (int i = 0; i < n; ++i) Rr.Ft.at(q * n + i, se) = col[i];
      for (int i = 0; i < n; ++i) N.F.at(q * n + i, sn) = col[n + i];
    }
    /* stream [0; X_j] -> Y_j (record) and X~_j (next H) */
    for (int q = 0; q < n; ++q) {
      for (int i = 0; i < n; ++i) col[i] = T(0);
      for (int i = 0; i < n; ++i) col[n + i] = Rr.Y.at(q * n + i, se);
      apply_qt<T>(W, ld, 2 * n, n, tau, col);
      for (int i = 0; i < n; ++i) Rr.Y.at(q * n + i, se) = col[i];
      for (int i = 0; i < n; ++i) N.H.at(q * n + i, sn) = col[n + i];
    }
  }
}

/* ---------------------------------------------------------------------------
 * Householder QR and reflector application on register arrays, for the FP32
 * pair kernel below: the row counts of stages A (m_j + n) and C (m_j +
 * m_{j+1}) are dispatched at run time to instantiations in which every loop
 * bound is a compile-time constant, so the pivot block P[col][row], the
 * reflector scalars and the streamed column are register arrays.  Same
 * arithmetic as pair_kernel.
 * ------------------------------------------------------------------------ */
template <int R, int C>
__device__ __forceinline__ void hh_reg(float (&P)[C][R], float (&tau)[C])
{
#pragma unroll
  for (int k = 0; k < C; ++k) {
    tau[k] = 0.0f;
    if (k >= R) continue;
    const float alpha = P[k][k];
    float tail = 0.0f;
#pragma unroll
    for (int i = k + 1; i < R; ++i) tail = fmaf(P[k][i], P[k][i], tail);
    if (tail != 0.0f) {
      const float beta = -copysignf(sqrtf(fmaf(alpha, alpha, tail)), alpha);
      const float amb = alpha - beta;
      const float inv = 1.0f / (beta * amb);
      const float t = -(amb * amb) * inv;
      const float scale = beta * inv;
#pragma unroll
      for (int i = k + 1; i < R; ++i) P[k][i] *= scale;
      P[k][k] = beta;
#pragma unroll
      for (int j = k + 1; j < C; ++j) {
        float d = P[j][k];
#pragma unroll
        for (int i = k + 1; i < R; ++i) d = fmaf(P[k][i], P[j][i], d);
        d *= t;
        P[j][k] -= d;
#pragma unroll
        for (int i = k + 1; i < R; ++i) P[j][i] = fmaf(-d, P[k][i], P[j][i]);
      }
      tau[k] = t;
    }
  }
}

template <int R, int C>
__device__ __forceinline__ void apply_reg(const float (&P)[C][R], const float (&tau)[C], float (&col)[R])
{
#pragma unroll
  for (int k = 0; k < C; ++k) {
    if (k >= R) continue;
    const float t = tau[k];
    float d = col[k];
#pragma unroll
    for (int i = k + 1; i < R; ++i) d = fmaf(P[k][i], col[i], d);
    d *= t;
    col[k] -= d;
#pragma unroll
    for (int i = k + 1; i < R; ++i) col[i] = fmaf(-d, P[k][i], col[i]);
  }
}

/* ---------------------------------------------------------------------------
 * FP32 pair elimination with the pair's inputs staged asynchronously.
 * Each thread copies its pair's level equations into its own slice of shared
 * memory with 4-byte cp.async copies in four commit groups (stage A's pivot,
 * the H_{j+1} columns, stage C's rows, stage B's blocks), so every input of
 * the pair is in flight at once and stage A starts when its group lands.  The
 * intermediates (R~, rhs~, Y~, H~, o~) stay in the slice, over inputs already
 * consumed; records and the next level are written once.  Element e of
 * thread t's slice is at smem[e * BP + t] (no bank conflicts).
 * ------------------------------------------------------------------------ */
__device__ __forceinline__ void cp_async4(float* dst, const float* src)
{
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int G>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(G) : "memory"); }

template <int N, int BP>
struct PairSlice {
  static constexpr int NN = N * N, GW = N * N;   /* MX == N */
  static constexpr int Gj = 0, oj = GW, Hj = GW + N, Fj = Hj + NN, cj = Fj + NN;
  static constexpr int G1 = cj + N, o1 = G1 + GW, H1 = o1 + N, F1 = H1 + NN, c1 = F1 + NN;
  static constexpr int width = c1 + N;
  /* intermediates: R~ over G_j, rhs~ over o_j, Y~ over F_{j+1}, H~ over the
   * consumed H_{j+1} columns, o~ over c_{j+1} */
  static constexpr int Rt = Gj, rt = oj, Yt = F1, Ht = H1, ot = c1;
  float* t0;
  __device__ __forceinline__ float& operator[](int e) const { return t0[e * BP]; }
};

/* stage A with RA = m_j + N rows: pivot [G_j; F_{j+1}], rhs [o_j; c_{j+1}] */
template <int N, int BP, int RA>
__device__ __forceinline__ void ss_stage_a(const PairSlice<N, BP>& S)
{
  using L = PairSlice<N, BP>;
  constexpr int MJ = RA - N;
  float P[N][RA], v[RA], tau[N];
  cp_async_wait<3>();
#pragma unroll
  for (int q = 0; q < N; ++q) {
#pragma unroll
    for (int i = 0; i < MJ; ++i) P[q][i] = S[L::Gj + q * N + i];
#pragma unroll
    for (int i = 0; i < N; ++i) P[q][MJ + i] = S[L::F1 + q * N + i];
  }
#pragma unroll
  for (int i = 0; i < MJ; ++i) v[i] = S[L::oj + i];
#pragma unroll
  for (int i = 0; i < N; ++i) v[MJ + i] = S[L::c1 + i];
  hh_reg<RA, N>(P, tau);
  apply_reg<RA, N>(P, tau, v);
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < N; ++i) S[L::Rt + q * N + i] = (i <= q) ? P[q][i] : 0.0f;
#pragma unroll
  for (int i = 0; i < N; ++i) S[L::rt + i] = v[i];
#pragma unroll
  for (int i = 0; i < MJ; ++i) S[L::ot + i] = v[N + i];
  cp_async_wait<2>();
#pragma unroll 1
  for (int q = 0; q < N; ++q) { /* not unrolled: keeps the kernel's code small */
    float col[RA];
#pragma unroll
    for (int i = 0; i < MJ; ++i) col[i] = 0.0f;
#pragma unroll
    for (int i = 0; i < N; ++i) col[MJ + i] = S[L::H1 + q * N + i];
    apply_reg<RA, N>(P, tau, col);
#pragma unroll
    for (int i = 0; i < N; ++i) S[L::Yt + q * N + i] = col[i];
#pragma unroll
    for (int i = 0; i < MJ; ++i) S[L::Ht + q * N + i] = col[N + i];
  }
}

/* stage C with RC = m_j + m_{j+1} rows: pivot [H~_{j+1}; G_{j+1}] */
template <int N, int BP, int RC>
__device__ __forceinline__ void ss_stage_c(const PairSlice<N, BP>& S, const Eq<float>& Nx, int64_t sn, int mj)
{
  using L = PairSlice<N, BP>;
  float P[N][RC], v[RC], tau[N];
  cp_async_wait<1>();
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < RC; ++i) P[q][i] = i < mj ? S[L::Ht + q * N + i] : S[L::G1 + q * N + (i - mj)];
#pragma unroll
  for (int i = 0; i < RC; ++i) v[i] = i < mj ? S[L::ot + i] : S[L::o1 + (i - mj)];
  hh_reg<RC, N>(P, tau);
  apply_reg<RC, N>(P, tau, v);
  constexpr int G = RC < N ? RC : N;
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < G; ++i) Nx.G.at(q * N + i, sn) = (i <= q) ? P[q][i] : 0.0f;
#pragma unroll
  for (int i = 0; i < G; ++i) Nx.o.at(i, sn) = v[i];
  Nx.m[sn] = G;
}

/* stage B: pivot [H_j; R~_j] (2N rows) */
template <int N, int BP>
__device__ __forceinline__ void ss_stage_b(const PairSlice<N, BP>& S, const Eq<float>& Nx, const Rec<float>& Rr,
                                           int64_t sn, int64_t se)
{
  using L = PairSlice<N, BP>;
  constexpr int R2 = 2 * N;
  float P[N][R2], v[R2], tau[N];
  cp_async_wait<0>();
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < N; ++i) {
      P[q][i] = S[L::Hj + q * N + i];
      P[q][N + i] = S[L::Rt + q * N + i];
    }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    v[i] = S[L::cj + i];
    v[N + i] = S[L::rt + i];
  }
  hh_reg<R2, N>(P, tau);
  apply_reg<R2, N>(P, tau, v);
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < N; ++i) Rr.R.at(q * N + i, se) = (i <= q) ? P[q][i] : 0.0f;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    Rr.rhs.at(i, se) = v[i];
    Nx.c.at(i, sn) = v[N + i];
  }
#pragma unroll 1
  for (int q = 0; q < N; ++q) {
    float col[R2];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      col[i] = S[L::Fj + q * N + i];
      col[N + i] = 0.0f;
    }
    apply_reg<R2, N>(P, tau, col);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Rr.Ft.at(q * N + i, se) = col[i];
      Nx.F.at(q * N + i, sn) = col[N + i];
    }
  }
#pragma unroll 1
  for (int q = 0; q < N; ++q) {
    float col[R2];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      col[i] = 0.0f;
      col[N + i] = S[L::Yt + q * N + i];
    }
    apply_reg<R2, N>(P, tau, col);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Rr.Y.at(q * N + i, se) = col[i];
      Nx.H.at(q * N + i, sn) = col[N + i];
    }
  }
}

template <int N, int BP, int RA = N>
__device__ __forceinline__ void ss_dispatch_a(int ra, const PairSlice<N, BP>& S)
{
  if constexpr (RA <= 2 * N) {
    if (ra == RA) ss_stage_a<N, BP, RA>(S);
    else ss_dispatch_a<N, BP, RA + 1>(ra, S);
  }
}

template <int N, int BP, int RC = 1>
__device__ __forceinline__ void ss_dispatch_c(int rc, const PairSlice<N, BP>& S, const Eq<float>& Nx, int64_t sn,
                                              int mj)
{
  if constexpr (RC <= 2 * N) {
    if (rc == RC) ss_stage_c<N, BP, RC>(S, Nx, sn, mj);
    else ss_dispatch_c<N, BP, RC + 1>(rc, S, Nx, sn, mj);
  }
}

constexpr int kPairSsBP = 64; /* default block size; 32 and 128 are tuning choices */

template <int N, int BP = kPairSsBP>
__global__ void __launch_bounds__(BP) pair_ss_kernel(Args<float, float> a, int)
{
  using L = PairSlice<N, BP>;
  extern __shared__ __align__(16) float ss_smem[];
  const int64_t item = (int64_t)blockIdx.x * BP + threadIdx.x;
  if (item >= a.ct.npairs) return;
  const int t = find_track(a.ct.pair, a.ntracks, item);
  const int64_t p = item - a.ct.pair[t];
  const int64_t sj = a.ct.slot[t] + 2 * p, sj1 = sj + 1;
  const int64_t sn = a.nt.slot[t] + p, se = a.ct.solve[t] + p;
  const Eq<float>& C = a.ce;
  const int mj = C.m[sj], mj1 = C.m[sj1];
  const L S{ss_smem + threadIdx.x};
  auto cp = [&](int e, const Soa<float>& src, int es, int64_t s) { cp_async4(&S[e], &src.at(es, s)); };
  /* group 0: stage A's pivot and right-hand side */
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i < mj) cp(L::Gj + q * N + i, C.G, q * N + i, sj);
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (i < mj) cp(L::oj + i, C.o, i, sj);
#pragma unroll
  for (int e = 0; e < N * N; ++e) cp(L::F1 + e, C.F, e, sj1);
#pragma unroll
  for (int i = 0; i < N; ++i) cp(L::c1 + i, C.c, i, sj1);
  cp_async_commit();
  /* group 1: the H_{j+1} columns */
#pragma unroll
  for (int e = 0; e < N * N; ++e) cp(L::H1 + e, C.H, e, sj1);
  cp_async_commit();
  /* group 2: stage C's observation rows of step j+1 */
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i < mj1) cp(L::G1 + q * N + i, C.G, q * N + i, sj1);
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (i < mj1) cp(L::o1 + i, C.o, i, sj1);
  cp_async_commit();
  /* group 3: stage B's blocks of step j (none for a track's first pair) */
  if (p > 0) {
#pragma unroll
    for (int e = 0; e < N * N; ++e) {
      cp(L::Hj + e, C.H, e, sj);
      cp(L::Fj + e, C.F, e, sj);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) cp(L::cj + i, C.c, i, sj);
  }
  cp_async_commit();

  ss_dispatch_a<N, BP>(mj + N, S);
  if (mj + mj1 == 0) a.ne.m[sn] = 0;
  else ss_dispatch_c<N, BP>(mj + mj1, S, a.ne, sn, mj);
  if (p == 0) { /* no stage B: the record is stage A's */
    cp_async_wait<0>();
#pragma unroll
    for (int e = 0; e < N * N; ++e) {
      a.cr.R.at(e, se) = S[L::Rt + e];
      a.cr.Y.at(e, se) = S[L::Yt + e];
      a.cr.Ft.at(e, se) = 0.0f;
    }
#pragma unroll
    for (int i = 0; i < N; ++i) a.cr.rhs.at(i, se) = S[L::rt + i];
    return;
  }
  ss_stage_b<N, BP>(S, a.ne, a.cr, sn, se);
}

/* ---------------------------------------------------------------------------
 * odd-length tracks: single last step + fix-up, or the one-step base case
 * ------------------------------------------------------------------------ */
template <typename T, typename TI>
__global__ void tail_kernel(Args<T, TI> a)
{
  extern __shared__ unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.ct.ntail) return;
  const int n = a.n, mx = a.mx;
  const Eq<TI>& C = a.ce;
  const Eq<T>& N = a.ne;
  const Rec<T>& Rr = a.cr;
  PV<T> ws{smem + threadIdx.x, (int)blockDim.x};
  const int t = (int)a.ct.tail[item];
  const int64_t L = a.ct.L[t];
  const int64_t sb = a.ct.slot[t];

  if (L == 1) { /* base case: x = R^{-1} Q^T o, S = R^{-1} R^{-T} */
    const int m0 = C.m[sb];
    const int64_t os = orig_step(a.track_start, a.level, t, 0);
    double* x = a.state + os * n;
    double* S = a.cov ? a.cov + os * (int64_t)n * n : nullptr;
    if (m0 < n) {
      for (int i = 0; i < n; ++i) x[i] = NAN;
      if (S) for (int e = 0; e < n * n; ++e) S[e] = NAN;
      atomicOr(a.flag, 2);
      return;
    }
    const int ld = m0;
    PV<T> W = ws, tau = ws + mx * (n + 1), dv = tau + n, Ri = dv + n;
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < m0; ++i) W[q * ld + i] = (T)C.G.at(q * mx + i, sb);
    for (int i = 0; i < m0; ++i) W[n * ld + i] = (T)C.o.at(i, sb);
    householder<T>(W, ld, m0, n, n + 1, tau);
    bool bad = false;
    for (int i = 0; i < n; ++i) {
      bad |= (W[i * ld + i] == T(0));
      dv[i] = T(1) / W[i * ld + i];
    }
    if (a.baseR.p)
      for (int q = 0; q < n; ++q)
        for (int i = 0; i < n; ++i) a.baseR.at(q * n + i, t) = (i <= q) ? W[q * ld + i] : T(0);
    auto Ru = [&](int i, int j) -> T { return W[j * ld + i]; };
    auto Di = [&](int i) -> T { return dv[i]; };
    auto xv = [&](int i) -> T& { return W[n * ld + i]; };
    solve_upper(Ru, Di, n, xv);
    for (int i = 0; i < n; ++i) x[i] = ukg_df::widen(W[n * ld + i]);
    if (S) {
      for (int q = 0; q < n; ++q) {
        for (int i = 0; i < n; ++i) Ri[q * n + i] = (i == q) ? T(1) : T(0);
        auto rc = [&](int i) -> T& { return Ri[q * n + i]; };
        solve_upper(Ru, Di, n, rc);
      }
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          T s = T(0);
          for (int k = (i > j ? i : j); k < n; ++k) s = fma(Ri[k * n + i], Ri[k * n + j], s);
          S[(int64_t)j * n + i] = ukg_df::widen(s);
        }
    }
    if (bad) atomicOr(a.flag, 2);
    return;
  }

  /* single last step s = L-1 of an odd-length level (L >= 3) */
  const int64_t s = sb + L - 1;
  const int64_t es = a.ct.solve[t] + (L - 1) / 2;
  const int64_t sn = a.nt.slot[t] + L / 2 - 1;
  const int ms = C.m[s], mt = ms < n ? ms : n;
  const int ldS = ms > 0 ? ms : 1, ldT = n + mt;
  PV<T> WS = ws, WT = ws + mx * (n + 1), WF = WT + 2 * n * (2 * n + 1), tau = WF + 2 * n * (n + 1);
  /* stage A on [G_s | o_s] */
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < ms; ++i) WS[q * ldS + i] = (T)C.G.at(q * mx + i, s);
  for (int i = 0; i < ms; ++i) WS[n * ldS + i] = (T)C.o.at(i, s);
  householder<T>(WS, ldS, ms, n, n + 1, tau);
  /* stage B on [H_s F_s c_s; R~_s 0 o'_s] */
  for (int q = 0; q < n; ++q) {
    for (int i = 0; i < n; ++i) WT[q * ldT + i] = (T)C.H.at(q * n + i, s);
    for (int i = 0; i < mt; ++i) WT[q * ldT + n + i] = (i <= q) ? WS[q * ldS + i] : T(0);
    for (int i = 0; i < n; ++i) WT[(n + q) * ldT + i] = (T)C.F.at(q * n + i, s);
    for (int i = 0; i < mt; ++i) WT[(n + q) * ldT + n + i] = T(0);
  }
  for (int i = 0; i < n; ++i) WT[2 * n * ldT + i] = (T)C.c.at(i, s);
  for (int i = 0; i < mt; ++i) WT[2 * n * ldT + n + i] = WS[n * ldS + i];
  householder<T>(WT, ldT, n + mt, n, 2 * n + 1, tau);
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < n; ++i) {
      Rr.R.at(q * n + i, es) = (i <= q) ? WT[q * ldT + i] : T(0);
      Rr.Ft.at(q * n + i, es) = WT[(n + q) * ldT + i];
      Rr.Y.at(q * n + i, es) = T(0);
    }
  for (int i = 0; i < n; ++i) Rr.rhs.at(i, es) = WT[2 * n * ldT + i];
  /* fix-up: QR of [G~_{L-2} o; Z_s o''_s] becomes the next observation */
  const int gp = N.m[sn], rF = gp + mt, ldF = rF > 0 ? rF : 1;
  for (int q = 0; q < n; ++q) {
    for (int i = 0; i < gp; ++i) WF[q * ldF + i] = N.G.at(q * mx + i, sn);
    for (int i = 0; i < mt; ++i) WF[q * ldF + gp + i] = WT[(n + q) * ldT + n + i];
  }
  for (int i = 0; i < gp; ++i) WF[n * ldF + i] = N.o.at(i, sn);
  for (int i = 0; i < mt; ++i) WF[n * ldF + gp + i] = WT[2 * n * ldT + n + i];
  householder<T>(WF, ldF, rF, n, n + 1, tau);
  const int g2 = rF < n ? rF : n;
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < g2; ++i) N.G.at(q * mx + i, sn) = (i <= q) ? WF[q * ldF + i] : T(0);
  for (int i = 0; i < g2; ++i) N.o.at(i, sn) = WF[n * ldF + i];
  N.m[sn] = g2;
}

/* ---------------------------------------------------------------------------
 * FP32 tail work (states only) with register-resident blocks: the same
 * arithmetic as tail_kernel, each QR an instantiation with compile-time rows
 * (dispatched on the run-time row count).  Hand-offs between the stages (R~
 * and o' of the single step's observation, its leftover rows Z and o'') go
 * through a per-thread slice of shared memory, element e at [e*32 + lane].
 * ------------------------------------------------------------------------ */
constexpr int kTailBS = 32;

template <int N>
struct TailSlice {
  static constexpr int Rt = 0, op = N * N, Z = N * N + N, opp = 2 * N * N + N, width = 2 * N * N + 2 * N;
  float* t0;
  __device__ __forceinline__ float& operator[](int e) const { return t0[e * kTailBS]; }
};

/* observation QR of the single last step: [G_s | o_s], MS rows */
template <int N, int MS>
__device__ __forceinline__ void tail_obs(const Eq<float>& C, int64_t s, const TailSlice<N>& S)
{
  float P[N][MS], v[MS], tau[N];
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < MS; ++i) P[q][i] = C.G.at(q * N + i, s);
#pragma unroll
  for (int i = 0; i < MS; ++i) v[i] = C.o.at(i, s);
  hh_reg<MS, N>(P, tau);
  apply_reg<MS, N>(P, tau, v);
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < MS; ++i) S[TailSlice<N>::Rt + q * N + i] = (i <= q) ? P[q][i] : 0.0f;
#pragma unroll
  for (int i = 0; i < MS; ++i) S[TailSlice<N>::op + i] = v[i];
}

/* evolution QR of the single last step: [H_s F_s c_s; R~ 0 o'], N+MT rows */
template <int N, int MT>
__device__ __forceinline__ void tail_evo(const Eq<float>& C, const Rec<float>& Rr, int64_t s, int64_t es,
                                         const TailSlice<N>& S)
{
  using L = TailSlice<N>;
  constexpr int R = N + MT;
  float P[N][R], v[R], tau[N];
#pragma unroll
  for (int q = 0; q < N; ++q) {
#pragma unroll
    for (int i = 0; i < N; ++i) P[q][i] = C.H.at(q * N + i, s);
#pragma unroll
    for (int i = 0; i < MT; ++i) P[q][N + i] = (i <= q) ? S[L::Rt + q * N + i] : 0.0f;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = C.c.at(i, s);
#pragma unroll
  for (int i = 0; i < MT; ++i) v[N + i] = S[L::op + i];
  hh_reg<R, N>(P, tau);
  apply_reg<R, N>(P, tau, v);
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Rr.R.at(q * N + i, es) = (i <= q) ? P[q][i] : 0.0f;
      Rr.Y.at(q * N + i, es) = 0.0f;
    }
#pragma unroll
  for (int i = 0; i < N; ++i) Rr.rhs.at(i, es) = v[i];
#pragma unroll
  for (int i = 0; i < MT; ++i) S[L::opp + i] = v[N + i];
#pragma unroll 1
  for (int q = 0; q < N; ++q) {
    float col[R];
#pragma unroll
    for (int i = 0; i < N; ++i) col[i] = C.F.at(q * N + i, s);
#pragma unroll
    for (int i = 0; i < MT; ++i) col[N + i] = 0.0f;
    apply_reg<R, N>(P, tau, col);
#pragma unroll
    for (int i = 0; i < N; ++i) Rr.Ft.at(q * N + i, es) = col[i];
#pragma unroll
    for (int i = 0; i < MT; ++i) S[L::Z + q * N + i] = col[N + i];
  }
}

/* fix-up: QR of [G~ o (gp rows of the next level's slot); Z o''], RF rows */
template <int N, int RF>
__device__ __forceinline__ void tail_fix(const Eq<float>& Nx, int64_t sn, int gp, const TailSlice<N>& S)
{
  using L = TailSlice<N>;
  float P[N][RF], v[RF], tau[N];
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < RF; ++i) P[q][i] = i < gp ? Nx.G.at(q * N + i, sn) : S[L::Z + q * N + (i - gp)];
#pragma unroll
  for (int i = 0; i < RF; ++i) v[i] = i < gp ? Nx.o.at(i, sn) : S[L::opp + (i - gp)];
  hh_reg<RF, N>(P, tau);
  apply_reg<RF, N>(P, tau, v);
  constexpr int G2 = RF < N ? RF : N;
#pragma unroll
  for (int q = 0; q < N; ++q)
#pragma unroll
    for (int i = 0; i < G2; ++i) Nx.G.at(q * N + i, sn) = (i <= q) ? P[q][i] : 0.0f;
#pragma unroll
  for (int i = 0; i < G2; ++i) Nx.o.at(i, sn) = v[i];
  Nx.m[sn] = G2;
}

template <int N, int K = 1>
__device__ __forceinline__ void tail_obs_d(int ms, const Eq<float>& C, int64_t s, const TailSlice<N>& S)
{
  if constexpr (K <= N) {
    if (ms == K) tail_obs<N, K>(C, s, S);
    else tail_obs_d<N, K + 1>(ms, C, s, S);
  }
}
template <int N, int K = 0>
__device__ __forceinline__ void tail_evo_d(int mt, const Eq<float>& C, const Rec<float>& Rr, int64_t s, int64_t es,
                                           const TailSlice<N>& S)
{
  if constexpr (K <= N) {
    if (mt == K) tail_evo<N, K>(C, Rr, s, es, S);
    else tail_evo_d<N, K + 1>(mt, C, Rr, s, es, S);
  }
}
template <int N, int K = 1>
__device__ __forceinline__ void tail_fix_d(int rf, const Eq<float>& Nx, int64_t sn, int gp, const TailSlice<N>& S)
{
  if constexpr (K <= 2 * N) {
    if (rf == K) tail_fix<N, K>(Nx, sn, gp, S);
    else tail_fix_d<N, K + 1>(rf, Nx, sn, gp, S);
  }
}

template <int N>
__global__ void __launch_bounds__(kTailBS) tail_reg_kernel(Args<float, float> a)
{
  __shared__ float tail_smem[TailSlice<N>::width * kTailBS];
  const int64_t item = (int64_t)blockIdx.x * kTailBS + threadIdx.x;
  if (item >= a.ct.ntail) return;
  const Eq<float>& C = a.ce;
  const int t = (int)a.ct.tail[item];
  const int64_t L = a.ct.L[t];
  const int64_t sb = a.ct.slot[t];
  if (L == 1) { /* base case: x = R^{-1} Q^T o */
    const int m0 = C.m[sb];
    double* x = a.state + orig_step(a.track_start, a.level, t, 0) * N;
    if (m0 < N) {
#pragma unroll
      for (int i = 0; i < N; ++i) x[i] = NAN;
      atomicOr(a.flag, 2);
      return;
    }
    float P[N][N], v[N], tau[N];
#pragma unroll
    for (int q = 0; q < N; ++q)
#pragma unroll
      for (int i = 0; i < N; ++i) P[q][i] = C.G.at(q * N + i, sb);
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = C.o.at(i, sb);
    hh_reg<N, N>(P, tau);
    apply_reg<N, N>(P, tau, v);
    bool bad = false;
    if (a.baseR.p)
#pragma unroll
      for (int q = 0; q < N; ++q)
#pragma unroll
        for (int i = 0; i < N; ++i) a.baseR.at(q * N + i, t) = (i <= q) ? P[q][i] : 0.0f;
#pragma unroll
    for (int i = N - 1; i >= 0; --i) {
      float sm = v[i];
#pragma unroll
      for (int k = i + 1; k < N; ++k) sm = fmaf(-P[k][i], v[k], sm);
      bad |= P[i][i] == 0.0f;
      v[i] = sm * (1.0f / P[i][i]);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) x[i] = ukg_df::f32_to_f64(v[i]);
    if (bad) atomicOr(a.flag, 2);
    return;
  }
  const TailSlice<N> S{tail_smem + threadIdx.x};
  const int64_t s = sb + L - 1;
  const int64_t es = a.ct.solve[t] + (L - 1) / 2;
  const int64_t sn = a.nt.slot[t] + L / 2 - 1;
  const int ms = C.m[s], mt = ms < N ? ms : N;
  if (ms > 0) tail_obs_d<N>(ms, C, s, S);
  tail_evo_d<N>(mt, C, a.cr, s, es, S);
  const int gp = a.ne.m[sn], rf = gp + mt;
  if (rf > 0) tail_fix_d<N>(rf, a.ne, sn, gp, S);
  else a.ne.m[sn] = 0;
}

/* ---------------------------------------------------------------------------
 * back-substitution and covariance recurrence for the even steps of a level
 *
 * With B = [Ft Y] and Sigma = [[Smm Smp]; [Smp^T Spp]] the joint covariance of
 * the odd neighbours (x_{j-1}, x_{j+1}):
 *   x_j            = R^{-1} (rhs - Ft x_{j-1} - Y x_{j+1})
 *   S_j            = R^{-1} (I + B Sigma B^T) R^{-T}
 *   cov(x_j, x_{j-1}) = -R^{-1} (B Sigma)[:, 0:n]
 *   cov(x_j, x_{j+1}) = -R^{-1} (B Sigma)[:, n:2n]
 * (the reference's formulas, Solve_Estimates 703-903, grouped by columns of
 * B Sigma, which are streamed one at a time).  In a refinement sweep the
 * right-hand side is y (yrhs) and `state` holds the correction d.
 * ------------------------------------------------------------------------ */
template <typename T, int NT = 0, int BS = 0>
__global__ void __launch_bounds__(BS ? BS : 1024) solve_kernel(Args<T, T> a, int want_cov)
{
  extern __shared__ unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.ct.nsolve) return;
  const int n = NT ? NT : a.n;
  const int64_t nn = (int64_t)n * n;
  const Rec<T>& Rr = a.cr;
  const int t = find_track(a.ct.solve, a.ntracks, item);
  const int64_t e = item - a.ct.solve[t];
  const int64_t j = 2 * e, L = a.ct.L[t];
  const bool hp = j > 0, hn = j + 1 < L;
  const int64_t se = item; /* records are indexed by the solve prefix */
  const int64_t oj = orig_step(a.track_start, a.level, t, j);
  const int64_t om = hp ? orig_step(a.track_start, a.level, t, j - 1) : 0;
  const int64_t op = hn ? orig_step(a.track_start, a.level, t, j + 1) : 0;

  using View = typename ViewOf<T, BS>::type;
  View ws = ViewOf<T, BS>::make(smem);
  View Rs = ws, Fs = ws + n * n, Ys = ws + 2 * n * n, M = ws + 3 * n * n, sg = ws + 4 * n * n, pv = sg + 2 * n,
       dv = pv + n;
  bool bad = false;
  for (int k = 0; k < n * n; ++k) {
    Rs[k] = Rr.R.at(k, se);
    Fs[k] = hp ? Rr.Ft.at(k, se) : T(0);
    Ys[k] = hn ? Rr.Y.at(k, se) : T(0);
  }
  for (int i = 0; i < n; ++i) {
    const T d = Rs[i * n + i];
    bad |= (d == T(0));
    dv[i] = T(1) / d;
  }
  auto Ru = [&](int i, int jj) -> T { return Rs[jj * n + i]; };
  auto Di = [&](int i) -> T { return dv[i]; };

  /* state */
  for (int i = 0; i < n; ++i) pv[i] = a.yrhs.p ? a.yrhs.at(i, se) : Rr.rhs.at(i, se);
  if (hp) {
    const double* xm = a.state + om * n;
    for (int k = 0; k < n; ++k) {
      const T xk = ukg_df::narrow<T>(xm[k]);
      for (int i = 0; i < n; ++i) pv[i] = fma(-Fs[k * n + i], xk, pv[i]);
    }
  }
  if (hn) {
    const double* xp = a.state + op * n;
    for (int k = 0; k < n; ++k) {
      const T xk = ukg_df::narrow<T>(xp[k]);
      for (int i = 0; i < n; ++i) pv[i] = fma(-Ys[k * n + i], xk, pv[i]);
    }
  }
  auto pvr = [&](int i) -> T& { return pv[i]; };
  solve_upper(Ru, Di, n, pvr);
  double* xo = a.state + oj * n;
  for (int i = 0; i < n; ++i) xo[i] = ukg_df::widen(pv[i]);
  if (!want_cov) {
    if (bad) atomicOr(a.flag, 2);
    return;
  }

  const double* Smm = hp ? a.cov + om * nn : nullptr;
  const double* Spp = hn ? a.cov + op * nn : nullptr;
  const int64_t smp = (hp && hn) ? a.nt.slot[t] + (j + 1) / 2 : 0; /* U of the next level */
  for (int k = 0; k < n * n; ++k) M[k] = T(0);
  const int q0 = hp ? 0 : n, q1 = hn ? 2 * n : n;
  for (int q = q0; q < q1; ++q) {
    /* column q of Sigma */
    if (q < n) {
      for (int i = 0; i < n; ++i) sg[i] = ukg_df::narrow<T>(Smm[(int64_t)q * n + i]);
      for (int i = 0; i < n; ++i) sg[n + i] = hn ? a.nr.U.at(i * n + q, smp) : T(0); /* Smp[q, :] */
    } else {
      const int qq = q - n;
      for (int i = 0; i < n; ++i) sg[i] = hp ? a.nr.U.at(qq * n + i, smp) : T(0);
      for (int i = 0; i < n; ++i) sg[n + i] = ukg_df::narrow<T>(Spp[(int64_t)qq * n + i]);
    }
    /* pv = B sigma */
    for (int i = 0; i < n; ++i) pv[i] = T(0);
    if (hp)
      for (int k = 0; k < n; ++k) {
        const T sk = sg[k];
        for (int i = 0; i < n; ++i) pv[i] = fma(Fs[k * n + i], sk, pv[i]);
      }
    if (hn)
      for (int k = 0; k < n; ++k) {
        const T sk = sg[n + k];
        for (int i = 0; i < n; ++i) pv[i] = fma(Ys[k * n + i], sk, pv[i]);
      }
    /* M += pv b_q^T, b_q = column q of B */
    View bq = q < n ? Fs + q * n : Ys + (q - n) * n;
    for (int c = 0; c < n; ++c) {
      const T bc = bq[c];
      for (int i = 0; i < n; ++i) M[c * n + i] = fma(pv[i], bc, M[c * n + i]);
    }
    if (a.level == 0) continue; /* level 0's off-diagonal blocks are not needed */
    /* off-diagonal block column: -R^{-1} pv */
    solve_upper(Ru, Di, n, pvr);
    if (q < n) { /* cov(x_{j-1}, x_j) = cov(x_j, x_{j-1})^T: row q */
      const int64_t sU = a.ct.slot[t] + j;
      for (int i = 0; i < n; ++i) Rr.U.at(i * n + q, sU) = -pv[i];
    } else {
      const int64_t sU = a.ct.slot[t] + j + 1;
      for (int i = 0; i < n; ++i) Rr.U.at((q - n) * n + i, sU) = -pv[i];
    }
  }
  for (int i = 0; i < n; ++i) M[i * n + i] += T(1);
  /* S = R^{-1} M R^{-T}: solve the columns, transpose, solve again, transpose */
  for (int c = 0; c < n; ++c) {
    auto mc = [&](int i) -> T& { return M[c * n + i]; };
    solve_upper(Ru, Di, n, mc);
  }
  for (int c = 0; c < n; ++c)
    for (int i = c + 1; i < n; ++i) {
      const T tmp = M[c * n + i];
      M[c * n + i] = M[i * n + c];
      M[i * n + c] = tmp;
    }
  for (int c = 0; c < n; ++c) {
    auto mc = [&](int i) -> T& { return M[c * n + i]; };
    solve_upper(Ru, Di, n, mc);
  }
  double* So = a.cov + oj * nn;
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < n; ++i) So[(int64_t)c * n + i] = ukg_df::widen(M[i * n + c]);
  if (bad) atomicOr(a.flag, 2);
}

/* ---------------------------------------------------------------------------
 * back-substitution with covariances, register-tiled (n = 4, 6)
 *
 * The same arithmetic as solve_kernel with want_cov, in the same order (the
 * results are equal bit for bit), but R, the reciprocals of its diagonal and
 * the n x n accumulator M live in registers; only F~ and Y (2 n^2 entries) use
 * the thread's shared-memory slice.  solve_kernel's slices (4 n^2 + 4 n
 * entries) hold four warps per SM; here about ten fit, which the FP64 pipe and
 * the double-float arithmetic both need to hide their latencies.
 * ------------------------------------------------------------------------ */
template <typename T, int N, int BS>
__global__ void __launch_bounds__(BS) solve_cov_reg_kernel(Args<T, T> a)
{
  extern __shared__ unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  const int64_t item = (int64_t)blockIdx.x * BS + threadIdx.x;
  if (item >= a.ct.nsolve) return;
  constexpr int nn = N * N;
  const Rec<T>& Rr = a.cr;
  const int t = find_track(a.ct.solve, a.ntracks, item);
  const int64_t e = item - a.ct.solve[t];
  const int64_t j = 2 * e, L = a.ct.L[t];
  const bool hp = j > 0, hn = j + 1 < L;
  const int64_t se = item;
  const int64_t oj = orig_step(a.track_start, a.level, t, j);
  const int64_t om = hp ? orig_step(a.track_start, a.level, t, j - 1) : 0;
  const int64_t op = hn ? orig_step(a.track_start, a.level, t, j + 1) : 0;
  PVc<T, BS> Fs{smem + threadIdx.x}, Ys = Fs + nn;
  T R[N][N], dv[N];
  bool bad = false;
#pragma unroll
  for (int c = 0; c < N; ++c)
#pragma unroll
    for (int i = 0; i <= c; ++i) R[i][c] = Rr.R.at(c * N + i, se);
  for (int k = 0; k < nn; ++k) {
    Fs[k] = hp ? Rr.Ft.at(k, se) : T(0);
    Ys[k] = hn ? Rr.Y.at(k, se) : T(0);
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    bad |= (R[i][i] == T(0));
    dv[i] = T(1) / R[i][i];
  }
  /* x <- R^{-1} x, the order of solve_upper */
  auto solve = [&](T (&x)[N]) {
#pragma unroll
    for (int jj = N - 1; jj >= 0; --jj) {
      const T xj = x[jj] * dv[jj];
      x[jj] = xj;
#pragma unroll
      for (int i = 0; i < jj; ++i) x[i] = fma(-xj, R[i][jj], x[i]);
    }
  };

  /* state */
  T pv[N];
#pragma unroll
  for (int i = 0; i < N; ++i) pv[i] = a.yrhs.p ? a.yrhs.at(i, se) : Rr.rhs.at(i, se);
  if (hp) {
    const double* xm = a.state + om * N;
    for (int k = 0; k < N; ++k) {
      const T xk = ukg_df::narrow<T>(xm[k]);
#pragma unroll
      for (int i = 0; i < N; ++i) pv[i] = fma(-Fs[k * N + i], xk, pv[i]);
    }
  }
  if (hn) {
    const double* xp = a.state + op * N;
    for (int k = 0; k < N; ++k) {
      const T xk = ukg_df::narrow<T>(xp[k]);
#pragma unroll
      for (int i = 0; i < N; ++i) pv[i] = fma(-Ys[k * N + i], xk, pv[i]);
    }
  }
  solve(pv);
  double* xo = a.state + oj * N;
#pragma unroll
  for (int i = 0; i < N; ++i) xo[i] = ukg_df::widen(pv[i]);

  const double* Smm = hp ? a.cov + om * nn : nullptr;
  const double* Spp = hn ? a.cov + op * nn : nullptr;
  const int64_t smp = (hp && hn) ? a.nt.slot[t] + (j + 1) / 2 : 0; /* U of the next level */
  T M[N][N]; /* M[c][i]: column c, row i */
#pragma unroll
  for (int c = 0; c < N; ++c)
#pragma unroll
    for (int i = 0; i < N; ++i) M[c][i] = T(0);
  const int q0 = hp ? 0 : N, q1 = hn ? 2 * N : N;
#pragma unroll 1
  for (int q = q0; q < q1; ++q) {
    T sg[2 * N];
    if (q < N) {
#pragma unroll
      for (int i = 0; i < N; ++i) sg[i] = ukg_df::narrow<T>(Smm[(int64_t)q * N + i]);
#pragma unroll
      for (int i = 0; i < N; ++i) sg[N + i] = hn ? a.nr.U.at(i * N + q, smp) : T(0); /* Smp[q, :] */
    } else {
      const int qq = q - N;
#pragma unroll
      for (int i = 0; i < N; ++i) sg[i] = hp ? a.nr.U.at(qq * N + i, smp) : T(0);
#pragma unroll
      for (int i = 0; i < N; ++i) sg[N + i] = ukg_df::narrow<T>(Spp[(int64_t)qq * N + i]);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) pv[i] = T(0);
    if (hp)
#pragma unroll
      for (int k = 0; k < N; ++k) {
        const T sk = sg[k];
#pragma unroll
        for (int i = 0; i < N; ++i) pv[i] = fma(Fs[k * N + i], sk, pv[i]);
      }
    if (hn)
#pragma unroll
      for (int k = 0; k < N; ++k) {
        const T sk = sg[N + k];
#pragma unroll
        for (int i = 0; i < N; ++i) pv[i] = fma(Ys[k * N + i], sk, pv[i]);
      }
    PVc<T, BS> bq = q < N ? Fs + q * N : Ys + (q - N) * N; /* column q of B = [F~ | Y] */
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const T bc = bq[c];
#pragma unroll
      for (int i = 0; i < N; ++i) M[c][i] = fma(pv[i], bc, M[c][i]);
    }
    if (a.level == 0) continue; /* level 0's off-diagonal blocks are not needed */
    solve(pv);
    if (q < N) { /* cov(x_{j-1}, x_j) = cov(x_j, x_{j-1})^T: row q */
      const int64_t sU = a.ct.slot[t] + j;
#pragma unroll
      for (int i = 0; i < N; ++i) Rr.U.at(i * N + q, sU) = -pv[i];
    } else {
      const int64_t sU = a.ct.slot[t] + j + 1;
#pragma unroll
      for (int i = 0; i < N; ++i) Rr.U.at((q - N) * N + i, sU) = -pv[i];
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) M[i][i] += T(1);
  /* S = R^{-1} M R^{-T}: solve the columns, transpose, solve again, transpose */
#pragma unroll
  for (int c = 0; c < N; ++c) solve(M[c]);
#pragma unroll
  for (int c = 0; c < N; ++c)
#pragma unroll
    for (int i = c + 1; i < N; ++i) {
      const T tmp = M[c][i];
      M[c][i] = M[i][c];
      M[i][c] = tmp;
    }
#pragma unroll
  for (int c = 0; c < N; ++c) solve(M[c]);
  double* So = a.cov + oj * nn;
#pragma unroll
  for (int c = 0; c < N; ++c)
#pragma unroll
    for (int i = 0; i < N; ++i) So[(int64_t)c * N + i] = ukg_df::widen(M[i][c]);
  if (bad) atomicOr(a.flag, 2);
}

/* ---------------------------------------------------------------------------
 * refinement sweep kernels (FP32 factors, FP64 residual)
 * ------------------------------------------------------------------------ */

/* w <- Cov^{-1} w for a covariance factor (cov, type): with Cov^{-1} = V^T V
 * for the weighing V of kalman_covariance_matrix_weigh -- 'W': W^T (W w),
 * 'w': diag(cov)^2 w, 'C': L^{-T} L^{-1} w (L = chol(cov)), 'U'/'F':
 * L^{-T} L^{-1} w (L = tril(cov)).  FP64; L, dinv, tmp as in weigh_column.  */
__device__ bool apply_precision(char type, const double* cov, int ldc, int rows, PV<double> L, PV<double> dinv,
                                PV<double> w, PV<double> tmp)
{
  if (type == 'W') {
    for (int i = 0; i < rows; ++i) {
      double s = 0.0;
      for (int j = 0; j < rows; ++j) s = fma(cov[(int64_t)j * ldc + i], w[j], s);
      tmp[i] = s;
    }
    for (int j = 0; j < rows; ++j) {
      double s = 0.0;
      for (int i = 0; i < rows; ++i) s = fma(cov[(int64_t)j * ldc + i], tmp[i], s);
      w[j] = s;
    }
    return true;
  }
  if (type == 'w') {
    for (int i = 0; i < rows; ++i) w[i] *= cov[i] * cov[i];
    return true;
  }
  const bool ok = lower_factor(type, cov, ldc, rows, L, dinv);
  for (int j = 0; j < rows; ++j) { /* L^{-1} */
    const double xj = w[j] * dinv[j];
    w[j] = xj;
    for (int i = j + 1; i < rows; ++i) w[i] = fma(-xj, L[j * rows + i], w[i]);
  }
  for (int j = rows - 1; j >= 0; --j) { /* L^{-T} */
    double s = w[j];
    for (int i = j + 1; i < rows; ++i) s = fma(-L[j * rows + i], w[i], s);
    w[j] = s * dinv[j];
  }
  return ok;
}

/* The refinement's right-hand side z = A^T (b - A x) of the weighted
 * least-squares system, in FP64 from the caller's raw equations.  With the
 * raw residuals r_i = c_i + F_i x_{i-1} - H_i x_i and s_i = o_i - G_i x_i:
 *   wE_i = K_i^{-1} r_i,   z_i = H_i^T wE_i + G_i^T C_i^{-1} s_i - F_{i+1}^T wE_{i+1}.
 * residual_kernel stores wE_i and the first two terms; atr_kernel adds the
 * third and rounds z to FP32.  FP64 is needed: at the solution r is the
 * (nonzero) least-squares residual, and z -> 0 is formed by cancellation.    */
__global__ void residual_kernel(Args<float, float> a, RawDev raw, Soa<double> wE, Soa<double> zp, int64_t nsteps)
{
  extern __shared__ unsigned char smem_raw[];
  double* smem = reinterpret_cast<double*>(smem_raw);
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nsteps) return;
  const int n = a.n, mx = a.mx, mm = raw.mmax;
  PV<double> ws{smem + threadIdx.x, (int)blockDim.x};
  PV<double> L = ws, dinv = ws + mx * mx, w = dinv + mx, tmp = w + mx, z = tmp + mx;
  const int t = find_track(a.track_start, a.ntracks, g);
  const int64_t i = g - a.track_start[t];
  const int64_t q = a.ct.slot[t] + i;
  const int64_t nn = (int64_t)n * n;
  const double* x = a.state + g * n;
  for (int c = 0; c < n; ++c) z[c] = 0.0;
  if (i > 0) {
    const double* xm = x - n;
    const double* H = raw.H + g * nn;
    const double* F = raw.F + g * nn;
    for (int p = 0; p < n; ++p) {
      double s = raw.c[g * n + p];
      for (int c = 0; c < n; ++c) s = fma(F[c * n + p], xm[c], fma(-H[c * n + p], x[c], s));
      w[p] = s;
    }
    apply_precision(raw.K_type[g], raw.K + g * nn, n, n, L, dinv, w, tmp);
    for (int p = 0; p < n; ++p) wE.at(p, q) = w[p];
    for (int c = 0; c < n; ++c) {
      double s = z[c];
      for (int p = 0; p < n; ++p) s = fma(H[c * n + p], w[p], s);
      z[c] = s;
    }
  }
  const int m = a.ce.m[q];
  if (m > 0) {
    const double* G = raw.G + g * (int64_t)mm * n;
    for (int p = 0; p < m; ++p) {
      double s = raw.o[g * mm + p];
      for (int c = 0; c < n; ++c) s = fma(-G[(int64_t)c * mm + p], x[c], s);
      w[p] = s;
    }
    apply_precision(raw.C_type[g], raw.C + g * (int64_t)mm * mm, mm, m, L, dinv, w, tmp);
    for (int c = 0; c < n; ++c) {
      double s = z[c];
      for (int p = 0; p < m; ++p) s = fma(G[(int64_t)c * mm + p], w[p], s);
      z[c] = s;
    }
  }
  for (int c = 0; c < n; ++c) zp.at(c, q) = z[c];
}

__global__ void atr_kernel(Args<float, float> a, RawDev raw, Soa<double> wE, Soa<double> zp, Soa<float> z0,
                           int64_t nsteps)
{
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nsteps) return;
  const int n = a.n;
  const int t = find_track(a.track_start, a.ntracks, g);
  const int64_t g0 = a.track_start[t], k = a.track_start[t + 1] - g0, i = g - g0;
  const int64_t q = a.ct.slot[t] + i;
  const double* F1 = raw.F + (g + 1) * (int64_t)n * n;
  for (int c = 0; c < n; ++c) {
    double s = zp.at(c, q);
    if (i + 1 < k)
      for (int p = 0; p < n; ++p) s = fma(-F1[c * n + p], wE.at(p, q + 1), s);
    z0.at(c, q) = ukg_df::f64_to_f32(s);
  }
}

/* The same right-hand side z, for the double-float weighed equations that
 * weigh_df_kernel leaves at level 0 (FP32 high parts in the level-0 arrays,
 * low parts in `lo`): with the weighed evolution H~ x_i + F~ x_{i-1} = c~ and
 * observation G~ x_i = o~ (F~ = -V F),
 *   r~_i = c~_i - H~_i x_i - F~_i x_{i-1},   s~_i = o~_i - G~_i x_i,
 *   z_i  = H~_i^T r~_i + G~_i^T s~_i + F~_{i+1}^T r~_{i+1}
 * in df arithmetic on the FP32 pipe.  Block b handles steps g0 = b(B-1) ..
 * g0+B-1: every thread forms u = F~^T r~ for its step, the first B-1 also z,
 * and thread k adds thread k+1's u, so the next step's term needs no second
 * pass.  The level-0 arrays are element-major, so every load is coalesced.
 * Writes z rounded to FP32.                                                  */
template <int N, int MM, int B>
__global__ void __launch_bounds__(B, 4) residual_df_kernel(Args<float, float> a, Eq<float> lo, Soa<float> z0,
                                                           int64_t nsteps)
{
  using namespace ukg_df;
  constexpr int MX = MM > N ? MM : N; /* leading dimension of the level-0 G */
  __shared__ float ush[2 * N][B];
  const int tid = threadIdx.x;
  const int64_t g = (int64_t)blockIdx.x * (B - 1) + tid;
  const bool live = g < nsteps, own = tid < B - 1;
  const Eq<float>& E = a.ce;
  df z[N], u[N];
#pragma unroll
  for (int c = 0; c < N; ++c) z[c] = u[c] = make(0.0f);
  int64_t q = 0;
  bool has_next = false;
  if (live) {
    const int t = find_track(a.track_start, a.ntracks, g);
    const int64_t i = g - a.track_start[t];
    has_next = g + 1 < a.track_start[t + 1];
    q = a.ct.slot[t] + i;
    auto ld = [&](const Soa<float>& h, const Soa<float>& l, int e) { return df{h.at(e, q), l.at(e, q)}; };
    const double* xg = a.state + g * N;
    df xn[N]; /* -x_i */
#pragma unroll
    for (int c = 0; c < N; ++c) xn[c] = neg(split(xg[c]));
    if (i > 0) {
      df xm[N]; /* -x_{i-1} */
#pragma unroll
      for (int c = 0; c < N; ++c) xm[c] = neg(split(xg[c - N]));
      df r[N];
#pragma unroll
      for (int p = 0; p < N; ++p) {
        acc sr = start(ld(E.c, lo.c, p));
#pragma unroll
        for (int c = 0; c < N; ++c) {
          add_prod(sr, ld(E.H, lo.H, c * N + p), xn[c]);
          add_prod(sr, ld(E.F, lo.F, c * N + p), xm[c]);
        }
        r[p] = finish(sr);
      }
#pragma unroll
      for (int c = 0; c < N; ++c) {
        acc su = start(make(0.0f)), sz = start(make(0.0f));
#pragma unroll
        for (int p = 0; p < N; ++p) {
          add_prod(su, ld(E.F, lo.F, c * N + p), r[p]);
          if (own) add_prod(sz, ld(E.H, lo.H, c * N + p), r[p]);
        }
        u[c] = finish(su);
        z[c] = finish(sz);
      }
    }
    const int m = E.m[q];
    if (own && m > 0) {
      df s[MM];
#pragma unroll
      for (int p = 0; p < MM; ++p) {
        s[p] = make(0.0f);
        if (p < m) {
          acc sp = start(ld(E.o, lo.o, p));
#pragma unroll
          for (int c = 0; c < N; ++c) add_prod(sp, ld(E.G, lo.G, c * MX + p), xn[c]);
          s[p] = finish(sp);
        }
      }
#pragma unroll
      for (int c = 0; c < N; ++c) {
        acc sz = start(z[c]);
#pragma unroll
        for (int p = 0; p < MM; ++p)
          if (p < m) add_prod(sz, ld(E.G, lo.G, c * MX + p), s[p]);
        z[c] = finish(sz);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < N; ++c) {
    ush[2 * c][tid] = u[c].hi;
    ush[2 * c + 1][tid] = u[c].lo;
  }
  __syncthreads();
  if (live && own) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      df zc = z[c];
      if (has_next) zc = add(zc, df{ush[2 * c][tid + 1], ush[2 * c + 1][tid + 1]});
      z0.at(c, q) = round_df(zc);
    }
  }
}

/* R^T y = z, even steps of a level: y_j = R_j^{-T} z_j                       */
__global__ void rt_even_kernel(Args<float, float> a, Soa<float> zc, Soa<float> yc)
{
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.ct.nsolve) return;
  const int n = a.n;
  const int t = find_track(a.ct.solve, a.ntracks, item);
  const int64_t j = 2 * (item - a.ct.solve[t]);
  const int64_t sz = a.ct.slot[t] + j;
  const Soa<float>& R = a.cr.R;
  auto Ru = [&](int i, int jj) -> float { return R.at(jj * n + i, item); };
  auto Di = [&](int i) -> float { return 1.0f / R.at(i * n + i, item); };
  auto yv = [&](int i) -> float& { return yc.at(i, item); };
  for (int i = 0; i < n; ++i) yc.at(i, item) = zc.at(i, sz);
  solve_upper_t(Ru, Di, n, yv);
}

/* the odd steps' right-hand sides lose the even rows' contributions and
 * become the next level's: z' = z_{2p+1} - Y_{2p}^T y_{2p} - Ft_{2p+2}^T y_{2p+2} */
__global__ void rt_odd_kernel(Args<float, float> a, Soa<float> zc, Soa<float> yc, Soa<float> zn)
{
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.ct.npairs) return;
  const int n = a.n;
  const int t = find_track(a.ct.pair, a.ntracks, item);
  const int64_t p = item - a.ct.pair[t], L = a.ct.L[t];
  const int64_t so = a.ct.slot[t] + 2 * p + 1, sn = a.nt.slot[t] + p;
  const int64_t e0 = a.ct.solve[t] + p, e1 = e0 + 1;
  const bool right = 2 * p + 2 <= L - 1;
  for (int c = 0; c < n; ++c) {
    float s = zc.at(c, so);
    for (int r = 0; r < n; ++r) s = fma(-a.cr.Y.at(c * n + r, e0), yc.at(r, e0), s);
    if (right)
      for (int r = 0; r < n; ++r) s = fma(-a.cr.Ft.at(c * n + r, e1), yc.at(r, e1), s);
    zn.at(c, sn) = s;
  }
}

/* one-step levels: d = R_b^{-1} R_b^{-T} z                                   */
__global__ void rt_base_kernel(Args<float, float> a, Soa<float> zc, Soa<float> tmp)
{
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.ct.ntail) return;
  const int n = a.n;
  const int t = (int)a.ct.tail[item];
  if (a.ct.L[t] != 1) return;
  const int64_t sz = a.ct.slot[t];
  auto Ru = [&](int i, int jj) -> float { return a.baseR.at(jj * n + i, t); };
  auto Di = [&](int i) -> float { return 1.0f / a.baseR.at(i * n + i, t); };
  auto v = [&](int i) -> float& { return tmp.at(i, item); };
  for (int i = 0; i < n; ++i) tmp.at(i, item) = zc.at(i, sz);
  solve_upper_t(Ru, Di, n, v);
  solve_upper(Ru, Di, n, v);
  double* d = a.state + orig_step(a.track_start, a.level, t, 0) * n;
  for (int i = 0; i < n; ++i) d[i] = ukg_df::widen(tmp.at(i, item));
}

/* ---------------------------------------------------------------------------
 * FP32 state-only back-substitution and refinement transpose solves with the
 * blocks in registers (compile-time n): every load of a thread is issued
 * before its arithmetic, which keeps many loads in flight per SM.  Same
 * arithmetic as solve_kernel (want_cov = 0), rt_even_kernel and rt_odd_kernel.
 * ------------------------------------------------------------------------ */
template <int N>
__global__ void __launch_bounds__(128) solve_state_reg_kernel(Args<float, float> a)
{
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.ct.nsolve) return;
  const int t = find_track(a.ct.solve, a.ntracks, item);
  const int64_t j = 2 * (item - a.ct.solve[t]), L = a.ct.L[t];
  const bool hp = j > 0, hn = j + 1 < L;
  const Rec<float>& Rr = a.cr;
  float R[N][N], pv[N];
#pragma unroll
  for (int k = 0; k < N; ++k)
#pragma unroll
    for (int i = 0; i <= k; ++i) R[k][i] = Rr.R.at(k * N + i, item);
#pragma unroll
  for (int i = 0; i < N; ++i) pv[i] = a.yrhs.p ? a.yrhs.at(i, item) : Rr.rhs.at(i, item);
  if (hp) {
    const double* xm = a.state + orig_step(a.track_start, a.level, t, j - 1) * N;
    float F[N][N], x[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
      x[k] = ukg_df::f64_to_f32(xm[k]);
#pragma unroll
      for (int i = 0; i < N; ++i) F[k][i] = Rr.Ft.at(k * N + i, item);
    }
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
      for (int i = 0; i < N; ++i) pv[i] = fmaf(-F[k][i], x[k], pv[i]);
  }
  if (hn) {
    const double* xp = a.state + orig_step(a.track_start, a.level, t, j + 1) * N;
    float Y[N][N], x[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
      x[k] = ukg_df::f64_to_f32(xp[k]);
#pragma unroll
      for (int i = 0; i < N; ++i) Y[k][i] = Rr.Y.at(k * N + i, item);
    }
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
      for (int i = 0; i < N; ++i) pv[i] = fmaf(-Y[k][i], x[k], pv[i]);
  }
  bool bad = false;
#pragma unroll
  for (int i = N - 1; i >= 0; --i) {
    float sm = pv[i];
#pragma unroll
    for (int k = i + 1; k < N; ++k) sm = fmaf(-R[k][i], pv[k], sm);
    bad |= R[i][i] == 0.0f;
    pv[i] = sm * (1.0f / R[i][i]);
  }
  double* xo = a.state + orig_step(a.track_start, a.level, t, j) * N;
#pragma unroll
  for (int i = 0; i < N; ++i) xo[i] = ukg_df::f32_to_f64(pv[i]);
  if (bad) atomicOr(a.flag, 2);
}

template <int N>
__global__ void __launch_bounds__(128) rt_even_reg_kernel(Args<float, float> a, Soa<float> zc, Soa<float> yc)
{
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.ct.nsolve) return;
  const int t = find_track(a.ct.solve, a.ntracks, item);
  const int64_t sz = a.ct.slot[t] + 2 * (item - a.ct.solve[t]);
  float R[N][N], y[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    y[k] = zc.at(k, sz);
#pragma unroll
    for (int i = 0; i <= k; ++i) R[k][i] = a.cr.R.at(k * N + i, item);
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    float sm = y[i];
#pragma unroll
    for (int k = 0; k < i; ++k) sm = fmaf(-R[i][k], y[k], sm);
    y[i] = sm * (1.0f / R[i][i]);
    yc.at(i, item) = y[i];
  }
}

template <int N>
__global__ void __launch_bounds__(128) rt_odd_reg_kernel(Args<float, float> a, Soa<float> zc, Soa<float> yc,
                                                         Soa<float> zn)
{
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.ct.npairs) return;
  const int t = find_track(a.ct.pair, a.ntracks, item);
  const int64_t p = item - a.ct.pair[t], L = a.ct.L[t];
  const int64_t so = a.ct.slot[t] + 2 * p + 1, sn = a.nt.slot[t] + p;
  const int64_t e0 = a.ct.solve[t] + p, e1 = e0 + 1;
  const bool right = 2 * p + 2 <= L - 1;
  float Y[N][N], y0[N], z[N];
#pragma unroll
  for (int c = 0; c < N; ++c) {
    z[c] = zc.at(c, so);
    y0[c] = yc.at(c, e0);
#pragma unroll
    for (int r = 0; r < N; ++r) Y[c][r] = a.cr.Y.at(c * N + r, e0);
  }
  if (right) {
    float F[N][N], y1[N];
#pragma unroll
    for (int c = 0; c < N; ++c) {
      y1[c] = yc.at(c, e1);
#pragma unroll
      for (int r = 0; r < N; ++r) F[c][r] = a.cr.Ft.at(c * N + r, e1);
    }
#pragma unroll
    for (int c = 0; c < N; ++c)
#pragma unroll
      for (int r = 0; r < N; ++r) z[c] = fmaf(-F[c][r], y1[r], z[c]);
  }
#pragma unroll
  for (int c = 0; c < N; ++c) {
    float sm = z[c];
#pragma unroll
    for (int r = 0; r < N; ++r) sm = fmaf(-Y[c][r], y0[r], sm);
    zn.at(c, sn) = sm;
  }
}

/* rt_base_kernel with the track's base-case R and right-hand side in
 * registers: the same two triangular solves in the same order (the results
 * are identical), without a round trip to memory per operation.            */
template <int N>
__global__ void __launch_bounds__(128) rt_base_reg_kernel(Args<float, float> a, Soa<float> zc)
{
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.ct.ntail) return;
  const int t = (int)a.ct.tail[item];
  if (a.ct.L[t] != 1) return;
  const int64_t sz = a.ct.slot[t];
  float R[N][N], v[N]; /* R[j][i]: row i of column j, i <= j */
#pragma unroll
  for (int j = 0; j < N; ++j) {
    v[j] = zc.at(j, sz);
#pragma unroll
    for (int i = 0; i <= j; ++i) R[j][i] = a.baseR.at(j * N + i, t);
  }
#pragma unroll
  for (int i = 0; i < N; ++i) { /* R^T y = z */
    float sm = v[i];
#pragma unroll
    for (int k = 0; k < i; ++k) sm = fmaf(-R[i][k], v[k], sm);
    v[i] = sm * (1.0f / R[i][i]);
  }
#pragma unroll
  for (int j = N - 1; j >= 0; --j) { /* R d = y */
    const float xj = v[j] * (1.0f / R[j][j]);
    v[j] = xj;
#pragma unroll
    for (int i = 0; i < j; ++i) v[i] = fmaf(-xj, R[j][i], v[i]);
  }
  double* d = a.state + orig_step(a.track_start, a.level, t, 0) * N;
#pragma unroll
  for (int i = 0; i < N; ++i) d[i] = ukg_df::f32_to_f64(v[i]);
}

struct RegSolves {
  void (*solve)(Args<float, float>) = nullptr;
  void (*rt_even)(Args<float, float>, Soa<float>, Soa<float>) = nullptr;
  void (*rt_odd)(Args<float, float>, Soa<float>, Soa<float>, Soa<float>) = nullptr;
  void (*rt_base)(Args<float, float>, Soa<float>) = nullptr;
};
RegSolves reg_solves(int n)
{
  RegSolves r;
  if (n == 6)
    r.solve = solve_state_reg_kernel<6>, r.rt_even = rt_even_reg_kernel<6>, r.rt_odd = rt_odd_reg_kernel<6>,
    r.rt_base = rt_base_reg_kernel<6>;
  if (n == 4)
    r.solve = solve_state_reg_kernel<4>, r.rt_even = rt_even_reg_kernel<4>, r.rt_odd = rt_odd_reg_kernel<4>,
    r.rt_base = rt_base_reg_kernel<4>;
  return r;
}

__global__ void add_kernel(double* x, const double* d, int64_t count)
{
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < count) x[g] += d[g];
}

#include "oddeven_cta.cuh"

/* ---------------------------------------------------------------------------
 * host side: plan, workspace, launches
 * ------------------------------------------------------------------------ */
constexpr int kMaxLevels = 64;
constexpr int kResidBS = 128;

/* double-float weighing and residual kernels for (n, mx), or null (FP32
 * weighing and the FP64 residual) */
struct DfKernels {
  void (*weigh)(Args<float, float>, Eq<float>, RawDev, int64_t, int) = nullptr;
  void (*resid)(Args<float, float>, Eq<float>, Soa<float>, int64_t) = nullptr;
  int weigh_bs = kWeighBS;
};
DfKernels df_kernels(int n, int mmax, int weigh_bs = kWeighBS)
{
  DfKernels k;
  const int mx = mmax > n ? mmax : n;
  k.weigh_bs = weigh_bs;
#define UKG_DFW(N_)                                                                                                 \
  if (n == N_ && mx == N_)                                                                                          \
    k.weigh = weigh_bs == 64 ? weigh_df_kernel<N_, N_, 64>                                                          \
              : weigh_bs == 256 ? weigh_df_kernel<N_, N_, 256> : weigh_df_kernel<N_, N_, 128>;
  UKG_DFW(6) UKG_DFW(4)
#undef UKG_DFW
#define UKG_DF(N_, M_)                                                                                              \
  if (n == N_ && mmax == M_) k.resid = residual_df_kernel<N_, M_, kResidBS>;
  UKG_DF(6, 6) UKG_DF(6, 3) UKG_DF(6, 2) UKG_DF(4, 4) UKG_DF(4, 2)
#undef UKG_DF
  if (!k.weigh || !k.resid) k = DfKernels(); /* both or neither */
  return k;
}

/* Launch tuning (kalman_gpu_set_tuning): process-wide, read once at the
 * start of every call.  Defaults: a thread per item below 9 states, a thread
 * block per item from 9 on; four CTAs per SM; the block sizes the FP32
 * kernels were written for.                                                  */
kalman_gpu_tuning_t default_tuning() { return kalman_gpu_tuning_t{9, 4, kPairSsBP, kWeighBS}; }
std::mutex g_tune_mu;
kalman_gpu_tuning_t g_tune = default_tuning();
kalman_gpu_tuning_t tuning_now()
{
  std::lock_guard<std::mutex> lock(g_tune_mu);
  return g_tune;
}

struct LevelPlan {
  int64_t S = 0, E = 0, npairs = 0, nsolve = 0, ntail = 0;
  size_t off_L = 0, off_slot = 0, off_pair = 0, off_solve = 0, off_tail = 0; /* in int64 entries */
};

/* Everything the launches need besides the arrays: per-level track tables
 * (host copy, uploaded into the workspace) and the workspace layout.        */
struct Plan {
  int nlev = 0;
  bool fp32 = false, refine = false;
  LevelPlan lp[kMaxLevels];
  size_t tab_entries = 0, off_ts = 0;
  size_t o_tab = 0, o_flag = 0;
  size_t o_eq0 = 0, o_m0 = 0;      /* level 0 (T)                            */
  size_t o_eqA = 0, o_mA = 0;      /* odd levels (T)                         */
  size_t o_eqB = 0, o_mB = 0;      /* even levels >= 2 in FP32 mode          */
  size_t o_rec[kMaxLevels] = {0}, o_U[kMaxLevels] = {0};
  size_t o_z[kMaxLevels] = {0}, o_y[kMaxLevels] = {0}, o_baseR = 0, o_dx = 0, o_tmp = 0, o_rE = 0, o_rO = 0;
  size_t o_eq0lo = 0; /* low parts of the double-float level-0 equations */
  size_t bytes = 0;
  int64_t S0 = 0, S1 = 0, S2 = 0;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

/* Builds the plan.  Track t has k_t >> l steps at level l.  When tab is not
 * NULL the tables are written into it (tab_cap entries).  Returns the number
 * of table entries needed, or 0 if the recursion is deeper than kMaxLevels. */
size_t build_plan(const kalman_gpu_problem_t* p, bool want_cov, bool fp32, bool refine, Plan& P, int64_t* tab,
                  size_t tab_cap, bool cta)
{
  const int n = p->n, T = p->ntracks;
  const int mx = p->mmax > n ? p->mmax : n;
  const int64_t nn = (int64_t)n * n;
  P.fp32 = fp32;
  P.refine = refine;
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

  /* workspace layout */
  const size_t ts = fp32 ? sizeof(float) : sizeof(double);
  size_t bytes = 0;
  auto take = [&](size_t b) { size_t o = bytes; bytes = align_up(bytes + b, 256); return o; };
  P.o_tab = take(pos * sizeof(int64_t));
  P.o_flag = take(sizeof(int));
  const int64_t eqd = 2 * nn + n + (int64_t)mx * n + mx; /* equation entries per slot */
  P.S0 = std::max<int64_t>(P.lp[0].S, 1);
  P.S1 = std::max<int64_t>(P.nlev > 1 ? P.lp[1].S : 0, 1);
  P.S2 = std::max<int64_t>(P.nlev > 2 ? P.lp[2].S : 0, 1);
  P.o_eq0 = take((size_t)P.S0 * eqd * ts);
  P.o_m0 = take((size_t)P.S0 * sizeof(int32_t));
  P.o_eqA = take((size_t)P.S1 * eqd * ts);
  P.o_mA = take((size_t)P.S1 * sizeof(int32_t));
  if (fp32) {
    P.o_eqB = take((size_t)P.S2 * eqd * ts);
    P.o_mB = take((size_t)P.S2 * sizeof(int32_t));
  }
  for (int l = 0; l < P.nlev; ++l) {
    const int64_t E = std::max<int64_t>(P.lp[l].E, 1), S = std::max<int64_t>(P.lp[l].S, 1);
    P.o_rec[l] = take((size_t)E * (3 * nn + n) * ts);
    P.o_U[l] = (want_cov && l > 0) ? take((size_t)S * nn * ts) : 0;
    if (refine) {
      P.o_z[l] = take((size_t)S * n * sizeof(float));
      P.o_y[l] = take((size_t)E * n * sizeof(float));
    }
  }
  if (refine) {
    P.o_baseR = take((size_t)std::max(T, 1) * nn * sizeof(float));
    P.o_tmp = take((size_t)std::max(T, 1) * n * sizeof(float));
    P.o_dx = take((size_t)std::max<int64_t>(p->nsteps, 1) * n * sizeof(double));
    /* the per-thread path refines with the double-float residual where it is
       compiled (low parts of the level-0 equations); the CTA path, and the
       per-thread path elsewhere, with the FP64 residual (its two arrays) */
    if (!cta && df_kernels(n, p->mmax).resid) {
      P.o_eq0lo = take((size_t)P.S0 * eqd * sizeof(float));
    } else { /* the FP64 residual's intermediate arrays */
      P.o_rE = take((size_t)P.S0 * n * sizeof(double));
      P.o_rO = take((size_t)P.S0 * n * sizeof(double));
    }
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

template <typename T>
Eq<T> eq_at(char* B, size_t off, size_t off_m, int64_t stride, int n, int mx)
{
  const int64_t nn = (int64_t)n * n;
  T* e = (T*)(B + off);
  Eq<T> d;
  d.F = Soa<T>{e, stride};
  d.H = Soa<T>{e + nn * stride, stride};
  d.c = Soa<T>{e + 2 * nn * stride, stride};
  d.G = Soa<T>{e + (2 * nn + n) * stride, stride};
  d.o = Soa<T>{e + (2 * nn + n + (int64_t)mx * n) * stride, stride};
  d.m = (int32_t*)(B + off_m);
  return d;
}

/* The pair and solve kernels used for a state dimension: instantiations with
 * compile-time n, mx and block size for the common small shapes, the
 * runtime-dimension kernels otherwise.                                       */
template <typename T>
struct Kernels {
  void (*pair)(Args<T, T>, int) = nullptr;
  void (*solve)(Args<T, T>, int) = nullptr;
  void (*solve_cov)(Args<T, T>) = nullptr; /* register-tiled back-substitution with covariances */
  int bp = 0, bs = 0;     /* fixed block sizes of the specialised kernels (0: pick) */
  size_t pair_smem = 0;   /* dynamic shared memory of the pair kernel (0: per-thread workspace) */
};

template <typename T>
Kernels<T> choose_kernels(int n, int mx, int pair_bp = kPairSsBP)
{
  Kernels<T> k;
  if constexpr (sizeof(T) == sizeof(float)) {
    if (n == mx && (n == 6 || n == 4)) {
      if (n == 6)
        k.pair = pair_bp == 32 ? pair_ss_kernel<6, 32> : pair_bp == 128 ? pair_ss_kernel<6, 128> : pair_ss_kernel<6, 64>;
      else
        k.pair = pair_bp == 32 ? pair_ss_kernel<4, 32> : pair_bp == 128 ? pair_ss_kernel<4, 128> : pair_ss_kernel<4, 64>;
      k.solve = n == 6 ? solve_kernel<T, 6, 64> : solve_kernel<T, 4, 64>;
      k.bp = pair_bp;
      k.bs = 64;
      k.pair_smem = (size_t)pair_bp * sizeof(float) * (n == 6 ? PairSlice<6, 64>::width : PairSlice<4, 64>::width);
      return k;
    }
  }
  if (n == mx && n == 6) {
    k.pair = pair_kernel<T, T, 6, 6, 128>;
    k.solve = solve_kernel<T, 6, 64>;
    if constexpr (sizeof(T) != sizeof(float)) k.solve_cov = solve_cov_reg_kernel<T, 6, 64>;
    k.bp = 128;
    k.bs = 64;
  } else if (n == mx && n == 4) {
    k.pair = pair_kernel<T, T, 4, 4, 128>;
    k.solve = solve_kernel<T, 4, 64>;
    if constexpr (sizeof(T) != sizeof(float)) k.solve_cov = solve_cov_reg_kernel<T, 4, 64>;
    k.bp = 128;
    k.bs = 64;
  } else if (n == mx && n == 8) {
    k.pair = pair_kernel<T, T, 8, 8, 128>;
    k.solve = solve_kernel<T, 8, 64>; /* the register-tiled form spills at n = 8 */
    k.bp = 128;
    k.bs = 64;
  } else {
    k.pair = pair_kernel<T, T>;
    k.solve = solve_kernel<T>;
  }
  return k;
}

/* Uploads the tables, runs every kernel of the smoother on stream st using
 * the device workspace at B (at least P.bytes), waits, reports the flags.   */
/* copies the plan tables from page-locked, device-mapped host memory: a kernel
 * rather than a DMA, so the upload never queues behind large copies of the
 * caller's arrays on a copy engine (the host path overlaps those with
 * smoothing) */
__global__ void upload_tables_kernel(int64_t* __restrict__ dst, const int64_t* __restrict__ src, int64_t count)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

/* tab_dev: the device address of tab when tab is page-locked and mapped (the
 * tables are then uploaded by a kernel); null: tab is ordinary host memory
 * (uploaded with cudaMemcpyAsync) */
template <typename T>
int run_plan(uint32_t options, const kalman_gpu_problem_t* p, cudaStream_t st, const Plan& P, const int64_t* tab,
             char* B, const int64_t* tab_dev = nullptr, bool enqueue_only = false)
{
  const int n = p->n, T_ = p->ntracks, nlev = P.nlev;
  const int mx = p->mmax > n ? p->mmax : n;
  const bool want_cov = !(options & KALMAN_NO_COVARIANCE) && p->covariance;
  const int64_t nn = (int64_t)n * n;
  const LevelPlan* lp = P.lp;
  int64_t* dtab = (int64_t*)(B + P.o_tab);
  int* dflag = (int*)(B + P.o_flag);
  if (tab_dev)
    upload_tables_kernel<<<(unsigned)std::min<size_t>((P.tab_entries + 255) / 256, 1024), 256, 0, st>>>(
        dtab, tab_dev, (int64_t)P.tab_entries);
  else if (tab) /* null: the tables are already in the workspace */
    cudaMemcpyAsync(dtab, tab, P.tab_entries * sizeof(int64_t), cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(dflag, 0, sizeof(int), st);

  auto tables = [&](int l) {
    Tables d;
    memset(&d, 0, sizeof(d));
    if (l >= nlev) return d;
    const LevelPlan& L = lp[l];
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
  auto eq0 = [&]() { return eq_at<T>(B, P.o_eq0, P.o_m0, P.S0, n, mx); };
  auto eqT = [&](int l) { /* equations of level l >= 1 in the arithmetic type */
    if (l & 1) return eq_at<T>(B, P.o_eqA, P.o_mA, P.S1, n, mx);
    if (P.fp32) return eq_at<T>(B, P.o_eqB, P.o_mB, P.S2, n, mx);
    return eq_at<T>(B, P.o_eq0, P.o_m0, P.S0, n, mx); /* FP64: even levels reuse level 0's region */
  };
  auto rec = [&](int l) {
    Rec<T> r;
    memset(&r, 0, sizeof(r));
    if (l >= nlev) return r;
    const int64_t E = std::max<int64_t>(lp[l].E, 1);
    T* d = (T*)(B + P.o_rec[l]);
    r.R = Soa<T>{d, E};
    r.Ft = Soa<T>{d + nn * E, E};
    r.Y = Soa<T>{d + 2 * nn * E, E};
    r.rhs = Soa<T>{d + 3 * nn * E, E};
    if (want_cov && l > 0) r.U = Soa<T>{(T*)(B + P.o_U[l]), std::max<int64_t>(lp[l].S, 1)};
    return r;
  };

  /* ---- launch configuration ---- */
  const int rmax = 2 * mx;
  const size_t ts = sizeof(T);
  const size_t pt_weigh = (size_t)(mx * mx + 3 * mx) * ts;
  const int mmx = p->mmax;
  const int blk = std::max(std::max(n * n, mmx * mmx), std::max(mmx * n, 1));
  const size_t weigh_smem = 16 + (size_t)kWeighBS * blk * sizeof(double) + (size_t)kWeighBS * pt_weigh;
  int optin = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  /* bulk copies need 16-byte aligned sources */
  const uintptr_t align_bits = (uintptr_t)p->H | (uintptr_t)p->F | (uintptr_t)p->c | (uintptr_t)p->K |
                               (uintptr_t)p->G | (uintptr_t)p->o | (uintptr_t)p->C;
  const bool staged = sizeof(T) == sizeof(float) && weigh_smem <= (size_t)optin && (align_bits & 15) == 0;
  const size_t pt_pair = (size_t)(rmax * (n + 1) + n + rmax) * ts;
  const size_t pt_tail = (size_t)(mx * (n + 1) + 2 * n * (2 * n + 1) + 2 * n * (n + 1) + 2 * n + nn) * ts;
  const size_t pt_solve = (size_t)(4 * nn + 4 * n) * ts;
  const size_t pt_res = (size_t)(mx * mx + 3 * mx + n) * sizeof(double);
  int bw, bp, bt, bs, br;
  if (pick_block(pt_weigh, 128, &bw) || pick_block(pt_pair, 128, &bp) || pick_block(pt_tail, 32, &bt) ||
      pick_block(pt_solve, 64, &bs) || pick_block(pt_res, 128, &br))
    return ukg_set_error(KALMAN_GPU_EINVAL, "state dimension %d (observation rows %d) needs more shared memory per "
                         "thread than this build's odd-even kernels use", n, mx);
  const kalman_gpu_tuning_t tune = tuning_now();
  const Kernels<T> K = choose_kernels<T>(n, mx, tune.pair_block);
  if (K.bp) bp = K.bp;
  if (K.bs) bs = K.bs;
  ukg_allow_dynamic_smem((const void*)weigh_kernel<T>);
  if (staged)
    ukg_allow_dynamic_smem((const void*)weigh_staged_kernel<T>);
  const size_t pair_smem = K.pair_smem ? K.pair_smem : bp * pt_pair;
  ukg_allow_dynamic_smem((const void*)K.pair);
  ukg_allow_dynamic_smem((const void*)tail_kernel<T, T>);
  ukg_allow_dynamic_smem((const void*)K.solve);
  ukg_allow_dynamic_smem((const void*)residual_kernel);

  auto grid = [](int64_t items, int block) { return (unsigned)((items + block - 1) / block); };
  constexpr bool kDD = std::is_same<T, ukg_df::dd>::value; /* double-float: own kernel classes */
  const int kWeigh = kDD ? UKG_K_DF_WEIGH : UKG_K_WEIGH, kTail = kDD ? UKG_K_DF_TAIL : UKG_K_TAIL;
  const int kPair = P.fp32 ? UKG_K_PAIR32 : kDD ? UKG_K_DF_PAIR : UKG_K_PAIR;
  const int kSolve = P.fp32 ? UKG_K_SOLVE32 : kDD ? UKG_K_DF_SOLVE : UKG_K_SOLVE;
  Soa<T> baseR{P.refine ? (T*)(B + P.o_baseR) : nullptr, std::max(T_, 1)};

  /* double-float level-0 weighing and refinement residual where compiled */
  DfKernels DK;
  if constexpr (sizeof(T) == sizeof(float)) DK = df_kernels(n, p->mmax, tune.weigh_block);
  const bool use_df = DK.resid != nullptr && P.refine && P.o_eq0lo != 0;
  if (!use_df) DK = DfKernels();
  if (P.refine && !use_df && (P.o_rE == 0 || P.o_rO == 0)) /* offset 0 is the tables: never write there */
    return ukg_set_error(KALMAN_GPU_EINVAL, "internal: the workspace has no FP64 residual arrays");
  Eq<float> eq0lo;
  memset(&eq0lo, 0, sizeof(eq0lo));
  RegSolves RS; /* register-resident FP32 solves where compiled */
  if constexpr (sizeof(T) == sizeof(float)) RS = reg_solves(n);
  if (use_df) eq0lo = eq_at<float>(B, P.o_eq0lo, P.o_m0, P.S0, n, mx);

  /* ---- level 0: weighing ---- */
  const RawDev raw{p->H, p->F, p->c, p->K, p->G, p->o, p->C, p->K_type, p->C_type, p->obs_rows, p->mmax};
  {
    Args<T, T> w;
    memset(&w, 0, sizeof(w));
    w.ct = tables(0);
    w.ce = eq0();
    w.n = n;
    w.mx = mx;
    w.ntracks = T_;
    w.track_start = dtab + P.off_ts;
    w.flag = dflag;
    bool done = false;
    if constexpr (sizeof(T) == sizeof(float)) {
      const int wbs = DK.weigh_bs;
      const size_t smem_df = 16 + (size_t)wbs * blk * sizeof(double);
      if (DK.weigh && smem_df <= (size_t)optin) {
        ukg_allow_dynamic_smem((const void*)DK.weigh);
        UKG_LAUNCH(UKG_K_WEIGH, st,
                   (DK.weigh<<<grid(p->nsteps, wbs), wbs, smem_df, st>>>(w, eq0lo, raw, p->nsteps,
                                                                          (align_bits & 15) == 0)));
        done = true;
      }
    }
    if (done) {
    } else if (staged)
      UKG_LAUNCH(UKG_K_WEIGH, st,
                 (weigh_staged_kernel<T><<<grid(p->nsteps, kWeighBS), kWeighBS, weigh_smem, st>>>(w, raw, p->nsteps,
                                                                                                   blk)));
    else
      UKG_LAUNCH(kWeigh, st, (weigh_kernel<T><<<grid(p->nsteps, bw), bw, bw * pt_weigh, st>>>(w, raw, p->nsteps)));
  }
  auto common = [&](auto& a, int l) {
    a.ct = tables(l);
    a.nt = tables(l + 1);
    a.cr = rec(l);
    a.nr = rec(l + 1);
    a.n = n;
    a.mx = mx;
    a.level = l;
    a.ntracks = T_;
    a.track_start = dtab + P.off_ts;
    a.state = p->state;
    a.cov = want_cov ? p->covariance : nullptr;
    a.flag = dflag;
    a.baseR = baseR;
  };
  /* ---- forward elimination ---- */
  for (int l = 0; l < nlev; ++l) {
    Args<T, T> a;
    memset(&a, 0, sizeof(a));
    common(a, l);
    a.ce = l == 0 ? eq0() : eqT(l);
    if (l + 1 < nlev) a.ne = eqT(l + 1);
    if (lp[l].npairs > 0)
      UKG_LAUNCH(kPair, st, (K.pair<<<grid(lp[l].npairs, bp), bp, pair_smem, st>>>(a, rmax)));
    if (lp[l].ntail > 0)
    {
      bool done = false;
      if constexpr (sizeof(T) == sizeof(float)) {
        if (!want_cov && n == mx && (n == 6 || n == 4)) {
          auto tk = n == 6 ? tail_reg_kernel<6> : tail_reg_kernel<4>;
          UKG_LAUNCH(UKG_K_TAIL, st, (tk<<<grid(lp[l].ntail, kTailBS), kTailBS, 0, st>>>(a)));
          done = true;
        }
      }
      if (!done)
        UKG_LAUNCH(kTail, st, (tail_kernel<T, T><<<grid(lp[l].ntail, bt), bt, bt * pt_tail, st>>>(a)));
    }
  }
  /* ---- back-substitution ---- */
  for (int l = nlev - 2; l >= 0; --l) {
    Args<T, T> a;
    memset(&a, 0, sizeof(a));
    common(a, l);
    if (lp[l].nsolve == 0) continue;
    if constexpr (sizeof(T) == sizeof(float)) {
      if (RS.solve && !want_cov) {
        UKG_LAUNCH(kSolve, st, (RS.solve<<<grid(lp[l].nsolve, 128), 128, 0, st>>>(a)));
        continue;
      }
    }
    if (want_cov && K.solve_cov) {
      const size_t smem_cov = (size_t)64 * 2 * nn * ts;
      ukg_allow_dynamic_smem((const void*)K.solve_cov);
      UKG_LAUNCH(kSolve, st, (K.solve_cov<<<grid(lp[l].nsolve, 64), 64, smem_cov, st>>>(a)));
      continue;
    }
    UKG_LAUNCH(kSolve, st, (K.solve<<<grid(lp[l].nsolve, bs), bs, bs * pt_solve, st>>>(a, want_cov ? 1 : 0)));
  }
  /* ---- refinement sweeps (FP32 factors only) ---- */
  if constexpr (sizeof(T) == sizeof(float)) {
    const int requested = (int)((options >> 21) & 3u);
    const int sweeps = P.refine ? (requested ? requested : 2) : 0;
    double* dx = P.refine ? (double*)(B + P.o_dx) : nullptr;
    for (int sw = 0; sw < sweeps; ++sw) {
      {
        Args<float, float> r;
        memset(&r, 0, sizeof(r));
        common(r, 0);
        r.ce = eq0();
        Soa<float> z0{(float*)(B + P.o_z[0]), std::max<int64_t>(lp[0].S, 1)};
        if (DK.resid) {
          UKG_LAUNCH(UKG_K_RESID, st,
                     (DK.resid<<<grid(p->nsteps, kResidBS - 1), kResidBS, 0, st>>>(r, eq0lo, z0, p->nsteps)));
        } else {
          Soa<double> wE{(double*)(B + P.o_rE), P.S0}, zp{(double*)(B + P.o_rO), P.S0};
          UKG_LAUNCH(UKG_K_RESID, st,
                     (residual_kernel<<<grid(p->nsteps, br), br, br * pt_res, st>>>(r, raw, wE, zp, p->nsteps)));
          UKG_LAUNCH(UKG_K_RESID, st,
                     (atr_kernel<<<grid(p->nsteps, 128), 128, 0, st>>>(r, raw, wE, zp, z0, p->nsteps)));
        }
      }
      for (int l = 0; l < nlev; ++l) {
        Args<float, float> a;
        memset(&a, 0, sizeof(a));
        common(a, l);
        a.state = dx;
        a.cov = nullptr;
        Soa<float> zc{(float*)(B + P.o_z[l]), std::max<int64_t>(lp[l].S, 1)};
        Soa<float> yc{(float*)(B + P.o_y[l]), std::max<int64_t>(lp[l].E, 1)};
        if (lp[l].nsolve > 0) {
          if (RS.rt_even)
            UKG_LAUNCH(UKG_K_RT, st, (RS.rt_even<<<grid(lp[l].nsolve, 128), 128, 0, st>>>(a, zc, yc)));
          else
            UKG_LAUNCH(UKG_K_RT, st, (rt_even_kernel<<<grid(lp[l].nsolve, 128), 128, 0, st>>>(a, zc, yc)));
        }
        if (lp[l].npairs > 0 && l + 1 < nlev) {
          Soa<float> zn{(float*)(B + P.o_z[l + 1]), std::max<int64_t>(lp[l + 1].S, 1)};
          if (RS.rt_odd)
            UKG_LAUNCH(UKG_K_RT, st, (RS.rt_odd<<<grid(lp[l].npairs, 128), 128, 0, st>>>(a, zc, yc, zn)));
          else
            UKG_LAUNCH(UKG_K_RT, st, (rt_odd_kernel<<<grid(lp[l].npairs, 128), 128, 0, st>>>(a, zc, yc, zn)));
        }
        if (lp[l].ntail > 0) {
          Soa<float> tmp{(float*)(B + P.o_tmp), std::max(T_, 1)};
          if (RS.rt_base)
            UKG_LAUNCH(UKG_K_RT, st, (RS.rt_base<<<grid(lp[l].ntail, 128), 128, 0, st>>>(a, zc)));
          else
            UKG_LAUNCH(UKG_K_RT, st, (rt_base_kernel<<<grid(lp[l].ntail, 128), 128, 0, st>>>(a, zc, tmp)));
        }
      }
      for (int l = nlev - 2; l >= 0; --l) {
        Args<float, float> a;
        memset(&a, 0, sizeof(a));
        common(a, l);
        a.state = dx;
        a.cov = nullptr;
        a.yrhs = Soa<float>{(float*)(B + P.o_y[l]), std::max<int64_t>(lp[l].E, 1)};
        if (lp[l].nsolve == 0) continue;
        if (RS.solve)
          UKG_LAUNCH(UKG_K_RSOLVE, st, (RS.solve<<<grid(lp[l].nsolve, 128), 128, 0, st>>>(a)));
        else
          UKG_LAUNCH(UKG_K_RSOLVE, st, (K.solve<<<grid(lp[l].nsolve, bs), bs, bs * pt_solve, st>>>(a, 0)));
      }
      const int64_t cnt = p->nsteps * n;
      UKG_LAUNCH(UKG_K_REFINE, st, (add_kernel<<<grid(cnt, 256), 256, 0, st>>>(p->state, dx, cnt)));
    }
  }
  if (enqueue_only) return 0;
  int hflag = 0;
  cudaMemcpyAsync(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return ukg_set_error(KALMAN_GPU_ECUDA, "odd-even smoother: %s", cudaGetErrorString(e));
  ukg_prof_collect();
  if (hflag & 8) return ukg_set_error(KALMAN_GPU_ECUDA, "a bulk copy into shared memory did not complete in time");
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

/* page-locked, device-mapped host buffer for the plan tables (one per host
 * thread; every call waits for its kernels, so the next call may refill it) */
struct MappedTables {
  int64_t* host = nullptr;
  int64_t* dev = nullptr;
  size_t entries = 0;
};
thread_local MappedTables tl_mtab;

int ensure_mapped_tables(size_t entries)
{
  MappedTables& m = tl_mtab;
  if (m.entries < entries) {
    if (m.host) cudaFreeHost(m.host);
    m = MappedTables();
    const size_t want = std::max<size_t>(entries, 1 << 16);
    cudaError_t e = cudaHostAlloc((void**)&m.host, want * sizeof(int64_t), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&m.dev, m.host, 0);
    if (e != cudaSuccess) {
      cudaGetLastError();
      if (m.host) cudaFreeHost(m.host);
      m = MappedTables();
      return ukg_set_error(KALMAN_GPU_ENOMEM, "page-locked plan tables (%zu entries): %s", entries,
                           cudaGetErrorString(e));
    }
    m.entries = want;
  }
  return 0;
}

/* The workspace grows by stream-ordered allocation on the call's stream
 * (cudaFreeAsync / cudaMallocAsync): cudaFree and cudaMalloc synchronize the
 * whole device, which would stall the calls other host threads have running
 * on their own streams.  Every call synchronizes its stream before returning,
 * so the next call, on any stream, finds the allocation complete.           */
int ensure_workspace(size_t bytes, void** out, cudaStream_t st)
{
  int dev = 0;
  cudaGetDevice(&dev);
  Workspace& w = tl_ws;
  if (w.dev && (w.dev_bytes < bytes || w.device != dev)) {
    if (w.device == dev) cudaFreeAsync(w.dev, st);
    else cudaFree(w.dev);
    w.dev = nullptr;
    w.dev_bytes = 0;
  }
  if (!w.dev) {
    size_t want = ukg_with_slack(bytes);
    const cudaError_t e = (cudaError_t)ukg_malloc_async(&w.dev, want, st);
    if (e != cudaSuccess) {
      w.dev = nullptr;
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

extern "C" int64_t ukg_oddeven_workspace_held(void) { return (int64_t)tl_ws.dev_bytes; }

extern "C" void ukg_release_oddeven_workspace(void)
{
  if (tl_ws.dev) cudaFree(tl_ws.dev);
  tl_ws = Workspace();
  if (tl_mtab.host) cudaFreeHost(tl_mtab.host);
  tl_mtab = MappedTables();
}

/* ---------------------------------------------------------------------------
 * larger state dimensions: one CTA per item (oddeven_cta.cuh), FP64
 * ------------------------------------------------------------------------ */
constexpr int kCtaMaxN = 128;
static_assert(kCtaMaxN <= 32 * ctak::kRtQ && kCtaMaxN <= cta::kMaxCov && 2 * kCtaMaxN <= cta::kMaxPanelRows,
              "CTA kernels: per-lane state registers, covariance and panel buffers");

int64_t cta_scratch_per_cta(int n, int mmax)
{
  const int64_t rmax = std::max(n, mmax);
  const int64_t weigh = rmax * rmax + rmax * (2 * n + 1) + rmax * cta::NT;
  const int64_t tail = 7 * (int64_t)n * n + 5 * n + (int64_t)std::max(n, mmax) * (n + 1) + n;
  const int64_t mx = rmax; /* max(n, mmax) */
  const int64_t pair = std::max(std::max(2 * (int64_t)n * (3 * n + 1), (mx + n) * (2 * n + 1)), 2 * mx * (n + 1));
  const int64_t solve = 7 * (int64_t)n * n + n;
  return std::max(std::max(weigh, tail), std::max(pair, solve)) + 32;
}

/* thread blocks of the CTA kernels' persistent grid: per_sm on every SM */
int cta_count(int per_sm)
{
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::max(sms, 1) * std::max(per_sm, 1);
}

/* thread per item below tune.cta_min_n states (and up to 8 observation
 * rows), one thread block per item from there on                           */
bool use_cta(const kalman_gpu_problem_t* p, const kalman_gpu_tuning_t& tune)
{
  const int mxp = p->mmax > p->n ? p->mmax : p->n;
  return p->n >= tune.cta_min_n || mxp > 8;
}

template <typename T>
int run_plan_cta(uint32_t options, const kalman_gpu_problem_t* p, cudaStream_t st, const Plan& P,
                 const int64_t* tab_dev, char* B, void* scratch, int64_t per_cta, int ncta,
                 bool enqueue_only = false)
{
  const int n = p->n, T_ = p->ntracks, nlev = P.nlev;
  const int mx = p->mmax > n ? p->mmax : n;
  const bool want_cov = !(options & KALMAN_NO_COVARIANCE) && p->covariance;
  const int64_t nn = (int64_t)n * n;
  const LevelPlan* lp = P.lp;
  int64_t* dtab = (int64_t*)(B + P.o_tab);
  int* dflag = (int*)(B + P.o_flag);
  if (P.refine && (P.o_rE == 0 || P.o_rO == 0)) /* offset 0 is the tables: never write there */
    return ukg_set_error(KALMAN_GPU_EINVAL, "internal: the workspace has no FP64 residual arrays");
  if (tab_dev) /* null: the tables are already in the workspace */
    upload_tables_kernel<<<(unsigned)std::min<size_t>((P.tab_entries + 255) / 256, 1024), 256, 0, st>>>(
        dtab, tab_dev, (int64_t)P.tab_entries);
  cudaMemsetAsync(dflag, 0, sizeof(int), st);
  auto tables = [&](int l) {
    Tables d;
    memset(&d, 0, sizeof(d));
    if (l >= nlev) return d;
    const LevelPlan& L = lp[l];
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
  auto eqa = [&](size_t off, size_t off_m, int64_t S) {
    T* e = (T*)(B + off);
    ctak::EqA<T> d;
    d.F = {e, nn};
    d.H = {e + nn * S, nn};
    d.c = {e + 2 * nn * S, n};
    d.G = {e + (2 * nn + n) * S, (int64_t)mx * n};
    d.o = {e + (2 * nn + n + (int64_t)mx * n) * S, mx};
    d.m = (int32_t*)(B + off_m);
    return d;
  };
  auto eq_level = [&](int l) { /* level 0; odd levels; even levels >= 2 (their own region in FP32) */
    if (l == 0) return eqa(P.o_eq0, P.o_m0, P.S0);
    if (l & 1) return eqa(P.o_eqA, P.o_mA, P.S1);
    return P.fp32 ? eqa(P.o_eqB, P.o_mB, P.S2) : eqa(P.o_eq0, P.o_m0, P.S0);
  };
  auto rec = [&](int l) {
    ctak::RecA<T> r;
    memset(&r, 0, sizeof(r));
    if (l >= nlev) return r;
    const int64_t E = std::max<int64_t>(lp[l].E, 1);
    T* d = (T*)(B + P.o_rec[l]);
    r.R = {d, nn};
    r.Ft = {d + nn * E, nn};
    r.Y = {d + 2 * nn * E, nn};
    r.rhs = {d + 3 * nn * E, n};
    if (want_cov && l > 0) r.U = {(T*)(B + P.o_U[l]), nn};
    return r;
  };
  Soa<T> baseR{P.refine ? (T*)(B + P.o_baseR) : nullptr, std::max(T_, 1)};
  auto common = [&](ctak::CArgs<T>& a, int l) {
    memset(&a, 0, sizeof(a));
    a.ct = tables(l);
    a.nt = tables(l + 1);
    a.cr = rec(l);
    a.nr = rec(l + 1);
    a.n = n;
    a.mx = mx;
    a.level = l;
    a.ntracks = T_;
    a.track_start = dtab + P.off_ts;
    a.state = p->state;
    a.cov = want_cov ? p->covariance : nullptr;
    a.flag = dflag;
    a.scratch = (T*)scratch;
    a.scratch_per_cta = per_cta * (int64_t)(sizeof(double) / sizeof(T));
    a.baseR = baseR;
  };
  auto grid = [&](int64_t items) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(items, ncta)); };
  constexpr bool kDD = std::is_same<T, ukg_df::dd>::value; /* double-float: own kernel classes */
  const int kWeigh = kDD ? UKG_K_DF_WEIGH : UKG_K_WEIGH, kTail = kDD ? UKG_K_DF_TAIL : UKG_K_TAIL;
  const ctak::RawA raw{p->H, p->F, p->c, p->K, p->G, p->o, p->C, p->K_type, p->C_type, p->obs_rows, p->mmax};
  {
    ctak::CArgs<T> a;
    common(a, 0);
    a.ce = eq_level(0);
    /* the weighing needs less scratch than the pair kernel: where two of its
       CTAs fit one slot, twice as many run (more warps on its latency) */
    const int64_t rmax = std::max(n, p->mmax);
    const int64_t wneed = rmax * rmax + rmax * (2 * n + 1) + rmax * cta::NT;
    if (2 * wneed <= a.scratch_per_cta) {
      a.scratch_per_cta /= 2;
      const unsigned g2 = (unsigned)std::max<int64_t>(1, std::min<int64_t>(p->nsteps, 2 * (int64_t)ncta));
      UKG_LAUNCH(kWeigh, st, (ctak::weigh_cta<T><<<g2, cta::NT, 0, st>>>(a, raw, p->nsteps)));
    } else {
      UKG_LAUNCH(kWeigh, st, (ctak::weigh_cta<T><<<grid(p->nsteps), cta::NT, 0, st>>>(a, raw, p->nsteps)));
    }
  }
  const int kPair = P.fp32 ? UKG_K_PAIR32 : kDD ? UKG_K_DF_PAIR : UKG_K_PAIR;
  const int kSolve = P.fp32 ? UKG_K_SOLVE32 : kDD ? UKG_K_DF_SOLVE : UKG_K_SOLVE;
  for (int l = 0; l < nlev; ++l) {
    ctak::CArgs<T> a;
    common(a, l);
    a.ce = eq_level(l);
    if (l + 1 < nlev) a.ne = eq_level(l + 1);
    if (lp[l].npairs > 0) {
      if (n >= cta::kBlockedMinN)
        UKG_LAUNCH(kPair, st, (ctak::pair_cta<T, true><<<grid(lp[l].npairs), cta::NT, 0, st>>>(a)));
      else
        UKG_LAUNCH(kPair, st, (ctak::pair_cta<T, false><<<grid(lp[l].npairs), cta::NT, 0, st>>>(a)));
    }
    if (lp[l].ntail > 0) {
      if (n >= cta::kBlockedMinN)
        UKG_LAUNCH(kTail, st, (ctak::tail_cta<T, true><<<grid(lp[l].ntail), cta::NT, 0, st>>>(a)));
      else
        UKG_LAUNCH(kTail, st, (ctak::tail_cta<T, false><<<grid(lp[l].ntail), cta::NT, 0, st>>>(a)));
    }
  }
  for (int l = nlev - 2; l >= 0; --l) {
    ctak::CArgs<T> a;
    common(a, l);
    if (lp[l].nsolve > 0)
      UKG_LAUNCH(kSolve, st, (ctak::solve_cta<T><<<grid(lp[l].nsolve), cta::NT, 0, st>>>(a, want_cov ? 1 : 0)));
  }
  /* ---- refinement sweeps (FP32 factors): FP64 residual, transpose solves, solves ---- */
  if constexpr (sizeof(T) == sizeof(float)) {
    const int requested = (int)((options >> 21) & 3u);
    const int sweeps = P.refine ? (requested ? requested : 2) : 0;
    double* dx = P.refine ? (double*)(B + P.o_dx) : nullptr;
    auto pargs = [&](int l) { /* for rt_base_kernel and atr_kernel (no level arrays) */
      Args<float, float> a;
      memset(&a, 0, sizeof(a));
      a.ct = tables(l);
      a.nt = tables(l + 1);
      a.n = n;
      a.mx = mx;
      a.level = l;
      a.ntracks = T_;
      a.track_start = dtab + P.off_ts;
      a.state = dx;
      a.flag = dflag;
      a.baseR = baseR;
      return a;
    };
    const RawDev rawd{p->H, p->F, p->c, p->K, p->G, p->o, p->C, p->K_type, p->C_type, p->obs_rows, p->mmax};
    /* the residual's scratch (a factor and four vectors, FP64) is small: two
       of its CTAs per slot where they fit */
    const int64_t rr = std::max(n, p->mmax), rneed = rr * rr + 4 * rr;
    const bool r2 = 2 * rneed <= per_cta;
    const int64_t rper = r2 ? per_cta / 2 : per_cta;
    const unsigned rgrid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(p->nsteps, (r2 ? 2 : 1) * (int64_t)ncta));
    for (int sw = 0; sw < sweeps; ++sw) {
      Soa<double> wE{(double*)(B + P.o_rE), P.S0}, zp{(double*)(B + P.o_rO), P.S0};
      Soa<float> z0{(float*)(B + P.o_z[0]), std::max<int64_t>(lp[0].S, 1)};
      {
        ctak::CArgs<float> a;
        common(a, 0);
        a.ce = eq_level(0);
        UKG_LAUNCH(UKG_K_RESID, st,
                   (ctak::residual_cta<<<rgrid, cta::NT, 0, st>>>(a, raw, wE, zp, (double*)scratch, rper,
                                                                           p->nsteps)));
        Args<float, float> r = pargs(0);
        r.state = p->state;
        UKG_LAUNCH(UKG_K_RESID, st,
                   (atr_kernel<<<(unsigned)((p->nsteps + 127) / 128), 128, 0, st>>>(r, rawd, wE, zp, z0, p->nsteps)));
      }
      for (int l = 0; l < nlev; ++l) {
        Args<float, float> a = pargs(l);
        ctak::CArgs<float> ca;
        common(ca, l);
        Soa<float> zc{(float*)(B + P.o_z[l]), std::max<int64_t>(lp[l].S, 1)};
        Soa<float> yc{(float*)(B + P.o_y[l]), std::max<int64_t>(lp[l].E, 1)};
        if (lp[l].nsolve > 0)
          UKG_LAUNCH(UKG_K_RT, st,
                     (ctak::rt_even_aos<<<(unsigned)((lp[l].nsolve * 32 + 127) / 128), 128, 0, st>>>(ca, zc, yc)));
        if (lp[l].npairs > 0 && l + 1 < nlev) {
          Soa<float> zn{(float*)(B + P.o_z[l + 1]), std::max<int64_t>(lp[l + 1].S, 1)};
          UKG_LAUNCH(UKG_K_RT, st,
                     (ctak::rt_odd_aos<<<(unsigned)((lp[l].npairs * 32 + 127) / 128), 128, 0, st>>>(ca, zc, yc, zn)));
        }
        if (lp[l].ntail > 0) {
          Soa<float> tmp{(float*)(B + P.o_tmp), std::max(T_, 1)};
          UKG_LAUNCH(UKG_K_RT, st, (rt_base_kernel<<<(unsigned)((lp[l].ntail + 127) / 128), 128, 0, st>>>(a, zc, tmp)));
        }
      }
      for (int l = nlev - 2; l >= 0; --l) {
        ctak::CArgs<float> a;
        common(a, l);
        a.state = dx;
        a.cov = nullptr;
        a.yrhs = Soa<float>{(float*)(B + P.o_y[l]), std::max<int64_t>(lp[l].E, 1)};
        if (lp[l].nsolve > 0)
          UKG_LAUNCH(UKG_K_RSOLVE, st, (ctak::solve_cta<float><<<grid(lp[l].nsolve), cta::NT, 0, st>>>(a, 0)));
      }
      const int64_t cnt = p->nsteps * n;
      UKG_LAUNCH(UKG_K_REFINE, st, (add_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(p->state, dx, cnt)));
    }
  }
  if (enqueue_only) return 0;
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

extern "C" int ukg_oddeven_device(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream)
{
  if (p->nsteps == 0) return 0;
  const bool want_cov = !(options & KALMAN_NO_COVARIANCE) && p->covariance;
  const int mxp = p->mmax > p->n ? p->mmax : p->n;
  const kalman_gpu_tuning_t tune = tuning_now();
  if (use_cta(p, tune)) { /* larger shapes: CTA kernels (FP64, or FP32 + refinement) */
    if (mxp > kCtaMaxN)
      return ukg_set_error(KALMAN_GPU_EINVAL, "state dimension %d (observation rows %d) above this build's limit %d",
                           p->n, p->mmax, kCtaMaxN);
    const bool dd = (options & KALMAN_GPU_FP32_REFINE) && want_cov; /* double-float with covariances */
    const bool f32 = (options & KALMAN_GPU_FP32_REFINE) && !dd;
    Plan P;
    const size_t need = build_plan(p, want_cov, f32, f32, P, nullptr, 0, true);
    if (need == 0) return ukg_set_error(KALMAN_GPU_EINVAL, "tracks longer than 2^%d steps", kMaxLevels - 1);
    if (int e = ensure_mapped_tables(need)) return e;
    build_plan(p, want_cov, f32, f32, P, tl_mtab.host, need, true);
    const int ncta = cta_count(tune.ctas_per_sm);
    const int64_t per = cta_scratch_per_cta(p->n, p->mmax);
    const size_t scratch_off = align_up(P.bytes, 256);
    void* base = nullptr;
    if (int e = ensure_workspace(scratch_off + (size_t)ncta * per * sizeof(double), &base, (cudaStream_t)cuda_stream))
      return e;
    if (f32)
      return run_plan_cta<float>(options, p, (cudaStream_t)cuda_stream, P, tl_mtab.dev, (char*)base,
                                 (char*)base + scratch_off, per, ncta);
    if (dd)
      return run_plan_cta<ukg_df::dd>(options, p, (cudaStream_t)cuda_stream, P, tl_mtab.dev, (char*)base,
                                      (char*)base + scratch_off, per, ncta);
    return run_plan_cta<double>(options, p, (cudaStream_t)cuda_stream, P, tl_mtab.dev, (char*)base,
                                (char*)base + scratch_off, per, ncta);
  }
  const bool dd = (options & KALMAN_GPU_FP32_REFINE) && want_cov; /* double-float with covariances */
  const bool fp32 = (options & KALMAN_GPU_FP32_REFINE) && !dd;
  Plan P;
  const size_t need = build_plan(p, want_cov, fp32, fp32, P, nullptr, 0, false);
  if (need == 0) return ukg_set_error(KALMAN_GPU_EINVAL, "tracks longer than 2^%d steps", kMaxLevels - 1);
  if (int e = ensure_mapped_tables(need)) return e;
  int64_t* tab = tl_mtab.host;
  build_plan(p, want_cov, fp32, fp32, P, tab, need, false);
  void* base = nullptr;
  if (int e = ensure_workspace(P.bytes, &base, (cudaStream_t)cuda_stream)) return e;
  if (fp32) return run_plan<float>(options, p, (cudaStream_t)cuda_stream, P, tab, (char*)base, tl_mtab.dev);
  if (dd) return run_plan<ukg_df::dd>(options, p, (cudaStream_t)cuda_stream, P, tab, (char*)base, tl_mtab.dev);
  return run_plan<double>(options, p, (cudaStream_t)cuda_stream, P, tab, (char*)base, tl_mtab.dev);
}

/* Device bytes the ordinary odd-even entry point caches for problem p under
 * these options (the workspace of ukg_oddeven_device, with its 1/8 slack):
 * a caller that budgets HBM (the serving loop) reads the library's own
 * figure instead of modelling it.  -1 on a malformed problem.              */
extern "C" int kalman_gpu_check_bounded_wait(void* cuda_stream)
{
  ukg_clear_error();
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return ukg_set_error(KALMAN_GPU_ENODEV, "no CUDA device");
  }
  cudaStream_t st = (cudaStream_t)cuda_stream;
  int* dflag = nullptr;
  if (ukg_malloc_async((void**)&dflag, sizeof(int), st) != 0)
    return ukg_set_error(KALMAN_GPU_ENOMEM, "allocating the check's flag failed");
  int hflag = 0;
  cudaMemsetAsync(dflag, 0, sizeof(int), st);
  bounded_wait_check_kernel<<<1, 32, 0, st>>>(dflag);
  cudaMemcpyAsync(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(dflag, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return ukg_set_error(KALMAN_GPU_ECUDA, "bounded-wait check: %s", cudaGetErrorString(e));
  if (hflag & 8) return ukg_set_error(KALMAN_GPU_ECUDA, "a bulk copy into shared memory did not complete in time");
  return 0;
}

extern "C" int64_t kalman_gpu_oddeven_workspace_bytes(uint32_t options, const kalman_gpu_problem_t* p)
{
  ukg_clear_error();
  if (ukg_validate_problem(p, 0)) return -1;
  if (p->nsteps == 0) return 0;
  const bool want_cov = !(options & KALMAN_NO_COVARIANCE) && p->covariance;
  const bool f32 = (options & KALMAN_GPU_FP32_REFINE) && !want_cov; /* with covariances: double-float, 8 bytes */
  Plan P;
  const kalman_gpu_tuning_t tune = tuning_now();
  const bool cta = use_cta(p, tune);
  if (build_plan(p, want_cov, f32, f32, P, nullptr, 0, cta) == 0) {
    ukg_set_error(KALMAN_GPU_EINVAL, "tracks longer than 2^%d steps", kMaxLevels - 1);
    return -1;
  }
  size_t bytes = P.bytes;
  if (cta)
    bytes = align_up(P.bytes, 256) +
            (size_t)cta_count(tune.ctas_per_sm) * cta_scratch_per_cta(p->n, p->mmax) * sizeof(double);
  return (int64_t)ukg_with_slack(bytes);
}

extern "C" int kalman_gpu_set_tuning(const kalman_gpu_tuning_t* t)
{
  ukg_clear_error();
  kalman_gpu_tuning_t v = t ? *t : default_tuning();
  if (v.cta_min_n < 1 || v.cta_min_n > kCtaMaxN + 1)
    return ukg_set_error(KALMAN_GPU_EINVAL, "cta_min_n %d outside 1..%d", v.cta_min_n, kCtaMaxN + 1);
  if (v.ctas_per_sm < 1 || v.ctas_per_sm > 16)
    return ukg_set_error(KALMAN_GPU_EINVAL, "ctas_per_sm %d outside 1..16", v.ctas_per_sm);
  if (v.pair_block != 32 && v.pair_block != 64 && v.pair_block != 128)
    return ukg_set_error(KALMAN_GPU_EINVAL, "pair_block %d is not 32, 64 or 128", v.pair_block);
  if (v.weigh_block != 64 && v.weigh_block != 128 && v.weigh_block != 256)
    return ukg_set_error(KALMAN_GPU_EINVAL, "weigh_block %d is not 64, 128 or 256", v.weigh_block);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune = v;
  return 0;
}

extern "C" void kalman_gpu_get_tuning(kalman_gpu_tuning_t* t)
{
  if (t) *t = tuning_now();
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
  if (options & KALMAN_GPU_FP32_REFINE)
    return ukg_set_error(KALMAN_GPU_EINVAL, "the allocation-free entry point runs the plain FP64 smoother only "
                         "(KALMAN_GPU_FP32_REFINE is not accepted)");
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
  const size_t need = build_plan(p, want_cov, false, false, P, nullptr, 0, false);
  if (need == 0 || need > kNoallocTabEntries)
    return ukg_set_error(KALMAN_GPU_EINVAL, "the allocation-free entry point plans at most %zu table entries "
                         "(this problem needs %zu: too many tracks)", kNoallocTabEntries, need);
  build_plan(p, want_cov, false, false, P, g_noalloc_tab, kNoallocTabEntries, false);
  if (P.bytes > (size_t)KALMAN_GPU_NOALLOC_SCRATCH_BYTES)
    return ukg_set_error(KALMAN_GPU_EINVAL, "this problem needs %zu bytes of scratch; the allocation-free entry "
                         "point has %zu (use kalman_gpu_smooth_oddeven_packed)", P.bytes,
                         (size_t)KALMAN_GPU_NOALLOC_SCRATCH_BYTES);
  const int prof = ukg_prof_pause(); /* profiling would create CUDA events */
  /* the per-thread kernels at every shape, also n >= 9 or mmax > 8 where the
     ordinary entry point switches to CTA kernels (their per-CTA panels are
     not part of this fixed scratch) */
  const int status = run_plan<double>(options, p, (cudaStream_t)cuda_stream, P, g_noalloc_tab,
                                      (char*)g_noalloc_addr[dev]);
  ukg_prof_resume(prof);
  return status;
}

/* ---------------------------------------------------------------------------
 * Prepared plans replayed as CUDA graphs (kalman_gpu_plan_*).
 *
 * For callers that smooth problems of one fixed shape again and again -- a
 * tracker re-smoothing a sliding window of the same length every frame, a
 * service whose requests come in a few fixed sizes -- every host step of a
 * call (plan tables, workspace, launch configuration, a hundred-odd kernel
 * launches) is done once: the tables are uploaded to a workspace the plan
 * owns and the whole launch sequence is captured into a CUDA graph; each
 * execution is one graph launch on the caller's stream, asynchronous, with
 * the current contents of the caller's device arrays.  The reference has no
 * counterpart (it rebuilds its step structures on every call).
 * ------------------------------------------------------------------------ */
struct kalman_gpu_plan {
  int device = -1;
  bool cta = false;
  void* work = nullptr;
  int* dflag = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t last = nullptr;
  bool launched = false;
};

extern "C" void kalman_gpu_plan_destroy(kalman_gpu_plan_t* pl)
{
  if (!pl) return;
  if (pl->launched) cudaStreamSynchronize(pl->last);
  if (pl->exec) cudaGraphExecDestroy(pl->exec);
  if (pl->graph) cudaGraphDestroy(pl->graph);
  if (pl->work) cudaFree(pl->work);
  delete pl;
}

extern "C" kalman_gpu_plan_t* kalman_gpu_plan_create(uint32_t options, const kalman_gpu_problem_t* p)
{
  ukg_clear_error();
  if (ukg_validate_problem(p, 0)) return nullptr;
  if (p->location != KALMAN_GPU_DEVICE) {
    ukg_set_error(KALMAN_GPU_EINVAL, "a plan takes device arrays (it is replayed on their current contents)");
    return nullptr;
  }
  if (p->nsteps == 0) {
    ukg_set_error(KALMAN_GPU_EINVAL, "a plan needs at least one step");
    return nullptr;
  }
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    ukg_set_error(KALMAN_GPU_ENODEV, "no CUDA device is available");
    return nullptr;
  }
  const bool want_cov = !(options & KALMAN_NO_COVARIANCE) && p->covariance;
  const int mxp = p->mmax > p->n ? p->mmax : p->n;
  const kalman_gpu_tuning_t tune = tuning_now();
  const bool cta = use_cta(p, tune);
  if (cta && mxp > kCtaMaxN) {
    ukg_set_error(KALMAN_GPU_EINVAL, "state dimension %d (observation rows %d) above this build's limit %d", p->n,
                  p->mmax, kCtaMaxN);
    return nullptr;
  }
  const bool dd = (options & KALMAN_GPU_FP32_REFINE) && want_cov; /* double-float with covariances */
  const bool fp32 = (options & KALMAN_GPU_FP32_REFINE) && !dd;
  Plan P;
  const size_t need = build_plan(p, want_cov, fp32, fp32, P, nullptr, 0, cta);
  if (need == 0) {
    ukg_set_error(KALMAN_GPU_EINVAL, "tracks longer than 2^%d steps", kMaxLevels - 1);
    return nullptr;
  }
  std::vector<int64_t> tab(need);
  build_plan(p, want_cov, fp32, fp32, P, tab.data(), need, cta);
  kalman_gpu_plan* pl = new kalman_gpu_plan();
  pl->cta = cta;
  cudaGetDevice(&pl->device);
  const int ncta = cta ? cta_count(tune.ctas_per_sm) : 0;
  const int64_t per = cta ? cta_scratch_per_cta(p->n, p->mmax) : 0;
  const size_t scratch_off = align_up(P.bytes, 256);
  const size_t bytes = cta ? scratch_off + (size_t)ncta * per * sizeof(double) : P.bytes;
  cudaError_t e = cudaMalloc(&pl->work, bytes);
  if (e == cudaSuccess)
    e = cudaMemcpy((char*)pl->work + P.o_tab, tab.data(), need * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ukg_set_error(KALMAN_GPU_ENOMEM, "plan workspace of %zu bytes: %s", bytes, cudaGetErrorString(e));
    kalman_gpu_plan_destroy(pl);
    return nullptr;
  }
  pl->dflag = (int*)((char*)pl->work + P.o_flag);
  cudaStream_t cs = nullptr;
  e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    const int prof = ukg_prof_pause(); /* no profiling events inside the graph */
    int st;
    if (cta && fp32)
      st = run_plan_cta<float>(options, p, cs, P, nullptr, (char*)pl->work, (char*)pl->work + scratch_off, per, ncta,
                               true);
    else if (cta && dd)
      st = run_plan_cta<ukg_df::dd>(options, p, cs, P, nullptr, (char*)pl->work, (char*)pl->work + scratch_off, per,
                                    ncta, true);
    else if (dd)
      st = run_plan<ukg_df::dd>(options, p, cs, P, nullptr, (char*)pl->work, nullptr, true);
    else if (cta)
      st = run_plan_cta<double>(options, p, cs, P, nullptr, (char*)pl->work, (char*)pl->work + scratch_off, per, ncta,
                                true);
    else if (fp32)
      st = run_plan<float>(options, p, cs, P, nullptr, (char*)pl->work, nullptr, true);
    else
      st = run_plan<double>(options, p, cs, P, nullptr, (char*)pl->work, nullptr, true);
    ukg_prof_resume(prof);
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(cs, &g);
    pl->graph = g;
    e = st ? cudaErrorUnknown : ee;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&pl->exec, pl->graph, 0);
  if (cs) cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (!kalman_gpu_last_status())
      ukg_set_error(KALMAN_GPU_ECUDA, "capturing the plan into a CUDA graph: %s", cudaGetErrorString(e));
    kalman_gpu_plan_destroy(pl);
    return nullptr;
  }
  return pl;
}

extern "C" int kalman_gpu_plan_execute(kalman_gpu_plan_t* pl, void* cuda_stream)
{
  ukg_clear_error();
  if (!pl || !pl->exec) return ukg_set_error(KALMAN_GPU_EINVAL, "no plan");
  cudaStream_t st = (cudaStream_t)cuda_stream;
  const cudaError_t e = cudaGraphLaunch(pl->exec, st);
  if (e != cudaSuccess) return ukg_set_error(KALMAN_GPU_ECUDA, "plan launch: %s", cudaGetErrorString(e));
  pl->last = st;
  pl->launched = true;
  return 0;
}

extern "C" int kalman_gpu_plan_status(kalman_gpu_plan_t* pl)
{
  ukg_clear_error();
  if (!pl || !pl->exec) return ukg_set_error(KALMAN_GPU_EINVAL, "no plan");
  if (!pl->launched) return 0;
  int hflag = 0;
  cudaError_t e = cudaStreamSynchronize(pl->last);
  if (e == cudaSuccess) e = cudaMemcpy(&hflag, pl->dflag, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return ukg_set_error(KALMAN_GPU_ECUDA, "plan: %s", cudaGetErrorString(e));
  if (hflag & 8) return ukg_set_error(KALMAN_GPU_ECUDA, "a bulk copy into shared memory did not complete in time");
  if (hflag & 4) return ukg_set_error(KALMAN_GPU_EINVAL, "malformed input: observation rows outside [0, mmax] or an "
                                     "unknown covariance type");
  if (hflag & 1) return ukg_set_error(KALMAN_GPU_ESINGULAR, "a covariance factor is not positive definite");
  if (hflag & 2) return ukg_set_error(KALMAN_GPU_ESINGULAR, "zero pivot: the smoothing problem is not observable");
  return 0;
}
