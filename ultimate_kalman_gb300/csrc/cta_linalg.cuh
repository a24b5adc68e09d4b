/*
 * cta_linalg.cuh -- dense linear algebra for one thread block (CTA) on small
 * matrices held row-major in global scratch: block reductions, Householder QR
 * with one thread per column, triangular solves with one thread per
 * right-hand side, weighing by a covariance factor.  Used by the CTA kernels
 * of the odd-even and associative smoothers for larger state dimensions.
 * Templates over the arithmetic type (FP64, or FP32 for the precision form).
 */
#pragma once
#include <cstdint>

namespace cta {

constexpr int NT = 128; /* threads per CTA; rows of a panel beyond NT are looped */
constexpr int kMaxPanelRows = 256; /* 2 x the largest state dimension (128) */

/* slot-major view: entry e of slot s at p[s * w + e] */
template <typename T>
struct Aos {
  T* p;
  int64_t w;
  __device__ __forceinline__ T& at(int e, int64_t s) const { return p[s * w + e]; }
};
/* sum over the CTA, returned to every thread; red holds >= 33 entries */
template <typename T>
static __device__ __forceinline__ T block_sum(T v, T* red)
{
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    T s = T(0);
    for (int w = 0; w < NT / 32; ++w) s += red[w];
    red[32] = s;
  }
  __syncthreads();
  const T r = red[32];
  __syncthreads(); /* red may be reused right away */
  return r;
}

/* Householder QR of the row-major panel A (ld) on its first `rows` rows: the
 * first npiv columns are triangularized (reflectors stored below the
 * diagonal, LAPACK dlarfg convention), Q^T is applied to all `cols` columns. */
template <typename T>
static __device__ void householder(T* A, int ld, int rows, int npiv, int cols, T* red)
{
  __shared__ T vs[kMaxPanelRows];
  const int tid = threadIdx.x;
  const int kmax = rows < npiv ? rows : npiv;
  for (int k = 0; k < kmax; ++k) {
    T part = T(0);
    for (int i = k + 1 + tid; i < rows; i += NT) {
      const T x = A[(int64_t)i * ld + k];
      part = fma(x, x, part);
    }
    const T tail = block_sum(part, red);
    const T alpha = A[(int64_t)k * ld + k];
    if (tail == T(0)) continue; /* identity reflector: every thread agrees */
    const T beta = -copysign(sqrt(fma(alpha, alpha, tail)), alpha);
    const T amb = alpha - beta;
    const T inv = T(1) / (beta * amb);
    const T t = -(amb * amb) * inv, scale = beta * inv;
    /* the reflector goes to shared memory too: every column update reads it */
    for (int i = k + 1 + tid; i < rows; i += NT) {
      const T v = A[(int64_t)i * ld + k] * scale;
      A[(int64_t)i * ld + k] = v;
      vs[i] = v;
    }
    __syncthreads();
    for (int j = k + 1 + tid; j < cols; j += NT) {
      /* four partial sums: independent FMA chains */
      T d0 = A[(int64_t)k * ld + j], d1 = T(0), d2 = T(0), d3 = T(0);
      int i = k + 1;
      for (; i + 3 < rows; i += 4) {
        d0 = fma(vs[i], A[(int64_t)i * ld + j], d0);
        d1 = fma(vs[i + 1], A[(int64_t)(i + 1) * ld + j], d1);
        d2 = fma(vs[i + 2], A[(int64_t)(i + 2) * ld + j], d2);
        d3 = fma(vs[i + 3], A[(int64_t)(i + 3) * ld + j], d3);
      }
      for (; i < rows; ++i) d0 = fma(vs[i], A[(int64_t)i * ld + j], d0);
      T d = (d0 + d1) + (d2 + d3);
      d *= t;
      A[(int64_t)k * ld + j] -= d;
      for (int i = k + 1; i < rows; ++i) A[(int64_t)i * ld + j] = fma(-d, vs[i], A[(int64_t)i * ld + j]);
    }
    if (tid == 0) A[(int64_t)k * ld + k] = beta;
    __syncthreads();
  }
}

/* The same QR, blocked (the LAPACK dgeqrf scheme): panels of kWyNB columns
 * are copied to shared memory and factored there (a warp per column for the
 * in-panel updates), then the panel's reflectors are applied to the trailing
 * columns together, one thread per column: w = V^T c (kWyNB dots), then
 * u_b = tau_b (w_b - sum_{l<b} (v_l^T v_b) u_l) (the sequence H_{kb-1}..H_0
 * unrolled through the reflectors' Gram matrix), c <- c - V u.  Each trailing
 * column is streamed twice per panel instead of twice per reflector, and V is
 * read from shared memory.  Same result as householder() up to rounding;
 * reflectors are stored below the diagonal in the same convention.          */
constexpr int kWyNB = 16;
constexpr int kWyRows = 8; /* trailing-column rows loaded together */

/* shared-memory entries householder_wy works in: the panel (rows x kWyNB,
 * zero-padded), the reflectors' Gram matrix, their tau factors and column
 * scales, partial dot products (4 warps x kWyNB), look-ahead norms (4) */
constexpr int kWyShared = kMaxPanelRows * kWyNB + kWyNB * kWyNB + 2 * kWyNB + 4 * kWyNB + 4;

/* Applies the panel's reflectors H_{kb-1} .. H_0 to CW columns c, c + dc of
 * the row-major C (rows 0..prow-1): w = V^T c, then u_b = tau_b (w_b -
 * sum_{l<b} (v_l^T v_b) u_l), c <- c - V u.  V (unit form) and the Gram
 * matrix are in shared memory.                                               */
template <int CW, typename T>
static __device__ __forceinline__ void wy_columns(T* C, int ld, int prow, int c, int dc, const T* Vs, const T* Gs,
                                                  const T* taus, int kb)
{
  T w[CW][kWyNB];
#pragma unroll
  for (int q = 0; q < CW; ++q)
#pragma unroll
    for (int b = 0; b < kWyNB; ++b) w[q][b] = T(0);
  /* rows in groups of kWyRows: their loads are in flight together */
  int i = 0;
#pragma unroll 1
  for (; i + kWyRows <= prow; i += kWyRows) {
    T cv[CW][kWyRows];
#pragma unroll
    for (int u = 0; u < kWyRows; ++u)
#pragma unroll
      for (int q = 0; q < CW; ++q) cv[q][u] = C[(int64_t)(i + u) * ld + c + q * dc];
#pragma unroll
    for (int u = 0; u < kWyRows; ++u)
#pragma unroll
      for (int b = 0; b < kWyNB; ++b) {
        const T v = Vs[(i + u) * kWyNB + b];
#pragma unroll
        for (int q = 0; q < CW; ++q) w[q][b] = fma(v, cv[q][u], w[q][b]);
      }
  }
#pragma unroll 1
  for (; i < prow; ++i)
#pragma unroll
    for (int q = 0; q < CW; ++q) {
      const T ci = C[(int64_t)i * ld + c + q * dc];
#pragma unroll
      for (int b = 0; b < kWyNB; ++b) w[q][b] = fma(Vs[i * kWyNB + b], ci, w[q][b]);
    }
  /* an opaque zero offset keeps the Gram matrix in shared memory instead of
     120 loop-invariant registers */
  int g0 = 0;
  asm volatile("" : "+r"(g0));
#pragma unroll
  for (int b = 0; b < kWyNB; ++b) {
    const T tb = b < kb ? taus[b] : T(0);
#pragma unroll
    for (int q = 0; q < CW; ++q) {
      T sm = w[q][b];
#pragma unroll
      for (int l = 0; l < b; ++l) sm = fma(-Gs[g0 + l * kWyNB + b], w[q][l], sm);
      w[q][b] = tb * sm; /* w now holds u */
    }
  }
  i = 0;
#pragma unroll 1
  for (; i + kWyRows <= prow; i += kWyRows) {
    T cv[CW][kWyRows];
#pragma unroll
    for (int u = 0; u < kWyRows; ++u)
#pragma unroll
      for (int q = 0; q < CW; ++q) cv[q][u] = C[(int64_t)(i + u) * ld + c + q * dc];
#pragma unroll
    for (int u = 0; u < kWyRows; ++u) {
#pragma unroll
      for (int b = 0; b < kWyNB; ++b) {
        const T v = Vs[(i + u) * kWyNB + b];
#pragma unroll
        for (int q = 0; q < CW; ++q) cv[q][u] = fma(-v, w[q][b], cv[q][u]);
      }
#pragma unroll
      for (int q = 0; q < CW; ++q) C[(int64_t)(i + u) * ld + c + q * dc] = cv[q][u];
    }
  }
#pragma unroll 1
  for (; i < prow; ++i)
#pragma unroll
    for (int q = 0; q < CW; ++q) {
      T ci = C[(int64_t)i * ld + c + q * dc];
#pragma unroll
      for (int b = 0; b < kWyNB; ++b) ci = fma(-Vs[i * kWyNB + b], w[q][b], ci);
      C[(int64_t)i * ld + c + q * dc] = ci;
    }
}

template <typename T>
static __device__ void householder_wy(T* A, int ld, int rows, int npiv, int cols, T* red, T* sh)
{
  static_assert(NT == 8 * kWyNB, "the panel factorization maps the CTA to kWyNB columns x 8 row groups");
  T* Vs = sh;                              /* Vs[i * kWyNB + b] */
  T* Gs = sh + kMaxPanelRows * kWyNB;      /* Gs[l * kWyNB + b] = v_l^T v_b, l < b */
  T* taus = Gs + kWyNB * kWyNB;
  T* scl = taus + kWyNB;                   /* reflector b's entries below the diagonal, unscaled until write-back */
  T* dpart = scl + kWyNB;                  /* [warp][column] */
  T* nrm4 = dpart + 4 * kWyNB;             /* [warp]: look-ahead norm of the next column */
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int jc = tid & (kWyNB - 1), rg = tid >> 4; /* panel factorization: column, row group */
  const int kmax = rows < npiv ? rows : npiv;
  for (int k0 = 0; k0 < kmax; k0 += kWyNB) {
    const int kb = kmax - k0 < kWyNB ? kmax - k0 : kWyNB;
    const int prow = rows - k0;
    T* P = A + (int64_t)k0 * ld + k0; /* the panel: rows k0.., columns k0..k0+kb-1 */
    for (int e = tid; e < prow * kWyNB; e += NT) {
      const int i = e / kWyNB, b = e - i * kWyNB;
      Vs[e] = b < kb ? P[(int64_t)i * ld + b] : T(0);
    }
    __syncthreads();
    /* panel factorization, thread (jc, rg) on column jc, rows rg, rg + 8, ...:
       reflector k is x (column k below the diagonal, left unscaled) times
       scale; for each later column j, d_j = tau (a_kj + scale x^T a_j) and
       a_j <- a_j - d_j scale x; two barriers per reflector */
    bool ahead = false;
    for (int k = 0; k < kb; ++k) {
      T tail;
      if (ahead) {
        tail = (nrm4[0] + nrm4[1]) + (nrm4[2] + nrm4[3]);
      } else {
        T part = T(0);
        for (int i = k + 1 + tid; i < prow; i += NT) {
          const T x = Vs[i * kWyNB + k];
          part = fma(x, x, part);
        }
        tail = block_sum(part, red);
      }
      const T alpha = Vs[k * kWyNB + k];
      if (tail == T(0)) { /* identity reflector: every thread agrees */
        if (tid == 0) {
          taus[k] = T(0);
          scl[k] = T(1);
        }
        ahead = false;
        continue;
      }
      const T beta = -copysign(sqrt(fma(alpha, alpha, tail)), alpha);
      const T amb = alpha - beta;
      const T inv = T(1) / (beta * amb);
      const T t = -(amb * amb) * inv, scale = beta * inv;
      const bool act = jc > k && jc < kb;
      const T akj = act ? Vs[k * kWyNB + jc] : T(0);
      T part = T(0);
      if (act)
        for (int i = k + 1 + rg; i < prow; i += 8) part = fma(Vs[i * kWyNB + k], Vs[i * kWyNB + jc], part);
      part += __shfl_xor_sync(0xffffffffu, part, 16);
      if (lane < 16) dpart[warp * kWyNB + jc] = part;
      __syncthreads();
      const T d = act ? (akj + scale * ((dpart[jc] + dpart[kWyNB + jc]) + (dpart[2 * kWyNB + jc] + dpart[3 * kWyNB + jc]))) * t
                      : T(0);
      const T ds = d * scale;
      T sq = T(0);
      if (act)
        for (int i = k + 1 + rg; i < prow; i += 8) {
          const T v = fma(-ds, Vs[i * kWyNB + k], Vs[i * kWyNB + jc]);
          Vs[i * kWyNB + jc] = v;
          if (i > k + 1) sq = fma(v, v, sq);
        }
      sq += __shfl_xor_sync(0xffffffffu, sq, 16);
      if (k + 1 < kb && lane == k + 1) nrm4[warp] = sq; /* column k + 1's lanes are k + 1 and k + 17 */
      if (act && rg == 0) Vs[k * kWyNB + jc] = akj - d;
      if (tid == 0) {
        Vs[k * kWyNB + k] = beta;
        taus[k] = t;
        scl[k] = scale;
      }
      ahead = k + 1 < kb;
      __syncthreads();
    }
    /* R and the scaled reflectors back to the panel; V in shared memory in unit form */
    for (int e = tid; e < prow * kWyNB; e += NT) {
      const int i = e / kWyNB, b = e - i * kWyNB;
      if (b < kb) {
        T v = Vs[e];
        if (i > b) v *= scl[b];
        P[(int64_t)i * ld + b] = v;
        Vs[e] = i > b ? v : i == b ? T(1) : T(0);
      }
    }
    __syncthreads();
    const int c0 = k0 + kb; /* first trailing column */
    if (c0 >= cols) continue;
    for (int e = tid; e < kWyNB * kWyNB; e += NT) {
      const int l = e / kWyNB, b = e - l * kWyNB;
      T g0 = T(0), g1 = T(0);
      if (l < b && b < kb) {
        int i = b;
        for (; i + 1 < prow; i += 2) {
          g0 = fma(Vs[i * kWyNB + l], Vs[i * kWyNB + b], g0);
          g1 = fma(Vs[(i + 1) * kWyNB + l], Vs[(i + 1) * kWyNB + b], g1);
        }
        if (i < prow) g0 = fma(Vs[i * kWyNB + l], Vs[i * kWyNB + b], g0);
      }
      Gs[e] = g0 + g1;
    }
    __syncthreads();
    T* C = A + (int64_t)k0 * ld; /* rows k0.. */
    int c = c0 + tid;
    if constexpr (sizeof(T) == sizeof(float)) /* two columns per thread: twice the loads in flight */
      for (; c + NT < cols; c += 2 * NT) wy_columns<2>(C, ld, prow, c, NT, Vs, Gs, taus, kb);
    for (; c < cols; c += NT) wy_columns<1>(C, ld, prow, c, 0, Vs, Gs, taus, kb);
    __syncthreads();
  }
}

/* QR of a panel with whichever of the two forms suits its size: kernels for
 * states from 64 on instantiate the blocked form (at n = 128 the odd-even pair
 * kernel runs 2.3x faster with it), the others keep the unblocked form and
 * its small shared-memory footprint (at n = 48 the panels then stay in L1). */
template <bool kBlocked, typename T>
static __device__ __forceinline__ void panel_qr(T* A, int ld, int rows, int npiv, int cols, T* red, T* sh)
{
  if (kBlocked && npiv >= kWyNB && cols > npiv) householder_wy(A, ld, rows, npiv, cols, red, sh);
  else householder(A, ld, rows, npiv, cols, red);
}
constexpr int kBlockedMinN = 64;

/* x <- R^{-1} x for every column c0 <= c < c1 of the row-major X (ldx), R the
 * upper triangle of the row-major Rm (ldr), n x n: one thread per column */
template <typename T>
static __device__ void solve_upper_cols(const T* Rm, int ldr, int n, T* X, int ldx, int c0, int c1)
{
  for (int c = c0 + threadIdx.x; c < c1; c += NT)
    for (int i = n - 1; i >= 0; --i) {
      T s0 = X[(int64_t)i * ldx + c], s1 = T(0);
      int k = i + 1;
      for (; k + 1 < n; k += 2) {
        s0 = fma(-Rm[(int64_t)i * ldr + k], X[(int64_t)k * ldx + c], s0);
        s1 = fma(-Rm[(int64_t)i * ldr + k + 1], X[(int64_t)(k + 1) * ldx + c], s1);
      }
      if (k < n) s0 = fma(-Rm[(int64_t)i * ldr + k], X[(int64_t)k * ldx + c], s0);
      X[(int64_t)i * ldx + c] = (s0 + s1) / Rm[(int64_t)i * ldr + i];
    }
  __syncthreads();
}

/* x <- R^{-1} x for one vector x (n entries, shared by the CTA) */
template <typename T>
static __device__ void solve_upper_vec(const T* Rm, int ldr, int n, T* x)
{
  for (int i = n - 1; i >= 0; --i) {
    if (threadIdx.x == 0) x[i] /= Rm[(int64_t)i * ldr + i];
    __syncthreads();
    const T xi = x[i];
    for (int k = threadIdx.x; k < i; k += NT) x[k] = fma(-Rm[(int64_t)k * ldr + i], xi, x[k]);
    __syncthreads();
  }
}

static __device__ __forceinline__ bool valid_cov_type(char t) { return t == 'W' || t == 'w' || t == 'C' || t == 'U' || t == 'F'; }

/* Cholesky factor of an SPD matrix held column-major in L (rows x rows, ld
 * rows; its lower triangle is read and overwritten, the strict upper triangle
 * is ignored), blocked by kChNB columns: each column block is copied to
 * shared memory and factored there, then the trailing lower triangle takes the
 * block's rank-kChNB update, a warp per column with lanes along it (coalesced).
 * A pivot that is not positive is replaced by 1 and reported: returns false
 * in every thread.                                                           */
constexpr int kChNB = 8;
constexpr int kMaxCov = 128; /* largest covariance dimension of the CTA kernels */

template <typename T>
static __device__ bool cholesky_cm(T* L, int rows)
{
  __shared__ T Ps[kChNB][kMaxCov];
  __shared__ int bad_c;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) bad_c = 0;
  for (int j0 = 0; j0 < rows; j0 += kChNB) {
    const int nb = rows - j0 < kChNB ? rows - j0 : kChNB;
    for (int jj = warp; jj < kChNB; jj += NT / 32)
      for (int i = j0 + lane; i < rows; i += 32) Ps[jj][i] = jj < nb ? L[(int64_t)(j0 + jj) * rows + i] : T(0);
    __syncthreads();
    for (int jj = 0; jj < nb; ++jj) {
      const int j = j0 + jj;
      if (tid == 0) {
        const T d = Ps[jj][j];
        if (!(d > T(0))) bad_c = 1;
        Ps[jj][j] = d > T(0) ? sqrt(d) : T(1);
      }
      __syncthreads();
      const T ljj = Ps[jj][j];
      for (int i = j + 1 + tid; i < rows; i += NT) Ps[jj][i] /= ljj;
      __syncthreads();
      for (int kk = jj + 1 + warp; kk < nb; kk += NT / 32) {
        const T mk = Ps[jj][j0 + kk];
        for (int i = j0 + kk + lane; i < rows; i += 32) Ps[kk][i] = fma(-Ps[jj][i], mk, Ps[kk][i]);
      }
      __syncthreads();
    }
    for (int jj = warp; jj < nb; jj += NT / 32)
      for (int i = j0 + jj + lane; i < rows; i += 32) L[(int64_t)(j0 + jj) * rows + i] = Ps[jj][i];
    for (int l = j0 + nb + warp; l < rows; l += NT / 32) {
      T pl[kChNB];
#pragma unroll
      for (int jj = 0; jj < kChNB; ++jj) pl[jj] = Ps[jj][l];
      for (int i = l + lane; i < rows; i += 32) {
        T v = L[(int64_t)l * rows + i];
#pragma unroll
        for (int jj = 0; jj < kChNB; ++jj) v = fma(-Ps[jj][i], pl[jj], v);
        L[(int64_t)l * rows + i] = v;
      }
    }
    __syncthreads();
  }
  const bool ok = bad_c == 0;
  __syncthreads();
  return ok;
}

/* B <- L^{-1} B for CW columns c, c + dc of the row-major B (rows x cols,
 * ldb) and the lower triangular, column-major L (ld rows), four rows at a
 * time: each L entry loaded once per CW columns, each B entry once per four
 * rows, 4 CW independent chains.                                            */
template <int CW, typename T>
static __device__ __forceinline__ void fsub_cols(const T* L, int rows, T* B, int ldb, int c, int dc)
{
  for (int i0 = 0; i0 < rows; i0 += 4) {
    const int nq = rows - i0 < 4 ? rows - i0 : 4;
    T s[CW][4];
#pragma unroll
    for (int w = 0; w < CW; ++w)
#pragma unroll
      for (int q = 0; q < 4; ++q) s[w][q] = q < nq ? B[(int64_t)(i0 + q) * ldb + c + w * dc] : T(0);
    if (nq == 4) {
#pragma unroll 2
      for (int k = 0; k < i0; ++k) {
        T bk[CW];
#pragma unroll
        for (int w = 0; w < CW; ++w) bk[w] = B[(int64_t)k * ldb + c + w * dc];
        const T* Lk = L + (int64_t)k * rows + i0;
        const T l0 = Lk[0], l1 = Lk[1], l2 = Lk[2], l3 = Lk[3];
#pragma unroll
        for (int w = 0; w < CW; ++w) {
          s[w][0] = fma(-l0, bk[w], s[w][0]);
          s[w][1] = fma(-l1, bk[w], s[w][1]);
          s[w][2] = fma(-l2, bk[w], s[w][2]);
          s[w][3] = fma(-l3, bk[w], s[w][3]);
        }
      }
    } else {
      for (int k = 0; k < i0; ++k) {
#pragma unroll
        for (int w = 0; w < CW; ++w) {
          const T bk = B[(int64_t)k * ldb + c + w * dc];
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (q < nq) s[w][q] = fma(-L[(int64_t)k * rows + i0 + q], bk, s[w][q]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (q < nq) {
        const T dq = L[(int64_t)(i0 + q) * rows + i0 + q];
#pragma unroll
        for (int w = 0; w < CW; ++w) {
#pragma unroll
          for (int r = 0; r < q; ++r) s[w][q] = fma(-L[(int64_t)(i0 + r) * rows + i0 + q], s[w][r], s[w][q]);
          s[w][q] /= dq;
          B[(int64_t)(i0 + q) * ldb + c + w * dc] = s[w][q];
        }
      }
  }
}

/* B <- L^{-1} B for the row-major B (rows x cols, ldb) and the lower
 * triangular, column-major L (ld rows): one thread per column (two where the
 * columns go past the CTA's threads), four rows at a time.                 */
template <typename T>
static __device__ void forward_subst_cm(const T* L, int rows, T* B, int ldb, int cols)
{
  int c = threadIdx.x;
  for (; c + NT < cols; c += 2 * NT) fsub_cols<2>(L, rows, B, ldb, c, NT);
  for (; c < cols; c += NT) fsub_cols<1>(L, rows, B, ldb, c, 0);
  __syncthreads();
}

/* w <- L^{-1} w (lower = true) or L^{-T} w for the column-major lower
 * triangular L (ld rows) and the CTA-shared vector w; run by warp 0, columns of
 * L read along their length, and followed by a CTA barrier.                 */
template <typename T>
static __device__ void tri_solve_vec_cm(const T* L, int rows, T* w, bool lower)
{
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    if (lower)
      for (int j = 0; j < rows; ++j) {
        const T wj = w[j] / L[(int64_t)j * rows + j];
        __syncwarp();
        if (lane == 0) w[j] = wj;
        for (int i = j + 1 + lane; i < rows; i += 32) w[i] = fma(-L[(int64_t)j * rows + i], wj, w[i]);
        __syncwarp();
      }
    else
      for (int j = rows - 1; j >= 0; --j) {
        T d = T(0);
        for (int i = j + 1 + lane; i < rows; i += 32) d = fma(L[(int64_t)j * rows + i], w[i], d);
        for (int off = 16; off > 0; off >>= 1) d += __shfl_xor_sync(0xffffffffu, d, off);
        const T wj = (w[j] - d) / L[(int64_t)j * rows + j];
        __syncwarp();
        if (lane == 0) w[j] = wj;
        __syncwarp();
      }
  }
  __syncthreads();
}

/* Copies between a column-major block (ld lds) and a row-major block (ld ldd)
 * through a 32 x 33 shared tile, so that both sides are read and written
 * along rows of 32 consecutive entries.  f converts each element.           */
template <typename T>
struct Tile {
  T t[32][33];
};
template <typename D, typename S, typename F>
static __device__ void cm_to_rm(const S* src, int64_t lds, int rows, int cols, D* dst, int64_t ldd, F f, Tile<D>& tl)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int r0 = 0; r0 < rows; r0 += 32)
    for (int c0 = 0; c0 < cols; c0 += 32) {
      for (int cc = warp; cc < 32; cc += NT / 32)
        if (c0 + cc < cols && r0 + lane < rows) tl.t[cc][lane] = f(src[(int64_t)(c0 + cc) * lds + r0 + lane]);
      __syncthreads();
      for (int rr = warp; rr < 32; rr += NT / 32)
        if (r0 + rr < rows && c0 + lane < cols) dst[(int64_t)(r0 + rr) * ldd + c0 + lane] = tl.t[lane][rr];
      __syncthreads();
    }
}
struct Ident {
  template <typename V>
  __device__ __forceinline__ V operator()(V v) const { return v; }
};
/* kUpper: entries below the diagonal are written as zeros */
template <bool kUpper = false, typename D, typename S>
static __device__ void rm_to_cm(const S* src, int64_t lds, int rows, int cols, D* dst, int64_t ldd, Tile<S>& tl)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int r0 = 0; r0 < rows; r0 += 32)
    for (int c0 = 0; c0 < cols; c0 += 32) {
      for (int rr = warp; rr < 32; rr += NT / 32)
        if (r0 + rr < rows && c0 + lane < cols) tl.t[rr][lane] = src[(int64_t)(r0 + rr) * lds + c0 + lane];
      __syncthreads();
      for (int cc = warp; cc < 32; cc += NT / 32)
        if (c0 + cc < cols && r0 + lane < rows)
          dst[(int64_t)(c0 + cc) * ldd + r0 + lane] = kUpper && r0 + lane > c0 + cc ? D(0) : tl.t[lane][cc];
      __syncthreads();
    }
}

/* Weighs the row-major panel B (rows x cols, ldb) by the covariance factor
 * (cov column-major rows x rows, ld ldc, type): 'W' B <- W B, 'w' B <- diag B,
 * 'C' B <- chol(cov)^{-1} B, 'U'/'F' B <- tril(cov)^{-1} B (the lower
 * triangle of cov in both).  L (rows x rows) is scratch, used column-major.
 * Returns false (in every thread) for a factor that is not positive definite
 * or has a zero pivot. */
template <typename T>
static __device__ bool weigh_panel(char type, const double* cov, int ldc, int rows, T* B, int ldb, int cols, T* L,
                                  T* red, T* tmp)
{
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (type == 'w') {
    for (int e = tid; e < rows * cols; e += NT) {
      const int i = e / cols, c = e - i * cols;
      B[(int64_t)i * ldb + c] *= T(cov[i]);
    }
    __syncthreads();
    return true;
  }
  if (type == 'W') { /* B <- W B, one thread per column, W read from the caller's array */
    for (int c = tid; c < cols; c += NT) {
      for (int i = 0; i < rows; ++i) {
        T s0 = T(0), s1 = T(0);
        int j = 0;
        for (; j + 1 < rows; j += 2) {
          s0 = fma(T(cov[(int64_t)j * ldc + i]), B[(int64_t)j * ldb + c], s0);
          s1 = fma(T(cov[(int64_t)(j + 1) * ldc + i]), B[(int64_t)(j + 1) * ldb + c], s1);
        }
        if (j < rows) s0 = fma(T(cov[(int64_t)j * ldc + i]), B[(int64_t)j * ldb + c], s0);
        tmp[(int64_t)i * NT + tid] = s0 + s1;
      }
      for (int i = 0; i < rows; ++i) B[(int64_t)i * ldb + c] = tmp[(int64_t)i * NT + tid];
    }
    __syncthreads();
    return true;
  }
  if (type != 'C' && type != 'U' && type != 'F') return true;
  for (int j = warp; j < rows; j += NT / 32)
    for (int i = lane; i < rows; i += 32) L[(int64_t)j * rows + i] = i >= j ? T(cov[(int64_t)j * ldc + i]) : T(0);
  __syncthreads();
  bool ok = true;
  if (type == 'C') {
    ok = cholesky_cm(L, rows);
  } else {
    __shared__ int bad_s;
    if (tid == 0) {
      bad_s = 0;
      for (int j = 0; j < rows; ++j)
        if (L[(int64_t)j * rows + j] == T(0)) bad_s = 1;
    }
    __syncthreads();
    ok = bad_s == 0;
    __syncthreads();
  }
  forward_subst_cm(L, rows, B, ldb, cols);
  return ok;
}

}  // namespace cta
