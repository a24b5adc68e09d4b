/*
 * cta_linalg.cuh -- dense linear algebra for one thread block (CTA) on small
 * matrices held row-major in global scratch: block reductions, Householder QR
 * with one thread per column, triangular solves with one thread per
 * right-hand side, weighing by a covariance factor.  Used by the CTA kernels
 * of the odd-even and associative smoothers for larger state dimensions.
 * FP64.
 */
#pragma once
#include <cstdint>

namespace cta {

constexpr int NT = 128; /* threads per CTA; rows of a panel beyond NT are looped */

/* slot-major view: entry e of slot s at p[s * w + e] */
template <typename T>
struct Aos {
  T* p;
  int64_t w;
  __device__ __forceinline__ T& at(int e, int64_t s) const { return p[s * w + e]; }
};
/* sum over the CTA, returned to every thread; red holds >= 33 doubles */
static __device__ __forceinline__ double block_sum(double v, double* red)
{
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < NT / 32; ++w) s += red[w];
    red[32] = s;
  }
  __syncthreads();
  const double r = red[32];
  __syncthreads(); /* red may be reused right away */
  return r;
}

/* Householder QR of the row-major panel A (ld) on its first `rows` rows: the
 * first npiv columns are triangularized (reflectors stored below the
 * diagonal, LAPACK dlarfg convention), Q^T is applied to all `cols` columns. */
static __device__ void householder(double* A, int ld, int rows, int npiv, int cols, double* red)
{
  const int tid = threadIdx.x;
  const int kmax = rows < npiv ? rows : npiv;
  for (int k = 0; k < kmax; ++k) {
    double part = 0.0;
    for (int i = k + 1 + tid; i < rows; i += NT) {
      const double x = A[(int64_t)i * ld + k];
      part = fma(x, x, part);
    }
    const double tail = block_sum(part, red);
    const double alpha = A[(int64_t)k * ld + k];
    if (tail == 0.0) continue; /* identity reflector: every thread agrees */
    const double beta = -copysign(sqrt(fma(alpha, alpha, tail)), alpha);
    const double amb = alpha - beta;
    const double inv = 1.0 / (beta * amb);
    const double t = -(amb * amb) * inv, scale = beta * inv;
    for (int i = k + 1 + tid; i < rows; i += NT) A[(int64_t)i * ld + k] *= scale;
    __syncthreads();
    for (int j = k + 1 + tid; j < cols; j += NT) {
      double d = A[(int64_t)k * ld + j];
      for (int i = k + 1; i < rows; ++i) d = fma(A[(int64_t)i * ld + k], A[(int64_t)i * ld + j], d);
      d *= t;
      A[(int64_t)k * ld + j] -= d;
      for (int i = k + 1; i < rows; ++i) A[(int64_t)i * ld + j] = fma(-d, A[(int64_t)i * ld + k], A[(int64_t)i * ld + j]);
    }
    if (tid == 0) A[(int64_t)k * ld + k] = beta;
    __syncthreads();
  }
}

/* x <- R^{-1} x for every column c0 <= c < c1 of the row-major X (ldx), R the
 * upper triangle of the row-major Rm (ldr), n x n: one thread per column */
static __device__ void solve_upper_cols(const double* Rm, int ldr, int n, double* X, int ldx, int c0, int c1)
{
  for (int c = c0 + threadIdx.x; c < c1; c += NT)
    for (int i = n - 1; i >= 0; --i) {
      double s = X[(int64_t)i * ldx + c];
      for (int k = i + 1; k < n; ++k) s = fma(-Rm[(int64_t)i * ldr + k], X[(int64_t)k * ldx + c], s);
      X[(int64_t)i * ldx + c] = s / Rm[(int64_t)i * ldr + i];
    }
  __syncthreads();
}

/* x <- R^{-1} x for one vector x (n entries, shared by the CTA) */
static __device__ void solve_upper_vec(const double* Rm, int ldr, int n, double* x)
{
  for (int i = n - 1; i >= 0; --i) {
    if (threadIdx.x == 0) x[i] /= Rm[(int64_t)i * ldr + i];
    __syncthreads();
    const double xi = x[i];
    for (int k = threadIdx.x; k < i; k += NT) x[k] = fma(-Rm[(int64_t)k * ldr + i], xi, x[k]);
    __syncthreads();
  }
}

static __device__ __forceinline__ bool valid_cov_type(char t) { return t == 'W' || t == 'w' || t == 'C' || t == 'U' || t == 'F'; }

/* Weighs the row-major panel B (rows x cols, ldb) by the covariance factor
 * (cov column-major rows x rows, ld ldc, type): 'W' B <- W B, 'w' B <- diag B,
 * 'C' B <- chol(cov)^{-1} B, 'U'/'F' B <- tril(cov)^{-1} B.  L (rows x rows
 * row-major, ld rows) is scratch.  Returns false (in every thread) for a
 * factor that is not positive definite or has a zero pivot. */
static __device__ bool weigh_panel(char type, const double* cov, int ldc, int rows, double* B, int ldb, int cols, double* L,
                            double* red, double* tmp)
{
  const int tid = threadIdx.x;
  if (type == 'w') {
    for (int e = tid; e < rows * cols; e += NT) {
      const int i = e / cols, c = e - i * cols;
      B[(int64_t)i * ldb + c] *= cov[i];
    }
    __syncthreads();
    return true;
  }
  if (type == 'W') { /* B <- W B, one thread per column, W read from the caller's array */
    for (int c = tid; c < cols; c += NT) {
      for (int i = 0; i < rows; ++i) {
        double s = 0.0;
        for (int j = 0; j < rows; ++j) s = fma(cov[(int64_t)j * ldc + i], B[(int64_t)j * ldb + c], s);
        tmp[(int64_t)i * NT + tid] = s;
      }
      for (int i = 0; i < rows; ++i) B[(int64_t)i * ldb + c] = tmp[(int64_t)i * NT + tid];
    }
    __syncthreads();
    return true;
  }
  if (type != 'C' && type != 'U' && type != 'F') return true;
  for (int e = tid; e < rows * rows; e += NT) {
    const int i = e / rows, j = e - i * rows;
    L[e] = i >= j ? cov[(int64_t)j * ldc + i] : 0.0;
  }
  __syncthreads();
  __shared__ int bad_s;
  if (tid == 0) bad_s = 0;
  __syncthreads();
  if (type == 'C') { /* right-looking Cholesky, in place in L */
    for (int j = 0; j < rows; ++j) {
      if (tid == 0) {
        const double d = L[(int64_t)j * rows + j];
        if (!(d > 0.0)) bad_s = 1;
        L[(int64_t)j * rows + j] = d > 0.0 ? sqrt(d) : 1.0;
      }
      __syncthreads();
      const double ljj = L[(int64_t)j * rows + j];
      for (int i = j + 1 + tid; i < rows; i += NT) L[(int64_t)i * rows + j] /= ljj;
      __syncthreads();
      for (int i = j + 1 + tid; i < rows; i += NT) {
        const double lij = L[(int64_t)i * rows + j];
        for (int l = j + 1; l <= i; ++l) L[(int64_t)i * rows + l] = fma(-lij, L[(int64_t)l * rows + j], L[(int64_t)i * rows + l]);
      }
      __syncthreads();
    }
  } else {
    if (tid == 0)
      for (int j = 0; j < rows; ++j)
        if (L[(int64_t)j * rows + j] == 0.0) bad_s = 1;
    __syncthreads();
  }
  /* forward substitution, one thread per column */
  for (int c = tid; c < cols; c += NT)
    for (int i = 0; i < rows; ++i) {
      double s = B[(int64_t)i * ldb + c];
      for (int k = 0; k < i; ++k) s = fma(-L[(int64_t)i * rows + k], B[(int64_t)k * ldb + c], s);
      B[(int64_t)i * ldb + c] = s / L[(int64_t)i * rows + i];
    }
  __syncthreads();
  const bool ok = bad_s == 0;
  __syncthreads();
  return ok;
}

}  // namespace cta
