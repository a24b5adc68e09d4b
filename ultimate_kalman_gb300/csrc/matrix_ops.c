/*
 * matrix_ops.c -- the host-side matrix helpers of the kalman.h / matrix_ops.h
 * API (UltimateKalman c/matrix_ops.h:137-236, c/kalman.h:44-45).
 *
 * Clients use these to build equations and to read results (for example the
 * reference's examples build random orthonormal matrices with
 * matrix_create_mutate_qr, and convert returned covariance factors with
 * kalman_covariance_matrix_explicit).  They operate on single small matrices
 * on the host.  The smoothers of this library never call them; the smoothing
 * runs in the CUDA kernels.
 *
 * Semantics follow the reference: every *create* function returns a new
 * malloc'd matrix owned by the caller; mutate functions work in place; QR is
 * Householder with LAPACK's compact storage (R above the diagonal, reflector
 * tails below, scalars in the returned TAU column).  Shape errors record a
 * message (kalman_gpu_last_error) and leave outputs unchanged or NaN instead
 * of aborting.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ukgpu_internal.h"

double kalman_nan = NAN;

#define EL(A, i, j) ((A)->elements[(size_t)(j) * (A)->ld + (i)])

#ifndef NDEBUG
void matrix_set(kalman_matrix_t* A, int32_t i, int32_t j, double v)
{
  if (!A || i < 0 || j < 0 || i >= A->row_dim || j >= A->col_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_set(%d,%d) out of range", i, j);
    return;
  }
  EL(A, i, j) = v;
}

double matrix_get(kalman_matrix_t* A, int32_t i, int32_t j)
{
  if (!A || i < 0 || j < 0 || i >= A->row_dim || j >= A->col_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_get(%d,%d) out of range", i, j);
    return NAN;
  }
  return EL(A, i, j);
}
#endif

kalman_matrix_t* matrix_create(int32_t rows, int32_t cols)
{
  kalman_matrix_t* A = (kalman_matrix_t*)malloc(sizeof(kalman_matrix_t));
  A->row_dim = rows;
  A->col_dim = cols;
  A->ld = rows;
  A->elements = (rows > 0 && cols > 0) ? (double*)malloc(sizeof(double) * (size_t)rows * cols) : NULL;
  return A;
}

void matrix_free(kalman_matrix_t* A)
{
  if (!A) return;
  free(A->elements);
  free(A);
}

int32_t matrix_rows(kalman_matrix_t* A) { return A ? A->row_dim : 0; }
int32_t matrix_cols(kalman_matrix_t* A) { return A ? A->col_dim : 0; }
int32_t matrix_ld(kalman_matrix_t* A) { return A ? A->ld : 0; }

kalman_matrix_t* matrix_create_constant(int32_t rows, int32_t cols, double c)
{
  kalman_matrix_t* A = matrix_create(rows, cols);
  for (int32_t j = 0; j < cols; j++)
    for (int32_t i = 0; i < rows; i++) EL(A, i, j) = c;
  return A;
}

kalman_matrix_t* matrix_create_identity(int32_t rows, int32_t cols)
{
  kalman_matrix_t* A = matrix_create_constant(rows, cols, 0.0);
  for (int32_t i = 0; i < rows && i < cols; i++) EL(A, i, i) = 1.0;
  return A;
}

kalman_matrix_t* matrix_create_from_rowwise(double* naked, int32_t rows, int32_t cols)
{
  kalman_matrix_t* A = matrix_create(rows, cols);
  for (int32_t i = 0; i < rows; i++)
    for (int32_t j = 0; j < cols; j++) EL(A, i, j) = naked[(size_t)i * cols + j];
  return A;
}

void matrix_mutate_copy(kalman_matrix_t* C, kalman_matrix_t* A)
{
  if (!A && !C) return;
  if (!A || !C || A->row_dim != C->row_dim || A->col_dim != C->col_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_mutate_copy: shape mismatch");
    return;
  }
  for (int32_t j = 0; j < A->col_dim; j++)
    for (int32_t i = 0; i < A->row_dim; i++) EL(C, i, j) = EL(A, i, j);
}

kalman_matrix_t* matrix_create_copy(kalman_matrix_t* A)
{
  if (!A) return NULL;
  kalman_matrix_t* C = matrix_create(A->row_dim, A->col_dim);
  matrix_mutate_copy(C, A);
  return C;
}

kalman_matrix_t* matrix_create_sub(kalman_matrix_t* A, int32_t first_row, int32_t rows, int32_t first_col, int32_t cols)
{
  if (!A || first_row < 0 || first_col < 0 || first_row + rows > A->row_dim || first_col + cols > A->col_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_create_sub: block out of range");
    return matrix_create_constant(rows, cols, NAN);
  }
  kalman_matrix_t* C = matrix_create(rows, cols);
  for (int32_t j = 0; j < cols; j++)
    for (int32_t i = 0; i < rows; i++) EL(C, i, j) = EL(A, first_row + i, first_col + j);
  return C;
}

void matrix_mutate_copy_sub(kalman_matrix_t* C, int32_t first_row, int32_t first_col, kalman_matrix_t* A)
{
  if (!A && !C) return;
  if (!A || !C || C->row_dim < first_row + A->row_dim || C->col_dim < first_col + A->col_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_mutate_copy_sub: block out of range");
    return;
  }
  for (int32_t j = 0; j < A->col_dim; j++)
    for (int32_t i = 0; i < A->row_dim; i++) EL(C, first_row + i, first_col + j) = EL(A, i, j);
}

void matrix_print(kalman_matrix_t* A, char* format)
{
  if (!A) return;
  printf("matrix_print %d %d\n", A->row_dim, A->col_dim);
  if (!format) format = "%f";
  for (int32_t i = 0; i < A->row_dim; i++) {
    for (int32_t j = 0; j < A->col_dim; j++) {
      printf(format, EL(A, i, j));
      printf(" ");
    }
    printf("\n");
  }
}

void matrix_mutate_chop(kalman_matrix_t* A, int32_t rows, int32_t cols)
{
  if (!A || rows < 0 || cols < 0 || rows > A->row_dim || cols > A->col_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_mutate_chop: bad size");
    return;
  }
  A->row_dim = rows;
  A->col_dim = cols;
}

void matrix_mutate_scale(kalman_matrix_t* A, double s)
{
  if (!A) return;
  for (int32_t j = 0; j < A->col_dim; j++)
    for (int32_t i = 0; i < A->row_dim; i++) EL(A, i, j) *= s;
}

void matrix_mutate_triu(kalman_matrix_t* A)
{
  if (!A) return;
  for (int32_t j = 0; j < A->col_dim; j++)
    for (int32_t i = j + 1; i < A->row_dim; i++) EL(A, i, j) = 0.0;
}

kalman_matrix_t* matrix_create_transpose(kalman_matrix_t* A)
{
  kalman_matrix_t* T = matrix_create(A->col_dim, A->row_dim);
  for (int32_t j = 0; j < A->col_dim; j++)
    for (int32_t i = 0; i < A->row_dim; i++) EL(T, j, i) = EL(A, i, j);
  return T;
}

static kalman_matrix_t* elementwise(kalman_matrix_t* A, kalman_matrix_t* B, double sb, const char* name)
{
  if (!A || !B || A->row_dim != B->row_dim || A->col_dim != B->col_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "%s: shape mismatch", name);
    return matrix_create_constant(matrix_rows(A), matrix_cols(A), NAN);
  }
  kalman_matrix_t* C = matrix_create(A->row_dim, A->col_dim);
  for (int32_t j = 0; j < A->col_dim; j++)
    for (int32_t i = 0; i < A->row_dim; i++) EL(C, i, j) = EL(A, i, j) + sb * EL(B, i, j);
  return C;
}

kalman_matrix_t* matrix_create_add(kalman_matrix_t* A, kalman_matrix_t* B) { return elementwise(A, B, 1.0, "add"); }
kalman_matrix_t* matrix_create_subtract(kalman_matrix_t* A, kalman_matrix_t* B)
{
  return elementwise(A, B, -1.0, "subtract");
}

void matrix_mutate_gemm(double alpha, kalman_matrix_t* A, kalman_matrix_t* B, double beta, kalman_matrix_t* C)
{
  if (!A || !B || !C || A->col_dim != B->row_dim || C->row_dim != A->row_dim || C->col_dim != B->col_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_mutate_gemm: shape mismatch");
    return;
  }
  for (int32_t j = 0; j < C->col_dim; j++)
    for (int32_t i = 0; i < C->row_dim; i++) {
      double s = 0.0;
      for (int32_t k = 0; k < A->col_dim; k++) s += EL(A, i, k) * EL(B, k, j);
      EL(C, i, j) = alpha * s + (beta == 0.0 ? 0.0 : beta * EL(C, i, j));
    }
}

kalman_matrix_t* matrix_create_multiply(kalman_matrix_t* A, kalman_matrix_t* B)
{
  kalman_matrix_t* C = matrix_create_constant(matrix_rows(A), matrix_cols(B), 0.0);
  matrix_mutate_gemm(1.0, A, B, 0.0, C);
  return C;
}

/* triangle "U": solve U X = B with the upper triangle; "L": the lower one    */
void matrix_mutate_trisolve(char* triangle, kalman_matrix_t* U, kalman_matrix_t* b)
{
  if (!U || !b || U->row_dim != U->col_dim || b->row_dim != U->col_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_mutate_trisolve: shape mismatch");
    return;
  }
  const int n = U->row_dim;
  const int upper = triangle && (triangle[0] == 'U' || triangle[0] == 'u');
  for (int32_t c = 0; c < b->col_dim; c++) {
    double* x = b->elements + (size_t)c * b->ld;
    if (upper) {
      for (int j = n - 1; j >= 0; j--) {
        if (EL(U, j, j) == 0.0) ukg_set_error(KALMAN_GPU_ESINGULAR, "matrix_mutate_trisolve: zero pivot");
        x[j] /= EL(U, j, j);
        for (int i = 0; i < j; i++) x[i] -= x[j] * EL(U, i, j);
      }
    } else {
      for (int j = 0; j < n; j++) {
        if (EL(U, j, j) == 0.0) ukg_set_error(KALMAN_GPU_ESINGULAR, "matrix_mutate_trisolve: zero pivot");
        x[j] /= EL(U, j, j);
        for (int i = j + 1; i < n; i++) x[i] -= x[j] * EL(U, i, j);
      }
    }
  }
}

kalman_matrix_t* matrix_create_trisolve(char* triangle, kalman_matrix_t* U, kalman_matrix_t* b)
{
  kalman_matrix_t* x = matrix_create_copy(b);
  matrix_mutate_trisolve(triangle, U, x);
  return x;
}

void matrix_mutate_chol(kalman_matrix_t* L)
{
  if (!L || L->row_dim != L->col_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_mutate_chol: matrix is not square");
    return;
  }
  const int n = L->row_dim;
  for (int j = 0; j < n; j++) {
    double d = EL(L, j, j);
    for (int k = 0; k < j; k++) d -= EL(L, j, k) * EL(L, j, k);
    if (!(d > 0.0)) {
      ukg_set_error(KALMAN_GPU_ESINGULAR, "matrix_mutate_chol: not positive definite");
      d = NAN;
    }
    d = sqrt(d);
    EL(L, j, j) = d;
    for (int i = j + 1; i < n; i++) {
      double s = EL(L, i, j);
      for (int k = 0; k < j; k++) s -= EL(L, i, k) * EL(L, j, k);
      EL(L, i, j) = s / d;
    }
    for (int i = 0; i < j; i++) EL(L, i, j) = 0.0;
  }
}

kalman_matrix_t* matrix_create_chol(kalman_matrix_t* A)
{
  kalman_matrix_t* L = matrix_create_copy(A);
  matrix_mutate_chol(L);
  return L;
}

kalman_matrix_t* matrix_create_vconcat(kalman_matrix_t* A, kalman_matrix_t* B)
{
  const int ar = matrix_rows(A), br = matrix_rows(B);
  if (ar + br == 0) return NULL;
  if (ar == 0) return matrix_create_copy(B);
  if (br == 0) return matrix_create_copy(A);
  const int cols = A->col_dim > B->col_dim ? A->col_dim : B->col_dim;
  kalman_matrix_t* C = matrix_create_constant(ar + br, cols, 0.0);
  for (int32_t j = 0; j < A->col_dim; j++)
    for (int32_t i = 0; i < ar; i++) EL(C, i, j) = EL(A, i, j);
  for (int32_t j = 0; j < B->col_dim; j++)
    for (int32_t i = 0; i < br; i++) EL(C, ar + i, j) = EL(B, i, j);
  return C;
}

kalman_matrix_t* matrix_create_mutate_qr(kalman_matrix_t* A)
{
  const int m = A->row_dim, n = A->col_dim, r = m < n ? m : n;
  kalman_matrix_t* tau = matrix_create_constant(n, 1, 0.0);
  for (int k = 0; k < r; k++) {
    double alpha = EL(A, k, k), tail = 0.0;
    for (int i = k + 1; i < m; i++) tail += EL(A, i, k) * EL(A, i, k);
    if (tail == 0.0) continue;
    const double beta = -copysign(sqrt(alpha * alpha + tail), alpha);
    const double t = (beta - alpha) / beta, s = 1.0 / (alpha - beta);
    for (int i = k + 1; i < m; i++) EL(A, i, k) *= s;
    EL(A, k, k) = beta;
    tau->elements[k] = t;
    for (int j = k + 1; j < n; j++) {
      double d = EL(A, k, j);
      for (int i = k + 1; i < m; i++) d += EL(A, i, k) * EL(A, i, j);
      d *= t;
      EL(A, k, j) -= d;
      for (int i = k + 1; i < m; i++) EL(A, i, j) -= d * EL(A, i, k);
    }
  }
  return tau;
}

void matrix_mutate_apply_qt(kalman_matrix_t* QR, kalman_matrix_t* TAU, kalman_matrix_t* C)
{
  const int m = QR->row_dim, r = QR->row_dim < QR->col_dim ? QR->row_dim : QR->col_dim;
  if (!C || C->row_dim != m) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_mutate_apply_qt: shape mismatch");
    return;
  }
  for (int k = 0; k < r; k++) {
    const double t = TAU->elements[k];
    if (t == 0.0) continue;
    for (int j = 0; j < C->col_dim; j++) {
      double d = EL(C, k, j);
      for (int i = k + 1; i < m; i++) d += EL(QR, i, k) * EL(C, i, j);
      d *= t;
      EL(C, k, j) -= d;
      for (int i = k + 1; i < m; i++) EL(C, i, j) -= d * EL(QR, i, k);
    }
  }
}

kalman_matrix_t* matrix_create_mldivide(kalman_matrix_t* A, kalman_matrix_t* B)
{
  if (!A || !B || A->row_dim != A->col_dim || B->row_dim != A->row_dim) {
    ukg_set_error(KALMAN_GPU_EINVAL, "matrix_create_mldivide: shape mismatch");
    return matrix_create_constant(matrix_cols(A), matrix_cols(B), NAN);
  }
  kalman_matrix_t* R = matrix_create_copy(A);
  kalman_matrix_t* tau = matrix_create_mutate_qr(R);
  kalman_matrix_t* X = matrix_create_copy(B);
  matrix_mutate_apply_qt(R, tau, X);
  matrix_mutate_trisolve("U", R, X);
  matrix_free(R);
  matrix_free(tau);
  return X;
}

kalman_matrix_t* matrix_create_inverse(kalman_matrix_t* A)
{
  kalman_matrix_t* I = matrix_create_identity(A->row_dim, A->col_dim);
  kalman_matrix_t* X = matrix_create_mldivide(A, I);
  matrix_free(I);
  return X;
}

/* kalman_covariance_matrix_weigh (c/kalman_base.c:61-175) */
kalman_matrix_t* kalman_covariance_matrix_weigh(kalman_matrix_t* cov, char type, kalman_matrix_t* A)
{
  if (!cov || !A) {
    ukg_set_error(KALMAN_GPU_EINVAL, "kalman_covariance_matrix_weigh: NULL argument");
    return NULL;
  }
  switch (type) {
  case 'W':
    return matrix_create_multiply(cov, A);
  case 'w': {
    kalman_matrix_t* W = matrix_create_copy(A);
    for (int32_t j = 0; j < A->col_dim; j++)
      for (int32_t i = 0; i < A->row_dim; i++) EL(W, i, j) *= EL(cov, i, 0);
    return W;
  }
  case 'C': {
    kalman_matrix_t* L = matrix_create_chol(cov);
    kalman_matrix_t* W = matrix_create_trisolve("L", L, A);
    matrix_free(L);
    return W;
  }
  case 'U':
  case 'F':
    return matrix_create_trisolve("L", cov, A);
  default:
    ukg_set_error(KALMAN_GPU_EINVAL, "unknown covariance-matrix type %c", type);
    return matrix_create_constant(A->row_dim, A->col_dim, NAN);
  }
}

/* kalman_covariance_matrix_explicit (c/kalman_base.c:178-214) */
kalman_matrix_t* kalman_covariance_matrix_explicit(kalman_matrix_t* cov, char type)
{
  if (!cov) return NULL;
  switch (type) {
  case 'w': {
    kalman_matrix_t* C = matrix_create_constant(cov->row_dim, cov->row_dim, 0.0);
    for (int32_t j = 0; j < cov->row_dim; j++) EL(C, j, j) = 1.0 / (EL(cov, j, 0) * EL(cov, j, 0));
    return C;
  }
  case 'W': {
    kalman_matrix_t* WT = matrix_create_transpose(cov);
    kalman_matrix_t* WTW = matrix_create_multiply(WT, cov);
    kalman_matrix_t* C = matrix_create_inverse(WTW);
    matrix_free(WT);
    matrix_free(WTW);
    return C;
  }
  case 'U':
  case 'F': {
    kalman_matrix_t* LT = matrix_create_transpose(cov);
    kalman_matrix_t* C = matrix_create_multiply(cov, LT);
    matrix_free(LT);
    return C;
  }
  case 'C':
    return matrix_create_copy(cov);
  default:
    ukg_set_error(KALMAN_GPU_EINVAL, "unknown covariance-matrix type %c", type);
    return NULL;
  }
}
