/*
 * matrix_ops.h -- dense-matrix type and helper functions of the GB300 Kalman
 * smoother library (libukgpu.so).
 *
 * The matrix type and every declaration below keep the binary interface of
 * UltimateKalman's c/matrix_ops.h (release 2.1.0), because c/kalman.h includes
 * that header (c/kalman.h:21) and clients build their inputs with these calls:
 *
 *   kalman_matrix_t            c/matrix_ops.h:137-147   (column-major, ld)
 *   matrix_get / matrix_set    c/matrix_ops.h:149-155   (macros under NDEBUG)
 *   matrix_create ... add      c/matrix_ops.h:160-236
 *
 * These functions are host-side helpers that clients use to build equations
 * and read results.  The smoothers in this library never call them: the
 * smoothing itself runs in CUDA kernels (see kalman_gpu.h).  They allocate
 * with malloc and are freed by matrix_free, as in the reference.
 */
#ifndef MATRIX_OPS_H
#define MATRIX_OPS_H

#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Element (i,j) lives at elements[j*ld + i].  A matrix with no rows or no
 * columns has elements == NULL.                                             */
typedef struct matrix_st {
  int32_t row_dim;
  int32_t col_dim;
  int32_t ld;
  double* elements;
}
kalman_matrix_t
#ifdef KALMAN_MATRIX_SHORT_TYPE
, matrix_t
#endif
;

#ifdef NDEBUG
#define matrix_set(A,i,j,v) ( ((A)->elements)[ (j)*((A)->ld) + (i) ] = (v) )
#define matrix_get(A,i,j)   ( ((A)->elements)[ (j)*((A)->ld) + (i) ] )
#else
void   matrix_set(kalman_matrix_t* A, int32_t i, int32_t j, double v);
double matrix_get(kalman_matrix_t* A, int32_t i, int32_t j);
#endif

kalman_matrix_t* matrix_create(int32_t rows, int32_t cols);
kalman_matrix_t* matrix_create_constant(int32_t rows, int32_t cols, double c);
kalman_matrix_t* matrix_create_copy(kalman_matrix_t* A);
kalman_matrix_t* matrix_create_sub(kalman_matrix_t* A, int32_t first_row, int32_t rows, int32_t first_col, int32_t cols);
void             matrix_mutate_copy_sub(kalman_matrix_t* C, int32_t first_row, int32_t first_col, kalman_matrix_t* A);
void             matrix_free(kalman_matrix_t* A);

int32_t matrix_rows(kalman_matrix_t* A);
int32_t matrix_cols(kalman_matrix_t* A);
int32_t matrix_ld  (kalman_matrix_t* A);

kalman_matrix_t* matrix_create_identity(int32_t rows, int32_t cols);
kalman_matrix_t* matrix_create_from_rowwise(double* naked, int32_t rows, int32_t cols);

void matrix_print(kalman_matrix_t* A, char* format);

void matrix_mutate_gemm    (double ALPHA, kalman_matrix_t* A, kalman_matrix_t* B, double BETA, kalman_matrix_t* C);
void matrix_mutate_scale   (kalman_matrix_t* A, double s);
void matrix_mutate_triu    (kalman_matrix_t* A);
void matrix_mutate_chop    (kalman_matrix_t* A, int32_t rows, int32_t cols);
void matrix_mutate_copy    (kalman_matrix_t* C, kalman_matrix_t* A);
void matrix_mutate_trisolve(char* triangle, kalman_matrix_t* U, kalman_matrix_t* b);
void matrix_mutate_chol    (kalman_matrix_t* L);

/* Householder QR in LAPACK's compact form: A is overwritten by R (upper
 * triangle) and the reflector tails (below it); the returned column holds
 * the reflector scalars tau.                                                */
kalman_matrix_t* matrix_create_mutate_qr(kalman_matrix_t* A);
/* C <- Q^T C for the Q held by (QR, TAU).                                    */
void matrix_mutate_apply_qt(kalman_matrix_t* QR, kalman_matrix_t* TAU, kalman_matrix_t* C);

kalman_matrix_t* matrix_create_trisolve (char* triangle, kalman_matrix_t* U, kalman_matrix_t* b);
kalman_matrix_t* matrix_create_chol     (kalman_matrix_t* L);
kalman_matrix_t* matrix_create_vconcat  (kalman_matrix_t* A, kalman_matrix_t* B);
kalman_matrix_t* matrix_create_inverse  (kalman_matrix_t* A);
kalman_matrix_t* matrix_create_transpose(kalman_matrix_t* A);
kalman_matrix_t* matrix_create_mldivide (kalman_matrix_t* A, kalman_matrix_t* B);
kalman_matrix_t* matrix_create_multiply (kalman_matrix_t* A, kalman_matrix_t* B);
kalman_matrix_t* matrix_create_subtract (kalman_matrix_t* A, kalman_matrix_t* B);
kalman_matrix_t* matrix_create_add      (kalman_matrix_t* A, kalman_matrix_t* B);

#ifdef __cplusplus
}
#endif

#endif /* MATRIX_OPS_H */
