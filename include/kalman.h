/*
 * kalman.h -- public C API of libukgpu.so, a GB300 drop-in for the parallel
 * smoothers of UltimateKalman (release 2.1.0).
 *
 * Every declaration keeps the name, argument meaning and binary layout of the
 * reference header c/kalman.h, so that a client built against the reference
 * links against this library unchanged:
 *
 *   kalman_covariance_matrix_weigh/_explicit   c/kalman.h:44-45
 *   kalman_step_equations_t                    c/kalman.h:56-75
 *   kalman_options_t                           c/kalman.h:81-88
 *   kalman_create ... kalman_perftest          c/kalman.h:117-142
 *   kalman_smooth_oddeven / _associative       c/kalman.h:148-149
 *
 * Differences a client can observe:
 *  - kalman_t is opaque here; the reference exposes its vtable struct, but no
 *    client touches its fields.
 *  - The library implements KALMAN_ALGORITHM_ODDEVEN and _ASSOCIATIVE on the
 *    GPU.  ULTIMATE and CONVENTIONAL (sequential filters) are not provided;
 *    kalman_create_options() with them records an error and returns NULL, and
 *    kalman_create() selects ODDEVEN.
 *  - Errors never abort the process.  They fill the affected outputs with NaN
 *    and record a message readable through kalman_gpu_last_error()
 *    (kalman_gpu.h).
 */
#ifndef ULTIMATE_KALMAN_H
#define ULTIMATE_KALMAN_H

#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>

#include "matrix_ops.h"

#ifdef __cplusplus
extern "C" {
#endif

extern double kalman_nan;

/* Step-index width.  The reference chooses it with one of these macros
 * (c/kalman.h:24-38, c/build.sh:3-4); its build script defaults to int32 and
 * so does this library.                                                      */
#if defined(KALMAN_STEP_INDEX_TYPE_INT64)
typedef int64_t kalman_step_index_t;
#elif defined(KALMAN_STEP_INDEX_TYPE_UINT64)
typedef uint64_t kalman_step_index_t;
#elif defined(KALMAN_STEP_INDEX_TYPE_UINT32)
typedef uint32_t kalman_step_index_t;
#else
typedef int32_t kalman_step_index_t;
#endif

/* Covariance factors.  cov_type is one of
 *   'W'  cov holds W with C = (W^T W)^{-1}; weighing multiplies by W
 *   'w'  cov is a column of inverse standard deviations (diagonal W)
 *   'C'  cov is the covariance itself; weighing solves with its Cholesky factor
 *   'U','F'  cov is a lower-triangular factor L with C = L L^T
 * (c/kalman_base.c:80-169 and 178-214).                                      */
kalman_matrix_t* kalman_covariance_matrix_weigh   (kalman_matrix_t* cov, char cov_type, kalman_matrix_t* A);
kalman_matrix_t* kalman_covariance_matrix_explicit(kalman_matrix_t* cov, char type);

/* One step of the smoothing problem, as filled in by clients that call the
 * parallel smoothers directly.  Step 0 carries no H, F, c, K.  A missing
 * observation is o == NULL.  After smoothing, state (n x 1), covariance (n x n)
 * and covariance_type ('C') are set and owned by the caller.                 */
typedef struct kalman_step_equations_st {
  kalman_step_index_t step;
  int32_t dimension;

  char C_type;
  char K_type;

  kalman_matrix_t* H;
  kalman_matrix_t* F;
  kalman_matrix_t* K;
  kalman_matrix_t* c;

  kalman_matrix_t* G;
  kalman_matrix_t* o;
  kalman_matrix_t* C;

  kalman_matrix_t* state;
  kalman_matrix_t* covariance;
  char             covariance_type;
} kalman_step_equations_t;

typedef enum {
  KALMAN_NONE                   = 0,
  KALMAN_ALGORITHM_ULTIMATE     = 1 << 0,
  KALMAN_ALGORITHM_CONVENTIONAL = 1 << 1,
  KALMAN_ALGORITHM_ODDEVEN      = 1 << 2,
  KALMAN_ALGORITHM_ASSOCIATIVE  = 1 << 3,
  KALMAN_NO_COVARIANCE          = 1 << 16
} kalman_options_t;

typedef struct kalman_st kalman_t;

kalman_t* kalman_create(void);
kalman_t* kalman_create_options(uint32_t options);
void      kalman_free(kalman_t* kalman);

kalman_step_index_t kalman_earliest(kalman_t* kalman);
kalman_step_index_t kalman_latest  (kalman_t* kalman);

void kalman_evolve (kalman_t* kalman, int32_t n_i, kalman_matrix_t* H_i, kalman_matrix_t* F_i, kalman_matrix_t* c_i,
                    kalman_matrix_t* K_i, char K_type);
void kalman_observe(kalman_t* kalman, kalman_matrix_t* G_i, kalman_matrix_t* o_i, kalman_matrix_t* C_i, char C_type);
void kalman_smooth (kalman_t* kalman);

kalman_matrix_t* kalman_estimate       (kalman_t* kalman, kalman_step_index_t si);
kalman_matrix_t* kalman_covariance     (kalman_t* kalman, kalman_step_index_t si);
char             kalman_covariance_type(kalman_t* kalman, kalman_step_index_t si);
void             kalman_forget         (kalman_t* kalman, kalman_step_index_t si);
void             kalman_rollback       (kalman_t* kalman, kalman_step_index_t si);
kalman_matrix_t* kalman_perftest(kalman_t* kalman,
                                 kalman_matrix_t* H, kalman_matrix_t* F, kalman_matrix_t* c,
                                 kalman_matrix_t* K, char K_type,
                                 kalman_matrix_t* G, kalman_matrix_t* o,
                                 kalman_matrix_t* C, char C_type,
                                 int32_t count, int32_t decimation);

/* The parallel smoothers (c/kalman.h:148-149), on the GPU.                   */
void kalman_smooth_oddeven    (kalman_options_t options, kalman_step_equations_t** equations, kalman_step_index_t length);
void kalman_smooth_associative(kalman_options_t options, kalman_step_equations_t** equations, kalman_step_index_t length);

#ifdef __cplusplus
}
#endif

#endif /* ULTIMATE_KALMAN_H */
