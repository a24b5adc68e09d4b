/*
 * kalman_oracle.c -- TEST INFRASTRUCTURE, not part of the product.
 *
 * A CPU restatement, in plain C and FP64, of the two parallel smoothers of
 * UltimateKalman 2.1.0.  It is the checker for the CUDA kernels of
 * libukgpu.so (tests/ and __graft_entry__.smoke() call it) and the timed CPU
 * baseline of bench.py.  Nothing in the product links it.
 *
 * It reads the packed problem layout of include/kalman_gpu.h with HOST
 * pointers.  All states of a track must have the same dimension n.
 *
 * Odd-even smoother (c/kalman_oddeven_smoother.c):
 *   weighing            steps_weigh 1620-1659, kalman_base.c:61-175
 *   stage A             G_F_to_R_tilde 379-457   QR of [G_j; F_{j+1}]
 *   stage B             H_R_tilde_to_R 460-523   QR of [H_j; R~_j]
 *   stage C             H_tilde_G_to_G_tilde 526-560  QR of [H~_{j+1}; G_{j+1}]
 *   odd-length fix      smooth_recursive 1452-1476 (use-after-free of
 *                       G_tilde at 1469/1471 does not arise here)
 *   renaming            Variables_Renaming 563-597
 *   base case           smooth_recursive 1360-1423
 *   back-substitution   Solve_Estimates 614-975 (states and the covariance
 *                       recurrence with the off-diagonal blocks S_off/S1_off)
 * Each "QR, then apply Q^T" of the reference is restated as one Householder
 * triangularization of an augmented block matrix: the reflectors built from
 * the pivot columns are applied to the remaining columns, which is what
 * dgeqrf + dormqr('L','T') compute.  Reflectors follow LAPACK dlarfg's sign
 * convention, so R matches LAPACK's up to rounding.
 *
 * Extensions beyond the reference, where the reference aborts: a pair of
 * consecutive unobserved steps, and an unobserved last step of an odd-length
 * level, are handled by carrying empty observation
 * blocks instead of calling QR on NULL.
 *
 * Associative smoother (c/kalman_associative_smoother.c):
 *   filtering elements  build_filtering_element_new 309-505
 *   filtering combine   filteringAssociativeOperation 889-980
 *   smoothing elements  build_smoothing_element_new 697-753
 *   smoothing combine   smoothingAssociativeOperation 982-1016
 *   read-out            filtered_to_state_new 1054-1071, smoothed_to_state_new
 *                       1073-1091, kalman_smooth_associative 1199-1240
 * Like the reference it ignores H (taken as the identity) and requires a
 * square weighted G at step 0.  Deviations: the last step's covariance is the
 * filtered Z (the reference copies an unset field and returns NaN, line 1221);
 * an unobserved step gets e = 0, J = 0 (the reference dereferences NULL), and
 * an unobserved step 1 gets b = F m0 + c (the reference adds m0 + c, line 394).
 * The scans run sequentially per track here; tracks run in parallel.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/kalman_gpu.h"

#define IDX(i, j, ld) ((size_t)(j) * (size_t)(ld) + (size_t)(i))

/* -------------------------------------------------------------------------- */
/* dense kernels on column-major blocks                                        */
/* -------------------------------------------------------------------------- */

/* Householder triangularization of the rows x cols block W.  Reflectors are
 * built from the first npiv columns (min(rows,npiv) of them) and applied to
 * every later column.  On return the upper triangle of the pivot columns is R;
 * below it lie the reflector tails.                                           */
static void hh_triangularize(double* W, int ld, int rows, int npiv, int cols)
{
  int nref = rows < npiv ? rows : npiv;
  for (int k = 0; k < nref; k++) {
    double* v = W + IDX(0, k, ld);
    double alpha = v[k];
    double tail = 0.0;
    for (int i = k + 1; i < rows; i++) tail += v[i] * v[i];
    if (tail == 0.0) continue;                 /* reflector is the identity */
    double beta = -copysign(sqrt(alpha * alpha + tail), alpha);
    double tau = (beta - alpha) / beta;
    double scale = 1.0 / (alpha - beta);
    for (int i = k + 1; i < rows; i++) v[i] *= scale;
    v[k] = beta;
    for (int j = k + 1; j < cols; j++) {
      double* a = W + IDX(0, j, ld);
      double d = a[k];
      for (int i = k + 1; i < rows; i++) d += v[i] * a[i];
      d *= tau;
      a[k] -= d;
      for (int i = k + 1; i < rows; i++) a[i] -= d * v[i];
    }
  }
}

/* x <- U^{-1} x for the upper triangle of U (n x n).  Returns 1 on a zero
 * pivot.                                                                      */
static int solve_upper(const double* U, int ld, int n, double* x, int incx)
{
  int bad = 0;
  for (int j = n - 1; j >= 0; j--) {
    double d = U[IDX(j, j, ld)];
    if (d == 0.0) bad = 1;
    double xj = x[(size_t)j * incx] / d;
    x[(size_t)j * incx] = xj;
    for (int i = 0; i < j; i++) x[(size_t)i * incx] -= xj * U[IDX(i, j, ld)];
  }
  return bad;
}

/* x <- L^{-1} x for the lower triangle of L.                                 */
static int solve_lower(const double* L, int ld, int n, double* x, int incx)
{
  int bad = 0;
  for (int j = 0; j < n; j++) {
    double d = L[IDX(j, j, ld)];
    if (d == 0.0) bad = 1;
    double xj = x[(size_t)j * incx] / d;
    x[(size_t)j * incx] = xj;
    for (int i = j + 1; i < n; i++) x[(size_t)i * incx] -= xj * L[IDX(i, j, ld)];
  }
  return bad;
}

/* In-place lower Cholesky factor (dpotrf 'L'); the strict upper part is
 * zeroed.  Returns 1 if the matrix is not positive definite.                  */
static int cholesky_lower(double* A, int ld, int n)
{
  for (int j = 0; j < n; j++) {
    double d = A[IDX(j, j, ld)];
    for (int k = 0; k < j; k++) d -= A[IDX(j, k, ld)] * A[IDX(j, k, ld)];
    if (!(d > 0.0)) return 1;
    d = sqrt(d);
    A[IDX(j, j, ld)] = d;
    for (int i = j + 1; i < n; i++) {
      double s = A[IDX(i, j, ld)];
      for (int k = 0; k < j; k++) s -= A[IDX(i, k, ld)] * A[IDX(j, k, ld)];
      A[IDX(i, j, ld)] = s / d;
    }
    for (int i = 0; i < j; i++) A[IDX(i, j, ld)] = 0.0;
  }
  return 0;
}

/* C (m x p) = op(A) op(B) (+ C if acc); op = transpose when the flag is set. */
static void gemm(int m, int p, int q, const double* A, int lda, int ta, const double* B, int ldb, int tb,
                 double* C, int ldc, int acc, double alpha)
{
  for (int j = 0; j < p; j++)
    for (int i = 0; i < m; i++) {
      double s = 0.0;
      for (int k = 0; k < q; k++) {
        double a = ta ? A[IDX(k, i, lda)] : A[IDX(i, k, lda)];
        double b = tb ? B[IDX(j, k, ldb)] : B[IDX(k, j, ldb)];
        s += a * b;
      }
      C[IDX(i, j, ldc)] = (acc ? C[IDX(i, j, ldc)] : 0.0) + alpha * s;
    }
}

/* X <- A^{-1} X for a general n x n A, by Householder QR of [A | X] (the
 * reference's matrix_create_mldivide, c/matrix_ops.c:610-630).  ws holds
 * n*(n+p) doubles.                                                           */
static int solve_general(const double* A, int lda, int n, double* X, int ldx, int p, double* ws)
{
  for (int j = 0; j < n; j++) memcpy(ws + IDX(0, j, n), A + IDX(0, j, lda), sizeof(double) * n);
  for (int j = 0; j < p; j++) memcpy(ws + IDX(0, n + j, n), X + IDX(0, j, ldx), sizeof(double) * n);
  hh_triangularize(ws, n, n, n, n + p);
  int bad = 0;
  for (int j = 0; j < p; j++) {
    bad |= solve_upper(ws, n, n, ws + IDX(0, n + j, n), 1);
    memcpy(X + IDX(0, j, ldx), ws + IDX(0, n + j, n), sizeof(double) * n);
  }
  return bad;
}

/* Weighs the rows x cols block A (leading dimension lda) in place by the
 * covariance factor cov of the given type (kalman_covariance_matrix_weigh,
 * c/kalman_base.c:61-175).  ws holds rows*(rows+cols) doubles.                */
static int weigh(char type, const double* cov, int ldc, int rows, double* A, int lda, int cols, double* ws)
{
  switch (type) {
  case 'W': {
    double* T = ws;
    gemm(rows, cols, rows, cov, ldc, 0, A, lda, 0, T, rows, 0, 1.0);
    for (int j = 0; j < cols; j++) memcpy(A + IDX(0, j, lda), T + IDX(0, j, rows), sizeof(double) * rows);
    return 0;
  }
  case 'w':
    for (int j = 0; j < cols; j++)
      for (int i = 0; i < rows; i++) A[IDX(i, j, lda)] *= cov[i];
    return 0;
  case 'C': {
    double* L = ws;
    for (int j = 0; j < rows; j++) memcpy(L + IDX(0, j, rows), cov + IDX(0, j, ldc), sizeof(double) * rows);
    if (cholesky_lower(L, rows, rows)) return 1;
    int bad = 0;
    for (int j = 0; j < cols; j++) bad |= solve_lower(L, rows, rows, A + IDX(0, j, lda), 1);
    return bad;
  }
  case 'U':
  case 'F': {
    int bad = 0;
    for (int j = 0; j < cols; j++) bad |= solve_lower(cov, ldc, rows, A + IDX(0, j, lda), 1);
    return bad;
  }
  default:
    return 1;
  }
}

/* Explicit covariance from a factor (kalman_covariance_matrix_explicit,
 * c/kalman_base.c:178-214).  out is rows x rows; ws holds 3*rows*rows.       */
static int explicit_cov(char type, const double* cov, int ldc, int rows, double* out, double* ws)
{
  switch (type) {
  case 'w':
    memset(out, 0, sizeof(double) * rows * rows);
    for (int i = 0; i < rows; i++) out[IDX(i, i, rows)] = 1.0 / (cov[i] * cov[i]);
    return 0;
  case 'C':
    for (int j = 0; j < rows; j++) memcpy(out + IDX(0, j, rows), cov + IDX(0, j, ldc), sizeof(double) * rows);
    return 0;
  case 'U':
  case 'F':
    gemm(rows, rows, rows, cov, ldc, 0, cov, ldc, 1, out, rows, 0, 1.0);
    return 0;
  case 'W': {
    /* (W^T W)^{-1} = W^{-1} W^{-T}                                           */
    double* Wi = ws; /* rows x rows */
    memset(Wi, 0, sizeof(double) * rows * rows);
    for (int i = 0; i < rows; i++) Wi[IDX(i, i, rows)] = 1.0;
    if (solve_general(cov, ldc, rows, Wi, rows, rows, ws + rows * rows)) return 1;
    gemm(rows, rows, rows, Wi, rows, 0, Wi, rows, 1, out, rows, 0, 1.0);
    return 0;
  }
  default:
    return 1;
  }
}

/* -------------------------------------------------------------------------- */
/* odd-even smoother                                                           */
/* -------------------------------------------------------------------------- */

typedef struct {
  int n, mx;
  int64_t L;
  double *F, *H, *c;     /* [L][n*n], [L][n*n], [L][n]: H x_s + F x_{s-1} = c */
  double *G, *o;         /* [L][mx*n] (ld mx), [L][mx]: G x_s = o             */
  int32_t* m;            /* rows of G                                         */
  double *R, *Ft, *Y, *cr; /* per even step e = s/2: R x_s + Ft x_{s-1} + Y x_{s+1} = cr */
  double* U;             /* [L][n*n]: U[q] = cov(x_{q-1}, x_q)                */
} olevel;

static void olevel_alloc(olevel* lv, int n, int mx, int64_t L)
{
  memset(lv, 0, sizeof(*lv));
  lv->n = n; lv->mx = mx; lv->L = L;
  size_t nn = (size_t)n * n, E = (size_t)(L + 1) / 2;
  lv->F = calloc((size_t)L * nn, sizeof(double));
  lv->H = calloc((size_t)L * nn, sizeof(double));
  lv->c = calloc((size_t)L * n, sizeof(double));
  lv->G = calloc((size_t)L * mx * n, sizeof(double));
  lv->o = calloc((size_t)L * mx, sizeof(double));
  lv->m = calloc((size_t)L, sizeof(int32_t));
  lv->R = calloc(E * nn, sizeof(double));
  lv->Ft = calloc(E * nn, sizeof(double));
  lv->Y = calloc(E * nn, sizeof(double));
  lv->cr = calloc(E * n, sizeof(double));
  lv->U = NULL;
}

static void olevel_free_equations(olevel* lv)
{
  free(lv->F); free(lv->H); free(lv->c); free(lv->G); free(lv->o); free(lv->m);
  lv->F = lv->H = lv->c = lv->G = lv->o = NULL; lv->m = NULL;
}

static void olevel_free(olevel* lv)
{
  olevel_free_equations(lv);
  free(lv->R); free(lv->Ft); free(lv->Y); free(lv->cr); free(lv->U);
}

/* copy the upper triangle of the rows x n block src into dst (zeros below)  */
static void copy_triu(double* dst, int ldd, const double* src, int lds, int rows, int n)
{
  for (int j = 0; j < n; j++)
    for (int i = 0; i < rows; i++) dst[IDX(i, j, ldd)] = (i <= j) ? src[IDX(i, j, lds)] : 0.0;
}

static void copy_block(double* dst, int ldd, const double* src, int lds, int rows, int cols)
{
  for (int j = 0; j < cols; j++)
    for (int i = 0; i < rows; i++) dst[IDX(i, j, ldd)] = src ? src[IDX(i, j, lds)] : 0.0;
}

/* Forward elimination of pair (j, j+1) of level lv, j = 2p; writes the
 * back-substitution record of step j and step p of the next level.  The last
 * pair of an odd-length level also eliminates the single last step and folds
 * its leftover rows into step p of the next level.                           */
static void oe_pair(const olevel* lv, olevel* nx, int64_t p, double* ws)
{
  const int n = lv->n, mx = lv->mx;
  const size_t nn = (size_t)n * n;
  const int64_t j = 2 * p, L = lv->L;
  const int mj = lv->m[j], mj1 = lv->m[j + 1];

  /* stage A: [G_j 0 o_j; F_{j+1} H_{j+1} c_{j+1}] */
  const int rA = mj + n, ldA = rA;
  double* WA = ws;
  copy_block(WA, ldA, lv->G + j * mx * n, mx, mj, n);
  copy_block(WA + mj, ldA, lv->F + (j + 1) * nn, n, n, n);
  copy_block(WA + IDX(0, n, ldA), ldA, NULL, 0, mj, n);
  copy_block(WA + IDX(mj, n, ldA), ldA, lv->H + (j + 1) * nn, n, n, n);
  copy_block(WA + IDX(0, 2 * n, ldA), ldA, lv->o + j * mx, mx, mj, 1);
  copy_block(WA + IDX(mj, 2 * n, ldA), ldA, lv->c + (j + 1) * n, n, n, 1);
  hh_triangularize(WA, ldA, rA, n, 2 * n + 1);
  /* R~_j = WA[0:n,0:n], X_j = WA[0:n,n:2n], o'_j = WA[0:n,2n]
     H~_{j+1} = WA[n:rA,n:2n], c'_{j+1} = WA[n:rA,2n]                         */

  /* stage C: [H~_{j+1} c'_{j+1}; G_{j+1} o_{j+1}] -> next step p observation */
  const int rC = mj + mj1, ldC = rC > 0 ? rC : 1;
  double* WC = WA + (size_t)ldA * (2 * n + 1);
  copy_block(WC, ldC, WA + IDX(n, n, ldA), ldA, mj, n);
  copy_block(WC + IDX(0, n, ldC), ldC, WA + IDX(n, 2 * n, ldA), ldA, mj, 1);
  copy_block(WC + mj, ldC, lv->G + (j + 1) * mx * n, mx, mj1, n);
  copy_block(WC + IDX(mj, n, ldC), ldC, lv->o + (j + 1) * mx, mx, mj1, 1);
  hh_triangularize(WC, ldC, rC, n, n + 1);
  const int g = rC < n ? rC : n;
  copy_triu(nx->G + p * mx * n, mx, WC, ldC, g, n);
  copy_block(nx->o + p * mx, mx, WC + IDX(0, n, ldC), ldC, g, 1);
  nx->m[p] = g;

  /* stage B */
  const int64_t e = p;
  if (j == 0) {
    copy_triu(lv->R + e * nn, n, WA, ldA, n, n);
    memset(lv->Ft + e * nn, 0, sizeof(double) * nn);
    copy_block(lv->Y + e * nn, n, WA + IDX(0, n, ldA), ldA, n, n);
    copy_block(lv->cr + e * n, n, WA + IDX(0, 2 * n, ldA), ldA, n, 1);
  } else {
    /* [H_j F_j 0 c_j; R~_j 0 X_j o'_j] */
    const int ldB = 2 * n;
    double* WB = WC + (size_t)ldC * (n + 1);
    copy_block(WB, ldB, lv->H + j * nn, n, n, n);
    copy_triu(WB + n, ldB, WA, ldA, n, n);
    copy_block(WB + IDX(0, n, ldB), ldB, lv->F + j * nn, n, n, n);
    copy_block(WB + IDX(n, n, ldB), ldB, NULL, 0, n, n);
    copy_block(WB + IDX(0, 2 * n, ldB), ldB, NULL, 0, n, n);
    copy_block(WB + IDX(n, 2 * n, ldB), ldB, WA + IDX(0, n, ldA), ldA, n, n);
    copy_block(WB + IDX(0, 3 * n, ldB), ldB, lv->c + j * n, n, n, 1);
    copy_block(WB + IDX(n, 3 * n, ldB), ldB, WA + IDX(0, 2 * n, ldA), ldA, n, 1);
    hh_triangularize(WB, ldB, 2 * n, n, 3 * n + 1);
    copy_triu(lv->R + e * nn, n, WB, ldB, n, n);
    copy_block(lv->Ft + e * nn, n, WB + IDX(0, n, ldB), ldB, n, n);
    copy_block(lv->Y + e * nn, n, WB + IDX(0, 2 * n, ldB), ldB, n, n);
    copy_block(lv->cr + e * n, n, WB + IDX(0, 3 * n, ldB), ldB, n, 1);
    /* renaming: Z_j, X~_j, o''_j become step p's evolution equation */
    copy_block(nx->F + p * nn, n, WB + IDX(n, n, ldB), ldB, n, n);
    copy_block(nx->H + p * nn, n, WB + IDX(n, 2 * n, ldB), ldB, n, n);
    copy_block(nx->c + p * n, n, WB + IDX(n, 3 * n, ldB), ldB, n, 1);
  }

  if ((L & 1) && p == L / 2 - 1) {
    /* single last step s = L-1: stage A on G_s alone, then stage B */
    const int64_t s = L - 1;
    const int ms = lv->m[s], mt = ms < n ? ms : n, ldS = ms > 0 ? ms : 1;
    double* WS = ws;
    copy_block(WS, ldS, lv->G + s * mx * n, mx, ms, n);
    copy_block(WS + IDX(0, n, ldS), ldS, lv->o + s * mx, mx, ms, 1);
    hh_triangularize(WS, ldS, ms, n, n + 1);
    const int ldT = n + mt;
    double* WT = WS + (size_t)ldS * (n + 1);
    copy_block(WT, ldT, lv->H + s * nn, n, n, n);
    copy_triu(WT + n, ldT, WS, ldS, mt, n);
    copy_block(WT + IDX(0, n, ldT), ldT, lv->F + s * nn, n, n, n);
    copy_block(WT + IDX(n, n, ldT), ldT, NULL, 0, mt, n);
    copy_block(WT + IDX(0, 2 * n, ldT), ldT, lv->c + s * n, n, n, 1);
    copy_block(WT + IDX(n, 2 * n, ldT), ldT, WS + IDX(0, n, ldS), ldS, mt, 1);
    hh_triangularize(WT, ldT, n + mt, n, 2 * n + 1);
    const int64_t es = s / 2;
    copy_triu(lv->R + es * nn, n, WT, ldT, n, n);
    copy_block(lv->Ft + es * nn, n, WT + IDX(0, n, ldT), ldT, n, n);
    memset(lv->Y + es * nn, 0, sizeof(double) * nn);
    copy_block(lv->cr + es * n, n, WT + IDX(0, 2 * n, ldT), ldT, n, 1);
    /* fix: fold [Z_s o''_s] into the observation of next-level step p */
    const int gp = nx->m[p], rF = gp + mt, ldF = rF > 0 ? rF : 1;
    double* WF = WT + (size_t)ldT * (2 * n + 1);
    copy_block(WF, ldF, nx->G + p * mx * n, mx, gp, n);
    copy_block(WF + IDX(0, n, ldF), ldF, nx->o + p * mx, mx, gp, 1);
    copy_block(WF + gp, ldF, WT + IDX(n, n, ldT), ldT, mt, n);
    copy_block(WF + IDX(gp, n, ldF), ldF, WT + IDX(n, 2 * n, ldT), ldT, mt, 1);
    hh_triangularize(WF, ldF, rF, n, n + 1);
    const int g2 = rF < n ? rF : n;
    copy_triu(nx->G + p * mx * n, mx, WF, ldF, g2, n);
    copy_block(nx->o + p * mx, mx, WF + IDX(0, n, ldF), ldF, g2, 1);
    nx->m[p] = g2;
  }
}

typedef struct {
  double* state;  /* track-local outputs, [k][n] */
  double* cov;    /* [k][n*n] or NULL          */
  int singular;
} oout;

static inline int64_t orig_index(int64_t q, int level) { return ((q + 1) << level) - 1; }

/* single-step level: x = R^{-1} Q^T o, S = R^{-1} R^{-T} (smooth_recursive
 * 1360-1423)                                                                 */
static void oe_base(const olevel* lv, int level, oout* out, double* ws)
{
  const int n = lv->n, mx = lv->mx, m0 = lv->m[0];
  const int64_t t = orig_index(0, level);
  double* x = out->state + t * n;
  if (m0 < n) {
    for (int i = 0; i < n; i++) x[i] = NAN;
    if (out->cov) for (int i = 0; i < n * n; i++) out->cov[t * n * n + i] = NAN;
    out->singular = 1;
    return;
  }
  const int ld = m0;
  double* W = ws;
  copy_block(W, ld, lv->G, mx, m0, n);
  copy_block(W + IDX(0, n, ld), ld, lv->o, mx, m0, 1);
  hh_triangularize(W, ld, m0, n, n + 1);
  for (int i = 0; i < n; i++) x[i] = W[IDX(i, n, ld)];
  out->singular |= solve_upper(W, ld, n, x, 1);
  if (out->cov) {
    double* Ri = W + (size_t)ld * (n + 1); /* R^{-1}, then S */
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) Ri[IDX(i, j, n)] = (i == j) ? 1.0 : 0.0;
    for (int j = 0; j < n; j++) solve_upper(W, ld, n, Ri + IDX(0, j, n), 1);
    gemm(n, n, n, Ri, n, 0, Ri, n, 1, out->cov + t * n * n, n, 0, 1.0);
  }
}

/* back-substitution for the even steps of a level (Solve_Estimates)        */
static void oe_solve(const olevel* lv, const olevel* nx, int level, int64_t e, oout* out, double* ws, int want_cov)
{
  const int n = lv->n;
  const size_t nn = (size_t)n * n;
  const int64_t L = lv->L, j = 2 * e;
  const int hp = j > 0, hn = j + 1 < L;
  const int64_t tj = orig_index(j, level), tm = orig_index(j - 1, level), tp = orig_index(j + 1, level);
  const double *R = lv->R + e * nn, *Ft = lv->Ft + e * nn, *Y = lv->Y + e * nn;
  double* x = out->state + tj * n;
  for (int i = 0; i < n; i++) x[i] = lv->cr[e * n + i];
  if (hp) gemm(n, 1, n, Ft, n, 0, out->state + tm * n, n, 0, x, n, 1, -1.0);
  if (hn) gemm(n, 1, n, Y, n, 0, out->state + tp * n, n, 0, x, n, 1, -1.0);
  out->singular |= solve_upper(R, n, n, x, 1);
  if (!want_cov) return;

  const double *Smm = hp ? out->cov + tm * nn : NULL, *Spp = hn ? out->cov + tp * nn : NULL;
  const double* Smp = (hp && hn) ? nx->U + ((j + 1) / 2) * nn : NULL;
  double *A1 = ws, *A2 = ws + nn, *M = ws + 2 * nn;
  memset(A1, 0, sizeof(double) * nn);
  memset(A2, 0, sizeof(double) * nn);
  if (hp) gemm(n, n, n, Ft, n, 0, Smm, n, 0, A1, n, 0, 1.0);          /* Ft Smm   */
  if (hp && hn) gemm(n, n, n, Y, n, 0, Smp, n, 1, A1, n, 1, 1.0);     /* + Y Smp^T */
  if (hn) gemm(n, n, n, Y, n, 0, Spp, n, 0, A2, n, 0, 1.0);           /* Y Spp    */
  if (hp && hn) gemm(n, n, n, Ft, n, 0, Smp, n, 0, A2, n, 1, 1.0);    /* + Ft Smp */
  /* M = I + A1 Ft^T + A2 Y^T */
  for (int jj = 0; jj < n; jj++)
    for (int i = 0; i < n; i++) M[IDX(i, jj, n)] = (i == jj) ? 1.0 : 0.0;
  if (hp) gemm(n, n, n, A1, n, 0, Ft, n, 1, M, n, 1, 1.0);
  if (hn) gemm(n, n, n, A2, n, 0, Y, n, 1, M, n, 1, 1.0);
  /* S = R^{-1} M R^{-T}: solve columns, transpose, solve again */
  for (int jj = 0; jj < n; jj++) solve_upper(R, n, n, M + IDX(0, jj, n), 1);
  double* S = out->cov + tj * nn;
  for (int jj = 0; jj < n; jj++)
    for (int i = 0; i < n; i++) S[IDX(i, jj, n)] = M[IDX(jj, i, n)];
  for (int jj = 0; jj < n; jj++) solve_upper(R, n, n, S + IDX(0, jj, n), 1);
  /* S now holds (R^{-1} (R^{-1} M)^T) = (R^{-1} M R^{-T})^T; transpose back */
  for (int jj = 0; jj < n; jj++)
    for (int i = jj + 1; i < n; i++) {
      double a = S[IDX(i, jj, n)];
      S[IDX(i, jj, n)] = S[IDX(jj, i, n)];
      S[IDX(jj, i, n)] = a;
    }
  /* off-diagonal blocks: cov(x_j, x_{j-1}) = -R^{-1} A1, cov(x_j, x_{j+1}) = -R^{-1} A2 */
  if (hp) {
    for (int jj = 0; jj < n; jj++) solve_upper(R, n, n, A1 + IDX(0, jj, n), 1);
    double* Uj = lv->U + j * nn; /* cov(x_{j-1}, x_j) = (cov(x_j, x_{j-1}))^T */
    for (int jj = 0; jj < n; jj++)
      for (int i = 0; i < n; i++) Uj[IDX(i, jj, n)] = -A1[IDX(jj, i, n)];
  }
  if (hn) {
    for (int jj = 0; jj < n; jj++) solve_upper(R, n, n, A2 + IDX(0, jj, n), 1);
    double* Up = lv->U + (j + 1) * nn;
    for (size_t i = 0; i < nn; i++) Up[i] = -A2[i];
  }
}

static int oe_nthreads(int requested)
{
#ifdef _OPENMP
  return requested > 0 ? requested : omp_get_max_threads();
#else
  (void)requested;
  return 1;
#endif
}

/* weighs step s of a packed problem into slot q of level 0 */
static int oe_weigh_step(const kalman_gpu_problem_t* P, int64_t s, int first, olevel* lv, int64_t q, double* ws)
{
  const int n = P->n, mx = lv->mx, mm = P->mmax;
  const size_t nn = (size_t)n * n;
  int bad = 0;
  if (!first) {
    double* H = lv->H + q * nn;
    double* F = lv->F + q * nn;
    double* c = lv->c + q * n;
    memcpy(H, P->H + s * nn, sizeof(double) * nn);
    for (size_t i = 0; i < nn; i++) F[i] = -P->F[s * nn + i];
    memcpy(c, P->c + s * n, sizeof(double) * n);
    const double* K = P->K + s * nn;
    char kt = P->K_type[s];
    bad |= weigh(kt, K, n, n, H, n, n, ws);
    bad |= weigh(kt, K, n, n, F, n, n, ws);
    bad |= weigh(kt, K, n, n, c, n, 1, ws);
  }
  int m = P->obs_rows ? P->obs_rows[s] : 0;
  lv->m[q] = m;
  if (m > 0) {
    double* G = lv->G + q * mx * n;
    double* o = lv->o + q * mx;
    copy_block(G, mx, P->G + s * (size_t)mm * n, mm, m, n);
    memcpy(o, P->o + s * (size_t)mm, sizeof(double) * m);
    const double* C = P->C + s * (size_t)mm * mm;
    char ct = P->C_type[s];
    bad |= weigh(ct, C, mm, m, G, mx, n, ws);
    bad |= weigh(ct, C, mm, m, o, mx, 1, ws);
  }
  return bad;
}

static size_t oe_ws_doubles(int n, int mx)
{
  size_t a = (size_t)(mx + n) * (2 * n + 1), c = (size_t)(2 * mx) * (n + 1), b = (size_t)(2 * n) * (3 * n + 1);
  size_t s = (size_t)mx * (n + 1) + (size_t)(2 * n) * (2 * n + 1) + (size_t)(2 * n) * (n + 1);
  size_t w = (size_t)mx * (mx + 2 * n + 2);
  size_t t = a + b + c;
  if (s > t) t = s;
  if (w > t) t = w;
  return t + 8 * (size_t)n * n + 64;
}

/* Odd-even smoothing of one track (k steps starting at global step s0). */
static int oe_track(uint32_t options, const kalman_gpu_problem_t* P, int64_t s0, int64_t k, int threads)
{
  const int n = P->n;
  const int mx = P->mmax > n ? P->mmax : n;
  const int want_cov = !(options & KALMAN_NO_COVARIANCE) && P->covariance != NULL;
  const size_t nn = (size_t)n * n;
  oout out = {P->state + s0 * n, want_cov ? P->covariance + s0 * nn : NULL, 0};
  if (k <= 0) return 0;
  int status = 0;

  int nlev = 1;
  for (int64_t L = k; L > 1; L /= 2) nlev++;
  olevel* lv = calloc((size_t)nlev, sizeof(olevel));
  olevel_alloc(&lv[0], n, mx, k);
  const size_t wsd = oe_ws_doubles(n, mx);
  int bad = 0;
#pragma omp parallel num_threads(threads) reduction(| : bad)
  {
    double* ws = malloc(sizeof(double) * wsd);
#pragma omp for schedule(static, 16)
    for (int64_t q = 0; q < k; q++) bad |= oe_weigh_step(P, s0 + q, q == 0, &lv[0], q, ws);
    free(ws);
  }
  if (bad) status = KALMAN_GPU_ESINGULAR;

  int d = 0;
  for (; lv[d].L > 1; d++) {
    olevel_alloc(&lv[d + 1], n, mx, lv[d].L / 2);
    const int64_t pairs = lv[d].L / 2;
#pragma omp parallel num_threads(threads)
    {
      double* ws = malloc(sizeof(double) * wsd);
#pragma omp for schedule(static, 16)
      for (int64_t p = 0; p < pairs; p++) oe_pair(&lv[d], &lv[d + 1], p, ws);
      free(ws);
    }
    olevel_free_equations(&lv[d]);
  }
  {
    double* ws = malloc(sizeof(double) * wsd);
    oe_base(&lv[d], d, &out, ws);
    free(ws);
  }
  for (int l = d - 1; l >= 0; l--) {
    if (want_cov) lv[l].U = calloc((size_t)lv[l].L * nn, sizeof(double));
    const int64_t evens = (lv[l].L + 1) / 2;
    int sing = 0;
#pragma omp parallel num_threads(threads) reduction(| : sing)
    {
      double* ws = malloc(sizeof(double) * wsd);
      oout o2 = out;
      o2.singular = 0;
#pragma omp for schedule(static, 16)
      for (int64_t e = 0; e < evens; e++) oe_solve(&lv[l], &lv[l + 1], l, e, &o2, ws, want_cov);
      sing |= o2.singular;
      free(ws);
    }
    out.singular |= sing;
    free(lv[l + 1].U);
    lv[l + 1].U = NULL;
  }
  for (int l = 0; l <= d; l++) olevel_free(&lv[l]);
  free(lv);
  if (out.singular && !status) status = KALMAN_GPU_ESINGULAR;
  return status;
}

/* -------------------------------------------------------------------------- */
/* associative smoother                                                        */
/* -------------------------------------------------------------------------- */

typedef struct {
  double *A, *b, *Z, *e, *J; /* filtering element */
} felem;

/* filtering combine (filteringAssociativeOperation): out = si (x) sj       */
static int assoc_combine_f(int n, const double* Ai, const double* bi, const double* Zi, const double* ei,
                           const double* Ji, const double* Aj, const double* bj, const double* Zj,
                           const double* ej, const double* Jj, double* A, double* b, double* Z, double* e,
                           double* J, double* ws)
{
  const size_t nn = (size_t)n * n;
  double *T = ws, *X = ws + nn, *Yt = ws + 2 * nn, *V = ws + 3 * nn, *v = ws + 4 * nn, *sw = ws + 4 * nn + 2 * n;
  int bad = 0;
  /* X^T = (I + Zi Jj)^{-T} Aj^T */
  gemm(n, n, n, Zi, n, 0, Jj, n, 0, V, n, 0, 1.0);
  for (int i = 0; i < n; i++) V[IDX(i, i, n)] += 1.0;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) T[IDX(i, j, n)] = V[IDX(j, i, n)];
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) X[IDX(i, j, n)] = Aj[IDX(j, i, n)];
  bad |= solve_general(T, n, n, X, n, n, sw); /* X holds X^T */
  /* Y^T = (I + Jj Zi)^{-T} Ai */
  gemm(n, n, n, Jj, n, 0, Zi, n, 0, V, n, 0, 1.0);
  for (int i = 0; i < n; i++) V[IDX(i, i, n)] += 1.0;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) T[IDX(i, j, n)] = V[IDX(j, i, n)];
  for (size_t i = 0; i < nn; i++) Yt[i] = Ai[i];
  bad |= solve_general(T, n, n, Yt, n, n, sw); /* Yt holds Y^T */
  /* A = X Ai */
  gemm(n, n, n, X, n, 1, Ai, n, 0, A, n, 0, 1.0);
  /* b = X (bi + Zi ej) + bj */
  for (int i = 0; i < n; i++) v[i] = bi[i];
  gemm(n, 1, n, Zi, n, 0, ej, n, 0, v, n, 1, 1.0);
  gemm(n, 1, n, X, n, 1, v, n, 0, b, n, 0, 1.0);
  for (int i = 0; i < n; i++) b[i] += bj[i];
  /* Z = X Zi Aj^T + Zj */
  gemm(n, n, n, X, n, 1, Zi, n, 0, V, n, 0, 1.0);
  gemm(n, n, n, V, n, 0, Aj, n, 1, Z, n, 0, 1.0);
  for (size_t i = 0; i < nn; i++) Z[i] += Zj[i];
  /* e = Y (ej - Jj bi) + ei */
  for (int i = 0; i < n; i++) v[i] = ej[i];
  gemm(n, 1, n, Jj, n, 0, bi, n, 0, v, n, 1, -1.0);
  gemm(n, 1, n, Yt, n, 1, v, n, 0, e, n, 0, 1.0);
  for (int i = 0; i < n; i++) e[i] += ei[i];
  /* J = Y Jj Ai + Ji */
  gemm(n, n, n, Jj, n, 0, Ai, n, 0, V, n, 0, 1.0);
  gemm(n, n, n, Yt, n, 1, V, n, 0, J, n, 0, 1.0);
  for (size_t i = 0; i < nn; i++) J[i] += Ji[i];
  return bad;
}

static int as_track(uint32_t options, const kalman_gpu_problem_t* P, int64_t s0, int64_t k)
{
  const int n = P->n, mm = P->mmax;
  const size_t nn = (size_t)n * n;
  const int want_cov = !(options & KALMAN_NO_COVARIANCE) && P->covariance != NULL;
  if (k <= 0) return 0;
  int bad = 0;
  const int mx = mm > n ? mm : n;
  double* ws = malloc(sizeof(double) * (20 * nn + 8 * (size_t)mx * mx + 8 * (size_t)mx * n + 64 * n + 64));
  double* Pf = malloc(sizeof(double) * (size_t)k * nn);  /* filtered covariances */
  double* xf = malloc(sizeof(double) * (size_t)k * n);   /* filtered states      */
  felem cur = {malloc(sizeof(double) * nn), malloc(sizeof(double) * n), malloc(sizeof(double) * nn),
               malloc(sizeof(double) * n), malloc(sizeof(double) * nn)};
  felem el = {malloc(sizeof(double) * nn), malloc(sizeof(double) * n), malloc(sizeof(double) * nn),
              malloc(sizeof(double) * n), malloc(sizeof(double) * nn)};
  felem nw = {malloc(sizeof(double) * nn), malloc(sizeof(double) * n), malloc(sizeof(double) * nn),
              malloc(sizeof(double) * n), malloc(sizeof(double) * nn)};

  /* step 0: QR of the weighted (square) G_0 gives m0 and P0 */
  {
    const int m0 = P->obs_rows ? P->obs_rows[s0] : 0;
    if (m0 != n) { bad = 2; goto done; }
    double* W = ws; /* n x (n+1) */
    copy_block(W, n, P->G + s0 * (size_t)mm * n, mm, n, n);
    copy_block(W + IDX(0, n, n), n, P->o + s0 * (size_t)mm, mm, n, 1);
    double* sw = W + (size_t)n * (n + 1);
    bad |= weigh(P->C_type[s0], P->C + s0 * (size_t)mm * mm, mm, n, W, n, n + 1, sw);
    hh_triangularize(W, n, n, n, n + 1);
    for (int i = 0; i < n; i++) xf[i] = W[IDX(i, n, n)];
    bad |= solve_upper(W, n, n, xf, 1);
    /* P0 = (R^T R)^{-1} = R^{-1} R^{-T} */
    double* Ri = sw;
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) Ri[IDX(i, j, n)] = (i == j) ? 1.0 : 0.0;
    for (int j = 0; j < n; j++) solve_upper(W, n, n, Ri + IDX(0, j, n), 1);
    gemm(n, n, n, Ri, n, 0, Ri, n, 1, Pf, n, 0, 1.0);
  }

  /* sequential filtering scan: element i (i >= 1) combined into cur */
  for (int64_t i = 1; i < k; i++) {
    const int64_t s = s0 + i;
    const double* F = P->F + s * nn;
    const double* c = P->c + s * n;
    double *Kx = ws, *sw = ws + nn;
    bad |= explicit_cov(P->K_type[s], P->K + s * nn, n, n, Kx, sw);
    if (i == 1) { /* K_1 += F P0 F^T */
      double* T = sw;
      gemm(n, n, n, F, n, 0, Pf, n, 0, T, n, 0, 1.0);
      gemm(n, n, n, T, n, 0, F, n, 1, Kx, n, 1, 1.0);
    }
    const int m = P->obs_rows ? P->obs_rows[s] : 0;
    felem* E = (i == 1) ? &cur : &el;
    if (m == 0) {
      memcpy(E->Z, Kx, sizeof(double) * nn);
      if (i == 1) {
        memset(E->A, 0, sizeof(double) * nn);
        for (int r = 0; r < n; r++) E->b[r] = c[r];
        gemm(n, 1, n, F, n, 0, xf, n, 0, E->b, n, 1, 1.0);
      } else {
        memcpy(E->A, F, sizeof(double) * nn);
        memcpy(E->b, c, sizeof(double) * n);
      }
      memset(E->e, 0, sizeof(double) * n);
      memset(E->J, 0, sizeof(double) * nn);
    } else {
      const double* G = P->G + s * (size_t)mm * n;
      const double* o = P->o + s * (size_t)mm;
      double* Cx = sw;                       /* m x m */
      double* S = Cx + (size_t)m * m;        /* m x m */
      double* KGt = S + (size_t)m * m;       /* n x m */
      double* GtS = KGt + (size_t)n * m;     /* n x m: G^T S^{-1} */
      double* Kg = GtS + (size_t)n * m;      /* n x m: gain       */
      double* r = Kg + (size_t)n * m;        /* m                 */
      double* T = r + mx;                    /* n x n             */
      double* T2 = T + nn;                   /* n x n             */
      double* sw2 = T2 + nn;
      bad |= explicit_cov(P->C_type[s], P->C + s * (size_t)mm * mm, mm, m, Cx, sw2);
      gemm(n, m, n, Kx, n, 0, G, mm, 1, KGt, n, 0, 1.0);          /* K G^T        */
      gemm(m, m, n, G, mm, 0, KGt, n, 0, S, m, 0, 1.0);           /* G K G^T      */
      for (size_t q = 0; q < (size_t)m * m; q++) S[q] += Cx[q];
      /* G^T S^{-1} = (S^{-T} G)^T */
      double* St = Cx; /* reuse: S^T */
      for (int a = 0; a < m; a++)
        for (int b2 = 0; b2 < m; b2++) St[IDX(a, b2, m)] = S[IDX(b2, a, m)];
      double* SG = sw2; /* m x n */
      copy_block(SG, m, G, mm, m, n);
      bad |= solve_general(St, m, m, SG, m, n, sw2 + (size_t)m * n);
      for (int a = 0; a < n; a++)
        for (int b2 = 0; b2 < m; b2++) GtS[IDX(a, b2, n)] = SG[IDX(b2, a, m)];
      gemm(n, m, n, Kx, n, 0, GtS, n, 0, Kg, n, 0, 1.0);          /* gain          */
      if (i == 1) {
        memset(E->A, 0, sizeof(double) * nn);
        double* m1 = T; /* F m0 + c */
        for (int q = 0; q < n; q++) m1[q] = c[q];
        gemm(n, 1, n, F, n, 0, xf, n, 0, m1, n, 1, 1.0);
        for (int q = 0; q < m; q++) r[q] = o[q];
        gemm(m, 1, n, G, mm, 0, m1, n, 0, r, m, 1, -1.0);
        for (int q = 0; q < n; q++) E->b[q] = m1[q];
        gemm(n, 1, m, Kg, n, 0, r, m, 0, E->b, n, 1, 1.0);
        double* KS = sw2; /* n x m */
        gemm(n, m, m, Kg, n, 0, S, m, 0, KS, n, 0, 1.0);
        memcpy(E->Z, Kx, sizeof(double) * nn);
        gemm(n, n, m, KS, n, 0, Kg, n, 1, E->Z, n, 1, -1.0);
      } else {
        double* GF = sw2; /* m x n */
        gemm(m, n, n, G, mm, 0, F, n, 0, GF, m, 0, 1.0);
        memcpy(E->A, F, sizeof(double) * nn);
        gemm(n, n, m, Kg, n, 0, GF, m, 0, E->A, n, 1, -1.0);
        for (int q = 0; q < m; q++) r[q] = o[q];
        gemm(m, 1, n, G, mm, 0, c, n, 0, r, m, 1, -1.0);
        for (int q = 0; q < n; q++) E->b[q] = c[q];
        gemm(n, 1, m, Kg, n, 0, r, m, 0, E->b, n, 1, 1.0);
        double* KG = T; /* n x n */
        gemm(n, n, m, Kg, n, 0, G, mm, 0, KG, n, 0, 1.0);
        memcpy(E->Z, Kx, sizeof(double) * nn);
        gemm(n, n, n, KG, n, 0, Kx, n, 0, E->Z, n, 1, -1.0);
      }
      /* e = F^T G^T S^{-1} (o - G c), J = F^T G^T S^{-1} G F */
      for (int q = 0; q < m; q++) r[q] = o[q];
      gemm(m, 1, n, G, mm, 0, c, n, 0, r, m, 1, -1.0);
      double* FtGtS = sw2; /* n x m */
      gemm(n, m, n, F, n, 1, GtS, n, 0, FtGtS, n, 0, 1.0);
      gemm(n, 1, m, FtGtS, n, 0, r, m, 0, E->e, n, 0, 1.0);
      double* GF = FtGtS + (size_t)n * m;
      gemm(m, n, n, G, mm, 0, F, n, 0, GF, m, 0, 1.0);
      gemm(n, n, m, FtGtS, n, 0, GF, m, 0, E->J, n, 0, 1.0);
    }
    if (i > 1) {
      bad |= assoc_combine_f(n, cur.A, cur.b, cur.Z, cur.e, cur.J, el.A, el.b, el.Z, el.e, el.J, nw.A, nw.b,
                             nw.Z, nw.e, nw.J, ws + 2 * nn);
      felem t = cur; cur = nw; nw = t;
    }
    memcpy(xf + i * n, cur.b, sizeof(double) * n);
    memcpy(Pf + i * nn, cur.Z, sizeof(double) * nn);
  }

  /* smoothing: the last step keeps its filtered estimate; then the reverse
     scan, which sequentially is g_acc <- E_i g_acc + g_i, L <- E_i L E_i^T + L_i */
  {
    double* xs = P->state + s0 * n;
    double* Ps = want_cov ? P->covariance + s0 * nn : NULL;
    double *Eacc = ws, *gacc = ws + nn, *Lacc = ws + nn + n;
    double *Ei = Lacc + nn, *gi = Ei + nn, *Li = gi + n, *T = Li + nn, *T2 = T + nn, *sw = T2 + nn;
    (void)Eacc;
    memcpy(gacc, xf + (k - 1) * n, sizeof(double) * n);
    memcpy(Lacc, Pf + (k - 1) * nn, sizeof(double) * nn);
    memcpy(xs + (k - 1) * n, gacc, sizeof(double) * n);
    if (Ps) memcpy(Ps + (k - 1) * nn, Lacc, sizeof(double) * nn);
    for (int64_t i = k - 2; i >= 0; i--) {
      const int64_t s = s0 + i + 1;
      const double* F = P->F + s * nn;
      const double* c = P->c + s * n;
      const double* Pi = Pf + i * nn;
      const double* xi = xf + i * n;
      double* Q = sw;
      bad |= explicit_cov(P->K_type[s], P->K + s * nn, n, n, Q, sw + nn);
      /* E = P F^T (F P F^T + Q)^{-1};  E^T = (F P F^T + Q)^{-T} (P F^T)^T */
      double* PFt = T;
      gemm(n, n, n, Pi, n, 0, F, n, 1, PFt, n, 0, 1.0);
      double* Mq = T2;
      memcpy(Mq, Q, sizeof(double) * nn);
      gemm(n, n, n, F, n, 0, PFt, n, 0, Mq, n, 1, 1.0);
      double* Mt = sw + nn; /* (F P F^T + Q)^T */
      for (int a = 0; a < n; a++)
        for (int b2 = 0; b2 < n; b2++) Mt[IDX(a, b2, n)] = Mq[IDX(b2, a, n)];
      double* Et = Mq; /* (P F^T)^T */
      for (int a = 0; a < n; a++)
        for (int b2 = 0; b2 < n; b2++) Et[IDX(a, b2, n)] = PFt[IDX(b2, a, n)];
      bad |= solve_general(Mt, n, n, Et, n, n, sw + 2 * nn);
      for (int a = 0; a < n; a++)
        for (int b2 = 0; b2 < n; b2++) Ei[IDX(a, b2, n)] = Et[IDX(b2, a, n)];
      /* g = x - E (F x + c) */
      double* v = T;
      for (int q = 0; q < n; q++) v[q] = c[q];
      gemm(n, 1, n, F, n, 0, xi, n, 0, v, n, 1, 1.0);
      for (int q = 0; q < n; q++) gi[q] = xi[q];
      gemm(n, 1, n, Ei, n, 0, v, n, 0, gi, n, 1, -1.0);
      /* L = P - E F P */
      double* EF = T;
      gemm(n, n, n, Ei, n, 0, F, n, 0, EF, n, 0, 1.0);
      memcpy(Li, Pi, sizeof(double) * nn);
      gemm(n, n, n, EF, n, 0, Pi, n, 0, Li, n, 1, -1.0);
      /* combine with the accumulated later elements */
      double* g2 = T2;
      memcpy(g2, gi, sizeof(double) * n);
      gemm(n, 1, n, Ei, n, 0, gacc, n, 0, g2, n, 1, 1.0);
      memcpy(gacc, g2, sizeof(double) * n);
      double* EL = T;
      gemm(n, n, n, Ei, n, 0, Lacc, n, 0, EL, n, 0, 1.0);
      memcpy(T2, Li, sizeof(double) * nn);
      gemm(n, n, n, EL, n, 0, Ei, n, 1, T2, n, 1, 1.0);
      memcpy(Lacc, T2, sizeof(double) * nn);
      memcpy(xs + i * n, gacc, sizeof(double) * n);
      if (Ps) memcpy(Ps + i * nn, Lacc, sizeof(double) * nn);
    }
  }
done:
  free(cur.A); free(cur.b); free(cur.Z); free(cur.e); free(cur.J);
  free(el.A); free(el.b); free(el.Z); free(el.e); free(el.J);
  free(nw.A); free(nw.b); free(nw.Z); free(nw.e); free(nw.J);
  free(ws); free(Pf); free(xf);
  if (bad == 2) return KALMAN_GPU_EINVAL;
  return bad ? KALMAN_GPU_ESINGULAR : 0;
}

/* -------------------------------------------------------------------------- */
/* entry points (called through ctypes by tests/ and bench.py)                */
/* -------------------------------------------------------------------------- */

/* Odd-even smoothing of every track.  threads <= 0: all available.  A single
 * track runs each level in parallel (as the reference's foreach_in_range);
 * several tracks run in parallel, one track per thread.                      */
int oracle_smooth_oddeven(uint32_t options, const kalman_gpu_problem_t* P, int threads)
{
  int nt = oe_nthreads(threads), status = 0;
  if (P->ntracks == 1) return oe_track(options, P, P->track_start[0], P->track_start[1] - P->track_start[0], nt);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt) reduction(max : status)
  for (int t = 0; t < P->ntracks; t++) {
    int s = oe_track(options, P, P->track_start[t], P->track_start[t + 1] - P->track_start[t], 1);
    if (s > status) status = s;
  }
  return status;
}

int oracle_smooth_associative(uint32_t options, const kalman_gpu_problem_t* P, int threads)
{
  int nt = oe_nthreads(threads), status = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt) reduction(max : status)
  for (int t = 0; t < P->ntracks; t++) {
    int s = as_track(options, P, P->track_start[t], P->track_start[t + 1] - P->track_start[t]);
    if (s > status) status = s;
  }
  return status;
}

int oracle_max_threads(void) { return oe_nthreads(0); }
