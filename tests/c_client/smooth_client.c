/*
 * smooth_client.c -- a plain C client of libukgpu.so that uses only the
 * reference API of kalman.h / matrix_ops.h, the way a program written against
 * UltimateKalman's C library does (c/kalman.h:117-131): kalman_create_options,
 * one kalman_evolve + kalman_observe per step (the first step evolves with
 * its dimension only), kalman_smooth, then kalman_estimate /
 * kalman_covariance per step, every returned matrix freed with matrix_free.
 * The test suite compiles it with gcc against include/ and links it with
 * -lukgpu; nothing of the library's own additions is used except
 * kalman_gpu_last_status / kalman_gpu_last_error to report failures.
 *
 * usage: smooth_client IN OUT oddeven|associative
 *   IN  (native-endian binary): int32 n, int32 k, then per step s:
 *        s > 0: H, F (n x n), c (n), char K_type, K (n x n, or n x 1 for 'w')
 *        int32 m; if m > 0: G (m x n), o (m), char C_type, C (m x m or m x 1)
 *        matrices column-major FP64
 *   OUT: int32 status, then per step the state (n) and covariance (n x n,
 *        column-major)
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "kalman.h"
#include "kalman_gpu.h"
#include "matrix_ops.h"

static int read_exact(FILE* f, void* p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

static kalman_matrix_t* read_matrix(FILE* f, int rows, int cols)
{
  kalman_matrix_t* A = matrix_create(rows, cols);
  for (int j = 0; j < cols; ++j)
    for (int i = 0; i < rows; ++i) {
      double v;
      if (!read_exact(f, &v, sizeof v)) {
        matrix_free(A);
        return NULL;
      }
      A->elements[(size_t)j * A->ld + i] = v;
    }
  return A;
}

int main(int argc, char** argv)
{
  if (argc != 4) {
    fprintf(stderr, "usage: %s IN OUT oddeven|associative\n", argv[0]);
    return 2;
  }
  FILE* in = fopen(argv[1], "rb");
  if (!in) return 2;
  int32_t n = 0, k = 0;
  if (!read_exact(in, &n, 4) || !read_exact(in, &k, 4) || n < 1 || k < 1) return 2;
  const uint32_t alg = strcmp(argv[3], "associative") == 0 ? KALMAN_ALGORITHM_ASSOCIATIVE : KALMAN_ALGORITHM_ODDEVEN;
  kalman_t* kf = kalman_create_options(alg);
  if (!kf) return 3;
  for (int32_t s = 0; s < k; ++s) {
    if (s == 0) {
      kalman_evolve(kf, n, NULL, NULL, NULL, NULL, 'C');
    } else {
      kalman_matrix_t* H = read_matrix(in, n, n);
      kalman_matrix_t* F = read_matrix(in, n, n);
      kalman_matrix_t* c = read_matrix(in, n, 1);
      char kt = 0;
      if (!H || !F || !c || !read_exact(in, &kt, 1)) return 2;
      kalman_matrix_t* K = read_matrix(in, n, kt == 'w' ? 1 : n);
      if (!K) return 2;
      kalman_evolve(kf, n, H, F, c, K, kt);
      matrix_free(H);
      matrix_free(F);
      matrix_free(c);
      matrix_free(K);
    }
    int32_t m = 0;
    if (!read_exact(in, &m, 4)) return 2;
    if (m > 0) {
      kalman_matrix_t* G = read_matrix(in, m, n);
      kalman_matrix_t* o = read_matrix(in, m, 1);
      char ct = 0;
      if (!G || !o || !read_exact(in, &ct, 1)) return 2;
      kalman_matrix_t* C = read_matrix(in, m, ct == 'w' ? 1 : m);
      if (!C) return 2;
      kalman_observe(kf, G, o, C, ct);
      matrix_free(G);
      matrix_free(o);
      matrix_free(C);
    } else {
      kalman_observe(kf, NULL, NULL, NULL, 'C');
    }
  }
  fclose(in);
  kalman_smooth(kf);
  const int32_t status = kalman_gpu_last_status();
  FILE* out = fopen(argv[2], "wb");
  if (!out) return 2;
  fwrite(&status, 4, 1, out);
  for (int32_t s = 0; s < k; ++s) {
    kalman_matrix_t* x = kalman_estimate(kf, s);
    kalman_matrix_t* P = kalman_covariance(kf, s);
    for (int i = 0; i < n; ++i) {
      const double v = x ? x->elements[i] : kalman_nan;
      fwrite(&v, 8, 1, out);
    }
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double v = P ? P->elements[(size_t)j * P->ld + i] : kalman_nan;
        fwrite(&v, 8, 1, out);
      }
    if (x) matrix_free(x);
    if (P) matrix_free(P);
  }
  fclose(out);
  printf("status %d: %s\n", status, status ? kalman_gpu_last_error() : "ok");
  kalman_free(kf);
  return 0;
}
