/*
 * filter.cu -- filtered estimates on the device: the sequential UltimateKalman
 * filter (c/kalman_ultimate.c: evolve 140-330, observe 332-470, estimate
 * 472-557) run for every track of a packed problem at once, one thread block
 * per track (kalman_gpu_filter_packed).
 *
 * Per track the block keeps the factor of the current state's information,
 * an upper-trapezoidal R (z rows, z <= n) and its right-hand side y:
 *   evolve to step i   QR, eliminating x_{i-1}, of
 *                        [ R        0     | y    ]   (z rows)
 *                        [ -V F_i   V H_i | V c_i ]   (n rows; V from K_i)
 *                      the last z rows become [R~ | y~] for x_i;
 *   observe            QR of [R~ | y~; W G_i | W o_i] (W from C_i; no rows
 *                      when the step is unobserved) -> R, y with
 *                      z = min(z + m_i, n) rows;
 *   estimate           x_{i|i} = R^{-1} y and P_{i|i} = R^{-1} R^{-T} once
 *                      z = n (NaN before, as the reference's estimate).
 * The QR reductions, weighing and triangular solves are the CTA routines of
 * the smoothers (cta_linalg.cuh).  FP64.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include <cuda_runtime.h>

#include "cta_linalg.cuh"
#include "profiling.h"
#include "ukgpu_internal.h"

namespace {

using cta::NT;

struct FilterArgs {
  int n, mmax, ntracks;
  const int64_t* track_start; /* device */
  const double *H, *F, *c, *K, *G, *o, *C;
  const char *K_type, *C_type;
  const int32_t* obs_rows;
  double* state;
  double* cov; /* may be null */
  double* scratch;
  int64_t per_cta;
  int* flag; /* 1: an estimate was undetermined (NaN written), 4: malformed input */
};

/* per-CTA scratch: the evolve panel (z + n) x (2n + 1), the observe panel
 * (n + mmax) x (n + 1), the weighing factor rmax^2 and product tmp, R^{-1} */
int64_t filter_scratch(int n, int mmax)
{
  const int64_t rmax = n > mmax ? n : mmax;
  const int64_t evolve = 2 * (int64_t)n * (2 * n + 1);
  const int64_t observe = (int64_t)(n + mmax) * (n + 1);
  const int64_t weigh = rmax * rmax + rmax * NT;
  return evolve + observe + weigh + (int64_t)n * n + 32;
}

__global__ void __launch_bounds__(NT) filter_cta(FilterArgs a)
{
  __shared__ double red[33];
  __shared__ int zs;
  const int n = a.n, mm = a.mmax, tid = threadIdx.x;
  const int64_t nn = (int64_t)n * n;
  const int le = 2 * n + 1, lo = n + 1;
  double* E = a.scratch + (int64_t)blockIdx.x * a.per_cta; /* evolve panel, row-major, ld le */
  double* O = E + 2 * (int64_t)n * le;                      /* observe panel, row-major, ld lo */
  double* Lw = O + (int64_t)(n + mm) * lo;                   /* weighing factor */
  double* tmp = Lw + (int64_t)(n > mm ? n : mm) * (n > mm ? n : mm);
  double* Ri = tmp + (int64_t)(n > mm ? n : mm) * NT;       /* R^{-1}, row-major */
  for (int t = blockIdx.x; t < a.ntracks; t += gridDim.x) {
    const int64_t s0 = a.track_start[t], s1 = a.track_start[t + 1];
    int z = 0; /* rows of the current factor, held in O's first rows as [R | y] */
    for (int64_t s = s0; s < s1; ++s) {
      bool bad = false;
      if (s > s0) { /* evolve: [R 0 | y; -V F  V H | V c], n pivots */
        for (int e = tid; e < z * le; e += NT) {
          const int r = e / le, q = e - r * le;
          /* R's upper triangle only: the QR that made it keeps its reflectors below */
          E[e] = q < n ? (q >= r ? O[(int64_t)r * lo + q] : 0.0) : q < 2 * n ? 0.0 : O[(int64_t)r * lo + n];
        }
        double* B = E + (int64_t)z * le;
        for (int e = tid; e < n * le; e += NT) {
          const int r = e / le, q = e - r * le;
          B[e] = q < n ? -a.F[s * nn + (int64_t)q * n + r]
                       : q < 2 * n ? a.H[s * nn + (int64_t)(q - n) * n + r] : a.c[s * n + r];
        }
        __syncthreads();
        const char kt = a.K_type[s];
        if (tid == 0 && !cta::valid_cov_type(kt)) atomicOr(a.flag, 4);
        bad |= !cta::weigh_panel(kt, a.K + s * nn, n, n, B, le, le, Lw, red, tmp);
        cta::householder(E, le, z + n, n, le, red);
        /* the last z rows: [0 | R~ | y~] -> O's first z rows */
        for (int e = tid; e < z * lo; e += NT) {
          const int r = e / lo, q = e - r * lo;
          O[e] = E[(int64_t)(n + r) * le + n + q];
        }
        __syncthreads();
      }
      /* observe: [R~ | y~ (z rows); W G | W o (m rows)], n pivots */
      int m = a.obs_rows[s];
      if (m < 0 || m > mm) {
        if (tid == 0) atomicOr(a.flag, 4);
        m = 0;
      }
      if (m > 0) {
        double* B = O + (int64_t)z * lo;
        for (int e = tid; e < m * lo; e += NT) {
          const int r = e / lo, q = e - r * lo;
          B[e] = q < n ? a.G[s * (int64_t)mm * n + (int64_t)q * mm + r] : a.o[s * mm + r];
        }
        __syncthreads();
        const char ct = a.C_type[s];
        if (tid == 0 && !cta::valid_cov_type(ct)) atomicOr(a.flag, 4);
        bad |= !cta::weigh_panel(ct, a.C + s * (int64_t)mm * mm, mm, m, B, lo, lo, Lw, red, tmp);
      }
      const int rows = z + m;
      if (rows > 0) cta::householder(O, lo, rows, n, lo, red);
      z = rows < n ? rows : n; /* rows below the factor are the residual, dropped */
      if (bad && tid == 0) atomicOr(a.flag, 1);
      /* estimate */
      if (tid == 0) {
        int ok = z == n;
        for (int i = 0; ok && i < n; ++i)
          if (O[(int64_t)i * lo + i] == 0.0) ok = 0;
        zs = ok;
      }
      __syncthreads();
      double* x = a.state + s * n;
      double* P = a.cov ? a.cov + s * nn : nullptr;
      if (!zs) {
        for (int i = tid; i < n; i += NT) x[i] = NAN;
        if (P)
          for (int e = tid; e < nn; e += NT) P[e] = NAN;
        if (tid == 0) atomicOr(a.flag, 1);
        __syncthreads();
        continue;
      }
      /* x = R^{-1} y, with y copied out of the panel (the panel stays the factor) */
      double* yv = tmp;
      for (int i = tid; i < n; i += NT) yv[i] = O[(int64_t)i * lo + n];
      __syncthreads();
      cta::solve_upper_vec(O, lo, n, yv);
      for (int i = tid; i < n; i += NT) x[i] = yv[i];
      if (P) { /* P = R^{-1} R^{-T}, column-major out */
        for (int e = tid; e < nn; e += NT) Ri[e] = (e / n == e % n) ? 1.0 : 0.0;
        __syncthreads();
        cta::solve_upper_cols(O, lo, n, Ri, n, 0, n);
        for (int e = tid; e < nn; e += NT) {
          const int r = e / n, q = e - r * n;
          double sm = 0.0;
          for (int k = (r > q ? r : q); k < n; ++k) sm = fma(Ri[(int64_t)r * n + k], Ri[(int64_t)q * n + k], sm);
          P[(int64_t)q * n + r] = sm;
        }
      }
      __syncthreads();
    }
  }
}

struct Workspace {
  void* p = nullptr;
  size_t bytes = 0;
};
thread_local Workspace tl_ws;

int ensure(size_t bytes)
{
  if (tl_ws.bytes >= bytes) return 0;
  if (tl_ws.p) cudaFree(tl_ws.p);
  tl_ws.p = nullptr;
  tl_ws.bytes = 0;
  if (cudaMalloc(&tl_ws.p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return ukg_set_error(KALMAN_GPU_ENOMEM, "filter workspace of %zu bytes", bytes);
  }
  tl_ws.bytes = bytes;
  return 0;
}

}  // namespace

extern "C" void ukg_release_filter_workspace(void)
{
  if (tl_ws.p) cudaFree(tl_ws.p);
  tl_ws = Workspace{};
}

extern "C" int kalman_gpu_filter_packed(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream)
{
  ukg_clear_error();
  const bool want_cov = !(options & (1u << 16)) && p && p->covariance;
  if (int e = ukg_validate_problem(p, 0)) return e;
  if (p->location != KALMAN_GPU_DEVICE)
    return ukg_set_error(KALMAN_GPU_EINVAL, "filter: the problem's arrays must be device arrays");
  if (p->n > cta::kMaxCov || p->mmax > cta::kMaxCov)
    return ukg_set_error(KALMAN_GPU_EINVAL, "filter: state dimension %d / observation rows %d above %d", p->n,
                         p->mmax, cta::kMaxCov);
  if (p->nsteps == 0) return KALMAN_GPU_OK;
  cudaStream_t st = (cudaStream_t)cuda_stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int ncta = p->ntracks < sms * 4 ? p->ntracks : sms * 4;
  const int64_t per = filter_scratch(p->n, p->mmax);
  const size_t tab = ((size_t)(p->ntracks + 1) * sizeof(int64_t) + 255) / 256 * 256;
  if (int e = ensure(tab + 256 + (size_t)ncta * per * sizeof(double))) return e;
  char* base = (char*)tl_ws.p;
  int64_t* dts = (int64_t*)base;
  int* dflag = (int*)(base + tab);
  cudaMemcpyAsync(dts, p->track_start, (size_t)(p->ntracks + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(dflag, 0, sizeof(int), st);
  FilterArgs a;
  a.n = p->n;
  a.mmax = p->mmax;
  a.ntracks = p->ntracks;
  a.track_start = dts;
  a.H = p->H;
  a.F = p->F;
  a.c = p->c;
  a.K = p->K;
  a.G = p->G;
  a.o = p->o;
  a.C = p->C;
  a.K_type = p->K_type;
  a.C_type = p->C_type;
  a.obs_rows = p->obs_rows;
  a.state = p->state;
  a.cov = want_cov ? p->covariance : nullptr;
  a.scratch = (double*)(base + tab + 256);
  a.per_cta = per;
  a.flag = dflag;
  UKG_LAUNCH(UKG_K_FILTER, st, (filter_cta<<<ncta, NT, 0, st>>>(a)));
  int hflag = 0;
  cudaMemcpyAsync(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return ukg_set_error(KALMAN_GPU_ECUDA, "filter: %s", cudaGetErrorString(e));
  if (hflag & 4) return ukg_set_error(KALMAN_GPU_EINVAL, "filter: malformed input (observation rows or covariance types)");
  if (hflag & 1)
    return ukg_set_error(KALMAN_GPU_ESINGULAR, "filter: some steps' states are not yet determined (NaN written there)");
  return KALMAN_GPU_OK;
}
