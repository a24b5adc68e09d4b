/*
 * filter.cu -- filtered estimates on the device: the sequential UltimateKalman
 * filter (c/kalman_ultimate.c: evolve 140-345, observe 347-557 with its
 * estimate 508-545) run for every track of a packed problem at once, one
 * thread block per track (kalman_gpu_filter_packed).  The reference keeps the
 * covariance as the factor R (its covariance_type 'W'); here P = R^{-1} R^{-T}
 * is written explicitly, as the smoothers write theirs.
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

/* ---------------------------------------------------------------------------
 * Small states (n, mmax <= 8): one warp per track, lane j holding column j of
 * the current panel in registers (fixed shapes, unused rows exactly zero, so
 * no row counts reach register indices):
 *   evolve panel  rows 0..N-1 the weighed [-F | H | c], rows N..2N-1 the
 *                 carried [R | 0 | y] (zero rows past z), N pivots; rows
 *                 N..2N-1 of columns N..2N are the information on x_i
 *   observe panel rows 0..N-1 that information (shifted to lanes 0..N), rows
 *                 N..N+7 the weighed [G | o] (zero past m), N pivots
 * Reflectors are formed by the pivot column's lane and broadcast by shuffles.
 * Weighing factors, R and R^{-1} for the estimate go through a small
 * per-warp shared-memory area.
 * ------------------------------------------------------------------------ */
constexpr int kWarpsPerBlock = 4;
constexpr int kWarpMaxN = 8;

/* QR with NP pivots of the panel held as one column per lane (R rows, NC
 * columns: lanes from NC on hold nothing and stay idle) */
template <int R, int NP, int NC>
__device__ __forceinline__ void warp_qr(double (&col)[R], int lane)
{
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    double tail = 0.0;
#pragma unroll
    for (int i = k + 1; i < R; ++i) tail = fma(col[i], col[i], tail);
    tail = __shfl_sync(0xffffffffu, tail, k);
    const double alpha = __shfl_sync(0xffffffffu, col[k], k);
    if (tail == 0.0) continue; /* identity reflector: uniform over the warp */
    const double beta = -copysign(sqrt(fma(alpha, alpha, tail)), alpha);
    const double amb = alpha - beta;
    const double inv = 1.0 / (beta * amb);
    const double t = -(amb * amb) * inv, scale = beta * inv;
    double v[R];
#pragma unroll
    for (int i = k + 1; i < R; ++i) v[i] = __shfl_sync(0xffffffffu, col[i], k) * scale;
    if (lane == k) {
      col[k] = beta;
#pragma unroll
      for (int i = k + 1; i < R; ++i) col[i] = v[i];
    } else if (lane > k && lane < NC) {
      double d = col[k];
#pragma unroll
      for (int i = k + 1; i < R; ++i) d = fma(v[i], col[i], d);
      d *= t;
      col[k] -= d;
#pragma unroll
      for (int i = k + 1; i < R; ++i) col[i] = fma(-d, v[i], col[i]);
    }
  }
}

/* rows r0 .. r0+rows-1 of this lane's column <- V (those rows) for the factor
 * of a covariance (column-major, ld ldc): 'W' W x, 'w' diag x, 'C'
 * chol(cov)^{-1} x, 'U'/'F' tril(cov)^{-1} x.  sL: rows^2 doubles of the
 * warp's shared area.  Returns false for a factor that is not positive
 * definite or has a zero pivot (the same in every lane). */
template <int R, int R0, int MAXR>
__device__ __forceinline__ bool warp_weigh(double (&col)[R], char type, const double* cov, int ldc, int rows,
                                           double* sL, double* sInv, int lane, int ncols)
{
  bool ok = true;
  const bool act = lane < ncols; /* lanes past the panel's columns hold zeros */
  if (type == 'w') {
#pragma unroll
    for (int i = 0; i < MAXR; ++i)
      if (act && i < rows) col[R0 + i] *= cov[i];
    return true;
  }
  if (type == 'W') {
    if (!act) return true;
    double x[MAXR];
#pragma unroll
    for (int i = 0; i < MAXR; ++i) {
      double sm = 0.0;
#pragma unroll
      for (int k = 0; k < MAXR; ++k)
        if (i < rows && k < rows) sm = fma(cov[(int64_t)k * ldc + i], col[R0 + k], sm);
      x[i] = sm;
    }
#pragma unroll
    for (int i = 0; i < MAXR; ++i)
      if (i < rows) col[R0 + i] = x[i];
    return true;
  }
  if (type != 'C' && type != 'U' && type != 'F') return true;
  /* the factor, column-major rows x rows, lower triangle */
  for (int e = lane; e < rows * rows; e += 32) {
    const int j = e / rows, i = e - j * rows;
    sL[e] = i >= j ? cov[(int64_t)j * ldc + i] : 0.0;
  }
  __syncwarp();
  if (type == 'C') {
    if (lane == 0) /* Cholesky by one lane: at most 8 x 8; one division per column */
      for (int j = 0; j < rows; ++j) {
        double d = sL[j * rows + j];
        for (int k = 0; k < j; ++k) d = fma(-sL[k * rows + j], sL[k * rows + j], d);
        const bool pd = d > 0.0;
        const double ljj = pd ? sqrt(d) : 1.0;
        const double ri = 1.0 / ljj;
        sL[j * rows + j] = pd ? ljj : -1.0; /* -1 marks a failed pivot (sqrt >= 0 otherwise) */
        sInv[j] = ri;
        for (int i = j + 1; i < rows; ++i) {
          double x = sL[j * rows + i];
          for (int k = 0; k < j; ++k) x = fma(-sL[k * rows + i], sL[k * rows + j], x);
          sL[j * rows + i] = x * ri;
        }
      }
    __syncwarp();
    for (int j = 0; j < rows; ++j)
      if (sL[j * rows + j] < 0.0) ok = false;
  } else {
    if (lane < rows) sInv[lane] = 1.0 / sL[lane * rows + lane];
    __syncwarp();
    for (int j = 0; j < rows; ++j)
      if (sL[j * rows + j] == 0.0) ok = false;
  }
  /* forward substitution on this lane's rows */
#pragma unroll
  for (int i = 0; i < MAXR; ++i)
    if (act && i < rows) {
      double x = col[R0 + i];
#pragma unroll
      for (int k = 0; k < MAXR; ++k)
        if (k < i) x = fma(-sL[k * rows + i], col[R0 + k], x);
      col[R0 + i] = x * sInv[i];
    }
  __syncwarp();
  return ok;
}

template <int N>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) filter_warp(FilterArgs a)
{
  constexpr int RE = 2 * N, RO = N + kWarpMaxN;
  __shared__ double area[kWarpsPerBlock][kWarpMaxN * kWarpMaxN + 2 * N * N + N + kWarpMaxN + N];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int t = blockIdx.x * kWarpsPerBlock + w;
  if (t >= a.ntracks) return; /* uniform over the warp */
  double* sL = area[w];
  double* sR = sL + kWarpMaxN * kWarpMaxN; /* R, column-major N x N */
  double* sRi = sR + N * N;                 /* R^{-1}, column-major */
  double* sy = sRi + N * N;
  double* sInv = sy + N;          /* reciprocal pivots of the weighing factor */
  double* sInvR = sInv + kWarpMaxN; /* reciprocal diagonal of R */
  const int mm = a.mmax;
  const int64_t nn = (int64_t)N * N;
  const int64_t s0 = a.track_start[t], s1 = a.track_start[t + 1];
  double Rc[N]; /* this lane's column of the carried [R | y] (lanes 0..N), zero rows past z */
#pragma unroll
  for (int r = 0; r < N; ++r) Rc[r] = 0.0;
  int z = 0;
  int flag = 0;
  for (int64_t s = s0; s < s1; ++s) {
    double oc[RO]; /* the observe panel: lanes 0..N-1 R~'s columns, lane N y~ */
    if (s > s0) {
      double ec[RE];
      /* rows 0..N-1: [-F | H | c] of step s; rows N..2N-1: [R | 0 | y] */
#pragma unroll
      for (int r = 0; r < N; ++r) {
        double v = 0.0;
        if (lane < N) v = -a.F[s * nn + (int64_t)lane * N + r];
        else if (lane < 2 * N) v = a.H[s * nn + (int64_t)(lane - N) * N + r];
        else if (lane == 2 * N) v = a.c[s * N + r];
        ec[r] = v;
      }
#pragma unroll
      for (int r = 0; r < N; ++r) {
        const double yr = __shfl_sync(0xffffffffu, Rc[r], N);
        ec[N + r] = lane < N ? Rc[r] : lane == 2 * N ? yr : 0.0;
      }
      const char kt = a.K_type[s];
      if (!cta::valid_cov_type(kt)) flag |= 4;
      if (!warp_weigh<RE, 0, N>(ec, kt, a.K + s * nn, N, N, sL, sInv, lane, 2 * N + 1)) flag |= 1;
      warp_qr<RE, N, 2 * N + 1>(ec, lane);
      /* rows N..2N-1 of lanes N..2N -> lanes 0..N */
#pragma unroll
      for (int r = 0; r < N; ++r) oc[r] = __shfl_sync(0xffffffffu, ec[N + r], (lane + N) & 31);
      if (lane > N) {
#pragma unroll
        for (int r = 0; r < N; ++r) oc[r] = 0.0;
      }
    } else {
#pragma unroll
      for (int r = 0; r < N; ++r) oc[r] = 0.0;
    }
    int m = a.obs_rows[s];
    if (m < 0 || m > mm || m > kWarpMaxN) {
      flag |= 4;
      m = 0;
    }
#pragma unroll
    for (int r = 0; r < kWarpMaxN; ++r) {
      double v = 0.0;
      if (r < m) {
        if (lane < N) v = a.G[s * (int64_t)mm * N + (int64_t)lane * mm + r];
        else if (lane == N) v = a.o[s * mm + r];
      }
      oc[N + r] = v;
    }
    if (m > 0) {
      const char ct = a.C_type[s];
      if (!cta::valid_cov_type(ct)) flag |= 4;
      if (!warp_weigh<RO, N, kWarpMaxN>(oc, ct, a.C + s * (int64_t)mm * mm, mm, m, sL, sInv, lane, N + 1)) flag |= 1;
    }
    warp_qr<RO, N, N + 1>(oc, lane);
#pragma unroll
    for (int r = 0; r < N; ++r) Rc[r] = (lane <= N && (lane == N || r <= lane)) ? oc[r] : 0.0;
    z = z + m < N ? z + m : N;
    /* estimate */
    double* x = a.state + s * N;
    double* P = a.cov ? a.cov + s * nn : nullptr;
    bool det = z == N;
    if (lane < N) {
#pragma unroll
      for (int r = 0; r < N; ++r) sR[lane * N + r] = Rc[r];
    } else if (lane == N) {
#pragma unroll
      for (int r = 0; r < N; ++r) sy[r] = Rc[r];
    }
    __syncwarp();
    for (int i = 0; i < N; ++i)
      if (sR[i * N + i] == 0.0) det = false;
    if (!det) {
      if (lane < N) x[lane] = NAN;
      if (P)
        for (int e = lane; e < N * N; e += 32) P[e] = NAN;
      flag |= 1;
      __syncwarp();
      continue;
    }
    if (lane < N) sInvR[lane] = 1.0 / sR[lane * N + lane];
    __syncwarp();
    if (lane < N) { /* column lane of R^{-1}: R u = e_lane */
      double u[N];
#pragma unroll
      for (int i = N - 1; i >= 0; --i) {
        double v = i == lane ? 1.0 : 0.0;
#pragma unroll
        for (int k = i + 1; k < N; ++k) v = fma(-sR[k * N + i], u[k], v);
        u[i] = v * sInvR[i];
      }
#pragma unroll
      for (int i = 0; i < N; ++i) sRi[lane * N + i] = u[i];
    }
    __syncwarp();
    if (lane < N) {
      double xi = 0.0;
#pragma unroll
      for (int k = 0; k < N; ++k) xi = fma(sRi[k * N + lane], sy[k], xi);
      x[lane] = xi;
      if (P) { /* P(:, lane) = sum_k Ri(:, k) Ri(lane, k) */
#pragma unroll
        for (int i = 0; i < N; ++i) {
          double sm = 0.0;
#pragma unroll
          for (int k = 0; k < N; ++k) sm = fma(sRi[k * N + i], sRi[k * N + lane], sm);
          P[(int64_t)lane * N + i] = sm;
        }
      }
    }
    __syncwarp();
  }
  if (flag && lane == 0) atomicOr(a.flag, flag);
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
  if (p->n <= kWarpMaxN && p->mmax <= kWarpMaxN) {
    const unsigned blocks = (unsigned)((p->ntracks + kWarpsPerBlock - 1) / kWarpsPerBlock);
    const int bs = 32 * kWarpsPerBlock;
    switch (p->n) {
      case 1: UKG_LAUNCH(UKG_K_FILTER, st, (filter_warp<1><<<blocks, bs, 0, st>>>(a))); break;
      case 2: UKG_LAUNCH(UKG_K_FILTER, st, (filter_warp<2><<<blocks, bs, 0, st>>>(a))); break;
      case 3: UKG_LAUNCH(UKG_K_FILTER, st, (filter_warp<3><<<blocks, bs, 0, st>>>(a))); break;
      case 4: UKG_LAUNCH(UKG_K_FILTER, st, (filter_warp<4><<<blocks, bs, 0, st>>>(a))); break;
      case 5: UKG_LAUNCH(UKG_K_FILTER, st, (filter_warp<5><<<blocks, bs, 0, st>>>(a))); break;
      case 6: UKG_LAUNCH(UKG_K_FILTER, st, (filter_warp<6><<<blocks, bs, 0, st>>>(a))); break;
      case 7: UKG_LAUNCH(UKG_K_FILTER, st, (filter_warp<7><<<blocks, bs, 0, st>>>(a))); break;
      default: UKG_LAUNCH(UKG_K_FILTER, st, (filter_warp<8><<<blocks, bs, 0, st>>>(a))); break;
    }
  } else {
    UKG_LAUNCH(UKG_K_FILTER, st, (filter_cta<<<ncta, NT, 0, st>>>(a)));
  }
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
