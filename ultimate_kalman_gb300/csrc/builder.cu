/*
 * builder.cu -- device-side equation builder: expands one time-invariant
 * model and an observation stream into the packed per-step arrays the
 * smoothers read (kalman_gpu_expand_invariant).  It stands in for the
 * reference's host-side kalman_evolve / kalman_observe loop
 * (c/kalman_explicit_representation.c:164-244) for such tracks.
 *
 * Pure data movement, bound by HBM writes: one grid-stride pass per field,
 * consecutive threads on consecutive entries of the destination.
 */
#include <cuda_runtime.h>

#include "profiling.h"
#include "ukgpu_internal.h"

namespace {

constexpr int kBuildThreads = 256;

/* dst[(first + i) * rows * cols + j * rows + r] for i < k, from column-major
 * sources (ld = their rows): step 0 from s0 (r0 x c0; null: all zero), the
 * other steps from s1 (r1 x c1); entries outside the source are zero.      */
__global__ void expand_matrix(double* __restrict__ dst, int64_t first, int64_t k, int rows, int cols,
                              const double* __restrict__ s0, int r0, int c0, const double* __restrict__ s1, int r1,
                              int c1)
{
  const int per = rows * cols; /* <= 128 x 128 */
  const int64_t total = k * per, e0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e0 >= total) return;
  /* (step, entry) of this thread's entries, advanced by the grid stride without
     64-bit divisions in the loop */
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t sq = stride / per;
  const int sr = (int)(stride - sq * per);
  int64_t i = e0 / per;
  int w = (int)(e0 - i * per);
  double* out = dst + first * per;
  for (int64_t e = e0; e < total; e += stride) {
    const int j = w / rows, r = w - j * rows;
    double v = 0.0;
    if (i == 0) {
      if (s0 && r < r0 && j < c0) v = s0[(int64_t)j * r0 + r];
    } else if (s1 && r < r1 && j < c1) {
      v = s1[(int64_t)j * r1 + r];
    }
    out[e] = v;
    i += sq;
    w += sr;
    if (w >= per) {
      w -= per;
      ++i;
    }
  }
}

/* the observation vectors: o[(first + i) * mmax + r] */
__global__ void expand_obs(double* __restrict__ dst, int64_t first, int64_t k, int mmax, const double* __restrict__ o0,
                           int m0, const double* __restrict__ o, int64_t ldo, int m)
{
  const int64_t total = k * mmax;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / mmax;
    const int r = (int)(e - i * mmax);
    double v = 0.0;
    if (i == 0) {
      if (r < m0) v = o0[r];
    } else if (r < m) {
      v = o[(i - 1) * ldo + r];
    }
    dst[(first + i) * mmax + r] = v;
  }
}

__global__ void expand_steps(char* __restrict__ kt, char* __restrict__ ct, int32_t* __restrict__ rows, int64_t first,
                             int64_t k, char ktype, char c0type, char ctype, int m0, int m,
                             const int32_t* __restrict__ obs)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < k; i += (int64_t)gridDim.x * blockDim.x) {
    kt[first + i] = i == 0 ? 'C' : ktype;
    ct[first + i] = i == 0 ? c0type : ctype;
    rows[first + i] = i == 0 ? m0 : obs ? obs[i - 1] : m;
  }
}

unsigned blocks_for(int64_t total)
{
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (total + kBuildThreads - 1) / kBuildThreads;
  const int64_t cap = (int64_t)(sms > 0 ? sms : 1) * 8; /* 8 blocks of 256 per SM, grid-stride beyond */
  return (unsigned)(want < 1 ? 1 : want < cap ? want : cap);
}

bool cov_type_ok(char t) { return t == 'W' || t == 'w' || t == 'C' || t == 'U' || t == 'F'; }

}  // namespace

extern "C" int kalman_gpu_expand_invariant(const kalman_gpu_problem_t* p, int64_t first, int64_t k,
                                           const kalman_gpu_invariant_model_t* md, const double* o, int64_t ldo,
                                           const int32_t* obs_rows, void* cuda_stream)
{
  ukg_clear_error();
  if (!p || !md) return ukg_set_error(KALMAN_GPU_EINVAL, "expand_invariant: null problem or model");
  if (p->location != KALMAN_GPU_DEVICE)
    return ukg_set_error(KALMAN_GPU_EINVAL, "expand_invariant: the problem's arrays must be device arrays");
  const int n = p->n, mmax = p->mmax;
  if (n <= 0 || mmax <= 0 || k <= 0 || first < 0 || first + k > p->nsteps)
    return ukg_set_error(KALMAN_GPU_EINVAL, "expand_invariant: steps [%lld, %lld) outside the problem's %lld steps",
                         (long long)first, (long long)(first + k), (long long)p->nsteps);
  if (md->m0 < 0 || md->m0 > mmax || md->m < 0 || md->m > mmax)
    return ukg_set_error(KALMAN_GPU_EINVAL, "expand_invariant: observation rows (%d, %d) outside [0, %d]", md->m0,
                         md->m, mmax);
  if (!cov_type_ok(md->K_type) || !cov_type_ok(md->C_type) || !cov_type_ok(md->C0_type))
    return ukg_set_error(KALMAN_GPU_EINVAL, "expand_invariant: covariance types must be one of W w C U F");
  if (k > 1 && (!md->H || !md->F || !md->c || !md->K || (md->m > 0 && (!md->G || !md->C || !o || ldo < md->m))))
    return ukg_set_error(KALMAN_GPU_EINVAL, "expand_invariant: missing model matrices or observations");
  if (md->m0 > 0 && (!md->G0 || !md->o0 || !md->C0))
    return ukg_set_error(KALMAN_GPU_EINVAL, "expand_invariant: missing step-0 observation");
  if (!p->H || !p->F || !p->c || !p->K || !p->K_type || !p->G || !p->o || !p->C || !p->C_type || !p->obs_rows)
    return ukg_set_error(KALMAN_GPU_EINVAL, "expand_invariant: null destination array");
  cudaStream_t st = (cudaStream_t)cuda_stream;
  auto W = [](const double* a) { return const_cast<double*>(a); };
  const int64_t nn = (int64_t)n * n;
  /* a 'w' covariance is a vector of rows x 1 (diagonal inverse standard
     deviations): it fills the first column of its packed block */
  const int kc = md->K_type == 'w' ? 1 : n, cc = md->C_type == 'w' ? 1 : md->m, c0c = md->C0_type == 'w' ? 1 : md->m0;
  const int64_t nG = k * mmax * (int64_t)n, nC = k * mmax * (int64_t)mmax;
  UKG_LAUNCH(UKG_K_BUILD, st, (expand_matrix<<<blocks_for(k * nn), kBuildThreads, 0, st>>>(
                                  W(p->H), first, k, n, n, nullptr, 0, 0, md->H, n, n)));
  UKG_LAUNCH(UKG_K_BUILD, st, (expand_matrix<<<blocks_for(k * nn), kBuildThreads, 0, st>>>(
                                  W(p->F), first, k, n, n, nullptr, 0, 0, md->F, n, n)));
  UKG_LAUNCH(UKG_K_BUILD, st, (expand_matrix<<<blocks_for(k * n), kBuildThreads, 0, st>>>(
                                  W(p->c), first, k, n, 1, nullptr, 0, 0, md->c, n, 1)));
  UKG_LAUNCH(UKG_K_BUILD, st, (expand_matrix<<<blocks_for(k * nn), kBuildThreads, 0, st>>>(
                                  W(p->K), first, k, n, n, nullptr, 0, 0, md->K, n, kc)));
  UKG_LAUNCH(UKG_K_BUILD, st, (expand_matrix<<<blocks_for(nG), kBuildThreads, 0, st>>>(
                                  W(p->G), first, k, mmax, n, md->G0, md->m0, n, md->G, md->m, n)));
  UKG_LAUNCH(UKG_K_BUILD, st, (expand_matrix<<<blocks_for(nC), kBuildThreads, 0, st>>>(
                                  W(p->C), first, k, mmax, mmax, md->C0, md->m0, c0c, md->C, md->m, cc)));
  UKG_LAUNCH(UKG_K_BUILD, st, (expand_obs<<<blocks_for(k * mmax), kBuildThreads, 0, st>>>(
                                  W(p->o), first, k, mmax, md->o0, md->m0, o, ldo, md->m)));
  UKG_LAUNCH(UKG_K_BUILD, st, (expand_steps<<<blocks_for(k), kBuildThreads, 0, st>>>(
                                  const_cast<char*>(p->K_type), const_cast<char*>(p->C_type),
                                  const_cast<int32_t*>(p->obs_rows), first, k, md->K_type, md->C0_type, md->C_type,
                                  md->m0, md->m, obs_rows)));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return ukg_set_error(KALMAN_GPU_ECUDA, "expand_invariant: %s", cudaGetErrorString(e));
  return KALMAN_GPU_OK;
}
