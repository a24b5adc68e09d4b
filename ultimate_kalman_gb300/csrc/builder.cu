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

/* Observation blocks of ld rows_s (compact) re-laid with ld rows_d >= rows_s:
 * dst[s][j * rows_d + r] = src[s][j * cols_s... ] inside the source block,
 * zero outside.  One thread per destination entry, grid-stride.            */
__global__ void pad_blocks(double* __restrict__ dst, const double* __restrict__ src, int64_t nsteps, int rows_d,
                           int cols_d, int rows_s, int cols_s)
{
  const int per = rows_d * cols_d;
  const int64_t total = nsteps * per;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = e / per;
    const int w = (int)(e - s * per), j = w / rows_d, r = w - j * rows_d;
    dst[e] = (r < rows_s && j < cols_s) ? src[s * rows_s * cols_s + (int64_t)j * rows_s + r] : 0.0;
  }
}

/* covariance types and row counts; a row count outside [0, rows_s] becomes
 * -1, which the smoother's weighing reports as malformed input             */
__global__ void pad_steps(char* __restrict__ ct, int32_t* __restrict__ rows, const char* __restrict__ ct_s,
                          const int32_t* __restrict__ rows_s, int64_t nsteps, int mc)
{
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nsteps; s += (int64_t)gridDim.x * blockDim.x) {
    const int32_t m = rows_s[s];
    ct[s] = ct_s[s];
    rows[s] = (m >= 0 && m <= mc) ? m : -1;
  }
}

/* each track's first-step observation (G0, o0, C0 with ld m0max, type, rows)
 * written over the padded blocks of its first step first[t] (-1: an empty
 * track)                                                                    */
__global__ void place_first_obs(double* __restrict__ G, double* __restrict__ o, double* __restrict__ C,
                                char* __restrict__ ct, int32_t* __restrict__ rows, const int64_t* __restrict__ first,
                                int ntracks, int n, int mp, const double* __restrict__ G0, const double* __restrict__ o0,
                                const double* __restrict__ C0, const char* __restrict__ C0t,
                                const int32_t* __restrict__ rows0, int m0max)
{
  const int per = mp * n + mp + mp * mp;
  const int64_t total = (int64_t)ntracks * per;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(e / per);
    const int w = (int)(e - (int64_t)t * per);
    const int64_t s = first[t];
    if (s < 0) continue;
    if (w < mp * n) {
      const int j = w / mp, r = w - j * mp;
      G[s * mp * n + w] = r < m0max ? G0[(int64_t)t * m0max * n + (int64_t)j * m0max + r] : 0.0;
    } else if (w < mp * n + mp) {
      const int r = w - mp * n;
      o[s * mp + r] = r < m0max ? o0[(int64_t)t * m0max + r] : 0.0;
    } else {
      const int w2 = w - mp * n - mp, j = w2 / mp, r = w2 - j * mp;
      C[s * mp * mp + w2] = (r < m0max && j < m0max) ? C0[(int64_t)t * m0max * m0max + (int64_t)j * m0max + r] : 0.0;
    }
    if (w == 0) {
      const int32_t m = rows0[t];
      ct[s] = C0t[t];
      rows[s] = (m >= 0 && m <= m0max) ? m : -1;
    }
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

/* Lays out the observations of a problem whose steps carry mc = p->mmax rows
 * and whose tracks' first-step observations come from f0, as the ordinary
 * packed layout with mp >= max(mc, f0->m0max) rows: G, o, C, C_type and
 * obs_rows of every step into the given device arrays (first[t]: the first
 * step of track t, -1 for an empty track, a device array).  Queued on st.  */
extern "C" int ukg_pad_first_obs(const kalman_gpu_problem_t* p, const kalman_gpu_first_obs_t* f0, int mp, double* G,
                                 double* o, double* C, char* ct, int32_t* rows, const int64_t* first, void* cuda_stream)
{
  cudaStream_t st = (cudaStream_t)cuda_stream;
  const int n = p->n, mc = p->mmax;
  const int64_t N = p->nsteps;
  UKG_LAUNCH(UKG_K_BUILD, st, (pad_blocks<<<blocks_for(N * mp * n), kBuildThreads, 0, st>>>(
                                  G, p->G, N, mp, n, mc, n)));
  UKG_LAUNCH(UKG_K_BUILD, st, (pad_blocks<<<blocks_for(N * mp), kBuildThreads, 0, st>>>(
                                  o, p->o, N, mp, 1, mc, 1)));
  UKG_LAUNCH(UKG_K_BUILD, st, (pad_blocks<<<blocks_for(N * mp * mp), kBuildThreads, 0, st>>>(
                                  C, p->C, N, mp, mp, mc, mc)));
  UKG_LAUNCH(UKG_K_BUILD, st, (pad_steps<<<blocks_for(N), kBuildThreads, 0, st>>>(
                                  ct, rows, p->C_type, p->obs_rows, N, mc)));
  const int per = mp * n + mp + mp * mp;
  UKG_LAUNCH(UKG_K_BUILD, st, (place_first_obs<<<blocks_for((int64_t)p->ntracks * per), kBuildThreads, 0, st>>>(
                                  G, o, C, ct, rows, first, p->ntracks, n, mp, f0->G0, f0->o0, f0->C0, f0->C0_type,
                                  f0->obs_rows0, f0->m0max)));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return ukg_set_error(KALMAN_GPU_ECUDA, "first-step observations: %s", cudaGetErrorString(e));
  return KALMAN_GPU_OK;
}
