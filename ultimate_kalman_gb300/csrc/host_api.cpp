/*
 * host_api.cpp -- the host side of libukgpu.so.
 *
 *  - error state (kalman_gpu_last_status / _last_error);
 *  - the packed entry points of kalman_gpu.h, which stage host arrays to the
 *    device and back when the caller passes host memory;
 *  - the reference API of kalman.h for the parallel smoothers:
 *      kalman_smooth_oddeven / kalman_smooth_associative  (c/kalman.h:148-149)
 *    marshal the caller's kalman_step_equations_t array into the packed layout,
 *    run the CUDA smoother and write state/covariance back into the equations;
 *      kalman_create_options ... kalman_covariance      (c/kalman.h:117-142)
 *    keep the semantics of the reference's explicit representation
 *    (c/kalman_explicit_representation.c:164-267 and c/kalman_base.c:231-460):
 *    evolve/observe store copies of the equations, smooth runs a smoother over
 *    the stored steps, estimate/covariance return caller-owned copies or
 *    NaN-filled matrices.
 *
 * Nothing here computes a smoothing step on the CPU: the smoothers run only in
 * the CUDA kernels of oddeven.cu and associative.cu, and fail with an error
 * (NaN outputs) when no device is usable.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <deque>
#include <mutex>
#include <set>
#include <thread>
#include <vector>

#include "ukgpu_internal.h"

/* -------------------------------------------------------------------------- */
/* error state                                                                 */
/* -------------------------------------------------------------------------- */

static thread_local int tl_status = 0;
static thread_local char tl_message[512] = "";

extern "C" int ukg_set_error(int status, const char* fmt, ...)
{
  tl_status = status;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(tl_message, sizeof(tl_message), fmt, ap);
  va_end(ap);
  return status;
}

extern "C" void ukg_clear_error(void)
{
  tl_status = 0;
  tl_message[0] = 0;
}

extern "C" int kalman_gpu_last_status(void) { return tl_status; }
extern "C" const char* kalman_gpu_last_error(void) { return tl_message; }
extern "C" void kalman_gpu_clear_error(void) { ukg_clear_error(); }

/* -------------------------------------------------------------------------- */
/* packed problems                                                             */
/* -------------------------------------------------------------------------- */

extern "C" int ukg_validate_problem(const kalman_gpu_problem_t* p, int need_cov)
{
  if (!p) return ukg_set_error(KALMAN_GPU_EINVAL, "problem is NULL");
  if (p->n < 1) return ukg_set_error(KALMAN_GPU_EINVAL, "state dimension %d < 1", p->n);
  if (p->mmax < 0) return ukg_set_error(KALMAN_GPU_EINVAL, "mmax %d < 0", p->mmax);
  if (p->ntracks < 1 || !p->track_start) return ukg_set_error(KALMAN_GPU_EINVAL, "no tracks");
  if (p->location != KALMAN_GPU_DEVICE && p->location != KALMAN_GPU_HOST)
    return ukg_set_error(KALMAN_GPU_EINVAL, "unknown array location %d", p->location);
  if (p->track_start[0] != 0) return ukg_set_error(KALMAN_GPU_EINVAL, "track_start[0] must be 0");
  for (int t = 0; t < p->ntracks; ++t)
    if (p->track_start[t + 1] < p->track_start[t])
      return ukg_set_error(KALMAN_GPU_EINVAL, "track_start is decreasing at track %d", t);
  if (p->track_start[p->ntracks] != p->nsteps)
    return ukg_set_error(KALMAN_GPU_EINVAL, "track_start[ntracks] != nsteps");
  if (p->nsteps > 0) {
    if (!p->H || !p->F || !p->c || !p->K || !p->K_type || !p->obs_rows || !p->state)
      return ukg_set_error(KALMAN_GPU_EINVAL, "a required array is NULL");
    if (p->mmax > 0 && (!p->G || !p->o || !p->C || !p->C_type))
      return ukg_set_error(KALMAN_GPU_EINVAL, "observation arrays are NULL");
    if (need_cov && !p->covariance) return ukg_set_error(KALMAN_GPU_EINVAL, "covariance output is NULL");
  }
  /* obs_rows is checked where it is read, on the device, for host and device
     arrays alike (a value outside [0, mmax] is reported as malformed input):
     a pass over the host copy here would hold up the first transfer */
  return 0;
}

namespace {

struct Stage {
  int device = -1;
  void* p = nullptr; /* two staging buffers, back to back */
  size_t bytes = 0;
  cudaStream_t h2d = nullptr, d2h = nullptr;
  cudaEvent_t h2d_done[2] = {nullptr, nullptr}, computed[2] = {nullptr, nullptr}, d2h_done[2] = {nullptr, nullptr};
};
thread_local Stage tl_stage; /* device staging of host-located packed problems */

void stage_release(Stage& S)
{
  if (S.p) cudaFree(S.p);
  for (int b = 0; b < 2; ++b) {
    if (S.h2d_done[b]) cudaEventDestroy(S.h2d_done[b]);
    if (S.computed[b]) cudaEventDestroy(S.computed[b]);
    if (S.d2h_done[b]) cudaEventDestroy(S.d2h_done[b]);
  }
  if (S.h2d) cudaStreamDestroy(S.h2d);
  if (S.d2h) cudaStreamDestroy(S.d2h);
  S = Stage();
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int device_ready()
{
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return ukg_set_error(KALMAN_GPU_ENODEV, "no CUDA device is available (%s)",
                         e == cudaSuccess ? "device count is 0" : cudaGetErrorString(e));
  }
  return 0;
}

typedef int (*device_smoother)(uint32_t, const kalman_gpu_problem_t*, void*);

/* Runs a device smoother on a packed problem held in host memory.  The tracks
 * are cut into chunks of about a sixteenth of the steps (at least 2^20 steps
 * a chunk); chunk k's inputs are copied into staging buffer k mod 2 on a copy
 * stream while chunk k-1 is smoothed on the caller's stream, and its states
 * (and covariances) are copied back on a second copy stream while chunk k+1
 * is smoothed -- so the host link, which bounds this path, stays busy.      */
/* The padded observation arrays of kalman_gpu_smooth_oddeven_first_obs on
 * the device (one buffer per host thread, grown by stream-ordered
 * allocation), and the tracks' first-step indices in page-locked, device-
 * mapped host memory, read by the padding kernel itself: a copy on the
 * compute stream would queue on the copy engine behind the next chunk's
 * arrays and stall the smoothing.  Every call synchronizes its stream before
 * returning, so the next call may refill the indices.                        */
struct PadCache {
  int device = -1;
  void* dev = nullptr;
  size_t bytes = 0;
  int64_t* idx = nullptr;
  int64_t* idx_dev = nullptr;
  size_t idx_cap = 0;
};
thread_local PadCache tl_pad;

void pad_release()
{
  if (tl_pad.dev) cudaFree(tl_pad.dev);
  if (tl_pad.idx) cudaFreeHost(tl_pad.idx);
  tl_pad = PadCache();
}

/* kalman_gpu_smooth_oddeven_first_obs on device arrays: pads the compact
 * observations (p->mmax rows, first steps from f0) to the packed layout with
 * max(p->mmax, f0->m0max) rows, then runs the odd-even smoother on it.      */
int first_obs_device(uint32_t options, const kalman_gpu_problem_t* p, const kalman_gpu_first_obs_t* f0,
                     cudaStream_t st)
{
  const int64_t N = p->nsteps, n = p->n;
  const int T = p->ntracks;
  const int mp = std::max(p->mmax, f0->m0max);
  size_t off[5], bytes = 0;
  const size_t sz[5] = {(size_t)N * mp * n * 8, (size_t)N * mp * 8, (size_t)N * mp * mp * 8, (size_t)N, (size_t)N * 4};
  for (int i = 0; i < 5; ++i) {
    off[i] = bytes;
    bytes = align_up(bytes + sz[i], 256);
  }
  int dev = 0;
  cudaGetDevice(&dev);
  PadCache& c = tl_pad;
  if (c.dev && (c.bytes < bytes || c.device != dev)) {
    if (c.device == dev) cudaFreeAsync(c.dev, st);
    else cudaFree(c.dev);
    c.dev = nullptr;
    c.bytes = 0;
  }
  if (!c.dev) {
    const size_t want = ukg_with_slack(bytes);
    if (ukg_malloc_async(&c.dev, want, st) != 0) {
      c.dev = nullptr;
      return ukg_set_error(KALMAN_GPU_ENOMEM, "padded observations: %zu bytes of device memory", want);
    }
    c.bytes = want;
    c.device = dev;
  }
  if (c.idx_cap < (size_t)std::max(T, 1)) {
    if (c.idx) cudaFreeHost(c.idx);
    c.idx = c.idx_dev = nullptr;
    c.idx_cap = 0;
    cudaError_t e = cudaHostAlloc((void**)&c.idx, (size_t)std::max(T, 1) * 8, cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&c.idx_dev, c.idx, 0);
    if (e != cudaSuccess) {
      cudaGetLastError();
      if (c.idx) cudaFreeHost(c.idx);
      c.idx = c.idx_dev = nullptr;
      return ukg_set_error(KALMAN_GPU_ENOMEM, "page-locked first-step table");
    }
    c.idx_cap = (size_t)std::max(T, 1);
  }
  for (int t = 0; t < T; ++t) c.idx[t] = p->track_start[t + 1] > p->track_start[t] ? p->track_start[t] : -1;
  char* B = (char*)c.dev;
  const int64_t* first = c.idx_dev;
  double *G = (double*)(B + off[0]), *o = (double*)(B + off[1]), *C = (double*)(B + off[2]);
  char* ct = (char*)(B + off[3]);
  int32_t* rows = (int32_t*)(B + off[4]);
  if (int e = ukg_pad_first_obs(p, f0, mp, G, o, C, ct, rows, first, st)) return e;
  kalman_gpu_problem_t d = *p;
  d.location = KALMAN_GPU_DEVICE;
  d.mmax = mp;
  d.G = G;
  d.o = o;
  d.C = C;
  d.C_type = ct;
  d.obs_rows = rows;
  return ukg_oddeven_device(options, &d, st);
}

int run_host_problem(device_smoother fn, uint32_t options, const kalman_gpu_problem_t* p, bool want_cov,
                     cudaStream_t st, const kalman_gpu_first_obs_t* f0 = nullptr)
{
  const int64_t N = p->nsteps, n = p->n, mm = p->mmax;
  /* chunks of whole tracks, about 32 of them: the smoothing of the last chunk,
     which no transfer hides, stays short */
  const int64_t target = std::max<int64_t>(N / 32, (int64_t)1 << 19);
  std::vector<int> cut{0};
  for (int t = 1; t < p->ntracks; ++t)
    if (p->track_start[t] - p->track_start[cut.back()] >= target) cut.push_back(t);
  cut.push_back(p->ntracks);
  const int nchunks = (int)cut.size() - 1;
  int64_t cmax = 0, tmax = 0;
  for (int k = 0; k < nchunks; ++k) {
    cmax = std::max<int64_t>(cmax, p->track_start[cut[k + 1]] - p->track_start[cut[k]]);
    tmax = std::max<int64_t>(tmax, cut[k + 1] - cut[k]);
  }

  /* bytes per step of each array: H F c K K_type G o C C_type obs_rows | state cov */
  const size_t per[12] = {(size_t)(n * n * 8), (size_t)(n * n * 8), (size_t)(n * 8), (size_t)(n * n * 8), 1,
                          (size_t)(mm * n * 8), (size_t)(mm * 8), (size_t)(mm * mm * 8), 1, 4, (size_t)(n * 8),
                          want_cov ? (size_t)(n * n * 8) : 0};
  const void* src[10] = {p->H, p->F, p->c, p->K, p->K_type, p->G, p->o, p->C, p->C_type, p->obs_rows};
  size_t off[12], half = 0;
  for (int i = 0; i < 12; ++i) {
    off[i] = half;
    half = align_up(half + per[i] * (size_t)cmax, 256);
  }
  /* with separate first-step observations, bytes per track of G0 o0 C0 C0_type obs_rows0 */
  const int64_t m0 = f0 ? f0->m0max : 0;
  const size_t per0[5] = {(size_t)(m0 * n * 8), (size_t)(m0 * 8), (size_t)(m0 * m0 * 8), 1, 4};
  const void* src0[5] = {f0 ? f0->G0 : nullptr, f0 ? f0->o0 : nullptr, f0 ? f0->C0 : nullptr,
                         f0 ? f0->C0_type : nullptr, f0 ? f0->obs_rows0 : nullptr};
  size_t off0[5] = {0, 0, 0, 0, 0};
  if (f0)
    for (int i = 0; i < 5; ++i) {
      off0[i] = half;
      half = align_up(half + per0[i] * (size_t)tmax, 256);
    }
  int dev = 0;
  cudaGetDevice(&dev);
  Stage& S = tl_stage;
  if (S.p && (S.bytes < 2 * half || S.device != dev)) stage_release(S);
  if (!S.p) {
    cudaError_t e = cudaMalloc(&S.p, 2 * half);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S.h2d, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S.d2h, cudaStreamNonBlocking);
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
      e = cudaEventCreateWithFlags(&S.h2d_done[b], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S.computed[b], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S.d2h_done[b], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      stage_release(S);
      return ukg_set_error(KALMAN_GPU_ENOMEM, "staging %zu bytes of the problem on the device failed: %s",
                           2 * half, cudaGetErrorString(e));
    }
    S.bytes = 2 * half;
    S.device = dev;
  }
  /* the events of an earlier call are complete: that call synchronized */
  auto buffer = [&](int b) { return (char*)S.p + (size_t)b * half; };
  auto copy_in = [&](int k) {
    const int64_t g0 = p->track_start[cut[k]], g1 = p->track_start[cut[k + 1]];
    char* D = buffer(k & 1);
    for (int i = 0; i < 10; ++i)
      if (per[i] && src[i])
        cudaMemcpyAsync(D + off[i], (const char*)src[i] + (size_t)g0 * per[i], (size_t)(g1 - g0) * per[i],
                        cudaMemcpyHostToDevice, S.h2d);
    if (f0)
      for (int i = 0; i < 5; ++i)
        cudaMemcpyAsync(D + off0[i], (const char*)src0[i] + (size_t)cut[k] * per0[i],
                        (size_t)(cut[k + 1] - cut[k]) * per0[i], cudaMemcpyHostToDevice, S.h2d);
    cudaEventRecord(S.h2d_done[k & 1], S.h2d);
  };
  bool used[2] = {false, false};
  int status = 0;
  char first_error[512] = "";
  copy_in(0);
  for (int k = 0; k < nchunks; ++k) {
    if (k + 1 < nchunks) copy_in(k + 1); /* overlaps this chunk's smoothing */
    const int b = k & 1;
    const int64_t g0 = p->track_start[cut[k]], g1 = p->track_start[cut[k + 1]];
    std::vector<int64_t> ts(cut[k + 1] - cut[k] + 1);
    for (size_t i = 0; i < ts.size(); ++i) ts[i] = p->track_start[cut[k] + (int)i] - g0;
    char* D = buffer(b);
    kalman_gpu_problem_t d = *p;
    d.location = KALMAN_GPU_DEVICE;
    d.ntracks = cut[k + 1] - cut[k];
    d.nsteps = g1 - g0;
    d.track_start = ts.data();
    d.H = (const double*)(D + off[0]);
    d.F = (const double*)(D + off[1]);
    d.c = (const double*)(D + off[2]);
    d.K = (const double*)(D + off[3]);
    d.K_type = (const char*)(D + off[4]);
    d.G = (const double*)(D + off[5]);
    d.o = (const double*)(D + off[6]);
    d.C = (const double*)(D + off[7]);
    d.C_type = (const char*)(D + off[8]);
    d.obs_rows = (const int32_t*)(D + off[9]);
    d.state = (double*)(D + off[10]);
    d.covariance = want_cov ? (double*)(D + off[11]) : nullptr;
    cudaStreamWaitEvent(st, S.h2d_done[b], 0);
    if (used[b]) cudaStreamWaitEvent(st, S.d2h_done[b], 0); /* chunk k-2's outputs are read back */
    int s;
    if (f0) {
      kalman_gpu_first_obs_t fc = *f0;
      fc.G0 = (const double*)(D + off0[0]);
      fc.o0 = (const double*)(D + off0[1]);
      fc.C0 = (const double*)(D + off0[2]);
      fc.C0_type = (const char*)(D + off0[3]);
      fc.obs_rows0 = (const int32_t*)(D + off0[4]);
      s = first_obs_device(options, &d, &fc, st); /* returns after the smoothing completed */
    } else {
      s = fn(options, &d, st);
    }
    if (s == KALMAN_GPU_ECUDA) {
      cudaStreamSynchronize(S.h2d);
      cudaStreamSynchronize(S.d2h);
      return s;
    }
    if (s && !status) {
      status = s;
      snprintf(first_error, sizeof(first_error), "%s", kalman_gpu_last_error());
    }
    cudaEventRecord(S.computed[b], st);
    cudaStreamWaitEvent(S.d2h, S.computed[b], 0);
    cudaMemcpyAsync((char*)p->state + (size_t)g0 * per[10], d.state, (size_t)(g1 - g0) * per[10],
                    cudaMemcpyDeviceToHost, S.d2h);
    if (want_cov)
      cudaMemcpyAsync((char*)p->covariance + (size_t)g0 * per[11], d.covariance, (size_t)(g1 - g0) * per[11],
                      cudaMemcpyDeviceToHost, S.d2h);
    cudaEventRecord(S.d2h_done[b], S.d2h);
    used[b] = true;
  }
  cudaError_t e = cudaStreamSynchronize(S.d2h);
  if (e == cudaSuccess) e = cudaStreamSynchronize(S.h2d);
  if (e != cudaSuccess) return ukg_set_error(KALMAN_GPU_ECUDA, "copying the problem: %s", cudaGetErrorString(e));
  if (status) return ukg_set_error(status, "%s", first_error);
  return 0;
}

int smooth_packed(device_smoother fn, uint32_t options, const kalman_gpu_problem_t* p, void* stream)
{
  ukg_clear_error();
  const bool want_cov = !(options & KALMAN_NO_COVARIANCE) && p && p->covariance;
  if (int e = ukg_validate_problem(p, 0)) return e;
  if (p->nsteps == 0) return 0;
  if (int e = device_ready()) return e;
  cudaStream_t st = (cudaStream_t)stream;
  if (p->location == KALMAN_GPU_HOST) return run_host_problem(fn, options, p, want_cov, st);
  return fn(options, p, st);
}

}  // namespace

extern "C" int kalman_gpu_smooth_oddeven_packed(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream)
{
  return smooth_packed(ukg_oddeven_device, options, p, cuda_stream);
}

extern "C" int kalman_gpu_smooth_oddeven_first_obs(uint32_t options, const kalman_gpu_problem_t* p,
                                                   const kalman_gpu_first_obs_t* f0, void* cuda_stream)
{
  ukg_clear_error();
  if (!f0 || f0->m0max < 1 || !f0->G0 || !f0->o0 || !f0->C0 || !f0->C0_type || !f0->obs_rows0)
    return ukg_set_error(KALMAN_GPU_EINVAL, "first-step observations: m0max >= 1 and every array are needed");
  if (int e = ukg_validate_problem(p, 0)) return e;
  if (p->nsteps == 0) return 0;
  if (int e = device_ready()) return e;
  const bool want_cov = !(options & KALMAN_NO_COVARIANCE) && p->covariance;
  cudaStream_t st = (cudaStream_t)cuda_stream;
  if (p->location == KALMAN_GPU_HOST) return run_host_problem(ukg_oddeven_device, options, p, want_cov, st, f0);
  return first_obs_device(options, p, f0, st);
}

extern "C" int kalman_gpu_smooth_associative_packed(uint32_t options, const kalman_gpu_problem_t* p,
                                                    void* cuda_stream)
{
  return smooth_packed(ukg_associative_device, options, p, cuda_stream);
}

extern "C" void ukg_release_oddeven_workspace(void);
extern "C" void ukg_release_associative_workspace(void);
extern "C" int64_t ukg_oddeven_workspace_held(void);
extern "C" int64_t ukg_associative_workspace_held(void);

extern "C" void ukg_allow_dynamic_smem(const void* kernel)
{
  static std::mutex mu;
  static std::set<std::pair<int, const void*>> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!done.insert({dev, kernel}).second) return;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  int stat = 0;
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kernel) == cudaSuccess) stat = (int)fa.sharedSizeBytes;
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - stat);
  cudaGetLastError();
}

extern "C" void ukg_trim_pool(void)
{
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
    cudaMemPoolTrimTo(pool, 0);
  cudaGetLastError();
}

extern "C" int ukg_malloc_async(void** ptr, size_t bytes, void* cuda_stream)
{
  cudaStream_t st = (cudaStream_t)cuda_stream;
  cudaError_t e = cudaMallocAsync(ptr, bytes, st);
  if (e == cudaSuccess) return 0;
  cudaGetLastError();
  cudaStreamSynchronize(st);
  ukg_trim_pool();
  e = cudaMallocAsync(ptr, bytes, st);
  if (e != cudaSuccess) cudaGetLastError();
  return (int)e;
}

extern "C" int64_t kalman_gpu_workspace_held(void)
{
  return ukg_oddeven_workspace_held() + ukg_associative_workspace_held() + (int64_t)tl_stage.bytes +
         (int64_t)tl_pad.bytes;
}

namespace {
void pack_release();
}

extern "C" void kalman_gpu_release(void)
{
  ukg_release_oddeven_workspace();
  ukg_release_associative_workspace();
  ukg_release_filter_workspace();
  stage_release(tl_stage);
  pack_release();
  pad_release();
  ukg_trim_pool();
}

/* -------------------------------------------------------------------------- */
/* marshalling kalman_step_equations_t arrays                                  */
/* -------------------------------------------------------------------------- */

namespace {

int rows_of(const kalman_matrix_t* A) { return A ? A->row_dim : 0; }
int cols_of(const kalman_matrix_t* A) { return A ? A->col_dim : 0; }

void copy_block(double* dst, int ld, const kalman_matrix_t* A)
{
  for (int j = 0; j < A->col_dim; ++j)
    for (int i = 0; i < A->row_dim; ++i) dst[(size_t)j * ld + i] = A->elements[(size_t)j * A->ld + i];
}

kalman_matrix_t* new_matrix(int rows, int cols)
{
  kalman_matrix_t* M = (kalman_matrix_t*)malloc(sizeof(kalman_matrix_t));
  M->row_dim = rows;
  M->col_dim = cols;
  M->ld = rows;
  M->elements = (rows > 0 && cols > 0) ? (double*)malloc(sizeof(double) * rows * cols) : nullptr;
  return M;
}

void free_matrix(kalman_matrix_t* M)
{
  if (!M) return;
  free(M->elements);
  free(M);
}

/* a matrix the packing may read: elements present, leading dimension at least
 * the row count */
bool readable(const kalman_matrix_t* A) { return A && A->elements && A->ld >= A->row_dim && A->row_dim >= 0; }

bool valid_cov(const kalman_matrix_t* Cm, char type, int dim)
{
  if (!readable(Cm)) return false;
  if (type == 'w') return Cm->row_dim == dim && Cm->col_dim >= 1;
  if (type == 'W' || type == 'C' || type == 'U' || type == 'F') return Cm->row_dim == dim && Cm->col_dim == dim;
  return false;
}

/* Host staging of the packed image of an equations array (page-locked when
 * possible, so the copies to the device run at full speed).                 */
struct HostPack {
  std::vector<int64_t> track_start;
  double *H = nullptr, *F = nullptr, *c = nullptr, *K = nullptr, *G = nullptr, *o = nullptr, *C = nullptr;
  double *state = nullptr, *cov = nullptr;
  char *Kt = nullptr, *Ct = nullptr;
  int32_t* m = nullptr;
  void* block = nullptr; /* the calling thread's cached staging buffer (tl_pack) */
};

/* The packed image of an equations array is staged in one page-locked host
 * buffer per host thread, kept between calls (grow-only; released by
 * kalman_gpu_release): page-locking tens of GB on every call would cost more
 * than the smoothing.                                                        */
struct PackCache {
  void* p = nullptr;
  size_t bytes = 0;
  bool pinned = false;
};
thread_local PackCache tl_pack;

void pack_release()
{
  if (tl_pack.p) {
    if (tl_pack.pinned) cudaFreeHost(tl_pack.p);
    else free(tl_pack.p);
  }
  tl_pack = PackCache();
}

void* pack_buffer(size_t bytes)
{
  if (tl_pack.p && tl_pack.bytes >= bytes) return tl_pack.p;
  pack_release();
  if (cudaHostAlloc(&tl_pack.p, bytes, cudaHostAllocDefault) == cudaSuccess) {
    tl_pack.pinned = true;
  } else {
    cudaGetLastError();
    tl_pack.p = malloc(bytes);
    tl_pack.pinned = false;
  }
  tl_pack.bytes = tl_pack.p ? bytes : 0;
  return tl_pack.p;
}

/* f(lo, hi) over [0, N) in contiguous ranges on up to 32 host threads (one
 * range per 16,384 steps at least); per-step marshalling is independent.    */
template <class Fn>
void parallel_steps(int64_t N, Fn f)
{
  const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
  const int64_t T = std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(hw, 32), N / 16384));
  if (T == 1) {
    f((int64_t)0, N);
    return;
  }
  std::vector<std::thread> pool;
  for (int64_t t = 0; t < T; ++t) pool.emplace_back(f, N * t / T, N * (t + 1) / T);
  for (auto& th : pool) th.join();
}

int pack_equations(kalman_step_equations_t** eq, int64_t N, const kalman_step_index_t* lengths, int ntracks,
                   bool want_cov, HostPack& hp, kalman_gpu_problem_t& P)
{
  if (!eq) return ukg_set_error(KALMAN_GPU_EINVAL, "equations is NULL");
  for (int64_t s = 0; s < N; ++s)
    if (!eq[s]) return ukg_set_error(KALMAN_GPU_EINVAL, "equations[%lld] is NULL", (long long)s);
  /* Steps may have different state dimensions n_s, and fewer evolution rows
   * l_s than states (c/kalman.h:56-75; the reference's test catalogue grows
   * the state, matlab/examples/kalmanTest.m:93-94).  The packed problem has
   * one dimension, so every step is padded to n = max n_s with dummy
   * components d_s (slots n_s .. n-1) that no real equation touches: evolution
   * rows l_s .. n-1 read d_s = 0 * d_{s-1} + e (unit noise, as far as there
   * are dummy slots; zero rows after that), and every step observes d_s = 0
   * with unit weight.  The least-squares problem then separates into the
   * caller's problem and an independent one for the dummies, so the real
   * components' estimates and covariances are unchanged; they are unpacked at
   * each step's own size.  Without padding (all n_s = l_s = n) the packed
   * arrays are exactly the caller's matrices.                              */
  int n = 0;
  for (int64_t s = 0; s < N; ++s) n = std::max(n, (int)eq[s]->dimension);
  if (n < 1) return ukg_set_error(KALMAN_GPU_EINVAL, "state dimension %d < 1", n);
  hp.track_start.assign(ntracks + 1, 0);
  for (int t = 0; t < ntracks; ++t) {
    if (lengths[t] < 0) return ukg_set_error(KALMAN_GPU_EINVAL, "negative track length");
    hp.track_start[t + 1] = hp.track_start[t] + (int64_t)lengths[t];
  }
  if (hp.track_start[ntracks] != N) return ukg_set_error(KALMAN_GPU_EINVAL, "track lengths do not sum to the step count");
  int mmax = 0;
  std::vector<char> first(N, 0);
  for (int t = 0; t < ntracks; ++t)
    if (lengths[t] > 0) first[hp.track_start[t]] = 1;
  for (int64_t s = 0; s < N; ++s) {
    const kalman_step_equations_t* e = eq[s];
    const int ns = e->dimension;
    if (ns < 1) return ukg_set_error(KALMAN_GPU_EINVAL, "step %lld has state dimension %d", (long long)s, ns);
    if (!first[s]) {
      const int np = eq[s - 1]->dimension, l = rows_of(e->H);
      if (l < 1 || l > n || cols_of(e->H) != ns || rows_of(e->F) != l || cols_of(e->F) != np || rows_of(e->c) != l ||
          cols_of(e->c) != 1 || !readable(e->H) || !readable(e->F) || !readable(e->c))
        return ukg_set_error(KALMAN_GPU_EINVAL, "step %lld: H must be l x %d, F l x %d and c l x 1 with 1 <= l <= %d",
                             (long long)s, ns, np, n);
      if (!valid_cov(e->K, e->K_type, l))
        return ukg_set_error(KALMAN_GPU_EINVAL, "step %lld: bad evolution covariance (type '%c')", (long long)s,
                             e->K_type ? e->K_type : '?');
    }
    int m = 0;
    if (e->o) {
      m = rows_of(e->o);
      if (m < 1 || cols_of(e->o) != 1 || rows_of(e->G) != m || cols_of(e->G) != ns || !readable(e->G) ||
          !readable(e->o))
        return ukg_set_error(KALMAN_GPU_EINVAL, "step %lld: G must be m x %d and o m x 1", (long long)s, ns);
      if (!valid_cov(e->C, e->C_type, m))
        return ukg_set_error(KALMAN_GPU_EINVAL, "step %lld: bad observation covariance (type '%c')", (long long)s,
                             e->C_type ? e->C_type : '?');
    }
    mmax = std::max(mmax, m + (n - ns)); /* the observation and the dummies' zero observation */
  }
  const size_t nn = (size_t)n * n, mm = (size_t)mmax;
  const size_t dbl = N * (3 * nn + n + mm * n + mm + mm * mm + n + (want_cov ? nn : 0));
  const size_t bytes = dbl * sizeof(double) + 2 * N + 4 * N + 64;
  hp.block = pack_buffer(bytes);
  if (!hp.block) return ukg_set_error(KALMAN_GPU_ENOMEM, "host allocation of %zu bytes failed", bytes);
  double* d = (double*)hp.block;
  hp.H = d; d += N * nn;
  hp.F = d; d += N * nn;
  hp.K = d; d += N * nn;
  hp.c = d; d += N * n;
  hp.G = d; d += N * mm * n;
  hp.o = d; d += N * mm;
  hp.C = d; d += N * mm * mm;
  hp.state = d; d += N * n;
  hp.cov = want_cov ? d : nullptr; d += want_cov ? N * nn : 0;
  hp.m = (int32_t*)d;
  hp.Kt = (char*)(hp.m + N);
  hp.Ct = hp.Kt + N;
  /* unit weight on pad rows beyond a covariance block of `rows` (ld) */
  auto pad_cov = [](double* B, int ld, char type, int rows, int total) {
    for (int i = rows; i < total; ++i) {
      if (type == 'w') B[i] = 1.0;
      else B[(size_t)i * ld + i] = 1.0;
    }
  };
  parallel_steps(N, [&](int64_t lo, int64_t hi) {
    const size_t cnt = (size_t)(hi - lo);
    memset(hp.H + lo * nn, 0, cnt * nn * sizeof(double));
    memset(hp.F + lo * nn, 0, cnt * nn * sizeof(double));
    memset(hp.K + lo * nn, 0, cnt * nn * sizeof(double));
    memset(hp.c + lo * n, 0, cnt * n * sizeof(double));
    memset(hp.G + lo * mm * n, 0, cnt * mm * n * sizeof(double));
    memset(hp.o + lo * mm, 0, cnt * mm * sizeof(double));
    memset(hp.C + lo * mm * mm, 0, cnt * mm * mm * sizeof(double));
    for (int64_t s = lo; s < hi; ++s) {
      const kalman_step_equations_t* e = eq[s];
      const int ns = e->dimension, dummies = n - ns;
      hp.Kt[s] = 'C';
      hp.Ct[s] = 'C';
      if (!first[s]) {
        const int l = e->H->row_dim;
        copy_block(hp.H + s * nn, n, e->H);
        copy_block(hp.F + s * nn, n, e->F);
        copy_block(hp.c + s * n, n, e->c);
        if (e->K_type == 'w') {
          for (int i = 0; i < l; ++i) hp.K[s * nn + i] = e->K->elements[i];
        } else {
          copy_block(hp.K + s * nn, n, e->K);
        }
        hp.Kt[s] = e->K_type;
        pad_cov(hp.K + s * nn, n, e->K_type, l, n);
        for (int r = l; r < n && r - l < dummies; ++r) hp.H[s * nn + (size_t)(ns + r - l) * n + r] = 1.0;
      }
      const int m = e->o ? e->o->row_dim : 0;
      if (m > 0) {
        copy_block(hp.G + s * mm * n, (int)mm, e->G);
        for (int i = 0; i < m; ++i) hp.o[s * mm + i] = e->o->elements[i];
        if (e->C_type == 'w') {
          for (int i = 0; i < m; ++i) hp.C[s * mm * mm + i] = e->C->elements[i];
        } else {
          copy_block(hp.C + s * mm * mm, (int)mm, e->C);
        }
        hp.Ct[s] = e->C_type;
      }
      if (dummies > 0) { /* d_s = 0, unit weight */
        for (int j = 0; j < dummies; ++j) hp.G[s * mm * n + (size_t)(ns + j) * mm + m + j] = 1.0;
        pad_cov(hp.C + s * mm * mm, (int)mm, hp.Ct[s], m, m + dummies);
      }
      hp.m[s] = m + dummies;
    }
  });
  memset(&P, 0, sizeof(P));
  P.n = n;
  P.mmax = mmax;
  P.ntracks = ntracks;
  P.location = KALMAN_GPU_HOST;
  P.nsteps = N;
  P.track_start = hp.track_start.data();
  P.H = hp.H; P.F = hp.F; P.c = hp.c; P.K = hp.K; P.K_type = hp.Kt;
  P.G = hp.G; P.o = hp.o; P.C = hp.C; P.C_type = hp.Ct; P.obs_rows = hp.m;
  P.state = hp.state;
  P.covariance = hp.cov;
  return 0;
}

/* writes the results into the equations (caller-owned matrices, type 'C'):
 * each step's leading dimension x dimension part of the packed results,
 * whose stride is n0 (the padded dimension); one host thread per range      */
void unpack_results(kalman_step_equations_t** eq, int64_t N, int n0, const double* state, const double* cov,
                    bool failed)
{
  parallel_steps(N, [&](int64_t lo, int64_t hi) {
    for (int64_t s = lo; s < hi; ++s) {
      kalman_step_equations_t* e = eq[s];
      if (!e) continue;
      const int n = e->dimension;
      if (n < 1 || (!failed && n > n0)) continue;
      const size_t nn0 = (size_t)n0 * n0;
      free_matrix(e->state);
      free_matrix(e->covariance);
      e->state = new_matrix(n, 1);
      for (int i = 0; i < n; ++i) e->state->elements[i] = failed ? NAN : state[s * n0 + i];
      e->covariance = nullptr;
      if (cov || failed) {
        e->covariance = new_matrix(n, n);
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i)
            e->covariance->elements[(size_t)j * n + i] = failed ? NAN : cov[s * nn0 + (size_t)j * n0 + i];
      }
      e->covariance_type = 'C';
    }
  });
}

int smooth_equations(bool associative, uint32_t options, kalman_step_equations_t** eq, int64_t N,
                     const kalman_step_index_t* lengths, int ntracks)
{
  ukg_clear_error();
  if (N <= 0) return 0;
  /* the reference's associative smoother always returns covariances */
  const bool want_cov = associative || !(options & KALMAN_NO_COVARIANCE);
  if (associative) options &= ~(uint32_t)KALMAN_NO_COVARIANCE;
  HostPack hp;
  kalman_gpu_problem_t P;
  int status = 0;
  if (associative && eq) /* it takes H as the identity: evolutions must be square (l_s = n_s) */
    for (int64_t s = 0; s < N && !status; ++s)
      if (eq[s] && eq[s]->H && eq[s]->H->row_dim != eq[s]->dimension)
        status = ukg_set_error(KALMAN_GPU_EINVAL, "step %lld: the associative smoother needs as many evolution "
                               "rows as states (%d, not %d)", (long long)s, eq[s]->dimension, eq[s]->H->row_dim);
  if (status == 0) status = pack_equations(eq, N, lengths, ntracks, want_cov, hp, P);
  if (status == 0) status = device_ready();
  if (status == 0)
    status = run_host_problem(associative ? ukg_associative_device : ukg_oddeven_device, options, &P, want_cov,
                              (cudaStream_t)0);
  const bool values = (status == 0 || status == KALMAN_GPU_ESINGULAR) && hp.block;
  if (eq) unpack_results(eq, N, values ? P.n : 0, hp.state, want_cov ? hp.cov : nullptr, !values);
  return status;
}

}  // namespace

extern "C" void kalman_smooth_oddeven(kalman_options_t options, kalman_step_equations_t** equations,
                                      kalman_step_index_t length)
{
  kalman_step_index_t L = length;
  smooth_equations(false, (uint32_t)options, equations, (int64_t)length, &L, 1);
}

extern "C" void kalman_smooth_associative(kalman_options_t options, kalman_step_equations_t** equations,
                                          kalman_step_index_t length)
{
  kalman_step_index_t L = length;
  smooth_equations(true, (uint32_t)options, equations, (int64_t)length, &L, 1);
}

extern "C" int kalman_gpu_smooth_tracks(uint32_t options, kalman_step_equations_t** equations,
                                        const kalman_step_index_t* track_lengths, int32_t ntracks)
{
  ukg_clear_error();
  if (ntracks < 1 || !track_lengths) return ukg_set_error(KALMAN_GPU_EINVAL, "no tracks");
  int64_t N = 0;
  for (int t = 0; t < ntracks; ++t) {
    if (track_lengths[t] < 0) return ukg_set_error(KALMAN_GPU_EINVAL, "negative track length");
    N += track_lengths[t];
  }
  const bool assoc = (options & KALMAN_ALGORITHM_ASSOCIATIVE) && !(options & KALMAN_ALGORITHM_ODDEVEN);
  return smooth_equations(assoc, options, equations, N, track_lengths, ntracks);
}

/* -------------------------------------------------------------------------- */
/* kalman_t: the explicit representation                                       */
/* -------------------------------------------------------------------------- */

struct kalman_st {
  uint32_t options;
  std::deque<kalman_step_equations_t*> steps; /* steps.front() has logical index `first` */
  int64_t first;
  kalman_step_equations_t* current;
};

namespace {

/* a copy the library owns; NULL for a NULL or unreadable matrix (negative
 * dimensions, no elements, leading dimension below the row count), which the
 * smoothing then refuses as a missing block */
kalman_matrix_t* copy_or_null(const kalman_matrix_t* A)
{
  if (!A || A->row_dim < 0 || A->col_dim < 0) return nullptr;
  if (A->row_dim > 0 && A->col_dim > 0 && !readable(A)) return nullptr;
  kalman_matrix_t* B = new_matrix(A->row_dim, A->col_dim);
  for (int j = 0; j < A->col_dim; ++j)
    for (int i = 0; i < A->row_dim; ++i) B->elements[(size_t)j * B->ld + i] = A->elements[(size_t)j * A->ld + i];
  return B;
}

kalman_step_equations_t* step_new()
{
  kalman_step_equations_t* s = (kalman_step_equations_t*)calloc(1, sizeof(kalman_step_equations_t));
  s->step = -1;
  s->dimension = -1;
  s->covariance_type = 'C';
  return s;
}

void step_release_observation(kalman_step_equations_t* s)
{
  free_matrix(s->G); s->G = nullptr;
  free_matrix(s->o); s->o = nullptr;
  free_matrix(s->C); s->C = nullptr;
  free_matrix(s->state); s->state = nullptr;
  free_matrix(s->covariance); s->covariance = nullptr;
}

void step_delete(kalman_step_equations_t* s)
{
  if (!s) return;
  step_release_observation(s);
  free_matrix(s->H);
  free_matrix(s->F);
  free_matrix(s->K);
  free_matrix(s->c);
  free(s);
}

kalman_matrix_t* nan_matrix(int rows, int cols)
{
  kalman_matrix_t* M = new_matrix(rows, cols);
  for (int i = 0; i < rows * cols; ++i) M->elements[i] = NAN;
  return M;
}

int64_t resolve(kalman_t* k, kalman_step_index_t si)
{
  int64_t last = k->first + (int64_t)k->steps.size() - 1;
  return si < 0 ? last : (int64_t)si;
}

kalman_step_equations_t* step_at(kalman_t* k, int64_t si)
{
  int64_t pos = si - k->first;
  if (pos < 0 || pos >= (int64_t)k->steps.size()) return nullptr;
  return k->steps[(size_t)pos];
}

}  // namespace

extern "C" kalman_t* kalman_create_options(uint32_t options)
{
  const uint32_t alg = options & (KALMAN_ALGORITHM_ULTIMATE | KALMAN_ALGORITHM_CONVENTIONAL |
                                  KALMAN_ALGORITHM_ODDEVEN | KALMAN_ALGORITHM_ASSOCIATIVE);
  if (alg != KALMAN_ALGORITHM_ODDEVEN && alg != KALMAN_ALGORITHM_ASSOCIATIVE) {
    ukg_set_error(KALMAN_GPU_EINVAL, "algorithm bits 0x%x: this library provides KALMAN_ALGORITHM_ODDEVEN and "
                  "KALMAN_ALGORITHM_ASSOCIATIVE only", alg);
    return nullptr;
  }
  kalman_t* k = new kalman_st();
  k->options = options;
  k->first = 0;
  k->current = nullptr;
  return k;
}

extern "C" kalman_t* kalman_create(void) { return kalman_create_options(KALMAN_ALGORITHM_ODDEVEN); }

extern "C" void kalman_free(kalman_t* k)
{
  if (!k) return;
  for (auto* s : k->steps) step_delete(s);
  if (k->current) step_delete(k->current);
  delete k;
}

extern "C" kalman_step_index_t kalman_earliest(kalman_t* k)
{
  if (!k || k->steps.empty()) return -1;
  return (kalman_step_index_t)k->steps.front()->step;
}

extern "C" kalman_step_index_t kalman_latest(kalman_t* k)
{
  if (!k || k->steps.empty()) return -1;
  return (kalman_step_index_t)k->steps.back()->step;
}

extern "C" void kalman_evolve(kalman_t* k, int32_t n_i, kalman_matrix_t* H_i, kalman_matrix_t* F_i,
                              kalman_matrix_t* c_i, kalman_matrix_t* K_i, char K_type)
{
  if (!k) return;
  if (k->current) step_delete(k->current);
  kalman_step_equations_t* s = step_new();
  k->current = s;
  s->dimension = n_i;
  if (k->steps.empty()) {
    s->step = 0;
    return;
  }
  s->step = k->steps.back()->step + 1;
  s->H = copy_or_null(H_i);
  s->F = copy_or_null(F_i);
  s->c = copy_or_null(c_i);
  s->K = copy_or_null(K_i);
  s->K_type = K_type;
}

extern "C" void kalman_observe(kalman_t* k, kalman_matrix_t* G_i, kalman_matrix_t* o_i, kalman_matrix_t* C_i,
                               char C_type)
{
  if (!k || !k->current) {
    ukg_set_error(KALMAN_GPU_EINVAL, "kalman_observe without a preceding kalman_evolve");
    return;
  }
  kalman_step_equations_t* s = k->current;
  if (o_i) {
    s->G = copy_or_null(G_i);
    s->o = copy_or_null(o_i);
    s->C = copy_or_null(C_i);
    s->C_type = C_type;
  }
  if (k->steps.empty()) k->first = s->step;
  k->steps.push_back(s);
  k->current = nullptr;
}

extern "C" void kalman_smooth(kalman_t* k)
{
  if (!k || k->steps.empty()) return;
  std::vector<kalman_step_equations_t*> v(k->steps.begin(), k->steps.end());
  if (k->options & KALMAN_ALGORITHM_ODDEVEN)
    kalman_smooth_oddeven((kalman_options_t)k->options, v.data(), (kalman_step_index_t)v.size());
  if (k->options & KALMAN_ALGORITHM_ASSOCIATIVE)
    kalman_smooth_associative((kalman_options_t)k->options, v.data(), (kalman_step_index_t)v.size());
}

extern "C" kalman_matrix_t* kalman_estimate(kalman_t* k, kalman_step_index_t si)
{
  if (!k || k->steps.empty()) return nullptr;
  kalman_step_equations_t* s = step_at(k, resolve(k, si));
  if (!s) return nullptr;
  if (!s->state) return nan_matrix(s->dimension, 1);
  return copy_or_null(s->state);
}

extern "C" kalman_matrix_t* kalman_covariance(kalman_t* k, kalman_step_index_t si)
{
  if (!k || k->steps.empty()) return nullptr;
  kalman_step_equations_t* s = step_at(k, resolve(k, si));
  if (!s) return nullptr;
  if (!s->covariance) return nan_matrix(s->dimension, s->dimension);
  return copy_or_null(s->covariance);
}

extern "C" char kalman_covariance_type(kalman_t* k, kalman_step_index_t si)
{
  if (!k || k->steps.empty()) return '-';
  kalman_step_equations_t* s = step_at(k, resolve(k, si));
  return s ? s->covariance_type : '-';
}

extern "C" void kalman_forget(kalman_t* k, kalman_step_index_t si)
{
  if (!k || k->steps.empty()) return;
  const int64_t last = k->first + (int64_t)k->steps.size() - 1;
  int64_t upto = si < 0 ? last - 1 : (int64_t)si;
  if (upto > last - 1) return; /* the last step is never forgotten */
  if (upto < k->first) return;
  while (k->first <= upto) {
    step_delete(k->steps.front());
    k->steps.pop_front();
    ++k->first;
  }
}

extern "C" void kalman_rollback(kalman_t* k, kalman_step_index_t si)
{
  if (!k || k->steps.empty()) return;
  const int64_t last = k->first + (int64_t)k->steps.size() - 1;
  if (si > last || si < k->first) return;
  while (!k->steps.empty()) {
    kalman_step_equations_t* s = k->steps.back();
    k->steps.pop_back();
    if (s->step == si) {
      step_release_observation(s); /* back to "just after evolve" */
      if (k->current) step_delete(k->current);
      k->current = s;
      break;
    }
    step_delete(s);
  }
}

extern "C" kalman_matrix_t* kalman_perftest(kalman_t* k, kalman_matrix_t* H, kalman_matrix_t* F, kalman_matrix_t* c,
                                            kalman_matrix_t* K, char K_type, kalman_matrix_t* G, kalman_matrix_t* o,
                                            kalman_matrix_t* C, char C_type, int32_t count, int32_t decimation)
{
  /* the reference's sequential-filter timing loop (c/kalman_base.c:464-512):
     evolve, observe, estimate, forget, averaging wall time per decimation block */
  if (decimation < 1) decimation = 1;
  kalman_matrix_t* t = nan_matrix(count / decimation, 1);
  const int n = cols_of(G);
  struct timespec b, e;
  clock_gettime(CLOCK_MONOTONIC, &b);
  int j = 0;
  for (int i = 0; i < count; ++i) {
    kalman_evolve(k, n, H, F, c, K, K_type);
    kalman_observe(k, G, o, C, C_type);
    free_matrix(kalman_estimate(k, -1));
    kalman_forget(k, -1);
    if ((i % decimation) == decimation - 1 && j < count / decimation) {
      clock_gettime(CLOCK_MONOTONIC, &e);
      t->elements[j++] = ((e.tv_sec - b.tv_sec) + 1e-9 * (e.tv_nsec - b.tv_nsec)) / decimation;
      b = e;
    }
  }
  return t;
}

/* the reference's thread controls (c/parallel.h:31-32): the GPU build sizes its
   launches itself, so these are accepted and ignored                          */
extern "C" void parallel_set_thread_limit(int number_of_threads) { (void)number_of_threads; }
extern "C" void parallel_set_blocksize(int blocksize_in) { (void)blocksize_in; }
