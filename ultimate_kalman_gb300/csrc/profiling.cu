/*
 * profiling.cu -- per-kernel timing, launch counting and an FP64 throughput
 * probe for libukgpu.so.
 *
 * When enabled (kalman_gpu_profile_enable), every kernel launch of the
 * smoothers is bracketed by CUDA events recorded on the launching stream; the
 * elapsed times are summed per kernel class when the smoother call has
 * synchronized.  Launches are counted always.  The state is per host thread.
 */
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "ukgpu_internal.h"
#include "profiling.h"

namespace {

struct Pending {
  int kind;
  cudaEvent_t a, b;
};

struct ProfState {
  bool on = false;
  int64_t launches = 0;
  double ms[UKG_K_COUNT] = {0};
  int64_t count[UKG_K_COUNT] = {0};
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
};
thread_local ProfState tl;

const char* kNames[UKG_K_COUNT] = {"weigh_kernel", "pair_kernel", "tail_kernel", "solve_kernel",
                                   "assoc_element_kernel", "assoc_scan_kernel", "assoc_smooth_kernel",
                                   "refine_kernel", "fp32_pair_kernel", "fp32_solve_kernel",
                                   "refine_residual_kernel", "refine_rt_kernel", "refine_solve_kernel",
                                   "build_kernel", "filter_kernel", "df_weigh_kernel", "df_pair_kernel",
                                   "df_tail_kernel", "df_solve_kernel"};

cudaEvent_t get_event()
{
  if (!tl.pool.empty()) {
    cudaEvent_t e = tl.pool.back();
    tl.pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

}  // namespace

void ukg_prof_before(cudaStream_t st, int kind, cudaEvent_t* mark)
{
  tl.launches++;
  if (!tl.on) return;
  *mark = get_event();
  cudaEventRecord(*mark, st);
}

void ukg_prof_after(cudaStream_t st, int kind, cudaEvent_t mark)
{
  if (!tl.on) return;
  cudaEvent_t b = get_event();
  cudaEventRecord(b, st);
  tl.pending.push_back(Pending{kind, mark, b});
}

void ukg_prof_collect(void)
{
  for (auto& p : tl.pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      tl.ms[p.kind] += ms;
      tl.count[p.kind] += 1;
    }
    tl.pool.push_back(p.a);
    tl.pool.push_back(p.b);
  }
  tl.pending.clear();
  cudaGetLastError();
}

int ukg_prof_pause(void)
{
  const int was = tl.on ? 1 : 0;
  tl.on = false;
  return was;
}

void ukg_prof_resume(int previous) { tl.on = previous != 0; }

extern "C" void kalman_gpu_profile_enable(int on)
{
  tl.on = on != 0;
  for (int k = 0; k < UKG_K_COUNT; ++k) {
    tl.ms[k] = 0;
    tl.count[k] = 0;
  }
}

extern "C" int kalman_gpu_profile_read(int max_kinds, const char** names, double* total_ms, int64_t* launches)
{
  ukg_prof_collect();
  int n = 0;
  for (int k = 0; k < UKG_K_COUNT && n < max_kinds; ++k) {
    if (tl.count[k] == 0) continue;
    if (names) names[n] = kNames[k];
    if (total_ms) total_ms[n] = tl.ms[k];
    if (launches) launches[n] = tl.count[k];
    ++n;
  }
  return n;
}

extern "C" int64_t kalman_gpu_launch_count(void) { return tl.launches; }

/* ---------------------------------------------------------------------------
 * FP64 pipe probe: independent fused multiply-add chains, 8 per thread
 * ------------------------------------------------------------------------ */
__global__ void fp64_fma_probe(double* out, int iters, double a, double b, int lanes)
{
  if ((int)(threadIdx.x & 31) >= lanes) return; /* partially active warps */
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 1234.5) out[blockIdx.x] = s; /* keeps the chains alive */
}

__global__ void fp32_fma_probe(float* out, int iters, float a, float b)
{
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 1234.5f) out[blockIdx.x] = s;
}

extern "C" double kalman_gpu_measure_fp32_tflops(void)
{
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0.0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  float* out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * sms * 8) != cudaSuccess) return 0.0;
  const int blocks = sms * 8, threads = 256, iters = 16384;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  fp32_fma_probe<<<blocks, threads>>>(out, iters, 0.9999f, 1e-4f);
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(a);
    fp32_fma_probe<<<blocks, threads>>>(out, iters, 0.9999f, 1e-4f);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  return 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
}

extern "C" double kalman_gpu_measure_fp64_tflops(int active_lanes)
{
  if (active_lanes < 1 || active_lanes > 32) active_lanes = 32;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0.0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * sms * 8) != cudaSuccess) return 0.0;
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  fp64_fma_probe<<<blocks, threads>>>(out, iters, 0.999999, 1e-7, active_lanes); /* warm-up */
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(a);
    fp64_fma_probe<<<blocks, threads>>>(out, iters, 0.999999, 1e-7, active_lanes);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * iters * (double)blocks * (threads / 32) * active_lanes;
  return flops / (best * 1e-3) / 1e12;
}
