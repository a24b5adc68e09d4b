/*
 * ukgpu_internal.h -- declarations shared by the translation units of
 * libukgpu.so (not installed; clients include include/kalman.h and
 * include/kalman_gpu.h).
 */
#ifndef UKGPU_INTERNAL_H
#define UKGPU_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#include "kalman_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* thread-local last error (host_api.cpp) */
int  ukg_set_error(int status, const char* fmt, ...);
void ukg_clear_error(void);

/* device smoothers on a packed problem whose arrays are in device memory
 * (oddeven.cu / associative.cu); cuda_stream may be NULL                      */
int ukg_oddeven_device(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream);
int ukg_associative_device(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream);

/* frees the filter's cached device workspace (filter.cu) */
void ukg_release_filter_workspace(void);

/* checks the arguments of a packed problem that do not need device access   */
int ukg_validate_problem(const kalman_gpu_problem_t* p, int need_cov);
/* Lets `kernel` launch with up to the device's opt-in maximum of dynamic
 * shared memory.  The attribute is process-wide, so it is raised once per
 * (device, kernel) to the maximum rather than set per call: per-call values
 * raced between host threads smoothing different shapes (one thread lowered
 * the limit just before another launched a larger request).              */
void ukg_allow_dynamic_smem(const void* kernel);
/* cudaMallocAsync from the device's default pool; if that fails, waits for
 * the stream, returns the pool's unused memory to the device (memory freed by
 * earlier workspaces stays reserved in the pool until trimmed) and tries once
 * more.  Returns the CUDA error code (0 on success).                         */
int ukg_malloc_async(void** ptr, size_t bytes, void* cuda_stream);
/* returns the default pool's unused memory of the current device            */
void ukg_trim_pool(void);
/* builder.cu: the padded observation layout of a problem with separate
 * first-step observations (kalman_gpu_smooth_oddeven_first_obs)            */
int ukg_pad_first_obs(const kalman_gpu_problem_t* p, const kalman_gpu_first_obs_t* f0, int mp, double* G, double* o,
                      double* C, char* ct, int32_t* rows, const int64_t* first, void* cuda_stream);
/* Workspace bytes to allocate for a problem needing `bytes`: 1/8 more, so a
 * slightly larger next problem reuses it, but at most 1 GiB more (a 150 GB
 * workspace must not hold 19 GB it will never use).                          */
static inline size_t ukg_with_slack(size_t bytes)
{
  const size_t extra = bytes >> 3;
  return bytes + (extra < ((size_t)1 << 30) ? extra : ((size_t)1 << 30));
}

#ifdef __cplusplus
}
#endif

#endif
