/* profiling.h -- internal hooks of profiling.cu (per-kernel CUDA-event timing) */
#ifndef UKGPU_PROFILING_H
#define UKGPU_PROFILING_H

#include <cuda_runtime.h>

enum {
  UKG_K_WEIGH = 0,
  UKG_K_PAIR,
  UKG_K_TAIL,
  UKG_K_SOLVE,
  UKG_K_AS_ELEMENT,
  UKG_K_AS_SCAN,
  UKG_K_AS_SMOOTH,
  UKG_K_REFINE,
  UKG_K_PAIR32,
  UKG_K_SOLVE32,
  UKG_K_RESID,
  UKG_K_RT,
  UKG_K_RSOLVE,
  UKG_K_BUILD,
  UKG_K_FILTER,
  UKG_K_DF_WEIGH, /* the precision form with covariances: double-float kernels */
  UKG_K_DF_PAIR,
  UKG_K_DF_TAIL,
  UKG_K_DF_SOLVE,
  UKG_K_COUNT
};

void ukg_prof_before(cudaStream_t st, int kind, cudaEvent_t* mark);
void ukg_prof_after(cudaStream_t st, int kind, cudaEvent_t mark);
void ukg_prof_collect(void);
/* turns event timing off for the calling thread; returns the previous state */
int  ukg_prof_pause(void);
void ukg_prof_resume(int previous);

/* brackets one kernel launch statement */
#define UKG_LAUNCH(kind, stream, launch)              \
  do {                                                \
    cudaEvent_t ukg_mark_ = nullptr;                  \
    ukg_prof_before((stream), (kind), &ukg_mark_);    \
    launch;                                           \
    ukg_prof_after((stream), (kind), ukg_mark_);      \
  } while (0)

#endif
