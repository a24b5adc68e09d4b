/*
 * associative.cu -- the associative-scan (Sarkka-Garcia-Fernandez) smoother on
 * the GPU.  (Kernels follow in the next commit; until then the entry point
 * reports that it is unavailable.)
 */
#include <cuda_runtime.h>

#include "ukgpu_internal.h"

extern "C" void ukg_release_associative_workspace(void) {}

extern "C" int ukg_associative_device(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream)
{
  (void)options; (void)p; (void)cuda_stream;
  return ukg_set_error(KALMAN_GPU_EINVAL, "the associative smoother is not built yet");
}
