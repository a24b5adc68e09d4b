/*
 * kalman_gpu.h -- entry points that libukgpu.so adds beside the reference API
 * of kalman.h.  None of them has a counterpart in UltimateKalman; each one
 * exists because the GPU boundary needs it:
 *
 *  - error reporting: the reference aborts on errors (assert), a library on a
 *    shared GPU must not;
 *  - a batched entry over many independent tracks (one launch sequence for
 *    thousands of smoothing problems);
 *  - a device-resident entry that takes packed arrays already in GPU memory,
 *    so a caller can keep inputs in HBM and skip the host marshalling.
 *
 * Packed layout (host or device arrays, FP64, column-major blocks):
 *
 *   steps of all tracks are concatenated; track t owns global steps
 *   [track_start[t], track_start[t+1]).  The first step of every track has no
 *   evolution equation: its H, F, c, K slots are ignored.
 *
 *   H, F       [nsteps][n*n]     evolution  H_i x_i = F_i x_{i-1} + c_i + e_i
 *   c          [nsteps][n]
 *   K          [nsteps][n*n]     covariance factor of e_i, type K_type[i]
 *                                ('w': the first n entries hold the column)
 *   G          [nsteps][mmax*n]  observation G_i x_i = o_i + d_i, ld = mmax
 *   o          [nsteps][mmax]
 *   C          [nsteps][mmax*mmax] covariance factor of d_i, ld = mmax,
 *                                type C_type[i] ('w': first m_i entries)
 *   obs_rows   [nsteps]          m_i, the rows of G_i; 0 = no observation
 *   state      [nsteps][n]       output
 *   covariance [nsteps][n*n]     output (may be NULL with KALMAN_NO_COVARIANCE)
 *
 * The covariance-type letters are those of kalman.h.
 */
#ifndef KALMAN_GPU_H
#define KALMAN_GPU_H

#include <stdint.h>
#include "kalman.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes returned by the int-valued entry points and recorded for the
 * void-valued reference entry points.                                        */
enum {
  KALMAN_GPU_OK        = 0,
  KALMAN_GPU_EINVAL    = 1,  /* bad argument or unsupported shape            */
  KALMAN_GPU_ECUDA     = 2,  /* CUDA runtime error                           */
  KALMAN_GPU_ENOMEM    = 3,  /* device or pinned-host allocation failed      */
  KALMAN_GPU_ESINGULAR = 4,  /* a zero pivot: the problem is not observable;
                                affected outputs are NaN                     */
  KALMAN_GPU_ENODEV    = 5   /* no CUDA device                               */
};

/* Option bit added to kalman_options_t: factor in FP32 and refine the
 * estimates with FP64 residuals of the least-squares system.                 */
#define KALMAN_GPU_FP32_REFINE (1u << 20)
/* Number of refinement sweeps with KALMAN_GPU_FP32_REFINE (1..3; 0 selects the
 * default, 2).  Each sweep multiplies the error by about eps32 * cond(A)^2.  */
#define KALMAN_GPU_REFINE_SWEEPS(k) (((uint32_t)(k) & 3u) << 21)

/* Last error of the calling thread: status code and a one-line message.     */
int         kalman_gpu_last_status(void);
const char* kalman_gpu_last_error(void);
void        kalman_gpu_clear_error(void);

/* Where the arrays of a kalman_gpu_problem_t live.  Host arrays are copied to
 * the device and the outputs back inside the call (page-locked host memory
 * makes the copies faster).                                                  */
#define KALMAN_GPU_DEVICE 0
#define KALMAN_GPU_HOST   1

typedef struct kalman_gpu_problem_st {
  int32_t n;
  int32_t mmax;
  int32_t ntracks;
  int32_t location;             /* KALMAN_GPU_DEVICE or KALMAN_GPU_HOST     */
  int64_t nsteps;
  const int64_t* track_start;   /* always a HOST array of ntracks+1 entries  */
  const double*  H;
  const double*  F;
  const double*  c;
  const double*  K;
  const char*    K_type;
  const double*  G;
  const double*  o;
  const double*  C;
  const char*    C_type;
  const int32_t* obs_rows;
  double*        state;
  double*        covariance;
} kalman_gpu_problem_t;

/* Odd-even (Gargir-Toledo) smoothing of every track of a packed problem, on
 * the given CUDA stream (NULL: the legacy default stream).  Returns a status
 * code.  With device arrays the call returns once the work is queued on the
 * stream, except that it waits for the stream to report singular pivots;
 * with host arrays it returns when the outputs are back in host memory.     */
int kalman_gpu_smooth_oddeven_packed    (uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream);
/* Associative-scan (Sarkka-Garcia-Fernandez) smoothing of a packed problem.  */
int kalman_gpu_smooth_associative_packed(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream);

/* First-step observations apart from the packed rows (no reference
 * counterpart).  A track's first step often has more observation rows than
 * its other steps (a prior folded into a square observation: n rows against
 * m), and the packed layout stores every step with mmax rows -- padding that
 * is a quarter of the bytes of a 6-state, 3-observation problem.  Here p
 * describes every step with p->mmax observation rows, except that the first
 * step of each track takes its observation from f0 (arrays in the same
 * location as p's; the first steps' own G, o, C, C_type, obs_rows slots are
 * ignored):
 *   G0         [ntracks][m0max*n]      ld = m0max
 *   o0         [ntracks][m0max]
 *   C0         [ntracks][m0max*m0max]  ld = m0max, type C0_type[t]
 *   C0_type    [ntracks]
 *   obs_rows0  [ntracks]               rows of track t's first observation
 * The odd-even smoother then runs as kalman_gpu_smooth_oddeven_packed would
 * on the padded problem (the same results, bit for bit): with host arrays the
 * library copies the compact arrays and pads them on the device, so the host
 * link carries no padding.                                                   */
typedef struct kalman_gpu_first_obs_st {
  int32_t m0max;
  const double*  G0;
  const double*  o0;
  const double*  C0;
  const char*    C0_type;
  const int32_t* obs_rows0;
} kalman_gpu_first_obs_t;
int kalman_gpu_smooth_oddeven_first_obs(uint32_t options, const kalman_gpu_problem_t* p,
                                        const kalman_gpu_first_obs_t* f0, void* cuda_stream);

/* Batched form of kalman_smooth_oddeven / kalman_smooth_associative: the
 * equations of ntracks independent tracks are stored one track after the
 * other; track t has track_lengths[t] steps.  Results are written into the
 * equations as the single-track entry points do.                            */
int kalman_gpu_smooth_tracks(uint32_t options, kalman_step_equations_t** equations,
                             const kalman_step_index_t* track_lengths, int32_t ntracks);

/* Filtered estimates (the sequential UltimateKalman filter of
 * c/kalman_ultimate.c: evolve 140-345, observe 347-557 with its estimate 508-545) for
 * every step of every track of a packed problem with DEVICE arrays: state[s]
 * = x_{s|s} and, unless KALMAN_NO_COVARIANCE, covariance[s] = P_{s|s}
 * (column-major), from the equations of the track's steps up to s.  Steps
 * whose state is not yet determined get NaN and the call returns
 * KALMAN_GPU_ESINGULAR.  Tracks run in parallel, steps in sequence.  n and
 * mmax <= 128.  Returns when the results are in place.  No counterpart in the
 * reference's ABI (its filter runs one step per kalman_evolve/observe call). */
int kalman_gpu_filter_packed(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream);

/* Device-side equation builder for tracks whose model does not change along
 * the track (no reference counterpart: it stands in for the kalman_evolve /
 * kalman_observe loop of c/kalman_explicit_representation.c:164-244, which
 * builds every step's matrices on the host).  Fills steps first .. first+k-1
 * of the packed DEVICE arrays that p points to (H, F, c, K, K_type, G, o, C,
 * C_type, obs_rows; step `first` is the track's step 0):
 *   step 0:        no evolution (H, F, c, K zero, K_type 'C'); the observation
 *                  G0 (m0 x n), o0 (m0), C0 (m0 x m0, type C0_type);
 *   steps 1..k-1:  the evolution H, F (n x n), c (n), K (n x n, type K_type);
 *                  the observation G (m x n), C (m x m, type C_type) and
 *                  o + (i-1)*ldo (m entries), with obs_rows[i-1] rows (NULL:
 *                  m at every step; 0 marks a missing observation).
 * Model matrices are column-major with ld = rows, in device memory; unused
 * rows of the packed G, o, C are zero.  m0, m <= p->mmax.  Queued on
 * cuda_stream; returns a status code.                                       */
typedef struct kalman_gpu_invariant_model_st {
  int32_t m0, m;
  const double *H, *F, *c, *K;
  char K_type;
  const double *G0, *o0, *C0;
  char C0_type;
  const double *G, *C;
  char C_type;
} kalman_gpu_invariant_model_t;
int kalman_gpu_expand_invariant(const kalman_gpu_problem_t* p, int64_t first, int64_t k,
                                const kalman_gpu_invariant_model_t* model, const double* o, int64_t ldo,
                                const int32_t* obs_rows, void* cuda_stream);

/* Kernel timing.  While enabled (per host thread), each kernel launch of the
 * smoothers is bracketed by CUDA events on its stream.  _read returns, per
 * kernel class that ran since it was enabled, its name, summed time (ms) and
 * launch count.                                                              */
void    kalman_gpu_profile_enable(int on);
int     kalman_gpu_profile_read(int max_kinds, const char** names, double* total_ms, int64_t* launches);
/* Number of kernels this host thread has launched through the library.      */
int64_t kalman_gpu_launch_count(void);
/* Measures the FP64 fused-multiply-add throughput of the current device in
 * TFLOP/s, with `active_lanes` (1..32) active threads per warp.  A diagnostic
 * for roofline reporting; takes a few milliseconds.                          */
double  kalman_gpu_measure_fp64_tflops(int active_lanes);
/* The same for FP32 fused multiply-adds (all lanes active).                 */
double  kalman_gpu_measure_fp32_tflops(void);
/* Checks the device-side failure path of the library's bounded waits: one
 * thread block arms an mbarrier for a transfer that nothing delivers, waits
 * with the same bound as the kernels' waits on their bulk copies (about a
 * second), and reports the outcome through the same error flag.  Returns
 * KALMAN_GPU_ECUDA with the message of a copy that did not complete in time
 * (the expected outcome), KALMAN_GPU_OK if the wait was satisfied, or the
 * status of a CUDA error.  No asynchronous copy is in flight when the block
 * exits.  A diagnostic; takes about a second.                               */
int     kalman_gpu_check_bounded_wait(void* cuda_stream);

/* Allocation-free odd-even smoothing of a packed problem held in DEVICE
 * memory.  No counterpart in the reference: it exists for callers that must
 * not allocate device memory while they run -- real-time tracking loops with
 * a no-allocation rule (cudaMalloc/cudaFree may synchronize the device and
 * take unbounded time) and plugins whose host program owns all device memory.
 * The smoother's scratch comes from a fixed array of
 * KALMAN_GPU_NOALLOC_SCRATCH_BYTES that every device loading the library
 * holds until the process exits (about 24,000 steps of a 6-state model with
 * covariances fit); larger problems are rejected with KALMAN_GPU_EINVAL.  The
 * caller passes the input and output arrays.  The first call on a device looks
 * up the array's device address (make it before any stream capture).  Calls
 * share the array: they are serialized and each waits for its kernels; work
 * that overlapped a call on the GPU would race on it.  Every call blocks the
 * host until its kernels have finished: it synchronizes the stream to read the
 * status.  It runs the plain FP64 smoother (per-thread kernels at every state
 * dimension up to the scratch limit); KALMAN_GPU_FP32_REFINE is refused with
 * KALMAN_GPU_EINVAL.                                                         */
#define KALMAN_GPU_NOALLOC_SCRATCH_BYTES (64u << 20)
int kalman_gpu_smooth_oddeven_noalloc(uint32_t options, const kalman_gpu_problem_t* p, void* cuda_stream);

/* Prepared plans, replayed as CUDA graphs.  No counterpart in the reference
 * (which rebuilds its step structures on every call).
 *
 * For callers that smooth problems of one fixed shape again and again (a
 * tracker re-smoothing a sliding window of the same length every frame, a
 * service with a few fixed request sizes): kalman_gpu_plan_create takes a
 * problem of device arrays (location KALMAN_GPU_DEVICE), builds the plan
 * tables into a workspace the plan owns and captures the whole launch
 * sequence into a CUDA graph.  kalman_gpu_plan_execute replays it on a stream
 * -- asynchronously, with the current contents of the same device arrays, so
 * the caller refills them between executions; the track lengths, n, mmax,
 * the array addresses and the options are those of the creation.
 * kalman_gpu_plan_status waits for the last execution and returns its status
 * (the KALMAN_GPU_* codes above).  create returns NULL on failure (see
 * kalman_gpu_last_error).  A plan belongs to the device current at its
 * creation; executions of one plan must not overlap on the GPU (they share
 * its workspace). */
typedef struct kalman_gpu_plan kalman_gpu_plan_t;
kalman_gpu_plan_t* kalman_gpu_plan_create(uint32_t options, const kalman_gpu_problem_t* p);
int kalman_gpu_plan_execute(kalman_gpu_plan_t* plan, void* cuda_stream);
int kalman_gpu_plan_status(kalman_gpu_plan_t* plan);
void kalman_gpu_plan_destroy(kalman_gpu_plan_t* plan);

/* HBM accounting for callers that budget device memory (a serving loop
 * admitting requests by memory; no reference counterpart).
 * kalman_gpu_oddeven_workspace_bytes: device bytes kalman_gpu_smooth_oddeven_packed
 * caches for problem p under these options (its workspace grows to the
 * largest problem a host thread has smoothed and is kept); -1 if p is
 * malformed.  kalman_gpu_workspace_held: device bytes of workspace and
 * staging the calling host thread holds now (all entry points).            */
int64_t kalman_gpu_oddeven_workspace_bytes(uint32_t options, const kalman_gpu_problem_t* p);
int64_t kalman_gpu_workspace_held(void);

/* Launch tuning of the odd-even smoother (no reference counterpart; the
 * reference's only knob is the TBB grain, parallel_set_blocksize).  The
 * setting is process-wide and applies to calls (and plans) that start after
 * it; the project's autotuner (ultimate_kalman_gb300/autotune.py) measures
 * the choices per problem class and records the best.
 *   cta_min_n    state dimension from which one thread block takes a work
 *                item (a step pair, a tail, an even step) instead of one
 *                thread; 1..129 (129: never below 129 states), default 9.
 *                Shapes with more than 8 observation rows always use blocks.
 *   ctas_per_sm  thread blocks per SM of the block-per-item kernels'
 *                persistent grid, 1..16, default 4.
 *   pair_block   threads per block of the FP32 register-tile pair kernel
 *                (precision form, n = 4 and 6): 32, 64 or 128, default 64.
 *   weigh_block  steps per block of the double-float weighing kernel
 *                (precision form, n = 4 and 6): 64, 128 or 256, default 128.
 * kalman_gpu_set_tuning(NULL) restores the defaults; values outside these
 * ranges are refused with KALMAN_GPU_EINVAL (the setting is unchanged).    */
typedef struct kalman_gpu_tuning_st {
  int32_t cta_min_n;
  int32_t ctas_per_sm;
  int32_t pair_block;
  int32_t weigh_block;
} kalman_gpu_tuning_t;
int  kalman_gpu_set_tuning(const kalman_gpu_tuning_t* t);
void kalman_gpu_get_tuning(kalman_gpu_tuning_t* t);

/* Releases the device workspace and pinned staging buffers cached by the
 * library for the current device.                                            */
void kalman_gpu_release(void);

#ifdef __cplusplus
}
#endif

#endif /* KALMAN_GPU_H */
