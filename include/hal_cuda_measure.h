/* hal_cuda_measure.h -- measurement hooks of libhal_cuda.so.
 *
 * These entry points are instrumentation, not part of the drop-in boundary of
 * include/hal_cuda.h: no HAL-CPP interface has a counterpart, and model code
 * never needs them.  Benchmarks and profiling runs use them to time single
 * kernels with CUDA events and to count the library's kernel launches.  They
 * are exported by the same library as the backend calls and use its handles
 * and status codes.
 */
#ifndef HAL_CUDA_MEASURE_H
#define HAL_CUDA_MEASURE_H

#include "hal_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- library ------------------------------------------------------------ */

/* Number of kernel launches this library has issued in this process (all
 * handles).  Used by benchmarks to report their launch counts. */
int64_t hal_cuda_launch_count(void);

/* Measured FP64 add issue rate of the current device (operations per second,
 * best of three timed launches of independent add chains on every SM).  The
 * FP64 stencils (hal_cuda_diffuse*, hal_cuda_advect*) are bound by this rate
 * on GB300, whose FP64 pipe is a small fraction of its FP32 one; benchmarks
 * use it as their roofline. */
int hal_cuda_fp64_issue_rate(double *opsPerSecond);

/* Check of the FP64 ADI's division (DiffusionADI's back substitution,
 * hal_cuda_pdegrid_diffusion_adi and the exact hal_cuda_adi calls): for every
 * num[i] and den[j] the device divides once by IEEE division (__ddiv_rn) and
 * once as the sweeps do -- from den's reciprocal as a double-word with one
 * Markstein correction, with IEEE division for a numerator that is -0,
 * subnormal, nonzero below 2^-900 or from 2^900 in magnitude, inf or NaN --
 * and *mismatches receives the number of pairs whose bit patterns differ.
 * Every den[j] must lie in [2^-20, 2^20], the range in which the sweeps use
 * that division; host arrays. */
int hal_cuda_check_plan_division(const double *num, int64_t nNum, const double *den, int32_t nDen,
                                 int64_t *mismatches);

/* ---- explicit diffusion -------------------------------------------------- */

/* Profiling of the FP64 stencils above (zero-flux forms): average device time
 * (ms) of one launch on the arrays the last call of that kind uploaded, over
 * `iters` individually timed launches.  Deltas accumulate on the device. */
#define HAL_CUDA_STENCIL_DIFFUSE_VAR 0
#define HAL_CUDA_STENCIL_ADVECT 1
#define HAL_CUDA_STENCIL_ADVECT_VAR 2
int hal_cuda_stencil64_profile(hal_cuda_diffusion *h, int32_t kind, int32_t iters, double xVel,
                               double yVel, int32_t wrapX, int32_t wrapY, float *ms);

/* Failure-detection test hook of the two-tick kernel
 * (hal_cuda_diffusion_set_blocking(h, 2)): with stall set, every staged
 * tile's mbarrier expects 16 bytes more than its tensor copy brings, so the
 * kernel's bounded wait runs out -- no fault, no hang: each CTA waits
 * waitSeconds (0: the 2 s default) twice, records the failure in the handle's
 * device error word and returns without writing its tile.  The next
 * synchronising call (hal_cuda_diffusion_get_field) then returns
 * HAL_CUDA_ETIMEOUT, and the handle refuses every later tick, as after a real
 * staging failure.  stall 0 restores normal launches (of a handle that has not
 * stopped). */
int hal_cuda_diffusion_test_stall(hal_cuda_diffusion *h, int32_t stall, double waitSeconds);

/* Profiling: average device time (ms) of one fused-tick launch over `iters`
 * individually timed ticks (CUDA events, no graph).  The field advances. */
int hal_cuda_diffusion_profile(hal_cuda_diffusion *h, int32_t iters, double diffRate,
                               double decay, int32_t wrapX, int32_t wrapY, float *ms);

/* ---- ADI ------------------------------------------------------------------ */

/* Steady-state profiling: for each sweep, a CUDA graph of `iters`
 * back-to-back launches on the same inputs (the x-sweep rewrites w, the
 * y-sweep the other parity's field), replayed once to warm up and once timed;
 * ms[0] / ms[1] = the mean device time of one x- / y-sweep launch.  The
 * resident field does not change. */
int hal_cuda_adi_profile_graph(hal_cuda_adi *h, int32_t iters, double diffRate, double decay,
                               int32_t wrapX, int32_t wrapY, float *ms);

/* Profiling: runs `iters` ticks with each sweep launched on its own between
 * CUDA events on the handle's stream (no graph), and returns the average
 * device time of one launch of each kernel: ms[0] = x-sweep
 * (AdiSweep<kSweepW>), ms[1] = y-sweep with commit (AdiSweep<kSweepTick>).
 * The resident field advances by `iters` ticks. */
int hal_cuda_adi_profile(hal_cuda_adi *h, int32_t iters, double diffRate, double decay,
                         int32_t wrapX, int32_t wrapY, float *ms);

/* ---- agent forces ----------------------------------------------------------- */

/* Profiling: `iters` resident dispatches with each kernel launch between CUDA
 * events; ms[0..5] = average device time of one launch of: bin count
 * (including the counts memset), scan (three launches together), unstable
 * scatter, stabilize, forces, and the whole dispatch. */
int hal_cuda_agents_profile(hal_cuda_agents *h, int32_t iters, double interactionRad,
                            double springConstant, int32_t wrapX, int32_t wrapY, float *ms);

/* ---- batched wells ---------------------------------------------------------- */

/* Profiling: average device ms over `iters` ticks launched one kernel at a
 * time: ms[0] explicit tiles, ms[1] ADI x-sweep tiles, ms[2] ADI y-sweep
 * tiles, ms[3] agent pass, ms[4] whole tick.  Fields advance. */
int hal_cuda_wells_profile(hal_cuda_wells *h, int32_t iters, double interactionRad,
                           double springConstant, float *ms);

#ifdef __cplusplus
}
#endif

#endif
