/*
 * hal_cuda.h -- C ABI of the GB300 (sm_103a) compute backend for HAL-CPP.
 *
 * This is the drop-in boundary.  HAL-CPP's three per-tick strategy interfaces
 *   Hal::IDiffusionBackend2D     (include/Hal/Pde/IDiffusionBackend2D.h:13-33)
 *   Hal::IAdiDiffusionBackend2D  (include/Hal/Pde/IAdiDiffusionBackend2D.h:12-32)
 *   Hal::IAgentForceBackend2D    (include/Hal/Agents/IAgentForceBackend2D.h:15-37)
 * are implemented by the C++ classes Hal::Cuda::CudaDiffusionBackend2D,
 * CudaAdiDiffusionBackend2D and CudaAgentForceBackend2D, which call only the
 * functions below.  Signatures carry plain pointers and sizes; nothing here
 * needs CUDA or C++ headers.  The Vulkan classes these replace are
 *   Hal::Gpu::GpuDiffusionBackend2D     (src/Gpu/GpuDiffusionBackend2D.cpp:22-52)
 *   Hal::Gpu::GpuAdiDiffusionBackend2D  (src/Gpu/GpuAdiDiffusionBackend2D.cpp:24-50)
 *   Hal::Gpu::GpuAgentForceBackend2D    (src/Gpu/GpuAgentForceBackend2D.cpp:24-68)
 * and their kernel hosts DiffusionKernel2D / AdiKernel2D / AgentForceKernel2D.
 *
 * Conventions
 *   - Field layout is HAL's row-major i = x*yDim + y (y contiguous).
 *   - Every call returns an int status: HAL_CUDA_OK or one of the error codes.
 *     hal_cuda_last_error() gives the message of the calling thread's last
 *     failure.  HAL_CUDA_EINVAL maps to std::invalid_argument in the C++
 *     wrappers, every other error to std::runtime_error (the reference's
 *     convention: IDiffusionBackend2D.cpp:26-31, AdiKernel2D.cpp:66-70).
 *   - A handle is sized at creation (as the Vulkan backends are,
 *     GpuDiffusionBackend2D.h:18-20) and owns its device buffers and one CUDA
 *     stream.  A handle must not be used from two threads at once; separate
 *     handles may run on separate threads.
 *   - Calls that take host arrays are synchronous: results are in host
 *     memory when they return (DiffusionKernel2D.cpp:159-171).  The resident
 *     calls (set_field / run_ticks / get_field) keep the field in device
 *     memory between calls; run_ticks only enqueues work on the handle's
 *     stream, hal_cuda_*_sync waits for it.
 *   - Arithmetic is FP32 on the device (as in the Vulkan backends); the
 *     double-precision interface calls convert on the device.
 *   - Dirichlet boundaries ("ghost tables"): the reference's boundary
 *     callable bc(x, y) (PDEequations.h:50-98, ADIequations.h:339-378) is only
 *     evaluated one cell outside the grid, so it is passed as a table of
 *     2*yDim + 2*xDim values: [0, yDim) = bc(-1, y); [yDim, 2*yDim) =
 *     bc(xDim, y); then xDim values bc(x, -1); then xDim values bc(x, yDim).
 *     A NULL table selects the zero-flux form.  Wrapped axes ignore their
 *     part of the table, as the reference does.
 */
#ifndef HAL_CUDA_H
#define HAL_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HAL_CUDA_OK 0
#define HAL_CUDA_EINVAL 1   /* bad argument or size mismatch */
#define HAL_CUDA_ENOMEM 2   /* device or pinned-host allocation failed */
#define HAL_CUDA_EDEVICE 3  /* CUDA runtime error, no device, launch failure */
#define HAL_CUDA_ETIMEOUT 4 /* a bounded device-side wait gave up */
#define HAL_CUDA_ENOTSUP 5  /* a size or mode this build does not handle */

/* Longest line the FP32 partitioned ADI sweeps solve (the Vulkan AdiKernel2D
 * caps lines at kMaxLine = 1024, AdiKernel2D.h:41).  The resident ADI ticks
 * take lines up to this length; the interface calls (hal_cuda_diffuse_adi,
 * _adi_bc) take any length, solving longer lines in FP64 as the CPU backend
 * does. */
#define HAL_CUDA_ADI_MAX_LINE 4096

typedef struct hal_cuda_diffusion hal_cuda_diffusion; /* explicit stencil */
typedef struct hal_cuda_adi hal_cuda_adi;             /* ADI (implicit) */
typedef struct hal_cuda_agents hal_cuda_agents;       /* agent forces */

/* ---- library ------------------------------------------------------------ */

/* Version string of this library. */
const char *hal_cuda_version(void);

/* Message of the calling thread's most recent failed call ("" if none). */
const char *hal_cuda_last_error(void);

/* Number of visible CUDA devices; selects device `device` for handles created
 * afterwards on this thread (default 0).  Replaces ComputeContext creation
 * (include/Hal/Gpu/ComputeContext.h:18-49). */
int hal_cuda_device_count(int32_t *count);
int hal_cuda_set_device(int32_t device);

/* ---- explicit diffusion: IDiffusionBackend2D ---------------------------- */

/* GpuDiffusionBackend2D(ComputeContext&, xDim, yDim)
 * (include/Hal/Gpu/GpuDiffusionBackend2D.h:18-20). */
int hal_cuda_diffusion_create(int32_t xDim, int32_t yDim, hal_cuda_diffusion **out);
int hal_cuda_diffusion_destroy(hal_cuda_diffusion *h);

/* IDiffusionBackend2D::Diffuse (IDiffusionBackend2D.h:26-32): deltas[i] +=
 * diffRate * (sum of the four neighbour differences of field at i), zero-flux
 * or periodic per axis.  field/deltas are host arrays of fieldLen/deltasLen
 * doubles; EINVAL unless both equal xDim*yDim (Internal::CheckFieldSizes,
 * src/Pde/IDiffusionBackend2D.cpp:20-33) and xDim/yDim equal the handle's. */
int hal_cuda_diffuse(hal_cuda_diffusion *h, const double *field, int64_t fieldLen,
                     double *deltas, int64_t deltasLen, double diffRate, int32_t xDim,
                     int32_t yDim, int32_t wrapX, int32_t wrapY);

/* Same with a Dirichlet ghost table (Internal::Diffusion2<BCFn>,
 * PDEequations.h:264-287); ghost may be NULL (zero-flux). */
int hal_cuda_diffuse_bc(hal_cuda_diffusion *h, const double *field, double *deltas,
                        double diffRate, int32_t wrapX, int32_t wrapY, const double *ghost);

/* Per-cell rate diffusion (Internal::Diffusion2(field, deltas, diffRatesX,
 * diffRatesY, ...), src/Pde/PDEequations.cpp:199-230): deltas += the
 * rate-weighted neighbour differences; all arrays xDim*yDim in layout A.
 * FP64, bit-identical to the reference. */
int hal_cuda_diffuse_var(hal_cuda_diffusion *h, const double *field, double *deltas,
                         const double *ratesX, const double *ratesY, int32_t wrapX, int32_t wrapY);

/* First-order upwind advection at a uniform velocity (Internal::Advection2
 * (field, deltas, xVel, yVel, ...), src/Pde/PDEequations.cpp:380-412).
 * FP64, bit-identical to the reference. */
int hal_cuda_advect(hal_cuda_diffusion *h, const double *field, double *deltas, double xVel,
                    double yVel, int32_t wrapX, int32_t wrapY);

/* Upwind advection with per-cell velocities (Internal::Advection2(field,
 * deltas, xVels, yVels, ...), src/Pde/PDEequations.cpp:535-575): face
 * fluxes from the upwind cell.  FP64, bit-identical to the reference. */
int hal_cuda_advect_var(hal_cuda_diffusion *h, const double *field, double *deltas,
                        const double *xVels, const double *yVels, int32_t wrapX, int32_t wrapY);

/* Dirichlet forms of the two advection calls, with ghost tables in the layout
 * of the file header.  hal_cuda_advect_bc: Internal::Advection2<BCFn>
 * (include/Hal/Pde/PDEequations.h:413-447), an off-grid upwind neighbour
 * gives (bc - centre) * 2.  hal_cuda_advect_var_bc: Advection2<BCFn,
 * XVelBCFn, YVelBCFn> (:720-778), the off-grid field value and velocities
 * are the tables' values (only the x part of ghostXVel and the y part of
 * ghostYVel are read).  A NULL table reads as 0 (the zero-flux value). */
int hal_cuda_advect_bc(hal_cuda_diffusion *h, const double *field, double *deltas, double xVel,
                       double yVel, int32_t wrapX, int32_t wrapY, const double *ghost);
int hal_cuda_advect_var_bc(hal_cuda_diffusion *h, const double *field, double *deltas,
                           const double *xVels, const double *yVels, int32_t wrapX, int32_t wrapY,
                           const double *ghost, const double *ghostXVel, const double *ghostYVel);

/* Resident field (DiffusionKernel2D::UploadField / RunSteps,
 * src/Gpu/DiffusionKernel2D.cpp:173-304).  len must be xDim*yDim. */
int hal_cuda_diffusion_set_field(hal_cuda_diffusion *h, const float *field, int64_t len);
int hal_cuda_diffusion_get_field(hal_cuda_diffusion *h, float *field, int64_t len);

/* Per-tick terms of a HAL model tick on PDEGrid2D (PDEGrid2D.h:103-186):
 * dense source field (len xDim*yDim, NULL clears it), point sources
 * (cell index, value; nPoints 0 clears them), Dirichlet ghost table (NULL =
 * zero-flux).  Stored on the device until changed. */
int hal_cuda_diffusion_set_source(hal_cuda_diffusion *h, const float *dense, int64_t len);
int hal_cuda_diffusion_set_point_sources(hal_cuda_diffusion *h, int32_t nPoints,
                                         const int32_t *cells, const float *values);
int hal_cuda_diffusion_set_dirichlet(hal_cuda_diffusion *h, const float *ghost);

/* Agent uptake coupling of the explicit tick: every agent of `agents`
 * (binned by its last dispatch or step) multiplies its cell by -uptake each
 * tick, as a model's PDEGrid2D::Mul(cell, -uptake) per agent
 * (PDEGrid2D.h:126-130, examples/CompetitiveRelease.cpp:147) before
 * Update.  The agent handle's grid must match; agents NULL removes the
 * coupling.  Coupled ticks run one per launch. */
int hal_cuda_diffusion_set_uptake(hal_cuda_diffusion *h, hal_cuda_agents *agents, double uptake);

/* Ticks per launch of the resident explicit tick: 1, 2 (temporal blocking:
 * a CTA stages its tile with a 2-cell halo by TMA and computes two ticks in
 * shared memory, so a pair of ticks reads and writes the field once), or 0
 * (the default: 1, which measures faster on GB300 at every size -- the
 * one-tick kernel streams large fields at over 80% of HBM peak, and the
 * two-tick kernel spends more instructions per cell than it saves in
 * bytes).  Two ticks need yDim % 4 == 0 (ENOTSUP otherwise).  With 2 the
 * dense source and the point sources are added as one pre-summed array, so
 * results match the one-tick launches to FP32 rounding, not bit for bit. */
int hal_cuda_diffusion_set_blocking(hal_cuda_diffusion *h, int32_t ticksPerLaunch);

/* Uniform advection velocity of every following tick (PDEGrid2D::Advection
 * (xVel, yVel[, bc]), PDEGrid2D.h:351-375, after the diffusion term): first-
 * order upwind, with the handle's Dirichlet table when one is set.  EINVAL
 * if |xVel| + |yVel| > 0.5 (CheckAdvectionStable, PDEGrid2D.h:444-450).
 * (0, 0), the default, is pure diffusion. */
int hal_cuda_diffusion_set_velocity(hal_cuda_diffusion *h, double xVel, double yVel);

/* `ticks` fused ticks on the resident field, each
 *   f' = f + diffRate*L_bc(f) [+ advection] - decay*f + src + points
 *        - uptake*count*f
 * (PDEGrid2D::Diffusion + MulAll(-decay) + Add + Mul + Update).  EINVAL if
 * diffRate > 0.25 (PDEGrid2D::CheckDiffusionStable, PDEGrid2D.h:436-442).
 * Asynchronous on the handle's stream; a run of ticks is replayed from a
 * CUDA graph. */
int hal_cuda_diffusion_run_ticks(hal_cuda_diffusion *h, int32_t ticks, double diffRate,
                                 double decay, int32_t wrapX, int32_t wrapY);

/* DiffusionKernel2D::RunSteps(field, steps, diffRate, wrapX, wrapY)
 * (src/Gpu/DiffusionKernel2D.cpp:244-304): upload, `steps` plain stencil
 * steps with commit, download.  field is a host array of len floats. */
int hal_cuda_diffusion_run_steps(hal_cuda_diffusion *h, float *field, int64_t len,
                                 int32_t steps, double diffRate, int32_t wrapX, int32_t wrapY);

int hal_cuda_diffusion_sync(hal_cuda_diffusion *h);

/* The handle's CUDA stream (a cudaStream_t), or replace it with the caller's
 * (NULL restores the handle's own).  Resident calls run on this stream. */
void *hal_cuda_diffusion_stream(hal_cuda_diffusion *h);
int hal_cuda_diffusion_set_stream(hal_cuda_diffusion *h, void *stream);

/* ---- ADI: IAdiDiffusionBackend2D --------------------------------------- */

/* GpuAdiDiffusionBackend2D(ComputeContext&, xDim, yDim)
 * (include/Hal/Gpu/GpuAdiDiffusionBackend2D.h).  Any size whose cell count
 * fits int32; with a side above HAL_CUDA_ADI_MAX_LINE the resident ticks
 * (run_ticks, profile) return EINVAL and only the interface calls run. */
int hal_cuda_adi_create(int32_t xDim, int32_t yDim, hal_cuda_adi **out);
int hal_cuda_adi_destroy(hal_cuda_adi *h);

/* IAdiDiffusionBackend2D::DiffuseADI (IAdiDiffusionBackend2D.h:25-31):
 * deltas[i] += v[i] - field[i], v = one ADI step of field
 * (Internal::Diffusion2DADI, ADIequations.h:306-337).  Host double arrays;
 * size checks as hal_cuda_diffuse.  Sides up to HAL_CUDA_ADI_MAX_LINE run the
 * FP32 partitioned solve (max error 2e-6 (1 + r) of the field); with a longer
 * side the step is the FP64 Thomas solve per line, bit-exact to the CPU
 * backend. */
int hal_cuda_diffuse_adi(hal_cuda_adi *h, const double *field, int64_t fieldLen,
                         double *deltas, int64_t deltasLen, double diffRate, int32_t xDim,
                         int32_t yDim, int32_t wrapX, int32_t wrapY);

/* Same with a Dirichlet ghost table (Diffusion2DADI<BCFn>,
 * ADIequations.h:339-378). */
int hal_cuda_diffuse_adi_bc(hal_cuda_adi *h, const double *field, double *deltas,
                            double diffRate, int32_t wrapX, int32_t wrapY, const double *ghost);

/* Exact mode of the two interface calls above (no reference counterpart: a
 * choice of this backend).  With exact nonzero, hal_cuda_diffuse_adi and
 * _adi_bc solve every size with the FP64 Thomas solve per line, bit-exact to
 * the CPU backend (CpuAdiDiffusionBackend2D); 0, the default, keeps the FP32
 * partitioned solve for sides up to HAL_CUDA_ADI_MAX_LINE.  The resident
 * ticks are not affected. */
int hal_cuda_adi_set_exact(hal_cuda_adi *h, int32_t exact);

/* Resident field and per-tick terms, as for the explicit handle. */
int hal_cuda_adi_set_field(hal_cuda_adi *h, const float *field, int64_t len);
int hal_cuda_adi_get_field(hal_cuda_adi *h, float *field, int64_t len);
int hal_cuda_adi_set_source(hal_cuda_adi *h, const float *dense, int64_t len);
int hal_cuda_adi_set_dirichlet(hal_cuda_adi *h, const float *ghost);

/* Agent uptake coupling: every agent of `agents` (binned by its last
 * dispatch) multiplies its cell by -uptake each tick, as a model's
 * PDEGrid2D::Mul(cell, -uptake) per agent (PDEGrid2D.h:126-130).  The agent
 * handle's grid must match.  agents NULL removes the coupling. */
int hal_cuda_adi_set_uptake(hal_cuda_adi *h, hal_cuda_agents *agents, double uptake);

/* `ticks` ADI ticks on the resident field, each
 *   f' = ADI(f) - decay*f + src - uptake*count*f
 * (PDEGrid2D::DiffusionADI + MulAll + Add + Mul + Update).  Asynchronous;
 * replayed from a CUDA graph. */
int hal_cuda_adi_run_ticks(hal_cuda_adi *h, int32_t ticks, double diffRate, double decay,
                           int32_t wrapX, int32_t wrapY);

/* `ticks` coupled ticks of a model like examples/CompetitiveRelease.cpp:
 * each tick is one resident step of `agents` (hal_cuda_agents_step with the
 * linear law: bins, forces, SphericalAgent2D's move) followed by one
 * hal_cuda_adi_run_ticks tick whose commit takes up -uptake*count*f with
 * the counts of that step's bins.  `agents` must be the handle coupled by
 * hal_cuda_adi_set_uptake (same grid); its axes wrap as the field's.  The
 * results equal alternating hal_cuda_agents_step(agents, 1, ...) and
 * hal_cuda_adi_run_ticks(h, 1, ...) calls bit for bit; here the ticks run
 * on the ADI handle's stream as one cached CUDA graph, ordered after the
 * agent handle's queued work and before its later work.  Asynchronous. */
int hal_cuda_adi_run_coupled(hal_cuda_adi *h, hal_cuda_agents *agents, int32_t ticks, double diffRate,
                             double decay, int32_t wrapX, int32_t wrapY, double interactionRad,
                             double springConstant, double friction, double maxVel);

/* AdiKernel2D::RunSteps(field, steps, diffRate, wrapX, wrapY)
 * (src/Gpu/AdiKernel2D.cpp:296-364): upload, `steps` ADI steps, download. */
int hal_cuda_adi_run_steps(hal_cuda_adi *h, float *field, int64_t len, int32_t steps,
                           double diffRate, int32_t wrapX, int32_t wrapY);

/* The same ticks as hal_cuda_adi_run_ticks, end to end from host memory:
 * field and src (src may be NULL) are uploaded, `ticks` ticks run, the field
 * is downloaded into `field`.  Synchronous. */
int hal_cuda_adi_run_ticks_host(hal_cuda_adi *h, float *field, const float *src, int64_t len,
                                int32_t ticks, double diffRate, double decay, int32_t wrapX,
                                int32_t wrapY);

int hal_cuda_adi_sync(hal_cuda_adi *h);
void *hal_cuda_adi_stream(hal_cuda_adi *h);
int hal_cuda_adi_set_stream(hal_cuda_adi *h, void *stream);

/* ---- agent forces: IAgentForceBackend2D --------------------------------- */

/* GpuAgentForceBackend2D(ComputeContext&, xDim, yDim, maxAgents)
 * (src/Gpu/GpuAgentForceBackend2D.cpp:9-18). */
int hal_cuda_agents_create(int32_t xDim, int32_t yDim, int32_t maxAgents,
                           hal_cuda_agents **out);
int hal_cuda_agents_destroy(hal_cuda_agents *h);

/* IAgentForceBackend2D::AccumulateForces (IAgentForceBackend2D.h:28-36):
 * positions (posLen = 2n doubles, x0 y0 x1 y1 ...), radii (radLen = n), out
 * velocityDeltas (2n doubles, overwritten).  EINVAL unless posLen ==
 * 2*radLen, xDim/yDim match the handle and n <= maxAgents
 * (GpuAgentForceBackend2D.cpp:34-46).  Positions, radii and the force sum
 * stay FP64 on the device, with IEEE operations in the CPU backend's order:
 * bins, bucket order and velocity deltas are bit-identical to
 * CpuAgentForceBackend2D's. */
int hal_cuda_accumulate_forces(hal_cuda_agents *h, const double *positions, int64_t posLen,
                               const double *radii, int64_t radLen, double *velocityDeltas,
                               double interactionRad, double springConstant, int32_t xDim,
                               int32_t yDim, int32_t wrapX, int32_t wrapY);

/* Overlap force laws.  SphericalAgent2D::SumForces (include/Hal/Agents/
 * SphericalAgent2D.h:74-102) takes a functor overlapFun(touchDist, other) ->
 * force, where touchDist = (r_i + r_j) - d is positive for overlapping agents;
 * a device kernel cannot call a host functor, so the law is one of:
 *   HAL_CUDA_FORCE_LINEAR          scale * touchDist (the interface's law,
 *                                  CpuAgentForceBackend2D.cpp:165)
 *   HAL_CUDA_FORCE_LINEAR_CLAMPED  0 when touchDist < 0, else scale * touchDist
 *                                  (examples/OffLatticeExample.cpp:147-154)
 *   HAL_CUDA_FORCE_POWER           pow(scale * touchDist, exponent)
 *                                  (examples/Chemotaxis.cpp:128-130)
 * A positive force pushes the agents apart. */
#define HAL_CUDA_FORCE_LINEAR 0
#define HAL_CUDA_FORCE_LINEAR_CLAMPED 1
#define HAL_CUDA_FORCE_POWER 2

typedef struct hal_cuda_force_law
{
    int32_t kind;    /* HAL_CUDA_FORCE_* */
    double scale;    /* the spring constant / force scaler */
    double exponent; /* HAL_CUDA_FORCE_POWER only */
} hal_cuda_force_law;

/* Order in which each agent visits its neighbours.  The cell window is
 * walked x-major then y in both; within a cell:
 *   HAL_CUDA_ORDER_BACKEND    ascending agent index, wrapped displacement
 *                             AgentForceDisp (CpuAgentForceBackend2D.cpp:
 *                             30-45, 112-175);
 *   HAL_CUDA_ORDER_AGENTGRID  descending agent index, wrapped displacement
 *                             DispX/DispY (src/Grids/GridGeometry2D.cpp:
 *                             132-150): AgentGrid2D::GetAgentsRadApprox
 *                             (include/Hal/Grids/AgentGrid2D.h:337-369) on a
 *                             grid whose agents were created in index order
 *                             (each square lists its newest agent first,
 *                             AgentPT2D.h:200-241). */
#define HAL_CUDA_ORDER_BACKEND 0
#define HAL_CUDA_ORDER_AGENTGRID 1

/* SphericalAgent2D::SumForces(interactionRad, overlapFun) for every agent at
 * once, FP64 (IEEE operations in the reference's order).  velocities (2n
 * doubles, may be NULL for zeros) are the agents' xVel/yVel before the call;
 * velocitiesOut (2n) receives them after it (velocities plus the forces'
 * change; with NULL velocities, the velocity deltas).  forceSums (n doubles,
 * may be NULL) receives each agent's SumForces return value: the sum of its
 * positive forces, which models gate division on (OffLatticeExample.cpp:
 * 156-165).  With HAL_CUDA_ORDER_AGENTGRID and the LINEAR or LINEAR_CLAMPED
 * law the results are bit-identical to SumForces on an AgentGrid2D whose
 * agents were created in index order; the POWER law calls the device's pow,
 * which can differ from the host's in the last bit.  Bins as in
 * hal_cuda_accumulate_forces; sizes as there. */
int hal_cuda_sum_forces(hal_cuda_agents *h, const double *positions, const double *radii, int64_t n,
                        const double *velocities, double *velocitiesOut, double *forceSums,
                        double interactionRad, const hal_cuda_force_law *law, int32_t order,
                        int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY);

/* Resident agents (AgentForceKernel2D::UploadAgents / Dispatch /
 * DownloadVelocityDeltas, src/Gpu/AgentForceKernel2D.cpp:173-290). */
int hal_cuda_agents_upload(hal_cuda_agents *h, const float *positions, const float *radii,
                           int32_t n);
int hal_cuda_agents_dispatch(hal_cuda_agents *h, double interactionRad, double springConstant,
                             int32_t wrapX, int32_t wrapY);
int hal_cuda_agents_download(hal_cuda_agents *h, float *velocityDeltas, int32_t n);

/* Device-resident agent integration (SphericalAgent2D, include/Hal/Agents/
 * SphericalAgent2D.h:133-162; MoveSafePT, include/Hal/Agents/AgentPT2D.h:
 * 157-186).  The handle keeps each agent's velocity (xVel, yVel) beside its
 * position; hal_cuda_agents_upload sets the velocities to zero
 * (DefaultInit).  One tick of hal_cuda_agents_step is a dispatch whose force
 * kernel then updates every agent i, in FP32 with each operation rounded to
 * nearest:
 *   vel_i += delta_i (the velocityDeltas of the dispatch);
 *   CapVelocity(maxVel) when maxVel >= 0 and finite;
 *   ForceMove: pos_i + vel_i if on the grid, else per axis: wrap a wrapped
 *     axis, keep the old coordinate of a closed axis that was left;
 *   ApplyFriction(friction): vel_i *= friction.
 * Positions stay on the device across ticks; the next tick bins the moved
 * agents.  hal_cuda_agents_download still returns the last tick's deltas.
 * Ticks are enqueued on the handle's stream; get_state synchronises. */
int hal_cuda_agents_set_velocities(hal_cuda_agents *h, const float *velocities, int32_t n);
int hal_cuda_agents_get_state(hal_cuda_agents *h, float *positions, float *velocities, int32_t n);
int hal_cuda_agents_step(hal_cuda_agents *h, int32_t ticks, double interactionRad,
                         double springConstant, int32_t wrapX, int32_t wrapY, double friction,
                         double maxVel);

/* The bins of the last dispatch: cellOffsets (xDim*yDim+1 int32, exclusive
 * prefix of per-cell counts, cellOffsets[C] == n) and bucketAgents (n int32,
 * agent indices grouped by cell, ascending within a cell) -- the scratch of
 * CpuAgentForceBackend2D (src/Agents/CpuAgentForceBackend2D.cpp:85-109).
 * Either pointer may be NULL. */
int hal_cuda_agents_get_bins(hal_cuda_agents *h, int32_t *cellOffsets, int32_t *bucketAgents);

/* The resident dispatch and step with a force law (HAL_CUDA_ORDER_BACKEND
 * order, FP32): as hal_cuda_agents_dispatch / hal_cuda_agents_step with the
 * law in place of the linear spring.  With withSums != 0 the force kernel also
 * writes each agent's sum of positive forces (SumForces' return value, in
 * FP32), which hal_cuda_agents_get_force_sums downloads (n = the uploaded
 * count; the sums of the step's last tick, at the positions it started from);
 * EINVAL when the last dispatch or step computed none. */
int hal_cuda_agents_dispatch_law(hal_cuda_agents *h, double interactionRad,
                                 const hal_cuda_force_law *law, int32_t withSums, int32_t wrapX,
                                 int32_t wrapY);
int hal_cuda_agents_step_law(hal_cuda_agents *h, int32_t ticks, double interactionRad,
                             const hal_cuda_force_law *law, int32_t withSums, int32_t wrapX,
                             int32_t wrapY, double friction, double maxVel);
int hal_cuda_agents_get_force_sums(hal_cuda_agents *h, float *forceSums, int32_t n);

int hal_cuda_agents_sync(hal_cuda_agents *h);
void *hal_cuda_agents_stream(hal_cuda_agents *h);
int hal_cuda_agents_set_stream(hal_cuda_agents *h, void *stream);

/* ---- device-resident PDEGrid2D -------------------------------------------
 * Hal::PDEGrid2D (include/Hal/Grids/PDEGrid2D.h:17-458) with its committed
 * field and its delta buffer kept in device memory, FP64.  Get reads the
 * committed field; the per-cell operations and the PDE operators accumulate
 * into the deltas; update commits them (field += deltas, deltas = 0, the
 * update count + 1).  Every call reproduces the reference's arithmetic bit
 * for bit, except hal_cuda_pdegrid_stats' average (a parallel sum; within
 * rounding of GetAvg).  Work is enqueued on the handle's stream; calls that
 * return values, or read caller arrays, synchronise it first.  EINVAL with
 * the reference's message where PDEGrid2D throws std::invalid_argument. */
typedef struct hal_cuda_pdegrid hal_cuda_pdegrid;

/* PDEGrid2D(xDim, yDim, wrapX, wrapY): field and deltas zero, count 0. */
int hal_cuda_pdegrid_create(int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY,
                            hal_cuda_pdegrid **out);
int hal_cuda_pdegrid_destroy(hal_cuda_pdegrid *h);

/* SetState(field, deltas, updateCt) (PDEGrid2D.h:58-75); deltas may be NULL
 * (zeros).  get_state: GetField / GetDeltas / UpdateCt, any pointer NULL to
 * skip it.  Arrays hold xDim*yDim doubles in HAL's layout. */
int hal_cuda_pdegrid_set_state(hal_cuda_pdegrid *h, const double *field, const double *deltas,
                               int32_t updateCt);
int hal_cuda_pdegrid_get_state(hal_cuda_pdegrid *h, double *field, double *deltas, int32_t *updateCt);
/* xDim, yDim, wrapX, wrapY, updateCt into dims[0..4]. */
int hal_cuda_pdegrid_dims(hal_cuda_pdegrid *h, int32_t *dims);

/* Per-cell operations (PDEGrid2D.h:88-140) on cell i = x*yDim + y:
 *   SET    deltas[i] = v - field[i]
 *   ADD    deltas[i] += v
 *   MUL    deltas[i] += field[i] * v
 *   SCALE  deltas[i] += field[i] * (v - 1)                              */
#define HAL_CUDA_CELL_SET 0
#define HAL_CUDA_CELL_ADD 1
#define HAL_CUDA_CELL_MUL 2
#define HAL_CUDA_CELL_SCALE 3

/* n operations, applied as a loop of single calls in list order would:
 * entry k is operation ops[k] (or `op` for all when ops is NULL) at
 * cells[k] with value values[k] (or `value` when values is NULL). */
int hal_cuda_pdegrid_apply(hal_cuda_pdegrid *h, const int32_t *ops, int32_t op, const int32_t *cells,
                           const double *values, double value, int64_t n);

/* One operation per agent of the agent handle's last binning (dispatch,
 * step, accumulate_forces or sum_forces), at the agent's cell, the agents of
 * a cell in index order: e.g. MUL with value -uptake is each agent's
 * PDEGrid2D::Mul(Isq(), -uptake) (examples/CompetitiveRelease.cpp:147).
 * perAgent (n doubles by agent index, may be NULL) replaces value.  The grid
 * must have the agents' size.  Ordered after the agents' last work on their
 * stream, and their next work after this. */
int hal_cuda_pdegrid_apply_agents(hal_cuda_pdegrid *h, hal_cuda_agents *agents, int32_t op,
                                  double value, const double *perAgent);

/* SetAll / AddAll / MulAll (PDEGrid2D.h:188-217): the operation at every
 * cell; perCell (xDim*yDim, may be NULL) replaces value (SetAll(pVals)).
 * The value form (perCell NULL) is recorded and runs at the start of the next
 * call on the handle, or, when that call is hal_cuda_pdegrid_update, inside
 * its pass; results are the same as running it at once, and a launch failure
 * is reported by that next call. */
int hal_cuda_pdegrid_apply_all(hal_cuda_pdegrid *h, int32_t op, double value, const double *perCell);

/* Update (PDEGrid2D.h:178-186) and SetNonNegative (:244-255). */
int hal_cuda_pdegrid_update(hal_cuda_pdegrid *h);
int hal_cuda_pdegrid_set_non_negative(hal_cuda_pdegrid *h);

/* Get(i) of n cells of the committed field. */
int hal_cuda_pdegrid_get_cells(hal_cuda_pdegrid *h, const int32_t *cells, int64_t n, double *out);

/* GradientX / GradientY (PDEGrid2D.h:257-285) at n points (xs[k], ys[k]):
 * off-grid neighbours read the cell's own value (reflecting) or, with
 * useBoundary, boundaryValue; a wrapped axis wraps. */
int hal_cuda_pdegrid_gradient(hal_cuda_pdegrid *h, const int32_t *xs, const int32_t *ys, int64_t n,
                              int32_t useBoundary, double boundaryValue, double *gradX, double *gradY);

/* stats[0..4] = GetMax, GetMin, GetAvg, MaxDelta and MaxDeltaScaled(
 * denomOffset) (PDEGrid2D.h:142-241); a NaN denomOffset skips the last
 * (stats[4] = NaN).  GetMax / GetMin keep the reference's choice among equal
 * values (+0 and -0): the last in cell order. */
int hal_cuda_pdegrid_stats(hal_cuda_pdegrid *h, double denomOffset, double *stats);

/* The PDE operators, accumulating into the deltas (PDEGrid2D.h:289-400):
 * Diffusion(diffCoef[, bc]) (EINVAL above 0.25), Diffusion(ratesX, ratesY),
 * DiffusionADI(diffRate[, bc]), Advection(xVel, yVel[, bc]) (EINVAL when
 * |xVel| + |yVel| > 0.5), Advection(xVels, yVels[, bc, xVelBC, yVelBC]).
 * Boundary callables are ghost tables (file header), NULL for none; per-cell
 * arrays hold xDim*yDim doubles. */
int hal_cuda_pdegrid_diffusion(hal_cuda_pdegrid *h, double diffCoef, const double *ghost);
int hal_cuda_pdegrid_diffusion_var(hal_cuda_pdegrid *h, const double *ratesX, const double *ratesY);
int hal_cuda_pdegrid_diffusion_adi(hal_cuda_pdegrid *h, double diffRate, const double *ghost);
int hal_cuda_pdegrid_advection(hal_cuda_pdegrid *h, double xVel, double yVel, const double *ghost);
int hal_cuda_pdegrid_advection_var(hal_cuda_pdegrid *h, const double *xVels, const double *yVels,
                                   const double *ghost, const double *ghostXVel,
                                   const double *ghostYVel);

int hal_cuda_pdegrid_sync(hal_cuda_pdegrid *h);
void *hal_cuda_pdegrid_stream(hal_cuda_pdegrid *h);
int hal_cuda_pdegrid_set_stream(hal_cuda_pdegrid *h, void *stream);

/* ---- on-disk format: SavePDEGrid2D / LoadPDEGrid2D ------------------------
 * (src/Grids/PDEGridSerialization.cpp:34-62, through BinaryWriter /
 * BinaryReader): raw native-endian int32 xDim, int32 yDim, one byte each for
 * wrapX and wrapY, int32 updateCt, then xDim*yDim doubles of field and as
 * many of pending deltas, in HAL's layout.  Files are byte-identical to the
 * reference's.  Reads fail with EINVAL on a short read or invalid
 * dimensions (Internal::CheckLoadedDims, src/Grids/GridSerialization.cpp:
 * 14-32).  The write / read calls are host-only and need no GPU. */
int hal_cuda_pdegrid2d_write(const char *path, int32_t xDim, int32_t yDim, int32_t wrapX,
                             int32_t wrapY, int32_t updateCt, const double *field,
                             const double *deltas); /* deltas NULL: zeros */
int hal_cuda_pdegrid2d_read_header(const char *path, int32_t *xDim, int32_t *yDim, int32_t *wrapX,
                                   int32_t *wrapY, int32_t *updateCt);
/* EINVAL unless the file's grid is xDim x yDim; deltas may be NULL. */
int hal_cuda_pdegrid2d_read(const char *path, int32_t xDim, int32_t yDim, double *field,
                            double *deltas);

/* Checkpoint / resume of a resident field.  A resident tick commits its own
 * deltas, so save writes zero deltas; the wrap flags and the update count
 * (PDEGrid2D::UpdateCt) are the caller's.  load needs the handle's grid size
 * and returns ENOTSUP for a file with pending deltas; wrapX, wrapY and
 * updateCt may be NULL. */
int hal_cuda_diffusion_save(hal_cuda_diffusion *h, const char *path, int32_t wrapX, int32_t wrapY,
                            int32_t updateCt);
int hal_cuda_diffusion_load(hal_cuda_diffusion *h, const char *path, int32_t *wrapX, int32_t *wrapY,
                            int32_t *updateCt);
int hal_cuda_adi_save(hal_cuda_adi *h, const char *path, int32_t wrapX, int32_t wrapY,
                      int32_t updateCt);
int hal_cuda_adi_load(hal_cuda_adi *h, const char *path, int32_t *wrapX, int32_t *wrapY,
                      int32_t *updateCt);

/* ---- batched wells: many independent simulations per launch -------------
 * MultiWellExperiment::Step / StepMultiThread
 * (include/Hal/Tools/MultiWellExperiment.h:83-103) advance independent wells
 * one after another, or on host threads through Hal::MultiThread
 * (include/Hal/Concurrency/MultiThread.h:19-91).  Here every well's tick runs
 * in the same few launches:
 *   - one launch over the tiles of every explicit well (the fused tick of
 *     hal_cuda_diffusion_run_ticks);
 *   - two launches (x- and y-sweep) over the line groups of every ADI well
 *     (the tick of hal_cuda_adi_run_ticks);
 *   - one agent force pass over the concatenated agents and cells of every
 *     well that has agents (hal_cuda_agents_dispatch's kernels).
 * A tick is replayed from a CUDA graph.  Each well's field, and its agents'
 * velocity deltas, are bit-identical to running that well alone on the
 * single-grid handles. */
#define HAL_CUDA_WELL_EXPLICIT 0
#define HAL_CUDA_WELL_ADI 1
#define HAL_CUDA_WELLS_MAX_SIDE 4096

typedef struct hal_cuda_well_desc
{
    int32_t xDim, yDim;  /* grid of the well, each in [1, HAL_CUDA_WELLS_MAX_SIDE] */
    int32_t kind;        /* HAL_CUDA_WELL_EXPLICIT or HAL_CUDA_WELL_ADI */
    int32_t wrapX, wrapY;
    int32_t maxAgents;   /* capacity of the well's agent set, 0 for none */
    double diffRate;     /* D*dt/dx^2; at most 0.25 for an explicit well */
    double decay;        /* per-tick decay: f' = ... - decay*f */
} hal_cuda_well_desc;

typedef struct hal_cuda_wells hal_cuda_wells;

int hal_cuda_wells_create(const hal_cuda_well_desc *wells, int32_t nWells, hal_cuda_wells **out);
int hal_cuda_wells_destroy(hal_cuda_wells *h);

/* Field (HAL layout x*yDim + y, len = xDim*yDim floats) and constant dense
 * source (NULL clears it) of one well. */
int hal_cuda_wells_set_field(hal_cuda_wells *h, int32_t well, const float *field, int64_t len);
int hal_cuda_wells_get_field(hal_cuda_wells *h, int32_t well, float *field, int64_t len);
int hal_cuda_wells_set_source(hal_cuda_wells *h, int32_t well, const float *dense, int64_t len);

/* Agents of every well at once: counts[w] <= maxAgents of well w; positions
 * (x, y interleaved, the well's own coordinates) and radii concatenated in
 * well order (2*sum and sum floats). */
int hal_cuda_wells_set_agents(hal_cuda_wells *h, const int32_t *counts, const float *positions,
                              const float *radii);

/* `ticks` ticks of every well: its field tick, then its agents' force pass
 * (interactionRad, springConstant).  Asynchronous on the handle's stream. */
int hal_cuda_wells_run_ticks(hal_cuda_wells *h, int32_t ticks, double interactionRad,
                             double springConstant);

/* Motion of the wells' agents: when enabled, each tick's force pass also
 * applies SphericalAgent2D's update to every agent, in its own well, as
 * hal_cuda_agents_step does (vel += delta; CapVelocity(maxVel) when maxVel >=
 * 0; ForceMove with the well's wrap flags; ApplyFriction(friction)), so the
 * agents move on the device tick after tick.  set_agents sets the velocities
 * to zero; set_velocities (NULL: zero) and get_agents take 2*sum(counts)
 * values, well after well. */
int hal_cuda_wells_set_motion(hal_cuda_wells *h, int32_t enabled, double friction, double maxVel);
int hal_cuda_wells_set_velocities(hal_cuda_wells *h, const float *velocities, int64_t len);
int hal_cuda_wells_get_agents(hal_cuda_wells *h, float *positions, float *velocities, int64_t len);

/* Velocity deltas of the last force pass, every well's agents concatenated
 * in well order (len = 2*sum(counts) floats). */
int hal_cuda_wells_get_forces(hal_cuda_wells *h, float *velocityDeltas, int64_t len);

/* Autotuner of the ADI sweep tiles: times the batched x- and y-sweeps of
 * every ADI well with the lines per tile capped at 128, 64, 32, 16 and 8, on
 * the wells' own fields (their state does not change), and keeps the
 * fastest cap.  Runs by itself before the first run_ticks or profile;
 * calling it again re-tunes.  Returns the chosen cap and the mean ms of one
 * x- plus y-sweep launch with it and with the uncapped default (any pointer
 * may be NULL; both times are 0 without ADI wells).  The block size of the
 * agent force kernel (64, 128 or 256 threads) is tuned the same way, on the
 * wells' agents, at the first run_ticks or profile after set_agents and for
 * each new interaction radius and spring constant. */
int hal_cuda_wells_autotune(hal_cuda_wells *h, int32_t *rCap, float *msTuned, float *msDefault);
int hal_cuda_wells_sync(hal_cuda_wells *h);
void *hal_cuda_wells_stream(hal_cuda_wells *h);
int hal_cuda_wells_set_stream(hal_cuda_wells *h, void *stream);

/* ---- variable-rate ADI and its gradient ------------------------------------
 * No reference implementation exists (the reference has no variable-rate ADI
 * and no gradient code).  The step follows HAL's variable-rate explicit
 * stencil Internal::Diffusion2(..., pDiffRatesX, pDiffRatesY, ...)
 * (src/Pde/PDEequations.cpp:199-230): the face between cells j and j+1 of a
 * line carries cell j's rate D (D*dt/dx^2, one per cell, both axes):
 *   w = (I - Lx/2)^-1 (I + Ly/2) f;  v = (I - Ly/2)^-1 (I + Lx/2) w;
 *   f' = f + (((v - f) + f*(-decay)) + src)
 * which for a constant D is hal_cuda_adi_run_ticks' tick.  The gradient of
 * loss = 1/2 |f_T - target|^2 with respect to D, decay and src comes from
 * adjoint kernels (transposed stencils and transposed line solves in reverse
 * sweep order) over states recomputed from checkpoints.  Sides up to
 * HAL_CUDA_ADJOINT_MAX_SIDE, wrapped or zero-flux at any length (a wrapped
 * line that is not a power of two long is solved with a Sherman-Morrison
 * split, as TdmaSolver::TDMAperiodic does). */
#define HAL_CUDA_ADJOINT_MAX_SIDE 1024

typedef struct hal_cuda_adjoint hal_cuda_adjoint;

int hal_cuda_adjoint_create(int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY,
                            hal_cuda_adjoint **out);
int hal_cuda_adjoint_destroy(hal_cuda_adjoint *h);

/* Initial field f0 and target final field (len = xDim*yDim floats each), the
 * number of steps, and the checkpoint interval: a field is kept every
 * checkpointEvery steps and the states in between are recomputed during the
 * gradient; 0 keeps every state of the run (3 fields per step of device
 * memory) and recomputes nothing. */
int hal_cuda_adjoint_set_problem(hal_cuda_adjoint *h, const float *f0, const float *target,
                                 int64_t len, int32_t steps, int32_t checkpointEvery);

/* loss (and f_T when fT is not NULL) for the rate field D (xDim*yDim), decay
 * and source field (NULL: none). */
int hal_cuda_adjoint_forward(hal_cuda_adjoint *h, const float *D, double decay, const float *src,
                             double *loss, float *fT);

/* loss and its gradients: gradD, gradSrc (xDim*yDim each, may be NULL) and
 * gradDecay (may be NULL). */
int hal_cuda_adjoint_gradient(hal_cuda_adjoint *h, const float *D, double decay, const float *src,
                              double *loss, float *gradD, double *gradDecay, float *gradSrc);

/* Device time (ms, CUDA events) of the last forward and gradient calls,
 * from the first kernel to the last. */
int hal_cuda_adjoint_times(hal_cuda_adjoint *h, float *msForward, float *msGradient);

/* ---- agent forces without allocation --------------------------------------
 * No counterpart in the reference: the reference's backends allocate their
 * buffers.  This entry point is for callers that cannot call cudaMalloc -- a
 * host framework that owns all device memory in its own pool and forbids
 * cudaMalloc/cudaFree in its step loop (they synchronise the whole device), or
 * a plugin whose host hands it only pointers to inputs and outputs.  It runs
 * the same kernels as hal_cuda_agents_dispatch (FP32 positions, radii and
 * velocity deltas; same bins, same summation order) and allocates nothing: no
 * handle, no cudaMalloc/cudaFree, no allocating library call.  Its scratch is
 * one static device array of HAL_CUDA_NOALLOC_SCRATCH_BYTES that every GPU
 * loading this library holds until the process exits.
 *
 * positions (2n floats, x,y interleaved), radii (n) and velocityDeltas (2n) are
 * device memory of the current device; stream is a cudaStream_t of that device
 * (NULL: the legacy default stream).  The call only enqueues work: synchronise
 * the stream before reading velocityDeltas.  n above HAL_CUDA_NOALLOC_MAX_AGENTS
 * or xDim*yDim above HAL_CUDA_NOALLOC_MAX_CELLS returns HAL_CUDA_EINVAL.
 *
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call
 * before any stream capture.  The address is kept with the id of the CUDA
 * context it was looked up in, and looked up again by the first call after the
 * context changed (a cudaDeviceReset in between), which again must not be made
 * during a stream capture.  Every call on a device shares the one array and
 * it keeps the last call's contents: calls that overlap on the GPU (different
 * streams, or host threads racing on one device) race on it and give wrong
 * results.  Calls ordered on one stream are safe. */
#define HAL_CUDA_NOALLOC_MAX_AGENTS 65536
#define HAL_CUDA_NOALLOC_MAX_CELLS 65536
#define HAL_CUDA_NOALLOC_SCRATCH_BYTES (3u << 20)

int hal_cuda_agents_forces_noalloc(const float *positions, const float *radii, int32_t n,
                                   float *velocityDeltas, double interactionRad, double springConstant,
                                   int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY, void *stream);

#ifdef __cplusplus
}
#endif

#endif
