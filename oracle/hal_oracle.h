/*
 * hal_oracle.h -- CPU oracle for the HAL-CPP per-tick hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * CPU backends (explicit stencil, ADI/Thomas, cell-bucket agent forces and the
 * PDEGrid2D tick semantics).  It exists to check the CUDA path: only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark may load
 * it, never the product path.
 *
 * Every function follows the reference file:line named beside it, operation
 * for operation (same loop order, same floating-point expression order), so
 * that with -ffp-contract=off it reproduces the reference's FP64 results bit
 * for bit.  Parity is pinned by tests/test_oracle_pin.py against golden
 * vectors generated from the reference's own CPU code (tests/golden/).
 *
 * Layout everywhere: row-major i = x*yDim + y (y contiguous), as in
 * Hal::PDEGrid2D.
 *
 * Dirichlet "ghost" arrays: a boundary callable bc(x, y) of the reference is
 * only ever evaluated one cell outside the grid, so it is passed as a table
 * of 2*yDim + 2*xDim values:
 *   ghost[y]                    = bc(-1,   y)   (x below the grid)
 *   ghost[yDim + y]             = bc(xDim, y)   (x above the grid)
 *   ghost[2*yDim + x]           = bc(x, -1)     (y below the grid)
 *   ghost[2*yDim + xDim + x]    = bc(x, yDim)   (y above the grid)
 * A NULL ghost table means the zero-flux form of the stencil.
 */
#ifndef HAL_ORACLE_H
#define HAL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- explicit 5-point stencil -------------------------------------------- */

/* Internal::Diffusion2 (src/Pde/PDEequations.cpp:140-161) and, with a ghost
 * table, Internal::Diffusion2<BCFn> (include/Hal/Pde/PDEequations.h:264-287):
 * deltas[i] += diffRate * sum of the four neighbour differences. */
void oracle_diffusion2(const double *field, double *deltas, double diffRate,
                       int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                       const double *ghost);

/* Same stencil, rows [x0, x1) only (used by the multi-threaded baseline). */
void oracle_diffusion2_rows(const double *field, double *deltas, double diffRate,
                            int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                            const double *ghost, int32_t x0, int32_t x1);

/* ---- ADI -------------------------------------------------------------- */

/* Internal::Diffusion2DADI (include/Hal/Pde/ADIequations.h:306-337) and, with
 * a ghost table, its Dirichlet form (:339-378).  scratch holds xDim*yDim
 * doubles.  deltas[i] += v - field[i]. */
void oracle_adi2(const double *field, double *scratch, double *deltas,
                 double diffRate, int32_t xDim, int32_t yDim, int wrapX,
                 int wrapY, const double *ghost);

/* Multi-threaded form of oracle_adi2 (lines split over nthreads POSIX
 * threads; each line is solved exactly as in oracle_adi2, so the result is
 * identical).  Used only as the CPU baseline. */
void oracle_adi2_mt(const double *field, double *scratch, double *deltas,
                    double diffRate, int32_t xDim, int32_t yDim, int wrapX,
                    int wrapY, const double *ghost, int nthreads);

/* ---- PDEGrid2D tick (include/Hal/Grids/PDEGrid2D.h) --------------------- */

/* One model tick as a HAL model writes it:
 *   Diffusion(diffRate[, bc]) or DiffusionADI(diffRate[, bc])  (:289-347)
 *   MulAll(-decay)                                             (:212-218)
 *   Add(i, srcDense[i]) for every cell (if srcDense)           (:110-114)
 *   Add(srcIdx[k], srcVal[k]) for k < nSrc                     (:110-114)
 *   Mul(cell, -uptake) once per agent in the cell (uptakeCount)(:126-130)
 *   Update()                                                   (:178-186)
 * field is updated in place; deltas (xDim*yDim, zeroed on entry and on exit)
 * and scratch (ADI only) are work arrays.  mode 0 = explicit, 1 = ADI.
 * Returns 0, or -1 for an explicit rate above 0.25 (CheckDiffusionStable,
 * :436-442). */
int oracle_tick(int mode, double *field, double *deltas, double *scratch,
                int32_t xDim, int32_t yDim, double diffRate, int wrapX,
                int wrapY, const double *ghost, double decay,
                const double *srcDense, int32_t nSrc, const int32_t *srcIdx,
                const double *srcVal, const int32_t *uptakeCount,
                double uptake, int nthreads);

/* The same tick with PDEGrid2D::Advection(xVel, yVel[, bc]) (PDEGrid2D.h:
 * 351-375) after the diffusion term: first-order upwind at a uniform
 * velocity, with the Dirichlet form when a ghost table is given.  Returns -2
 * when |xVel| + |yVel| > 0.5 (CheckAdvectionStable, :444-450). */
int oracle_tick_adv(int mode, double *field, double *deltas, double *scratch,
                    int32_t xDim, int32_t yDim, double diffRate, double xVel, double yVel,
                    int wrapX, int wrapY, const double *ghost, double decay,
                    const double *srcDense, int32_t nSrc, const int32_t *srcIdx,
                    const double *srcVal, const int32_t *uptakeCount,
                    double uptake, int nthreads);

/* ---- cell-bucket agent forces (src/Agents/CpuAgentForceBackend2D.cpp) ---- */

/* Passes 1-3 (:85-109): counts -> exclusive offsets (numCells+1 entries,
 * offsets[numCells] == n) and the stable scatter of agent indices. */
void oracle_agent_bins(const double *positions, int32_t n, int32_t xDim,
                       int32_t yDim, int32_t *cellOffsets, int32_t *bucketAgents);

/* Pass 4 (:111-175) for agents [i0, i1): velocityDeltas[2i], [2i+1]
 * overwritten with the summed linear-spring response. */
void oracle_agent_forces(const double *positions, const double *radii,
                         int32_t n, double interactionRad, double springConstant,
                         int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                         const int32_t *cellOffsets, const int32_t *bucketAgents,
                         double *velocityDeltas, int32_t i0, int32_t i1);

/* CpuAgentForceBackend2D::AccumulateForces (:66-176) end to end.  Scratch
 * cellOffsets (xDim*yDim+1) and bucketAgents (n) are caller-provided.  Pass 4
 * is split over nthreads threads (identical result).  Returns 0. */
int oracle_accumulate_forces(const double *positions, const double *radii,
                             int32_t n, double *velocityDeltas,
                             double interactionRad, double springConstant,
                             int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                             int32_t *cellOffsets, int32_t *bucketAgents,
                             int nthreads);

/* ---- variable-rate diffusion and upwind advection ------------------------ */

/* Internal::Diffusion2(pField, pDeltas, pDiffRatesX, pDiffRatesY, ...)
 * (src/Pde/PDEequations.cpp:199-230): the +x/+y face uses the cell's rate (0
 * past a non-wrapped edge), the -x/-y face the neighbour's. */
/* SphericalAgent2D::SumForces (include/Hal/Agents/SphericalAgent2D.h:74-102)
 * of every agent, in index order.  kind: 0 linear scale*touchDist, 1 clamped
 * (0 when touchDist < 0), 2 pow(scale*touchDist, exponent).  order 1 visits
 * each square's agents newest first with the grid's DispX/DispY, as an
 * AgentGrid2D filled in index order does; order 0 ascending with
 * AgentForceDisp, as CpuAgentForceBackend2D does.  velIn (may be NULL for
 * zeros) -> velOut, sums (may be NULL) = the returned sums of positive
 * forces. */
void oracle_sum_forces(const double *positions, const double *radii, int32_t n,
                       const double *velIn, double *velOut, double *sums,
                       double interactionRad, int kind, double scale, double exponent,
                       int order, int32_t xDim, int32_t yDim, int wrapX, int wrapY);

/* A script of Hal::PDEGrid2D calls (include/Hal/Grids/PDEGrid2D.h) run on
 * field/deltas/updateCt in place.  Op k has iargs[3k..3k+2] = (offset of
 * its arrays in `arrays`, i or x, y) and dargs[2k..2k+1]:
 *   0-3 Set/Add/Mul/Scale(i, d0);  10-12 SetAll/AddAll/MulAll(d0);
 *   13 SetAll(arrays);  20 Diffusion(d0);  21 Diffusion(d0, ghost table);
 *   22 Diffusion(ratesX, ratesY);  30 DiffusionADI(d0);  31 DiffusionADI(d0,
 *   ghost);  40 Advection(d0, d1);  41 Advection(d0, d1, ghost);
 *   42 Advection(xVels, yVels);  43 the same with field, x- and y-velocity
 *   ghost tables;  50 Update();  51 SetNonNegative();  records: 60 Get(i),
 *   61 GetMax, 62 GetMin, 63 GetAvg, 64 MaxDelta, 65 MaxDeltaScaled(d0),
 *   66/67 GradientX/Y(x, y), 68/69 the same with boundary value d0.
 * Returns the number of records, -1 / -2 for a rejected diffusion /
 * advection rate. */
int oracle_pdegrid_script(int32_t xDim, int32_t yDim, int wrapX, int wrapY, double *field, double *deltas,
                          int32_t *updateCt, int32_t nOps, const int32_t *ops, const int32_t *iargs,
                          const double *dargs, const double *arrays, double *records);

void oracle_diffusion2_var(const double *field, double *deltas, const double *ratesX, const double *ratesY,
                           int32_t xDim, int32_t yDim, int wrapX, int wrapY);

/* Internal::Advection2 with a uniform velocity (src/Pde/PDEequations.cpp:
 * 380-412): first-order upwind. */
void oracle_advection2(const double *field, double *deltas, double xVel, double yVel, int32_t xDim, int32_t yDim,
                       int wrapX, int wrapY);

/* Internal::Advection2 with a per-cell velocity field
 * (src/Pde/PDEequations.cpp:535-575): upwind face fluxes. */
void oracle_advection2_var(const double *field, double *deltas, const double *xVels, const double *yVels,
                           int32_t xDim, int32_t yDim, int wrapX, int wrapY);

/* Dirichlet forms: Internal::Advection2<BCFn> (include/Hal/Pde/
 * PDEequations.h:413-447; an off-grid upwind neighbour gives
 * (bc - centre) * 2) and Advection2<BCFn, XVelBCFn, YVelBCFn> (:720-778; the
 * off-grid field and velocities are the boundary values themselves).  Each
 * callable is a ghost table in the layout above; NULL reads as 0. */
void oracle_advection2_bc(const double *field, double *deltas, double xVel, double yVel, int32_t xDim,
                          int32_t yDim, int wrapX, int wrapY, const double *ghost);
void oracle_advection2_var_bc(const double *field, double *deltas, const double *xVels, const double *yVels,
                              int32_t xDim, int32_t yDim, int wrapX, int wrapY, const double *ghost,
                              const double *ghostXVel, const double *ghostYVel);

/* ---- variable-rate ADI and its adjoint -----------------------------------
 * No reference implementation exists: the step is defined from HAL's
 * variable-rate explicit stencil (src/Pde/PDEequations.cpp:199-230; the face
 * between cells j and j+1 has cell j's rate) as
 *   w = (I - Lx/2)^-1 (I + Ly/2) f,  v = (I - Ly/2)^-1 (I + Lx/2) w,
 *   f' = f + (((v - f) + f*(-decay)) + src),
 * equal to Diffusion2DADI plus the PDEGrid2D tick for a constant rate.  D
 * holds one rate (D*dt/dx^2) per cell for both axes. */

/* One step; w (xDim*yDim) receives the x-sweep result, out the new field. */
void oracle_dadi_step(const double *f, const double *D, int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                      double decay, const double *src, double *w, double *out);

/* `steps` steps from f0; returns loss = 1/2 |f_T - target|^2 and, when the
 * pointers are not NULL, f_T and the gradients of the loss with respect to D
 * (per cell), decay and src (per cell), by reverse-mode differentiation of
 * the steps (every state kept, FP64). */
double oracle_dadi_loss_grad(const double *f0, const double *target, const double *D, double decay,
                             const double *src, int32_t xDim, int32_t yDim, int wrapX, int wrapY, int32_t steps,
                             double *fT, double *gD, double *gDecay, double *gSrc);

/* ---- agent integration step --------------------------------------------------
 * SphericalAgent2D's update after its forces (include/Hal/Agents/
 * SphericalAgent2D.h:133-162), per agent i with velocity delta d_i:
 *   vel += d;  CapVelocity(maxVel) when maxVel >= 0;
 *   ForceMove = MoveSafePT(pos + vel) (include/Hal/Agents/AgentPT2D.h:157-186):
 *     a point on the grid (GridGeometry2D::In, src/Grids/GridGeometry2D.cpp:
 *     120-124) is taken; otherwise a wrapped axis wraps (Wrap,
 *     src/MathUtil.cpp:48-53) and a closed axis whose coordinate left
 *     [0, dim) keeps the old one;
 *   ApplyFriction(friction): vel *= friction.
 * pos and vel (2n interleaved values) are updated in place.  The double form
 * is the reference's arithmetic; the float form is the same steps in FP32,
 * the precision of the resident device step. */
void oracle_agents_move(double *pos, double *vel, const double *deltas, int32_t n, int32_t xDim, int32_t yDim,
                        int wrapX, int wrapY, double friction, double maxVel);
void oracle_agents_move_f32(float *pos, float *vel, const float *deltas, int32_t n, int32_t xDim, int32_t yDim,
                            int wrapX, int wrapY, float friction, float maxVel);

/* ---- Hal::Rng / Hal::Rand (src/Rng.cpp, src/Rand.cpp) ----------------------
 * xoshiro256** seeded through splitmix64, plus the Marsaglia polar Gaussian
 * (src/GaussianSampler.cpp:23-47).  Used to rebuild the seeded scenes of the
 * reference's own tests. */
typedef struct oracle_rand
{
    uint64_t s[4];
    double v1, v2, sq;
    int phase;
} oracle_rand;

void oracle_rand_init(oracle_rand *r, uint64_t seed);
uint64_t oracle_rand_next(oracle_rand *r);
double oracle_rand_double(oracle_rand *r);
int32_t oracle_rand_int(oracle_rand *r, int32_t bound);
double oracle_rand_gaussian(oracle_rand *r, double mean, double stdDev);

#ifdef __cplusplus
}
#endif

#endif
