/*
 * hal_oracle.c -- CPU oracle for the HAL-CPP hot path (TEST INFRASTRUCTURE).
 *
 * A plain-C restatement of the reference CPU backends.  Each function keeps
 * the reference's loop order and floating-point expression order so that,
 * compiled with -ffp-contract=off, the FP64 results are bit-identical to the
 * reference's own CPU code (pinned against golden vectors made from it).
 * Nothing in the product path may call this file.
 */
#include "hal_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* MathUtil.cpp:41-46 (Wrap) and :381-385 (InDim). */
static int32_t o_wrap(int32_t val, int32_t max)
{
    int32_t mod = val % max;
    return (mod < 0) ? (max + mod) : mod;
}

static int o_in_dim(int32_t val, int32_t dim)
{
    return (val >= 0) && (val < dim);
}

/* Ghost lookups for a Dirichlet callable evaluated just outside the grid. */
static double o_ghost_x(const double *ghost, int32_t x, int32_t y, int32_t yDim)
{
    return (x < 0) ? ghost[y] : ghost[yDim + y];
}

static double o_ghost_y(const double *ghost, int32_t x, int32_t y, int32_t xDim,
                        int32_t yDim)
{
    return (y < 0) ? ghost[2 * yDim + x] : ghost[2 * yDim + xDim + x];
}

/* DeltaX2D (src/Pde/PDEequations.cpp:24-41) and its Dirichlet form
 * (include/Hal/Pde/PDEequations.h:50-69). */
static double o_delta_x(const double *f, double c, int32_t x, int32_t y,
                        int32_t xDim, int32_t yDim, int wrapX, const double *ghost)
{
    if (o_in_dim(x, xDim))
    {
        return f[x * yDim + y] - c;
    }
    if (wrapX)
    {
        return f[o_wrap(x, xDim) * yDim + y] - c;
    }
    if (ghost != NULL)
    {
        return (o_ghost_x(ghost, x, y, yDim) - c) * 2;
    }
    return 0;
}

/* DeltaY2D (src/Pde/PDEequations.cpp:43-60) and its Dirichlet form
 * (include/Hal/Pde/PDEequations.h:79-98). */
static double o_delta_y(const double *f, double c, int32_t x, int32_t y,
                        int32_t xDim, int32_t yDim, int wrapY, const double *ghost)
{
    if (o_in_dim(y, yDim))
    {
        return f[x * yDim + y] - c;
    }
    if (wrapY)
    {
        return f[x * yDim + o_wrap(y, yDim)] - c;
    }
    if (ghost != NULL)
    {
        return (o_ghost_y(ghost, x, y, xDim, yDim) - c) * 2;
    }
    return 0;
}

void oracle_diffusion2_rows(const double *field, double *deltas, double diffRate,
                            int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                            const double *ghost, int32_t x0, int32_t x1)
{
    /* src/Pde/PDEequations.cpp:148-160 */
    for (int32_t x = x0; x < x1; x++)
    {
        for (int32_t y = 0; y < yDim; y++)
        {
            int32_t i = x * yDim + y;
            double centerVal = field[i];
            double deltaSum = o_delta_x(field, centerVal, x + 1, y, xDim, yDim, wrapX, ghost);
            deltaSum += o_delta_x(field, centerVal, x - 1, y, xDim, yDim, wrapX, ghost);
            deltaSum += o_delta_y(field, centerVal, x, y + 1, xDim, yDim, wrapY, ghost);
            deltaSum += o_delta_y(field, centerVal, x, y - 1, xDim, yDim, wrapY, ghost);
            deltas[i] += deltaSum * diffRate;
        }
    }
}

void oracle_diffusion2(const double *field, double *deltas, double diffRate,
                       int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                       const double *ghost)
{
    oracle_diffusion2_rows(field, deltas, diffRate, xDim, yDim, wrapX, wrapY, ghost, 0, xDim);
}

/* ---- Thomas solver: include/Hal/Pde/TdmaSolver.h ------------------------ */

typedef struct o_tdma
{
    double *as, *bs, *cs, *ws, *ds, *ys, *zs, *us;
    int32_t len;
} o_tdma;

static int o_tdma_init(o_tdma *t, int32_t len)
{
    double *block = (double *)calloc((size_t)len * 8 + 8, sizeof(double));
    if (block == NULL)
    {
        return -1;
    }
    t->as = block;
    t->bs = t->as + len + 1;
    t->cs = t->bs + len + 1;
    t->ws = t->cs + len + 1;
    t->ds = t->ws + len + 1;
    t->ys = t->ds + len + 1;
    t->zs = t->ys + len + 1;
    t->us = t->zs + len + 1;
    t->len = len;
    return 0;
}

static void o_tdma_free(o_tdma *t)
{
    free(t->as);
}

/* The coefficient callables of ADISolveRow (ADIequations.h:225-270) and the
 * adjusted diagonal of TDMAperiodic (TdmaSolver.h:84-95), as data. */
typedef struct o_coeffs
{
    double offDiagonal;
    double endAdjust;
    int periodic;     /* diagonal is 1 - 2*offDiagonal everywhere */
    int adjusted;     /* apply the Sherman-Morrison end adjustment */
    double gamma, alpha, beta;
    int32_t len;
} o_coeffs;

static double o_get_b_raw(const o_coeffs *k, int32_t i)
{
    if (k->periodic)
    {
        return 1 - 2 * k->offDiagonal;
    }
    double weight = 2.0;
    if (i == 0)
    {
        weight += k->endAdjust;
    }
    if (i == (k->len - 1))
    {
        weight += k->endAdjust;
    }
    return 1 - weight * k->offDiagonal;
}

static double o_get_b(const o_coeffs *k, int32_t i)
{
    if (k->adjusted)
    {
        if (i == 0)
        {
            return o_get_b_raw(k, i) - k->gamma;
        }
        if (i == (k->len - 1))
        {
            return o_get_b_raw(k, i) - (k->alpha * k->beta) / k->gamma;
        }
    }
    return o_get_b_raw(k, i);
}

/* TdmaSolver::TDMA (TdmaSolver.h:26-66).  rhs[i] plays getIn(i); the solution
 * goes to out[i] in the order setOut is called (last to first). */
static void o_tdma_solve(o_tdma *t, const o_coeffs *k, int32_t n, const double *rhs,
                         double *out)
{
    double *as = t->as, *bs = t->bs, *cs = t->cs, *ws = t->ws, *ds = t->ds;
    bs[0] = o_get_b(k, 0);
    cs[0] = k->offDiagonal;
    ds[0] = rhs[0];
    for (int32_t i = 1; i < n; i++)
    {
        if (i < (n - 1))
        {
            cs[i] = k->offDiagonal;
        }
        bs[i] = o_get_b(k, i);
        as[i] = k->offDiagonal;
        ds[i] = rhs[i];
        ws[i] = as[i] / bs[i - 1];
        bs[i] = bs[i] - ws[i] * cs[i - 1];
        ds[i] = ds[i] - ws[i] * ds[i - 1];
    }
    int32_t i = n - 1;
    double x = ds[i] / bs[i];
    out[i] = x;
    for (i -= 1; i >= 0; i--)
    {
        x = (ds[i] - cs[i] * x) / bs[i];
        out[i] = x;
    }
}

/* ADISolveRow (ADIequations.h:225-270) with TDMA / TDMAperiodic
 * (TdmaSolver.h:26-120).  rhs holds getIn(0..len-1); out receives setOut's
 * values. */
static void o_adi_solve_row(o_tdma *t, int32_t len, double diffRate, int wrapDim,
                            int hasBC, const double *rhs, double *out)
{
    o_coeffs k;
    memset(&k, 0, sizeof(k));
    k.offDiagonal = -diffRate / 2.0;
    k.len = len;
    if (wrapDim)
    {
        k.periodic = 1;
        /* TdmaSolver.h:80-82 */
        const double gamma = -o_get_b(&k, 0);
        const double alpha = k.offDiagonal;
        const double beta = k.offDiagonal;
        k.gamma = gamma;
        k.alpha = alpha;
        k.beta = beta;
        k.adjusted = 1;
        o_tdma_solve(t, &k, len, rhs, t->ys);
        /* second right-hand side (TdmaSolver.h:102-110) */
        for (int32_t i = 0; i < len; i++)
        {
            if (i == 0)
            {
                t->us[i] = gamma;
            }
            else if (i == (len - 1))
            {
                t->us[i] = alpha;
            }
            else
            {
                t->us[i] = 0.0;
            }
        }
        o_tdma_solve(t, &k, len, t->us, t->zs);
        double vEnd = beta / gamma;
        double vy = t->ys[0] + t->ys[len - 1] * vEnd;
        double vz = t->zs[0] + t->zs[len - 1] * vEnd;
        double factor = vy / (1 + vz);
        for (int32_t i = 0; i < len; i++)
        {
            out[i] = t->ys[i] - factor * t->zs[i];
        }
        return;
    }
    k.endAdjust = hasBC ? 1.0 : -1.0;
    o_tdma_solve(t, &k, len, rhs, out);
}

/* ExplicitDiffusionY2ADI (src/Pde/ADIequations.cpp:34-47, Dirichlet form
 * ADIequations.h:79-94). */
static double o_explicit_y2(int32_t x, int32_t y, const double *f, double diffRate,
                            int32_t xDim, int32_t yDim, int wrapY, const double *ghost)
{
    int32_t i = x * yDim + y;
    double centerVal = f[i];
    double deltaSum = o_delta_y(f, centerVal, x, y + 1, xDim, yDim, wrapY, ghost);
    deltaSum += o_delta_y(f, centerVal, x, y - 1, xDim, yDim, wrapY, ghost);
    return centerVal + (deltaSum * diffRate) / 2;
}

/* ExplicitDiffusionX2ADI (src/Pde/ADIequations.cpp:19-32, Dirichlet form
 * ADIequations.h:54-69). */
static double o_explicit_x2(int32_t x, int32_t y, const double *f, double diffRate,
                            int32_t xDim, int32_t yDim, int wrapX, const double *ghost)
{
    int32_t i = x * yDim + y;
    double centerVal = f[i];
    double deltaSum = o_delta_x(f, centerVal, x + 1, y, xDim, yDim, wrapX, ghost);
    deltaSum += o_delta_x(f, centerVal, x - 1, y, xDim, yDim, wrapX, ghost);
    return centerVal + (deltaSum * diffRate) / 2;
}

/* ImplicitBoundarySource (ADIequations.h:198-220) with diffScaleFactor 2. */
static double o_implicit_source(int32_t i, int32_t len, int wrap, double diffRate,
                                double lowVal, double highVal)
{
    if (wrap)
    {
        return 0.0;
    }
    double source = 0.0;
    if (i == 0)
    {
        source += lowVal;
    }
    if (i == (len - 1))
    {
        source += highVal;
    }
    return source * 2.0 * diffRate / 2.0;
}

/* x-sweep lines y in [y0, y1) (ADIequations.h:316-324 / :351-362). */
static void o_adi_xsweep(o_tdma *t, double *rhs, double *out, const double *field,
                         double *scratch, double diffRate, int32_t xDim, int32_t yDim,
                         int wrapX, int wrapY, const double *ghost, int32_t y0, int32_t y1)
{
    for (int32_t y = y0; y < y1; y++)
    {
        for (int32_t i = 0; i < xDim; i++)
        {
            if (ghost == NULL)
            {
                rhs[i] = o_explicit_y2(i, y, field, diffRate, xDim, yDim, wrapY, NULL);
            }
            else
            {
                rhs[i] = o_explicit_y2(i, y, field, diffRate, xDim, yDim, wrapY, ghost) +
                         o_implicit_source(i, xDim, wrapX, diffRate, ghost[y], ghost[yDim + y]);
            }
        }
        o_adi_solve_row(t, xDim, diffRate, wrapX, ghost != NULL, rhs, out);
        for (int32_t i = 0; i < xDim; i++)
        {
            scratch[i * yDim + y] = out[i];
        }
    }
}

/* y-sweep lines x in [x0, x1) (ADIequations.h:325-336 / :363-377). */
static void o_adi_ysweep(o_tdma *t, double *rhs, double *out, const double *field,
                         const double *scratch, double *deltas, double diffRate,
                         int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                         const double *ghost, int32_t x0, int32_t x1)
{
    for (int32_t x = x0; x < x1; x++)
    {
        for (int32_t i = 0; i < yDim; i++)
        {
            if (ghost == NULL)
            {
                rhs[i] = o_explicit_x2(x, i, scratch, diffRate, xDim, yDim, wrapX, NULL);
            }
            else
            {
                rhs[i] = o_explicit_x2(x, i, scratch, diffRate, xDim, yDim, wrapX, ghost) +
                         o_implicit_source(i, yDim, wrapY, diffRate, ghost[2 * yDim + x],
                                           ghost[2 * yDim + xDim + x]);
            }
        }
        o_adi_solve_row(t, yDim, diffRate, wrapY, ghost != NULL, rhs, out);
        for (int32_t i = 0; i < yDim; i++)
        {
            int32_t index = x * yDim + i;
            deltas[index] += out[i] - field[index];
        }
    }
}

void oracle_adi2(const double *field, double *scratch, double *deltas,
                 double diffRate, int32_t xDim, int32_t yDim, int wrapX,
                 int wrapY, const double *ghost)
{
    oracle_adi2_mt(field, scratch, deltas, diffRate, xDim, yDim, wrapX, wrapY, ghost, 1);
}

typedef struct o_adi_job
{
    const double *field;
    double *scratch, *deltas;
    double diffRate;
    int32_t xDim, yDim;
    int wrapX, wrapY;
    const double *ghost;
    int32_t lo, hi;
    int sweep; /* 0 = x-sweep, 1 = y-sweep */
} o_adi_job;

static void *o_adi_worker(void *arg)
{
    o_adi_job *j = (o_adi_job *)arg;
    int32_t len = (j->xDim > j->yDim) ? j->xDim : j->yDim;
    o_tdma t;
    if (o_tdma_init(&t, len) != 0)
    {
        return NULL;
    }
    double *rhs = (double *)calloc((size_t)len, sizeof(double));
    double *out = (double *)calloc((size_t)len, sizeof(double));
    if (j->sweep == 0)
    {
        o_adi_xsweep(&t, rhs, out, j->field, j->scratch, j->diffRate, j->xDim, j->yDim,
                     j->wrapX, j->wrapY, j->ghost, j->lo, j->hi);
    }
    else
    {
        o_adi_ysweep(&t, rhs, out, j->field, j->scratch, j->deltas, j->diffRate, j->xDim,
                     j->yDim, j->wrapX, j->wrapY, j->ghost, j->lo, j->hi);
    }
    free(rhs);
    free(out);
    o_tdma_free(&t);
    return NULL;
}

static void o_run_sweep(o_adi_job *base, int sweep, int32_t lines, int nthreads)
{
    if (nthreads < 1)
    {
        nthreads = 1;
    }
    if (nthreads > lines)
    {
        nthreads = lines;
    }
    if (nthreads <= 1)
    {
        o_adi_job j = *base;
        j.sweep = sweep;
        j.lo = 0;
        j.hi = lines;
        o_adi_worker(&j);
        return;
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    o_adi_job *jobs = (o_adi_job *)malloc(sizeof(o_adi_job) * (size_t)nthreads);
    for (int k = 0; k < nthreads; k++)
    {
        jobs[k] = *base;
        jobs[k].sweep = sweep;
        jobs[k].lo = (int32_t)(((int64_t)lines * k) / nthreads);
        jobs[k].hi = (int32_t)(((int64_t)lines * (k + 1)) / nthreads);
        pthread_create(&th[k], NULL, o_adi_worker, &jobs[k]);
    }
    for (int k = 0; k < nthreads; k++)
    {
        pthread_join(th[k], NULL);
    }
    free(th);
    free(jobs);
}

void oracle_adi2_mt(const double *field, double *scratch, double *deltas,
                    double diffRate, int32_t xDim, int32_t yDim, int wrapX,
                    int wrapY, const double *ghost, int nthreads)
{
    o_adi_job base;
    base.field = field;
    base.scratch = scratch;
    base.deltas = deltas;
    base.diffRate = diffRate;
    base.xDim = xDim;
    base.yDim = yDim;
    base.wrapX = wrapX;
    base.wrapY = wrapY;
    base.ghost = ghost;
    /* all x-sweep lines complete before any y-sweep line starts, as in the
     * two consecutive loops of Diffusion2DADI */
    o_run_sweep(&base, 0, yDim, nthreads);
    o_run_sweep(&base, 1, xDim, nthreads);
}

/* ---- explicit stencil, threaded rows (baseline only) --------------------- */

typedef struct o_rows_job
{
    const double *field;
    double *deltas;
    double diffRate;
    int32_t xDim, yDim;
    int wrapX, wrapY;
    const double *ghost;
    int32_t lo, hi;
} o_rows_job;

static void *o_rows_worker(void *arg)
{
    o_rows_job *j = (o_rows_job *)arg;
    oracle_diffusion2_rows(j->field, j->deltas, j->diffRate, j->xDim, j->yDim, j->wrapX,
                           j->wrapY, j->ghost, j->lo, j->hi);
    return NULL;
}

static void o_diffusion2_mt(const double *field, double *deltas, double diffRate,
                            int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                            const double *ghost, int nthreads)
{
    if (nthreads > xDim)
    {
        nthreads = xDim;
    }
    if (nthreads <= 1)
    {
        oracle_diffusion2(field, deltas, diffRate, xDim, yDim, wrapX, wrapY, ghost);
        return;
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    o_rows_job *jobs = (o_rows_job *)malloc(sizeof(o_rows_job) * (size_t)nthreads);
    for (int k = 0; k < nthreads; k++)
    {
        o_rows_job j = {field, deltas, diffRate, xDim, yDim, wrapX, wrapY, ghost,
                        (int32_t)(((int64_t)xDim * k) / nthreads),
                        (int32_t)(((int64_t)xDim * (k + 1)) / nthreads)};
        jobs[k] = j;
        pthread_create(&th[k], NULL, o_rows_worker, &jobs[k]);
    }
    for (int k = 0; k < nthreads; k++)
    {
        pthread_join(th[k], NULL);
    }
    free(th);
    free(jobs);
}

/* ---- PDEGrid2D tick -------------------------------------------------- */

int oracle_tick(int mode, double *field, double *deltas, double *scratch,
                int32_t xDim, int32_t yDim, double diffRate, int wrapX,
                int wrapY, const double *ghost, double decay,
                const double *srcDense, int32_t nSrc, const int32_t *srcIdx,
                const double *srcVal, const int32_t *uptakeCount,
                double uptake, int nthreads)
{
    return oracle_tick_adv(mode, field, deltas, scratch, xDim, yDim, diffRate, 0.0, 0.0, wrapX, wrapY, ghost,
                           decay, srcDense, nSrc, srcIdx, srcVal, uptakeCount, uptake, nthreads);
}

int oracle_tick_adv(int mode, double *field, double *deltas, double *scratch,
                    int32_t xDim, int32_t yDim, double diffRate, double xVel, double yVel,
                    int wrapX, int wrapY, const double *ghost, double decay,
                    const double *srcDense, int32_t nSrc, const int32_t *srcIdx,
                    const double *srcVal, const int32_t *uptakeCount,
                    double uptake, int nthreads)
{
    int32_t length = xDim * yDim;
    if (mode == 0)
    {
        /* PDEGrid2D::CheckDiffusionStable (PDEGrid2D.h:436-442) */
        if (diffRate > 0.25)
        {
            return -1;
        }
        o_diffusion2_mt(field, deltas, diffRate, xDim, yDim, wrapX, wrapY, ghost, nthreads);
    }
    else
    {
        oracle_adi2_mt(field, scratch, deltas, diffRate, xDim, yDim, wrapX, wrapY, ghost,
                       nthreads);
    }
    if (xVel != 0.0 || yVel != 0.0)
    {
        /* PDEGrid2D::Advection(xVel, yVel[, bc]) (PDEGrid2D.h:351-375), after
         * CheckAdvectionStable (:444-450) */
        if (fabs(xVel) + fabs(yVel) > 0.5)
        {
            return -2;
        }
        oracle_advection2_bc(field, deltas, xVel, yVel, xDim, yDim, wrapX, wrapY, ghost);
    }
    if (decay != 0.0)
    {
        /* MulAll(-decay) -> Mul(i, val): deltas[i] += field[i] * val (:126-130) */
        double val = -decay;
        for (int32_t i = 0; i < length; i++)
        {
            deltas[i] += field[i] * val;
        }
    }
    if (srcDense != NULL)
    {
        for (int32_t i = 0; i < length; i++)
        {
            deltas[i] += srcDense[i];
        }
    }
    for (int32_t k = 0; k < nSrc; k++)
    {
        deltas[srcIdx[k]] += srcVal[k];
    }
    if (uptakeCount != NULL)
    {
        double val = -uptake;
        for (int32_t i = 0; i < length; i++)
        {
            for (int32_t a = 0; a < uptakeCount[i]; a++)
            {
                deltas[i] += field[i] * val;
            }
        }
    }
    /* Update() (:178-186) */
    for (int32_t i = 0; i < length; i++)
    {
        field[i] += deltas[i];
    }
    memset(deltas, 0, sizeof(double) * (size_t)length);
    return 0;
}

/* ---- agents: src/Agents/CpuAgentForceBackend2D.cpp ------------------------ */

/* AgentForceCellCoord (:14-27) */
static int32_t o_cell_coord(double v, int32_t dim)
{
    int32_t c = (int32_t)floor(v);
    if (c < 0)
    {
        c = 0;
    }
    else if (c >= dim)
    {
        c = dim - 1;
    }
    return c;
}

/* AgentForceDisp (:30-45) */
static double o_disp(double a, double b, int32_t dim, int wrap)
{
    double d = b - a;
    if (wrap)
    {
        double dimF = (double)dim;
        if (fabs(d) > (dimF * 0.5))
        {
            d = (a > b) ? (d + dimF) : (d - dimF);
        }
    }
    return d;
}

/* AgentForceWrapIndex (:47-52) */
static int32_t o_wrap_index(int32_t v, int32_t dim)
{
    int32_t m = v % dim;
    return (m < 0) ? (m + dim) : m;
}

void oracle_agent_bins(const double *positions, int32_t n, int32_t xDim,
                       int32_t yDim, int32_t *cellOffsets, int32_t *bucketAgents)
{
    int32_t numCells = xDim * yDim;
    memset(cellOffsets, 0, sizeof(int32_t) * ((size_t)numCells + 1));
    for (int32_t i = 0; i < n; i++)
    {
        int32_t cellX = o_cell_coord(positions[(size_t)i * 2], xDim);
        int32_t cellY = o_cell_coord(positions[(size_t)i * 2 + 1], yDim);
        cellOffsets[(size_t)(cellX * yDim + cellY) + 1]++;
    }
    for (int32_t c = 0; c < numCells; c++)
    {
        cellOffsets[(size_t)c + 1] += cellOffsets[(size_t)c];
    }
    int32_t *cursors = (int32_t *)malloc(sizeof(int32_t) * ((size_t)numCells + 1));
    memcpy(cursors, cellOffsets, sizeof(int32_t) * (size_t)numCells);
    for (int32_t i = 0; i < n; i++)
    {
        int32_t cellX = o_cell_coord(positions[(size_t)i * 2], xDim);
        int32_t cellY = o_cell_coord(positions[(size_t)i * 2 + 1], yDim);
        int32_t cell = cellX * yDim + cellY;
        bucketAgents[cursors[cell]] = i;
        cursors[cell]++;
    }
    free(cursors);
}

void oracle_agent_forces(const double *positions, const double *radii,
                         int32_t n, double interactionRad, double springConstant,
                         int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                         const int32_t *cellOffsets, const int32_t *bucketAgents,
                         double *velocityDeltas, int32_t i0, int32_t i1)
{
    (void)n;
    for (int32_t i = i0; i < i1; i++)
    {
        double posX = positions[(size_t)i * 2];
        double posY = positions[(size_t)i * 2 + 1];
        double rad = radii[i];

        int32_t xStart = (int32_t)floor(posX - interactionRad);
        int32_t xEnd = (int32_t)ceil(posX + interactionRad);
        int32_t yStart = (int32_t)floor(posY - interactionRad);
        int32_t yEnd = (int32_t)ceil(posY + interactionRad);

        double velDeltaX = 0.0;
        double velDeltaY = 0.0;
        for (int32_t xSq = xStart; xSq < xEnd; xSq++)
        {
            int32_t retX = xSq;
            int inX = (retX >= 0) && (retX < xDim);
            if (!wrapX && !inX)
            {
                continue;
            }
            if (wrapX && !inX)
            {
                retX = o_wrap_index(retX, xDim);
            }
            for (int32_t ySq = yStart; ySq < yEnd; ySq++)
            {
                int32_t retY = ySq;
                int inY = (retY >= 0) && (retY < yDim);
                if (!wrapY && !inY)
                {
                    continue;
                }
                if (wrapY && !inY)
                {
                    retY = o_wrap_index(retY, yDim);
                }
                int32_t cell = retX * yDim + retY;
                int32_t start = cellOffsets[cell];
                int32_t end = cellOffsets[cell + 1];
                for (int32_t k = start; k < end; k++)
                {
                    int32_t j = bucketAgents[k];
                    if (j == i)
                    {
                        continue;
                    }
                    double xComp = o_disp(posX, positions[(size_t)j * 2], xDim, wrapX);
                    double yComp = o_disp(posY, positions[(size_t)j * 2 + 1], yDim, wrapY);
                    double dist = sqrt((xComp * xComp) + (yComp * yComp));
                    if ((dist < interactionRad) && (dist > 0.0))
                    {
                        double touchDist = (rad + radii[j]) - dist;
                        double force = springConstant * touchDist;
                        velDeltaX -= (xComp / dist) * force;
                        velDeltaY -= (yComp / dist) * force;
                    }
                }
            }
        }
        velocityDeltas[(size_t)i * 2] = velDeltaX;
        velocityDeltas[(size_t)i * 2 + 1] = velDeltaY;
    }
}

typedef struct o_force_job
{
    const double *positions, *radii;
    int32_t n;
    double R, k;
    int32_t xDim, yDim;
    int wrapX, wrapY;
    const int32_t *offsets, *bucket;
    double *out;
    int32_t lo, hi;
} o_force_job;

static void *o_force_worker(void *arg)
{
    o_force_job *j = (o_force_job *)arg;
    oracle_agent_forces(j->positions, j->radii, j->n, j->R, j->k, j->xDim, j->yDim,
                        j->wrapX, j->wrapY, j->offsets, j->bucket, j->out, j->lo, j->hi);
    return NULL;
}

int oracle_accumulate_forces(const double *positions, const double *radii,
                             int32_t n, double *velocityDeltas,
                             double interactionRad, double springConstant,
                             int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                             int32_t *cellOffsets, int32_t *bucketAgents,
                             int nthreads)
{
    oracle_agent_bins(positions, n, xDim, yDim, cellOffsets, bucketAgents);
    if (nthreads > n)
    {
        nthreads = n;
    }
    if (nthreads <= 1)
    {
        oracle_agent_forces(positions, radii, n, interactionRad, springConstant, xDim, yDim,
                            wrapX, wrapY, cellOffsets, bucketAgents, velocityDeltas, 0, n);
        return 0;
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    o_force_job *jobs = (o_force_job *)malloc(sizeof(o_force_job) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++)
    {
        o_force_job j = {positions, radii, n, interactionRad, springConstant, xDim, yDim,
                         wrapX, wrapY, cellOffsets, bucketAgents, velocityDeltas,
                         (int32_t)(((int64_t)n * t) / nthreads),
                         (int32_t)(((int64_t)n * (t + 1)) / nthreads)};
        jobs[t] = j;
        pthread_create(&th[t], NULL, o_force_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++)
    {
        pthread_join(th[t], NULL);
    }
    free(th);
    free(jobs);
    return 0;
}

/* ---- SphericalAgent2D::SumForces (include/Hal/Agents/SphericalAgent2D.h:74-102)
 * over an AgentGrid2D (include/Hal/Grids/AgentGrid2D.h:337-369) ---------- */

/* GridGeometry2D::DispX/DispY (src/Grids/GridGeometry2D.cpp:132-150) with
 * DispWrap (src/MathUtil.cpp:363-379) on a wrapped axis. */
static double o_disp_grid(double p1, double p2, int32_t dim, int wrap)
{
    if (wrap)
    {
        double dimF = (double)dim;
        if (fabs(p1 - p2) > (dimF / 2))
        {
            if (p1 > p2)
            {
                p2 = p2 + dimF;
            }
            else
            {
                p1 = p1 + dimF;
            }
        }
    }
    return p2 - p1;
}

/* The overlap force laws of the examples: linear (the backend's spring),
 * clamped Hooke's law (examples/OffLatticeExample.cpp:147-154) and a power
 * law (examples/Chemotaxis.cpp:128-130). */
static double o_overlap_force(int kind, double touchDist, double scale, double exponent)
{
    if (kind == 1)
    {
        if (touchDist < 0)
        {
            return 0;
        }
        return scale * touchDist;
    }
    if (kind == 2)
    {
        return pow(scale * touchDist, exponent);
    }
    return scale * touchDist;
}

void oracle_sum_forces(const double *positions, const double *radii, int32_t n,
                       const double *velIn, double *velOut, double *sums,
                       double interactionRad, int kind, double scale, double exponent,
                       int order, int32_t xDim, int32_t yDim, int wrapX, int wrapY)
{
    int32_t numCells = xDim * yDim;
    int32_t *offsets = (int32_t *)malloc(sizeof(int32_t) * ((size_t)numCells + 1));
    int32_t *bucket = (int32_t *)malloc(sizeof(int32_t) * ((size_t)n + 1));
    oracle_agent_bins(positions, n, xDim, yDim, offsets, bucket);
    for (int32_t i = 0; i < n; i++)
    {
        double posX = positions[(size_t)i * 2];
        double posY = positions[(size_t)i * 2 + 1];
        double rad = radii[i];
        double xVel = velIn ? velIn[(size_t)i * 2] : 0.0;
        double yVel = velIn ? velIn[(size_t)i * 2 + 1] : 0.0;
        double sum = 0;
        /* GetAgentsRadApprox: the squares of the window, x-major, skipping
         * or wrapping off-grid squares */
        int32_t xStart = (int32_t)floor(posX - interactionRad);
        int32_t xEnd = (int32_t)ceil(posX + interactionRad);
        int32_t yStart = (int32_t)floor(posY - interactionRad);
        int32_t yEnd = (int32_t)ceil(posY + interactionRad);
        for (int32_t xSq = xStart; xSq < xEnd; xSq++)
        {
            for (int32_t ySq = yStart; ySq < yEnd; ySq++)
            {
                int32_t retX = xSq;
                int32_t retY = ySq;
                int inX = (retX >= 0) && (retX < xDim);
                int inY = (retY >= 0) && (retY < yDim);
                if ((!wrapX && !inX) || (!wrapY && !inY))
                {
                    continue;
                }
                if (wrapX && !inX)
                {
                    retX = o_wrap_index(retX, xDim);
                }
                if (wrapY && !inY)
                {
                    retY = o_wrap_index(retY, yDim);
                }
                int32_t cell = retX * yDim + retY;
                int32_t start = offsets[cell];
                int32_t end = offsets[cell + 1];
                int32_t cnt = end - start;
                for (int32_t t = 0; t < cnt; t++)
                {
                    /* a square's agents: newest first on a grid filled in
                     * index order (AgentPT2D.h:200-241), else ascending */
                    int32_t j = bucket[order == 1 ? end - 1 - t : start + t];
                    if (j == i)
                    {
                        continue;
                    }
                    double xComp, yComp;
                    if (order == 1)
                    {
                        xComp = o_disp_grid(posX, positions[(size_t)j * 2], xDim, wrapX);
                        yComp = o_disp_grid(posY, positions[(size_t)j * 2 + 1], yDim, wrapY);
                    }
                    else
                    {
                        xComp = o_disp(posX, positions[(size_t)j * 2], xDim, wrapX);
                        yComp = o_disp(posY, positions[(size_t)j * 2 + 1], yDim, wrapY);
                    }
                    double dist = sqrt((xComp * xComp) + (yComp * yComp));
                    if ((dist < interactionRad) && (dist > 0.0))
                    {
                        double touchDist = (rad + radii[j]) - dist;
                        double force = o_overlap_force(kind, touchDist, scale, exponent);
                        xVel -= (xComp / dist) * force;
                        yVel -= (yComp / dist) * force;
                        if (force > 0)
                        {
                            sum += fabs(force);
                        }
                    }
                }
            }
        }
        velOut[(size_t)i * 2] = xVel;
        velOut[(size_t)i * 2 + 1] = yVel;
        if (sums)
        {
            sums[i] = sum;
        }
    }
    free(offsets);
    free(bucket);
}

/* ---- Hal::Rng (src/Rng.cpp) and the polar Gaussian -------------------- */

/* SplitMix64Next (src/Rng.cpp:61-68) */
static uint64_t o_splitmix(uint64_t *state)
{
    *state += 0x9E3779B97F4A7C15ULL;
    uint64_t z = *state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static uint64_t o_rotl(uint64_t x, int k)
{
    return (x << k) | (x >> (64 - k));
}

void oracle_rand_init(oracle_rand *r, uint64_t seed)
{
    /* Rng::Rng(uint64_t) (src/Rng.cpp:85-93) */
    uint64_t st = seed;
    r->s[0] = o_splitmix(&st);
    r->s[1] = o_splitmix(&st);
    r->s[2] = o_splitmix(&st);
    r->s[3] = o_splitmix(&st);
    r->v1 = 0;
    r->v2 = 0;
    r->sq = 0;
    r->phase = 0;
}

uint64_t oracle_rand_next(oracle_rand *r)
{
    /* xoshiro256** step (src/Rng.cpp:104-117) */
    const uint64_t result = o_rotl(r->s[1] * 5, 7) * 9;
    const uint64_t t = r->s[1] << 17;
    r->s[2] ^= r->s[0];
    r->s[3] ^= r->s[1];
    r->s[1] ^= r->s[2];
    r->s[0] ^= r->s[3];
    r->s[2] ^= t;
    r->s[3] = o_rotl(r->s[3], 45);
    return result;
}

double oracle_rand_double(oracle_rand *r)
{
    /* Rng::NextDouble (src/Rng.cpp:139-144) */
    const uint64_t mantissaBits = oracle_rand_next(r) >> 11;
    return (double)mantissaBits * (1.0 / 9007199254740992.0);
}

int32_t oracle_rand_int(oracle_rand *r, int32_t bound)
{
    /* Rng::BoundedUint64 / NextInt (src/Rng.cpp:119-137) */
    uint64_t b = (uint64_t)bound;
    const uint64_t threshold = (~b + 1) % b;
    uint64_t v = oracle_rand_next(r);
    while (v < threshold)
    {
        v = oracle_rand_next(r);
    }
    return (int32_t)(v % b);
}

double oracle_rand_gaussian(oracle_rand *r, double mean, double stdDev)
{
    /* GaussianSampler::Sample (src/GaussianSampler.cpp:23-47) */
    double x;
    if (r->phase == 0)
    {
        do
        {
            double u1 = oracle_rand_double(r);
            double u2 = oracle_rand_double(r);
            r->v1 = 2 * u1 - 1;
            r->v2 = 2 * u2 - 1;
            r->sq = r->v1 * r->v1 + r->v2 * r->v2;
        } while ((r->sq >= 1) || (r->sq == 0));
        x = r->v1 * sqrt(-2 * log(r->sq) / r->sq);
    }
    else
    {
        x = r->v2 * sqrt(-2 * log(r->sq) / r->sq);
    }
    r->phase = 1 - r->phase;
    return x * stdDev + mean;
}

/* ---- variable-rate ADI and its adjoint -------------------------------------
 * The reference has no variable-rate ADI and no gradient code.  This is the
 * builder's definition, written from HAL's variable-rate explicit stencil
 * Internal::Diffusion2(pField, pDeltas, pDiffRatesX, pDiffRatesY, ...)
 * (src/Pde/PDEequations.cpp:199-230): the face between cells j and j+1 of a
 * line has the rate of cell j (the +x/+y face uses the cell's own rate, the
 * -x/-y face the neighbour's), and a non-wrapped edge has no face.  With L
 * the face-weighted Laplacian of a line, one step is
 *   b1 = (I + L_y/2) f;  w = (I - L_x/2)^-1 b1;
 *   b2 = (I + L_x/2) w;  v = (I - L_y/2)^-1 b2;
 *   f' = f + (((v - f) + f * (-decay)) + src)      (PDEGrid2D tick order)
 * which for a constant rate D = r is Internal::Diffusion2DADI
 * (include/Hal/Pde/ADIequations.h:306-337) followed by the tick. */

/* Face weight on the low (eL) and high (eR) side of cell j of a line whose
 * face weights are e[j] = face (j, j+1) and, wrapped, e[n-1] = face (n-1, 0). */
static void o_var_faces(const double *e, int32_t n, int wrap, int32_t j, double *eL, double *eR)
{
    *eL = (j > 0) ? e[j - 1] : (wrap ? e[n - 1] : 0.0);
    *eR = (j < n - 1) ? e[j] : (wrap ? e[n - 1] : 0.0);
}

/* out = (I + s*L) u along one line (s = +1/2 or -1/2). */
static void o_var_apply(const double *e, int32_t n, int wrap, double s, const double *u, double *out)
{
    for (int32_t j = 0; j < n; j++)
    {
        double eL, eR;
        o_var_faces(e, n, wrap, j, &eL, &eR);
        double lo = (j > 0) ? u[j - 1] : (wrap ? u[n - 1] : u[j]);
        double hi = (j < n - 1) ? u[j + 1] : (wrap ? u[0] : u[j]);
        out[j] = u[j] + s * (eR * (hi - u[j]) + eL * (lo - u[j]));
    }
}

/* Solves (I - L/2) x = d along one line: Thomas, or for a wrapped line
 * Sherman-Morrison around Thomas (as TdmaSolver::TDMAperiodic does,
 * include/Hal/Pde/TdmaSolver.h:68-120).  work holds 6n doubles. */
static void o_var_solve(const double *e, int32_t n, int wrap, const double *d, double *x, double *work)
{
    double *a = work, *b = work + n, *c = work + 2 * n, *y = work + 3 * n, *z = work + 4 * n,
           *u = work + 5 * n;
    for (int32_t j = 0; j < n; j++)
    {
        double eL, eR;
        o_var_faces(e, n, wrap, j, &eL, &eR);
        a[j] = -0.5 * eL;
        c[j] = -0.5 * eR;
        b[j] = 1.0 + 0.5 * (eL + eR);
    }
    if (n == 1)
    {
        /* a wrapped single cell couples only to itself: L = 0 */
        x[0] = wrap ? d[0] / (a[0] + b[0] + c[0]) : d[0] / b[0];
        return;
    }
    double gamma = 0.0, a0 = a[0], cn = c[n - 1];
    if (wrap)
    {
        gamma = -b[0];
        b[0] -= gamma;
        b[n - 1] -= a0 * cn / gamma;
    }
    /* Thomas on (a, b, c) for the right-hand sides d -> y and (wrapped) u -> z */
    for (int32_t pass = 0; pass < (wrap ? 2 : 1); pass++)
    {
        const double *rhs = (pass == 0) ? d : u;
        double *out = (pass == 0) ? y : z;
        if (pass == 1)
        {
            for (int32_t j = 0; j < n; j++)
            {
                u[j] = 0.0;
            }
            u[0] = gamma;
            u[n - 1] = cn;
        }
        double *cp = x; /* scratch for the modified super-diagonal */
        double denom = b[0];
        cp[0] = c[0] / denom;
        out[0] = rhs[0] / denom;
        for (int32_t j = 1; j < n; j++)
        {
            denom = b[j] - a[j] * cp[j - 1];
            cp[j] = (j < n - 1) ? c[j] / denom : 0.0;
            out[j] = (rhs[j] - a[j] * out[j - 1]) / denom;
        }
        for (int32_t j = n - 2; j >= 0; j--)
        {
            out[j] -= cp[j] * out[j + 1];
        }
    }
    if (!wrap)
    {
        for (int32_t j = 0; j < n; j++)
        {
            x[j] = y[j];
        }
        return;
    }
    /* v = (1, 0, ..., a0/gamma) */
    double vy = y[0] + (a0 / gamma) * y[n - 1];
    double vz = z[0] + (a0 / gamma) * z[n - 1];
    double fct = vy / (1.0 + vz);
    for (int32_t j = 0; j < n; j++)
    {
        x[j] = y[j] - fct * z[j];
    }
}

/* Gathers line `l` of a row-major xDim x yDim array along x (dir 0: fixed y
 * = l) or along y (dir 1: fixed x = l). */
static void o_line_get(const double *g, int32_t xDim, int32_t yDim, int dir, int32_t l, double *out)
{
    if (dir == 0)
    {
        for (int32_t x = 0; x < xDim; x++)
        {
            out[x] = g[(size_t)x * yDim + l];
        }
    }
    else
    {
        memcpy(out, g + (size_t)l * yDim, sizeof(double) * (size_t)yDim);
    }
}

static void o_line_put(double *g, int32_t xDim, int32_t yDim, int dir, int32_t l, const double *in)
{
    if (dir == 0)
    {
        for (int32_t x = 0; x < xDim; x++)
        {
            g[(size_t)x * yDim + l] = in[x];
        }
    }
    else
    {
        memcpy(g + (size_t)l * yDim, in, sizeof(double) * (size_t)yDim);
    }
}

/* out = (I + s*L_dir) u, or with solve != 0 out = (I - L_dir/2)^-1 u, over
 * every line of direction dir; D holds the cell rates. */
static void o_var_sweep(const double *D, int32_t xDim, int32_t yDim, int wrapX, int wrapY, int dir, int solve,
                        double s, const double *u, double *out, double *work)
{
    const int32_t n = (dir == 0) ? xDim : yDim;
    const int32_t lines = (dir == 0) ? yDim : xDim;
    const int wrap = (dir == 0) ? wrapX : wrapY;
    double *e = work, *ul = work + n, *ol = work + 2 * n, *ws = work + 3 * n;
    for (int32_t l = 0; l < lines; l++)
    {
        o_line_get(D, xDim, yDim, dir, l, e);
        o_line_get(u, xDim, yDim, dir, l, ul);
        if (solve)
        {
            o_var_solve(e, n, wrap, ul, ol, ws);
        }
        else
        {
            o_var_apply(e, n, wrap, s, ul, ol);
        }
        o_line_put(out, xDim, yDim, dir, l, ol);
    }
}

/* Adds, for every face of direction dir, -1/2 (p_j+1 - p_j)(q_j+1 - q_j)
 * to the rate gradient of the face's owner cell j:  d<p, L q>/d e_face =
 * -(p_j+1 - p_j)(q_j+1 - q_j). */
static void o_var_face_grad(const double *p, const double *q, int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                            int dir, double *gD)
{
    for (int32_t x = 0; x < xDim; x++)
    {
        for (int32_t y = 0; y < yDim; y++)
        {
            int32_t nx = x, ny = y;
            if (dir == 0)
            {
                nx = x + 1;
                if (nx == xDim)
                {
                    if (!wrapX)
                    {
                        continue;
                    }
                    nx = 0;
                }
            }
            else
            {
                ny = y + 1;
                if (ny == yDim)
                {
                    if (!wrapY)
                    {
                        continue;
                    }
                    ny = 0;
                }
            }
            size_t i = (size_t)x * yDim + y, j = (size_t)nx * yDim + ny;
            if (i == j)
            {
                continue; /* a wrapped line of one cell has no effective face */
            }
            gD[i] += -0.5 * (p[j] - p[i]) * (q[j] - q[i]);
        }
    }
}

void oracle_dadi_step(const double *f, const double *D, int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                      double decay, const double *src, double *w, double *out)
{
    size_t len = (size_t)xDim * yDim;
    int32_t nmax = xDim > yDim ? xDim : yDim;
    double *b = malloc(sizeof(double) * len);
    double *work = malloc(sizeof(double) * (size_t)nmax * 9);
    o_var_sweep(D, xDim, yDim, wrapX, wrapY, 1, 0, 0.5, f, b, work);  /* b1 = (I + Ly/2) f */
    o_var_sweep(D, xDim, yDim, wrapX, wrapY, 0, 1, 0.0, b, w, work);  /* w = Ax^-1 b1 */
    o_var_sweep(D, xDim, yDim, wrapX, wrapY, 0, 0, 0.5, w, b, work);  /* b2 = (I + Lx/2) w */
    o_var_sweep(D, xDim, yDim, wrapX, wrapY, 1, 1, 0.0, b, out, work); /* v = Ay^-1 b2 */
    for (size_t i = 0; i < len; i++)
    {
        double delta = out[i] - f[i];
        delta += f[i] * (-decay);
        if (src != NULL)
        {
            delta += src[i];
        }
        out[i] = f[i] + delta;
    }
    free(b);
    free(work);
}

double oracle_dadi_loss_grad(const double *f0, const double *target, const double *D, double decay,
                             const double *src, int32_t xDim, int32_t yDim, int wrapX, int wrapY, int32_t steps,
                             double *fT, double *gD, double *gDecay, double *gSrc)
{
    size_t len = (size_t)xDim * yDim;
    int grad = (gD != NULL || gDecay != NULL || gSrc != NULL);
    /* all states f_0..f_T and intermediates w_t (the FP64 oracle keeps every
     * step; the GPU path checkpoints) */
    double *fs = malloc(sizeof(double) * len * (size_t)(steps + 1));
    double *ws = malloc(sizeof(double) * len * (size_t)(steps > 0 ? steps : 1));
    memcpy(fs, f0, sizeof(double) * len);
    for (int32_t t = 0; t < steps; t++)
    {
        oracle_dadi_step(fs + len * t, D, xDim, yDim, wrapX, wrapY, decay, src, ws + len * t, fs + len * (t + 1));
    }
    const double *f = fs + len * (size_t)steps;
    double loss = 0.0;
    for (size_t i = 0; i < len; i++)
    {
        double r = f[i] - target[i];
        loss += 0.5 * r * r;
    }
    if (fT != NULL)
    {
        memcpy(fT, f, sizeof(double) * len);
    }
    if (grad)
    {
        int32_t nmax = xDim > yDim ? xDim : yDim;
        double *g = malloc(sizeof(double) * len);
        double *b2 = malloc(sizeof(double) * len);
        double *t1 = malloc(sizeof(double) * len);
        double *b1 = malloc(sizeof(double) * len);
        double *v = malloc(sizeof(double) * len);
        double *work = malloc(sizeof(double) * (size_t)nmax * 9);
        double *dD = calloc(len, sizeof(double));
        double *dS = calloc(len, sizeof(double));
        double dK = 0.0;
        for (size_t i = 0; i < len; i++)
        {
            g[i] = f[i] - target[i];
        }
        for (int32_t t = steps - 1; t >= 0; t--)
        {
            const double *ft = fs + len * t, *wt = ws + len * t;
            /* v_t from the step's own sweeps */
            o_var_sweep(D, xDim, yDim, wrapX, wrapY, 0, 0, 0.5, wt, t1, work);
            o_var_sweep(D, xDim, yDim, wrapX, wrapY, 1, 1, 0.0, t1, v, work);
            /* f' = v - decay f + src */
            for (size_t i = 0; i < len; i++)
            {
                dS[i] += g[i];
                dK += -g[i] * ft[i];
            }
            /* v = Ay^-1 b2:  b2bar = Ay^-1 g (Ay symmetric), dD += 1/2 <b2bar, dLy v> */
            o_var_sweep(D, xDim, yDim, wrapX, wrapY, 1, 1, 0.0, g, b2, work);
            o_var_face_grad(b2, v, xDim, yDim, wrapX, wrapY, 1, dD);
            /* b2 = (I + Lx/2) w:  wbar = (I + Lx/2) b2bar, dD += 1/2 <b2bar, dLx w> */
            o_var_face_grad(b2, wt, xDim, yDim, wrapX, wrapY, 0, dD);
            o_var_sweep(D, xDim, yDim, wrapX, wrapY, 0, 0, 0.5, b2, t1, work);
            /* w = Ax^-1 b1:  b1bar = Ax^-1 wbar, dD += 1/2 <b1bar, dLx w> */
            o_var_sweep(D, xDim, yDim, wrapX, wrapY, 0, 1, 0.0, t1, b1, work);
            o_var_face_grad(b1, wt, xDim, yDim, wrapX, wrapY, 0, dD);
            /* b1 = (I + Ly/2) f:  fbar = (I + Ly/2) b1bar - decay g, dD += 1/2 <b1bar, dLy f> */
            o_var_face_grad(b1, ft, xDim, yDim, wrapX, wrapY, 1, dD);
            o_var_sweep(D, xDim, yDim, wrapX, wrapY, 1, 0, 0.5, b1, t1, work);
            for (size_t i = 0; i < len; i++)
            {
                g[i] = t1[i] - decay * g[i];
            }
        }
        if (gD != NULL)
        {
            memcpy(gD, dD, sizeof(double) * len);
        }
        if (gSrc != NULL)
        {
            memcpy(gSrc, dS, sizeof(double) * len);
        }
        if (gDecay != NULL)
        {
            *gDecay = dK;
        }
        free(g);
        free(b2);
        free(t1);
        free(b1);
        free(v);
        free(work);
        free(dD);
        free(dS);
    }
    free(fs);
    free(ws);
    return loss;
}

/* ---- variable-rate diffusion and upwind advection --------------------------- */

/* DisplacedX2D / DisplacedY2D (src/Pde/PDEequations.cpp:163-197): the value of
 * a per-cell array at a possibly off-grid neighbour, wrapped, or 0. */
/* DisplacedX2D / DisplacedY2D (src/Pde/PDEequations.cpp:163-197) and their
 * Dirichlet forms (include/Hal/Pde/PDEequations.h:589-616): the value at an
 * off-grid coordinate of a closed axis is 0, or the boundary value itself
 * (not doubled) when a ghost table is given. */
static double o_displaced_x(const double *v, int32_t x, int32_t y, int32_t xDim, int32_t yDim, int wrapX,
                            const double *ghost)
{
    if (o_in_dim(x, xDim))
    {
        return v[x * yDim + y];
    }
    if (wrapX)
    {
        return v[o_wrap(x, xDim) * yDim + y];
    }
    return ghost != NULL ? o_ghost_x(ghost, x, y, yDim) : 0.0;
}

static double o_displaced_y(const double *v, int32_t x, int32_t y, int32_t xDim, int32_t yDim, int wrapY,
                            const double *ghost)
{
    if (o_in_dim(y, yDim))
    {
        return v[x * yDim + y];
    }
    if (wrapY)
    {
        return v[x * yDim + o_wrap(y, yDim)];
    }
    return ghost != NULL ? o_ghost_y(ghost, x, y, xDim, yDim) : 0.0;
}

void oracle_diffusion2_var(const double *field, double *deltas, const double *ratesX, const double *ratesY,
                           int32_t xDim, int32_t yDim, int wrapX, int wrapY)
{
    for (int32_t x = 0; x < xDim; x++)
    {
        for (int32_t y = 0; y < yDim; y++)
        {
            int32_t i = x * yDim + y;
            double c = field[i];
            double dp1x = ((x == xDim - 1) && !wrapX) ? o_displaced_x(ratesX, x + 1, y, xDim, yDim, wrapX, NULL) : ratesX[i];
            double dm1x = o_displaced_x(ratesX, x - 1, y, xDim, yDim, wrapX, NULL);
            double dp1y = ((y == yDim - 1) && !wrapY) ? o_displaced_y(ratesY, x, y + 1, xDim, yDim, wrapY, NULL) : ratesY[i];
            double dm1y = o_displaced_y(ratesY, x, y - 1, xDim, yDim, wrapY, NULL);
            double s = o_delta_x(field, c, x + 1, y, xDim, yDim, wrapX, NULL) * dp1x;
            s += o_delta_x(field, c, x - 1, y, xDim, yDim, wrapX, NULL) * dm1x;
            s += o_delta_y(field, c, x, y + 1, xDim, yDim, wrapY, NULL) * dp1y;
            s += o_delta_y(field, c, x, y - 1, xDim, yDim, wrapY, NULL) * dm1y;
            deltas[i] += s;
        }
    }
}

void oracle_advection2_bc(const double *field, double *deltas, double xVel, double yVel, int32_t xDim,
                          int32_t yDim, int wrapX, int wrapY, const double *ghost)
{
    for (int32_t x = 0; x < xDim; x++)
    {
        for (int32_t y = 0; y < yDim; y++)
        {
            int32_t i = x * yDim + y;
            double c = field[i];
            if (xVel > 0)
            {
                deltas[i] += o_delta_x(field, c, x - 1, y, xDim, yDim, wrapX, ghost) * xVel;
            }
            else if (xVel < 0)
            {
                deltas[i] -= o_delta_x(field, c, x + 1, y, xDim, yDim, wrapX, ghost) * xVel;
            }
            if (yVel > 0)
            {
                deltas[i] += o_delta_y(field, c, x, y - 1, xDim, yDim, wrapY, ghost) * yVel;
            }
            else if (yVel < 0)
            {
                deltas[i] -= o_delta_y(field, c, x, y + 1, xDim, yDim, wrapY, ghost) * yVel;
            }
        }
    }
}

void oracle_advection2(const double *field, double *deltas, double xVel, double yVel, int32_t xDim, int32_t yDim,
                       int wrapX, int wrapY)
{
    oracle_advection2_bc(field, deltas, xVel, yVel, xDim, yDim, wrapX, wrapY, NULL);
}

void oracle_advection2_var_bc(const double *field, double *deltas, const double *xVels, const double *yVels,
                              int32_t xDim, int32_t yDim, int wrapX, int wrapY, const double *ghost,
                              const double *ghostXVel, const double *ghostYVel)
{
    for (int32_t x = 0; x < xDim; x++)
    {
        for (int32_t y = 0; y < yDim; y++)
        {
            int32_t i = x * yDim + y;
            double xVelP = ((x == xDim - 1) && !wrapX) ? o_displaced_x(xVels, x + 1, y, xDim, yDim, wrapX, ghostXVel) : xVels[i];
            double yVelP = ((y == yDim - 1) && !wrapY) ? o_displaced_y(yVels, x, y + 1, xDim, yDim, wrapY, ghostYVel) : yVels[i];
            double xVelM = o_displaced_x(xVels, x - 1, y, xDim, yDim, wrapX, ghostXVel);
            double yVelM = o_displaced_y(yVels, x, y - 1, xDim, yDim, wrapY, ghostYVel);
            double c = field[i];
            double xFluxP = 0.0, xFluxM = 0.0, yFluxP = 0.0, yFluxM = 0.0;
            if (xVelP > 0)
            {
                xFluxP = xVelP * c;
            }
            else if (xVelP < 0)
            {
                xFluxP = xVelP * o_displaced_x(field, x + 1, y, xDim, yDim, wrapX, ghost);
            }
            if (xVelM > 0)
            {
                xFluxM = xVelM * o_displaced_x(field, x - 1, y, xDim, yDim, wrapX, ghost);
            }
            else if (xVelM < 0)
            {
                xFluxM = xVelM * c;
            }
            if (yVelP > 0)
            {
                yFluxP = yVelP * c;
            }
            else if (yVelP < 0)
            {
                yFluxP = yVelP * o_displaced_y(field, x, y + 1, xDim, yDim, wrapY, ghost);
            }
            if (yVelM > 0)
            {
                yFluxM = yVelM * o_displaced_y(field, x, y - 1, xDim, yDim, wrapY, ghost);
            }
            else if (yVelM < 0)
            {
                yFluxM = yVelM * c;
            }
            deltas[i] += -xFluxP + xFluxM - yFluxP + yFluxM;
        }
    }
}

void oracle_advection2_var(const double *field, double *deltas, const double *xVels, const double *yVels,
                           int32_t xDim, int32_t yDim, int wrapX, int wrapY)
{
    oracle_advection2_var_bc(field, deltas, xVels, yVels, xDim, yDim, wrapX, wrapY, NULL, NULL, NULL);
}

/* ---- agent integration step ------------------------------------------------ */

/* Written once for both precisions: T is double or float, FMOD and SQRT the
 * matching libm functions. */
#define O_AGENTS_MOVE(NAME, T, FMOD, SQRT)                                                             \
    void NAME(T *pos, T *vel, const T *deltas, int32_t n, int32_t xDim, int32_t yDim, int wrapX,        \
              int wrapY, T friction, T maxVel)                                                          \
    {                                                                                                   \
        const T xd = (T)xDim, yd = (T)yDim;                                                             \
        for (int32_t i = 0; i < n; i++)                                                                 \
        {                                                                                               \
            T vx = vel[2 * i] + deltas[2 * i];                                                          \
            T vy = vel[2 * i + 1] + deltas[2 * i + 1];                                                  \
            if (maxVel >= 0)                                                                            \
            { /* CapVelocity, SphericalAgent2D.h:143-153 */                                             \
                T maxVelSq = maxVel * maxVel;                                                           \
                T normSq = (vx * vx) + (vy * vy);                                                       \
                if (normSq > maxVelSq)                                                                  \
                {                                                                                       \
                    T conv = maxVel / SQRT(normSq);                                                     \
                    vx *= conv;                                                                         \
                    vy *= conv;                                                                         \
                }                                                                                       \
            }                                                                                           \
            /* ForceMove -> MoveSafePT, AgentPT2D.h:157-186 */                                          \
            T px = pos[2 * i], py = pos[2 * i + 1];                                                     \
            T nx = px + vx, ny = py + vy;                                                               \
            int in = (nx >= 0) && (nx < xd) && (ny >= 0) && (ny < yd);                                  \
            if (!in)                                                                                    \
            {                                                                                           \
                if (wrapX)                                                                              \
                {                                                                                       \
                    T m = FMOD(nx, xd);                                                                 \
                    nx = (m < 0) ? (xd + m) : m;                                                        \
                }                                                                                       \
                else if (!((nx >= 0) && (nx < xd)))                                                     \
                {                                                                                       \
                    nx = px;                                                                            \
                }                                                                                       \
                if (wrapY)                                                                              \
                {                                                                                       \
                    T m = FMOD(ny, yd);                                                                 \
                    ny = (m < 0) ? (yd + m) : m;                                                        \
                }                                                                                       \
                else if (!((ny >= 0) && (ny < yd)))                                                     \
                {                                                                                       \
                    ny = py;                                                                            \
                }                                                                                       \
            }                                                                                           \
            pos[2 * i] = nx;                                                                            \
            pos[2 * i + 1] = ny;                                                                        \
            /* ApplyFriction, SphericalAgent2D.h:135-141 */                                             \
            vel[2 * i] = vx * friction;                                                                 \
            vel[2 * i + 1] = vy * friction;                                                             \
        }                                                                                               \
    }

O_AGENTS_MOVE(oracle_agents_move, double, fmod, sqrt)
O_AGENTS_MOVE(oracle_agents_move_f32, float, fmodf, sqrtf)

/* ---- Hal::PDEGrid2D call sequences (include/Hal/Grids/PDEGrid2D.h) --------
 * A script of calls on one grid, run as the reference's PDEGrid2D runs them:
 * see oracle_pdegrid_script in hal_oracle.h for the encoding. */

static void o_cell_op(int op, double *deltas, const double *field, int32_t i, double v)
{
    switch (op)
    {
    case 0: /* Set (:88-99) */
        deltas[i] = v - field[i];
        break;
    case 1: /* Add (:101-112) */
        deltas[i] += v;
        break;
    case 2: /* Mul (:114-126) */
        deltas[i] += field[i] * v;
        break;
    default: /* Scale (:128-140) */
        deltas[i] += field[i] * (v - 1);
        break;
    }
}

/* DisplacedFieldX / DisplacedFieldY (:400-430) */
static double o_displaced(const double *f, int32_t x, int32_t y, int alongX, int32_t xDim, int32_t yDim,
                          int wrapX, int wrapY, double oob)
{
    if (alongX)
    {
        if (o_in_dim(x, xDim))
        {
            return f[x * yDim + y];
        }
        if (wrapX)
        {
            return f[o_wrap(x, xDim) * yDim + y];
        }
        return oob;
    }
    if (o_in_dim(y, yDim))
    {
        return f[x * yDim + y];
    }
    if (wrapY)
    {
        return f[x * yDim + o_wrap(y, yDim)];
    }
    return oob;
}

int oracle_pdegrid_script(int32_t xDim, int32_t yDim, int wrapX, int wrapY, double *field, double *deltas,
                          int32_t *updateCt, int32_t nOps, const int32_t *ops, const int32_t *iargs,
                          const double *dargs, const double *arrays, double *records)
{
    int32_t length = xDim * yDim;
    double *scratch = (double *)malloc(sizeof(double) * ((size_t)length + 1));
    int32_t nRec = 0;
    for (int32_t k = 0; k < nOps; k++)
    {
        const int32_t *ia = iargs + 3 * (size_t)k;
        const double *da = dargs + 2 * (size_t)k;
        const double *arr = arrays + ia[0];
        int op = ops[k];
        if (op >= 0 && op <= 3)
        {
            o_cell_op(op, deltas, field, ia[1], da[0]);
        }
        else if (op >= 10 && op <= 12)
        {
            /* SetAll / AddAll / MulAll (:188-217) */
            for (int32_t i = 0; i < length; i++)
            {
                o_cell_op(op - 10, deltas, field, i, da[0]);
            }
        }
        else if (op == 13)
        {
            for (int32_t i = 0; i < length; i++)
            {
                o_cell_op(0, deltas, field, i, arr[i]);
            }
        }
        else if (op == 20 || op == 21)
        {
            if (da[0] > 0.25)
            {
                free(scratch);
                return -1;
            }
            oracle_diffusion2(field, deltas, da[0], xDim, yDim, wrapX, wrapY, op == 21 ? arr : NULL);
        }
        else if (op == 22)
        {
            oracle_diffusion2_var(field, deltas, arr, arr + length, xDim, yDim, wrapX, wrapY);
        }
        else if (op == 30 || op == 31)
        {
            oracle_adi2(field, scratch, deltas, da[0], xDim, yDim, wrapX, wrapY, op == 31 ? arr : NULL);
        }
        else if (op == 40 || op == 41)
        {
            if ((fabs(da[0]) + fabs(da[1])) > 0.5)
            {
                free(scratch);
                return -2;
            }
            oracle_advection2_bc(field, deltas, da[0], da[1], xDim, yDim, wrapX, wrapY, op == 41 ? arr : NULL);
        }
        else if (op == 42)
        {
            oracle_advection2_var(field, deltas, arr, arr + length, xDim, yDim, wrapX, wrapY);
        }
        else if (op == 43)
        {
            int32_t g = 2 * (xDim + yDim);
            oracle_advection2_var_bc(field, deltas, arr, arr + length, xDim, yDim, wrapX, wrapY, arr + 2 * length,
                                     arr + 2 * length + g, arr + 2 * length + 2 * g);
        }
        else if (op == 50)
        {
            /* Update (:178-186) */
            for (int32_t i = 0; i < length; i++)
            {
                field[i] += deltas[i];
            }
            memset(deltas, 0, sizeof(double) * (size_t)length);
            (*updateCt)++;
        }
        else if (op == 51)
        {
            /* SetNonNegative (:244-255) */
            for (int32_t i = 0; i < length; i++)
            {
                if ((field[i] + deltas[i]) < 0)
                {
                    deltas[i] = 0 - field[i];
                }
            }
        }
        else if (op == 60)
        {
            records[nRec++] = field[ia[1]];
        }
        else if (op == 61 || op == 62)
        {
            /* GetMax / GetMin (:142-164): std::max(field, max) keeps the
             * later of equal values */
            double m = (op == 61) ? -DBL_MAX : DBL_MAX;
            for (int32_t i = 0; i < length; i++)
            {
                if (op == 61)
                {
                    m = (field[i] < m) ? m : field[i];
                }
                else
                {
                    m = (m < field[i]) ? m : field[i];
                }
            }
            records[nRec++] = m;
        }
        else if (op == 63)
        {
            double tot = 0;
            for (int32_t i = 0; i < length; i++)
            {
                tot += field[i];
            }
            records[nRec++] = tot / length;
        }
        else if (op == 64 || op == 65)
        {
            /* MaxDelta / MaxDeltaScaled (:219-241) */
            double maxDif = 0;
            for (int32_t i = 0; i < length; i++)
            {
                double v = (op == 64) ? fabs(deltas[i]) : fabs(deltas[i] / (fabs(field[i]) + da[0]));
                maxDif = (maxDif < v) ? v : maxDif;
            }
            records[nRec++] = maxDif;
        }
        else if (op >= 66 && op <= 69)
        {
            /* GradientX / GradientY (:257-285) */
            int32_t x = ia[1], y = ia[2];
            double own = field[x * yDim + y];
            double oob = (op >= 68) ? da[0] : own;
            if (op == 66 || op == 68)
            {
                records[nRec++] = o_displaced(field, x + 1, y, 1, xDim, yDim, wrapX, wrapY, oob) -
                                  o_displaced(field, x - 1, y, 1, xDim, yDim, wrapX, wrapY, oob);
            }
            else
            {
                records[nRec++] = o_displaced(field, x, y + 1, 0, xDim, yDim, wrapX, wrapY, oob) -
                                  o_displaced(field, x, y - 1, 0, xDim, yDim, wrapX, wrapY, oob);
            }
        }
    }
    free(scratch);
    return nRec;
}
