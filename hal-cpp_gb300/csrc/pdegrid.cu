// pdegrid.cu -- a device-resident Hal::PDEGrid2D (include/Hal/Grids/PDEGrid2D.h).
//
// PDEGrid2D keeps a committed field and a delta buffer: Get reads the field,
// Set/Add/Mul/Scale and the PDE operators accumulate into the deltas, and
// Update commits them (PDEGrid2D.h:17-186).  This handle keeps both buffers in
// HBM in FP64 and reproduces every call bit for bit:
//   * per-cell operations arrive as lists (from the host, or one per agent of
//     an agent handle's last binning); entries of one cell are applied by one
//     thread in list order, so repeated cells accumulate exactly as a loop of
//     single calls does;
//   * the explicit stencils are the FP64 functors of the interface path
//     (IEEE operations in the reference's order);
//   * DiffusionADI is the reference's Thomas solve per line
//     (include/Hal/Pde/ADIequations.h:225-337, TdmaSolver.h:26-120) in FP64.
//     Its matrix is the same for every line of a sweep, so the modified
//     diagonal, the elimination multipliers and, on a periodic axis, the
//     Sherman-Morrison vector are computed once on the host with the
//     reference's operations; each line then runs the right-hand-side part
//     of the elimination and the back substitution, one thread per line, in
//     the reference's order.  The x-sweep reads its lines across the
//     contiguous y index (coalesced); its output is transposed so that the
//     y-sweep reads coalesced too, and the y-sweep's result is transposed
//     back while it is added into the deltas.
#include "common.cuh"
#include "adi64.h"
#include "stencil64.cuh"
#include "agents_wells.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <numeric>
#include <vector>

using namespace halcuda::stencil64;

namespace halcuda
{
    namespace
    {
        // ---- per-cell operations (PDEGrid2D.h:88-140) ---------------------
        constexpr int kOpSet = HAL_CUDA_CELL_SET;
        constexpr int kOpAdd = HAL_CUDA_CELL_ADD;
        constexpr int kOpMul = HAL_CUDA_CELL_MUL;
        constexpr int kOpScale = HAL_CUDA_CELL_SCALE;

        // One operation on a cell's delta d given its committed value f:
        // Set d = v - f, Add d += v, Mul d += f * v, Scale d += f * (v - 1).
        __device__ __forceinline__ double ApplyOp(int op, double d, double f, double v)
        {
            switch (op)
            {
            case kOpSet:
                return __dsub_rn(v, f);
            case kOpAdd:
                return __dadd_rn(d, v);
            case kOpMul:
                return __dadd_rn(d, __dmul_rn(f, v));
            default:
                return __dadd_rn(d, __dmul_rn(f, __dsub_rn(v, 1.0)));
            }
        }

        // Runs of a cell-sorted operation list: run r covers entries
        // [runStart[r], runStart[r + 1]) of one cell, in list order.
        __global__ void ApplyRuns(const int32_t *__restrict__ cells, const int8_t *__restrict__ ops,
                                  const double *__restrict__ vals, const int32_t *__restrict__ runStart, int32_t nRuns,
                                  const double *__restrict__ f, double *__restrict__ deltas)
        {
            const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
            if (r >= nRuns)
            {
                return;
            }
            const int32_t s = runStart[r], e = runStart[r + 1];
            const int64_t c = cells[s];
            const double fc = f[c];
            double d = deltas[c];
            for (int32_t k = s; k < e; k++)
            {
                d = ApplyOp(ops[k], d, fc, vals[k]);
            }
            deltas[c] = d;
        }

        // One operation per agent of a binning, each at its agent's cell, in
        // agent index order within a cell (the bucket order): the thread of
        // the first slot of each occupied cell applies the cell's agents.
        __global__ void ApplyAgents(const int32_t *__restrict__ offsets, const int32_t *__restrict__ bucket,
                                    const int32_t *__restrict__ cellOf, int32_t n, int op, double value,
                                    const double *__restrict__ perAgent, const double *__restrict__ f,
                                    double *__restrict__ deltas)
        {
            const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
            if (s >= n)
            {
                return;
            }
            const int32_t c = cellOf[bucket[s]];
            if (offsets[c] != s)
            {
                return;
            }
            const int32_t e = offsets[c + 1];
            const double fc = f[c];
            double d = deltas[c];
            for (int32_t k = s; k < e; k++)
            {
                d = ApplyOp(op, d, fc, perAgent != nullptr ? perAgent[bucket[k]] : value);
            }
            deltas[c] = d;
        }

        // SetAll / AddAll / MulAll (PDEGrid2D.h:188-217): the operation at
        // every cell, the value a scalar or (SetAll(pVals)) one per cell.
        __global__ void ApplyAll(int op, double value, const double *__restrict__ perCell, int64_t n,
                                 const double *__restrict__ f, double *__restrict__ deltas)
        {
            for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
                 i += static_cast<int64_t>(gridDim.x) * blockDim.x)
            {
                deltas[i] = ApplyOp(op, deltas[i], f[i], perCell != nullptr ? perCell[i] : value);
            }
        }

        // Update (PDEGrid2D.h:178-186): field += deltas, deltas = 0.
        __global__ void Commit(int64_t n, double *__restrict__ f, double *__restrict__ deltas)
        {
            for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
                 i += static_cast<int64_t>(gridDim.x) * blockDim.x)
            {
                f[i] = __dadd_rn(f[i], deltas[i]);
                deltas[i] = 0.0;
            }
        }

        // A value-form SetAll / AddAll / MulAll deferred to the Update right
        // after it, in one pass: deltas = op(deltas, field, value), then
        // field += deltas and deltas = 0, the two kernels' operations in
        // their order.
        __global__ void ApplyAllCommit(int op, double value, int64_t n, double *__restrict__ f,
                                       double *__restrict__ deltas)
        {
            for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
                 i += static_cast<int64_t>(gridDim.x) * blockDim.x)
            {
                const double fi = f[i];
                const double d = ApplyOp(op, deltas[i], fi, value);
                f[i] = __dadd_rn(fi, d);
                deltas[i] = 0.0;
            }
        }

        // SetNonNegative (PDEGrid2D.h:244-255): Set(i, 0) where f + d < 0.
        __global__ void NonNegative(int64_t n, const double *__restrict__ f, double *__restrict__ deltas)
        {
            for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
                 i += static_cast<int64_t>(gridDim.x) * blockDim.x)
            {
                if (__dadd_rn(f[i], deltas[i]) < 0.0)
                {
                    deltas[i] = __dsub_rn(0.0, f[i]);
                }
            }
        }

        __global__ void Gather(const int32_t *__restrict__ cells, int64_t n, const double *__restrict__ f,
                               double *__restrict__ out)
        {
            const int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
            if (k < n)
            {
                out[k] = f[cells[k]];
            }
        }

        // ---- reductions: GetMax, GetMin, GetAvg, MaxDelta, MaxDeltaScaled ----
        // GetMax keeps max = (f < max) ? max : f over the cells in order, so
        // of equal values (+0 and -0 compare equal) the last one is kept; the
        // reduction carries the index to keep the same one.  GetMin likewise.
        struct Extreme
        {
            double v;
            int64_t i;
        };

        __device__ __forceinline__ Extreme MaxOf(Extreme a, Extreme b)  // a before b or after: by index
        {
            if (a.v < b.v)
            {
                return b;
            }
            if (b.v < a.v)
            {
                return a;
            }
            return (a.i > b.i) ? a : b;
        }

        __device__ __forceinline__ Extreme MinOf(Extreme a, Extreme b)
        {
            if (b.v < a.v)
            {
                return b;
            }
            if (a.v < b.v)
            {
                return a;
            }
            return (a.i > b.i) ? a : b;
        }

        constexpr int kRedThreads = 256;
        constexpr int kRedBlocks = 592;  // 4 per SM on 148-152 SMs

        // Per block: the extremes of its cells, the sum of the field (in a
        // fixed order, so the result is deterministic), max |d| and max
        // |d / (|f| + offset)|.  Partials go to out[block]; the host combines
        // them in block order.
        struct RedPartial
        {
            double maxV, minV, sum, maxDelta, maxScaled;
            long long maxI, minI;
        };

        __global__ void __launch_bounds__(kRedThreads) Reduce(int64_t n, const double *__restrict__ f,
                                                              const double *__restrict__ deltas, double offset,
                                                              bool scaled, RedPartial *__restrict__ out)
        {
            const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
            const int64_t lo = blockIdx.x * chunk;
            const int64_t hi = (lo + chunk < n) ? lo + chunk : n;
            Extreme mx = {-INFINITY, -1}, mn = {INFINITY, -1};
            double sum = 0.0, md = 0.0, ms = 0.0;
            for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
            {
                const double fv = f[i];
                const double dv = deltas[i];
                mx = MaxOf(mx, Extreme{fv, i});
                mn = MinOf(mn, Extreme{fv, i});
                sum = __dadd_rn(sum, fv);
                md = fmax(md, fabs(dv));
                if (scaled)
                {
                    ms = fmax(ms, fabs(__ddiv_rn(dv, __dadd_rn(fabs(fv), offset))));
                }
            }
            __shared__ RedPartial sh[kRedThreads];
            sh[threadIdx.x] = RedPartial{mx.v, mn.v, sum, md, ms, mx.i, mn.i};
            __syncthreads();
            for (int w = kRedThreads / 2; w > 0; w >>= 1)
            {
                if (threadIdx.x < w)
                {
                    RedPartial a = sh[threadIdx.x], b = sh[threadIdx.x + w];
                    const Extreme xm = MaxOf(Extreme{a.maxV, a.maxI}, Extreme{b.maxV, b.maxI});
                    const Extreme xn = MinOf(Extreme{a.minV, a.minI}, Extreme{b.minV, b.minI});
                    a.maxV = xm.v;
                    a.maxI = xm.i;
                    a.minV = xn.v;
                    a.minI = xn.i;
                    a.sum = __dadd_rn(a.sum, b.sum);
                    a.maxDelta = fmax(a.maxDelta, b.maxDelta);
                    a.maxScaled = fmax(a.maxScaled, b.maxScaled);
                    sh[threadIdx.x] = a;
                }
                __syncthreads();
            }
            if (threadIdx.x == 0)
            {
                out[blockIdx.x] = sh[0];
            }
        }

        // GradientX/GradientY (PDEGrid2D.h:257-285) at query points:
        // DisplacedField(x+1) - DisplacedField(x-1), off-grid the cell's own
        // value (reflecting) or a boundary value.
        __device__ __forceinline__ double DisplacedField(const double *f, int32_t a, int32_t b, bool alongX,
                                                         int32_t xDim, int32_t yDim, bool wrap, double oob)
        {
            const int32_t dim = alongX ? xDim : yDim;
            int32_t v = alongX ? a : b;
            if (v < 0 || v >= dim)
            {
                if (!wrap)
                {
                    return oob;
                }
                v %= dim;
                v = (v < 0) ? v + dim : v;
            }
            return alongX ? f[static_cast<int64_t>(v) * yDim + b] : f[static_cast<int64_t>(a) * yDim + v];
        }

        __global__ void Gradients(const int32_t *__restrict__ xs, const int32_t *__restrict__ ys, int64_t n,
                                  const double *__restrict__ f, int32_t xDim, int32_t yDim, int32_t wrapX,
                                  int32_t wrapY, int32_t useBoundary, double boundary, double *__restrict__ gx,
                                  double *__restrict__ gy)
        {
            const int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
            if (k >= n)
            {
                return;
            }
            const int32_t x = xs[k], y = ys[k];
            const double own = f[static_cast<int64_t>(x) * yDim + y];
            const double oob = useBoundary ? boundary : own;
            gx[k] = __dsub_rn(DisplacedField(f, x + 1, y, true, xDim, yDim, wrapX != 0, oob),
                              DisplacedField(f, x - 1, y, true, xDim, yDim, wrapX != 0, oob));
            gy[k] = __dsub_rn(DisplacedField(f, x, y + 1, false, xDim, yDim, wrapY != 0, oob),
                              DisplacedField(f, x, y - 1, false, xDim, yDim, wrapY != 0, oob));
        }

        // ---- ADI in FP64 ----------------------------------------------------
        // The line-independent part of one sweep's Thomas solve.
        struct LinePlan64Dev
        {
            const double *ws;    // elimination multipliers (index 0 unused)
            const double *bs;    // modified diagonal
            const double *zs;    // periodic: the Sherman-Morrison solution
            const double2 *bh;   // (bs[i], RN(1 / bs[i])): DivByPlan's b and yHi
            const int2 *lo;      // RN(1 / bs[i]) - yHi as (FP32 mantissa bits, exponent)
            double off;          // the off-diagonal -r/2
            double vEnd;         // periodic: beta / gamma
            double onePlusVz;    // periodic: 1 + (zs[0] + zs[L-1] * vEnd)
            int32_t L;
            int32_t periodic;
            int32_t fastDiv;     // every bs[i] in [2^-20, 2^20]: DivByPlan is exact
        };

        // ExplicitDiffusionY2ADI / X2ADI (src/Pde/ADIequations.cpp:19-47 and
        // the Dirichlet forms, include/Hal/Pde/ADIequations.h:54-94): the
        // cell plus half the rate times its two cross-axis differences.
        __device__ __forceinline__ double HalfStep(double c, double d1, double d2, double r)
        {
            return __dadd_rn(c, __dmul_rn(__dmul_rn(__dadd_rn(d1, d2), r), 0.5));
        }

        // ImplicitBoundarySource (ADIequations.h:198-220) at position i of a
        // line of length L; 0 on a wrapped axis.
        __device__ __forceinline__ double ImplicitSource(int32_t i, int32_t L, bool wrap, double r, double lo,
                                                         double hi)
        {
            if (wrap)
            {
                return 0.0;
            }
            double source = 0.0;
            if (i == 0)
            {
                source = __dadd_rn(source, lo);
            }
            if (i == L - 1)
            {
                source = __dadd_rn(source, hi);
            }
            return __dmul_rn(__dmul_rn(__dmul_rn(source, 2.0), r), 0.5);
        }

        // Difference to a cross-axis neighbour n of a line of length dim:
        // on the grid, wrapped, a doubled Dirichlet ghost, or 0.
        __device__ __forceinline__ double CrossDelta(const double *v, double c, int32_t n, int32_t dim, bool wrap,
                                                     int64_t base, int64_t stride, const double *ghost, int64_t gi)
        {
            return DeltaTerm64(v, c, n, dim, wrap, base, stride, ghost, gi);
        }

        // An approximation of n * yLo, for DivByPlan, without FP64
        // instructions: yLo = mLo * 2^eLo with mLo an FP32 value in +-[1, 2]
        // (0 for yLo = 0, with eLo very negative); n's top 20 mantissa bits
        // times mLo in FP32, the exponents added as integers.  Within 1e-5
        // of n * yLo relative, or 0 where n is +-0 or subnormal or the
        // product is below 2^-1022.
        __device__ __forceinline__ double ApproxTimesLo(double n, float mLo, int32_t eLo)
        {
            const uint32_t hi = static_cast<uint32_t>(__double2hiint(n));
            const int32_t en = static_cast<int32_t>((hi >> 20) & 0x7ffu);
            const float fn = __uint_as_float(0x3f800000u | ((hi & 0xfffffu) << 3));
            const uint32_t pb = __float_as_uint(fn * mLo);
            const int32_t te = en + eLo + static_cast<int32_t>((pb >> 23) & 0xffu) - 127;
            const uint32_t tHi = ((hi ^ pb) & 0x80000000u) | (static_cast<uint32_t>(te) << 20) | ((pb & 0x7fffffu) >> 3);
            const bool ok = te > 0 && en != 0;
            return __hiloint2double(ok ? static_cast<int32_t>(tHi) : 0, ok ? static_cast<int32_t>(pb << 29) : 0);
        }

        // n / b rounded to nearest, bit-equal to __ddiv_rn(n, b) for every n
        // that PlanDivisionOutOfRange accepts, from the plan's reciprocal of
        // b as a double-word: yHi = RN(1/b) and yLo = RN(1/b - yHi) (|yLo| <=
        // 2^-53 |yHi|).  With t within half of n*yLo (ApproxTimesLo's is
        // within 1e-5), n*yHi + t is within 2^-54 |n/b| of n/b, so q =
        // RN(n*yHi + t) is one of the two doubles around n/b (faithful); its
        // remainder n - b*q is then exact under an FMA, and RN(q + rem*yHi)
        // is the correctly rounded quotient by Markstein's theorem (P.
        // Markstein, "Computation of elementary functions on the IBM RISC
        // System/6000 processor", IBM J. Res. Dev. 34(1), 1990: y within half
        // an ulp of 1/b, q within one ulp of n/b).  The argument needs no
        // intermediate to underflow or overflow: the plan allows b in
        // [2^-20, 2^20] only (fastDiv), and n must lie in [2^-900, 2^900) in
        // magnitude.  n = +0 gives +0 (t = 0, q = +0, rem = +0, for b > 0);
        // n = -0 would give +0 too, so PlanDivisionOutOfRange refuses it.
        // Three dependent FP64 operations instead of a division's longer
        // sequence; hal_cuda_check_plan_division compares the two.
        __device__ __forceinline__ double DivByPlan(double n, double2 bh, int2 lo)
        {
            const double t = ApproxTimesLo(n, __int_as_float(lo.x), lo.y);
            const double q = __fma_rn(n, bh.y, t);
            const double rem = __fma_rn(-bh.x, q, n);
            return __fma_rn(rem, bh.y, q);
        }

        // Nonzero when DivByPlan may not be exact for the numerator n: -0,
        // subnormal, nonzero below 2^-900 or from 2^900 in magnitude, inf or
        // NaN.  Integer operations only, off the FP64 chain.
        __device__ __forceinline__ uint32_t PlanDivisionOutOfRange(double n)
        {
            const uint32_t hi = static_cast<uint32_t>(__double2hiint(n));
            const uint32_t e = (hi >> 20) & 0x7ffu;
            const bool plusZero = (hi | static_cast<uint32_t>(__double2loint(n))) == 0u;
            return ((e - 123u) > (1922u - 123u) && !plusZero) ? 1u : 0u;
        }

        // Right-hand side of one sweep at every cell (i, line) of lines laid
        // out v[i * lines + line], one thread per cell: for the x-sweep
        // ExplicitDiffusionY2ADI (ADIequations.h:316-324, Dirichlet :351-362),
        // for the y-sweep ExplicitDiffusionX2ADI (ADIequations.h:325-336,
        // Dirichlet :363-377) -- the cell plus half the rate times its two
        // cross-axis differences, to line + 1 then line - 1 -- plus, with a
        // ghost table, ImplicitBoundarySource along the line.  crossGhost[L +
        // i] / crossGhost[i] are the ghosts beyond line lines-1 / line 0 of
        // row i; alongLo[line] / alongLo[lines + line] those before element 0
        // / after element L-1 of a line (null: zero-flux).
        __global__ void AdiRhs64(const double *__restrict__ v, double *__restrict__ rhs, int32_t L, int32_t lines,
                                 int32_t wrapCross, int32_t wrapAlong, const double *__restrict__ crossGhost,
                                 const double *__restrict__ alongLo, double r)
        {
            const int32_t line = blockIdx.x * blockDim.x + threadIdx.x;
            if (line >= lines)
            {
                return;
            }
            for (int32_t i = blockIdx.y; i < L; i += gridDim.y)
            {
                const int64_t row = static_cast<int64_t>(i) * lines;
                const double c = v[row + line];
                double s = HalfStep(c, CrossDelta(v, c, line + 1, lines, wrapCross != 0, row, 1, crossGhost, L + i),
                                    CrossDelta(v, c, line - 1, lines, wrapCross != 0, row, 1, crossGhost, i), r);
                if (alongLo != nullptr)
                {
                    s = __dadd_rn(s, ImplicitSource(i, L, wrapAlong != 0, r, alongLo[line], alongLo[lines + line]));
                }
                rhs[row + line] = s;
            }
        }

        constexpr int kChainFwd = 16;  // elements loaded ahead in the elimination
        constexpr int kChainBwd = 8;   // ... and in the back substitution

        // Thomas solve of one line per thread, TdmaSolver::TDMA
        // (TdmaSolver.h:26-66) in its operations and order, over the
        // right-hand sides in d (element i of a line at d[i * lines + line]):
        // elimination in place, d[i] = d[i] - ws[i] * d[i - 1], then back
        // substitution x[i] = (d[i] - off * x[i + 1]) / bs[i] into out.
        // A warp's FP64 instruction costs tens of cycles on this part however
        // many lanes it runs, and a line is one dependent chain, so the chain
        // is all a thread does: AdiRhs64 computes the right-hand sides, the
        // transposes apply the periodic correction, each loop loads the next
        // batch of elements while it works on the current one, and the
        // divisions use the plan's reciprocals (DivByPlan, FAST).  A periodic
        // line (TDMAperiodic, TdmaSolver.h:96-119) leaves its factor (y0 +
        // yL * vEnd) / (1 + vz) in factor[line].
        template <bool FAST>
        __global__ void __launch_bounds__(32) AdiChain64(double *__restrict__ d, double *__restrict__ out,
                                                          LinePlan64Dev pl, int32_t lines,
                                                          double *__restrict__ factor)
        {
            const int32_t line = blockIdx.x * blockDim.x + threadIdx.x;
            if (line >= lines)
            {
                return;
            }
            const int32_t L = pl.L;
            auto at = [&](int32_t i) { return static_cast<int64_t>(i) * lines + line; };

            double rc[kChainFwd], wc[kChainFwd];
#pragma unroll
            for (int k = 0; k < kChainFwd; k++)
            {
                const int32_t i = min(k, L - 1);
                rc[k] = __ldcg(d + at(i));
                wc[k] = __ldg(pl.ws + i);
            }
            double prev = 0.0;
            for (int32_t i0 = 0; i0 < L; i0 += kChainFwd)
            {
                double rn[kChainFwd], wn[kChainFwd];
#pragma unroll
                for (int k = 0; k < kChainFwd; k++)
                {
                    const int32_t i = min(i0 + kChainFwd + k, L - 1);
                    rn[k] = __ldcg(d + at(i));
                    wn[k] = __ldg(pl.ws + i);
                }
#pragma unroll
                for (int k = 0; k < kChainFwd; k++)
                {
                    const int32_t i = i0 + k;
                    if (i < L)
                    {
                        prev = (i == 0) ? rc[k] : __dsub_rn(rc[k], __dmul_rn(wc[k], prev));
                        d[at(i)] = prev;
                    }
                }
#pragma unroll
                for (int k = 0; k < kChainFwd; k++)
                {
                    rc[k] = rn[k];
                    wc[k] = wn[k];
                }
            }

            // FAST: a numerator outside DivByPlan's range is only recorded
            // here, and the line is solved again with IEEE divisions below
            // (a test in the loop would put its branch on the chain)
            uint32_t redo = 0;
            double x = FAST ? DivByPlan(prev, pl.bh[L - 1], pl.lo[L - 1]) : __ddiv_rn(prev, pl.bs[L - 1]);
            if (FAST)
            {
                redo |= PlanDivisionOutOfRange(prev);
            }
            out[at(L - 1)] = x;
            double xLast = x;
            double dc[kChainBwd];
            double2 bc[kChainBwd];
            int2 lc[kChainBwd];
#pragma unroll
            for (int k = 0; k < kChainBwd; k++)
            {
                const int32_t i = max(L - 2 - k, 0);
                dc[k] = __ldcg(d + at(i));
                bc[k] = FAST ? __ldg(pl.bh + i) : make_double2(__ldg(pl.bs + i), 0.0);
                lc[k] = FAST ? __ldg(pl.lo + i) : make_int2(0, 0);
            }
            for (int32_t i0 = L - 2; i0 >= 0; i0 -= kChainBwd)
            {
                double dn[kChainBwd];
                double2 bn[kChainBwd];
                int2 ln[kChainBwd];
#pragma unroll
                for (int k = 0; k < kChainBwd; k++)
                {
                    const int32_t i = max(i0 - kChainBwd - k, 0);
                    dn[k] = __ldcg(d + at(i));
                    bn[k] = FAST ? __ldg(pl.bh + i) : make_double2(__ldg(pl.bs + i), 0.0);
                    ln[k] = FAST ? __ldg(pl.lo + i) : make_int2(0, 0);
                }
#pragma unroll
                for (int k = 0; k < kChainBwd; k++)
                {
                    const int32_t i = i0 - k;
                    if (i >= 0)
                    {
                        const double num = __dsub_rn(dc[k], __dmul_rn(pl.off, x));
                        x = FAST ? DivByPlan(num, bc[k], lc[k]) : __ddiv_rn(num, bc[k].x);
                        if (FAST)
                        {
                            redo |= PlanDivisionOutOfRange(num);
                        }
                        out[at(i)] = x;
                    }
                }
#pragma unroll
                for (int k = 0; k < kChainBwd; k++)
                {
                    dc[k] = dn[k];
                    bc[k] = bn[k];
                    lc[k] = ln[k];
                }
            }
            if (FAST && redo != 0)
            {
                x = __ddiv_rn(prev, pl.bs[L - 1]);
                out[at(L - 1)] = x;
                xLast = x;
                for (int32_t i = L - 2; i >= 0; i--)
                {
                    x = __ddiv_rn(__dsub_rn(__ldcg(d + at(i)), __dmul_rn(pl.off, x)), pl.bs[i]);
                    out[at(i)] = x;
                }
            }
            if (pl.periodic)
            {
                // x is now y0 (element 0), xLast yL (element L - 1)
                const double vy = __dadd_rn(x, __dmul_rn(xLast, pl.vEnd));
                factor[line] = __ddiv_rn(vy, pl.onePlusVz);
            }
        }

        // The sweeps' division (DivByPlan, or __ddiv_rn where
        // PlanDivisionOutOfRange says so) against __ddiv_rn for every num[i]
        // and divisor j (bh[j], lo[j]: its plan entries); the count of
        // differing bit patterns goes to *bad.
        __global__ void CheckPlanDivision(const double *__restrict__ num, int64_t nNum, const double2 *__restrict__ bh,
                                          const int2 *__restrict__ lo, int32_t nDen, unsigned long long *bad)
        {
            for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nNum;
                 i += static_cast<int64_t>(gridDim.x) * blockDim.x)
            {
                const double n = num[i];
                unsigned long long c = 0;
                for (int32_t j = 0; j < nDen; j++)
                {
                    const double a = __ddiv_rn(n, bh[j].x);
                    const double b = PlanDivisionOutOfRange(n) ? __ddiv_rn(n, bh[j].x) : DivByPlan(n, bh[j], lo[j]);
                    c += (__double_as_longlong(a) != __double_as_longlong(b)) ? 1ull : 0ull;
                }
                if (c != 0)
                {
                    atomicAdd(bad, c);
                }
            }
        }

        // Tiled transpose of a rows x cols FP64 array: out[c * rows + r] =
        // in[r * cols + c].  With deltas, instead deltas[c * rows + r] +=
        // in[r * cols + c] - f[c * rows + r] (the y-sweep's commit into the
        // deltas, ADIequations.h:331-335).  With fac, each input first takes
        // the periodic correction of its line c at element r, in - fac[c] *
        // zs[r] (TDMAperiodic's ys - factor * zs, TdmaSolver.h:115-118).
        template <bool COMMIT>
        __global__ void Transpose64(const double *__restrict__ in, double *__restrict__ out, int32_t rows,
                                    int32_t cols, const double *__restrict__ f, const double *__restrict__ fac,
                                    const double *__restrict__ zs)
        {
            __shared__ double tile[32][33];
            const int32_t c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
            for (int j = threadIdx.y; j < 32; j += blockDim.y)
            {
                const int32_t r = r0 + j, c = c0 + threadIdx.x;
                if (r < rows && c < cols)
                {
                    double v = in[static_cast<int64_t>(r) * cols + c];
                    if (fac != nullptr)
                    {
                        v = __dsub_rn(v, __dmul_rn(fac[c], zs[r]));
                    }
                    tile[j][threadIdx.x] = v;
                }
            }
            __syncthreads();
            for (int j = threadIdx.y; j < 32; j += blockDim.y)
            {
                const int32_t c = c0 + j, r = r0 + threadIdx.x;
                if (r < rows && c < cols)
                {
                    const int64_t o = static_cast<int64_t>(c) * rows + r;
                    if constexpr (COMMIT)
                    {
                        out[o] = __dadd_rn(out[o], __dsub_rn(tile[threadIdx.x][j], f[o]));
                    }
                    else
                    {
                        out[o] = tile[threadIdx.x][j];
                    }
                }
            }
        }

        inline unsigned Blocks(int64_t n, int t)
        {
            const int64_t b = (n + t - 1) / t;
            return static_cast<unsigned>(b < 1 ? 1 : (b > 2147483647 ? 2147483647 : b));
        }

        inline unsigned StrideBlocks(int64_t n)
        {
            return static_cast<unsigned>(std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 152 * 16));
        }

        // ---- host side of the ADI plan -------------------------------------
        // TdmaSolver::TDMA's elimination (TdmaSolver.h:26-66) applied to the
        // coefficients alone, in its operations: bs[i] = b_i - ws[i] * c,
        // ws[i] = a / bs[i - 1], with ADISolveRow's coefficients
        // (ADIequations.h:225-270): off-diagonal -r/2; diagonal 1 - w * off,
        // w = 2 plus endAdjust (+1 Dirichlet, -1 zero-flux) at each end; on a
        // wrapped axis TDMAperiodic's adjusted ends (TdmaSolver.h:68-95).
        // This file is compiled without floating-point contraction on the
        // host, so each operation rounds as the reference's does.
        struct LinePlan64Host
        {
            std::vector<double> ws, bs, zs;
            std::vector<double2> bh;
            std::vector<int2> lo;
            double off = 0, vEnd = 0, onePlusVz = 0;
            bool periodic = false;
            bool fastDiv = false;
        };

        // DivByPlan's entries for the divisor b: (b, hi) with hi = RN(1/b),
        // and lo = RN(1/b - hi) as an FP32 mantissa in +-[1, 2) (its bits)
        // and an exponent; 1 - b*hi is exact under an FMA, so lo = RN((1 -
        // b*hi) / b).  A lo below 2^-200 |hi| counts as 0 (its product with
        // any n is far below half an ulp of n/b).
        void PlanReciprocal(double b, double2 *bh, int2 *lo)
        {
            const double hi = 1.0 / b;
            const double l = std::fma(-b, hi, 1.0) / b;
            *bh = make_double2(b, hi);
            *lo = make_int2(0, -4096);
            if (l != 0.0 && std::fabs(l) >= std::ldexp(std::fabs(hi), -200))
            {
                int e = 0;
                const double fr = std::frexp(l, &e);  // l = fr * 2^e, |fr| in [0.5, 1)
                const float m = static_cast<float>(fr * 2.0);
                int32_t bits = 0;
                std::memcpy(&bits, &m, sizeof(bits));
                *lo = make_int2(bits, e - 1);
            }
        }

        // b in [2^-20, 2^20], where DivByPlan is exact for every n that
        // PlanDivisionOutOfRange accepts (the matrices of a diffusion rate
        // r >= 0 have diagonals of at least 1).
        bool PlanDivisorInRange(double b)
        {
            return b >= 0x1p-20 && b <= 0x1p20;
        }

        // Reciprocals of the modified diagonal and whether DivByPlan may
        // replace the back substitution's divisions.
        void AddReciprocals(LinePlan64Host &p)
        {
            const size_t n = p.bs.size();
            p.bh.assign(n, make_double2(0.0, 0.0));
            p.lo.assign(n, make_int2(0, 0));
            p.fastDiv = true;
            for (size_t i = 0; i < n; i++)
            {
                p.fastDiv = p.fastDiv && PlanDivisorInRange(p.bs[i]);
            }
            for (size_t i = 0; p.fastDiv && i < n; i++)
            {
                PlanReciprocal(p.bs[i], &p.bh[i], &p.lo[i]);
            }
        }

        struct PlanCoeffs
        {
            double off;
            double endAdjust;
            bool periodic, adjusted;
            double gamma, alpha, beta;
            int32_t len;

            double BRaw(int32_t i) const
            {
                if (periodic)
                {
                    return 1 - 2 * off;
                }
                double weight = 2.0;
                if (i == 0)
                {
                    weight += endAdjust;
                }
                if (i == len - 1)
                {
                    weight += endAdjust;
                }
                return 1 - weight * off;
            }

            double B(int32_t i) const
            {
                if (adjusted)
                {
                    if (i == 0)
                    {
                        return BRaw(i) - gamma;
                    }
                    if (i == len - 1)
                    {
                        return BRaw(i) - (alpha * beta) / gamma;
                    }
                }
                return BRaw(i);
            }
        };

        // The elimination's coefficients (ws, bs) of a matrix.
        void Eliminate(const PlanCoeffs &k, std::vector<double> &ws, std::vector<double> &bs)
        {
            const int32_t n = k.len;
            ws.assign(static_cast<size_t>(n), 0.0);
            bs.assign(static_cast<size_t>(n), 0.0);
            bs[0] = k.B(0);
            for (int32_t i = 1; i < n; i++)
            {
                bs[i] = k.B(i);
                ws[i] = k.off / bs[i - 1];
                bs[i] = bs[i] - ws[i] * k.off;
            }
        }

        // TDMA of one right-hand side with given coefficients (host).
        void SolveHost(const PlanCoeffs &k, const std::vector<double> &ws, const std::vector<double> &bs,
                       const std::vector<double> &rhs, std::vector<double> &out)
        {
            const int32_t n = k.len;
            std::vector<double> ds(rhs);
            for (int32_t i = 1; i < n; i++)
            {
                ds[i] = ds[i] - ws[i] * ds[i - 1];
            }
            out.assign(static_cast<size_t>(n), 0.0);
            double x = ds[n - 1] / bs[n - 1];
            out[n - 1] = x;
            for (int32_t i = n - 2; i >= 0; i--)
            {
                x = (ds[i] - k.off * x) / bs[i];
                out[i] = x;
            }
        }

        LinePlan64Host BuildPlan64(int32_t len, double r, bool wrap, bool dirichlet)
        {
            LinePlan64Host p;
            PlanCoeffs k{};
            k.off = -r / 2.0;
            k.len = len;
            p.off = k.off;
            if (wrap)
            {
                k.periodic = true;
                const double gamma = -k.B(0);
                k.gamma = gamma;
                k.alpha = k.off;
                k.beta = k.off;
                k.adjusted = true;
                Eliminate(k, p.ws, p.bs);
                std::vector<double> us(static_cast<size_t>(len), 0.0);
                for (int32_t i = 0; i < len; i++)
                {
                    us[i] = (i == 0) ? gamma : ((i == len - 1) ? k.alpha : 0.0);
                }
                SolveHost(k, p.ws, p.bs, us, p.zs);
                p.vEnd = k.beta / gamma;
                const double vz = p.zs[0] + p.zs[len - 1] * p.vEnd;
                p.onePlusVz = 1 + vz;
                p.periodic = true;
                AddReciprocals(p);
                return p;
            }
            k.endAdjust = dirichlet ? 1.0 : -1.0;
            Eliminate(k, p.ws, p.bs);
            p.zs.assign(static_cast<size_t>(len), 0.0);
            AddReciprocals(p);
            return p;
        }

        struct PlanBuf64
        {
            DevBuf<double> buf;  // ws, bs, zs
            LinePlan64Dev dev;
        };
    }

    struct PdeGrid
    {
        int32_t xDim = 0, yDim = 0;
        int32_t wrapX = 0, wrapY = 0;
        int32_t updateCt = 0;
        // a value-form *All call not yet run (see Prepare)
        bool pendingAll = false;
        int32_t pendingOp = 0;
        double pendingValue = 0.0;
        int device = 0;
        StreamSlot stream;
        DevBuf<double> f, d;
        Adi64 adi64;                     // DiffusionADI (plans and scratch)
        DevBuf<double> a0, a1, a2;       // uploaded per-cell arrays (rates, velocities)
        DevBuf<double> g0, g1, g2;       // uploaded ghost tables
        DevBuf<RedPartial> red;
        HostBuf<RedPartial> redHost;
        DevBuf<int32_t> ic0, ic1;        // uploaded index lists
        DevBuf<int8_t> iops;
        DevBuf<double> ivals, iout, iout2;
        cudaEvent_t evA = nullptr, evB = nullptr;

        int64_t Length() const
        {
            return static_cast<int64_t>(xDim) * yDim;
        }

        int Init(int32_t x, int32_t y, int32_t wx, int32_t wy)
        {
            xDim = x;
            yDim = y;
            wrapX = wx;
            wrapY = wy;
            device = CurrentDevice();
            HAL_TRY(CudaStatus(cudaSetDevice(device), "cudaSetDevice"));
            HAL_TRY(stream.Create("cudaStreamCreate"));
            HAL_TRY(f.Alloc(static_cast<size_t>(Length()), "cudaMalloc(pdegrid field)"));
            HAL_TRY(d.Alloc(static_cast<size_t>(Length()), "cudaMalloc(pdegrid deltas)"));
            HAL_TRY(CudaStatus(cudaMemset(f.p, 0, static_cast<size_t>(Length()) * sizeof(double)), "cudaMemset"));
            HAL_TRY(CudaStatus(cudaMemset(d.p, 0, static_cast<size_t>(Length()) * sizeof(double)), "cudaMemset"));
            HAL_TRY(red.Alloc(kRedBlocks, "cudaMalloc(reduction)"));
            HAL_TRY(redHost.Reserve(kRedBlocks, "cudaMallocHost(reduction)"));
            HAL_TRY(CudaStatus(cudaEventCreateWithFlags(&evA, cudaEventDisableTiming), "cudaEventCreate"));
            HAL_TRY(CudaStatus(cudaEventCreateWithFlags(&evB, cudaEventDisableTiming), "cudaEventCreate"));
            return HAL_CUDA_OK;
        }

        ~PdeGrid()
        {
            if (evA != nullptr)
            {
                cudaEventDestroy(evA);
            }
            if (evB != nullptr)
            {
                cudaEventDestroy(evB);
            }
        }

        // Copies n values of host array h into device buffer b (grown to
        // at least n), on the handle's stream.
        template <typename T>
        int Upload(DevBuf<T> &b, const T *h, size_t n, const char *what)
        {
            if (b.n < n || b.p == nullptr)
            {
                HAL_TRY(CudaStatus(cudaStreamSynchronize(stream.Get()), what));
                HAL_TRY(b.Alloc(n, what));
            }
            if (n > 0)
            {
                HAL_TRY(CudaStatus(cudaMemcpyAsync(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice, stream.Get()),
                                   what));
            }
            return HAL_CUDA_OK;
        }

        template <typename T>
        int Ensure(DevBuf<T> &b, size_t n, const char *what)
        {
            if (b.n < n || b.p == nullptr)
            {
                HAL_TRY(CudaStatus(cudaStreamSynchronize(stream.Get()), what));
                HAL_TRY(b.Alloc(n, what));
            }
            return HAL_CUDA_OK;
        }

        int GhostTable(const double *ghost, DevBuf<double> &buf, const double **out)
        {
            *out = nullptr;
            if (ghost != nullptr)
            {
                HAL_TRY(Upload(buf, ghost, 2 * (static_cast<size_t>(xDim) + yDim), "cudaMemcpy(ghost)"));
                *out = buf.p;
            }
            return HAL_CUDA_OK;
        }

        // Internal::Diffusion2DADI (ADIequations.h:306-337, Dirichlet
        // :339-378): deltas += v - f.
        int Adi(double r, const double *ghostHost)
        {
            const double *g = nullptr;
            HAL_TRY(GhostTable(ghostHost, g0, &g));
            return adi64.Run(f.p, d.p, xDim, yDim, wrapX, wrapY, r, g, stream.Get());
        }

        int Sync(const char *who)
        {
            return CudaStatus(cudaStreamSynchronize(stream.Get()), who);
        }
    };

    // ---- Adi64 -------------------------------------------------------------
    struct Adi64::Impl
    {
        DevBuf<double> wA, wB, vB, dS;  // scratch (grown on first use)
        DevBuf<double> fac;             // periodic factors of the current sweep's lines
        std::map<std::string, std::unique_ptr<PlanBuf64>> plans;

        int Ensure(DevBuf<double> &b, size_t n, cudaStream_t s, const char *what)
        {
            if (b.n < n || b.p == nullptr)
            {
                HAL_TRY(CudaStatus(cudaStreamSynchronize(s), what));
                HAL_TRY(b.Alloc(n, what));
            }
            return HAL_CUDA_OK;
        }

        int Plan(int32_t L, double r, bool wrap, bool dirichlet, LinePlan64Dev *out)
        {
            char key[96];
            snprintf(key, sizeof(key), "%d|%a|%d|%d", L, r, wrap ? 1 : 0, (dirichlet && !wrap) ? 1 : 0);
            auto it = plans.find(key);
            if (it == plans.end())
            {
                const LinePlan64Host h = BuildPlan64(L, r, wrap, dirichlet);
                auto pb = std::make_unique<PlanBuf64>();
                // layout (in doubles): bh [2L], lo [L], ws [L], bs [L], zs [L]
                const size_t Ls = static_cast<size_t>(L);
                std::vector<double> all(6 * Ls, 0.0);
                std::memcpy(all.data(), h.bh.data(), sizeof(double2) * Ls);
                std::memcpy(all.data() + 2 * Ls, h.lo.data(), sizeof(int2) * Ls);
                std::copy(h.ws.begin(), h.ws.end(), all.begin() + 3 * Ls);
                std::copy(h.bs.begin(), h.bs.end(), all.begin() + 4 * Ls);
                std::copy(h.zs.begin(), h.zs.end(), all.begin() + 5 * Ls);
                HAL_TRY(pb->buf.Alloc(all.size(), "cudaMalloc(ADI plan)"));
                HAL_TRY(CudaStatus(cudaMemcpy(pb->buf.p, all.data(), all.size() * sizeof(double),
                                              cudaMemcpyHostToDevice),
                                   "cudaMemcpy(ADI plan)"));
                pb->dev.bh = reinterpret_cast<const double2 *>(pb->buf.p);
                pb->dev.lo = reinterpret_cast<const int2 *>(pb->buf.p + 2 * Ls);
                pb->dev.ws = pb->buf.p + 3 * Ls;
                pb->dev.bs = pb->buf.p + 4 * Ls;
                pb->dev.zs = pb->buf.p + 5 * Ls;
                pb->dev.fastDiv = h.fastDiv ? 1 : 0;
                pb->dev.off = h.off;
                pb->dev.vEnd = h.vEnd;
                pb->dev.onePlusVz = h.onePlusVz;
                pb->dev.L = L;
                pb->dev.periodic = h.periodic ? 1 : 0;
                it = plans.emplace(key, std::move(pb)).first;
            }
            *out = it->second->dev;
            return HAL_CUDA_OK;
        }
    };

    Adi64::Adi64() : m_impl(new Impl())
    {
    }

    Adi64::~Adi64() = default;

    int Adi64::Run(const double *f, double *deltas, int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY,
                   double r, const double *g, cudaStream_t s)
    {
        Impl &m = *m_impl;
        const size_t n = static_cast<size_t>(xDim) * static_cast<size_t>(yDim);
        HAL_TRY(m.Ensure(m.wA, n, s, "cudaMalloc(ADI scratch)"));
        HAL_TRY(m.Ensure(m.wB, n, s, "cudaMalloc(ADI scratch)"));
        HAL_TRY(m.Ensure(m.vB, n, s, "cudaMalloc(ADI scratch)"));
        HAL_TRY(m.Ensure(m.dS, n, s, "cudaMalloc(ADI scratch)"));
        LinePlan64Dev px, py;
        HAL_TRY(m.Plan(xDim, r, wrapX != 0, g != nullptr, &px));
        HAL_TRY(m.Plan(yDim, r, wrapY != 0, g != nullptr, &py));
        // per sweep: the right-hand sides on every SM, the chains one line
        // per thread and one warp per block (the lines spread over the most
        // SMs), then the transpose that applies the periodic correction
        const size_t nFac = static_cast<size_t>(std::max(xDim, yDim));
        HAL_TRY(m.Ensure(m.fac, nFac, s, "cudaMalloc(ADI scratch)"));
        const int T = 32;
        const dim3 tb(32, 8);
        const auto rhsGrid = [](int32_t lines, int32_t L) {
            return dim3(Blocks(lines, 256), static_cast<unsigned>(std::min<int32_t>(std::max<int32_t>(L, 1), 65535)));
        };
        const auto chain = [&](const LinePlan64Dev &pl, int32_t lines, double *out) {
            if (pl.fastDiv)
            {
                AdiChain64<true><<<Blocks(lines, T), T, 0, s>>>(m.dS.p, out, pl, lines, m.fac.p);
            }
            else
            {
                AdiChain64<false><<<Blocks(lines, T), T, 0, s>>>(m.dS.p, out, pl, lines, m.fac.p);
            }
        };
        AdiRhs64<<<rhsGrid(yDim, xDim), 256, 0, s>>>(f, m.dS.p, xDim, yDim, wrapY, wrapX,
                                                        g ? g + 2 * static_cast<size_t>(yDim) : nullptr, g, r);
        chain(px, yDim, m.wA.p);
        Transpose64<false><<<dim3((yDim + 31) / 32, (xDim + 31) / 32), tb, 0, s>>>(
            m.wA.p, m.wB.p, xDim, yDim, nullptr, px.periodic ? m.fac.p : nullptr, px.zs);
        AdiRhs64<<<rhsGrid(xDim, yDim), 256, 0, s>>>(m.wB.p, m.dS.p, yDim, xDim, wrapX, wrapY, g,
                                                        g ? g + 2 * static_cast<size_t>(yDim) : nullptr, r);
        chain(py, xDim, m.vB.p);
        Transpose64<true><<<dim3((xDim + 31) / 32, (yDim + 31) / 32), tb, 0, s>>>(
            m.vB.p, deltas, yDim, xDim, f, py.periodic ? m.fac.p : nullptr, py.zs);
        CountLaunch(6);
        return LaunchStatus("DiffusionADI (FP64)");
    }
}

struct hal_cuda_pdegrid : public halcuda::PdeGrid
{
};

namespace
{
    using halcuda::CudaStatus;
    using halcuda::LaunchStatus;

    // Every entry point starts here.  A pending value-form *All call
    // (hal_cuda_pdegrid_apply_all) runs first, unless the caller is the
    // Update that takes it over (flush false).
    int Prepare(hal_cuda_pdegrid *h, const char *who, bool flush = true)
    {
        HAL_REQUIRE(h != nullptr, "%s: handle is NULL", who);
        HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
        if (flush && h->pendingAll)
        {
            h->pendingAll = false;
            const int64_t n = h->Length();
            halcuda::ApplyAll<<<halcuda::StrideBlocks(n), 256, 0, h->stream.Get()>>>(
                h->pendingOp, h->pendingValue, nullptr, n, h->f.p, h->d.p);
            halcuda::CountLaunch();
            HAL_TRY(LaunchStatus(who));
        }
        return HAL_CUDA_OK;
    }
}

extern "C" int hal_cuda_pdegrid_create(int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY,
                                       hal_cuda_pdegrid **out)
{
    HAL_REQUIRE(out != nullptr, "hal_cuda_pdegrid_create: out is NULL");
    *out = nullptr;
    HAL_REQUIRE(xDim > 0 && yDim > 0, "hal_cuda_pdegrid_create: dimensions must be positive");
    HAL_REQUIRE(static_cast<int64_t>(xDim) * yDim <= INT32_MAX,
                "hal_cuda_pdegrid_create: xDim*yDim exceeds int32 (PDEGrid2D indexes cells with int32_t)");
    hal_cuda_pdegrid *h = new (std::nothrow) hal_cuda_pdegrid();
    if (h == nullptr)
    {
        halcuda::SetError("hal_cuda_pdegrid_create: out of host memory");
        return HAL_CUDA_ENOMEM;
    }
    const int rc = h->Init(xDim, yDim, wrapX != 0, wrapY != 0);
    if (rc != HAL_CUDA_OK)
    {
        delete h;
        return rc;
    }
    *out = h;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_pdegrid_destroy(hal_cuda_pdegrid *h)
{
    if (h != nullptr)
    {
        cudaSetDevice(h->device);
        cudaStreamSynchronize(h->stream.Get());
        delete h;
    }
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_pdegrid_set_state(hal_cuda_pdegrid *h, const double *field, const double *deltas,
                                          int32_t updateCt)
{
    HAL_TRY(Prepare(h, "hal_cuda_pdegrid_set_state"));
    HAL_REQUIRE(field != nullptr, "PDEGrid::SetState arrays must match the grid length");
    cudaStream_t s = h->stream.Get();
    const size_t bytes = static_cast<size_t>(h->Length()) * sizeof(double);
    HAL_TRY(CudaStatus(cudaMemcpyAsync(h->f.p, field, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpy(field)"));
    HAL_TRY(CudaStatus(deltas != nullptr ? cudaMemcpyAsync(h->d.p, deltas, bytes, cudaMemcpyHostToDevice, s)
                                         : cudaMemsetAsync(h->d.p, 0, bytes, s),
                       "cudaMemcpy(deltas)"));
    h->updateCt = updateCt;
    return h->Sync("hal_cuda_pdegrid_set_state");
}

extern "C" int hal_cuda_pdegrid_get_state(hal_cuda_pdegrid *h, double *field, double *deltas, int32_t *updateCt)
{
    HAL_TRY(Prepare(h, "hal_cuda_pdegrid_get_state"));
    cudaStream_t s = h->stream.Get();
    const size_t bytes = static_cast<size_t>(h->Length()) * sizeof(double);
    if (field != nullptr)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(field, h->f.p, bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpy(field)"));
    }
    if (deltas != nullptr)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(deltas, h->d.p, bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpy(deltas)"));
    }
    if (updateCt != nullptr)
    {
        *updateCt = h->updateCt;
    }
    return h->Sync("hal_cuda_pdegrid_get_state");
}

extern "C" int hal_cuda_pdegrid_apply(hal_cuda_pdegrid *h, const int32_t *ops, int32_t op, const int32_t *cells,
                                      const double *values, double value, int64_t n)
{
    const char *who = "hal_cuda_pdegrid_apply";
    HAL_TRY(Prepare(h, who));
    HAL_REQUIRE(n >= 0, "%s: negative count", who);
    if (n == 0)
    {
        return HAL_CUDA_OK;
    }
    HAL_REQUIRE(cells != nullptr, "%s: cells is NULL", who);
    HAL_REQUIRE(ops != nullptr || (op >= HAL_CUDA_CELL_SET && op <= HAL_CUDA_CELL_SCALE), "%s: unknown operation %d",
                who, op);
    const int64_t len = h->Length();
    // stable order by cell: entries of a cell keep their list order
    std::vector<int64_t> order(static_cast<size_t>(n));
    std::iota(order.begin(), order.end(), int64_t(0));
    for (int64_t k = 0; k < n; k++)
    {
        HAL_REQUIRE(cells[k] >= 0 && cells[k] < len, "%s: cell %d outside the grid of %lld cells", who, cells[k],
                    static_cast<long long>(len));
        if (ops != nullptr)
        {
            HAL_REQUIRE(ops[k] >= HAL_CUDA_CELL_SET && ops[k] <= HAL_CUDA_CELL_SCALE, "%s: unknown operation %d", who,
                        ops[k]);
        }
    }
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return cells[a] < cells[b]; });
    std::vector<int32_t> sc(static_cast<size_t>(n));
    std::vector<int8_t> so(static_cast<size_t>(n));
    std::vector<double> sv(static_cast<size_t>(n));
    std::vector<int32_t> runs;
    for (int64_t k = 0; k < n; k++)
    {
        const int64_t e = order[static_cast<size_t>(k)];
        sc[k] = cells[e];
        so[k] = static_cast<int8_t>(ops != nullptr ? ops[e] : op);
        sv[k] = values != nullptr ? values[e] : value;
        if (k == 0 || sc[k] != sc[k - 1])
        {
            runs.push_back(static_cast<int32_t>(k));
        }
    }
    runs.push_back(static_cast<int32_t>(n));
    const int32_t nRuns = static_cast<int32_t>(runs.size()) - 1;
    HAL_TRY(h->Upload(h->ic0, sc.data(), sc.size(), "cudaMemcpy(cells)"));
    HAL_TRY(h->Upload(h->iops, so.data(), so.size(), "cudaMemcpy(ops)"));
    HAL_TRY(h->Upload(h->ivals, sv.data(), sv.size(), "cudaMemcpy(values)"));
    HAL_TRY(h->Upload(h->ic1, runs.data(), runs.size(), "cudaMemcpy(runs)"));
    halcuda::ApplyRuns<<<halcuda::Blocks(nRuns, 256), 256, 0, h->stream.Get()>>>(
        h->ic0.p, h->iops.p, h->ivals.p, h->ic1.p, nRuns, h->f.p, h->d.p);
    halcuda::CountLaunch();
    HAL_TRY(LaunchStatus(who));
    // the host lists are copied out before this call returns
    return h->Sync(who);
}

extern "C" int hal_cuda_pdegrid_apply_agents(hal_cuda_pdegrid *h, hal_cuda_agents *agents, int32_t op, double value,
                                             const double *perAgent)
{
    const char *who = "hal_cuda_pdegrid_apply_agents";
    HAL_TRY(Prepare(h, who));
    HAL_REQUIRE(agents != nullptr, "%s: agents is NULL", who);
    HAL_REQUIRE(op >= HAL_CUDA_CELL_SET && op <= HAL_CUDA_CELL_SCALE, "%s: unknown operation %d", who, op);
    const halcuda::AgentBinsView v = halcuda::AgentsBins(agents);
    HAL_REQUIRE(v.xDim == h->xDim && v.yDim == h->yDim, "%s: agent grid %dx%d differs from the field %dx%d", who,
                v.xDim, v.yDim, h->xDim, h->yDim);
    HAL_REQUIRE(v.device == h->device, "%s: the agents live on another device", who);
    if (v.n == 0)
    {
        return HAL_CUDA_OK;
    }
    cudaStream_t s = h->stream.Get();
    const double *pa = nullptr;
    if (perAgent != nullptr)
    {
        HAL_TRY(h->Upload(h->ivals, perAgent, static_cast<size_t>(v.n), "cudaMemcpy(per-agent values)"));
        pa = h->ivals.p;
    }
    // the agents' last binning completes before, and their next one starts
    // after, this grid's use of it
    HAL_TRY(CudaStatus(cudaEventRecord(h->evA, v.stream), "cudaEventRecord"));
    HAL_TRY(CudaStatus(cudaStreamWaitEvent(s, h->evA, 0), "cudaStreamWaitEvent"));
    halcuda::ApplyAgents<<<halcuda::Blocks(v.n, 256), 256, 0, s>>>(v.offsets, v.bucket, v.cellOf, v.n, op, value, pa,
                                                                   h->f.p, h->d.p);
    halcuda::CountLaunch();
    HAL_TRY(LaunchStatus(who));
    HAL_TRY(CudaStatus(cudaEventRecord(h->evB, s), "cudaEventRecord"));
    HAL_TRY(CudaStatus(cudaStreamWaitEvent(v.stream, h->evB, 0), "cudaStreamWaitEvent"));
    if (perAgent != nullptr)
    {
        return h->Sync(who);  // the host values are read before the call returns
    }
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_pdegrid_apply_all(hal_cuda_pdegrid *h, int32_t op, double value, const double *perCell)
{
    const char *who = "hal_cuda_pdegrid_apply_all";
    HAL_TRY(Prepare(h, who));
    HAL_REQUIRE(op >= HAL_CUDA_CELL_SET && op <= HAL_CUDA_CELL_SCALE, "%s: unknown operation %d", who, op);
    cudaStream_t s = h->stream.Get();
    const int64_t n = h->Length();
    if (perCell == nullptr)
    {
        // deferred: the next call runs it first, and an Update right after
        // it runs it in its own pass (ApplyAllCommit)
        h->pendingAll = true;
        h->pendingOp = op;
        h->pendingValue = value;
        return HAL_CUDA_OK;
    }
    HAL_TRY(h->Upload(h->a0, perCell, static_cast<size_t>(n), "cudaMemcpy(values)"));
    const double *pc = h->a0.p;
    halcuda::ApplyAll<<<halcuda::StrideBlocks(n), 256, 0, s>>>(op, value, pc, n, h->f.p, h->d.p);
    halcuda::CountLaunch();
    HAL_TRY(LaunchStatus(who));
    return h->Sync(who);
}

extern "C" int hal_cuda_pdegrid_update(hal_cuda_pdegrid *h)
{
    HAL_TRY(Prepare(h, "hal_cuda_pdegrid_update", false));
    const int64_t n = h->Length();
    if (h->pendingAll)
    {
        h->pendingAll = false;
        halcuda::ApplyAllCommit<<<halcuda::StrideBlocks(n), 256, 0, h->stream.Get()>>>(
            h->pendingOp, h->pendingValue, n, h->f.p, h->d.p);
    }
    else
    {
        halcuda::Commit<<<halcuda::StrideBlocks(n), 256, 0, h->stream.Get()>>>(n, h->f.p, h->d.p);
    }
    halcuda::CountLaunch();
    h->updateCt++;
    return LaunchStatus("hal_cuda_pdegrid_update");
}

extern "C" int hal_cuda_pdegrid_set_non_negative(hal_cuda_pdegrid *h)
{
    HAL_TRY(Prepare(h, "hal_cuda_pdegrid_set_non_negative"));
    const int64_t n = h->Length();
    halcuda::NonNegative<<<halcuda::StrideBlocks(n), 256, 0, h->stream.Get()>>>(n, h->f.p, h->d.p);
    halcuda::CountLaunch();
    return LaunchStatus("hal_cuda_pdegrid_set_non_negative");
}

extern "C" int hal_cuda_pdegrid_get_cells(hal_cuda_pdegrid *h, const int32_t *cells, int64_t n, double *out)
{
    const char *who = "hal_cuda_pdegrid_get_cells";
    HAL_TRY(Prepare(h, who));
    HAL_REQUIRE(n >= 0 && (n == 0 || (cells != nullptr && out != nullptr)), "%s: NULL array", who);
    if (n == 0)
    {
        return HAL_CUDA_OK;
    }
    const int64_t len = h->Length();
    for (int64_t k = 0; k < n; k++)
    {
        HAL_REQUIRE(cells[k] >= 0 && cells[k] < len, "%s: cell %d outside the grid", who, cells[k]);
    }
    cudaStream_t s = h->stream.Get();
    HAL_TRY(h->Upload(h->ic0, cells, static_cast<size_t>(n), "cudaMemcpy(cells)"));
    HAL_TRY(h->Ensure(h->iout, static_cast<size_t>(n), "cudaMalloc(values)"));
    halcuda::Gather<<<halcuda::Blocks(n, 256), 256, 0, s>>>(h->ic0.p, n, h->f.p, h->iout.p);
    halcuda::CountLaunch();
    HAL_TRY(LaunchStatus(who));
    HAL_TRY(CudaStatus(cudaMemcpyAsync(out, h->iout.p, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDeviceToHost,
                                       s),
                       "cudaMemcpy(values)"));
    return h->Sync(who);
}

extern "C" int hal_cuda_pdegrid_gradient(hal_cuda_pdegrid *h, const int32_t *xs, const int32_t *ys, int64_t n,
                                         int32_t useBoundary, double boundaryValue, double *gradX, double *gradY)
{
    const char *who = "hal_cuda_pdegrid_gradient";
    HAL_TRY(Prepare(h, who));
    HAL_REQUIRE(n >= 0 && (n == 0 || (xs != nullptr && ys != nullptr && gradX != nullptr && gradY != nullptr)),
                "%s: NULL array", who);
    if (n == 0)
    {
        return HAL_CUDA_OK;
    }
    for (int64_t k = 0; k < n; k++)
    {
        HAL_REQUIRE(xs[k] >= 0 && xs[k] < h->xDim && ys[k] >= 0 && ys[k] < h->yDim, "%s: point (%d, %d) outside the grid",
                    who, xs[k], ys[k]);
    }
    cudaStream_t s = h->stream.Get();
    HAL_TRY(h->Upload(h->ic0, xs, static_cast<size_t>(n), "cudaMemcpy(points)"));
    HAL_TRY(h->Upload(h->ic1, ys, static_cast<size_t>(n), "cudaMemcpy(points)"));
    HAL_TRY(h->Ensure(h->iout, static_cast<size_t>(n), "cudaMalloc(gradients)"));
    HAL_TRY(h->Ensure(h->iout2, static_cast<size_t>(n), "cudaMalloc(gradients)"));
    halcuda::Gradients<<<halcuda::Blocks(n, 256), 256, 0, s>>>(h->ic0.p, h->ic1.p, n, h->f.p, h->xDim, h->yDim,
                                                               h->wrapX, h->wrapY, useBoundary, boundaryValue,
                                                               h->iout.p, h->iout2.p);
    halcuda::CountLaunch();
    HAL_TRY(LaunchStatus(who));
    const size_t bytes = static_cast<size_t>(n) * sizeof(double);
    HAL_TRY(CudaStatus(cudaMemcpyAsync(gradX, h->iout.p, bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpy(gradients)"));
    HAL_TRY(CudaStatus(cudaMemcpyAsync(gradY, h->iout2.p, bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpy(gradients)"));
    return h->Sync(who);
}

extern "C" int hal_cuda_pdegrid_stats(hal_cuda_pdegrid *h, double denomOffset, double *stats)
{
    const char *who = "hal_cuda_pdegrid_stats";
    HAL_TRY(Prepare(h, who));
    HAL_REQUIRE(stats != nullptr, "%s: stats is NULL", who);
    cudaStream_t s = h->stream.Get();
    const int64_t n = h->Length();
    const bool scaled = !std::isnan(denomOffset);
    halcuda::Reduce<<<halcuda::kRedBlocks, halcuda::kRedThreads, 0, s>>>(n, h->f.p, h->d.p, denomOffset, scaled,
                                                                         h->red.p);
    halcuda::CountLaunch();
    HAL_TRY(LaunchStatus(who));
    HAL_TRY(CudaStatus(cudaMemcpyAsync(h->redHost.p, h->red.p, halcuda::kRedBlocks * sizeof(halcuda::RedPartial),
                                       cudaMemcpyDeviceToHost, s),
                       "cudaMemcpy(reduction)"));
    HAL_TRY(h->Sync(who));
    // combine the blocks in order (the same rules as within a block)
    double maxV = -INFINITY, minV = INFINITY, sum = 0.0, md = 0.0, ms = 0.0;
    long long maxI = -1, minI = -1;
    for (int b = 0; b < halcuda::kRedBlocks; b++)
    {
        const halcuda::RedPartial &p = h->redHost.p[b];
        if (maxV < p.maxV || (!(p.maxV < maxV) && p.maxI > maxI))
        {
            maxV = p.maxV;
            maxI = p.maxI;
        }
        if (p.minV < minV || (!(minV < p.minV) && p.minI > minI))
        {
            minV = p.minV;
            minI = p.minI;
        }
        sum += p.sum;
        md = std::fmax(md, p.maxDelta);
        ms = std::fmax(ms, p.maxScaled);
    }
    // GetMax / GetMin start from lowest() / max() (PDEGrid2D.h:142-164),
    // which an all -inf (+inf) field never replaces
    const double lowest = -std::numeric_limits<double>::max();
    const double highest = std::numeric_limits<double>::max();
    stats[0] = (maxV < lowest) ? lowest : maxV;
    stats[1] = (highest < minV) ? highest : minV;
    stats[2] = sum / static_cast<double>(n);
    stats[3] = md;
    stats[4] = scaled ? ms : NAN;
    return HAL_CUDA_OK;
}

namespace
{
    // A stencil of stencil64.cuh over the whole grid, into the deltas.
    template <class Cell>
    int RunCells(hal_cuda_pdegrid *h, const Cell &cell, const char *who)
    {
        halcuda::stencil64::Cells64Kernel<<<halcuda::stencil64::Cells64Grid(h->xDim, h->yDim), 256, 0,
                                            h->stream.Get()>>>(cell, h->xDim, h->yDim);
        halcuda::CountLaunch();
        HAL_TRY(LaunchStatus(who));
        // host arrays (rates, velocities, ghost tables) were copied
        // asynchronously from the caller's memory: finish before returning
        return h->Sync(who);
    }

    int SignOf(double v)
    {
        return (v > 0) ? 1 : ((v < 0) ? -1 : 0);
    }
}

extern "C" int hal_cuda_pdegrid_diffusion(hal_cuda_pdegrid *h, double diffCoef, const double *ghost)
{
    const char *who = "hal_cuda_pdegrid_diffusion";
    HAL_TRY(Prepare(h, who));
    HAL_REQUIRE(!(diffCoef > 0.25), "Diffusion rate above stable maximum value of 0.25");
    const double *g = nullptr;
    HAL_TRY(h->GhostTable(ghost, h->g0, &g));
    const halcuda::stencil64::Diffuse64Cell cell{h->f.p, h->d.p, g, diffCoef, h->xDim, h->yDim, h->wrapX, h->wrapY};
    return RunCells(h, cell, who);
}

extern "C" int hal_cuda_pdegrid_diffusion_var(hal_cuda_pdegrid *h, const double *ratesX, const double *ratesY)
{
    const char *who = "hal_cuda_pdegrid_diffusion_var";
    HAL_TRY(Prepare(h, who));
    HAL_REQUIRE(ratesX != nullptr && ratesY != nullptr, "%s: NULL rate array", who);
    const size_t n = static_cast<size_t>(h->Length());
    HAL_TRY(h->Upload(h->a0, ratesX, n, "cudaMemcpy(rates)"));
    HAL_TRY(h->Upload(h->a1, ratesY, n, "cudaMemcpy(rates)"));
    const halcuda::stencil64::DiffuseVar64Cell cell{h->f.p, h->d.p, h->a0.p, h->a1.p, h->xDim, h->yDim, h->wrapX,
                                                    h->wrapY};
    return RunCells(h, cell, who);
}

extern "C" int hal_cuda_pdegrid_diffusion_adi(hal_cuda_pdegrid *h, double diffRate, const double *ghost)
{
    const char *who = "hal_cuda_pdegrid_diffusion_adi";
    HAL_TRY(Prepare(h, who));
    HAL_TRY(h->Adi(diffRate, ghost));
    return ghost != nullptr ? h->Sync(who) : HAL_CUDA_OK;
}

extern "C" int hal_cuda_pdegrid_advection(hal_cuda_pdegrid *h, double xVel, double yVel, const double *ghost)
{
    const char *who = "hal_cuda_pdegrid_advection";
    HAL_TRY(Prepare(h, who));
    HAL_REQUIRE(!((std::fabs(xVel) + std::fabs(yVel)) > 0.5),
                "Advection rate component sum above stable maximum value of 0.5");
    const double *g = nullptr;
    HAL_TRY(h->GhostTable(ghost, h->g0, &g));
    const halcuda::stencil64::Advect64Cell cell{h->f.p, h->d.p, g, xVel, yVel, h->xDim, h->yDim, h->wrapX, h->wrapY,
                                                SignOf(xVel), SignOf(yVel)};
    return RunCells(h, cell, who);
}

extern "C" int hal_cuda_pdegrid_advection_var(hal_cuda_pdegrid *h, const double *xVels, const double *yVels,
                                              const double *ghost, const double *ghostXVel, const double *ghostYVel)
{
    const char *who = "hal_cuda_pdegrid_advection_var";
    HAL_TRY(Prepare(h, who));
    HAL_REQUIRE(xVels != nullptr && yVels != nullptr, "%s: NULL velocity array", who);
    const size_t n = static_cast<size_t>(h->Length());
    HAL_TRY(h->Upload(h->a0, xVels, n, "cudaMemcpy(velocities)"));
    HAL_TRY(h->Upload(h->a1, yVels, n, "cudaMemcpy(velocities)"));
    const double *g = nullptr, *gx = nullptr, *gy = nullptr;
    HAL_TRY(h->GhostTable(ghost, h->g0, &g));
    HAL_TRY(h->GhostTable(ghostXVel, h->g1, &gx));
    HAL_TRY(h->GhostTable(ghostYVel, h->g2, &gy));
    const halcuda::stencil64::AdvectVar64Cell cell{h->f.p, h->d.p, h->a0.p, h->a1.p, g, gx, gy,
                                                   h->xDim, h->yDim, h->wrapX, h->wrapY};
    return RunCells(h, cell, who);
}

extern "C" int hal_cuda_pdegrid_sync(hal_cuda_pdegrid *h)
{
    HAL_TRY(Prepare(h, "hal_cuda_pdegrid_sync"));
    return h->Sync("hal_cuda_pdegrid_sync");
}

extern "C" void *hal_cuda_pdegrid_stream(hal_cuda_pdegrid *h)
{
    return h ? static_cast<void *>(h->stream.Get()) : nullptr;
}

extern "C" int hal_cuda_pdegrid_set_stream(hal_cuda_pdegrid *h, void *stream)
{
    HAL_TRY(Prepare(h, "hal_cuda_pdegrid_set_stream"));  // a pending *All runs on the old stream
    h->stream.Set(stream);
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_pdegrid_dims(hal_cuda_pdegrid *h, int32_t *dims)
{
    HAL_REQUIRE(h != nullptr && dims != nullptr, "hal_cuda_pdegrid_dims: NULL argument");
    dims[0] = h->xDim;
    dims[1] = h->yDim;
    dims[2] = h->wrapX;
    dims[3] = h->wrapY;
    dims[4] = h->updateCt;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_check_plan_division(const double *num, int64_t nNum, const double *den, int32_t nDen,
                                            int64_t *mismatches)
{
    using namespace halcuda;
    HAL_REQUIRE(num != nullptr && den != nullptr && mismatches != nullptr,
                "hal_cuda_check_plan_division: NULL argument");
    HAL_REQUIRE(nNum >= 0 && nDen >= 0, "hal_cuda_check_plan_division: negative count");
    std::vector<double2> bh(static_cast<size_t>(nDen));
    std::vector<int2> lo(static_cast<size_t>(nDen));
    for (int32_t j = 0; j < nDen; j++)
    {
        HAL_REQUIRE(PlanDivisorInRange(den[j]),
                    "hal_cuda_check_plan_division: divisor %d (%g) outside [2^-20, 2^20]", j, den[j]);
        PlanReciprocal(den[j], &bh[j], &lo[j]);
    }
    HAL_TRY(CudaStatus(cudaSetDevice(CurrentDevice()), "cudaSetDevice"));
    DevBuf<double> dNum;
    DevBuf<double2> dBh;
    DevBuf<int2> dLo;
    DevBuf<unsigned long long> dBad;
    HAL_TRY(dNum.Alloc(static_cast<size_t>(std::max<int64_t>(nNum, 1)), "cudaMalloc(division check)"));
    HAL_TRY(dBh.Alloc(static_cast<size_t>(std::max<int32_t>(nDen, 1)), "cudaMalloc(division check)"));
    HAL_TRY(dLo.Alloc(static_cast<size_t>(std::max<int32_t>(nDen, 1)), "cudaMalloc(division check)"));
    HAL_TRY(dBad.Alloc(1, "cudaMalloc(division check)"));
    HAL_TRY(CudaStatus(cudaMemcpy(dNum.p, num, sizeof(double) * nNum, cudaMemcpyHostToDevice), "cudaMemcpy"));
    HAL_TRY(CudaStatus(cudaMemcpy(dBh.p, bh.data(), sizeof(double2) * bh.size(), cudaMemcpyHostToDevice),
                       "cudaMemcpy"));
    HAL_TRY(CudaStatus(cudaMemcpy(dLo.p, lo.data(), sizeof(int2) * lo.size(), cudaMemcpyHostToDevice),
                       "cudaMemcpy"));
    HAL_TRY(CudaStatus(cudaMemset(dBad.p, 0, sizeof(unsigned long long)), "cudaMemset"));
    if (nNum > 0 && nDen > 0)
    {
        CheckPlanDivision<<<StrideBlocks(nNum), 256>>>(dNum.p, nNum, dBh.p, dLo.p, nDen, dBad.p);
        CountLaunch();
        HAL_TRY(LaunchStatus("CheckPlanDivision"));
    }
    unsigned long long bad = 0;
    HAL_TRY(CudaStatus(cudaMemcpy(&bad, dBad.p, sizeof(bad), cudaMemcpyDeviceToHost), "cudaMemcpy"));
    *mismatches = static_cast<int64_t>(bad);
    return HAL_CUDA_OK;
}
