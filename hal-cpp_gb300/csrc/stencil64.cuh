// stencil64.cuh -- the FP64 per-cell stencils of the reference's CPU code
// (src/Pde/PDEequations.cpp, include/Hal/Pde/PDEequations.h) as device
// functors, shared by the interface kernels (diffusion.cu) and the resident
// PDEGrid2D (pdegrid.cu).
#pragma once

#include <algorithm>
#include <cstdint>

namespace halcuda
{
    namespace stencil64
    {
        // The FP64 stencils below reproduce the reference's CPU arithmetic bit
        // for bit: IEEE operations in the reference's order, no contraction.
        // GB300 issues FP64 at a small fraction of its FP32 rate, so the
        // cells are indexed without 64-bit division (y from the block's x
        // index, x from its y index) and sign tests use the bit pattern.

        // v > 0 and v < 0 as IEEE comparisons (false for zeros and NaNs),
        // decided on the two 32-bit halves of v so that no FP64 compare is
        // issued: |v| is nonzero and at most infinity, then the sign bit.
        __device__ __forceinline__ int Sign64(double v)
        {
            const int hi = __double2hiint(v);
            const unsigned lo = static_cast<unsigned>(__double2loint(v));
            const unsigned mag = static_cast<unsigned>(hi) & 0x7fffffffu;
            const bool nonzero = (mag | lo) != 0u;
            const bool notNan = mag < 0x7ff00000u || (mag == 0x7ff00000u && lo == 0u);
            return (nonzero && notNan) ? (hi < 0 ? -1 : 1) : 0;
        }

        // vel * (vel > 0 ? ifPos : ifNeg), or +0 when vel is 0 or NaN: the
        // reference's upwind flux of one face.
        __device__ __forceinline__ double UpwindFlux64(double vel, double ifPos, double ifNeg)
        {
            const int sign = Sign64(vel);
            const double p = __dmul_rn(vel, sign > 0 ? ifPos : ifNeg);
            return sign != 0 ? p : 0.0;
        }

        // field[n] - c along one axis of a line: the neighbour at index n
        // (wrapped, a Dirichlet ghost doubled, or 0 off-grid) minus the cell.
        __device__ __forceinline__ double DeltaTerm64(const double *f, double c, int32_t n,
                                                      int32_t dim, bool wrap, int64_t base,
                                                      int64_t stride, const double *ghost,
                                                      int64_t ghostIdx)
        {
            if (n >= 0 && n < dim)
            {
                return __dsub_rn(f[base + n * stride], c);
            }
            if (wrap)
            {
                int32_t w = (n < 0) ? n + dim : n - dim;
                return __dsub_rn(f[base + w * stride], c);
            }
            if (ghost != nullptr)
            {
                return __dmul_rn(__dsub_rn(ghost[ghostIdx], c), 2.0);
            }
            return 0.0;
        }

        // DisplacedX2D / DisplacedY2D (src/Pde/PDEequations.cpp:163-197) and
        // their Dirichlet forms (include/Hal/Pde/PDEequations.h:589-616): a
        // per-cell value at neighbour n of a line, wrapped, or off-grid the
        // ghost-table value (not doubled), or 0 without a table.
        __device__ __forceinline__ double Displaced64(const double *v, int32_t n, int32_t dim, bool wrap,
                                                      int64_t base, int64_t stride, const double *ghost = nullptr,
                                                      int64_t ghostIdx = 0)
        {
            if (n >= 0 && n < dim)
            {
                return v[base + n * stride];
            }
            if (wrap)
            {
                int32_t w = (n < 0) ? n + dim : n - dim;
                return v[base + w * stride];
            }
            return ghost != nullptr ? ghost[ghostIdx] : 0.0;
        }

        // IDiffusionBackend2D::Diffuse: deltas[i] += sum * r, bit-identical
        // to Hal::CpuDiffusionBackend2D (src/Pde/PDEequations.cpp, the
        // uniform-rate Diffusion2 and its Dirichlet form).
        struct Diffuse64Cell
        {
            const double *__restrict__ f;
            double *__restrict__ deltas;
            const double *__restrict__ ghost;
            double r;
            int32_t xDim, yDim, wrapX, wrapY;

            __device__ __forceinline__ void operator()(int32_t x, int32_t y, int64_t i) const
            {
                const double c = f[i];
                const double *gx = ghost;
                const double *gy = ghost ? ghost + 2 * yDim : nullptr;
                const int64_t colBase = y;                               // column y, stride yDim
                const int64_t rowBase = static_cast<int64_t>(x) * yDim;  // row x, stride 1
                double s = DeltaTerm64(f, c, x + 1, xDim, wrapX, colBase, yDim, gx, yDim + y);
                s = __dadd_rn(s, DeltaTerm64(f, c, x - 1, xDim, wrapX, colBase, yDim, gx, y));
                s = __dadd_rn(s, DeltaTerm64(f, c, y + 1, yDim, wrapY, rowBase, 1, gy, xDim + x));
                s = __dadd_rn(s, DeltaTerm64(f, c, y - 1, yDim, wrapY, rowBase, 1, gy, x));
                deltas[i] = __dadd_rn(deltas[i], __dmul_rn(s, r));
            }
        };

        // Internal::Diffusion2 with per-cell rates (src/Pde/PDEequations.cpp:
        // 199-230): the +x face takes the cell's own rate except at a closed
        // last column, where the displaced (zero) rate applies.
        struct DiffuseVar64Cell
        {
            const double *__restrict__ f;
            double *__restrict__ deltas;
            const double *__restrict__ rx;
            const double *__restrict__ ry;
            int32_t xDim, yDim, wrapX, wrapY;

            __device__ __forceinline__ void operator()(int32_t x, int32_t y, int64_t i) const
            {
                const double c = f[i];
                const int64_t colBase = y, rowBase = static_cast<int64_t>(x) * yDim;
                const double dp1x =
                    ((x == xDim - 1) && !wrapX) ? Displaced64(rx, x + 1, xDim, wrapX, colBase, yDim) : rx[i];
                const double dm1x = Displaced64(rx, x - 1, xDim, wrapX, colBase, yDim);
                const double dp1y =
                    ((y == yDim - 1) && !wrapY) ? Displaced64(ry, y + 1, yDim, wrapY, rowBase, 1) : ry[i];
                const double dm1y = Displaced64(ry, y - 1, yDim, wrapY, rowBase, 1);
                double s = __dmul_rn(DeltaTerm64(f, c, x + 1, xDim, wrapX, colBase, yDim, nullptr, 0), dp1x);
                s = __dadd_rn(s, __dmul_rn(DeltaTerm64(f, c, x - 1, xDim, wrapX, colBase, yDim, nullptr, 0), dm1x));
                s = __dadd_rn(s, __dmul_rn(DeltaTerm64(f, c, y + 1, yDim, wrapY, rowBase, 1, nullptr, 0), dp1y));
                s = __dadd_rn(s, __dmul_rn(DeltaTerm64(f, c, y - 1, yDim, wrapY, rowBase, 1, nullptr, 0), dm1y));
                deltas[i] = __dadd_rn(deltas[i], s);
            }
        };

        // Internal::Advection2, uniform velocity (src/Pde/PDEequations.cpp:
        // 380-412; Dirichlet form include/Hal/Pde/PDEequations.h:413-447):
        // first-order upwind, each term added to deltas in turn.
        struct Advect64Cell
        {
            const double *__restrict__ f;
            double *__restrict__ deltas;
            const double *__restrict__ ghost;  // Dirichlet table or nullptr
            double xVel, yVel;
            int32_t xDim, yDim, wrapX, wrapY;
            int32_t xSign, ySign;  // +1 for vel > 0, -1 for vel < 0, else 0 (set on the host)

            __device__ __forceinline__ void operator()(int32_t x, int32_t y, int64_t i) const
            {
                const double c = f[i];
                const int64_t colBase = y, rowBase = static_cast<int64_t>(x) * yDim;
                const double *gy = ghost ? ghost + 2 * yDim : nullptr;
                double d = deltas[i];
                if (xSign > 0)
                {
                    d = __dadd_rn(d, __dmul_rn(DeltaTerm64(f, c, x - 1, xDim, wrapX, colBase, yDim, ghost, y), xVel));
                }
                else if (xSign < 0)
                {
                    d = __dsub_rn(d,
                                  __dmul_rn(DeltaTerm64(f, c, x + 1, xDim, wrapX, colBase, yDim, ghost, yDim + y), xVel));
                }
                if (ySign > 0)
                {
                    d = __dadd_rn(d, __dmul_rn(DeltaTerm64(f, c, y - 1, yDim, wrapY, rowBase, 1, gy, x), yVel));
                }
                else if (ySign < 0)
                {
                    d = __dsub_rn(d, __dmul_rn(DeltaTerm64(f, c, y + 1, yDim, wrapY, rowBase, 1, gy, xDim + x), yVel));
                }
                deltas[i] = d;
            }
        };

        // Internal::Advection2, per-cell velocity (src/Pde/PDEequations.cpp:
        // 535-575; Dirichlet form include/Hal/Pde/PDEequations.h:720-778):
        // upwind face fluxes, -xFluxP + xFluxM - yFluxP + yFluxM.
        struct AdvectVar64Cell
        {
            const double *__restrict__ f;
            double *__restrict__ deltas;
            const double *__restrict__ vx;
            const double *__restrict__ vy;
            const double *__restrict__ ghost;    // field boundary table or nullptr
            const double *__restrict__ ghostVx;  // x-velocity boundary table or nullptr
            const double *__restrict__ ghostVy;  // y-velocity boundary table or nullptr
            int32_t xDim, yDim, wrapX, wrapY;

            __device__ __forceinline__ void operator()(int32_t x, int32_t y, int64_t i) const
            {
                const int64_t colBase = y, rowBase = static_cast<int64_t>(x) * yDim;
                const double *gy = ghost ? ghost + 2 * yDim : nullptr;
                const double *gvy = ghostVy ? ghostVy + 2 * yDim : nullptr;
                const double xVelP = ((x == xDim - 1) && !wrapX)
                                         ? Displaced64(vx, x + 1, xDim, wrapX, colBase, yDim, ghostVx, yDim + y)
                                         : vx[i];
                const double yVelP = ((y == yDim - 1) && !wrapY)
                                         ? Displaced64(vy, y + 1, yDim, wrapY, rowBase, 1, gvy, xDim + x)
                                         : vy[i];
                const double xVelM = Displaced64(vx, x - 1, xDim, wrapX, colBase, yDim, ghostVx, y);
                const double yVelM = Displaced64(vy, y - 1, yDim, wrapY, rowBase, 1, gvy, x);
                const double c = f[i];
                // Each flux is velocity x upwind value, 0 when the velocity is
                // neither > 0 nor < 0.  The product is formed on every lane and
                // selected afterwards, so lanes of a warp with different signs
                // do not issue the FP64 multiply twice.
                const double xFluxP =
                    UpwindFlux64(xVelP, c, Displaced64(f, x + 1, xDim, wrapX, colBase, yDim, ghost, yDim + y));
                const double xFluxM = UpwindFlux64(xVelM, Displaced64(f, x - 1, xDim, wrapX, colBase, yDim, ghost, y), c);
                const double yFluxP = UpwindFlux64(yVelP, c, Displaced64(f, y + 1, yDim, wrapY, rowBase, 1, gy, xDim + x));
                const double yFluxM = UpwindFlux64(yVelM, Displaced64(f, y - 1, yDim, wrapY, rowBase, 1, gy, x), c);
                // -xFluxP + xFluxM is xFluxM - xFluxP exactly (IEEE a - b = a + (-b))
                double t = __dsub_rn(xFluxM, xFluxP);
                t = __dsub_rn(t, yFluxP);
                t = __dadd_rn(t, yFluxM);
                deltas[i] = __dadd_rn(deltas[i], t);
            }
        };

        // One thread per cell of an xDim x yDim field in layout A: y from the
        // block's x index (rows read coalesced), x from its y index, striding
        // by gridDim.y when xDim exceeds the grid's y limit.
        template <class Cell>
        __global__ void __launch_bounds__(256) Cells64Kernel(Cell cell, int32_t xDim, int32_t yDim)
        {
            const int32_t y = static_cast<int32_t>(blockIdx.x * blockDim.x + threadIdx.x);
            if (y >= yDim)
            {
                return;
            }
            for (int32_t x = static_cast<int32_t>(blockIdx.y); x < xDim; x += static_cast<int32_t>(gridDim.y))
            {
                cell(x, y, static_cast<int64_t>(x) * yDim + y);
            }
        }

        // One cell per thread.  (A grid of one resident wave with threads
        // walking x measured 4-9% slower on these FP64-bound kernels.)
        inline dim3 Cells64Grid(int32_t xDim, int32_t yDim)
        {
            return dim3(static_cast<unsigned>((yDim + 255) / 256), static_cast<unsigned>(std::min(xDim, 65535)));
        }
    }
}
