// CudaPDEGrid2D.h -- Hal::PDEGrid2D with its field resident on the GPU.
//
// The same calls as Hal::PDEGrid2D (include/Hal/Grids/PDEGrid2D.h:17-458), so
// model code written against PDEGrid2D compiles against this class by
// changing the grid's type.  The committed field and the delta buffer live in
// device memory (FP64) in the hal_cuda_pdegrid handle of hal_cuda.h, and every
// call gives the reference's bits: the per-cell operations Set/Add/Mul/Scale
// are queued on the host and sent as one list before the next operator,
// query or Update, which applies them in call order; the PDE operators run on
// the device; Get and the gradients read a host copy of the committed field,
// fetched once after each Update.  GetAvg is a parallel sum (within rounding
// of the reference's serial sum).  Errors throw as PDEGrid2D does:
// std::invalid_argument for the rate checks and size mismatches,
// std::runtime_error for device failures.
#pragma once

#include "hal_cuda.h"

#include <cstdint>
#include <vector>

namespace Hal
{
    namespace Cuda
    {
        class CudaAgentForceBackend2D;

        class CudaPDEGrid2D
        {
        public:
            CudaPDEGrid2D(int32_t xDim, int32_t yDim);
            CudaPDEGrid2D(int32_t xDim, int32_t yDim, bool wrapX, bool wrapY);
            ~CudaPDEGrid2D();
            CudaPDEGrid2D(const CudaPDEGrid2D &) = delete;
            CudaPDEGrid2D &operator=(const CudaPDEGrid2D &) = delete;

            int32_t Xdim() const { return m_xDim; }
            int32_t Ydim() const { return m_yDim; }
            int32_t Length() const { return m_xDim * m_yDim; }
            bool IsWrapX() const { return m_wrapX; }
            bool IsWrapY() const { return m_wrapY; }
            int32_t I(int32_t x, int32_t y) const { return x * m_yDim + y; }
            int32_t UpdateCt() const { return m_updateCt; }

            // The committed field (host copy) and the pending deltas.
            const std::vector<double> &GetField() const;
            std::vector<double> GetDeltas() const;
            void SetState(const std::vector<double> &field, const std::vector<double> &deltas, int32_t updateCt);

            double Get(int32_t x, int32_t y) const { return Get(I(x, y)); }
            double Get(int32_t i) const;

            void Set(int32_t x, int32_t y, double val) { Queue(HAL_CUDA_CELL_SET, I(x, y), val); }
            void Set(int32_t i, double val) { Queue(HAL_CUDA_CELL_SET, i, val); }
            void Add(int32_t x, int32_t y, double val) { Queue(HAL_CUDA_CELL_ADD, I(x, y), val); }
            void Add(int32_t i, double val) { Queue(HAL_CUDA_CELL_ADD, i, val); }
            void Mul(int32_t x, int32_t y, double val) { Queue(HAL_CUDA_CELL_MUL, I(x, y), val); }
            void Mul(int32_t i, double val) { Queue(HAL_CUDA_CELL_MUL, i, val); }
            void Scale(int32_t x, int32_t y, double val) { Queue(HAL_CUDA_CELL_SCALE, I(x, y), val); }
            void Scale(int32_t i, double val) { Queue(HAL_CUDA_CELL_SCALE, i, val); }

            // One operation per agent of the agent backend's last binning, at
            // its cell, in agent index order (e.g. HAL_CUDA_CELL_MUL with
            // -uptake: each agent's Mul(Isq(), -uptake)), without a host loop.
            void ApplyAgents(CudaAgentForceBackend2D &agents, int32_t op, double value,
                             const std::vector<double> &perAgent = {});

            double GetMax() const;
            double GetMin() const;
            double GetAvg() const;
            double MaxDelta() const;
            double MaxDeltaScaled(double denomOffset) const;

            void Update();
            void SetAll(double val);
            void SetAll(const double *pVals);
            void AddAll(double val);
            void MulAll(double val);
            void SetNonNegative();

            double GradientX(int32_t x, int32_t y) const;
            double GradientX(int32_t x, int32_t y, double boundaryValue) const;
            double GradientY(int32_t x, int32_t y) const;
            double GradientY(int32_t x, int32_t y, double boundaryValue) const;

            void Diffusion(double diffCoef);
            void Diffusion(double diffCoef, double boundaryValue);
            template <typename BCFn>
            void Diffusion(double diffCoef, BCFn bc)
            {
                DiffusionTable(diffCoef, GhostTable(bc));
            }
            void Diffusion(const std::vector<double> &diffRatesX, const std::vector<double> &diffRatesY);

            void DiffusionADI(double diffRate);
            void DiffusionADI(double diffRate, double boundaryValue);
            template <typename BCFn>
            void DiffusionADI(double diffRate, BCFn bc)
            {
                DiffusionADITable(diffRate, GhostTable(bc));
            }

            void Advection(double xVel, double yVel);
            void Advection(double xVel, double yVel, double boundaryValue);
            template <typename BCFn>
            void Advection(double xVel, double yVel, BCFn bc)
            {
                AdvectionTable(xVel, yVel, GhostTable(bc));
            }
            void Advection(const std::vector<double> &xVels, const std::vector<double> &yVels);
            template <typename BCFn, typename XVelBCFn, typename YVelBCFn>
            void Advection(const std::vector<double> &xVels, const std::vector<double> &yVels, BCFn bc,
                           XVelBCFn xVelBC, YVelBCFn yVelBC)
            {
                AdvectionVarTables(xVels, yVels, GhostTable(bc), GhostTable(xVelBC), GhostTable(yVelBC));
            }

            hal_cuda_pdegrid *Handle() const { return m_pHandle; }

        private:
            // A boundary callable evaluated one cell outside the grid, in the
            // ghost-table layout of hal_cuda.h (the only cells the reference
            // evaluates it at, PDEequations.h:50-98, ADIequations.h:339-378).
            template <typename BCFn>
            std::vector<double> GhostTable(BCFn bc) const
            {
                std::vector<double> g(2 * (static_cast<size_t>(m_xDim) + m_yDim));
                for (int32_t y = 0; y < m_yDim; y++)
                {
                    g[y] = bc(-1, y);
                    g[m_yDim + y] = bc(m_xDim, y);
                }
                for (int32_t x = 0; x < m_xDim; x++)
                {
                    g[2 * m_yDim + x] = bc(x, -1);
                    g[2 * m_yDim + m_xDim + x] = bc(x, m_yDim);
                }
                return g;
            }

            void Queue(int32_t op, int32_t i, double val);
            void Flush() const;
            void Stats(double denomOffset, double *out) const;
            double Gradient(int32_t x, int32_t y, bool alongX, bool useBoundary, double boundaryValue) const;
            void DiffusionTable(double diffCoef, const std::vector<double> &ghost);
            void DiffusionADITable(double diffRate, const std::vector<double> &ghost);
            void AdvectionTable(double xVel, double yVel, const std::vector<double> &ghost);
            void AdvectionVarTables(const std::vector<double> &xVels, const std::vector<double> &yVels,
                                    const std::vector<double> &ghost, const std::vector<double> &ghostXVel,
                                    const std::vector<double> &ghostYVel);
            void CheckCells(const std::vector<double> &a, const char *pWhat) const;

            hal_cuda_pdegrid *m_pHandle = nullptr;
            int32_t m_xDim, m_yDim;
            bool m_wrapX, m_wrapY;
            int32_t m_updateCt = 0;
            // queued per-cell operations, in call order
            mutable std::vector<int32_t> m_qOps, m_qCells;
            mutable std::vector<double> m_qVals;
            // host copy of the committed field
            mutable std::vector<double> m_field;
            mutable bool m_fieldValid = false;
        };
    }
}
