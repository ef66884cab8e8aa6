// Hal::Cuda::CudaPDEGrid2D over the hal_cuda_pdegrid C ABI.
#include "Hal/Cuda/CudaPDEGrid2D.h"

#include "Hal/Cuda/CudaBackends2D.h"

#include <cmath>
#include <stdexcept>

namespace Hal::Cuda
{
    void Check(int status, const char *pWhat);

    CudaPDEGrid2D::CudaPDEGrid2D(int32_t xDim, int32_t yDim)
        : CudaPDEGrid2D(xDim, yDim, false, false)
    {
    }

    CudaPDEGrid2D::CudaPDEGrid2D(int32_t xDim, int32_t yDim, bool wrapX, bool wrapY)
        : m_xDim(xDim),
          m_yDim(yDim),
          m_wrapX(wrapX),
          m_wrapY(wrapY)
    {
        Check(hal_cuda_pdegrid_create(xDim, yDim, wrapX, wrapY, &m_pHandle), "CudaPDEGrid2D");
    }

    CudaPDEGrid2D::~CudaPDEGrid2D()
    {
        hal_cuda_pdegrid_destroy(m_pHandle);
    }

    void CudaPDEGrid2D::Queue(int32_t op, int32_t i, double val)
    {
        m_qOps.push_back(op);
        m_qCells.push_back(i);
        m_qVals.push_back(val);
    }

    // Sends the queued per-cell operations (one list, applied in call order).
    void CudaPDEGrid2D::Flush() const
    {
        if (m_qOps.empty())
        {
            return;
        }
        const int rc = hal_cuda_pdegrid_apply(m_pHandle, m_qOps.data(), 0, m_qCells.data(), m_qVals.data(), 0.0,
                                              static_cast<int64_t>(m_qOps.size()));
        m_qOps.clear();
        m_qCells.clear();
        m_qVals.clear();
        Check(rc, "CudaPDEGrid2D: per-cell operations");
    }

    const std::vector<double> &CudaPDEGrid2D::GetField() const
    {
        if (!m_fieldValid)
        {
            m_field.resize(static_cast<size_t>(Length()));
            Check(hal_cuda_pdegrid_get_state(m_pHandle, m_field.data(), nullptr, nullptr), "CudaPDEGrid2D::GetField");
            m_fieldValid = true;
        }
        return m_field;
    }

    std::vector<double> CudaPDEGrid2D::GetDeltas() const
    {
        Flush();
        std::vector<double> d(static_cast<size_t>(Length()));
        Check(hal_cuda_pdegrid_get_state(m_pHandle, nullptr, d.data(), nullptr), "CudaPDEGrid2D::GetDeltas");
        return d;
    }

    void CudaPDEGrid2D::SetState(const std::vector<double> &field, const std::vector<double> &deltas,
                                 int32_t updateCt)
    {
        if (static_cast<int32_t>(field.size()) != Length() || static_cast<int32_t>(deltas.size()) != Length())
        {
            Check(HAL_CUDA_EINVAL, "PDEGrid::SetState arrays must match the grid length");
        }
        m_qOps.clear();
        m_qCells.clear();
        m_qVals.clear();
        Check(hal_cuda_pdegrid_set_state(m_pHandle, field.data(), deltas.data(), updateCt), "CudaPDEGrid2D::SetState");
        m_updateCt = updateCt;
        m_field = field;
        m_fieldValid = true;
    }

    double CudaPDEGrid2D::Get(int32_t i) const
    {
        return GetField()[static_cast<size_t>(i)];
    }

    void CudaPDEGrid2D::ApplyAgents(CudaAgentForceBackend2D &agents, int32_t op, double value,
                                    const std::vector<double> &perAgent)
    {
        Flush();
        Check(hal_cuda_pdegrid_apply_agents(m_pHandle, agents.Handle(), op, value,
                                            perAgent.empty() ? nullptr : perAgent.data()),
              "CudaPDEGrid2D::ApplyAgents");
    }

    void CudaPDEGrid2D::Stats(double denomOffset, double *out) const
    {
        Flush();
        Check(hal_cuda_pdegrid_stats(m_pHandle, denomOffset, out), "CudaPDEGrid2D: reduction");
    }

    double CudaPDEGrid2D::GetMax() const
    {
        double s[5];
        Stats(NAN, s);
        return s[0];
    }

    double CudaPDEGrid2D::GetMin() const
    {
        double s[5];
        Stats(NAN, s);
        return s[1];
    }

    double CudaPDEGrid2D::GetAvg() const
    {
        double s[5];
        Stats(NAN, s);
        return s[2];
    }

    double CudaPDEGrid2D::MaxDelta() const
    {
        double s[5];
        Stats(NAN, s);
        return s[3];
    }

    double CudaPDEGrid2D::MaxDeltaScaled(double denomOffset) const
    {
        double s[5];
        Stats(denomOffset, s);
        return s[4];
    }

    void CudaPDEGrid2D::Update()
    {
        Flush();
        Check(hal_cuda_pdegrid_update(m_pHandle), "CudaPDEGrid2D::Update");
        m_updateCt++;
        m_fieldValid = false;
    }

    void CudaPDEGrid2D::SetAll(double val)
    {
        Flush();
        Check(hal_cuda_pdegrid_apply_all(m_pHandle, HAL_CUDA_CELL_SET, val, nullptr), "CudaPDEGrid2D::SetAll");
    }

    void CudaPDEGrid2D::SetAll(const double *pVals)
    {
        Flush();
        Check(hal_cuda_pdegrid_apply_all(m_pHandle, HAL_CUDA_CELL_SET, 0.0, pVals), "CudaPDEGrid2D::SetAll");
    }

    void CudaPDEGrid2D::AddAll(double val)
    {
        Flush();
        Check(hal_cuda_pdegrid_apply_all(m_pHandle, HAL_CUDA_CELL_ADD, val, nullptr), "CudaPDEGrid2D::AddAll");
    }

    void CudaPDEGrid2D::MulAll(double val)
    {
        Flush();
        Check(hal_cuda_pdegrid_apply_all(m_pHandle, HAL_CUDA_CELL_MUL, val, nullptr), "CudaPDEGrid2D::MulAll");
    }

    void CudaPDEGrid2D::SetNonNegative()
    {
        Flush();
        Check(hal_cuda_pdegrid_set_non_negative(m_pHandle), "CudaPDEGrid2D::SetNonNegative");
    }

    // GradientX / GradientY (PDEGrid2D.h:257-285) on the host copy of the
    // committed field: DisplacedField(+1) - DisplacedField(-1), off-grid the
    // cell's own value or the boundary value, a wrapped axis wrapped.
    double CudaPDEGrid2D::Gradient(int32_t x, int32_t y, bool alongX, bool useBoundary, double boundaryValue) const
    {
        const std::vector<double> &f = GetField();
        const double oob = useBoundary ? boundaryValue : f[static_cast<size_t>(I(x, y))];
        auto displaced = [&](int32_t a, int32_t b) {
            const int32_t dim = alongX ? m_xDim : m_yDim;
            int32_t v = alongX ? a : b;
            if (v < 0 || v >= dim)
            {
                if (!(alongX ? m_wrapX : m_wrapY))
                {
                    return oob;
                }
                v %= dim;
                v = (v < 0) ? v + dim : v;
            }
            return alongX ? f[static_cast<size_t>(I(v, b))] : f[static_cast<size_t>(I(a, v))];
        };
        return alongX ? displaced(x + 1, y) - displaced(x - 1, y) : displaced(x, y + 1) - displaced(x, y - 1);
    }

    double CudaPDEGrid2D::GradientX(int32_t x, int32_t y) const
    {
        return Gradient(x, y, true, false, 0.0);
    }

    double CudaPDEGrid2D::GradientX(int32_t x, int32_t y, double boundaryValue) const
    {
        return Gradient(x, y, true, true, boundaryValue);
    }

    double CudaPDEGrid2D::GradientY(int32_t x, int32_t y) const
    {
        return Gradient(x, y, false, false, 0.0);
    }

    double CudaPDEGrid2D::GradientY(int32_t x, int32_t y, double boundaryValue) const
    {
        return Gradient(x, y, false, true, boundaryValue);
    }

    void CudaPDEGrid2D::CheckCells(const std::vector<double> &a, const char *pWhat) const
    {
        if (static_cast<int32_t>(a.size()) != Length())
        {
            Check(HAL_CUDA_EINVAL, pWhat);
        }
    }

    void CudaPDEGrid2D::Diffusion(double diffCoef)
    {
        Flush();
        Check(hal_cuda_pdegrid_diffusion(m_pHandle, diffCoef, nullptr), "CudaPDEGrid2D::Diffusion");
    }

    void CudaPDEGrid2D::Diffusion(double diffCoef, double boundaryValue)
    {
        DiffusionTable(diffCoef, std::vector<double>(2 * (static_cast<size_t>(m_xDim) + m_yDim), boundaryValue));
    }

    void CudaPDEGrid2D::DiffusionTable(double diffCoef, const std::vector<double> &ghost)
    {
        Flush();
        Check(hal_cuda_pdegrid_diffusion(m_pHandle, diffCoef, ghost.data()), "CudaPDEGrid2D::Diffusion");
    }

    void CudaPDEGrid2D::Diffusion(const std::vector<double> &diffRatesX, const std::vector<double> &diffRatesY)
    {
        CheckCells(diffRatesX, "CudaPDEGrid2D::Diffusion: rate arrays must hold xDim*yDim values");
        CheckCells(diffRatesY, "CudaPDEGrid2D::Diffusion: rate arrays must hold xDim*yDim values");
        Flush();
        Check(hal_cuda_pdegrid_diffusion_var(m_pHandle, diffRatesX.data(), diffRatesY.data()),
              "CudaPDEGrid2D::Diffusion");
    }

    void CudaPDEGrid2D::DiffusionADI(double diffRate)
    {
        Flush();
        Check(hal_cuda_pdegrid_diffusion_adi(m_pHandle, diffRate, nullptr), "CudaPDEGrid2D::DiffusionADI");
    }

    void CudaPDEGrid2D::DiffusionADI(double diffRate, double boundaryValue)
    {
        DiffusionADITable(diffRate, std::vector<double>(2 * (static_cast<size_t>(m_xDim) + m_yDim), boundaryValue));
    }

    void CudaPDEGrid2D::DiffusionADITable(double diffRate, const std::vector<double> &ghost)
    {
        Flush();
        Check(hal_cuda_pdegrid_diffusion_adi(m_pHandle, diffRate, ghost.data()), "CudaPDEGrid2D::DiffusionADI");
    }

    void CudaPDEGrid2D::Advection(double xVel, double yVel)
    {
        Flush();
        Check(hal_cuda_pdegrid_advection(m_pHandle, xVel, yVel, nullptr), "CudaPDEGrid2D::Advection");
    }

    void CudaPDEGrid2D::Advection(double xVel, double yVel, double boundaryValue)
    {
        AdvectionTable(xVel, yVel, std::vector<double>(2 * (static_cast<size_t>(m_xDim) + m_yDim), boundaryValue));
    }

    void CudaPDEGrid2D::AdvectionTable(double xVel, double yVel, const std::vector<double> &ghost)
    {
        Flush();
        Check(hal_cuda_pdegrid_advection(m_pHandle, xVel, yVel, ghost.data()), "CudaPDEGrid2D::Advection");
    }

    void CudaPDEGrid2D::Advection(const std::vector<double> &xVels, const std::vector<double> &yVels)
    {
        CheckCells(xVels, "CudaPDEGrid2D::Advection: velocity arrays must hold xDim*yDim values");
        CheckCells(yVels, "CudaPDEGrid2D::Advection: velocity arrays must hold xDim*yDim values");
        Flush();
        Check(hal_cuda_pdegrid_advection_var(m_pHandle, xVels.data(), yVels.data(), nullptr, nullptr, nullptr),
              "CudaPDEGrid2D::Advection");
    }

    void CudaPDEGrid2D::AdvectionVarTables(const std::vector<double> &xVels, const std::vector<double> &yVels,
                                           const std::vector<double> &ghost, const std::vector<double> &ghostXVel,
                                           const std::vector<double> &ghostYVel)
    {
        CheckCells(xVels, "CudaPDEGrid2D::Advection: velocity arrays must hold xDim*yDim values");
        CheckCells(yVels, "CudaPDEGrid2D::Advection: velocity arrays must hold xDim*yDim values");
        Flush();
        Check(hal_cuda_pdegrid_advection_var(m_pHandle, xVels.data(), yVels.data(), ghost.data(), ghostXVel.data(),
                                             ghostYVel.data()),
              "CudaPDEGrid2D::Advection");
    }
}
