// Hal::Cuda backends: thin C++ classes over the hal_cuda C ABI.
#include "Hal/Cuda/CudaBackends2D.h"

#include "Hal/Log/Logger.h"

#include <stdexcept>
#include <string>

namespace Hal::Cuda
{
    void Check(int status, const char *pWhat)
    {
        if (status == HAL_CUDA_OK)
        {
            return;
        }
        std::string msg = std::string(pWhat) + ": " + hal_cuda_last_error();
        Logger::Instance().Log(LogSeverity::Error, msg);
        if (status == HAL_CUDA_EINVAL)
        {
            throw std::invalid_argument(msg);
        }
        throw std::runtime_error(msg);
    }

    void SetDevice(int32_t device)
    {
        Check(hal_cuda_set_device(device), "Hal::Cuda::SetDevice");
    }

    namespace
    {
        const double *GhostOrNull(const std::vector<double> &ghost)
        {
            return ghost.empty() ? nullptr : ghost.data();
        }

        const float *GhostOrNull(const std::vector<float> &ghost)
        {
            return ghost.empty() ? nullptr : ghost.data();
        }

        void CheckGhost(size_t n, int32_t xDim, int32_t yDim, const char *pWhat)
        {
            if (n != 0 && n != 2 * static_cast<size_t>(xDim) + 2 * static_cast<size_t>(yDim))
            {
                std::string msg = std::string(pWhat) + ": Dirichlet table must hold 2*xDim + 2*yDim values";
                Logger::Instance().Log(LogSeverity::Error, msg);
                throw std::invalid_argument(msg);
            }
        }

        void CheckCells(const std::vector<double> &a, const std::vector<double> &b, int32_t xDim,
                        int32_t yDim, const char *pWhat)
        {
            const size_t n = static_cast<size_t>(xDim) * static_cast<size_t>(yDim);
            if (a.size() != n || b.size() != n)
            {
                std::string msg = std::string(pWhat) + ": field and deltas must hold xDim*yDim values";
                Logger::Instance().Log(LogSeverity::Error, msg);
                throw std::invalid_argument(msg);
            }
        }
    }

    // ---- explicit diffusion -------------------------------------------------

    CudaDiffusionBackend2D::CudaDiffusionBackend2D(int32_t xDim, int32_t yDim) : m_xDim(xDim), m_yDim(yDim)
    {
        Check(hal_cuda_diffusion_create(xDim, yDim, &m_pHandle), "CudaDiffusionBackend2D");
    }

    CudaDiffusionBackend2D::~CudaDiffusionBackend2D()
    {
        hal_cuda_diffusion_destroy(m_pHandle);
    }

    void CudaDiffusionBackend2D::Diffuse(const std::vector<double> &field, std::vector<double> &deltas,
                                         double diffRate, int32_t xDim, int32_t yDim, bool wrapX, bool wrapY)
    {
        Check(hal_cuda_diffuse(m_pHandle, field.data(), static_cast<int64_t>(field.size()), deltas.data(),
                               static_cast<int64_t>(deltas.size()), diffRate, xDim, yDim, wrapX, wrapY),
              "CudaDiffusionBackend2D::Diffuse");
    }

    void CudaDiffusionBackend2D::DiffuseDirichlet(const std::vector<double> &field, std::vector<double> &deltas,
                                                  double diffRate, bool wrapX, bool wrapY,
                                                  const std::vector<double> &ghost)
    {
        CheckCells(field, deltas, m_xDim, m_yDim, "CudaDiffusionBackend2D::DiffuseDirichlet");
        CheckGhost(ghost.size(), m_xDim, m_yDim, "CudaDiffusionBackend2D::DiffuseDirichlet");
        Check(hal_cuda_diffuse_bc(m_pHandle, field.data(), deltas.data(), diffRate, wrapX, wrapY, GhostOrNull(ghost)),
              "CudaDiffusionBackend2D::DiffuseDirichlet");
    }

    void CudaDiffusionBackend2D::DiffuseVariable(const std::vector<double> &field, std::vector<double> &deltas,
                                                 const std::vector<double> &diffRatesX,
                                                 const std::vector<double> &diffRatesY, bool wrapX, bool wrapY)
    {
        CheckCells(field, deltas, m_xDim, m_yDim, "CudaDiffusionBackend2D::DiffuseVariable");
        CheckCells(diffRatesX, diffRatesY, m_xDim, m_yDim, "CudaDiffusionBackend2D::DiffuseVariable");
        Check(hal_cuda_diffuse_var(m_pHandle, field.data(), deltas.data(), diffRatesX.data(), diffRatesY.data(), wrapX,
                                   wrapY),
              "CudaDiffusionBackend2D::DiffuseVariable");
    }

    void CudaDiffusionBackend2D::Advect(const std::vector<double> &field, std::vector<double> &deltas, double xVel,
                                        double yVel, bool wrapX, bool wrapY, const std::vector<double> &ghost)
    {
        CheckCells(field, deltas, m_xDim, m_yDim, "CudaDiffusionBackend2D::Advect");
        CheckGhost(ghost.size(), m_xDim, m_yDim, "CudaDiffusionBackend2D::Advect");
        Check(ghost.empty() ? hal_cuda_advect(m_pHandle, field.data(), deltas.data(), xVel, yVel, wrapX, wrapY)
                            : hal_cuda_advect_bc(m_pHandle, field.data(), deltas.data(), xVel, yVel, wrapX, wrapY,
                                                 ghost.data()),
              "CudaDiffusionBackend2D::Advect");
    }

    void CudaDiffusionBackend2D::AdvectVariable(const std::vector<double> &field, std::vector<double> &deltas,
                                                const std::vector<double> &xVels, const std::vector<double> &yVels,
                                                bool wrapX, bool wrapY, const std::vector<double> &ghost,
                                                const std::vector<double> &ghostXVel,
                                                const std::vector<double> &ghostYVel)
    {
        CheckCells(field, deltas, m_xDim, m_yDim, "CudaDiffusionBackend2D::AdvectVariable");
        CheckCells(xVels, yVels, m_xDim, m_yDim, "CudaDiffusionBackend2D::AdvectVariable");
        CheckGhost(ghost.size(), m_xDim, m_yDim, "CudaDiffusionBackend2D::AdvectVariable");
        CheckGhost(ghostXVel.size(), m_xDim, m_yDim, "CudaDiffusionBackend2D::AdvectVariable");
        CheckGhost(ghostYVel.size(), m_xDim, m_yDim, "CudaDiffusionBackend2D::AdvectVariable");
        const bool bc = !ghost.empty() || !ghostXVel.empty() || !ghostYVel.empty();
        Check(bc ? hal_cuda_advect_var_bc(m_pHandle, field.data(), deltas.data(), xVels.data(), yVels.data(), wrapX,
                                          wrapY, GhostOrNull(ghost), GhostOrNull(ghostXVel), GhostOrNull(ghostYVel))
                 : hal_cuda_advect_var(m_pHandle, field.data(), deltas.data(), xVels.data(), yVels.data(), wrapX,
                                       wrapY),
              "CudaDiffusionBackend2D::AdvectVariable");
    }

    void CudaDiffusionBackend2D::SetVelocity(double xVel, double yVel)
    {
        Check(hal_cuda_diffusion_set_velocity(m_pHandle, xVel, yVel), "CudaDiffusionBackend2D::SetVelocity");
    }

    void CudaDiffusionBackend2D::SetUptake(CudaAgentForceBackend2D *pAgents, double uptake)
    {
        Check(hal_cuda_diffusion_set_uptake(m_pHandle, pAgents ? pAgents->Handle() : nullptr, uptake),
              "CudaDiffusionBackend2D::SetUptake");
    }

    void CudaDiffusionBackend2D::SetField(const std::vector<float> &field)
    {
        Check(hal_cuda_diffusion_set_field(m_pHandle, field.data(), static_cast<int64_t>(field.size())),
              "CudaDiffusionBackend2D::SetField");
    }

    void CudaDiffusionBackend2D::GetField(std::vector<float> &field)
    {
        field.resize(static_cast<size_t>(m_xDim) * static_cast<size_t>(m_yDim));
        Check(hal_cuda_diffusion_get_field(m_pHandle, field.data(), static_cast<int64_t>(field.size())),
              "CudaDiffusionBackend2D::GetField");
    }

    void CudaDiffusionBackend2D::SetSource(const std::vector<float> &dense)
    {
        Check(hal_cuda_diffusion_set_source(m_pHandle, dense.empty() ? nullptr : dense.data(),
                                            static_cast<int64_t>(dense.size())),
              "CudaDiffusionBackend2D::SetSource");
    }

    void CudaDiffusionBackend2D::SetPointSources(const std::vector<int32_t> &cells, const std::vector<float> &values)
    {
        if (cells.size() != values.size())
        {
            Check(HAL_CUDA_EINVAL, "CudaDiffusionBackend2D::SetPointSources: cells and values differ in length");
        }
        Check(hal_cuda_diffusion_set_point_sources(m_pHandle, static_cast<int32_t>(cells.size()), cells.data(),
                                                   values.data()),
              "CudaDiffusionBackend2D::SetPointSources");
    }

    void CudaDiffusionBackend2D::SetDirichlet(const std::vector<float> &ghost)
    {
        CheckGhost(ghost.size(), m_xDim, m_yDim, "CudaDiffusionBackend2D::SetDirichlet");
        Check(hal_cuda_diffusion_set_dirichlet(m_pHandle, GhostOrNull(ghost)), "CudaDiffusionBackend2D::SetDirichlet");
    }

    void CudaDiffusionBackend2D::RunTicks(int32_t ticks, double diffRate, double decay, bool wrapX, bool wrapY)
    {
        Check(hal_cuda_diffusion_run_ticks(m_pHandle, ticks, diffRate, decay, wrapX, wrapY),
              "CudaDiffusionBackend2D::RunTicks");
    }

    void CudaDiffusionBackend2D::Sync()
    {
        Check(hal_cuda_diffusion_sync(m_pHandle), "CudaDiffusionBackend2D::Sync");
    }

    void CudaDiffusionBackend2D::RunSteps(std::vector<float> &field, int32_t steps, double diffRate, bool wrapX,
                                          bool wrapY)
    {
        Check(hal_cuda_diffusion_run_steps(m_pHandle, field.data(), static_cast<int64_t>(field.size()), steps,
                                           diffRate, wrapX, wrapY),
              "CudaDiffusionBackend2D::RunSteps");
    }

    // ---- ADI ------------------------------------------------------------------

    CudaAdiDiffusionBackend2D::CudaAdiDiffusionBackend2D(int32_t xDim, int32_t yDim) : m_xDim(xDim), m_yDim(yDim)
    {
        Check(hal_cuda_adi_create(xDim, yDim, &m_pHandle), "CudaAdiDiffusionBackend2D");
    }

    CudaAdiDiffusionBackend2D::~CudaAdiDiffusionBackend2D()
    {
        hal_cuda_adi_destroy(m_pHandle);
    }

    void CudaAdiDiffusionBackend2D::DiffuseADI(const std::vector<double> &field, std::vector<double> &deltas,
                                               double diffRate, int32_t xDim, int32_t yDim, bool wrapX, bool wrapY)
    {
        Check(hal_cuda_diffuse_adi(m_pHandle, field.data(), static_cast<int64_t>(field.size()), deltas.data(),
                                   static_cast<int64_t>(deltas.size()), diffRate, xDim, yDim, wrapX, wrapY),
              "CudaAdiDiffusionBackend2D::DiffuseADI");
    }

    void CudaAdiDiffusionBackend2D::DiffuseADIDirichlet(const std::vector<double> &field,
                                                        std::vector<double> &deltas, double diffRate, bool wrapX,
                                                        bool wrapY, const std::vector<double> &ghost)
    {
        CheckCells(field, deltas, m_xDim, m_yDim, "CudaAdiDiffusionBackend2D::DiffuseADIDirichlet");
        CheckGhost(ghost.size(), m_xDim, m_yDim, "CudaAdiDiffusionBackend2D::DiffuseADIDirichlet");
        Check(hal_cuda_diffuse_adi_bc(m_pHandle, field.data(), deltas.data(), diffRate, wrapX, wrapY,
                                      GhostOrNull(ghost)),
              "CudaAdiDiffusionBackend2D::DiffuseADIDirichlet");
    }

    void CudaAdiDiffusionBackend2D::SetField(const std::vector<float> &field)
    {
        Check(hal_cuda_adi_set_field(m_pHandle, field.data(), static_cast<int64_t>(field.size())),
              "CudaAdiDiffusionBackend2D::SetField");
    }

    void CudaAdiDiffusionBackend2D::GetField(std::vector<float> &field)
    {
        field.resize(static_cast<size_t>(m_xDim) * static_cast<size_t>(m_yDim));
        Check(hal_cuda_adi_get_field(m_pHandle, field.data(), static_cast<int64_t>(field.size())),
              "CudaAdiDiffusionBackend2D::GetField");
    }

    void CudaAdiDiffusionBackend2D::SetExact(bool exact)
    {
        Check(hal_cuda_adi_set_exact(m_pHandle, exact ? 1 : 0), "CudaAdiDiffusionBackend2D::SetExact");
    }

    void CudaAdiDiffusionBackend2D::SetSource(const std::vector<float> &dense)
    {
        Check(hal_cuda_adi_set_source(m_pHandle, dense.empty() ? nullptr : dense.data(),
                                      static_cast<int64_t>(dense.size())),
              "CudaAdiDiffusionBackend2D::SetSource");
    }

    void CudaAdiDiffusionBackend2D::SetDirichlet(const std::vector<float> &ghost)
    {
        CheckGhost(ghost.size(), m_xDim, m_yDim, "CudaAdiDiffusionBackend2D::SetDirichlet");
        Check(hal_cuda_adi_set_dirichlet(m_pHandle, GhostOrNull(ghost)), "CudaAdiDiffusionBackend2D::SetDirichlet");
    }

    void CudaAdiDiffusionBackend2D::SetUptake(CudaAgentForceBackend2D *pAgents, double uptake)
    {
        Check(hal_cuda_adi_set_uptake(m_pHandle, pAgents ? pAgents->Handle() : nullptr, uptake),
              "CudaAdiDiffusionBackend2D::SetUptake");
    }

    void CudaAdiDiffusionBackend2D::RunCoupled(CudaAgentForceBackend2D &agents, int32_t ticks, double diffRate,
                                               double decay, bool wrapX, bool wrapY, double interactionRad,
                                               double springConstant, double friction, double maxVel)
    {
        Check(hal_cuda_adi_run_coupled(m_pHandle, agents.Handle(), ticks, diffRate, decay, wrapX ? 1 : 0,
                                       wrapY ? 1 : 0, interactionRad, springConstant, friction, maxVel),
              "CudaAdiDiffusionBackend2D::RunCoupled");
    }

    void CudaAdiDiffusionBackend2D::RunTicks(int32_t ticks, double diffRate, double decay, bool wrapX, bool wrapY)
    {
        Check(hal_cuda_adi_run_ticks(m_pHandle, ticks, diffRate, decay, wrapX, wrapY),
              "CudaAdiDiffusionBackend2D::RunTicks");
    }

    void CudaAdiDiffusionBackend2D::Sync()
    {
        Check(hal_cuda_adi_sync(m_pHandle), "CudaAdiDiffusionBackend2D::Sync");
    }

    void CudaAdiDiffusionBackend2D::RunSteps(std::vector<float> &field, int32_t steps, double diffRate, bool wrapX,
                                             bool wrapY)
    {
        Check(hal_cuda_adi_run_steps(m_pHandle, field.data(), static_cast<int64_t>(field.size()), steps, diffRate,
                                     wrapX, wrapY),
              "CudaAdiDiffusionBackend2D::RunSteps");
    }

    // ---- agent forces ---------------------------------------------------------

    CudaAgentForceBackend2D::CudaAgentForceBackend2D(int32_t xDim, int32_t yDim, int32_t maxAgents)
        : m_xDim(xDim), m_yDim(yDim), m_maxAgents(maxAgents)
    {
        Check(hal_cuda_agents_create(xDim, yDim, maxAgents, &m_pHandle), "CudaAgentForceBackend2D");
    }

    CudaAgentForceBackend2D::~CudaAgentForceBackend2D()
    {
        hal_cuda_agents_destroy(m_pHandle);
    }

    void CudaAgentForceBackend2D::AccumulateForces(const std::vector<double> &positions,
                                                   const std::vector<double> &radii,
                                                   std::vector<double> &velocityDeltas, double interactionRad,
                                                   double springConstant, int32_t xDim, int32_t yDim, bool wrapX,
                                                   bool wrapY)
    {
        if (positions.size() != 2 * radii.size())
        {
            Check(HAL_CUDA_EINVAL, "CudaAgentForceBackend2D::AccumulateForces: positions must hold two values per "
                                   "radius");
        }
        velocityDeltas.resize(positions.size());
        Check(hal_cuda_accumulate_forces(m_pHandle, positions.data(), static_cast<int64_t>(positions.size()),
                                         radii.data(), static_cast<int64_t>(radii.size()), velocityDeltas.data(),
                                         interactionRad, springConstant, xDim, yDim, wrapX, wrapY),
              "CudaAgentForceBackend2D::AccumulateForces");
        m_count = static_cast<int32_t>(radii.size());
    }

    void CudaAgentForceBackend2D::SumForces(const std::vector<double> &positions, const std::vector<double> &radii,
                                            std::vector<double> &velocities, std::vector<double> &forceSums,
                                            double interactionRad, const hal_cuda_force_law &law, int32_t xDim,
                                            int32_t yDim, bool wrapX, bool wrapY, int32_t order)
    {
        if (positions.size() != 2 * radii.size())
        {
            Check(HAL_CUDA_EINVAL, "CudaAgentForceBackend2D::SumForces: positions must hold two values per radius");
        }
        if (!velocities.empty() && velocities.size() != positions.size())
        {
            Check(HAL_CUDA_EINVAL, "CudaAgentForceBackend2D::SumForces: velocities must hold two values per agent");
        }
        const bool haveVel = !velocities.empty();
        velocities.resize(positions.size());
        forceSums.resize(radii.size());
        Check(hal_cuda_sum_forces(m_pHandle, positions.data(), radii.data(), static_cast<int64_t>(radii.size()),
                                  haveVel ? velocities.data() : nullptr, velocities.data(), forceSums.data(),
                                  interactionRad, &law, order, xDim, yDim, wrapX, wrapY),
              "CudaAgentForceBackend2D::SumForces");
        m_count = static_cast<int32_t>(radii.size());
    }

    void CudaAgentForceBackend2D::DispatchLaw(double interactionRad, const hal_cuda_force_law &law, bool withSums,
                                              bool wrapX, bool wrapY)
    {
        Check(hal_cuda_agents_dispatch_law(m_pHandle, interactionRad, &law, withSums, wrapX, wrapY),
              "CudaAgentForceBackend2D::DispatchLaw");
    }

    void CudaAgentForceBackend2D::StepLaw(int32_t ticks, double interactionRad, const hal_cuda_force_law &law,
                                          bool withSums, bool wrapX, bool wrapY, double friction, double maxVel)
    {
        Check(hal_cuda_agents_step_law(m_pHandle, ticks, interactionRad, &law, withSums, wrapX, wrapY, friction,
                                       maxVel),
              "CudaAgentForceBackend2D::StepLaw");
    }

    void CudaAgentForceBackend2D::GetForceSums(std::vector<float> &forceSums)
    {
        forceSums.resize(static_cast<size_t>(m_count));
        Check(hal_cuda_agents_get_force_sums(m_pHandle, forceSums.data(), m_count),
              "CudaAgentForceBackend2D::GetForceSums");
    }

    void CudaAgentForceBackend2D::Upload(const std::vector<float> &positions, const std::vector<float> &radii)
    {
        if (positions.size() != 2 * radii.size())
        {
            Check(HAL_CUDA_EINVAL, "CudaAgentForceBackend2D::Upload: positions must hold two values per radius");
        }
        Check(hal_cuda_agents_upload(m_pHandle, positions.data(), radii.data(), static_cast<int32_t>(radii.size())),
              "CudaAgentForceBackend2D::Upload");
        m_count = static_cast<int32_t>(radii.size());
    }

    void CudaAgentForceBackend2D::Dispatch(double interactionRad, double springConstant, bool wrapX, bool wrapY)
    {
        Check(hal_cuda_agents_dispatch(m_pHandle, interactionRad, springConstant, wrapX, wrapY),
              "CudaAgentForceBackend2D::Dispatch");
    }

    void CudaAgentForceBackend2D::Download(std::vector<float> &velocityDeltas)
    {
        velocityDeltas.resize(2 * static_cast<size_t>(m_count));
        Check(hal_cuda_agents_download(m_pHandle, velocityDeltas.data(), m_count), "CudaAgentForceBackend2D::Download");
    }

    void CudaAgentForceBackend2D::SetVelocities(const std::vector<float> &velocities)
    {
        if (velocities.size() != 2 * static_cast<size_t>(m_count))
        {
            std::string msg = "CudaAgentForceBackend2D::SetVelocities: two values per uploaded agent";
            Logger::Instance().Log(LogSeverity::Error, msg);
            throw std::invalid_argument(msg);
        }
        Check(hal_cuda_agents_set_velocities(m_pHandle, velocities.empty() ? nullptr : velocities.data(), m_count),
              "CudaAgentForceBackend2D::SetVelocities");
    }

    void CudaAgentForceBackend2D::Step(int32_t ticks, double interactionRad, double springConstant, bool wrapX,
                                       bool wrapY, double friction, double maxVel)
    {
        Check(hal_cuda_agents_step(m_pHandle, ticks, interactionRad, springConstant, wrapX, wrapY, friction, maxVel),
              "CudaAgentForceBackend2D::Step");
    }

    void CudaAgentForceBackend2D::GetState(std::vector<float> &positions, std::vector<float> &velocities)
    {
        positions.resize(2 * static_cast<size_t>(m_count));
        velocities.resize(2 * static_cast<size_t>(m_count));
        Check(hal_cuda_agents_get_state(m_pHandle, positions.data(), velocities.data(), m_count),
              "CudaAgentForceBackend2D::GetState");
    }

    void CudaAgentForceBackend2D::GetBins(std::vector<int32_t> &cellOffsets, std::vector<int32_t> &bucketAgents)
    {
        cellOffsets.resize(static_cast<size_t>(m_xDim) * static_cast<size_t>(m_yDim) + 1);
        bucketAgents.resize(static_cast<size_t>(m_count));
        Check(hal_cuda_agents_get_bins(m_pHandle, cellOffsets.data(), bucketAgents.empty() ? nullptr : bucketAgents.data()),
              "CudaAgentForceBackend2D::GetBins");
    }

    // ---- CudaWells2D ---------------------------------------------------------

    CudaWells2D::CudaWells2D(const std::vector<hal_cuda_well_desc> &wells)
        : m_wells(wells)
    {
        Check(hal_cuda_wells_create(wells.data(), static_cast<int32_t>(wells.size()), &m_pHandle), "CudaWells2D");
    }

    CudaWells2D::~CudaWells2D()
    {
        hal_cuda_wells_destroy(m_pHandle);
    }

    void CudaWells2D::SetField(int32_t well, const std::vector<float> &field)
    {
        Check(hal_cuda_wells_set_field(m_pHandle, well, field.data(), static_cast<int64_t>(field.size())),
              "CudaWells2D::SetField");
    }

    void CudaWells2D::GetField(int32_t well, std::vector<float> &field)
    {
        if (well < 0 || well >= static_cast<int32_t>(m_wells.size()))
        {
            Check(HAL_CUDA_EINVAL, "CudaWells2D::GetField: no such well");
        }
        const hal_cuda_well_desc &d = m_wells[static_cast<size_t>(well)];
        field.resize(static_cast<size_t>(d.xDim) * static_cast<size_t>(d.yDim));
        Check(hal_cuda_wells_get_field(m_pHandle, well, field.data(), static_cast<int64_t>(field.size())),
              "CudaWells2D::GetField");
    }

    void CudaWells2D::SetSource(int32_t well, const std::vector<float> &dense)
    {
        Check(hal_cuda_wells_set_source(m_pHandle, well, dense.empty() ? nullptr : dense.data(),
                                        static_cast<int64_t>(dense.size())),
              "CudaWells2D::SetSource");
    }

    void CudaWells2D::SetAgents(const std::vector<int32_t> &counts, const std::vector<float> &positions,
                                const std::vector<float> &radii)
    {
        int64_t n = 0;
        for (int32_t c : counts)
        {
            n += c;
        }
        if (counts.size() != m_wells.size() || static_cast<int64_t>(radii.size()) != n ||
            static_cast<int64_t>(positions.size()) != 2 * n)
        {
            Check(HAL_CUDA_EINVAL, "CudaWells2D::SetAgents: one count per well, two positions and one radius per agent");
        }
        Check(hal_cuda_wells_set_agents(m_pHandle, counts.data(), positions.data(), radii.data()),
              "CudaWells2D::SetAgents");
        m_agents = n;
    }

    void CudaWells2D::RunTicks(int32_t ticks, double interactionRad, double springConstant)
    {
        Check(hal_cuda_wells_run_ticks(m_pHandle, ticks, interactionRad, springConstant), "CudaWells2D::RunTicks");
    }

    void CudaWells2D::GetForces(std::vector<float> &velocityDeltas)
    {
        velocityDeltas.resize(2 * static_cast<size_t>(m_agents));
        Check(hal_cuda_wells_get_forces(m_pHandle, velocityDeltas.data(), static_cast<int64_t>(velocityDeltas.size())),
              "CudaWells2D::GetForces");
    }

    void CudaWells2D::SetMotion(bool enabled, double friction, double maxVel)
    {
        Check(hal_cuda_wells_set_motion(m_pHandle, enabled, friction, maxVel), "CudaWells2D::SetMotion");
    }

    void CudaWells2D::SetVelocities(const std::vector<float> &velocities)
    {
        Check(hal_cuda_wells_set_velocities(m_pHandle, velocities.empty() ? nullptr : velocities.data(),
                                            static_cast<int64_t>(velocities.size())),
              "CudaWells2D::SetVelocities");
    }

    void CudaWells2D::GetAgents(std::vector<float> &positions, std::vector<float> &velocities)
    {
        positions.resize(2 * static_cast<size_t>(m_agents));
        velocities.resize(2 * static_cast<size_t>(m_agents));
        Check(hal_cuda_wells_get_agents(m_pHandle, positions.data(), velocities.data(),
                                        static_cast<int64_t>(positions.size())),
              "CudaWells2D::GetAgents");
    }

    void CudaWells2D::Sync()
    {
        Check(hal_cuda_wells_sync(m_pHandle), "CudaWells2D::Sync");
    }

    // ---- CudaAdjointAdi2D ------------------------------------------------------

    CudaAdjointAdi2D::CudaAdjointAdi2D(int32_t xDim, int32_t yDim, bool wrapX, bool wrapY)
        : m_xDim(xDim), m_yDim(yDim)
    {
        Check(hal_cuda_adjoint_create(xDim, yDim, wrapX, wrapY, &m_pHandle), "CudaAdjointAdi2D");
    }

    CudaAdjointAdi2D::~CudaAdjointAdi2D()
    {
        hal_cuda_adjoint_destroy(m_pHandle);
    }

    void CudaAdjointAdi2D::CheckCells(const std::vector<float> &v, bool allowEmpty, const char *pWhat) const
    {
        const size_t n = static_cast<size_t>(m_xDim) * static_cast<size_t>(m_yDim);
        if (v.size() != n && !(allowEmpty && v.empty()))
        {
            Check(HAL_CUDA_EINVAL, (std::string(pWhat) + ": arrays must hold xDim*yDim values").c_str());
        }
    }

    void CudaAdjointAdi2D::SetProblem(const std::vector<float> &f0, const std::vector<float> &target, int32_t steps,
                                      int32_t checkpointEvery)
    {
        CheckCells(f0, false, "CudaAdjointAdi2D::SetProblem");
        CheckCells(target, false, "CudaAdjointAdi2D::SetProblem");
        Check(hal_cuda_adjoint_set_problem(m_pHandle, f0.data(), target.data(), static_cast<int64_t>(f0.size()), steps,
                                           checkpointEvery),
              "CudaAdjointAdi2D::SetProblem");
    }

    double CudaAdjointAdi2D::Forward(const std::vector<float> &D, double decay, const std::vector<float> &src,
                                     std::vector<float> *pFT)
    {
        CheckCells(D, false, "CudaAdjointAdi2D::Forward");
        CheckCells(src, true, "CudaAdjointAdi2D::Forward");
        double loss = 0.0;
        if (pFT != nullptr)
        {
            pFT->resize(static_cast<size_t>(m_xDim) * static_cast<size_t>(m_yDim));
        }
        Check(hal_cuda_adjoint_forward(m_pHandle, D.data(), decay, src.empty() ? nullptr : src.data(), &loss,
                                       pFT != nullptr ? pFT->data() : nullptr),
              "CudaAdjointAdi2D::Forward");
        return loss;
    }

    double CudaAdjointAdi2D::Backward(const std::vector<float> &D, double decay, const std::vector<float> &src,
                                      std::vector<float> &gradD, double &gradDecay, std::vector<float> &gradSrc)
    {
        CheckCells(D, false, "CudaAdjointAdi2D::Backward");
        CheckCells(src, true, "CudaAdjointAdi2D::Backward");
        const size_t n = static_cast<size_t>(m_xDim) * static_cast<size_t>(m_yDim);
        gradD.resize(n);
        gradSrc.resize(n);
        double loss = 0.0;
        Check(hal_cuda_adjoint_gradient(m_pHandle, D.data(), decay, src.empty() ? nullptr : src.data(), &loss,
                                        gradD.data(), &gradDecay, gradSrc.data()),
              "CudaAdjointAdi2D::Backward");
        return loss;
    }

    void CudaAdjointAdi2D::Times(float &msForward, float &msBackward) const
    {
        Check(hal_cuda_adjoint_times(m_pHandle, &msForward, &msBackward), "CudaAdjointAdi2D::Times");
    }
}
