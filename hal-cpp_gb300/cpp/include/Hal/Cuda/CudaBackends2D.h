#pragma once

// CUDA (sm_103a) implementations of HAL-CPP's three per-tick strategy
// interfaces, over the C ABI in hal_cuda.h.  They stand where the Vulkan
// classes Hal::Gpu::GpuDiffusionBackend2D / GpuAdiDiffusionBackend2D /
// GpuAgentForceBackend2D stand (src/Gpu/GpuDiffusionBackend2D.cpp:22-52,
// GpuAdiDiffusionBackend2D.cpp:24-50, GpuAgentForceBackend2D.cpp:24-68):
// sized at construction, copy-deleted, and throwing std::invalid_argument
// for size mismatches and std::runtime_error for device failures, after
// logging through Hal::Logger (IDiffusionBackend2D.cpp:26-31,
// AdiKernel2D.cpp:66-70).  No ComputeContext: hal_cuda_set_device picks the
// GPU for handles created afterwards on the calling thread.
//
// Beyond the interfaces, each class exposes the device-resident tick that
// PDEGrid2D performs on the host (PDEGrid2D.h:103-186): set the field,
// sources and Dirichlet values once, run many ticks, read the field back.

#include "Hal/Agents/IAgentForceBackend2D.h"
#include "Hal/Pde/IAdiDiffusionBackend2D.h"
#include "Hal/Pde/IDiffusionBackend2D.h"

#include "hal_cuda.h"

#include <cstdint>
#include <vector>

namespace Hal::Cuda
{
    // Logs and throws for a non-OK status: std::invalid_argument for
    // HAL_CUDA_EINVAL, std::runtime_error otherwise.
    void Check(int status, const char *pWhat);

    // Selects the CUDA device for backends constructed afterwards on this
    // thread.
    void SetDevice(int32_t device);

    class CudaAgentForceBackend2D;

    class CudaDiffusionBackend2D final : public IDiffusionBackend2D
    {
    public:
        CudaDiffusionBackend2D(int32_t xDim, int32_t yDim);
        ~CudaDiffusionBackend2D() override;

        // IDiffusionBackend2D::Diffuse: deltas += one explicit step, FP64,
        // bit-identical to CpuDiffusionBackend2D.
        void Diffuse(const std::vector<double> &field,
                     std::vector<double>       &deltas,
                     double                     diffRate,
                     int32_t                    xDim,
                     int32_t                    yDim,
                     bool                       wrapX,
                     bool                       wrapY) override;

        // Internal::Diffusion2<BCFn> with the Dirichlet callable given as its
        // ghost table (2*yDim + 2*xDim values: bc(-1,y), bc(xDim,y),
        // bc(x,-1), bc(x,yDim)); an empty table means zero-flux.
        void DiffuseDirichlet(const std::vector<double> &field,
                              std::vector<double>       &deltas,
                              double                     diffRate,
                              bool                       wrapX,
                              bool                       wrapY,
                              const std::vector<double> &ghost);

        // Internal::Diffusion2 with per-cell rates (src/Pde/PDEequations.cpp:
        // 199-230); FP64, bit-identical to the CPU code.
        void DiffuseVariable(const std::vector<double> &field,
                             std::vector<double>       &deltas,
                             const std::vector<double> &diffRatesX,
                             const std::vector<double> &diffRatesY,
                             bool                       wrapX,
                             bool                       wrapY);

        // Internal::Advection2 at a uniform velocity (src/Pde/
        // PDEequations.cpp:380-412) or, with a non-empty ghost table, its
        // Dirichlet form (include/Hal/Pde/PDEequations.h:413-447).
        void Advect(const std::vector<double> &field,
                    std::vector<double>       &deltas,
                    double                     xVel,
                    double                     yVel,
                    bool                       wrapX,
                    bool                       wrapY,
                    const std::vector<double> &ghost = {});

        // Internal::Advection2 with per-cell velocities (src/Pde/
        // PDEequations.cpp:535-575) or, with ghost tables for the field and
        // the two velocity components, its Dirichlet form (:720-778).
        void AdvectVariable(const std::vector<double> &field,
                            std::vector<double>       &deltas,
                            const std::vector<double> &xVels,
                            const std::vector<double> &yVels,
                            bool                       wrapX,
                            bool                       wrapY,
                            const std::vector<double> &ghost = {},
                            const std::vector<double> &ghostXVel = {},
                            const std::vector<double> &ghostYVel = {});

        // Device-resident PDEGrid2D tick:
        // f' = f + r L(f) - decay f + src - uptake * (agents in the cell) * f.
        void SetField(const std::vector<float> &field);
        void GetField(std::vector<float> &field);
        void SetSource(const std::vector<float> &dense);
        void SetPointSources(const std::vector<int32_t> &cells, const std::vector<float> &values);
        void SetDirichlet(const std::vector<float> &ghost);
        // PDEGrid2D::Advection(xVel, yVel) in every following tick (upwind).
        void SetVelocity(double xVel, double yVel);
        // PDEGrid2D::Mul(cell, -uptake) once per agent of pAgents' last
        // binning, every following tick (nullptr removes the coupling).
        void SetUptake(CudaAgentForceBackend2D *pAgents, double uptake);
        void RunTicks(int32_t ticks, double diffRate, double decay, bool wrapX, bool wrapY);
        void Sync();

        // DiffusionKernel2D::RunSteps: upload, `steps` plain steps, download.
        void RunSteps(std::vector<float> &field, int32_t steps, double diffRate, bool wrapX, bool wrapY);

        int32_t XDim() const { return m_xDim; }
        int32_t YDim() const { return m_yDim; }

    private:
        hal_cuda_diffusion *m_pHandle = nullptr;
        int32_t             m_xDim;
        int32_t             m_yDim;
    };

    class CudaAdiDiffusionBackend2D final : public IAdiDiffusionBackend2D
    {
    public:
        CudaAdiDiffusionBackend2D(int32_t xDim, int32_t yDim);
        ~CudaAdiDiffusionBackend2D() override;

        // IAdiDiffusionBackend2D::DiffuseADI: deltas += one ADI step.
        void DiffuseADI(const std::vector<double> &field,
                        std::vector<double>       &deltas,
                        double                     diffRate,
                        int32_t                    xDim,
                        int32_t                    yDim,
                        bool                       wrapX,
                        bool                       wrapY) override;

        // Internal::Diffusion2DADI<BCFn> with a Dirichlet ghost table.
        void DiffuseADIDirichlet(const std::vector<double> &field,
                                 std::vector<double>       &deltas,
                                 double                     diffRate,
                                 bool                       wrapX,
                                 bool                       wrapY,
                                 const std::vector<double> &ghost);

        // exact: DiffuseADI and DiffuseADIDirichlet solve every size in
        // FP64, bit-exact to CpuAdiDiffusionBackend2D (default false: FP32
        // for sides up to HAL_CUDA_ADI_MAX_LINE).
        void SetExact(bool exact);

        // Device-resident PDEGrid2D::DiffusionADI tick:
        // f' = ADI(f) - decay f + src - uptake * (agents in the cell) * f.
        void SetField(const std::vector<float> &field);
        void GetField(std::vector<float> &field);
        void SetSource(const std::vector<float> &dense);
        void SetDirichlet(const std::vector<float> &ghost);
        void SetUptake(CudaAgentForceBackend2D *pAgents, double uptake);
        // `ticks` coupled ticks (the agents' resident step, then this field's
        // tick with their uptake) as one graph; agents must be the coupled
        // backend (SetUptake).  Equal to alternating agents.Step(1, ...) and
        // RunTicks(1, ...).
        void RunCoupled(CudaAgentForceBackend2D &agents, int32_t ticks, double diffRate, double decay, bool wrapX,
                        bool wrapY, double interactionRad, double springConstant, double friction, double maxVel);
        void RunTicks(int32_t ticks, double diffRate, double decay, bool wrapX, bool wrapY);
        void Sync();

        // AdiKernel2D::RunSteps: upload, `steps` plain ADI steps, download.
        void RunSteps(std::vector<float> &field, int32_t steps, double diffRate, bool wrapX, bool wrapY);

        int32_t XDim() const { return m_xDim; }
        int32_t YDim() const { return m_yDim; }

    private:
        hal_cuda_adi *m_pHandle = nullptr;
        int32_t       m_xDim;
        int32_t       m_yDim;
    };

    class CudaAgentForceBackend2D final : public IAgentForceBackend2D
    {
    public:
        CudaAgentForceBackend2D(int32_t xDim, int32_t yDim, int32_t maxAgents);
        ~CudaAgentForceBackend2D() override;

        // IAgentForceBackend2D::AccumulateForces: velocityDeltas resized to
        // positions.size() and overwritten.  Bins and forces are
        // bit-identical to the CPU backend's (FP64 throughout).
        void AccumulateForces(const std::vector<double> &positions,
                              const std::vector<double> &radii,
                              std::vector<double>       &velocityDeltas,
                              double                     interactionRad,
                              double                     springConstant,
                              int32_t                    xDim,
                              int32_t                    yDim,
                              bool                       wrapX,
                              bool                       wrapY) override;

        // SphericalAgent2D::SumForces (include/Hal/Agents/SphericalAgent2D.h:
        // 74-102) of every agent, FP64: velocities (2n, the agents' xVel/yVel;
        // empty for zeros) are updated in place with each neighbour's
        // -(disp/d) * law(touchDist), and forceSums (resized to n) receives
        // the sums of positive forces SumForces returns.  `order` is
        // HAL_CUDA_ORDER_AGENTGRID (an AgentGrid2D filled in index order:
        // bit-identical for the linear and clamped laws) or
        // HAL_CUDA_ORDER_BACKEND.  The law replaces the overlap functor.
        void SumForces(const std::vector<double> &positions,
                       const std::vector<double> &radii,
                       std::vector<double>       &velocities,
                       std::vector<double>       &forceSums,
                       double                     interactionRad,
                       const hal_cuda_force_law  &law,
                       int32_t                    xDim,
                       int32_t                    yDim,
                       bool                       wrapX,
                       bool                       wrapY,
                       int32_t                    order = HAL_CUDA_ORDER_AGENTGRID);

        // AgentForceKernel2D's resident form (FP32): upload, dispatch, download.
        void Upload(const std::vector<float> &positions, const std::vector<float> &radii);
        void Dispatch(double interactionRad, double springConstant, bool wrapX, bool wrapY);
        void Download(std::vector<float> &velocityDeltas);
        // Cell offsets (xDim*yDim + 1) and the agent order of the last binning.
        void GetBins(std::vector<int32_t> &cellOffsets, std::vector<int32_t> &bucketAgents);

        // Device-resident SphericalAgent2D ticks (SphericalAgent2D.h:133-162):
        // each tick computes the forces, then per agent vel += delta,
        // CapVelocity(maxVel) when maxVel >= 0, ForceMove (MoveSafePT) and
        // ApplyFriction(friction).  Upload sets the velocities to zero.
        void SetVelocities(const std::vector<float> &velocities);
        void Step(int32_t ticks, double interactionRad, double springConstant, bool wrapX, bool wrapY,
                  double friction, double maxVel = -1.0);
        // The resident dispatch and step with a force law in place of the
        // linear spring; with withSums the kernel also keeps each agent's sum
        // of positive forces (FP32), which GetForceSums downloads, e.g. to gate
        // division as OffLatticeExample.cpp:156-165 does.
        void DispatchLaw(double interactionRad, const hal_cuda_force_law &law, bool withSums, bool wrapX, bool wrapY);
        void StepLaw(int32_t ticks, double interactionRad, const hal_cuda_force_law &law, bool withSums, bool wrapX,
                     bool wrapY, double friction, double maxVel = -1.0);
        void GetForceSums(std::vector<float> &forceSums);
        void GetState(std::vector<float> &positions, std::vector<float> &velocities);

        hal_cuda_agents *Handle() const { return m_pHandle; }

    private:
        hal_cuda_agents *m_pHandle = nullptr;
        int32_t          m_xDim;
        int32_t          m_yDim;
        int32_t          m_maxAgents;
        int32_t          m_count = 0;
    };

    // Many independent wells (MultiWellExperiment::Step, include/Hal/Tools/
    // MultiWellExperiment.h:83-103) advanced together: each tick runs every
    // well's field tick and agent force pass in a few batched launches
    // replayed from a CUDA graph.  Each well equals its own single-grid run.
    class CudaWells2D
    {
    public:
        explicit CudaWells2D(const std::vector<hal_cuda_well_desc> &wells);
        ~CudaWells2D();
        CudaWells2D(const CudaWells2D &) = delete;
        CudaWells2D &operator=(const CudaWells2D &) = delete;

        void SetField(int32_t well, const std::vector<float> &field);
        void GetField(int32_t well, std::vector<float> &field);
        void SetSource(int32_t well, const std::vector<float> &dense);  // empty: no source
        // counts[w] agents per well; positions (x, y interleaved) and radii
        // concatenated in well order, in each well's own coordinates.
        void SetAgents(const std::vector<int32_t> &counts, const std::vector<float> &positions,
                       const std::vector<float> &radii);
        void RunTicks(int32_t ticks, double interactionRad, double springConstant);
        void GetForces(std::vector<float> &velocityDeltas);
        // Agents move after their forces each tick (SphericalAgent2D's update,
        // as CudaAgentForceBackend2D::Step), each within its own well.
        void SetMotion(bool enabled, double friction, double maxVel = -1.0);
        void SetVelocities(const std::vector<float> &velocities);
        void GetAgents(std::vector<float> &positions, std::vector<float> &velocities);
        void Sync();

        hal_cuda_wells *Handle() const { return m_pHandle; }

    private:
        hal_cuda_wells                *m_pHandle = nullptr;
        std::vector<hal_cuda_well_desc> m_wells;
        int64_t                        m_agents = 0;
    };

    // Forward / backward API of the variable-rate ADI (a rate D per cell, the
    // face convention of Internal::Diffusion2 with per-cell rates,
    // src/Pde/PDEequations.cpp:199-230) over `steps` PDEGrid2D ticks:
    // Forward gives loss = 1/2 |f_T - target|^2, Backward its gradient with
    // respect to D, decay and the source, by adjoint kernels over states
    // recomputed from checkpoints every `checkpointEvery` steps (0 keeps
    // every state).  The reference has no counterpart.
    class CudaAdjointAdi2D
    {
    public:
        CudaAdjointAdi2D(int32_t xDim, int32_t yDim, bool wrapX, bool wrapY);
        ~CudaAdjointAdi2D();
        CudaAdjointAdi2D(const CudaAdjointAdi2D &) = delete;
        CudaAdjointAdi2D &operator=(const CudaAdjointAdi2D &) = delete;

        void SetProblem(const std::vector<float> &f0, const std::vector<float> &target, int32_t steps,
                        int32_t checkpointEvery);
        // Returns the loss; fT (optional) receives the final field.  An empty
        // src means no source.
        double Forward(const std::vector<float> &D, double decay, const std::vector<float> &src,
                       std::vector<float> *pFT = nullptr);
        // Returns the loss and fills the three gradients.
        double Backward(const std::vector<float> &D, double decay, const std::vector<float> &src,
                        std::vector<float> &gradD, double &gradDecay, std::vector<float> &gradSrc);
        // Device ms of the last Forward and Backward.
        void Times(float &msForward, float &msBackward) const;

    private:
        void CheckCells(const std::vector<float> &v, bool allowEmpty, const char *pWhat) const;

        hal_cuda_adjoint *m_pHandle = nullptr;
        int32_t           m_xDim;
        int32_t           m_yDim;
    };
}
