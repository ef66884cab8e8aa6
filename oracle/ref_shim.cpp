// ref_shim.cpp -- C entry points over the reference's own CPU code.
//
// TEST INFRASTRUCTURE ONLY.  Compiled (by oracle/Makefile) together with the
// reference's CPU sources, read in place from the reference tree, into
// oracle/_ref/libhal_ref.so.  It lets the golden-vector generator
// (tests/golden/make_golden.py) and the oracle pin tests run the reference
// itself: Hal::CpuDiffusionBackend2D, Hal::CpuAdiDiffusionBackend2D,
// Hal::CpuAgentForceBackend2D, Hal::PDEGrid2D and Hal::Rand.  Nothing here is
// part of the product.
#include "Hal/Agents/SphericalAgent2D.h"
#include "Hal/Grids/AgentGrid2D.h"
#include "Hal/Grids/PDEGrid2D.h"
#include "Hal/Grids/PDEGridSerialization.h"
#include "Hal/Pde/ADIequations.h"
#include "Hal/Pde/CpuAdiDiffusionBackend2D.h"
#include "Hal/Pde/CpuDiffusionBackend2D.h"
#include "Hal/Pde/PDEequations.h"
#include "Hal/Pde/TdmaSolver.h"
#include "Hal/Rand.h"
#include "Hal/Log/Logger.h"

// The bins of CpuAgentForceBackend2D are private members; the golden vectors
// for the bit-exact binning check read them straight after AccumulateForces.
#define private public
#include "Hal/Agents/CpuAgentForceBackend2D.h"
#undef private

#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

namespace
{
    // A Dirichlet callable backed by the ghost table layout of hal_oracle.h.
    struct GhostBc
    {
        const double *pGhost;
        int32_t xDim;
        int32_t yDim;

        double operator()(int32_t x, int32_t y) const
        {
            if (x < 0)
            {
                return pGhost[y];
            }
            if (x >= xDim)
            {
                return pGhost[yDim + y];
            }
            if (y < 0)
            {
                return pGhost[2 * yDim + x];
            }
            return pGhost[2 * yDim + xDim + x];
        }
    };

    template <typename Fn>
    int Guard(Fn fn)
    {
        try
        {
            fn();
            return 0;
        }
        catch (const std::invalid_argument &)
        {
            return 1;
        }
        catch (...)
        {
            return 2;
        }
    }

    void Quiet()
    {
        static bool s_done = false;
        if (!s_done)
        {
            // Error-path tests provoke logged errors on purpose.
            Hal::Logger::Instance().SetMinSeverity(Hal::LogSeverity::Error);
            s_done = true;
        }
    }
}

// A minimal off-lattice model on the reference's own agent grid, as in its
// tests (tests/SphericalAgentTests.cpp:9-36).
class ShimCellGrid;

class ShimCell : public Hal::SphericalAgent2D<ShimCellGrid>
{
public:
    explicit ShimCell(ShimCellGrid *pGrid)
        : Hal::SphericalAgent2D<ShimCellGrid>(pGrid)
    {
    }
};

class ShimCellGrid : public Hal::AgentGrid2D<ShimCell, ShimCellGrid>
{
public:
    ShimCellGrid(int32_t xDim, int32_t yDim, bool wrapX, bool wrapY)
        : Hal::AgentGrid2D<ShimCell, ShimCellGrid>(xDim, yDim, wrapX, wrapY)
    {
    }
};

extern "C"
{
    // IDiffusionBackend2D::Diffuse through Hal::CpuDiffusionBackend2D.
    // Internal::Diffusion2 with per-cell rates and the two Advection2 forms
    // (src/Pde/PDEequations.cpp:199-230, 380-412, 535-575).
    int ref_diffuse_var(const double *field, double *deltas, const double *ratesX, const double *ratesY,
                        int32_t xDim, int32_t yDim, int wrapX, int wrapY)
    {
        Quiet();
        return Guard([&]()
                     { Hal::Internal::Diffusion2(field, deltas, ratesX, ratesY, xDim, yDim, wrapX != 0, wrapY != 0); });
    }

    int ref_advect(const double *field, double *deltas, double xVel, double yVel, int32_t xDim, int32_t yDim,
                   int wrapX, int wrapY)
    {
        Quiet();
        return Guard([&]()
                     { Hal::Internal::Advection2(field, deltas, xVel, yVel, xDim, yDim, wrapX != 0, wrapY != 0); });
    }

    int ref_advect_var(const double *field, double *deltas, const double *xVels, const double *yVels, int32_t xDim,
                       int32_t yDim, int wrapX, int wrapY)
    {
        Quiet();
        return Guard([&]()
                     { Hal::Internal::Advection2(field, deltas, xVels, yVels, xDim, yDim, wrapX != 0, wrapY != 0); });
    }

    // Hal::Internal::Advection2<BCFn> with a ghost-table callable.
    int ref_advect_bc(const double *field, double *deltas, double xVel, double yVel, int32_t xDim, int32_t yDim,
                      int wrapX, int wrapY, const double *ghost)
    {
        Quiet();
        return Guard([&]()
                     { Hal::Internal::Advection2(field, deltas, xVel, yVel, xDim, yDim, wrapX != 0, wrapY != 0,
                                                 GhostBc{ghost, xDim, yDim}); });
    }

    // Hal::Internal::Advection2<BCFn, XVelBCFn, YVelBCFn> with three
    // ghost-table callables (field, x velocity, y velocity).
    int ref_advect_var_bc(const double *field, double *deltas, const double *xVels, const double *yVels,
                          int32_t xDim, int32_t yDim, int wrapX, int wrapY, const double *ghost,
                          const double *ghostXVel, const double *ghostYVel)
    {
        Quiet();
        return Guard([&]()
                     { Hal::Internal::Advection2(field, deltas, xVels, yVels, xDim, yDim, wrapX != 0, wrapY != 0,
                                                 GhostBc{ghost, xDim, yDim}, GhostBc{ghostXVel, xDim, yDim},
                                                 GhostBc{ghostYVel, xDim, yDim}); });
    }

    // One agent update of a SphericalAgent2D model after its forces
    // (include/Hal/Agents/SphericalAgent2D.h:133-162): SetVelocity(vel +
    // delta), CapVelocity(maxVel) when maxVel >= 0, ForceMove (MoveSafePT),
    // ApplyFriction(friction).  Each agent is placed alone on the grid, moved
    // and disposed of, so the agents do not interact here.
    int ref_agents_move(double *pos, double *vel, const double *deltas, int32_t n, int32_t xDim, int32_t yDim,
                        int wrapX, int wrapY, double friction, double maxVel)
    {
        Quiet();
        return Guard([&]()
                     {
            ShimCellGrid grid(xDim, yDim, wrapX != 0, wrapY != 0);
            for (int32_t i = 0; i < n; i++)
            {
                ShimCell &a = grid.NewAgentPT(pos[2 * i], pos[2 * i + 1]);
                a.DefaultInit(0.5);
                a.SetVelocity(vel[2 * i] + deltas[2 * i], vel[2 * i + 1] + deltas[2 * i + 1]);
                if (maxVel >= 0)
                {
                    a.CapVelocity(maxVel);
                }
                a.ForceMove();
                a.ApplyFriction(friction);
                pos[2 * i] = a.Xpt();
                pos[2 * i + 1] = a.Ypt();
                vel[2 * i] = a.XVel();
                vel[2 * i + 1] = a.YVel();
                a.Dispose();
            } });
    }

    // SphericalAgent2D::SumForces (include/Hal/Agents/SphericalAgent2D.h:
    // 74-102) of every agent on the reference's own agent grid: the agents
    // are created in index order with their radii and velocities, then each
    // calls SumForces(interactionRad, law) in index order.  law 0: linear
    // scale*touchDist; 1: clamped as examples/OffLatticeExample.cpp:147-154;
    // 2: pow(scale*touchDist, exponent) as examples/Chemotaxis.cpp:128-130.
    // velOut receives the velocities after the call, sums the returned values.
    int ref_sum_forces(const double *pos, const double *rad, const double *velIn, int32_t n, int32_t xDim,
                       int32_t yDim, int wrapX, int wrapY, double interactionRad, int law, double scale,
                       double exponent, double *velOut, double *sums)
    {
        Quiet();
        return Guard([&]()
                     {
            ShimCellGrid grid(xDim, yDim, wrapX != 0, wrapY != 0);
            std::vector<ShimCell *> agents(static_cast<size_t>(n));
            for (int32_t i = 0; i < n; i++)
            {
                ShimCell &a = grid.NewAgentPT(pos[2 * i], pos[2 * i + 1]);
                a.DefaultInit(rad[i]);
                if (velIn != nullptr)
                {
                    a.SetVelocity(velIn[2 * i], velIn[2 * i + 1]);
                }
                agents[static_cast<size_t>(i)] = &a;
            }
            for (int32_t i = 0; i < n; i++)
            {
                ShimCell &a = *agents[static_cast<size_t>(i)];
                double sum = 0;
                if (law == 1)
                {
                    sum = a.SumForces(interactionRad, [scale](double overlap, ShimCell &)
                                      {
                        if (overlap < 0)
                        {
                            return 0.0;
                        }
                        return scale * overlap; });
                }
                else if (law == 2)
                {
                    sum = a.SumForces(interactionRad, [scale, exponent](double overlap, ShimCell &)
                                      { return std::pow(scale * overlap, exponent); });
                }
                else
                {
                    sum = a.SumForces(interactionRad, [scale](double overlap, ShimCell &)
                                      { return scale * overlap; });
                }
                velOut[2 * i] = a.XVel();
                velOut[2 * i + 1] = a.YVel();
                sums[i] = sum;
            } });
    }

    // A script of calls on the reference's own Hal::PDEGrid2D, in the
    // encoding of oracle_pdegrid_script (hal_oracle.h): the grid starts in
    // the given state, every call runs in order, query results go to
    // records, and the final state is written back.  Returns the number of
    // records through nRec.
    int ref_pdegrid_script(int32_t xDim, int32_t yDim, int wrapX, int wrapY, double *field, double *deltas,
                           int32_t *updateCt, int32_t nOps, const int32_t *ops, const int32_t *iargs,
                           const double *dargs, const double *arrays, double *records, int32_t *nRec)
    {
        Quiet();
        return Guard([&]()
                     {
            const size_t length = static_cast<size_t>(xDim) * static_cast<size_t>(yDim);
            Hal::PDEGrid2D grid(xDim, yDim, wrapX != 0, wrapY != 0);
            grid.SetState(std::vector<double>(field, field + length), std::vector<double>(deltas, deltas + length),
                          *updateCt);
            const int32_t g = 2 * (xDim + yDim);
            int32_t r = 0;
            for (int32_t k = 0; k < nOps; k++)
            {
                const int32_t *ia = iargs + 3 * static_cast<size_t>(k);
                const double *da = dargs + 2 * static_cast<size_t>(k);
                const double *arr = arrays + ia[0];
                const std::vector<double> a0(arr, arr + length);
                switch (ops[k])
                {
                case 0: grid.Set(ia[1], da[0]); break;
                case 1: grid.Add(ia[1], da[0]); break;
                case 2: grid.Mul(ia[1], da[0]); break;
                case 3: grid.Scale(ia[1], da[0]); break;
                case 10: grid.SetAll(da[0]); break;
                case 11: grid.AddAll(da[0]); break;
                case 12: grid.MulAll(da[0]); break;
                case 13: grid.SetAll(arr); break;
                case 20: grid.Diffusion(da[0]); break;
                case 21: grid.Diffusion(da[0], GhostBc{arr, xDim, yDim}); break;
                case 22: grid.Diffusion(a0, std::vector<double>(arr + length, arr + 2 * length)); break;
                case 30: grid.DiffusionADI(da[0]); break;
                case 31: grid.DiffusionADI(da[0], GhostBc{arr, xDim, yDim}); break;
                case 40: grid.Advection(da[0], da[1]); break;
                case 41: grid.Advection(da[0], da[1], GhostBc{arr, xDim, yDim}); break;
                case 42: grid.Advection(a0, std::vector<double>(arr + length, arr + 2 * length)); break;
                case 43:
                    grid.Advection(a0, std::vector<double>(arr + length, arr + 2 * length),
                                   GhostBc{arr + 2 * length, xDim, yDim}, GhostBc{arr + 2 * length + g, xDim, yDim},
                                   GhostBc{arr + 2 * length + 2 * g, xDim, yDim});
                    break;
                case 50: grid.Update(); break;
                case 51: grid.SetNonNegative(); break;
                case 60: records[r++] = grid.Get(ia[1]); break;
                case 61: records[r++] = grid.GetMax(); break;
                case 62: records[r++] = grid.GetMin(); break;
                case 63: records[r++] = grid.GetAvg(); break;
                case 64: records[r++] = grid.MaxDelta(); break;
                case 65: records[r++] = grid.MaxDeltaScaled(da[0]); break;
                case 66: records[r++] = grid.GradientX(ia[1], ia[2]); break;
                case 67: records[r++] = grid.GradientY(ia[1], ia[2]); break;
                case 68: records[r++] = grid.GradientX(ia[1], ia[2], da[0]); break;
                case 69: records[r++] = grid.GradientY(ia[1], ia[2], da[0]); break;
                default: throw std::runtime_error("unknown script op");
                }
            }
            std::memcpy(field, grid.GetField().data(), sizeof(double) * length);
            std::memcpy(deltas, grid.GetDeltas().data(), sizeof(double) * length);
            *updateCt = grid.UpdateCt();
            *nRec = r; });
    }

    // Hal::SavePDEGrid2D of a grid in the given state, through BinaryWriter.
    int ref_pdegrid2d_save(const char *path, int32_t xDim, int32_t yDim, int wrapX, int wrapY, int32_t updateCt,
                           const double *field, const double *deltas)
    {
        Quiet();
        return Guard([&]()
                     {
            const size_t n = static_cast<size_t>(xDim) * static_cast<size_t>(yDim);
            Hal::PDEGrid2D grid(xDim, yDim, wrapX != 0, wrapY != 0);
            grid.SetState(std::vector<double>(field, field + n), std::vector<double>(deltas, deltas + n), updateCt);
            Hal::BinaryWriter writer(path);
            Hal::SavePDEGrid2D(writer, grid);
            if (!writer.IsGood())
            {
                throw std::runtime_error("write failed");
            } });
    }

    // Hal::LoadPDEGrid2D: the grid's sizes, flags, update count, field and
    // deltas (field/deltas hold at most cap values).
    int ref_pdegrid2d_load(const char *path, int32_t *dims, int32_t *updateCt, double *field, double *deltas,
                           int64_t cap)
    {
        Quiet();
        return Guard([&]()
                     {
            Hal::BinaryReader reader(path);
            Hal::PDEGrid2D grid = Hal::LoadPDEGrid2D(reader);
            dims[0] = grid.Xdim();
            dims[1] = grid.Ydim();
            dims[2] = grid.IsWrapX();
            dims[3] = grid.IsWrapY();
            *updateCt = grid.UpdateCt();
            const std::vector<double> &f = grid.GetField();
            const std::vector<double> &d = grid.GetDeltas();
            if (static_cast<int64_t>(f.size()) > cap)
            {
                throw std::runtime_error("grid larger than the buffers");
            }
            std::memcpy(field, f.data(), f.size() * sizeof(double));
            std::memcpy(deltas, d.data(), d.size() * sizeof(double)); });
    }

    int ref_diffuse(const double *field, int64_t fieldLen, double *deltas, int64_t deltasLen,
                    double diffRate, int32_t xDim, int32_t yDim, int wrapX, int wrapY)
    {
        Quiet();
        return Guard([&]()
                     {
            std::vector<double> f(field, field + fieldLen);
            std::vector<double> d(deltas, deltas + deltasLen);
            Hal::CpuDiffusionBackend2D backend;
            backend.Diffuse(f, d, diffRate, xDim, yDim, wrapX != 0, wrapY != 0);
            std::memcpy(deltas, d.data(), sizeof(double) * d.size()); });
    }

    // Hal::Internal::Diffusion2<BCFn> with a ghost-table callable.
    int ref_diffuse_bc(const double *field, double *deltas, double diffRate, int32_t xDim,
                       int32_t yDim, int wrapX, int wrapY, const double *ghost)
    {
        Quiet();
        return Guard([&]()
                     { Hal::Internal::Diffusion2(field, deltas, diffRate, xDim, yDim, wrapX != 0, wrapY != 0,
                                                 GhostBc{ghost, xDim, yDim}); });
    }

    // IAdiDiffusionBackend2D::DiffuseADI through Hal::CpuAdiDiffusionBackend2D.
    int ref_diffuse_adi(const double *field, int64_t fieldLen, double *deltas, int64_t deltasLen,
                        double diffRate, int32_t xDim, int32_t yDim, int wrapX, int wrapY)
    {
        Quiet();
        return Guard([&]()
                     {
            std::vector<double> f(field, field + fieldLen);
            std::vector<double> d(deltas, deltas + deltasLen);
            Hal::CpuAdiDiffusionBackend2D backend;
            backend.DiffuseADI(f, d, diffRate, xDim, yDim, wrapX != 0, wrapY != 0);
            std::memcpy(deltas, d.data(), sizeof(double) * d.size()); });
    }

    // Hal::Internal::Diffusion2DADI<BCFn> with a ghost-table callable.
    int ref_diffuse_adi_bc(const double *field, double *deltas, double diffRate, int32_t xDim,
                           int32_t yDim, int wrapX, int wrapY, const double *ghost)
    {
        Quiet();
        return Guard([&]()
                     {
            std::vector<double> scratch(static_cast<size_t>(xDim) * static_cast<size_t>(yDim), 0.0);
            Hal::TdmaSolver tdma(xDim > yDim ? xDim : yDim);
            Hal::Internal::Diffusion2DADI(field, scratch.data(), deltas, diffRate, xDim, yDim, wrapX != 0,
                                          wrapY != 0, GhostBc{ghost, xDim, yDim}, tdma); });
    }

    // A HAL model's tick loop on Hal::PDEGrid2D: mode 0 = Diffusion, 1 =
    // DiffusionADI; then MulAll(-decay), Add(dense), Add(points),
    // Mul(cell,-uptake) per agent, Update().  field is updated in place.
    int ref_pdegrid_run(int mode, double *field, int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                        double diffRate, const double *ghost, double decay, const double *srcDense,
                        int32_t nSrc, const int32_t *srcIdx, const double *srcVal,
                        const int32_t *uptakeCount, double uptake, int32_t ticks)
    {
        Quiet();
        return Guard([&]()
                     {
            Hal::PDEGrid2D grid(xDim, yDim, wrapX != 0, wrapY != 0);
            int32_t length = xDim * yDim;
            std::vector<double> f(field, field + length);
            std::vector<double> zeros(static_cast<size_t>(length), 0.0);
            grid.SetState(f, zeros, 0);
            GhostBc bc{ghost, xDim, yDim};
            for (int32_t t = 0; t < ticks; t++)
            {
                if (mode == 0)
                {
                    if (ghost != nullptr)
                    {
                        grid.Diffusion(diffRate, bc);
                    }
                    else
                    {
                        grid.Diffusion(diffRate);
                    }
                }
                else
                {
                    if (ghost != nullptr)
                    {
                        grid.DiffusionADI(diffRate, bc);
                    }
                    else
                    {
                        grid.DiffusionADI(diffRate);
                    }
                }
                if (decay != 0.0)
                {
                    grid.MulAll(-decay);
                }
                if (srcDense != nullptr)
                {
                    for (int32_t i = 0; i < length; i++)
                    {
                        grid.Add(i, srcDense[i]);
                    }
                }
                for (int32_t k = 0; k < nSrc; k++)
                {
                    grid.Add(srcIdx[k], srcVal[k]);
                }
                if (uptakeCount != nullptr)
                {
                    for (int32_t i = 0; i < length; i++)
                    {
                        for (int32_t a = 0; a < uptakeCount[i]; a++)
                        {
                            grid.Mul(i, -uptake);
                        }
                    }
                }
                grid.Update();
            }
            std::memcpy(field, grid.GetField().data(), sizeof(double) * static_cast<size_t>(length)); });
    }

    // The same tick loop with PDEGrid2D::Advection(xVel, yVel[, bc]) after
    // the diffusion term.
    int ref_pdegrid_run_adv(int mode, double *field, int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                            double diffRate, double xVel, double yVel, const double *ghost, double decay, const double *srcDense,
                        int32_t nSrc, const int32_t *srcIdx, const double *srcVal,
                        const int32_t *uptakeCount, double uptake, int32_t ticks)
    {
        Quiet();
        return Guard([&]()
                     {
            Hal::PDEGrid2D grid(xDim, yDim, wrapX != 0, wrapY != 0);
            int32_t length = xDim * yDim;
            std::vector<double> f(field, field + length);
            std::vector<double> zeros(static_cast<size_t>(length), 0.0);
            grid.SetState(f, zeros, 0);
            GhostBc bc{ghost, xDim, yDim};
            for (int32_t t = 0; t < ticks; t++)
            {
                if (mode == 0)
                {
                    if (ghost != nullptr)
                    {
                        grid.Diffusion(diffRate, bc);
                    }
                    else
                    {
                        grid.Diffusion(diffRate);
                    }
                }
                else
                {
                    if (ghost != nullptr)
                    {
                        grid.DiffusionADI(diffRate, bc);
                    }
                    else
                    {
                        grid.DiffusionADI(diffRate);
                    }
                }
                if (xVel != 0.0 || yVel != 0.0)
                {
                    if (ghost != nullptr)
                    {
                        grid.Advection(xVel, yVel, bc);
                    }
                    else
                    {
                        grid.Advection(xVel, yVel);
                    }
                }
                if (decay != 0.0)
                {
                    grid.MulAll(-decay);
                }
                if (srcDense != nullptr)
                {
                    for (int32_t i = 0; i < length; i++)
                    {
                        grid.Add(i, srcDense[i]);
                    }
                }
                for (int32_t k = 0; k < nSrc; k++)
                {
                    grid.Add(srcIdx[k], srcVal[k]);
                }
                if (uptakeCount != nullptr)
                {
                    for (int32_t i = 0; i < length; i++)
                    {
                        for (int32_t a = 0; a < uptakeCount[i]; a++)
                        {
                            grid.Mul(i, -uptake);
                        }
                    }
                }
                grid.Update();
            }
            std::memcpy(field, grid.GetField().data(), sizeof(double) * static_cast<size_t>(length)); });
    }

    // IAgentForceBackend2D::AccumulateForces through
    // Hal::CpuAgentForceBackend2D; also returns its bins.  cellOffsets holds
    // xDim*yDim+1 entries and bucketAgents n entries (either may be null).
    int ref_accumulate_forces(const double *positions, int64_t posLen, const double *radii,
                              int64_t radLen, double *velocityDeltas, double interactionRad,
                              double springConstant, int32_t xDim, int32_t yDim, int wrapX, int wrapY,
                              int32_t *cellOffsets, int32_t *bucketAgents)
    {
        Quiet();
        return Guard([&]()
                     {
            std::vector<double> p(positions, positions + posLen);
            std::vector<double> r(radii, radii + radLen);
            std::vector<double> out;
            Hal::CpuAgentForceBackend2D backend;
            backend.AccumulateForces(p, r, out, interactionRad, springConstant, xDim, yDim, wrapX != 0,
                                     wrapY != 0);
            std::memcpy(velocityDeltas, out.data(), sizeof(double) * out.size());
            if (cellOffsets != nullptr)
            {
                std::memcpy(cellOffsets, backend.m_cellOffsets.data(),
                            sizeof(int32_t) * backend.m_cellOffsets.size());
            }
            if (bucketAgents != nullptr)
            {
                std::memcpy(bucketAgents, backend.m_bucketAgents.data(),
                            sizeof(int32_t) * backend.m_bucketAgents.size());
            } });
    }

    // Hal::Rand draws: kind 0 = Double(), 1 = Int(bound), 2 = Gaussian(0, 1).
    void ref_rand_draws(uint64_t seed, int kind, int32_t bound, int32_t n, double *out)
    {
        Hal::Rand rand(seed);
        for (int32_t i = 0; i < n; i++)
        {
            if (kind == 0)
            {
                out[i] = rand.Double();
            }
            else if (kind == 1)
            {
                out[i] = static_cast<double>(rand.Int(bound));
            }
            else
            {
                out[i] = rand.Gaussian(0.0, 1.0);
            }
        }
    }
}
