// Tests of the Hal::Cuda backends through HAL's strategy interfaces, in the
// shape of the reference's own interface tests: every check runs against an
// IDiffusionBackend2D& / IAdiDiffusionBackend2D& / IAgentForceBackend2D&
// (tests/IDiffusionBackend2DTests.cpp:23-144,
// tests/IAgentForceBackend2DTests.cpp:25-165, tests/AdiKernel2DTests.cpp:18-141),
// with the CPU oracle (oracle/hal_oracle.h) as the checker where the
// reference compares against its CPU backend.
//
// Prints one line per check and "backend_tests: N passed, M failed"; the exit
// status is 0 only if every check passed.
#include "Hal/Cuda/CudaBackends2D.h"
#include "Hal/Cuda/CudaPDEGrid2D.h"

extern "C"
{
#include "hal_oracle.h"
}

#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

namespace
{
    int g_passed = 0;
    int g_failed = 0;

    void Report(const char *pName, bool ok, const std::string &detail)
    {
        std::printf("%s %s %s\n", ok ? "PASS" : "FAIL", pName, detail.c_str());
        (ok ? g_passed : g_failed)++;
    }

    void Run(const char *pName, const std::function<std::string()> &body)
    {
        try
        {
            std::string err = body();
            Report(pName, err.empty(), err);
        }
        catch (const std::exception &e)
        {
            Report(pName, false, std::string("exception: ") + e.what());
        }
    }

    double MaxAbs(const std::vector<double> &a)
    {
        double m = 0.0;
        for (double v : a)
        {
            m = std::fmax(m, std::fabs(v));
        }
        return m;
    }

    double MaxAbsDiff(const std::vector<double> &a, const std::vector<double> &b)
    {
        double m = 0.0;
        for (size_t i = 0; i < a.size(); i++)
        {
            m = std::fmax(m, std::fabs(a[i] - b[i]));
        }
        return m;
    }

    std::string Fmt(const char *pFmt, double v)
    {
        char buf[128];
        std::snprintf(buf, sizeof(buf), pFmt, v);
        return buf;
    }

    // cos(2 pi x / nx) cos(2 pi y / ny): an eigenvector of both axis
    // Laplacians on a periodic grid.
    std::vector<double> Eigenmode(int32_t nx, int32_t ny)
    {
        std::vector<double> f(static_cast<size_t>(nx) * ny);
        const double pi = 3.14159265358979323846;
        for (int32_t x = 0; x < nx; x++)
        {
            for (int32_t y = 0; y < ny; y++)
            {
                f[static_cast<size_t>(x) * ny + y] = std::cos(2 * pi * x / nx) * std::cos(2 * pi * y / ny);
            }
        }
        return f;
    }

    // Explicit step: one Diffuse on the eigenmode scales it by
    // 1 - 4 r (sin^2(pi/nx) + sin^2(pi/ny)); the result also equals the CPU
    // stencil bit for bit.
    std::string ExplicitEigenmode(Hal::IDiffusionBackend2D &backend)
    {
        const int32_t nx = 16, ny = 20;
        const double r = 0.05;
        const double pi = 3.14159265358979323846;
        std::vector<double> f = Eigenmode(nx, ny);
        std::vector<double> d(f.size(), 0.0);
        backend.Diffuse(f, d, r, nx, ny, true, true);
        const double sx = std::sin(pi / nx), sy = std::sin(pi / ny);
        const double lambda = 1.0 - 4.0 * r * (sx * sx + sy * sy);
        double err = 0.0;
        for (size_t i = 0; i < f.size(); i++)
        {
            err = std::fmax(err, std::fabs(f[i] + d[i] - lambda * f[i]));
        }
        std::vector<double> exp(f.size(), 0.0);
        oracle_diffusion2(f.data(), exp.data(), r, nx, ny, 1, 1, nullptr);
        if (err > 1e-4)
        {
            return Fmt("eigenmode error %.3e > 1e-4", err);
        }
        if (std::memcmp(exp.data(), d.data(), d.size() * sizeof(double)) != 0)
        {
            return "deltas differ from the CPU stencil";
        }
        return "";
    }

    // ADI step on the eigenmode: the Crank-Nicolson factor of each axis,
    // (1 + r/2 mu) / (1 - r/2 mu) with mu = -4 sin^2(pi/n).
    std::string AdiEigenmode(Hal::IAdiDiffusionBackend2D &backend)
    {
        const int32_t nx = 12, ny = 18;
        const double r = 0.3;
        const double pi = 3.14159265358979323846;
        std::vector<double> f = Eigenmode(nx, ny);
        std::vector<double> d(f.size(), 0.0);
        backend.DiffuseADI(f, d, r, nx, ny, true, true);
        const double mx = -4.0 * std::pow(std::sin(pi / nx), 2), my = -4.0 * std::pow(std::sin(pi / ny), 2);
        const double g = (1 + 0.5 * r * mx) / (1 - 0.5 * r * mx) * (1 + 0.5 * r * my) / (1 - 0.5 * r * my);
        double err = 0.0;
        for (size_t i = 0; i < f.size(); i++)
        {
            err = std::fmax(err, std::fabs(f[i] + d[i] - g * f[i]));
        }
        return err <= 1e-4 ? "" : Fmt("CN factor error %.3e > 1e-4", err);
    }

    // ADI against the CPU solver cell for cell (zero-flux and periodic), and
    // mass conservation with zero-flux edges.
    std::string AdiMatchesCpu(Hal::IAdiDiffusionBackend2D &backend)
    {
        const int32_t nx = 20, ny = 14;
        std::vector<double> f(static_cast<size_t>(nx) * ny);
        for (int32_t x = 0; x < nx; x++)
        {
            for (int32_t y = 0; y < ny; y++)
            {
                f[static_cast<size_t>(x) * ny + y] = 1.0 + 0.3 * x - 0.2 * y + 0.5 * std::sin(0.7 * x * y);
            }
        }
        for (int wrap = 0; wrap < 2; wrap++)
        {
            std::vector<double> d(f.size(), 0.0), exp(f.size(), 0.0), scratch(f.size());
            backend.DiffuseADI(f, d, 0.6, nx, ny, wrap, wrap);
            oracle_adi2(f.data(), scratch.data(), exp.data(), 0.6, nx, ny, wrap, wrap, nullptr);
            const double err = MaxAbsDiff(d, exp) / MaxAbs(f);
            if (err > 1e-5)
            {
                return Fmt("ADI differs from the CPU solver: %.3e", err);
            }
            double mass = 0.0;
            for (double v : d)
            {
                mass += v;
            }
            if (std::fabs(mass) > 1e-3)
            {
                return Fmt("mass not conserved: %.3e", mass);
            }
        }
        return "";
    }

    // Cell-bucket forces against an all-pairs sum with no buckets.
    std::string BruteForceForces(Hal::IAgentForceBackend2D &backend)
    {
        const int32_t dim = 16, n = 60;
        const double R = 3.0, k = 0.4;
        oracle_rand rng;
        oracle_rand_init(&rng, 1234);
        std::vector<double> pos(2 * n), rad(n);
        for (int32_t i = 0; i < n; i++)
        {
            pos[2 * i] = oracle_rand_double(&rng) * dim;
            pos[2 * i + 1] = oracle_rand_double(&rng) * dim;
            rad[i] = 0.4 + 0.4 * oracle_rand_double(&rng);
        }
        std::vector<double> v;
        backend.AccumulateForces(pos, rad, v, R, k, dim, dim, true, true);
        std::vector<double> exp(2 * n, 0.0);
        for (int32_t i = 0; i < n; i++)
        {
            for (int32_t j = 0; j < n; j++)
            {
                if (j == i)
                {
                    continue;
                }
                double dx = pos[2 * j] - pos[2 * i], dy = pos[2 * j + 1] - pos[2 * i + 1];
                dx -= dim * std::round(dx / dim);
                dy -= dim * std::round(dy / dim);
                const double dist = std::sqrt(dx * dx + dy * dy);
                if (dist > 0.0 && dist < R)
                {
                    const double force = k * ((rad[i] + rad[j]) - dist);
                    exp[2 * i] -= dx / dist * force;
                    exp[2 * i + 1] -= dy / dist * force;
                }
            }
        }
        const double err = MaxAbsDiff(v, exp);
        return err <= 1e-12 ? "" : Fmt("all-pairs difference %.3e > 1e-12", err);
    }

    // The off-lattice example's force pass (examples/OffLatticeExample.cpp:
    // 145-165): SumForces with the clamped Hooke law from the cells' current
    // velocities, returning each cell's force sum; bit-identical to the
    // restatement of SumForces on the agent grid.
    std::string ClampedSumForces(Hal::Cuda::CudaAgentForceBackend2D &backend)
    {
        const int32_t dim = 64, n = 4000;
        oracle_rand rng;
        oracle_rand_init(&rng, 11);
        std::vector<double> pos(2 * n), rad(n, 0.25), vel(2 * n);
        for (int32_t i = 0; i < n; i++)
        {
            pos[2 * i] = 24.0 + oracle_rand_gaussian(&rng, 0.0, 4.0);
            pos[2 * i + 1] = 24.0 + oracle_rand_gaussian(&rng, 0.0, 4.0);
            vel[2 * i] = oracle_rand_double(&rng) - 0.5;
            vel[2 * i + 1] = oracle_rand_double(&rng) - 0.5;
        }
        const hal_cuda_force_law law = {HAL_CUDA_FORCE_LINEAR_CLAMPED, 0.25, 1.0};
        std::vector<double> v = vel, sums;
        backend.SumForces(pos, rad, v, sums, 0.5, law, dim, dim, false, false);
        std::vector<double> expV(2 * n), expS(n);
        oracle_sum_forces(pos.data(), rad.data(), n, vel.data(), expV.data(), expS.data(), 0.5,
                          HAL_CUDA_FORCE_LINEAR_CLAMPED, 0.25, 1.0, HAL_CUDA_ORDER_AGENTGRID, dim, dim, 0, 0);
        if (v != expV || sums != expS)
        {
            return Fmt("SumForces differs from the restatement: %.3e", MaxAbsDiff(v, expV) + MaxAbsDiff(sums, expS));
        }
        int32_t positive = 0;
        for (double s : sums)
        {
            positive += (s > 0.0) ? 1 : 0;
        }
        return positive > n / 4 ? "" : Fmt("only %.0f cells feel a force", static_cast<double>(positive));
    }

    // A model's tick on the resident PDEGrid2D, written as against
    // Hal::PDEGrid2D (examples/CompetitiveRelease.cpp:77-94,147): per-cell
    // uptake Mul and source Add calls, DiffusionADI with a boundary value,
    // an explicit step, MulAll decay and Update, three ticks.  Equal bit for
    // bit to the same calls on the restatement of PDEGrid2D.
    std::string ResidentGridModelTicks()
    {
        const int32_t nx = 40, ny = 33, n = nx * ny, ticks = 3, perTick = 50;
        oracle_rand rng;
        oracle_rand_init(&rng, 21);
        std::vector<double> f0(static_cast<size_t>(n));
        for (double &v : f0)
        {
            v = oracle_rand_double(&rng);
        }
        Hal::Cuda::CudaPDEGrid2D grid(nx, ny);
        grid.SetState(f0, std::vector<double>(static_cast<size_t>(n), 0.0), 0);
        std::vector<int32_t> ops, iargs;
        std::vector<double> dargs, arrays;
        auto op = [&](int32_t code, int32_t i, double d0, double d1 = 0.0, int32_t arr = 0) {
            ops.push_back(code);
            iargs.insert(iargs.end(), {arr, i, 0});
            dargs.insert(dargs.end(), {d0, d1});
        };
        const int32_t g = 2 * (nx + ny);
        arrays.assign(static_cast<size_t>(g), 1.0);  // the boundary value 1.0 as a ghost table
        for (int32_t t = 0; t < ticks; t++)
        {
            for (int32_t k = 0; k < perTick; k++)
            {
                const int32_t c = oracle_rand_int(&rng, n);
                grid.Mul(c, -0.03);
                op(2, c, -0.03);
                grid.Add(c, 0.01);
                op(1, c, 0.01);
            }
            grid.DiffusionADI(0.7, 1.0);
            op(31, 0, 0.7);
            grid.Diffusion(0.2);
            op(20, 0, 0.2);
            grid.MulAll(-0.001);
            op(12, 0, -0.001);
            grid.Update();
            op(50, 0, 0.0);
        }
        std::vector<double> f = f0, d(static_cast<size_t>(n), 0.0), rec(4);
        int32_t uc = 0;
        oracle_pdegrid_script(nx, ny, 0, 0, f.data(), d.data(), &uc, static_cast<int32_t>(ops.size()), ops.data(),
                              iargs.data(), dargs.data(), arrays.data(), rec.data());
        if (grid.GetField() != f || grid.GetDeltas() != d || grid.UpdateCt() != uc)
        {
            return Fmt("resident grid differs from the restatement: %.3e", MaxAbsDiff(grid.GetField(), f));
        }
        double mx = f[0];
        for (double v : f)
        {
            mx = (v < mx) ? mx : v;
        }
        return grid.GetMax() == mx ? "" : "GetMax differs";
    }

    // Bins and FP64 forces equal the CPU backend bit for bit on float32
    // positions.
    std::string ForcesMatchCpu(Hal::Cuda::CudaAgentForceBackend2D &backend)
    {
        const int32_t dim = 64, n = 4000;
        oracle_rand rng;
        oracle_rand_init(&rng, 7);
        std::vector<double> pos(2 * n), rad(n, 0.5);
        for (int32_t i = 0; i < 2 * n; i++)
        {
            pos[i] = static_cast<double>(static_cast<float>(oracle_rand_double(&rng) * dim));
        }
        std::vector<double> v;
        backend.AccumulateForces(pos, rad, v, 1.0, 0.1, dim, dim, false, false);
        std::vector<double> exp(2 * n);
        std::vector<int32_t> off(static_cast<size_t>(dim) * dim + 1), bucket(n);
        oracle_accumulate_forces(pos.data(), rad.data(), n, exp.data(), 1.0, 0.1, dim, dim, 0, 0, off.data(),
                                 bucket.data(), 1);
        std::vector<int32_t> gotOff, gotBucket;
        backend.GetBins(gotOff, gotBucket);
        if (gotOff != off || gotBucket != bucket)
        {
            return "bins differ from the CPU backend";
        }
        if (std::memcmp(v.data(), exp.data(), v.size() * sizeof(double)) != 0)
        {
            return "FP64 forces differ from the CPU backend";
        }
        return "";
    }

    std::string CoincidentAgents(Hal::IAgentForceBackend2D &backend)
    {
        std::vector<double> pos = {4.0, 4.0, 4.0, 4.0}, rad = {0.5, 0.5}, v;
        backend.AccumulateForces(pos, rad, v, 2.0, 1.0, 8, 8, false, false);
        if (v.size() != 4)
        {
            return "velocityDeltas not resized";
        }
        for (double x : v)
        {
            if (x != 0.0)
            {
                return "coincident agents pushed apart or NaN";
            }
        }
        return "";
    }

    template <typename Fn>
    std::string Throws(Fn fn, const char *pWhat)
    {
        try
        {
            fn();
        }
        catch (const std::invalid_argument &)
        {
            return "";
        }
        return std::string(pWhat) + " did not throw std::invalid_argument";
    }

    std::string SizeMismatches(Hal::IDiffusionBackend2D &diff, Hal::IAdiDiffusionBackend2D &adi,
                               Hal::IAgentForceBackend2D &agents)
    {
        std::vector<double> f(16 * 20), d(16 * 20 - 1), v;
        std::string e = Throws([&] { diff.Diffuse(f, d, 0.1, 16, 20, false, false); }, "Diffuse");
        if (e.empty())
        {
            std::vector<double> f2(12 * 18), d2(12 * 17);
            e = Throws([&] { adi.DiffuseADI(f2, d2, 0.1, 12, 18, false, false); }, "DiffuseADI");
        }
        if (e.empty())
        {
            std::vector<double> pos(5), rad(2);
            e = Throws([&] { agents.AccumulateForces(pos, rad, v, 1.0, 1.0, 16, 16, false, false); },
                       "AccumulateForces");
        }
        return e;
    }

    // Per-cell rate diffusion and both advection forms, zero-flux, periodic
    // and Dirichlet, bit for bit against the CPU restatement.
    std::string VariableStencils(Hal::Cuda::CudaDiffusionBackend2D &diff)
    {
        const int32_t nx = diff.XDim(), ny = diff.YDim();
        const size_t cells = static_cast<size_t>(nx) * ny, ng = 2 * static_cast<size_t>(nx + ny);
        oracle_rand rng;
        oracle_rand_init(&rng, 7);
        auto draw = [&](size_t n, double scale, double shift)
        {
            std::vector<double> v(n);
            for (double &x : v)
            {
                x = scale * oracle_rand_double(&rng) + shift;
            }
            return v;
        };
        const std::vector<double> f = draw(cells, 1.0, 0.0), d0 = draw(cells, 0.1, 0.0);
        const std::vector<double> rx = draw(cells, 0.24, 0.0), ry = draw(cells, 0.24, 0.0);
        const std::vector<double> vx = draw(cells, 1.0, -0.5), vy = draw(cells, 1.0, -0.5);
        const std::vector<double> g = draw(ng, 1.0, -0.3), gvx = draw(ng, 1.0, -0.5), gvy = draw(ng, 1.0, -0.5);
        for (int wrap = 0; wrap < 3; wrap++)
        {
            const bool wx = wrap == 1, wy = wrap >= 1;
            std::vector<double> got = d0, exp = d0;
            diff.DiffuseVariable(f, got, rx, ry, wx, wy);
            oracle_diffusion2_var(f.data(), exp.data(), rx.data(), ry.data(), nx, ny, wx, wy);
            if (got != exp)
            {
                return Fmt("DiffuseVariable differs (wrap %g)", wrap);
            }
            got = d0;
            exp = d0;
            diff.Advect(f, got, 0.3, -0.2, wx, wy, g);
            oracle_advection2_bc(f.data(), exp.data(), 0.3, -0.2, nx, ny, wx, wy, g.data());
            if (got != exp)
            {
                return Fmt("Advect (Dirichlet) differs (wrap %g)", wrap);
            }
            got = d0;
            exp = d0;
            diff.AdvectVariable(f, got, vx, vy, wx, wy);
            oracle_advection2_var(f.data(), exp.data(), vx.data(), vy.data(), nx, ny, wx, wy);
            if (got != exp)
            {
                return Fmt("AdvectVariable differs (wrap %g)", wrap);
            }
            got = d0;
            exp = d0;
            diff.AdvectVariable(f, got, vx, vy, wx, wy, g, gvx, gvy);
            oracle_advection2_var_bc(f.data(), exp.data(), vx.data(), vy.data(), nx, ny, wx, wy, g.data(), gvx.data(),
                                     gvy.data());
            if (got != exp)
            {
                return Fmt("AdvectVariable (Dirichlet) differs (wrap %g)", wrap);
            }
        }
        return "";
    }

    // Resident SphericalAgent2D ticks: one tick's update equals the oracle's
    // FP32 update of the tick's own deltas, bit for bit.
    std::string AgentStep(Hal::Cuda::CudaAgentForceBackend2D &agents)
    {
        const int32_t n = 3000, dim = 64;
        oracle_rand rng;
        oracle_rand_init(&rng, 31);
        std::vector<float> pos(2 * n), rad(n), vel(2 * n);
        for (int32_t i = 0; i < n; i++)
        {
            pos[2 * i] = static_cast<float>(oracle_rand_double(&rng) * dim * 0.999);
            pos[2 * i + 1] = static_cast<float>(oracle_rand_double(&rng) * dim * 0.999);
            rad[i] = static_cast<float>(0.3 + 0.4 * oracle_rand_double(&rng));
            vel[2 * i] = static_cast<float>(oracle_rand_double(&rng) - 0.5);
            vel[2 * i + 1] = static_cast<float>(oracle_rand_double(&rng) - 0.5);
        }
        agents.Upload(pos, rad);
        agents.SetVelocities(vel);
        agents.Step(1, 1.5, 0.2, true, false, 0.7, 0.6);
        std::vector<float> gotPos, gotVel, deltas;
        agents.GetState(gotPos, gotVel);
        agents.Download(deltas);
        oracle_agents_move_f32(pos.data(), vel.data(), deltas.data(), n, dim, dim, 1, 0, 0.7f, 0.6f);
        if (gotPos != pos || gotVel != vel)
        {
            return "resident agent step differs from the FP32 update of its deltas";
        }
        return "";
    }

    // A CompetitiveRelease-style model tick through the classes: the coupled
    // call equals alternating Step(1) / RunTicks(1) calls bit for bit, and the
    // explicit field's uptake equals the oracle tick with the bins' counts.
    std::string CoupledModel()
    {
        const int32_t nx = 48, ny = 64, n = 2500;
        oracle_rand rng;
        oracle_rand_init(&rng, 91);
        std::vector<float> pos(2 * n), rad(n, 0.5f), f0(static_cast<size_t>(nx) * ny),
            s0(static_cast<size_t>(nx) * ny);
        for (int32_t i = 0; i < n; i++)
        {
            pos[2 * i] = static_cast<float>(oracle_rand_double(&rng) * nx * 0.999);
            pos[2 * i + 1] = static_cast<float>(ny * 0.5 + (oracle_rand_double(&rng) - 0.5) * ny * 0.4);
        }
        for (size_t c = 0; c < f0.size(); c++)
        {
            f0[c] = static_cast<float>(oracle_rand_double(&rng));
            s0[c] = static_cast<float>(0.01 * oracle_rand_double(&rng));
        }
        const double uptake = 0.002, r = 3.0, decay = 0.01;
        std::vector<float> expF, expP, expV, gotF, gotP, gotV;
        {
            Hal::Cuda::CudaAgentForceBackend2D ag(nx, ny, n);
            Hal::Cuda::CudaAdiDiffusionBackend2D adi(nx, ny);
            ag.Upload(pos, rad);
            adi.SetField(f0);
            adi.SetSource(s0);
            adi.SetUptake(&ag, uptake);
            for (int t = 0; t < 9; t++)
            {
                // the handles' streams differ: the tick reads this step's bins,
                // and the next step rebins after the tick has read them
                ag.Step(1, 1.0, 0.1, false, false, 0.5, -1.0);
                hal_cuda_agents_sync(ag.Handle());
                adi.RunTicks(1, r, decay, false, false);
                adi.Sync();
            }
            adi.GetField(expF);
            ag.GetState(expP, expV);
        }
        {
            Hal::Cuda::CudaAgentForceBackend2D ag(nx, ny, n);
            Hal::Cuda::CudaAdiDiffusionBackend2D adi(nx, ny);
            ag.Upload(pos, rad);
            adi.SetField(f0);
            adi.SetSource(s0);
            adi.SetUptake(&ag, uptake);
            adi.RunCoupled(ag, 4, r, decay, false, false, 1.0, 0.1, 0.5, -1.0);
            adi.RunCoupled(ag, 5, r, decay, false, false, 1.0, 0.1, 0.5, -1.0);
            adi.GetField(gotF);
            ag.GetState(gotP, gotV);
        }
        if (gotF != expF || gotP != expP || gotV != expV)
        {
            return "RunCoupled differs from alternating Step / RunTicks calls";
        }
        // explicit uptake: one dispatch's bins, 20 ticks, against the oracle
        Hal::Cuda::CudaAgentForceBackend2D ag(nx, ny, n);
        Hal::Cuda::CudaDiffusionBackend2D diff(nx, ny);
        ag.Upload(pos, rad);
        ag.Dispatch(1.0, 0.1, false, false);
        std::vector<int32_t> off, bucket;
        ag.GetBins(off, bucket);
        std::vector<int32_t> counts(f0.size());
        for (size_t c = 0; c < counts.size(); c++)
        {
            counts[c] = off[c + 1] - off[c];
        }
        diff.SetField(f0);
        diff.SetSource(s0);
        diff.SetUptake(&ag, uptake);
        diff.RunTicks(20, 0.2, decay, false, false);
        diff.GetField(gotF);
        const size_t cells = f0.size();
        std::vector<double> exp(f0.begin(), f0.end()), deltas(cells, 0.0), scratch(cells),
            src64(s0.begin(), s0.end());
        for (int t = 0; t < 20; t++)
        {
            oracle_tick(0, exp.data(), deltas.data(), scratch.data(), nx, ny, 0.2, 0, 0, nullptr, decay, src64.data(),
                        0, nullptr, nullptr, counts.data(), uptake, 1);
        }
        std::vector<double> got64(gotF.begin(), gotF.end());
        const double err = MaxAbsDiff(got64, exp) / MaxAbs(exp);
        if (err > 1e-5)
        {
            return Fmt("explicit ticks with uptake differ from the oracle: %.3e", err);
        }
        return "";
    }

    double RelL2(const std::vector<float> &a, const std::vector<double> &b)
    {
        double num = 0.0, den = 0.0;
        for (size_t i = 0; i < b.size(); i++)
        {
            num += (a[i] - b[i]) * (a[i] - b[i]);
            den += b[i] * b[i];
        }
        return std::sqrt(num / (den > 0.0 ? den : 1.0));
    }

    // Three wells (explicit, ADI with a source, explicit with agents) in one
    // batched handle against the single-grid classes: identical fields and
    // forces.
    std::string Wells()
    {
        std::vector<hal_cuda_well_desc> d(3);
        d[0] = {40, 33, HAL_CUDA_WELL_EXPLICIT, 0, 1, 0, 0.2, 0.001};
        d[1] = {48, 48, HAL_CUDA_WELL_ADI, 1, 0, 0, 4.0, 0.01};
        d[2] = {24, 24, HAL_CUDA_WELL_EXPLICIT, 0, 0, 200, 0.15, 0.0};
        oracle_rand rng;
        oracle_rand_init(&rng, 77);
        auto draw = [&](size_t n, double scale)
        {
            std::vector<float> v(n);
            for (float &x : v)
            {
                x = static_cast<float>(scale * oracle_rand_double(&rng));
            }
            return v;
        };
        std::vector<std::vector<float>> f0;
        for (const hal_cuda_well_desc &w : d)
        {
            f0.push_back(draw(static_cast<size_t>(w.xDim) * w.yDim, 1.0));
        }
        const std::vector<float> src1 = draw(48 * 48, 0.01);
        std::vector<float> pos = draw(400, 23.99), rad(200, 0.5f);
        const int ticks = 7;
        Hal::Cuda::CudaWells2D wells(d);
        for (int w = 0; w < 3; w++)
        {
            wells.SetField(w, f0[static_cast<size_t>(w)]);
        }
        wells.SetSource(1, src1);
        wells.SetAgents({0, 0, 200}, pos, rad);
        wells.RunTicks(ticks, 1.0, 0.1);
        std::vector<float> got, exp, forces, expForces;
        wells.GetForces(forces);
        for (int w = 0; w < 3; w++)
        {
            wells.GetField(w, got);
            const hal_cuda_well_desc &x = d[static_cast<size_t>(w)];
            if (x.kind == HAL_CUDA_WELL_ADI)
            {
                Hal::Cuda::CudaAdiDiffusionBackend2D adi(x.xDim, x.yDim);
                adi.SetField(f0[static_cast<size_t>(w)]);
                adi.SetSource(src1);
                adi.RunTicks(ticks, x.diffRate, x.decay, x.wrapX != 0, x.wrapY != 0);
                adi.GetField(exp);
            }
            else
            {
                Hal::Cuda::CudaDiffusionBackend2D diff(x.xDim, x.yDim);
                diff.SetField(f0[static_cast<size_t>(w)]);
                diff.RunTicks(ticks, x.diffRate, x.decay, x.wrapX != 0, x.wrapY != 0);
                diff.GetField(exp);
            }
            if (got != exp)
            {
                return Fmt("well %g differs from its single-grid run", w);
            }
        }
        Hal::Cuda::CudaAgentForceBackend2D agents(24, 24, 200);
        agents.Upload(pos, rad);
        agents.Dispatch(1.0, 0.1, false, false);
        agents.Download(expForces);
        return forces == expForces ? "" : "well agent forces differ from the single-grid dispatch";
    }

    // The adjoint's forward/backward API against the FP64 CPU adjoint, and
    // the gradient's independence of the checkpoint interval.
    std::string Adjoint()
    {
        const int32_t n = 32, steps = 12;
        const size_t cells = static_cast<size_t>(n) * n;
        oracle_rand rng;
        oracle_rand_init(&rng, 5);
        std::vector<float> f0(cells), target(cells), D(cells), src(cells);
        for (size_t i = 0; i < cells; i++)
        {
            f0[i] = static_cast<float>(oracle_rand_double(&rng));
            target[i] = static_cast<float>(oracle_rand_double(&rng));
            D[i] = static_cast<float>(0.5 + 4.5 * oracle_rand_double(&rng));
            src[i] = static_cast<float>(0.01 * oracle_rand_double(&rng));
        }
        const double decay = 0.005;
        std::vector<double> f0d(f0.begin(), f0.end()), td(target.begin(), target.end()), Dd(D.begin(), D.end()),
            sd(src.begin(), src.end()), fT(cells), gD(cells), gS(cells);
        double gK = 0.0;
        const double lossRef = oracle_dadi_loss_grad(f0d.data(), td.data(), Dd.data(), decay, sd.data(), n, n, 0, 0,
                                                     steps, fT.data(), gD.data(), &gK, gS.data());
        Hal::Cuda::CudaAdjointAdi2D adj(n, n, false, false);
        std::vector<float> gotD, gotS, firstD;
        double gotK = 0.0;
        for (int every : {5, 0})
        {
            adj.SetProblem(f0, target, steps, every);
            const double lf = adj.Forward(D, decay, src);
            const double lb = adj.Backward(D, decay, src, gotD, gotK, gotS);
            if (std::fabs(lf - lossRef) > 1e-4 * lossRef || std::fabs(lb - lf) > 1e-6 * lf)
            {
                return Fmt("adjoint loss differs from the FP64 adjoint: %.3e", lf - lossRef);
            }
            if (RelL2(gotD, gD) > 2e-3 || RelL2(gotS, gS) > 2e-3 || std::fabs(gotK - gK) > 2e-3 * std::fabs(gK))
            {
                return Fmt("adjoint gradient differs from the FP64 adjoint: %.3e", RelL2(gotD, gD));
            }
            if (every == 0 && gotD != firstD)
            {
                return "gradient depends on the checkpoint interval";
            }
            firstD = gotD;
        }
        float msF = 0.0f, msB = 0.0f;
        adj.Times(msF, msB);
        return (msF > 0.0f && msB > 0.0f) ? "" : "adjoint times not recorded";
    }

    // Resident ticks (PDEGrid2D semantics: decay, dense source, Dirichlet)
    // against the CPU tick, explicit and ADI.
    std::string ResidentTicks(Hal::Cuda::CudaDiffusionBackend2D &diff, Hal::Cuda::CudaAdiDiffusionBackend2D &adi)
    {
        const int32_t nx = diff.XDim(), ny = diff.YDim();
        const size_t cells = static_cast<size_t>(nx) * ny;
        oracle_rand rng;
        oracle_rand_init(&rng, 99);
        std::vector<double> f(cells), src(cells), ghost(2 * (nx + ny), 0.0);
        for (size_t i = 0; i < cells; i++)
        {
            f[i] = static_cast<float>(oracle_rand_double(&rng));
            src[i] = static_cast<float>(0.01 * oracle_rand_double(&rng));
        }
        for (int32_t y = 0; y < ny; y++)
        {
            ghost[y] = 1.0;  // bc(-1, y) = 1, 0 elsewhere
        }
        std::vector<float> f32(f.begin(), f.end()), s32(src.begin(), src.end()), g32(ghost.begin(), ghost.end());
        for (int mode = 0; mode < 2; mode++)
        {
            const double r = mode == 0 ? 0.2 : 5.0;
            const int ticks = 30;
            std::vector<double> exp = f, deltas(cells, 0.0), scratch(cells);
            for (int t = 0; t < ticks; t++)
            {
                oracle_tick(mode, exp.data(), deltas.data(), scratch.data(), nx, ny, r, 0, 0, ghost.data(), 0.01,
                            src.data(), 0, nullptr, nullptr, nullptr, 0.0, 1);
            }
            std::vector<float> got;
            if (mode == 0)
            {
                diff.SetField(f32);
                diff.SetSource(s32);
                diff.SetDirichlet(g32);
                diff.RunTicks(ticks, r, 0.01, false, false);
                diff.GetField(got);
            }
            else
            {
                adi.SetField(f32);
                adi.SetSource(s32);
                adi.SetDirichlet(g32);
                adi.RunTicks(ticks, r, 0.01, false, false);
                adi.GetField(got);
            }
            std::vector<double> got64(got.begin(), got.end());
            const double err = MaxAbsDiff(got64, exp) / MaxAbs(exp);
            if (err > 1e-5)
            {
                return Fmt(mode == 0 ? "explicit ticks differ: %.3e" : "ADI ticks differ: %.3e", err);
            }
        }
        return "";
    }
}

int main()
{
    Hal::Cuda::CudaDiffusionBackend2D diffEig(16, 20);
    Hal::Cuda::CudaAdiDiffusionBackend2D adiEig(12, 18);
    Hal::Cuda::CudaAdiDiffusionBackend2D adiCpu(20, 14);
    Hal::Cuda::CudaAgentForceBackend2D agents16(16, 16, 64);
    Hal::Cuda::CudaAgentForceBackend2D agents64(64, 64, 4000);
    Hal::Cuda::CudaAgentForceBackend2D agents8(8, 8, 4);
    Hal::Cuda::CudaDiffusionBackend2D diffTick(40, 33);
    Hal::Cuda::CudaAdiDiffusionBackend2D adiTick(40, 33);

    Run("explicit_eigenmode", [&] { return ExplicitEigenmode(diffEig); });
    Run("adi_crank_nicolson_factor", [&] { return AdiEigenmode(adiEig); });
    Run("adi_matches_cpu_and_conserves_mass", [&] { return AdiMatchesCpu(adiCpu); });
    Run("forces_match_all_pairs", [&] { return BruteForceForces(agents16); });
    Run("forces_and_bins_match_cpu", [&] { return ForcesMatchCpu(agents64); });
    Run("coincident_agents", [&] { return CoincidentAgents(agents8); });
    Run("clamped_sum_forces_bit_exact", [&] { return ClampedSumForces(agents64); });
    Run("resident_pdegrid_model_ticks_bit_exact", [&] { return ResidentGridModelTicks(); });
    Run("size_mismatch_throws", [&] { return SizeMismatches(diffEig, adiEig, agents16); });
    Run("resident_ticks_match_cpu", [&] { return ResidentTicks(diffTick, adiTick); });
    Run("variable_rate_and_advection_bit_exact", [&] { return VariableStencils(diffTick); });
    Run("resident_agent_step_bit_exact", [&] { return AgentStep(agents64); });
    Run("batched_wells_equal_single_grids", [&] { return Wells(); });
    Run("adjoint_forward_backward_api", [&] { return Adjoint(); });
    Run("coupled_model_ticks", [&] { return CoupledModel(); });

    std::printf("backend_tests: %d passed, %d failed\n", g_passed, g_failed);
    return g_failed == 0 ? 0 : 1;
}
