// interface_bench.cpp -- per-call times of the three strategy interfaces.
//
// The counterpart of the reference's examples/BackendBenchmark.cpp:60-268 for
// the calls model code makes through the interfaces: one Diffuse, one
// DiffuseADI or one AccumulateForces per call, on std::vector<double> host
// data, so that every GPU call pays its upload, kernels and readback.  Each
// call goes through Hal::Cuda::*Backend2D (the GB300 backends) and, as the
// CPU baseline, through the CPU oracle (the C restatement of the reference's
// single-threaded CPU backends, bit-identical to them).  Inputs follow
// BackendBenchmark: the field 0.5 + 0.5 sin(2 pi (x + y) / n), wrapped axes,
// rate 0.2 (explicit) or 0.8 (ADI); agents uniform in a 256 x 256 wrapped
// domain with Rand(7), radius 0.5, interaction radius 2, spring constant 0.5.
// One warm-up call, then the mean over the repetitions (steady_clock).  Prints
// one JSON object per line.
#include "Hal/Cuda/CudaBackends2D.h"

#include "hal_oracle.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <functional>
#include <vector>

namespace
{
    double Seconds(const std::function<void()> &fn, int reps)
    {
        fn();  // warm-up (first call allocates and sets up)
        const auto t0 = std::chrono::steady_clock::now();
        for (int r = 0; r < reps; r++)
        {
            fn();
        }
        const auto t1 = std::chrono::steady_clock::now();
        return std::chrono::duration<double>(t1 - t0).count() / reps;
    }

    std::vector<double> Field(int32_t n)
    {
        std::vector<double> f(static_cast<size_t>(n) * n);
        for (int32_t x = 0; x < n; x++)
        {
            for (int32_t y = 0; y < n; y++)
            {
                f[static_cast<size_t>(x) * n + y] = 0.5 + 0.5 * std::sin(2.0 * 3.14159265358979323846 * (x + y) / n);
            }
        }
        return f;
    }

    void Line(const char *call, const char *size, double cpu, double gpu, const char *unit, double units)
    {
        std::printf("{\"call\": \"%s\", \"size\": \"%s\", \"cpu_s_per_call\": %.6e, \"gpu_s_per_call\": %.6e, "
                    "\"speedup\": %.3f, \"gpu_%s_per_s\": %.4e}\n",
                    call, size, cpu, gpu, cpu / gpu, unit, units / gpu);
        std::fflush(stdout);
    }
}

int main()
{
    char size[64];
    for (int32_t n : {64, 256, 512, 1024, 2048})
    {
        const std::vector<double> f = Field(n);
        std::vector<double> dg(f.size(), 0.0), dc(f.size(), 0.0);
        Hal::Cuda::CudaDiffusionBackend2D gpu(n, n);
        const int reps = (n >= 1024) ? 10 : 20;
        const double tg = Seconds([&] { gpu.Diffuse(f, dg, 0.2, n, n, true, true); }, reps);
        const double tc = Seconds([&] { oracle_diffusion2(f.data(), dc.data(), 0.2, n, n, 1, 1, nullptr); }, reps);
        std::snprintf(size, sizeof(size), "%dx%d", n, n);
        Line("Diffuse", size, tc, tg, "cell_updates", static_cast<double>(n) * n);
    }
    for (int32_t n : {64, 256, 512, 1024, 2048})
    {
        const std::vector<double> f = Field(n);
        std::vector<double> dg(f.size(), 0.0), dc(f.size(), 0.0), scratch(f.size());
        Hal::Cuda::CudaAdiDiffusionBackend2D gpu(n, n);
        const int reps = (n >= 1024) ? 5 : 20;
        const double tg = Seconds([&] { gpu.DiffuseADI(f, dg, 0.8, n, n, true, true); }, reps);
        const double tc = Seconds(
            [&] { oracle_adi2(f.data(), scratch.data(), dc.data(), 0.8, n, n, 1, 1, nullptr); }, reps);
        std::snprintf(size, sizeof(size), "%dx%d", n, n);
        Line("DiffuseADI", size, tc, tg, "cell_updates", static_cast<double>(n) * n);
        // the same call in exact mode (FP64 Thomas per line, bit-exact)
        gpu.SetExact(true);
        const double te = Seconds([&] { gpu.DiffuseADI(f, dg, 0.8, n, n, true, true); }, reps);
        Line("DiffuseADI (exact)", size, tc, te, "cell_updates", static_cast<double>(n) * n);
    }
    for (int32_t agents : {1000, 10000, 50000, 200000})
    {
        const int32_t n = 256;
        oracle_rand rng;
        oracle_rand_init(&rng, 7);
        std::vector<double> pos, rad;
        for (int32_t i = 0; i < agents; i++)
        {
            pos.push_back(oracle_rand_double(&rng) * n);
            pos.push_back(oracle_rand_double(&rng) * n);
            rad.push_back(0.5);
        }
        std::vector<double> vg, vc(pos.size());
        std::vector<int32_t> off(static_cast<size_t>(n) * n + 1), bucket(static_cast<size_t>(agents));
        Hal::Cuda::CudaAgentForceBackend2D gpu(n, n, agents);
        const int reps = (agents >= 200000) ? 3 : 10;
        const double tg = Seconds([&] { gpu.AccumulateForces(pos, rad, vg, 2.0, 0.5, n, n, true, true); }, reps);
        const double tc = Seconds(
            [&] {
                oracle_accumulate_forces(pos.data(), rad.data(), agents, vc.data(), 2.0, 0.5, n, n, 1, 1, off.data(),
                                         bucket.data(), 1);
            },
            reps);
        std::snprintf(size, sizeof(size), "%d agents in 256x256", agents);
        Line("AccumulateForces", size, tc, tg, "agents", static_cast<double>(agents));
    }
    return 0;
}
