// adi64.h -- Internal::Diffusion2DADI in FP64 on device arrays: the Thomas
// solve per line in the reference's operation order (pdegrid.cu), for any line
// length.  The device-resident PDEGrid2D uses it for DiffusionADI, and the ADI
// handle's interface calls (IAdiDiffusionBackend2D::DiffuseADI) use it for
// lines longer than the FP32 partitioned solve takes.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>

namespace halcuda
{
    class Adi64
    {
    public:
        Adi64();
        ~Adi64();
        Adi64(const Adi64 &) = delete;
        Adi64 &operator=(const Adi64 &) = delete;

        // deltas += v - f for the xDim x yDim field f (HAL's layout, device
        // FP64), v the ADI step of f at rate r (ADIequations.h:306-337); with
        // ghost (the device ghost table of hal_cuda.h, FP64), the Dirichlet
        // form (:339-378).  Enqueued on s; scratch grows on first use (after
        // synchronising s).
        int Run(const double *f, double *deltas, int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY, double r,
                const double *ghost, cudaStream_t s);

    private:
        struct Impl;
        std::unique_ptr<Impl> m_impl;
    };
}
