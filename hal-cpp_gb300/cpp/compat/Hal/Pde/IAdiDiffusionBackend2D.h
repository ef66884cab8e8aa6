#pragma once

// Stand-in for HAL-CPP's include/Hal/Pde/IAdiDiffusionBackend2D.h (:12-32),
// used only outside a HAL-CPP tree; same declaration as HAL's.
#include <cstdint>
#include <vector>

namespace Hal
{
    class IAdiDiffusionBackend2D
    {
    public:
        IAdiDiffusionBackend2D();
        virtual ~IAdiDiffusionBackend2D();
        IAdiDiffusionBackend2D(const IAdiDiffusionBackend2D &other) = delete;
        IAdiDiffusionBackend2D &operator=(const IAdiDiffusionBackend2D &other) = delete;

        virtual void DiffuseADI(const std::vector<double> &field,
                                std::vector<double>       &deltas,
                                double                     diffRate,
                                int32_t                    xDim,
                                int32_t                    yDim,
                                bool                       wrapX,
                                bool                       wrapY) = 0;
    };
}
