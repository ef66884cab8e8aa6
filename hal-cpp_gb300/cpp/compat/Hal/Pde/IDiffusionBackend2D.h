#pragma once

// Stand-in for HAL-CPP's include/Hal/Pde/IDiffusionBackend2D.h, used only when
// this backend is built outside a HAL-CPP tree.  The class must match HAL's
// declaration (include/Hal/Pde/IDiffusionBackend2D.h:13-33) signature for
// signature: it is the drop-in contract.  Inside HAL-CPP, HAL's own header is
// used instead.
#include <cstdint>
#include <vector>

namespace Hal
{
    class IDiffusionBackend2D
    {
    public:
        IDiffusionBackend2D();
        virtual ~IDiffusionBackend2D();
        IDiffusionBackend2D(const IDiffusionBackend2D &other) = delete;
        IDiffusionBackend2D &operator=(const IDiffusionBackend2D &other) = delete;

        virtual void Diffuse(const std::vector<double> &field,
                             std::vector<double>       &deltas,
                             double                     diffRate,
                             int32_t                    xDim,
                             int32_t                    yDim,
                             bool                       wrapX,
                             bool                       wrapY) = 0;
    };
}
