#pragma once

// Stand-in for HAL-CPP's include/Hal/Agents/IAgentForceBackend2D.h (:15-37),
// used only outside a HAL-CPP tree; same declaration as HAL's.
#include <cstdint>
#include <vector>

namespace Hal
{
    class IAgentForceBackend2D
    {
    public:
        IAgentForceBackend2D();
        virtual ~IAgentForceBackend2D();
        IAgentForceBackend2D(const IAgentForceBackend2D &other) = delete;
        IAgentForceBackend2D &operator=(const IAgentForceBackend2D &other) = delete;

        virtual void AccumulateForces(const std::vector<double> &positions,
                                      const std::vector<double> &radii,
                                      std::vector<double>       &velocityDeltas,
                                      double                     interactionRad,
                                      double                     springConstant,
                                      int32_t                    xDim,
                                      int32_t                    yDim,
                                      bool                       wrapX,
                                      bool                       wrapY) = 0;
    };
}
