// agents_wells.h -- the agent force pass over many independent wells at once
// (agents.cu), used by the batched wells handle (wells.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

struct hal_cuda_agents;

namespace halcuda
{
    // One well's grid inside the concatenated cell array.
    struct AgentWellDev
    {
        int64_t cellBase;       // first cell of the well in the concatenation
        int32_t xDim, yDim;
        int32_t wrapX, wrapY;
    };

    // Device arrays of one pass (n agents, `cells` concatenated cells).
    struct AgentWellsArgs
    {
        const float *pos;          // 2n, (x, y) interleaved, well-local coordinates
        const float *rad;          // n
        const int32_t *wellOf;     // n
        const AgentWellDev *wells;
        int32_t n;
        int64_t cells;
        float2 *posF, *sPos;       // n each
        float *sRad;               // n
        int32_t *cellOf, *arrival, *bucketTmp, *bucket;  // n each
        int32_t *counts;           // cells, zero on entry (each binning's scan clears them again)
        int32_t *offsets;          // cells + 1
        int32_t *tileSums;         // AgentScanTiles(cells)
        double interactionRad;
        float R, k;
        float *vel;                // 2n, overwritten
        int32_t forceThreads = 128;  // block size of the force kernel (64, 128 or 256)
        // Motion (SphericalAgent2D's update after the forces, the resident
        // step of hal_cuda_agents_step): with velState set, each agent's
        // velocity takes its delta, is capped (maxVel >= 0), moves the agent
        // (posOut, agent order, the well's own wrap) and takes the friction.
        float2 *velState = nullptr;  // n, or null: forces only
        float2 *posOut = nullptr;    // n: the positions, rewritten in place
        float friction = 1.0f, maxVel = -1.0f;
    };

    int32_t AgentScanTiles(int64_t cells);

    // The bins of an agent handle's last binning, for other handles that act
    // per agent on a grid of the same size (hal_cuda_pdegrid_apply_agents).
    struct AgentBinsView
    {
        const int32_t *offsets;  // xDim*yDim + 1
        const int32_t *bucket;   // n, ascending agent index within each cell
        const int32_t *cellOf;   // n, by agent index
        int32_t n, xDim, yDim;
        int device;
        cudaStream_t stream;     // the handle's stream
    };

    // Count, scan, scatter, stable rank and forces of every well's agents.
    int LaunchAgentWells(const AgentWellsArgs &a, cudaStream_t s);

    AgentBinsView AgentsBins(const hal_cuda_agents *a);
}
