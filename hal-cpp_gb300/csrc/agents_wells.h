// agents_wells.h -- the agent force pass over many independent wells at once
// (agents.cu), used by the batched wells handle (wells.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

struct hal_cuda_agents;

namespace halcuda
{
    // The wells' agents are binned in coarse bins of b x b cells, b = 2^shift
    // chosen per well from its agent capacity: the largest b <= 2^kWellMaxShift
    // whose bins hold at most one agent on average.  Sparse wells (the
    // batched workload's large wells: a few thousand agents in up to 1M
    // cells) thereby scan b^2 times fewer bins than cells, while dense wells
    // keep one cell per bin, whose force walk reads each window row as one
    // run of bins.  Within a bin the agents are ordered by (cell, agent
    // index), so each cell's agents are a run of its bin in the order of a
    // per-cell binning.
    constexpr int32_t kWellMaxShift = 3;

    inline int32_t WellBinShift(int32_t xDim, int32_t yDim, int32_t maxAgents)
    {
        const double cells = static_cast<double>(xDim) * static_cast<double>(yDim);
        int32_t shift = 0;
        while (shift < kWellMaxShift && static_cast<double>(maxAgents) * static_cast<double>(4 << (2 * shift)) <= cells)
        {
            shift++;
        }
        return shift;
    }

    inline int64_t WellBins(int32_t xDim, int32_t yDim, int32_t shift)
    {
        const int32_t b = 1 << shift;
        return static_cast<int64_t>((xDim + b - 1) >> shift) * ((yDim + b - 1) >> shift);
    }

    // One well's grid inside the concatenated bin array.
    struct AgentWellDev
    {
        int64_t binBase;        // first coarse bin of the well in the concatenation
        int32_t xDim, yDim;
        int32_t wrapX, wrapY;
        int32_t binsY;          // coarse bins along y
        int32_t binShift;       // bins of 2^binShift x 2^binShift cells
    };

    // Device arrays of one pass (n agents, `cells` concatenated cells).
    struct AgentWellsArgs
    {
        const float *pos;          // 2n, (x, y) interleaved, well-local coordinates
        const float *rad;          // n
        const int32_t *wellOf;     // n
        const AgentWellDev *wells;
        int32_t n;
        int64_t cells;             // coarse bins of all wells (WellBins summed)
        float2 *posF, *sPos;       // n each
        float *sRad;               // n
        int32_t *cellOf, *arrival, *bucketTmp, *bucket;  // n each (cellOf: the agent's bin)
        int32_t *sCell;            // n: each sorted slot's cell within its well
        int32_t *counts;           // cells (bins), zero on entry (each binning's scan clears them again)
        int32_t *offsets;          // cells (bins) + 1
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
