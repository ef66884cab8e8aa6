// tick_params.h -- parameters of one fused explicit tick (the TickKernel's
// input), shared by the single-grid handle (diffusion.cu) and the batched
// wells handle (wells.cu).
#pragma once

#include "common.cuh"

#include <cstdint>

namespace halcuda
{
    struct TickParams
    {
        const float *f;
        float *out;
        int32_t xDim, yDim;
        float r, negDecay;
        int32_t wrapX, wrapY;
        const float *src;          // dense source or null
        GhostView ghost;           // all null for zero-flux
        const int32_t *ptStart;    // point sources grouped by CTA (CSR), or null
        const int32_t *ptRow;
        const int32_t *ptCol;
        const float *ptVal;        // Uniform-velocity upwind advection (PDEGrid2D::Advection): the
        // weight of each neighbour difference is the diffusion rate plus the
        // upwind velocity from that side -- x-1: r + max(xVel, 0), x+1:
        // r + max(-xVel, 0), y-1: r + max(yVel, 0), y+1: r + max(-yVel, 0).
        // Read only by the advective variant of the tick.
        float kUp, kDn, kYm, kYp;
    };

    // Agent uptake of the single-grid tick's uptake variant (a second kernel
    // parameter, so that the other ticks keep their parameters): every agent
    // binned in a cell multiplies it by negUptake, as a model's
    // PDEGrid2D::Mul(cell, -uptake) per agent; the agent count of cell i is
    // cellOffsets[i + 1] - cellOffsets[i] (layout x*yDim + y).
    struct TickUptake
    {
        const int32_t *cellOffsets;
        float negUptake;
    };

    // Geometry of the tick's CTAs: 32 lanes x kTickWarps warps; a lane owns
    // VEC consecutive cells of kTickRowsPerThread consecutive rows.
    constexpr int kTickRowsPerThread = 3;
    constexpr int kTickWarps = 8;

    // Batched ticks: tile b = (grid index, CTA column, CTA row) of the
    // table's grids.  vec is 4 (every grid's yDim % 4 == 0) or 1.
    int LaunchTickTiles(const TickParams *table, const int4 *tiles, int32_t nTiles, int vec, cudaStream_t s);

    // ---- two ticks per launch (temporal blocking, tick_blocked.cu) --------
    // A CTA computes a kTickBlockRows x kTickBlockCols tile; the field must
    // have yDim % 4 == 0 and a 16-byte aligned base.
    constexpr int kTickBlockRows = 32;
    constexpr int kTickBlockCols = 128;

    struct TickBlockParams
    {
        const float *f;
        float *out;
        int32_t xDim, yDim;
        float r, negDecay;
        int32_t wrapX, wrapY;
        const float *S;            // dense source plus point sources, or null
        GhostView ghost;           // all null for zero-flux
        float kUp, kDn, kYm, kYp;  // per-side weights when advecting (see TickParams)
        int32_t adv;
        int32_t *err;              // set to 1 if a staging wait gave up
        // failure-detection test hook (hal_cuda_diffusion_test_stall):
        // bytes the staged copy's mbarrier expects beyond the copy, so that
        // its wait runs out, and the wait's limit in us (0: the default)
        uint32_t extraTx;
        uint32_t waitLimitUs;
    };

    // Opaque 128-byte tensor map (a CUtensorMap) over one field buffer.
    struct alignas(64) TickBlockTensorMap
    {
        unsigned char bytes[128];
    };

    bool MakeTickBlockTensorMap(TickBlockTensorMap &map, const float *field, int32_t xDim, int32_t yDim);
    int PrepareTickBlocked();
    void LaunchTickBlocked2(const TickBlockParams &p, const TickBlockTensorMap &map, cudaStream_t s);
}
