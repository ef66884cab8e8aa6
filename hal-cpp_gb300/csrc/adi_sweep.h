// adi_sweep.h -- parameters of one ADI half-sweep (the AdiSweep kernel's
// input), shared by the single-grid handle (adi.cu) and the batched wells
// handle (wells.cu), which fills one SweepParams per well and sweep.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace halcuda
{
    // Device view of an AdiLinePlanHost (adi_plan.h).
    struct LinePlanDev
    {
        int32_t L, P, B, periodic, nlast;
        float a;              // off-diagonal, a == c == -r/2
        const float *coef;    // [3][kCoefCount][M]
        const float *gband;   // [(P-1)][2B+1]
        const float *zsm;     // [L], periodic only
        float bog, invDenom;  // periodic: beta/gamma, 1/(1 + v.z_sm)
    };

    enum SweepMode : int
    {
        kSweepW = 0,      // x-sweep: out (transposed) = w
        kSweepTick = 1,   // y-sweep: out (transposed) = committed f'
        kSweepPlain = 2,  // y-sweep: out (transposed) = v
        kSweepDeltas = 3  // y-sweep: deltas (line-major, FP64) += v - f64
    };

    struct SweepParams
    {
        const float *in;          // Nlines lines of L floats, line-major
        int32_t L, Nlines;
        int32_t wrapLines;        // the explicit (cross-line) axis wraps
        const float *ghostLo;     // Dirichlet ghost line before line 0 (L values) or null
        const float *ghostHi;     // ghost line after line Nlines-1
        const float *implLo;      // Dirichlet value before position 0, per line, or null
        const float *implHi;      // Dirichlet value after position L-1, per line
        float halfR, r;
        LinePlanDev plan;         // lines of length L along the implicit axis
        int32_t R, LS;            // lines per CTA, shared-memory line stride (floats)
        float *out;               // transposed output: out[pos * Nlines + line]
        const float *f;           // kSweepTick: field before the step (output layout)
        const float *src;         // kSweepTick: dense source (output layout) or null
        const int32_t *cellOffsets;  // kSweepTick: agent bins (line-major), or null
        float negDecay, negUptake;
        const double *f64;        // kSweepDeltas: field (line-major)
        double *deltas;           // kSweepDeltas: deltas (line-major)
        int32_t *err;             // set to 1 if a bounded wait gave up
        // Floats between consecutive input lines (>= L) and between
        // consecutive output rows (>= Nlines).  A stride above the length
        // pads each line or row to a multiple of 4 floats: the padding of the
        // input lines must hold zeros, and the sweep writes zeros into the
        // padding of its output rows, so that the next sweep can stage every
        // line with 16-byte copies and write whole 16-byte units.
        int32_t inStride, outStride;
    };

    // Device copy of the line plan (adi_plan.h) of lines of length L at rate
    // r with the given ends (AdiEnds); owns its device buffers.
    class AdiDevicePlan
    {
    public:
        AdiDevicePlan() = default;
        ~AdiDevicePlan();
        AdiDevicePlan(const AdiDevicePlan &) = delete;
        AdiDevicePlan &operator=(const AdiDevicePlan &) = delete;

        int Build(int32_t L, double r, int ends);
        const LinePlanDev &Dev() const { return m_dev; }

    private:
        float *m_pCoef = nullptr;
        float *m_pGband = nullptr;
        float *m_pZsm = nullptr;
        LinePlanDev m_dev{};
    };

    // out[c][r] = in[r][c] for a rows x cols FP32 matrix.
    int LaunchTranspose(const float *in, float *out, int32_t rows, int32_t cols, cudaStream_t s);

    // The same with row strides: out[c * outStride + r] = in[r * inStride + c]
    // (inStride >= cols, outStride >= rows); padding is left untouched.
    int LaunchTransposeStrided(const float *in, int32_t inStride, float *out, int32_t outStride, int32_t rows,
                               int32_t cols, cudaStream_t s);

    // ---- batched sweeps (many independent grids in one launch) ------------
    //
    // A tile is (index into the SweepParams table, first line).  A grid's
    // lines per CTA (SweepParams::R) and shared-memory stride (LS) come from
    // SweepTileShape; every CTA of a launch has the largest thread count of
    // its tiles (at most kSweepTileThreads) and the largest shared memory.
    constexpr int32_t kSweepTileThreads = 512;

    struct SweepTileShape
    {
        int32_t R, LS;
        int32_t threads;  // threads the tile needs: (R / 2) * P, rounded up to a warp
        size_t smem;      // dynamic shared memory of one CTA
    };

    // Shape of the tiles of a grid whose lines have P = ceil(L/32) chunks:
    // the most lines per CTA (a power of two, at least 8, at most rCap)
    // that `budget` threads cover.  Budgets below kSweepTileThreads give
    // smaller CTAs, several of which share an SM (each thread keeps up to 128
    // registers).
    constexpr int32_t kSweepTileMaxR = 128;
    SweepTileShape SweepTileShapeFor(int32_t P, int32_t rCap = kSweepTileMaxR, int32_t budget = kSweepTileThreads);

    // Enables `smem` bytes of dynamic shared memory for the batched kernel of
    // `mode` (kSweepW or kSweepTick); call before capturing a launch.
    int PrepareSweepTiles(int mode, size_t smem);

    // Launches nTiles CTAs of `threads` threads (at least every tile's
    // SweepTileShape::threads) of the batched kernel of `mode` (smem
    // prepared).
    int LaunchSweepTiles(int mode, const SweepParams *table, const int2 *tiles, int32_t nTiles, size_t smem,
                         int32_t threads, cudaStream_t s);
}
