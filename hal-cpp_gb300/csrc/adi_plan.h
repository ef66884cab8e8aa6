// adi_plan.h -- host-side precomputation for the ADI line solves.
//
// Every line of one ADI sweep solves the same tridiagonal matrix (constant
// off-diagonals -r/2, constant interior diagonal, fixed end rows:
// ADISolveRow, include/Hal/Pde/ADIequations.h:225-270).  Only the right-hand
// side differs between lines.  So everything that depends on the matrix
// alone is computed once here, in FP64, and the device only runs
// O(1)-flop-per-element recurrences on the right-hand sides.
//
// Decomposition used on the device (a partitioned Thomas solve):
//   - the line of length L is cut into P = ceil(L/M) chunks of M rows;
//   - the last row of every chunk but the last is a separator s_k, the other
//     rows of chunk k form block k (M-1 rows; the last block has the rest);
//   - each block is solved by Thomas with the separators moved to the
//     right-hand side: x = z - s_{k-1} p - s_k q, where z = A_k^{-1} d and the
//     coupling vectors p = A_k^{-1}(a e_0), q = A_k^{-1}(c e_last) depend only
//     on the matrix;
//   - substituting into the separator rows gives a (P-1)x(P-1) tridiagonal
//     system whose matrix is again line-independent; its inverse G is
//     precomputed and, because it decays geometrically away from the
//     diagonal, stored as a band (entries below 2^-46 of the largest
//     diagonal entry dropped; the full matrix is kept when the band would be
//     wider).
// Periodic lines use the reference's Sherman-Morrison form
// (TdmaSolver::TDMAperiodic, include/Hal/Pde/TdmaSolver.h:68-120): the
// non-periodic system with adjusted end diagonals is solved as above, and the
// correction vector z_sm = A'^{-1}u is precomputed.
#pragma once

#include <cstdint>
#include <vector>

#ifdef __CUDACC__
#define HAL_HD __host__ __device__
#else
#define HAL_HD
#endif

namespace halcuda
{
    constexpr int kAdiM = 32;         // rows per chunk (registers per thread)
    constexpr int kAdiMaxChunks = 128;  // HAL_CUDA_ADI_MAX_LINE / kAdiM

    enum AdiEnds : int
    {
        kEndsZeroFlux = 0,
        kEndsDirichlet = 1,
        kEndsPeriodic = 2
    };

    // Coefficient arrays of one block type; entries past the block are the
    // identity (fw = 0, ib = 1, cb = 0, p = q = 0).
    enum AdiCoef : int
    {
        kCoefFw = 0,  // forward multiplier w_i = a / b'_{i-1}
        kCoefIb = 1,  // 1 / b'_i
        kCoefCb = 2,  // c / b'_i, 0 at the block's last row
        kCoefP = 3,   // A^{-1}(a e_0)
        kCoefQ = 4,   // A^{-1}(c e_last)
        kCoefCount = 5
    };

    struct AdiLinePlanHost
    {
        int32_t L = 0;
        int32_t P = 0;
        int32_t B = 0;       // band half-width of G
        int32_t ends = 0;
        double offDiag = 0;  // a = c = -r/2
        // [3 block types: first, middle, last][kCoefCount][kAdiM]
        std::vector<float> coef;
        // [(P-1)][2B+1], G[k][k-B+t]
        std::vector<float> gband;
        // periodic: z_sm (L values), beta/gamma, 1/(1 + v.z_sm)
        std::vector<float> zsm;
        double betaOverGamma = 0;
        double invDenom = 0;
        // largest |error| of the FP64 decomposition against a dense solve of
        // a test right-hand side (self-check, see BuildAdiLinePlan)
        double selfCheck = 0;
    };

    // Builds the plan for a line of length L (1 <= L <= kAdiM*kAdiMaxChunks)
    // at rate r with the given end condition.  Returns false if L is out of
    // range.
    bool BuildAdiLinePlan(int32_t L, double r, int ends, AdiLinePlanHost &out);

    // Block type of chunk k (0 = first, 1 = middle, 2 = last).  A single
    // chunk (P == 1) uses type 0, built with both end rows.
    HAL_HD inline int AdiBlockType(int32_t k, int32_t P)
    {
        if (k == 0)
        {
            return 0;
        }
        return (k == P - 1) ? 2 : 1;
    }
}
