// adi.cu -- ADI (alternating-direction implicit) diffusion on sm_103a.
//
// One ADI step (Internal::Diffusion2DADI, include/Hal/Pde/ADIequations.h:
// 306-378) is two sweeps:
//   x-sweep: for every column y, solve (I - r/2 Lx) w = (I + r/2 Ly) f along x
//            (lines of stride yDim) -> scratch w;
//   y-sweep: for every row x, solve (I - r/2 Ly) v = (I + r/2 Lx) w along y
//            (contiguous lines), then commit v.
// Each line is a tridiagonal system with the same matrix for every line of a
// sweep; adi_plan.h describes the partitioned Thomas solve used here and the
// FP64 precomputation it relies on.
//
// Kernel mapping (32-row chunks, one per thread, values kept in registers):
//   AdiColumnSweep -- a lane per column (coalesced 128-byte rows), a warp per
//     chunk of 32 rows, a thread-block cluster of up to 8 CTAs per 32-column
//     strip so that all chunks of a line sit in one cluster.  The separator
//     right-hand sides are exchanged through distributed shared memory.
//   AdiRowSweep -- a CTA stages R rows (plus the rows above and below, for
//     the explicit x part) in shared memory with coalesced loads, a thread
//     per (row, chunk) solves from shared memory, and the commit
//     (v - decay*f + source - uptake*count*f) streams back coalesced.
#include "common.cuh"
#include "adi_plan.h"

#include <cooperative_groups.h>

#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace cg = cooperative_groups;

namespace halcuda
{
    namespace
    {
        constexpr int M = kAdiM;
        constexpr int kCoefFloats = 3 * kCoefCount * M;
        constexpr int kRowThreads = 256;

        enum RowMode : int
        {
            kRowTick = 0,    // out = f + (v - f) - decay f + src - uptake n f
            kRowDeltas = 1,  // deltas (FP64) += v - f
            kRowPlain = 2    // out = v
        };

        enum NbrMode : int
        {
            kNbrGrid = 0,
            kNbrGhost = 1,
            kNbrNone = 2
        };

        __device__ __forceinline__ float NbrTerm(int mode, float v, float c)
        {
            return (mode == kNbrGrid) ? (v - c) : ((mode == kNbrGhost) ? (v - c) * 2.0f : 0.0f);
        }

        struct LinePlanDev
        {
            int32_t L, P, B, periodic, nlast;
            float a;              // off-diagonal, a == c == -r/2
            const float *coef;    // [3][kCoefCount][M]
            const float *gband;   // [(P-1)][2B+1]
            const float *zsm;     // [L], periodic only
            float bog, invDenom;  // periodic: beta/gamma, 1/(1 + v.z_sm)
        };

        __device__ __forceinline__ void ClusterArriveRelaxed()
        {
            asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory");
        }

        __device__ __forceinline__ void ClusterWait()
        {
            asm volatile("barrier.cluster.wait.aligned;\n" ::: "memory");
        }

        // Thomas forward elimination and back substitution of one block with
        // the identity padding described in adi_plan.h.
        __device__ __forceinline__ void BlockSolve(float (&z)[M], const float *cf)
        {
            const float *fw = cf + kCoefFw * M;
            const float *ib = cf + kCoefIb * M;
            const float *cb = cf + kCoefCb * M;
#pragma unroll
            for (int i = 1; i < M; i++)
            {
                z[i] = fmaf(-fw[i], z[i - 1], z[i]);
            }
            z[M - 1] *= ib[M - 1];
#pragma unroll
            for (int i = M - 2; i >= 0; i--)
            {
                z[i] = fmaf(-cb[i], z[i + 1], z[i] * ib[i]);
            }
        }

        // s_j = sum_m G[j][m] * (xA[m] + xB[m]) over the stored band.
        __device__ __forceinline__ float BandDot(const LinePlanDev &pl, int j, const float *xA,
                                                 const float *xB, int stride)
        {
            const int S = pl.P - 1;
            const int lo = max(0, j - pl.B);
            const int hi = min(S - 1, j + pl.B);
            const float *g = pl.gband + static_cast<int64_t>(j) * (2 * pl.B + 1);
            float acc = 0.0f;
            for (int m = lo; m <= hi; m++)
            {
                acc = fmaf(__ldg(g + (m - j + pl.B)), xA[m * stride] + xB[m * stride], acc);
            }
            return acc;
        }

        // z[idx] for a run-time idx without dynamic register indexing.
        __device__ __forceinline__ float SelectReg(const float (&z)[M], int idx)
        {
            float v = 0.0f;
#pragma unroll
            for (int i = 0; i < M; i++)
            {
                v = (i == idx) ? z[i] : v;
            }
            return v;
        }

        __device__ __forceinline__ float LoadAsFloat(const float *p)
        {
            return __ldg(p);
        }

        __device__ __forceinline__ float LoadAsFloat(const double *p)
        {
            return static_cast<float>(__ldg(p));
        }

        // ---------------------------------------------------------------
        // x-sweep: lines along x (stride yDim), a lane per column.
        // ---------------------------------------------------------------
        template <typename TIn>
        struct ColParams
        {
            const TIn *f;
            float *w;
            int32_t L;      // xDim (line length)
            int32_t ncols;  // yDim
            float halfR, r;
            int32_t wrapY;
            GhostView ghost;
            LinePlanDev plan;
        };

        // Right-hand side (I + r/2 Ly) f at (row, col) plus the Dirichlet
        // source of the implicit axis (ExplicitDiffusionY2ADI,
        // src/Pde/ADIequations.cpp:34-47; ImplicitBoundarySource,
        // ADIequations.h:198-220).  Called by all 32 lanes together.
        template <typename TIn>
        __device__ __forceinline__ float ColumnRhs(const ColParams<TIn> &p, int32_t row, int32_t col,
                                                   bool colOk, int lane)
        {
            const TIn *rowp = p.f + static_cast<int64_t>(row) * p.ncols;
            float c = colOk ? LoadAsFloat(rowp + col) : 0.0f;
            float left = __shfl_up_sync(0xffffffffu, c, 1);
            float right = __shfl_down_sync(0xffffffffu, c, 1);
            if (!colOk)
            {
                return 0.0f;
            }
            if (lane == 0 && col > 0)
            {
                left = LoadAsFloat(rowp + col - 1);
            }
            if (lane == 31 && col + 1 < p.ncols)
            {
                right = LoadAsFloat(rowp + col + 1);
            }
            float tp, tm;
            if (col + 1 < p.ncols)
            {
                tp = right - c;
            }
            else if (p.wrapY)
            {
                tp = LoadAsFloat(rowp) - c;
            }
            else if (p.ghost.yhi != nullptr)
            {
                tp = (__ldg(p.ghost.yhi + row) - c) * 2.0f;
            }
            else
            {
                tp = 0.0f;
            }
            if (col > 0)
            {
                tm = left - c;
            }
            else if (p.wrapY)
            {
                tm = LoadAsFloat(rowp + p.ncols - 1) - c;
            }
            else if (p.ghost.ylo != nullptr)
            {
                tm = (__ldg(p.ghost.ylo + row) - c) * 2.0f;
            }
            else
            {
                tm = 0.0f;
            }
            float d = fmaf(tp + tm, p.halfR, c);
            if (p.ghost.xlo != nullptr && !p.plan.periodic)
            {
                if (row == 0)
                {
                    d = fmaf(p.r, __ldg(p.ghost.xlo + col), d);
                }
                if (row == p.L - 1)
                {
                    d = fmaf(p.r, __ldg(p.ghost.xhi + col), d);
                }
            }
            return d;
        }

        template <typename TIn>
        __global__ void __launch_bounds__(512) AdiColumnSweep(ColParams<TIn> p)
        {
            __shared__ float sCoef[kCoefFloats];
            __shared__ float xA[kAdiMaxChunks * 32];
            __shared__ float xB[kAdiMaxChunks * 32];
            __shared__ float xZ0[32];
            __shared__ float xZL[32];

            cg::cluster_group cl = cg::this_cluster();
            const int lane = threadIdx.x;
            const int warp = threadIdx.y;
            const int W = blockDim.y;
            const unsigned K = cl.num_blocks();
            const int rank = static_cast<int>(cl.block_rank());
            const int tid = warp * 32 + lane;
            for (int q = tid; q < kCoefFloats; q += 32 * W)
            {
                sCoef[q] = __ldg(p.plan.coef + q);
            }
            __syncthreads();
            ClusterArriveRelaxed();

            const int P = p.plan.P;
            const int k = rank * W + warp;
            const int32_t col = blockIdx.y * 32 + lane;
            const bool colOk = col < p.ncols;
            const bool chunkOk = k < P;
            const int32_t base = k * M;

            float z[M];
#pragma unroll
            for (int i = 0; i < M; i++)
            {
                const int32_t row = base + i;
                z[i] = 0.0f;
                if (chunkOk && row < p.L)  // warp-uniform
                {
                    z[i] = ColumnRhs(p, row, col, colOk, lane);
                }
            }

            const int type = AdiBlockType(k, P);
            const float *cf = sCoef + type * kCoefCount * M;
            if (chunkOk)
            {
                BlockSolve(z, cf);
            }

            const float a = p.plan.a;
            ClusterWait();  // every CTA of the cluster is running
            if (chunkOk && k < P - 1)
            {
                const float vA = fmaf(-a, z[M - 2], z[M - 1]);
                for (unsigned q = 0; q < K; q++)
                {
                    cl.map_shared_rank(xA, q)[k * 32 + lane] = vA;
                }
            }
            if (chunkOk && k >= 1)
            {
                const float vB = -a * z[0];
                for (unsigned q = 0; q < K; q++)
                {
                    cl.map_shared_rank(xB, q)[(k - 1) * 32 + lane] = vB;
                }
            }
            if (p.plan.periodic && P > 1)
            {
                if (k == 0)
                {
                    for (unsigned q = 0; q < K; q++)
                    {
                        cl.map_shared_rank(xZ0, q)[lane] = z[0];
                    }
                }
                if (k == P - 1)
                {
                    const float zl = SelectReg(z, p.plan.nlast - 1);
                    for (unsigned q = 0; q < K; q++)
                    {
                        cl.map_shared_rank(xZL, q)[lane] = zl;
                    }
                }
            }
            cl.sync();

            if (chunkOk)
            {
                float sL = 0.0f, sR = 0.0f;
                if (P > 1)
                {
                    if (k < P - 1)
                    {
                        sR = BandDot(p.plan, k, xA + lane, xB + lane, 32);
                    }
                    if (k >= 1)
                    {
                        sL = BandDot(p.plan, k - 1, xA + lane, xB + lane, 32);
                    }
                }
                const float *pv = cf + kCoefP * M;
                const float *qv = cf + kCoefQ * M;
#pragma unroll
                for (int i = 0; i < M; i++)
                {
                    z[i] = fmaf(-sL, pv[i], fmaf(-sR, qv[i], z[i]));
                }
                if (k < P - 1)
                {
                    z[M - 1] = sR;
                }
                if (p.plan.periodic)
                {
                    float y0, yl;
                    if (P == 1)
                    {
                        y0 = z[0];
                        yl = SelectReg(z, p.L - 1);
                    }
                    else
                    {
                        const float s0 = BandDot(p.plan, 0, xA + lane, xB + lane, 32);
                        const float sl = BandDot(p.plan, P - 2, xA + lane, xB + lane, 32);
                        y0 = xZ0[lane] - s0 * sCoef[0 * kCoefCount * M + kCoefQ * M + 0];
                        yl = xZL[lane] - sl * sCoef[2 * kCoefCount * M + kCoefP * M + p.plan.nlast - 1];
                    }
                    const float factor = fmaf(yl, p.plan.bog, y0) * p.plan.invDenom;
#pragma unroll
                    for (int i = 0; i < M; i++)
                    {
                        const int32_t row = base + i;
                        if (row < p.L)
                        {
                            z[i] = fmaf(-factor, __ldg(p.plan.zsm + row), z[i]);
                        }
                    }
                }
                if (colOk)
                {
#pragma unroll
                    for (int i = 0; i < M; i++)
                    {
                        const int32_t row = base + i;
                        if (row < p.L)
                        {
                            p.w[static_cast<int64_t>(row) * p.ncols + col] = z[i];
                        }
                    }
                }
            }
        }

        // ---------------------------------------------------------------
        // y-sweep: contiguous lines, R rows per CTA staged in shared memory.
        // ---------------------------------------------------------------
        template <typename TF>
        struct RowParams
        {
            const float *w;        // x-sweep result
            const TF *f;           // field before the step (commit input)
            float *out;            // kRowTick / kRowPlain
            double *deltas;        // kRowDeltas
            const float *src;      // dense source or null
            const int32_t *cellOffsets;  // uptake counts (offsets[c+1]-offsets[c]) or null
            float negUptake, negDecay;
            int32_t xDim;
            int32_t L;             // yDim
            float halfR, r;
            int32_t wrapX;
            GhostView ghost;
            LinePlanDev plan;
            int32_t R;             // rows per CTA
            int32_t LP;            // padded row length in shared memory
        };

        __device__ __forceinline__ int PadIdx(int32_t y)
        {
            return (y / M) * (M + 1) + (y % M);
        }

        template <typename TF, int MODE>
        __global__ void __launch_bounds__(kRowThreads) AdiRowSweep(RowParams<TF> p)
        {
            extern __shared__ float smem[];
            float *sCoef = smem;
            float *sRows = sCoef + kCoefFloats;                 // (R+2) * LP
            float *xA = sRows + (p.R + 2) * p.LP;                // R * P
            float *xB = xA + p.R * p.plan.P;                     // R * P
            float *xZ0 = xB + p.R * p.plan.P;                    // R
            float *xZL = xZ0 + p.R;                              // R

            const int tid = threadIdx.x;
            const int nthreads = blockDim.x;
            const int P = p.plan.P;
            const int32_t x0 = blockIdx.x * p.R;

            for (int q = tid; q < kCoefFloats; q += nthreads)
            {
                sCoef[q] = __ldg(p.plan.coef + q);
            }
            // Stage rows x0-1 .. x0+R of w.
            for (int rr = 0; rr < p.R + 2; rr++)
            {
                int32_t xg = x0 - 1 + rr;
                const float *src = nullptr;
                const float *ghostRow = nullptr;
                if (xg >= 0 && xg < p.xDim)
                {
                    src = p.w + static_cast<int64_t>(xg) * p.L;
                }
                else if (p.wrapX)
                {
                    int32_t xw = (xg < 0) ? xg + p.xDim : xg - p.xDim;
                    src = p.w + static_cast<int64_t>(xw) * p.L;
                }
                else if (p.ghost.xlo != nullptr)
                {
                    ghostRow = (xg < 0) ? p.ghost.xlo : p.ghost.xhi;
                }
                float *dst = sRows + rr * p.LP;
                if (src != nullptr && (p.L % 4) == 0)
                {
                    const float4 *s4 = reinterpret_cast<const float4 *>(src);
                    for (int32_t q = tid; q < p.L / 4; q += nthreads)
                    {
                        float4 v = __ldg(s4 + q);
                        int32_t y = q * 4;
                        int o = PadIdx(y);
                        dst[o] = v.x;
                        dst[o + 1] = v.y;
                        dst[o + 2] = v.z;
                        dst[o + 3] = v.w;
                    }
                }
                else
                {
                    for (int32_t y = tid; y < p.L; y += nthreads)
                    {
                        float v = 0.0f;
                        if (src != nullptr)
                        {
                            v = __ldg(src + y);
                        }
                        else if (ghostRow != nullptr)
                        {
                            v = __ldg(ghostRow + y);
                        }
                        dst[PadIdx(y)] = v;
                    }
                }
            }
            __syncthreads();

            const int rho = tid / P;
            const int k = tid - rho * P;
            const int32_t x = x0 + rho;
            const bool active = (rho < p.R) && (x < p.xDim);
            const int type = AdiBlockType(k, P);
            const float *cf = sCoef + type * kCoefCount * M;

            float z[M];
            if (active)
            {
                const int upMode = (x - 1 >= 0 || p.wrapX) ? kNbrGrid : ((p.ghost.xlo != nullptr) ? kNbrGhost : kNbrNone);
                const int dnMode = (x + 1 < p.xDim || p.wrapX) ? kNbrGrid : ((p.ghost.xlo != nullptr) ? kNbrGhost : kNbrNone);
                const float *rowC = sRows + (rho + 1) * p.LP + k * (M + 1);
                const float *rowU = rowC - p.LP;
                const float *rowD = rowC + p.LP;
#pragma unroll
                for (int i = 0; i < M; i++)
                {
                    const int32_t y = k * M + i;
                    const float c = rowC[i];
                    // ExplicitDiffusionX2ADI order: x+1 then x-1
                    float d = fmaf(NbrTerm(dnMode, rowD[i], c) + NbrTerm(upMode, rowU[i], c), p.halfR, c);
                    if (p.ghost.ylo != nullptr && !p.plan.periodic)
                    {
                        if (y == 0)
                        {
                            d = fmaf(p.r, __ldg(p.ghost.ylo + x), d);
                        }
                        if (y == p.L - 1)
                        {
                            d = fmaf(p.r, __ldg(p.ghost.yhi + x), d);
                        }
                    }
                    z[i] = (y < p.L) ? d : 0.0f;
                }
                BlockSolve(z, cf);
                const float a = p.plan.a;
                if (k < P - 1)
                {
                    xA[rho * P + k] = fmaf(-a, z[M - 2], z[M - 1]);
                }
                if (k >= 1)
                {
                    xB[rho * P + k - 1] = -a * z[0];
                }
                if (p.plan.periodic && P > 1)
                {
                    if (k == 0)
                    {
                        xZ0[rho] = z[0];
                    }
                    if (k == P - 1)
                    {
                        xZL[rho] = SelectReg(z, p.plan.nlast - 1);
                    }
                }
            }
            __syncthreads();
            if (active)
            {
                const float *rA = xA + rho * P;
                const float *rB = xB + rho * P;
                float sL = 0.0f, sR = 0.0f;
                if (P > 1)
                {
                    if (k < P - 1)
                    {
                        sR = BandDot(p.plan, k, rA, rB, 1);
                    }
                    if (k >= 1)
                    {
                        sL = BandDot(p.plan, k - 1, rA, rB, 1);
                    }
                }
                const float *pv = cf + kCoefP * M;
                const float *qv = cf + kCoefQ * M;
#pragma unroll
                for (int i = 0; i < M; i++)
                {
                    z[i] = fmaf(-sL, pv[i], fmaf(-sR, qv[i], z[i]));
                }
                if (k < P - 1)
                {
                    z[M - 1] = sR;
                }
                if (p.plan.periodic)
                {
                    float y0, yl;
                    if (P == 1)
                    {
                        y0 = z[0];
                        yl = SelectReg(z, p.L - 1);
                    }
                    else
                    {
                        const float s0 = BandDot(p.plan, 0, rA, rB, 1);
                        const float sl = BandDot(p.plan, P - 2, rA, rB, 1);
                        y0 = xZ0[rho] - s0 * sCoef[0 * kCoefCount * M + kCoefQ * M + 0];
                        yl = xZL[rho] - sl * sCoef[2 * kCoefCount * M + kCoefP * M + p.plan.nlast - 1];
                    }
                    const float factor = fmaf(yl, p.plan.bog, y0) * p.plan.invDenom;
#pragma unroll
                    for (int i = 0; i < M; i++)
                    {
                        const int32_t y = k * M + i;
                        if (y < p.L)
                        {
                            z[i] = fmaf(-factor, __ldg(p.plan.zsm + y), z[i]);
                        }
                    }
                }
                // the halo reads of every thread finished before the barrier
                // above, so the row buffer can take the solution
                float *rowC = sRows + (rho + 1) * p.LP + k * (M + 1);
#pragma unroll
                for (int i = 0; i < M; i++)
                {
                    rowC[i] = z[i];
                }
            }
            __syncthreads();

            // Commit, streamed row by row with coalesced accesses.
            for (int rr = 0; rr < p.R; rr++)
            {
                const int32_t xr = x0 + rr;
                if (xr >= p.xDim)
                {
                    break;
                }
                const float *rowV = sRows + (rr + 1) * p.LP;
                const int64_t rowBase = static_cast<int64_t>(xr) * p.L;
                for (int32_t y = tid; y < p.L; y += nthreads)
                {
                    const float v = rowV[PadIdx(y)];
                    const int64_t i = rowBase + y;
                    if constexpr (MODE == kRowPlain)
                    {
                        p.out[i] = v;
                    }
                    else if constexpr (MODE == kRowDeltas)
                    {
                        const double fv = p.f[i];
                        p.deltas[i] = p.deltas[i] + (static_cast<double>(v) - fv);
                    }
                    else
                    {
                        const float fv = static_cast<float>(p.f[i]);
                        float d = v - fv;
                        d = fmaf(fv, p.negDecay, d);
                        if (p.src != nullptr)
                        {
                            d += __ldg(p.src + i);
                        }
                        if (p.cellOffsets != nullptr)
                        {
                            const int32_t n = __ldg(p.cellOffsets + i + 1) - __ldg(p.cellOffsets + i);
                            d = fmaf(fv, p.negUptake * static_cast<float>(n), d);
                        }
                        p.out[i] = fv + d;
                    }
                }
            }
        }

        // Device copy of one line plan.
        struct LinePlanBuf
        {
            DevBuf<float> coef, gband, zsm;
            LinePlanDev dev{};
            AdiLinePlanHost host;
        };

        int UploadPlan(int32_t L, double r, int ends, LinePlanBuf &pb)
        {
            if (!BuildAdiLinePlan(L, r, ends, pb.host))
            {
                SetError("ADI line length %d outside [1, %d]", L, HAL_CUDA_ADI_MAX_LINE);
                return HAL_CUDA_ENOTSUP;
            }
            if (!(pb.host.selfCheck < 1e-5))
            {
                SetError("ADI plan self-check failed (L=%d, r=%g, rel err %g)", L, r, pb.host.selfCheck);
                return HAL_CUDA_ENOTSUP;
            }
            const AdiLinePlanHost &h = pb.host;
            HAL_TRY(pb.coef.Alloc(h.coef.size(), "cudaMalloc(plan)"));
            HAL_TRY(CudaStatus(cudaMemcpy(pb.coef.p, h.coef.data(), h.coef.size() * sizeof(float),
                                          cudaMemcpyHostToDevice), "cudaMemcpy(plan)"));
            if (!h.gband.empty())
            {
                HAL_TRY(pb.gband.Alloc(h.gband.size(), "cudaMalloc(plan)"));
                HAL_TRY(CudaStatus(cudaMemcpy(pb.gband.p, h.gband.data(), h.gband.size() * sizeof(float),
                                              cudaMemcpyHostToDevice), "cudaMemcpy(plan)"));
            }
            if (!h.zsm.empty())
            {
                HAL_TRY(pb.zsm.Alloc(h.zsm.size(), "cudaMalloc(plan)"));
                HAL_TRY(CudaStatus(cudaMemcpy(pb.zsm.p, h.zsm.data(), h.zsm.size() * sizeof(float),
                                              cudaMemcpyHostToDevice), "cudaMemcpy(plan)"));
            }
            LinePlanDev &d = pb.dev;
            d.L = h.L;
            d.P = h.P;
            d.B = h.B;
            d.periodic = (ends == kEndsPeriodic);
            d.nlast = h.L - (h.P - 1) * M;
            d.a = static_cast<float>(h.offDiag);
            d.coef = pb.coef.p;
            d.gband = pb.gband.p;
            d.zsm = pb.zsm.p;
            d.bog = static_cast<float>(h.betaOverGamma);
            d.invDenom = static_cast<float>(h.invDenom);
            return HAL_CUDA_OK;
        }

        size_t RowSmemBytes(int32_t R, int32_t LP, int32_t P)
        {
            return sizeof(float) * (static_cast<size_t>(kCoefFloats) + static_cast<size_t>(R + 2) * LP +
                                    2 * static_cast<size_t>(R) * P + 2 * static_cast<size_t>(R));
        }

        template <typename TF, int MODE>
        int EnableRowSmem(size_t bytes)
        {
            static size_t s_enabled = 0;
            if (bytes > s_enabled)
            {
                HAL_TRY(CudaStatus(cudaFuncSetAttribute(AdiRowSweep<TF, MODE>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        static_cast<int>(bytes)),
                                   "cudaFuncSetAttribute(AdiRowSweep)"));
                s_enabled = bytes;
            }
            return HAL_CUDA_OK;
        }
    }

}

struct hal_cuda_agents;  // agents.cu

namespace halcuda
{
    // Device cell offsets of an agent handle's last dispatch and its grid.
    const int32_t *AgentsCellOffsets(const hal_cuda_agents *a, int32_t *xDim, int32_t *yDim);

    struct Adi
    {
        int32_t xDim = 0, yDim = 0;
        int device = 0;
        StreamSlot stream;
        DevBuf<float> field[2];
        int cur = 0;
        DevBuf<float> w;
        DevBuf<float> src;
        bool hasSrc = false;
        DevBuf<float> ghost;
        bool hasGhost = false;
        DevBuf<double> f64, d64;
        DevBuf<float> g32;  // ghost table of the FP64 interface call, in float
        const hal_cuda_agents *agents = nullptr;
        double uptake = 0.0;
        std::map<std::string, std::unique_ptr<LinePlanBuf>> plans;
        GraphCache graph[2];  // by the parity of the starting buffer

        void ResetGraphs()
        {
            graph[0].Reset();
            graph[1].Reset();
        }

        int Init(int32_t x, int32_t y)
        {
            xDim = x;
            yDim = y;
            device = CurrentDevice();
            HAL_TRY(CudaStatus(cudaSetDevice(device), "cudaSetDevice"));
            HAL_TRY(stream.Create("cudaStreamCreate"));
            size_t n = Length();
            HAL_TRY(field[0].Alloc(n, "cudaMalloc(field)"));
            HAL_TRY(field[1].Alloc(n, "cudaMalloc(field)"));
            HAL_TRY(w.Alloc(n, "cudaMalloc(scratch)"));
            HAL_TRY(CudaStatus(cudaMemset(field[0].p, 0, n * sizeof(float)), "cudaMemset"));
            return HAL_CUDA_OK;
        }

        size_t Length() const
        {
            return static_cast<size_t>(xDim) * static_cast<size_t>(yDim);
        }

        int Plan(int32_t L, double r, int ends, const LinePlanDev **out)
        {
            char key[96];
            snprintf(key, sizeof(key), "%d|%a|%d", L, r, ends);
            auto it = plans.find(key);
            if (it == plans.end())
            {
                if (plans.size() > 16)
                {
                    // plans captured in the cached graph may be freed
                    HAL_TRY(CudaStatus(cudaStreamSynchronize(stream.Get()), "cudaStreamSynchronize"));
                    ResetGraphs();
                    plans.clear();
                }
                auto pb = std::make_unique<LinePlanBuf>();
                HAL_TRY(UploadPlan(L, r, ends, *pb));
                it = plans.emplace(key, std::move(pb)).first;
            }
            *out = &it->second->dev;
            return HAL_CUDA_OK;
        }

        template <typename TIn>
        int LaunchColumn(const TIn *f, double r, bool wrapX, bool wrapY, const float *ghostTab,
                         cudaStream_t s)
        {
            const LinePlanDev *pl = nullptr;
            int ends = wrapX ? kEndsPeriodic : (ghostTab ? kEndsDirichlet : kEndsZeroFlux);
            HAL_TRY(Plan(xDim, r, ends, &pl));
            ColParams<TIn> p;
            p.f = f;
            p.w = w.p;
            p.L = xDim;
            p.ncols = yDim;
            p.halfR = static_cast<float>(r / 2.0);
            p.r = static_cast<float>(r);
            p.wrapY = wrapY;
            p.ghost = MakeGhostView(ghostTab, xDim, yDim);
            p.plan = *pl;
            const int P = pl->P;
            int K = (P + 7) / 8;
            if (K > 8)
            {
                K = 8;
            }
            int W = (P + K - 1) / K;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(K, (yDim + 31) / 32, 1);
            cfg.blockDim = dim3(32, W, 1);
            cfg.dynamicSmemBytes = 0;
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = K;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            cudaError_t e = cudaLaunchKernelEx(&cfg, AdiColumnSweep<TIn>, p);
            CountLaunch();
            return CudaStatus(e, "AdiColumnSweep launch");
        }

        template <typename TF, int MODE>
        int LaunchRow(const TF *f, float *out, double *deltas, double r, double decay, bool wrapX,
                      bool wrapY, const float *ghostTab, bool extras, cudaStream_t s)
        {
            const LinePlanDev *pl = nullptr;
            int ends = wrapY ? kEndsPeriodic : (ghostTab ? kEndsDirichlet : kEndsZeroFlux);
            HAL_TRY(Plan(yDim, r, ends, &pl));
            RowParams<TF> p;
            p.w = w.p;
            p.f = f;
            p.out = out;
            p.deltas = deltas;
            p.src = (extras && hasSrc) ? src.p : nullptr;
            p.cellOffsets = nullptr;
            p.negUptake = 0.0f;
            if (extras && agents != nullptr)
            {
                int32_t ax = 0, ay = 0;
                p.cellOffsets = AgentsCellOffsets(agents, &ax, &ay);
                p.negUptake = static_cast<float>(-uptake);
            }
            p.negDecay = static_cast<float>(-decay);
            p.xDim = xDim;
            p.L = yDim;
            p.halfR = static_cast<float>(r / 2.0);
            p.r = static_cast<float>(r);
            p.wrapX = wrapX;
            p.ghost = MakeGhostView(ghostTab, xDim, yDim);
            p.plan = *pl;
            const int P = pl->P;
            int R = kRowThreads / P;
            if (R < 1)
            {
                R = 1;
            }
            p.R = R;
            p.LP = P * (M + 1);
            int threads = ((R * P + 31) / 32) * 32;
            size_t smem = RowSmemBytes(R, p.LP, P);
            HAL_TRY((EnableRowSmem<TF, MODE>(smem)));
            unsigned blocks = static_cast<unsigned>((xDim + R - 1) / R);
            AdiRowSweep<TF, MODE><<<blocks, threads, smem, s>>>(p);
            CountLaunch();
            return LaunchStatus("AdiRowSweep launch");
        }

        int EnqueueTick(int c, double r, double decay, bool wrapX, bool wrapY, bool extras, int mode,
                        cudaStream_t s)
        {
            const float *g = (mode != kRowPlain && hasGhost) ? ghost.p : nullptr;
            HAL_TRY(LaunchColumn<float>(field[c].p, r, wrapX, wrapY, g, s));
            if (mode == kRowPlain)
            {
                return LaunchRow<float, kRowPlain>(field[c].p, field[c ^ 1].p, nullptr, r, decay, wrapX, wrapY,
                                                   nullptr, false, s);
            }
            return LaunchRow<float, kRowTick>(field[c].p, field[c ^ 1].p, nullptr, r, decay, wrapX, wrapY, g,
                                              extras, s);
        }

        int RunTicks(int32_t ticks, double r, double decay, bool wrapX, bool wrapY, bool plain)
        {
            if (ticks <= 0)
            {
                return HAL_CUDA_OK;
            }
            cudaStream_t s = stream.Get();
            // make sure both plans exist before capture (no allocation inside)
            const LinePlanDev *pl = nullptr;
            const float *g = (!plain && hasGhost) ? ghost.p : nullptr;
            HAL_TRY(Plan(xDim, r, wrapX ? kEndsPeriodic : (g ? kEndsDirichlet : kEndsZeroFlux), &pl));
            HAL_TRY(Plan(yDim, r, wrapY ? kEndsPeriodic : (g ? kEndsDirichlet : kEndsZeroFlux), &pl));
            char key[256];
            snprintf(key, sizeof(key), "%d|%a|%a|%d|%d|%d|%d|%d|%p|%p|%a", ticks, r, decay, wrapX, wrapY,
                     plain ? 1 : 0, hasSrc, hasGhost, static_cast<void *>(s),
                     static_cast<const void *>(agents), uptake);
            GraphCache &graph = this->graph[cur];
            if (graph.exec == nullptr || graph.key != key)
            {
                graph.Reset();
                // Warm the per-kernel shared-memory attribute outside capture.
                {
                    const LinePlanDev *py = nullptr;
                    HAL_TRY(Plan(yDim, r, wrapY ? kEndsPeriodic : (g ? kEndsDirichlet : kEndsZeroFlux), &py));
                    int R = kRowThreads / py->P;
                    R = R < 1 ? 1 : R;
                    size_t smem = RowSmemBytes(R, py->P * (M + 1), py->P);
                    HAL_TRY((EnableRowSmem<float, kRowTick>(smem)));
                    HAL_TRY((EnableRowSmem<float, kRowPlain>(smem)));
                }
                cudaGraph_t gr = nullptr;
                HAL_TRY(CudaStatus(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                                   "cudaStreamBeginCapture"));
                int c = cur;
                int rc = HAL_CUDA_OK;
                for (int32_t t = 0; t < ticks && rc == HAL_CUDA_OK; t++)
                {
                    rc = EnqueueTick(c, r, decay, wrapX, wrapY, true, plain ? kRowPlain : kRowTick, s);
                    c ^= 1;
                }
                cudaError_t e = cudaStreamEndCapture(s, &gr);
                if (rc != HAL_CUDA_OK)
                {
                    if (gr != nullptr)
                    {
                        cudaGraphDestroy(gr);
                    }
                    return rc;
                }
                HAL_TRY(CudaStatus(e, "cudaStreamEndCapture"));
                e = cudaGraphInstantiate(&graph.exec, gr, 0);
                cudaGraphDestroy(gr);
                HAL_TRY(CudaStatus(e, "cudaGraphInstantiate"));
                graph.key = key;
            }
            else
            {
                CountLaunch(2 * static_cast<int64_t>(ticks));
            }
            HAL_TRY(CudaStatus(cudaGraphLaunch(graph.exec, s), "cudaGraphLaunch"));
            cur ^= (ticks & 1);
            return HAL_CUDA_OK;
        }
    };
}

using halcuda::Adi;

struct hal_cuda_adi : public Adi
{
};

extern "C" int hal_cuda_adi_create(int32_t xDim, int32_t yDim, hal_cuda_adi **out)
{
    HAL_REQUIRE(out != nullptr, "hal_cuda_adi_create: out is NULL");
    *out = nullptr;
    HAL_REQUIRE(xDim > 0 && yDim > 0, "hal_cuda_adi_create: dimensions must be positive");
    if (xDim > HAL_CUDA_ADI_MAX_LINE || yDim > HAL_CUDA_ADI_MAX_LINE)
    {
        halcuda::SetError("hal_cuda_adi_create: ADI lines are limited to %d cells (got %d x %d)",
                          HAL_CUDA_ADI_MAX_LINE, xDim, yDim);
        return HAL_CUDA_ENOTSUP;
    }
    hal_cuda_adi *h = new (std::nothrow) hal_cuda_adi();
    if (h == nullptr)
    {
        halcuda::SetError("hal_cuda_adi_create: out of host memory");
        return HAL_CUDA_ENOMEM;
    }
    int rc = h->Init(xDim, yDim);
    if (rc != HAL_CUDA_OK)
    {
        delete h;
        return rc;
    }
    *out = h;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_adi_destroy(hal_cuda_adi *h)
{
    if (h != nullptr)
    {
        cudaSetDevice(h->device);
        cudaStreamSynchronize(h->stream.Get());
        delete h;
    }
    return HAL_CUDA_OK;
}

namespace
{
    int DiffuseAdiCommon(hal_cuda_adi *h, const double *field, double *deltas, double r, int32_t wrapX,
                         int32_t wrapY, const double *ghost, const char *who)
    {
        using namespace halcuda;
        HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
        size_t n = h->Length();
        if (h->f64.p == nullptr)
        {
            HAL_TRY(h->f64.Alloc(n, "cudaMalloc(f64)"));
            HAL_TRY(h->d64.Alloc(n, "cudaMalloc(d64)"));
            HAL_TRY(h->g32.Alloc(2 * (static_cast<size_t>(h->xDim) + h->yDim), "cudaMalloc(ghost)"));
        }
        cudaStream_t s = h->stream.Get();
        const float *g = nullptr;
        if (ghost != nullptr)
        {
            size_t ng = 2 * (static_cast<size_t>(h->xDim) + h->yDim);
            std::vector<float> gf(ng);
            for (size_t i = 0; i < ng; i++)
            {
                gf[i] = static_cast<float>(ghost[i]);
            }
            HAL_TRY(CudaStatus(cudaMemcpy(h->g32.p, gf.data(), ng * sizeof(float), cudaMemcpyHostToDevice),
                               "cudaMemcpy(ghost)"));
            g = h->g32.p;
        }
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->f64.p, field, n * sizeof(double), cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(field)"));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->d64.p, deltas, n * sizeof(double), cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(deltas)"));
        HAL_TRY(h->LaunchColumn<double>(h->f64.p, r, wrapX != 0, wrapY != 0, g, s));
        HAL_TRY((h->LaunchRow<double, halcuda::kRowDeltas>(h->f64.p, nullptr, h->d64.p, r, 0.0, wrapX != 0,
                                                           wrapY != 0, g, false, s)));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(deltas, h->d64.p, n * sizeof(double), cudaMemcpyDeviceToHost, s),
                           "cudaMemcpy(deltas)"));
        return CudaStatus(cudaStreamSynchronize(s), who);
    }
}

extern "C" int hal_cuda_diffuse_adi(hal_cuda_adi *h, const double *field, int64_t fieldLen, double *deltas,
                                    int64_t deltasLen, double diffRate, int32_t xDim, int32_t yDim,
                                    int32_t wrapX, int32_t wrapY)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffuse_adi: handle is NULL");
    int64_t length = static_cast<int64_t>(xDim) * yDim;
    HAL_REQUIRE(xDim > 0 && yDim > 0 && fieldLen == length && deltasLen == length,
                "CudaAdiDiffusionBackend2D::DiffuseADI: field and deltas must each hold xDim*yDim values");
    HAL_REQUIRE(xDim == h->xDim && yDim == h->yDim,
                "CudaAdiDiffusionBackend2D::DiffuseADI called with dimensions differing from construction");
    HAL_REQUIRE(field != nullptr && deltas != nullptr, "hal_cuda_diffuse_adi: NULL array");
    return DiffuseAdiCommon(h, field, deltas, diffRate, wrapX, wrapY, nullptr, "hal_cuda_diffuse_adi");
}

extern "C" int hal_cuda_diffuse_adi_bc(hal_cuda_adi *h, const double *field, double *deltas, double diffRate,
                                       int32_t wrapX, int32_t wrapY, const double *ghost)
{
    HAL_REQUIRE(h != nullptr && field != nullptr && deltas != nullptr, "hal_cuda_diffuse_adi_bc: NULL argument");
    return DiffuseAdiCommon(h, field, deltas, diffRate, wrapX, wrapY, ghost, "hal_cuda_diffuse_adi_bc");
}

extern "C" int hal_cuda_adi_set_field(hal_cuda_adi *h, const float *field, int64_t len)
{
    HAL_REQUIRE(h != nullptr && field != nullptr, "hal_cuda_adi_set_field: NULL argument");
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()), "hal_cuda_adi_set_field: field must hold xDim*yDim values");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    HAL_TRY(halcuda::CudaStatus(cudaMemcpyAsync(h->field[h->cur].p, field, h->Length() * sizeof(float),
                                                cudaMemcpyHostToDevice, s),
                                "cudaMemcpy(field)"));
    return halcuda::CudaStatus(cudaStreamSynchronize(s), "hal_cuda_adi_set_field");
}

extern "C" int hal_cuda_adi_get_field(hal_cuda_adi *h, float *field, int64_t len)
{
    HAL_REQUIRE(h != nullptr && field != nullptr, "hal_cuda_adi_get_field: NULL argument");
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()), "hal_cuda_adi_get_field: field must hold xDim*yDim values");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    HAL_TRY(halcuda::CudaStatus(cudaMemcpyAsync(field, h->field[h->cur].p, h->Length() * sizeof(float),
                                                cudaMemcpyDeviceToHost, s),
                                "cudaMemcpy(field)"));
    return halcuda::CudaStatus(cudaStreamSynchronize(s), "hal_cuda_adi_get_field");
}

extern "C" int hal_cuda_adi_set_source(hal_cuda_adi *h, const float *dense, int64_t len)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_adi_set_source: handle is NULL");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    if (dense == nullptr)
    {
        h->hasSrc = false;
        return HAL_CUDA_OK;
    }
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()), "hal_cuda_adi_set_source: source must hold xDim*yDim values");
    if (h->src.p == nullptr)
    {
        HAL_TRY(h->src.Alloc(h->Length(), "cudaMalloc(src)"));
    }
    HAL_TRY(halcuda::CudaStatus(cudaStreamSynchronize(h->stream.Get()), "cudaStreamSynchronize"));
    HAL_TRY(halcuda::CudaStatus(cudaMemcpy(h->src.p, dense, h->Length() * sizeof(float), cudaMemcpyHostToDevice),
                                "cudaMemcpy(src)"));
    h->hasSrc = true;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_adi_set_dirichlet(hal_cuda_adi *h, const float *ghost)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_adi_set_dirichlet: handle is NULL");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    if (ghost == nullptr)
    {
        h->hasGhost = false;
        return HAL_CUDA_OK;
    }
    size_t ng = 2 * (static_cast<size_t>(h->xDim) + h->yDim);
    if (h->ghost.p == nullptr)
    {
        HAL_TRY(h->ghost.Alloc(ng, "cudaMalloc(ghost)"));
    }
    HAL_TRY(halcuda::CudaStatus(cudaStreamSynchronize(h->stream.Get()), "cudaStreamSynchronize"));
    HAL_TRY(halcuda::CudaStatus(cudaMemcpy(h->ghost.p, ghost, ng * sizeof(float), cudaMemcpyHostToDevice),
                                "cudaMemcpy(ghost)"));
    h->hasGhost = true;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_adi_set_uptake(hal_cuda_adi *h, hal_cuda_agents *agents, double uptake)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_adi_set_uptake: handle is NULL");
    if (agents == nullptr)
    {
        h->agents = nullptr;
        h->uptake = 0.0;
        return HAL_CUDA_OK;
    }
    int32_t ax = 0, ay = 0;
    halcuda::AgentsCellOffsets(agents, &ax, &ay);
    HAL_REQUIRE(ax == h->xDim && ay == h->yDim,
                "hal_cuda_adi_set_uptake: agent grid %dx%d differs from the field %dx%d", ax, ay, h->xDim, h->yDim);
    h->agents = agents;
    h->uptake = uptake;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_adi_run_ticks(hal_cuda_adi *h, int32_t ticks, double diffRate, double decay, int32_t wrapX,
                                      int32_t wrapY)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_adi_run_ticks: handle is NULL");
    HAL_REQUIRE(ticks >= 0, "hal_cuda_adi_run_ticks: negative tick count");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return h->RunTicks(ticks, diffRate, decay, wrapX != 0, wrapY != 0, false);
}

extern "C" int hal_cuda_adi_run_steps(hal_cuda_adi *h, float *field, int64_t len, int32_t steps, double diffRate,
                                      int32_t wrapX, int32_t wrapY)
{
    HAL_REQUIRE(h != nullptr && field != nullptr, "hal_cuda_adi_run_steps: NULL argument");
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()), "AdiKernel2D::RunSteps: field must hold xDim*yDim values");
    HAL_REQUIRE(steps >= 0, "hal_cuda_adi_run_steps: negative step count");
    HAL_TRY(hal_cuda_adi_set_field(h, field, len));
    HAL_TRY(h->RunTicks(steps, diffRate, 0.0, wrapX != 0, wrapY != 0, true));
    return hal_cuda_adi_get_field(h, field, len);
}

extern "C" int hal_cuda_adi_run_ticks_host(hal_cuda_adi *h, float *field, const float *src, int64_t len,
                                           int32_t ticks, double diffRate, double decay, int32_t wrapX,
                                           int32_t wrapY)
{
    HAL_REQUIRE(h != nullptr && field != nullptr, "hal_cuda_adi_run_ticks_host: NULL argument");
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()),
                "hal_cuda_adi_run_ticks_host: field must hold xDim*yDim values");
    HAL_REQUIRE(ticks >= 0, "hal_cuda_adi_run_ticks_host: negative tick count");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    size_t bytes = h->Length() * sizeof(float);
    if (src != nullptr)
    {
        if (h->src.p == nullptr)
        {
            HAL_TRY(h->src.Alloc(h->Length(), "cudaMalloc(src)"));
        }
        HAL_TRY(halcuda::CudaStatus(cudaMemcpyAsync(h->src.p, src, bytes, cudaMemcpyHostToDevice, s),
                                    "cudaMemcpy(src)"));
        h->hasSrc = true;
    }
    else
    {
        h->hasSrc = false;
    }
    HAL_TRY(halcuda::CudaStatus(cudaMemcpyAsync(h->field[h->cur].p, field, bytes, cudaMemcpyHostToDevice, s),
                                "cudaMemcpy(field)"));
    HAL_TRY(h->RunTicks(ticks, diffRate, decay, wrapX != 0, wrapY != 0, false));
    HAL_TRY(halcuda::CudaStatus(cudaMemcpyAsync(field, h->field[h->cur].p, bytes, cudaMemcpyDeviceToHost, s),
                                "cudaMemcpy(field)"));
    return halcuda::CudaStatus(cudaStreamSynchronize(s), "hal_cuda_adi_run_ticks_host");
}

extern "C" int hal_cuda_adi_sync(hal_cuda_adi *h)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_adi_sync: handle is NULL");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return halcuda::CudaStatus(cudaStreamSynchronize(h->stream.Get()), "hal_cuda_adi_sync");
}

extern "C" void *hal_cuda_adi_stream(hal_cuda_adi *h)
{
    return h ? static_cast<void *>(h->stream.Get()) : nullptr;
}

extern "C" int hal_cuda_adi_set_stream(hal_cuda_adi *h, void *stream)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_adi_set_stream: handle is NULL");
    h->stream.Set(stream);
    h->ResetGraphs();
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_adi_profile(hal_cuda_adi *h, int32_t iters, double diffRate, double decay, int32_t wrapX,
                                    int32_t wrapY, float *ms)
{
    HAL_REQUIRE(h != nullptr && ms != nullptr, "hal_cuda_adi_profile: NULL argument");
    HAL_REQUIRE(iters > 0, "hal_cuda_adi_profile: iters must be positive");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    cudaEvent_t ev[3];
    for (auto &e : ev)
    {
        HAL_TRY(CudaStatus(cudaEventCreate(&e), "cudaEventCreate"));
    }
    const float *g = h->hasGhost ? h->ghost.p : nullptr;
    double tCol = 0.0, tRow = 0.0;
    int rc = HAL_CUDA_OK;
    for (int32_t t = 0; t < iters && rc == HAL_CUDA_OK; t++)
    {
        int c = h->cur;
        cudaEventRecord(ev[0], s);
        rc = h->LaunchColumn<float>(h->field[c].p, diffRate, wrapX != 0, wrapY != 0, g, s);
        if (rc != HAL_CUDA_OK)
        {
            break;
        }
        cudaEventRecord(ev[1], s);
        rc = h->LaunchRow<float, halcuda::kRowTick>(h->field[c].p, h->field[c ^ 1].p, nullptr, diffRate, decay,
                                                    wrapX != 0, wrapY != 0, g, true, s);
        if (rc != HAL_CUDA_OK)
        {
            break;
        }
        cudaEventRecord(ev[2], s);
        rc = CudaStatus(cudaEventSynchronize(ev[2]), "hal_cuda_adi_profile");
        float a = 0.0f, b = 0.0f;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[1], ev[2]);
        tCol += a;
        tRow += b;
        h->cur ^= 1;
    }
    for (auto &e : ev)
    {
        cudaEventDestroy(e);
    }
    HAL_TRY(rc);
    ms[0] = static_cast<float>(tCol / iters);
    ms[1] = static_cast<float>(tRow / iters);
    return HAL_CUDA_OK;
}
