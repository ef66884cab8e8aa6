// diffusion.cu -- explicit 5-point diffusion: the fused per-tick kernel, the
// FP64 IDiffusionBackend2D::Diffuse kernel, and the hal_cuda_diffusion handle.
//
// Math (reference src/Pde/PDEequations.cpp:140-161 and PDEequations.h:50-98,
// 264-287): for cell i = x*yDim + y with centre value c,
//   sum = d(x+1) + d(x-1) + d(y+1) + d(y-1),  d(n) = f[n] - c  on the grid,
//         f[wrap(n)] - c on a wrapped axis, (bc - c)*2 for a Dirichlet ghost,
//         0 for a zero-flux edge;
//   deltas[i] += sum * diffRate.
// The fused tick adds PDEGrid2D's MulAll(-decay), Add(source) and Update()
// (PDEGrid2D.h:103-186) in the same pass: f'[i] = c + (sum*r - c*decay + src).
#include "common.cuh"
#include "stencil64.cuh"
#include "tick_params.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

using namespace halcuda::stencil64;

namespace halcuda
{
    namespace
    {

        // Off-grid neighbour handling of one row (or column) of the stencil.
        enum NbrMode : int
        {
            kNbrGrid = 0,   // value on the grid (or wrapped onto it)
            kNbrGhost = 1,  // Dirichlet ghost: (bc - c) * 2
            kNbrNone = 2    // zero-flux: contributes 0
        };

        __device__ __forceinline__ float ModeWeight(int mode)
        {
            return (mode == kNbrGrid) ? 1.0f : ((mode == kNbrGhost) ? 2.0f : 0.0f);
        }


        // Loads VEC consecutive values of row x starting at column y0 (the
        // part inside the grid) and classifies the row as grid/ghost/none.
        template <int VEC>
        __device__ __forceinline__ int LoadRow(const TickParams &p, int32_t x, int32_t y0,
                                               float (&v)[VEC], bool lowSide)
        {
            int mode = kNbrGrid;
            int32_t row = x;
            if (x < 0 || x >= p.xDim)
            {
                if (p.wrapX)
                {
                    row = (x < 0) ? x + p.xDim : x - p.xDim;
                }
                else if (p.ghost.xlo != nullptr)
                {
                    const float *g = lowSide ? p.ghost.xlo : p.ghost.xhi;
#pragma unroll
                    for (int k = 0; k < VEC; k++)
                    {
                        v[k] = (y0 + k < p.yDim) ? __ldg(g + y0 + k) : 0.0f;
                    }
                    return kNbrGhost;
                }
                else
                {
#pragma unroll
                    for (int k = 0; k < VEC; k++)
                    {
                        v[k] = 0.0f;
                    }
                    return kNbrNone;
                }
            }
            const float *src = p.f + static_cast<int64_t>(row) * p.yDim + y0;
            if constexpr (VEC == 4)
            {
                float4 q = __ldg(reinterpret_cast<const float4 *>(src));
                v[0] = q.x;
                v[1] = q.y;
                v[2] = q.z;
                v[3] = q.w;
            }
            else
            {
#pragma unroll
                for (int k = 0; k < VEC; k++)
                {
                    v[k] = (y0 + k < p.yDim) ? __ldg(src + k) : 0.0f;
                }
            }
            return mode;
        }

        // One fused tick.  Each thread owns VEC consecutive cells (float4 when
        // yDim % 4 == 0) of kTickRowsPerThread consecutive rows.  Every load
        // of the thread -- the rows above, inside and below its strip, the
        // y neighbours of each row and the source -- is issued before the
        // first result is computed.
        // CTA (bx, by) of the tick of grid p: columns from bx * 32 * VEC, rows
        // from by * kTickWarps * kTickRowsPerThread.
        // The tick of a thread whose strip and every neighbour of it lie on
        // the grid (rows xs-1 .. xs+T, columns y0-1 .. y0+4): no wrap, ghost
        // or zero-flux cases, so every difference weight is 1.  The
        // arithmetic is the general path's with those weights (x * 1 and
        // fmaf(x, 1, y) round as x and x + y), so results are bit-identical.
        // UPT: the commit also multiplies each cell by upt.negUptake once per
        // agent binned in it (TickUptake).
        template <bool ADV, bool UPT>
        __device__ __forceinline__ void TickInterior(const TickParams &p, const TickUptake &upt, const int32_t bx,
                                                     const int32_t by, const int32_t y0, const int32_t xs)
        {
            constexpr int T = kTickRowsPerThread;
            const int64_t yD = p.yDim;
            float4 rows[T + 2];
#pragma unroll
            for (int j = 0; j < T + 2; j++)
            {
                rows[j] = __ldg(reinterpret_cast<const float4 *>(p.f + (xs - 1 + j) * yD + y0));
            }
            float left[T], right[T];
            float4 srcv[T];
#pragma unroll
            for (int t = 0; t < T; t++)
            {
                const float *rowp = p.f + (xs + t) * yD;
                left[t] = __ldg(rowp + y0 - 1);
                right[t] = __ldg(rowp + y0 + 4);
                srcv[t] = (p.src != nullptr) ? __ldg(reinterpret_cast<const float4 *>(p.src + (xs + t) * yD + y0))
                                             : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            int32_t ptBeg = 0, ptEnd = 0;
            if (p.ptStart != nullptr)
            {
                const int32_t gridX = (p.yDim + 32 * 4 - 1) / (32 * 4);
                const int32_t b = by * gridX + bx;
                ptBeg = __ldg(p.ptStart + b);
                ptEnd = __ldg(p.ptStart + b + 1);
            }
#pragma unroll
            for (int t = 0; t < T; t++)
            {
                const float up[4] = {rows[t].x, rows[t].y, rows[t].z, rows[t].w};
                const float cur[4] = {rows[t + 1].x, rows[t + 1].y, rows[t + 1].z, rows[t + 1].w};
                const float dn[4] = {rows[t + 2].x, rows[t + 2].y, rows[t + 2].z, rows[t + 2].w};
                const float sv[4] = {srcv[t].x, srcv[t].y, srcv[t].z, srcv[t].w};
                float o[4];
#pragma unroll
                for (int k = 0; k < 4; k++)
                {
                    const float c = cur[k];
                    const float yp = (k < 3) ? cur[k + 1] : right[t];
                    const float ym = (k > 0) ? cur[k - 1] : left[t];
                    float d;
                    if constexpr (ADV)
                    {
                        float sum = (dn[k] - c) * p.kDn;
                        sum = fmaf(up[k] - c, p.kUp, sum);
                        sum = fmaf(yp - c, p.kYp, sum);
                        sum = fmaf(ym - c, p.kYm, sum);
                        d = fmaf(c, p.negDecay, sum);
                    }
                    else
                    {
                        float sum = dn[k] - c;
                        sum = (up[k] - c) + sum;
                        sum = (yp - c) + sum;
                        sum = (ym - c) + sum;
                        d = sum * p.r;
                        d = fmaf(c, p.negDecay, d);
                    }
                    o[k] = d + sv[k];
                }
                const int32_t x = xs + t;
                if constexpr (UPT)
                {
                    // agent counts of the four cells: five consecutive offsets
                    const int32_t *oc = upt.cellOffsets + x * yD + y0;
                    const int4 o4 = __ldg(reinterpret_cast<const int4 *>(oc));
                    const int32_t o5 = __ldg(oc + 4);
                    const int32_t nc[4] = {o4.y - o4.x, o4.z - o4.y, o4.w - o4.z, o5 - o4.w};
#pragma unroll
                    for (int k = 0; k < 4; k++)
                    {
                        o[k] = fmaf(cur[k], upt.negUptake * static_cast<float>(nc[k]), o[k]);
                    }
                }
                for (int32_t q = ptBeg; q < ptEnd; q++)
                {
                    if (__ldg(p.ptRow + q) == x)
                    {
                        const int32_t col = __ldg(p.ptCol + q) - y0;
                        const float val = __ldg(p.ptVal + q);
#pragma unroll
                        for (int k = 0; k < 4; k++)
                        {
                            if (col == k)
                            {
                                o[k] += val;
                            }
                        }
                    }
                }
                *reinterpret_cast<float4 *>(p.out + x * yD + y0) =
                    make_float4(cur[0] + o[0], cur[1] + o[1], cur[2] + o[2], cur[3] + o[3]);
            }
        }

        template <int VEC, bool ADV = false, bool UPT = false>
        __device__ __forceinline__ void TickTile(const TickParams &p, const int32_t bx, const int32_t by,
                                                 const TickUptake &upt = TickUptake{nullptr, 0.0f})
        {
            constexpr int T = kTickRowsPerThread;
            const int lane = threadIdx.x;
            const int warp = threadIdx.y;
            const int32_t y0 = (bx * 32 + lane) * VEC;
            const int32_t xs = (by * kTickWarps + warp) * T;
            if (y0 >= p.yDim || xs >= p.xDim)
            {
                return;
            }
            if constexpr (VEC == 4)
            {
                if (xs >= 1 && xs + T < p.xDim && y0 >= 1 && y0 + 4 < p.yDim)
                {
                    TickInterior<ADV, UPT>(p, upt, bx, by, y0, xs);
                    return;
                }
            }
            const int nValid = min(VEC, p.yDim - y0);

            float rows[T + 2][VEC];
            int mode[T + 2];
#pragma unroll
            for (int j = 0; j < T + 2; j++)
            {
                const int32_t x = xs - 1 + j;
                if (x <= p.xDim)  // rows past the strip's last "below" row are unused
                {
                    mode[j] = LoadRow<VEC>(p, x, y0, rows[j], j == 0);
                }
                else
                {
                    mode[j] = kNbrNone;
#pragma unroll
                    for (int k = 0; k < VEC; k++)
                    {
                        rows[j][k] = 0.0f;
                    }
                }
            }
            float left[T], right[T], srcv[T][VEC];
            int leftMode = kNbrGrid, rightMode = kNbrGrid;
            const int32_t yr = y0 + nValid;  // column right of the last owned cell
            if (y0 == 0)
            {
                leftMode = p.wrapY ? kNbrGrid : ((p.ghost.ylo != nullptr) ? kNbrGhost : kNbrNone);
            }
            if (yr >= p.yDim)
            {
                rightMode = p.wrapY ? kNbrGrid : ((p.ghost.yhi != nullptr) ? kNbrGhost : kNbrNone);
            }
#pragma unroll
            for (int t = 0; t < T; t++)
            {
                const int32_t x = xs + t;
                left[t] = 0.0f;
                right[t] = 0.0f;
#pragma unroll
                for (int k = 0; k < VEC; k++)
                {
                    srcv[t][k] = 0.0f;
                }
                if (x < p.xDim)
                {
                    const float *rowp = p.f + static_cast<int64_t>(x) * p.yDim;
                    if (y0 > 0)
                    {
                        left[t] = __ldg(rowp + y0 - 1);
                    }
                    else if (p.wrapY)
                    {
                        left[t] = __ldg(rowp + p.yDim - 1);
                    }
                    else if (p.ghost.ylo != nullptr)
                    {
                        left[t] = __ldg(p.ghost.ylo + x);
                    }
                    if (yr < p.yDim)
                    {
                        right[t] = __ldg(rowp + yr);
                    }
                    else if (p.wrapY)
                    {
                        right[t] = __ldg(rowp);
                    }
                    else if (p.ghost.yhi != nullptr)
                    {
                        right[t] = __ldg(p.ghost.yhi + x);
                    }
                    if (p.src != nullptr)
                    {
                        const float *s = p.src + static_cast<int64_t>(x) * p.yDim + y0;
                        if constexpr (VEC == 4)
                        {
                            float4 q = __ldg(reinterpret_cast<const float4 *>(s));
                            srcv[t][0] = q.x;
                            srcv[t][1] = q.y;
                            srcv[t][2] = q.z;
                            srcv[t][3] = q.w;
                        }
                        else
                        {
#pragma unroll
                            for (int k = 0; k < VEC; k++)
                            {
                                srcv[t][k] = (k < nValid) ? __ldg(s + k) : 0.0f;
                            }
                        }
                    }
                }
            }

            const float wLeft = ModeWeight(leftMode);
            const float wRight = ModeWeight(rightMode);
            int32_t ptBeg = 0, ptEnd = 0;
            if (p.ptStart != nullptr)
            {
                const int32_t gridX = (p.yDim + 32 * VEC - 1) / (32 * VEC);
                int32_t b = by * gridX + bx;
                ptBeg = __ldg(p.ptStart + b);
                ptEnd = __ldg(p.ptStart + b + 1);
            }

#pragma unroll
            for (int t = 0; t < T; t++)
            {
                const int32_t x = xs + t;
                if (x >= p.xDim)
                {
                    break;
                }
                const float *up = rows[t];
                const float *cur = rows[t + 1];
                const float *dn = rows[t + 2];
                // difference weights: 1 on the grid, 2 for a Dirichlet ghost
                // ((bc - c) * 2), 0 past a zero-flux edge
                const float wUp = ModeWeight(mode[t]);
                const float wDn = ModeWeight(mode[t + 2]);
                float o[VEC];
#pragma unroll
                for (int k = 0; k < VEC; k++)
                {
                    const float c = cur[k];
                    const float yp = (k + 1 < nValid) ? cur[k + 1] : right[t];
                    const float wYp = (k + 1 < nValid) ? 1.0f : wRight;
                    const float ym = (k > 0) ? cur[k - 1] : left[t];
                    const float wYm = (k > 0) ? 1.0f : wLeft;
                    float d;
                    if constexpr (ADV)
                    {
                        // diffusion plus upwind advection: one weight per side
                        float sum = (dn[k] - c) * (wDn * p.kDn);
                        sum = fmaf(up[k] - c, wUp * p.kUp, sum);
                        sum = fmaf(yp - c, wYp * p.kYp, sum);
                        sum = fmaf(ym - c, wYm * p.kYm, sum);
                        d = fmaf(c, p.negDecay, sum);
                    }
                    else
                    {
                        // reference order: x+1, x-1, y+1, y-1
                        float sum = (dn[k] - c) * wDn;
                        sum = fmaf(up[k] - c, wUp, sum);
                        sum = fmaf(yp - c, wYp, sum);
                        sum = fmaf(ym - c, wYm, sum);
                        d = sum * p.r;
                        d = fmaf(c, p.negDecay, d);
                    }
                    o[k] = d + srcv[t][k];
                }
                if constexpr (UPT)
                {
                    const int32_t *oc = upt.cellOffsets + static_cast<int64_t>(x) * p.yDim + y0;
#pragma unroll
                    for (int k = 0; k < VEC; k++)
                    {
                        if (k < nValid)
                        {
                            const int32_t nc = __ldg(oc + k + 1) - __ldg(oc + k);
                            o[k] = fmaf(cur[k], upt.negUptake * static_cast<float>(nc), o[k]);
                        }
                    }
                }
                for (int32_t q = ptBeg; q < ptEnd; q++)
                {
                    if (__ldg(p.ptRow + q) == x)
                    {
                        int32_t col = __ldg(p.ptCol + q) - y0;
                        float val = __ldg(p.ptVal + q);
#pragma unroll
                        for (int k = 0; k < VEC; k++)
                        {
                            if (col == k)
                            {
                                o[k] += val;
                            }
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < VEC; k++)
                {
                    o[k] = cur[k] + o[k];
                }
                float *dst = p.out + static_cast<int64_t>(x) * p.yDim + y0;
                if constexpr (VEC == 4)
                {
                    *reinterpret_cast<float4 *>(dst) = make_float4(o[0], o[1], o[2], o[3]);
                }
                else
                {
#pragma unroll
                    for (int k = 0; k < VEC; k++)
                    {
                        if (k < nValid)
                        {
                            dst[k] = o[k];
                        }
                    }
                }
            }
        }

        // Four CTAs per SM (64 registers) measured fastest for the plain tick
        // (6.68 vs 6.78 us at 2048^2); the advective tick is fastest unbounded.
        template <int VEC, bool ADV>
        __global__ void __launch_bounds__(32 * kTickWarps, ADV ? 1 : 4)
            TickKernel(TickParams p)
        {
            // Programmatic dependent launch (LaunchTick): the next tick's grid
            // may be scheduled as soon as every CTA of this one has started,
            // so its launch overlaps this tick's last wave; each tick waits
            // for the previous one to complete before it reads or writes a
            // field (a no-op when launched without the attribute).
            asm volatile("griddepcontrol.launch_dependents;");
            asm volatile("griddepcontrol.wait;" ::: "memory");
            TickTile<VEC, ADV>(p, static_cast<int32_t>(blockIdx.x), static_cast<int32_t>(blockIdx.y));
        }

        // The tick with the agents' uptake term (hal_cuda_diffusion_set_uptake).
        template <int VEC, bool ADV>
        __global__ void __launch_bounds__(32 * kTickWarps, ADV ? 1 : 4)
            TickKernelUptake(TickParams p, TickUptake up)
        {
            asm volatile("griddepcontrol.launch_dependents;");
            asm volatile("griddepcontrol.wait;" ::: "memory");
            TickTile<VEC, ADV, true>(p, static_cast<int32_t>(blockIdx.x), static_cast<int32_t>(blockIdx.y), up);
        }

        // Batched form: CTA b runs tile tiles[b] = (grid, CTA column, CTA row).
        template <int VEC>
        __global__ void __launch_bounds__(32 * kTickWarps)
            TickTiles(const TickParams *__restrict__ table, const int4 *__restrict__ tiles)
        {
            const int4 t = tiles[blockIdx.x];
            TickTile<VEC>(table[t.x], t.y, t.z);
        }
    }

    namespace
    {
        // S[cell] += value for every point source, in list order by one
        // thread, so sums over repeated cells are deterministic.
        __global__ void AddPointsSerial(float *__restrict__ S, const int32_t *__restrict__ row,
                                        const int32_t *__restrict__ col, const float *__restrict__ val, int32_t n,
                                        int32_t yDim)
        {
            if (threadIdx.x == 0 && blockIdx.x == 0)
            {
                for (int32_t k = 0; k < n; k++)
                {
                    S[static_cast<int64_t>(row[k]) * yDim + col[k]] += val[k];
                }
            }
        }
    }

    int LaunchTickTiles(const TickParams *table, const int4 *tiles, int32_t nTiles, int vec, cudaStream_t s)
    {
        if (nTiles <= 0)
        {
            return HAL_CUDA_OK;
        }
        const dim3 block(32, kTickWarps);
        if (vec == 4)
        {
            TickTiles<4><<<static_cast<unsigned>(nTiles), block, 0, s>>>(table, tiles);
        }
        else
        {
            TickTiles<1><<<static_cast<unsigned>(nTiles), block, 0, s>>>(table, tiles);
        }
        CountLaunch();
        return LaunchStatus("TickTiles");
    }

    struct Diffusion
    {
        int32_t xDim = 0, yDim = 0;
        int device = 0;
        StreamSlot stream;
        DevBuf<float> field[2];
        int cur = 0;
        DevBuf<float> src;
        bool hasSrc = false;
        DevBuf<float> ghost;
        bool hasGhost = false;
        DevBuf<int32_t> ptStart, ptRow, ptCol;
        DevBuf<float> ptVal;
        bool hasPoints = false;
        double xVel = 0.0, yVel = 0.0;  // uniform advection of every tick (PDEGrid2D::Advection)
        // agent uptake coupling (hal_cuda_diffusion_set_uptake): the agent
        // handle whose last binning gives each cell's agent count
        const hal_cuda_agents *agents = nullptr;
        double uptake = 0.0;
        int32_t nPoints = 0;
        // Temporal blocking: ticks per launch 1 or 2 (0 = automatic, which
        // is 1).  The two-tick kernel stages tiles with a tensor map per field
        // buffer and reads the dense source and the point sources summed into
        // one array.  Measured on GB300 it is slower at every size (2048^2:
        // 12.0 vs 7.1 us per tick; 8192^2: 165 vs 94 us, where one tick per
        // launch already streams at 84% of HBM peak), so it is opt-in.
        int32_t blockMode = 0;
        TickBlockTensorMap tmap[2];
        bool tmapOk = false;
        DevBuf<float> combS;
        bool combDirty = true;
        DevBuf<int32_t> blockErr;
        bool stopped = false;  // a two-tick launch gave up waiting: no further ticks
        // failure-detection test hook (hal_cuda_diffusion_test_stall)
        uint32_t testExtraTx = 0, testWaitUs = 0;

        DevBuf<double> f64, d64, g64;
        DevBuf<double> a64, b64;  // per-cell rates or velocities of the FP64 stencil calls
        DevBuf<double> gv64;      // x- and y-velocity ghost tables of the Dirichlet advection form
        GraphCache graph[2];  // by the parity of the starting buffer
        dim3 grid, block;

        void ResetGraphs()
        {
            graph[0].Reset();
            graph[1].Reset();
        }
        bool vec4 = false;

        int Init(int32_t x, int32_t y)
        {
            xDim = x;
            yDim = y;
            device = CurrentDevice();
            HAL_TRY(CudaStatus(cudaSetDevice(device), "cudaSetDevice"));
            HAL_TRY(stream.Create("cudaStreamCreate"));
            size_t n = static_cast<size_t>(x) * static_cast<size_t>(y);
            HAL_TRY(field[0].Alloc(n, "cudaMalloc(field)"));
            HAL_TRY(field[1].Alloc(n, "cudaMalloc(field)"));
            HAL_TRY(CudaStatus(cudaMemset(field[0].p, 0, n * sizeof(float)), "cudaMemset"));
            vec4 = (yDim % 4) == 0;
            int vec = vec4 ? 4 : 1;
            block = dim3(32, kTickWarps);
            grid = dim3((yDim + 32 * vec - 1) / (32 * vec),
                        (xDim + kTickWarps * kTickRowsPerThread - 1) / (kTickWarps * kTickRowsPerThread));
            tmapOk = vec4 && MakeTickBlockTensorMap(tmap[0], field[0].p, xDim, yDim) &&
                     MakeTickBlockTensorMap(tmap[1], field[1].p, xDim, yDim);
            if (tmapOk)
            {
                HAL_TRY(PrepareTickBlocked());
                HAL_TRY(blockErr.Alloc(1, "cudaMalloc(err)"));
                HAL_TRY(CudaStatus(cudaMemset(blockErr.p, 0, sizeof(int32_t)), "cudaMemset"));
            }
            return HAL_CUDA_OK;
        }

        // (the two-tick kernel has no uptake term: coupled ticks run one per
        // launch)
        bool UseBlocked(int32_t ticks) const
        {
            return tmapOk && ticks >= 2 && blockMode == 2 && agents == nullptr;
        }

        // The dense source plus the point sources as one array (null if
        // neither is set or extras are off), rebuilt after either changes.
        int CombinedSource(bool useExtras, const float **out, cudaStream_t s)
        {
            *out = nullptr;
            if (!useExtras || (!hasSrc && !hasPoints))
            {
                return HAL_CUDA_OK;
            }
            if (combDirty)
            {
                if (combS.p == nullptr)
                {
                    HAL_TRY(combS.Alloc(Length(), "cudaMalloc(combined source)"));
                }
                const size_t bytes = Length() * sizeof(float);
                HAL_TRY(CudaStatus(hasSrc ? cudaMemcpyAsync(combS.p, src.p, bytes, cudaMemcpyDeviceToDevice, s)
                                          : cudaMemsetAsync(combS.p, 0, bytes, s),
                                   "combined source"));
                if (hasPoints)
                {
                    AddPointsSerial<<<1, 32, 0, s>>>(combS.p, ptRow.p, ptCol.p, ptVal.p, nPoints, yDim);
                    CountLaunch();
                    HAL_TRY(LaunchStatus("combined source"));
                }
                combDirty = false;
            }
            *out = combS.p;
            return HAL_CUDA_OK;
        }

        TickBlockParams BlockParams(const TickParams &t, const float *S) const
        {
            TickBlockParams b;
            b.f = t.f;
            b.out = t.out;
            b.xDim = t.xDim;
            b.yDim = t.yDim;
            b.r = t.r;
            b.negDecay = t.negDecay;
            b.wrapX = t.wrapX;
            b.wrapY = t.wrapY;
            b.S = S;
            b.ghost = t.ghost;
            b.kUp = t.kUp;
            b.kDn = t.kDn;
            b.kYm = t.kYm;
            b.kYp = t.kYp;
            b.adv = (t.kUp != t.r || t.kDn != t.r || t.kYm != t.r || t.kYp != t.r) ? 1 : 0;
            b.err = blockErr.p;
            b.extraTx = testExtraTx;
            b.waitLimitUs = testWaitUs;
            return b;
        }

        size_t Length() const
        {
            return static_cast<size_t>(xDim) * static_cast<size_t>(yDim);
        }

        TickParams Params(const float *in, float *out, double r, double decay, bool wrapX,
                          bool wrapY, bool useExtras) const
        {
            TickParams p;
            p.f = in;
            p.out = out;
            p.xDim = xDim;
            p.yDim = yDim;
            p.r = static_cast<float>(r);
            p.negDecay = static_cast<float>(-decay);
            p.wrapX = wrapX;
            p.wrapY = wrapY;
            p.src = (useExtras && hasSrc) ? src.p : nullptr;
            p.ghost = MakeGhostView((useExtras && hasGhost) ? ghost.p : nullptr, xDim, yDim);
            bool pts = useExtras && hasPoints;
            p.ptStart = pts ? ptStart.p : nullptr;
            p.ptRow = pts ? ptRow.p : nullptr;
            p.ptCol = pts ? ptCol.p : nullptr;
            p.ptVal = pts ? ptVal.p : nullptr;
            const double vx = useExtras ? xVel : 0.0, vy = useExtras ? yVel : 0.0;
            p.kUp = static_cast<float>(r + std::max(vx, 0.0));
            p.kDn = static_cast<float>(r + std::max(-vx, 0.0));
            p.kYm = static_cast<float>(r + std::max(vy, 0.0));
            p.kYp = static_cast<float>(r + std::max(-vy, 0.0));
            return p;
        }

        // The uptake of a tick with extras (cellOffsets null: none).
        TickUptake Uptake(bool useExtras) const
        {
            TickUptake u{nullptr, 0.0f};
            if (useExtras && agents != nullptr)
            {
                int32_t ax = 0, ay = 0;
                u.cellOffsets = AgentsCellOffsets(agents, &ax, &ay);
                u.negUptake = static_cast<float>(-uptake);
            }
            return u;
        }

        // One tick, launched with programmatic stream serialization (the
        // kernel's griddepcontrol.wait keeps the ticks ordered): 6.55 against
        // 6.70 us per 2048^2 tick in a graph, bit-identical fields.
        void LaunchTick(const TickParams &p, const TickUptake &up, cudaStream_t s) const
        {
            const bool adv = p.kUp != p.r || p.kDn != p.r || p.kYm != p.r || p.kYp != p.r;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = grid;
            cfg.blockDim = block;
            cfg.dynamicSmemBytes = 0;
            cfg.stream = s;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            at[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            if (up.cellOffsets != nullptr)
            {
                if (vec4)
                {
                    cudaLaunchKernelEx(&cfg, adv ? TickKernelUptake<4, true> : TickKernelUptake<4, false>, p, up);
                }
                else
                {
                    cudaLaunchKernelEx(&cfg, adv ? TickKernelUptake<1, true> : TickKernelUptake<1, false>, p, up);
                }
            }
            else if (vec4)
            {
                if (adv)
                {
                    cudaLaunchKernelEx(&cfg, TickKernel<4, true>, p);
                }
                else
                {
                    cudaLaunchKernelEx(&cfg, TickKernel<4, false>, p);
                }
            }
            else if (adv)
            {
                cudaLaunchKernelEx(&cfg, TickKernel<1, true>, p);
            }
            else
            {
                cudaLaunchKernelEx(&cfg, TickKernel<1, false>, p);
            }
        }

        // Enqueues `ticks` ticks from field[cur], replayed from a graph.
        int RunTicks(int32_t ticks, double r, double decay, bool wrapX, bool wrapY, bool extras)
        {
            if (stopped)
            {
                SetError("hal_cuda_diffusion_run_ticks: the handle stopped after a two-tick launch gave up waiting "
                         "for its tile; the field is undefined: destroy the handle and create a new one");
                return HAL_CUDA_ETIMEOUT;
            }
            if (ticks <= 0)
            {
                return HAL_CUDA_OK;
            }
            cudaStream_t s = stream.Get();
            const bool blocked = UseBlocked(ticks);
            const float *S = nullptr;
            if (blocked)
            {
                HAL_TRY(CombinedSource(extras, &S, s));
            }
            // launches: two ticks each when blocked (plus one single tick
            // for an odd count); each launch flips the buffers
            const int32_t launches = blocked ? ticks / 2 + (ticks & 1) : ticks;
            char key[256];
            snprintf(key, sizeof(key), "%d|%a|%a|%d|%d|%d|%d|%d|%d|%a|%a|%d|%p|%p|%a|%u|%u", ticks, r, decay, wrapX,
                     wrapY, extras ? 1 : 0, hasSrc, hasPoints, hasGhost, xVel, yVel, blocked ? 1 : 0,
                     static_cast<void *>(s), static_cast<const void *>(agents), uptake, testExtraTx, testWaitUs);
            GraphCache &graph = this->graph[cur];
            if (graph.exec == nullptr || graph.key != key)
            {
                graph.Reset();
                cudaGraph_t g = nullptr;
                HAL_TRY(CudaStatus(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                                   "cudaStreamBeginCapture"));
                int c = cur;
                int32_t t = 0;
                if (blocked)
                {
                    for (; t + 1 < ticks; t += 2)
                    {
                        const TickParams p = Params(field[c].p, field[c ^ 1].p, r, decay, wrapX, wrapY, extras);
                        LaunchTickBlocked2(BlockParams(p, S), tmap[c], s);
                        c ^= 1;
                    }
                }
                for (; t < ticks; t++)
                {
                    TickParams p = Params(field[c].p, field[c ^ 1].p, r, decay, wrapX, wrapY, extras);
                    LaunchTick(p, Uptake(extras), s);
                    c ^= 1;
                }
                cudaError_t e = cudaStreamEndCapture(s, &g);
                HAL_TRY(CudaStatus(e, "cudaStreamEndCapture"));
                e = cudaGraphInstantiate(&graph.exec, g, 0);
                cudaGraphDestroy(g);
                HAL_TRY(CudaStatus(e, "cudaGraphInstantiate"));
                graph.key = key;
            }
            HAL_TRY(CudaStatus(cudaGraphLaunch(graph.exec, s), "cudaGraphLaunch"));
            CountLaunch(launches);
            cur ^= (launches & 1);
            return HAL_CUDA_OK;
        }
    };
}

using halcuda::Diffusion;

struct hal_cuda_diffusion : public Diffusion
{
};

void halcuda::DiffusionDims(const hal_cuda_diffusion *h, int32_t *xDim, int32_t *yDim)
{
    *xDim = h->xDim;
    *yDim = h->yDim;
}

extern "C" int hal_cuda_diffusion_create(int32_t xDim, int32_t yDim, hal_cuda_diffusion **out)
{
    HAL_REQUIRE(out != nullptr, "hal_cuda_diffusion_create: out is NULL");
    *out = nullptr;
    HAL_REQUIRE(xDim > 0 && yDim > 0, "hal_cuda_diffusion_create: dimensions must be positive");
    HAL_REQUIRE(static_cast<int64_t>(xDim) * yDim < (int64_t(1) << 31),
                "hal_cuda_diffusion_create: xDim*yDim exceeds int32");
    hal_cuda_diffusion *h = new (std::nothrow) hal_cuda_diffusion();
    if (h == nullptr)
    {
        halcuda::SetError("hal_cuda_diffusion_create: out of host memory");
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

extern "C" int hal_cuda_diffusion_destroy(hal_cuda_diffusion *h)
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
    int DiffuseCommon(hal_cuda_diffusion *h, const double *field, double *deltas, double r,
                      int32_t wrapX, int32_t wrapY, const double *ghost, const char *who)
    {
        using namespace halcuda;
        HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
        size_t n = h->Length();
        size_t ng = ghost ? 2 * (static_cast<size_t>(h->xDim) + h->yDim) : 0;
        if (h->f64.p == nullptr)
        {
            HAL_TRY(h->f64.Alloc(n, "cudaMalloc(f64)"));
            HAL_TRY(h->d64.Alloc(n, "cudaMalloc(d64)"));
            HAL_TRY(h->g64.Alloc(2 * (static_cast<size_t>(h->xDim) + h->yDim), "cudaMalloc(g64)"));
        }
        cudaStream_t s = h->stream.Get();
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->f64.p, field, n * sizeof(double), cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(field)"));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->d64.p, deltas, n * sizeof(double), cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(deltas)"));
        if (ghost)
        {
            HAL_TRY(CudaStatus(cudaMemcpyAsync(h->g64.p, ghost, ng * sizeof(double), cudaMemcpyHostToDevice, s),
                               "cudaMemcpy(ghost)"));
        }
        const Diffuse64Cell cell{h->f64.p, h->d64.p, ghost ? h->g64.p : nullptr, r, h->xDim, h->yDim, wrapX, wrapY};
        Cells64Kernel<<<Cells64Grid(h->xDim, h->yDim), 256, 0, s>>>(cell, h->xDim, h->yDim);
        CountLaunch();
        HAL_TRY(LaunchStatus(who));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(deltas, h->d64.p, n * sizeof(double), cudaMemcpyDeviceToHost, s),
                           "cudaMemcpy(deltas)"));
        return CudaStatus(cudaStreamSynchronize(s), who);
    }
}

namespace
{
    enum Stencil64 : int
    {
        kVarDiffusion = HAL_CUDA_STENCIL_DIFFUSE_VAR,
        kAdvection = HAL_CUDA_STENCIL_ADVECT,
        kVarAdvection = HAL_CUDA_STENCIL_ADVECT_VAR
    };

    // ghost / ghostVx / ghostVy: device ghost tables of the Dirichlet forms
    // (field; x and y velocities), or nullptr for the zero-flux forms.
    void LaunchStencil64(hal_cuda_diffusion *h, int kind, double xVel, double yVel, int32_t wrapX, int32_t wrapY,
                         const double *ghost, const double *ghostVx, const double *ghostVy, cudaStream_t s)
    {
        using namespace halcuda;
        const dim3 grid = Cells64Grid(h->xDim, h->yDim);
        if (kind == kVarDiffusion)
        {
            const DiffuseVar64Cell cell{h->f64.p, h->d64.p, h->a64.p, h->b64.p, h->xDim, h->yDim, wrapX, wrapY};
            Cells64Kernel<<<grid, 256, 0, s>>>(cell, h->xDim, h->yDim);
        }
        else if (kind == kAdvection)
        {
            const int32_t xSign = xVel > 0 ? 1 : (xVel < 0 ? -1 : 0);
            const int32_t ySign = yVel > 0 ? 1 : (yVel < 0 ? -1 : 0);
            const Advect64Cell cell{h->f64.p, h->d64.p, ghost, xVel, yVel, h->xDim, h->yDim, wrapX, wrapY, xSign, ySign};
            Cells64Kernel<<<grid, 256, 0, s>>>(cell, h->xDim, h->yDim);
        }
        else
        {
            const AdvectVar64Cell cell{h->f64.p, h->d64.p, h->a64.p, h->b64.p, ghost, ghostVx, ghostVy,
                                       h->xDim,  h->yDim,  wrapX,    wrapY};
            Cells64Kernel<<<grid, 256, 0, s>>>(cell, h->xDim, h->yDim);
        }
    }

    // Upload field, deltas and (for the per-cell forms) two per-cell arrays,
    // run one FP64 stencil, download deltas.
    int Stencil64Common(hal_cuda_diffusion *h, int kind, const double *field, double *deltas, const double *a,
                        const double *b, double xVel, double yVel, int32_t wrapX, int32_t wrapY, const double *ghost,
                        const double *ghostVx, const double *ghostVy, const char *who)
    {
        using namespace halcuda;
        HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
        const size_t n = h->Length();
        if (h->f64.p == nullptr)
        {
            HAL_TRY(h->f64.Alloc(n, "cudaMalloc(f64)"));
            HAL_TRY(h->d64.Alloc(n, "cudaMalloc(d64)"));
            HAL_TRY(h->g64.Alloc(2 * (static_cast<size_t>(h->xDim) + h->yDim), "cudaMalloc(g64)"));
        }
        if (kind != kAdvection && h->b64.p == nullptr)
        {
            HAL_TRY(h->a64.Alloc(n, "cudaMalloc(a64)"));
            HAL_TRY(h->b64.Alloc(n, "cudaMalloc(b64)"));
        }
        const size_t ng = 2 * (static_cast<size_t>(h->xDim) + h->yDim);
        if ((ghostVx != nullptr || ghostVy != nullptr) && h->gv64.p == nullptr)
        {
            HAL_TRY(h->gv64.Alloc(2 * ng, "cudaMalloc(gv64)"));
        }
        cudaStream_t s = h->stream.Get();
        const size_t bytes = n * sizeof(double);
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->f64.p, field, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpy(field)"));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->d64.p, deltas, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpy(deltas)"));
        if (kind != kAdvection)
        {
            HAL_TRY(CudaStatus(cudaMemcpyAsync(h->a64.p, a, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpy(x array)"));
            HAL_TRY(CudaStatus(cudaMemcpyAsync(h->b64.p, b, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpy(y array)"));
        }
        const double *dGhost = nullptr, *dGhostVx = nullptr, *dGhostVy = nullptr;
        if (ghost != nullptr)
        {
            HAL_TRY(CudaStatus(cudaMemcpyAsync(h->g64.p, ghost, ng * sizeof(double), cudaMemcpyHostToDevice, s),
                               "cudaMemcpy(ghost)"));
            dGhost = h->g64.p;
        }
        if (ghostVx != nullptr)
        {
            HAL_TRY(CudaStatus(cudaMemcpyAsync(h->gv64.p, ghostVx, ng * sizeof(double), cudaMemcpyHostToDevice, s),
                               "cudaMemcpy(ghostVx)"));
            dGhostVx = h->gv64.p;
        }
        if (ghostVy != nullptr)
        {
            HAL_TRY(CudaStatus(
                cudaMemcpyAsync(h->gv64.p + ng, ghostVy, ng * sizeof(double), cudaMemcpyHostToDevice, s),
                "cudaMemcpy(ghostVy)"));
            dGhostVy = h->gv64.p + ng;
        }
        LaunchStencil64(h, kind, xVel, yVel, wrapX, wrapY, dGhost, dGhostVx, dGhostVy, s);
        CountLaunch();
        HAL_TRY(LaunchStatus(who));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(deltas, h->d64.p, bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpy(deltas)"));
        return CudaStatus(cudaStreamSynchronize(s), who);
    }
}

extern "C" int hal_cuda_diffuse_var(hal_cuda_diffusion *h, const double *field, double *deltas,
                                    const double *ratesX, const double *ratesY, int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && field != nullptr && deltas != nullptr && ratesX != nullptr && ratesY != nullptr,
                "hal_cuda_diffuse_var: NULL argument");
    return Stencil64Common(h, kVarDiffusion, field, deltas, ratesX, ratesY, 0.0, 0.0, wrapX, wrapY, nullptr, nullptr,
                           nullptr, "hal_cuda_diffuse_var");
}

extern "C" int hal_cuda_advect(hal_cuda_diffusion *h, const double *field, double *deltas, double xVel, double yVel,
                               int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && field != nullptr && deltas != nullptr, "hal_cuda_advect: NULL argument");
    return Stencil64Common(h, kAdvection, field, deltas, nullptr, nullptr, xVel, yVel, wrapX, wrapY, nullptr, nullptr,
                           nullptr, "hal_cuda_advect");
}

extern "C" int hal_cuda_advect_bc(hal_cuda_diffusion *h, const double *field, double *deltas, double xVel,
                                  double yVel, int32_t wrapX, int32_t wrapY, const double *ghost)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && field != nullptr && deltas != nullptr, "hal_cuda_advect_bc: NULL argument");
    return Stencil64Common(h, kAdvection, field, deltas, nullptr, nullptr, xVel, yVel, wrapX, wrapY, ghost, nullptr,
                           nullptr, "hal_cuda_advect_bc");
}

extern "C" int hal_cuda_advect_var(hal_cuda_diffusion *h, const double *field, double *deltas, const double *xVels,
                                   const double *yVels, int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && field != nullptr && deltas != nullptr && xVels != nullptr && yVels != nullptr,
                "hal_cuda_advect_var: NULL argument");
    return Stencil64Common(h, kVarAdvection, field, deltas, xVels, yVels, 0.0, 0.0, wrapX, wrapY, nullptr, nullptr,
                           nullptr, "hal_cuda_advect_var");
}

extern "C" int hal_cuda_advect_var_bc(hal_cuda_diffusion *h, const double *field, double *deltas,
                                      const double *xVels, const double *yVels, int32_t wrapX, int32_t wrapY,
                                      const double *ghost, const double *ghostXVel, const double *ghostYVel)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && field != nullptr && deltas != nullptr && xVels != nullptr && yVels != nullptr,
                "hal_cuda_advect_var_bc: NULL argument");
    return Stencil64Common(h, kVarAdvection, field, deltas, xVels, yVels, 0.0, 0.0, wrapX, wrapY, ghost, ghostXVel,
                           ghostYVel, "hal_cuda_advect_var_bc");
}

extern "C" int hal_cuda_stencil64_profile(hal_cuda_diffusion *h, int32_t kind, int32_t iters, double xVel,
                                          double yVel, int32_t wrapX, int32_t wrapY, float *ms)
{
    HAL_REQUIRE(h != nullptr && ms != nullptr, "hal_cuda_stencil64_profile: NULL argument");
    HAL_REQUIRE(iters > 0, "hal_cuda_stencil64_profile: iters must be positive");
    HAL_REQUIRE(kind == kVarDiffusion || kind == kAdvection || kind == kVarAdvection,
                "hal_cuda_stencil64_profile: unknown stencil kind");
    HAL_REQUIRE(h->f64.p != nullptr && (kind == kAdvection || h->b64.p != nullptr),
                "hal_cuda_stencil64_profile: no arrays uploaded by a call of this kind");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    cudaEvent_t e0, e1;
    HAL_TRY(CudaStatus(cudaEventCreate(&e0), "cudaEventCreate"));
    HAL_TRY(CudaStatus(cudaEventCreate(&e1), "cudaEventCreate"));
    double total = 0.0;
    int rc = HAL_CUDA_OK;
    for (int32_t t = 0; t < iters && rc == HAL_CUDA_OK; t++)
    {
        cudaEventRecord(e0, s);
        LaunchStencil64(h, kind, xVel, yVel, wrapX, wrapY, nullptr, nullptr, nullptr, s);
        CountLaunch();
        cudaEventRecord(e1, s);
        rc = LaunchStatus("hal_cuda_stencil64_profile");
        if (rc == HAL_CUDA_OK)
        {
            rc = CudaStatus(cudaEventSynchronize(e1), "hal_cuda_stencil64_profile");
        }
        float a = 0.0f;
        if (rc == HAL_CUDA_OK)
        {
            cudaEventElapsedTime(&a, e0, e1);
        }
        total += a;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    HAL_TRY(rc);
    *ms = static_cast<float>(total / iters);
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_diffuse(hal_cuda_diffusion *h, const double *field, int64_t fieldLen,
                                double *deltas, int64_t deltasLen, double diffRate, int32_t xDim,
                                int32_t yDim, int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffuse: handle is NULL");
    int64_t length = static_cast<int64_t>(xDim) * yDim;
    HAL_REQUIRE(xDim > 0 && yDim > 0 && fieldLen == length && deltasLen == length,
                "CudaDiffusionBackend2D::Diffuse: field and deltas must each hold xDim*yDim values");
    HAL_REQUIRE(xDim == h->xDim && yDim == h->yDim,
                "CudaDiffusionBackend2D::Diffuse called with dimensions differing from construction");
    HAL_REQUIRE(field != nullptr && deltas != nullptr, "hal_cuda_diffuse: NULL array");
    return DiffuseCommon(h, field, deltas, diffRate, wrapX, wrapY, nullptr, "hal_cuda_diffuse");
}

extern "C" int hal_cuda_diffuse_bc(hal_cuda_diffusion *h, const double *field, double *deltas,
                                   double diffRate, int32_t wrapX, int32_t wrapY, const double *ghost)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && field != nullptr && deltas != nullptr, "hal_cuda_diffuse_bc: NULL argument");
    return DiffuseCommon(h, field, deltas, diffRate, wrapX, wrapY, ghost, "hal_cuda_diffuse_bc");
}

extern "C" int hal_cuda_diffusion_set_field(hal_cuda_diffusion *h, const float *field, int64_t len)
{
    HAL_REQUIRE(h != nullptr && field != nullptr, "hal_cuda_diffusion_set_field: NULL argument");
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()),
                "hal_cuda_diffusion_set_field: field must hold xDim*yDim values");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    HAL_TRY(halcuda::CudaStatus(cudaMemcpyAsync(h->field[h->cur].p, field, h->Length() * sizeof(float),
                                                cudaMemcpyHostToDevice, s),
                                "cudaMemcpy(field)"));
    return halcuda::CudaStatus(cudaStreamSynchronize(s), "hal_cuda_diffusion_set_field");
}

extern "C" int hal_cuda_diffusion_get_field(hal_cuda_diffusion *h, float *field, int64_t len)
{
    HAL_REQUIRE(h != nullptr && field != nullptr, "hal_cuda_diffusion_get_field: NULL argument");
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()),
                "hal_cuda_diffusion_get_field: field must hold xDim*yDim values");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    HAL_TRY(halcuda::CudaStatus(cudaMemcpyAsync(field, h->field[h->cur].p, h->Length() * sizeof(float),
                                                cudaMemcpyDeviceToHost, s),
                                "cudaMemcpy(field)"));
    HAL_TRY(halcuda::CudaStatus(cudaStreamSynchronize(s), "hal_cuda_diffusion_get_field"));
    if (h->blockErr.p != nullptr)
    {
        int32_t err = 0;
        HAL_TRY(halcuda::CudaStatus(cudaMemcpy(&err, h->blockErr.p, sizeof(err), cudaMemcpyDeviceToHost),
                                    "cudaMemcpy(err)"));
        if (err != 0)
        {
            // the field is undefined from here on, and every later tick of
            // this handle is refused
            h->stopped = true;
            halcuda::SetError("hal_cuda_diffusion_get_field: a two-tick launch gave up waiting for its tile");
            return HAL_CUDA_ETIMEOUT;
        }
    }
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_diffusion_set_source(hal_cuda_diffusion *h, const float *dense, int64_t len)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffusion_set_source: handle is NULL");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    if (dense == nullptr)
    {
        h->hasSrc = false;
        h->combDirty = true;
        h->ResetGraphs();
        return HAL_CUDA_OK;
    }
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()),
                "hal_cuda_diffusion_set_source: source must hold xDim*yDim values");
    if (h->src.p == nullptr)
    {
        HAL_TRY(h->src.Alloc(h->Length(), "cudaMalloc(src)"));
    }
    HAL_TRY(halcuda::CudaStatus(cudaMemcpy(h->src.p, dense, h->Length() * sizeof(float), cudaMemcpyHostToDevice),
                                "cudaMemcpy(src)"));
    h->hasSrc = true;
    h->combDirty = true;
    h->ResetGraphs();
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_diffusion_set_point_sources(hal_cuda_diffusion *h, int32_t nPoints,
                                                    const int32_t *cells, const float *values)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffusion_set_point_sources: handle is NULL");
    HAL_REQUIRE(nPoints >= 0, "hal_cuda_diffusion_set_point_sources: negative count");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    h->ResetGraphs();
    h->combDirty = true;
    if (nPoints == 0)
    {
        h->hasPoints = false;
        h->nPoints = 0;
        return HAL_CUDA_OK;
    }
    HAL_REQUIRE(cells != nullptr && values != nullptr, "hal_cuda_diffusion_set_point_sources: NULL array");
    int64_t n = static_cast<int64_t>(h->Length());
    // Group the points by the CTA of the tick kernel that owns their cell.
    int vec = h->vec4 ? 4 : 1;
    int32_t gx = static_cast<int32_t>(h->grid.x);
    int32_t nBlocks = gx * static_cast<int32_t>(h->grid.y);
    std::vector<int32_t> blockOf(nPoints), start(nBlocks + 1, 0);
    for (int32_t k = 0; k < nPoints; k++)
    {
        HAL_REQUIRE(cells[k] >= 0 && cells[k] < n, "hal_cuda_diffusion_set_point_sources: cell %d out of range",
                    cells[k]);
        int32_t x = cells[k] / h->yDim;
        int32_t y = cells[k] % h->yDim;
        int32_t bx = y / (32 * vec);
        int32_t by = x / (halcuda::kTickWarps * halcuda::kTickRowsPerThread);
        blockOf[k] = by * gx + bx;
        start[blockOf[k] + 1]++;
    }
    for (int32_t b = 0; b < nBlocks; b++)
    {
        start[b + 1] += start[b];
    }
    std::vector<int32_t> row(nPoints), col(nPoints), cursor(start.begin(), start.end() - 1);
    std::vector<float> val(nPoints);
    for (int32_t k = 0; k < nPoints; k++)
    {
        int32_t slot = cursor[blockOf[k]]++;
        row[slot] = cells[k] / h->yDim;
        col[slot] = cells[k] % h->yDim;
        val[slot] = values[k];
    }
    HAL_TRY(h->ptStart.Alloc(nBlocks + 1, "cudaMalloc(points)"));
    HAL_TRY(h->ptRow.Alloc(nPoints, "cudaMalloc(points)"));
    HAL_TRY(h->ptCol.Alloc(nPoints, "cudaMalloc(points)"));
    HAL_TRY(h->ptVal.Alloc(nPoints, "cudaMalloc(points)"));
    HAL_TRY(halcuda::CudaStatus(cudaMemcpy(h->ptStart.p, start.data(), (nBlocks + 1) * sizeof(int32_t),
                                           cudaMemcpyHostToDevice), "cudaMemcpy(points)"));
    HAL_TRY(halcuda::CudaStatus(cudaMemcpy(h->ptRow.p, row.data(), nPoints * sizeof(int32_t), cudaMemcpyHostToDevice),
                                "cudaMemcpy(points)"));
    HAL_TRY(halcuda::CudaStatus(cudaMemcpy(h->ptCol.p, col.data(), nPoints * sizeof(int32_t), cudaMemcpyHostToDevice),
                                "cudaMemcpy(points)"));
    HAL_TRY(halcuda::CudaStatus(cudaMemcpy(h->ptVal.p, val.data(), nPoints * sizeof(float), cudaMemcpyHostToDevice),
                                "cudaMemcpy(points)"));
    h->hasPoints = true;
    h->nPoints = nPoints;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_diffusion_set_uptake(hal_cuda_diffusion *h, hal_cuda_agents *agents, double uptake)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffusion_set_uptake: handle is NULL");
    if (agents == nullptr)
    {
        h->agents = nullptr;
        h->uptake = 0.0;
        return HAL_CUDA_OK;
    }
    HAL_REQUIRE(std::isfinite(uptake), "hal_cuda_diffusion_set_uptake: uptake must be finite");
    int32_t ax = 0, ay = 0;
    halcuda::AgentsCellOffsets(agents, &ax, &ay);
    HAL_REQUIRE(ax == h->xDim && ay == h->yDim,
                "hal_cuda_diffusion_set_uptake: agent grid %dx%d differs from the field %dx%d", ax, ay, h->xDim,
                h->yDim);
    h->agents = agents;
    h->uptake = uptake;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_diffusion_test_stall(hal_cuda_diffusion *h, int32_t stall, double waitSeconds)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffusion_test_stall: handle is NULL");
    HAL_REQUIRE(waitSeconds >= 0.0 && waitSeconds <= 2.0, "hal_cuda_diffusion_test_stall: wait %g s outside [0, 2]",
                waitSeconds);
    // 16 bytes more than the copy brings: the mbarrier's phase never
    // completes, and the bounded wait runs out
    h->testExtraTx = stall ? 16u : 0u;
    h->testWaitUs = static_cast<uint32_t>(waitSeconds * 1e6);
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_diffusion_set_blocking(hal_cuda_diffusion *h, int32_t ticksPerLaunch)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffusion_set_blocking: handle is NULL");
    HAL_REQUIRE(ticksPerLaunch >= 0 && ticksPerLaunch <= 2, "hal_cuda_diffusion_set_blocking: %d ticks per launch",
                ticksPerLaunch);
    if (ticksPerLaunch == 2 && !h->tmapOk)
    {
        halcuda::SetError("hal_cuda_diffusion_set_blocking: two-tick launches need yDim %% 4 == 0");
        return HAL_CUDA_ENOTSUP;
    }
    h->blockMode = ticksPerLaunch;
    h->ResetGraphs();
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_diffusion_set_velocity(hal_cuda_diffusion *h, double xVel, double yVel)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffusion_set_velocity: handle is NULL");
    HAL_REQUIRE(std::isfinite(xVel) && std::isfinite(yVel), "hal_cuda_diffusion_set_velocity: velocity must be finite");
    HAL_REQUIRE(!(std::fabs(xVel) + std::fabs(yVel) > 0.5),
                "Advection rate component sum above stable maximum value of 0.5");
    h->xVel = xVel;
    h->yVel = yVel;
    h->ResetGraphs();
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_diffusion_set_dirichlet(hal_cuda_diffusion *h, const float *ghost)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffusion_set_dirichlet: handle is NULL");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    h->ResetGraphs();
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
    HAL_TRY(halcuda::CudaStatus(cudaMemcpy(h->ghost.p, ghost, ng * sizeof(float), cudaMemcpyHostToDevice),
                                "cudaMemcpy(ghost)"));
    h->hasGhost = true;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_diffusion_run_ticks(hal_cuda_diffusion *h, int32_t ticks, double diffRate,
                                            double decay, int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffusion_run_ticks: handle is NULL");
    HAL_REQUIRE(ticks >= 0, "hal_cuda_diffusion_run_ticks: negative tick count");
    HAL_REQUIRE(!(diffRate > 0.25), "Diffusion rate above stable maximum value of 0.25");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return h->RunTicks(ticks, diffRate, decay, wrapX != 0, wrapY != 0, true);
}

extern "C" int hal_cuda_diffusion_run_steps(hal_cuda_diffusion *h, float *field, int64_t len, int32_t steps,
                                            double diffRate, int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && field != nullptr, "hal_cuda_diffusion_run_steps: NULL argument");
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()),
                "DiffusionKernel2D::RunSteps: field must hold xDim*yDim values");
    HAL_REQUIRE(steps >= 0, "hal_cuda_diffusion_run_steps: negative step count");
    HAL_TRY(hal_cuda_diffusion_set_field(h, field, len));
    HAL_TRY(h->RunTicks(steps, diffRate, 0.0, wrapX != 0, wrapY != 0, false));
    return hal_cuda_diffusion_get_field(h, field, len);
}

extern "C" int hal_cuda_diffusion_sync(hal_cuda_diffusion *h)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffusion_sync: handle is NULL");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return halcuda::CudaStatus(cudaStreamSynchronize(h->stream.Get()), "hal_cuda_diffusion_sync");
}

extern "C" void *hal_cuda_diffusion_stream(hal_cuda_diffusion *h)
{
    return h ? static_cast<void *>(h->stream.Get()) : nullptr;
}

extern "C" int hal_cuda_diffusion_set_stream(hal_cuda_diffusion *h, void *stream)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_diffusion_set_stream: handle is NULL");
    h->stream.Set(stream);
    h->ResetGraphs();
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_diffusion_profile(hal_cuda_diffusion *h, int32_t iters, double diffRate, double decay,
                                          int32_t wrapX, int32_t wrapY, float *ms)
{
    HAL_REQUIRE(h != nullptr && ms != nullptr, "hal_cuda_diffusion_profile: NULL argument");
    HAL_REQUIRE(iters > 0, "hal_cuda_diffusion_profile: iters must be positive");
    HAL_REQUIRE(!(diffRate > 0.25), "Diffusion rate above stable maximum value of 0.25");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    cudaEvent_t e0, e1;
    HAL_TRY(CudaStatus(cudaEventCreate(&e0), "cudaEventCreate"));
    HAL_TRY(CudaStatus(cudaEventCreate(&e1), "cudaEventCreate"));
    double total = 0.0;
    int rc = HAL_CUDA_OK;
    for (int32_t t = 0; t < iters; t++)
    {
        int c = h->cur;
        TickParams p = h->Params(h->field[c].p, h->field[c ^ 1].p, diffRate, decay, wrapX != 0, wrapY != 0, true);
        cudaEventRecord(e0, s);
        h->LaunchTick(p, h->Uptake(true), s);
        CountLaunch();
        cudaEventRecord(e1, s);
        rc = LaunchStatus("TickKernel launch");
        if (rc == HAL_CUDA_OK)
        {
            rc = CudaStatus(cudaEventSynchronize(e1), "hal_cuda_diffusion_profile");
        }
        if (rc != HAL_CUDA_OK)
        {
            break;
        }
        float a = 0.0f;
        cudaEventElapsedTime(&a, e0, e1);
        total += a;
        h->cur ^= 1;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    HAL_TRY(rc);
    *ms = static_cast<float>(total / iters);
    return HAL_CUDA_OK;
}
