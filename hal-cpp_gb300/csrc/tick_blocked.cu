// tick_blocked.cu -- two fused explicit ticks per launch (temporal blocking).
//
// The one-tick kernel (diffusion.cu) reads the field and writes the next one:
// 8 bytes per cell-update.  When the ping-pong pair does not fit in L2 (fields
// of many millions of cells) every tick streams both through HBM.  Here a CTA
// stages a 32 x 128 tile of the field with a 2-cell halo in shared memory
// (one 2-D TMA copy, zero fill outside the field), computes the first tick on
// the tile plus a 1-cell ring, and the second tick on the tile, so each pair
// of ticks reads and writes the field once: 4 bytes per cell-update.
//
// Each tick is PDEGrid2D's (PDEGrid2D.h:103-186, 289-375):
//   f' = f + (sum over the four sides of w_side * (nbr - f) - decay * f + S)
// with w_side = r (+ the upwind velocity from that side when advecting), a
// neighbour difference weighted 1 on the grid (or wrapped onto it), 2 for a
// Dirichlet ghost ((bc - f) * 2) and 0 past a zero-flux edge, and S the dense
// source plus the point sources (summed into one array on the host).  The
// arithmetic per tick is the one-tick kernel's general path; only the source
// terms are pre-summed, so results agree with it to FP32 rounding.
#include "common.cuh"
#include "tick_params.h"

#include <cuda.h>
#include <cudaTypedefs.h>

namespace halcuda
{
    namespace
    {
        constexpr int kBX = kTickBlockRows;  // output rows (x) per CTA
        constexpr int kBY = kTickBlockCols;  // output columns (y) per CTA
        constexpr int kAR = kBX + 4;         // staged rows: x0-2 .. x0+kBX+1
        constexpr int kAC = kBY + 8;         // staged columns: y0-4 .. y0+kBY+3 (16-byte aligned box)
        constexpr int kBR = kBX + 2;         // first-tick rows: x0-1 .. x0+kBX
        constexpr int kThreads = 256;
        constexpr unsigned long long kWaitLimitNs = 2000000000ull;

        __device__ __forceinline__ unsigned long long GlobalTimerNs()
        {
            unsigned long long t;
            asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
            return t;
        }

        __device__ __forceinline__ uint32_t SmemAddr(const void *p)
        {
            return static_cast<uint32_t>(__cvta_generic_to_shared(p));
        }

        // Waits for phase 0 of the mbarrier at shared address bar for at most
        // limitNs of %globaltimer; returns whether the phase completed.
        __device__ __forceinline__ bool MbarWaitBounded(uint32_t bar, unsigned long long limitNs)
        {
            const unsigned long long t0 = GlobalTimerNs();
            uint32_t done = 0;
            while (!done)
            {
                asm volatile(
                    "{ .reg .pred ok; mbarrier.try_wait.parity.shared::cta.b64 ok, [%1], 0, %2; selp.u32 %0, 1, 0, "
                    "ok; }"
                    : "=r"(done)
                    : "r"(bar), "r"(1000000u)
                    : "memory");
                if (!done && GlobalTimerNs() - t0 > limitNs)
                {
                    return false;
                }
            }
            return true;
        }

        // Grid coordinate of an extended coordinate on one axis: itself on
        // the grid, wrapped on a periodic axis, else -1 (off the grid).
        __device__ __forceinline__ int32_t OnGrid(int32_t v, int32_t dim, bool wrap)
        {
            if (v >= 0 && v < dim)
            {
                return v;
            }
            if (wrap)
            {
                const int32_t m = v % dim;  // the halo can reach several periods past a tiny grid
                return (m < 0) ? m + dim : m;
            }
            return -1;
        }

        // Weight of the difference towards neighbour coordinate n on an axis.
        __device__ __forceinline__ float SideWeight(int32_t n, int32_t dim, bool wrap, float offGrid)
        {
            return (wrap || (n >= 0 && n < dim)) ? 1.0f : offGrid;
        }

        template <bool ADV>
        __device__ __forceinline__ float CellTick(const TickBlockParams &p, float c, float up, float dn, float ym,
                                                  float yp, float wUp, float wDn, float wYm, float wYp, float s)
        {
            float d;
            if constexpr (ADV)
            {
                float sum = (dn - c) * (wDn * p.kDn);
                sum = fmaf(up - c, wUp * p.kUp, sum);
                sum = fmaf(yp - c, wYp * p.kYp, sum);
                sum = fmaf(ym - c, wYm * p.kYm, sum);
                d = fmaf(c, p.negDecay, sum);
            }
            else
            {
                float sum = (dn - c) * wDn;
                sum = fmaf(up - c, wUp, sum);
                sum = fmaf(yp - c, wYp, sum);
                sum = fmaf(ym - c, wYm, sum);
                d = sum * p.r;
                d = fmaf(c, p.negDecay, d);
            }
            return c + (d + s);
        }

        __global__ void __launch_bounds__(kThreads) TickBlocked2(TickBlockParams p,
                                                                 const __grid_constant__ CUtensorMap tmap)
        {
            extern __shared__ __align__(128) float smem[];
            float *A = smem;            // kAR x kAC: the field around the tile
            float *B = A + kAR * kAC;   // kBR x kAC: the first tick (rows x0-1 ..)
            __shared__ __align__(8) unsigned long long mbar;
            __shared__ int s_fail;

            const int tid = threadIdx.x;
            const int32_t x0 = static_cast<int32_t>(blockIdx.y) * kBX;
            const int32_t y0 = static_cast<int32_t>(blockIdx.x) * kBY;
            const bool wrapX = p.wrapX != 0, wrapY = p.wrapY != 0;
            const float gw = (p.ghost.xlo != nullptr) ? 2.0f : 0.0f;  // off-grid difference weight

            // ---- stage rows x0-2 .. x0+kBX+1, columns y0-4 .. y0+kBY+3 ---------
            const uint32_t bar = SmemAddr(&mbar);
            const uint32_t bytes = static_cast<uint32_t>(kAR * kAC * sizeof(float));
            if (tid == 0)
            {
                s_fail = 0;
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
                asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                             "r"(bytes + p.extraTx)
                             : "memory");
                asm volatile(
                    "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                    " [%0], [%1, {%2, %3}], [%4];" ::"r"(SmemAddr(A)),
                    "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(y0 - 4), "r"(x0 - 2), "r"(bar)
                    : "memory");
            }
            __syncthreads();  // mbarrier initialised before anyone waits on it
            // bounded wait for the tile; one that gives up records the
            // failure and waits once more (bounded again), so that the copy
            // is not still writing into shared memory when the CTA exits
            const unsigned long long limitNs =
                (p.waitLimitUs != 0) ? 1000ull * static_cast<unsigned long long>(p.waitLimitUs) : kWaitLimitNs;
            if (!MbarWaitBounded(bar, limitNs))
            {
                s_fail = 1;
                MbarWaitBounded(bar, limitNs);
            }
            __syncthreads();
            if (s_fail)
            {
                if (tid == 0)
                {
                    atomicExch(p.err, 1);
                }
                return;
            }

            // ---- halo cells the copy filled with zeros: wrapped values and
            // Dirichlet ghosts (only tiles at an edge of the grid have any) --
            const bool edgeTile = x0 - 2 < 0 || x0 + kBX + 1 >= p.xDim || y0 - 4 < 0 || y0 + kBY + 3 >= p.yDim;
            if (edgeTile)
            {
                for (int i = tid; i < kAR * kAC; i += kThreads)
                {
                    const int32_t x = x0 - 2 + i / kAC;
                    const int32_t y = y0 - 4 + i % kAC;
                    const bool inX = x >= 0 && x < p.xDim, inY = y >= 0 && y < p.yDim;
                    if (inX && inY)
                    {
                        continue;  // staged by the copy
                    }
                    const int32_t xg = OnGrid(x, p.xDim, wrapX), yg = OnGrid(y, p.yDim, wrapY);
                    float v = 0.0f;
                    if (xg >= 0 && yg >= 0)
                    {
                        v = __ldg(p.f + static_cast<int64_t>(xg) * p.yDim + yg);  // wrapped
                    }
                    else if (p.ghost.xlo != nullptr)
                    {
                        if (xg >= 0 && y == -1)
                        {
                            v = __ldg(p.ghost.ylo + xg);
                        }
                        else if (xg >= 0 && y == p.yDim)
                        {
                            v = __ldg(p.ghost.yhi + xg);
                        }
                        else if (yg >= 0 && x == -1)
                        {
                            v = __ldg(p.ghost.xlo + yg);
                        }
                        else if (yg >= 0 && x == p.xDim)
                        {
                            v = __ldg(p.ghost.xhi + yg);
                        }
                    }
                    A[i] = v;
                }
                __syncthreads();
            }

            // ---- first tick on rows x0-1 .. x0+kBX, columns y0-1 .. y0+kBY --
            constexpr int kC1 = kBY + 2;
            for (int i = tid; i < kBR * kC1; i += kThreads)
            {
                const int rb = i / kC1;        // B row: x = x0 - 1 + rb
                const int cb = 3 + i % kC1;    // column index of both A and B: y = y0 - 4 + cb
                const int32_t x = x0 - 1 + rb;
                const int32_t y = y0 - 4 + cb;
                const int ia = (rb + 1) * kAC + cb;
                const int32_t xg = OnGrid(x, p.xDim, wrapX), yg = OnGrid(y, p.yDim, wrapY);
                float out;
                if (xg < 0 || yg < 0)
                {
                    out = A[ia];  // off the grid: keeps the ghost (or the zero) as the second tick's neighbour
                }
                else
                {
                    const float s = (p.S != nullptr) ? __ldg(p.S + static_cast<int64_t>(xg) * p.yDim + yg) : 0.0f;
                    const float wUp = SideWeight(x - 1, p.xDim, wrapX, gw);
                    const float wDn = SideWeight(x + 1, p.xDim, wrapX, gw);
                    const float wYm = SideWeight(y - 1, p.yDim, wrapY, gw);
                    const float wYp = SideWeight(y + 1, p.yDim, wrapY, gw);
                    out = (p.adv != 0) ? CellTick<true>(p, A[ia], A[ia - kAC], A[ia + kAC], A[ia - 1], A[ia + 1], wUp,
                                                        wDn, wYm, wYp, s)
                                       : CellTick<false>(p, A[ia], A[ia - kAC], A[ia + kAC], A[ia - 1], A[ia + 1], wUp,
                                                         wDn, wYm, wYp, s);
                }
                B[rb * kAC + cb] = out;
            }
            __syncthreads();

            // ---- second tick on the tile: float4 groups of columns ----------
            constexpr int kG = kBY / 4;
            for (int i = tid; i < kBX * kG; i += kThreads)
            {
                const int r = i / kG;
                const int g = i % kG;
                const int32_t x = x0 + r;
                const int32_t yb = y0 + 4 * g;
                if (x >= p.xDim || yb >= p.yDim)
                {
                    continue;
                }
                const int ib = (r + 1) * kAC + 4 + 4 * g;  // B index of (x, yb)
                const float4 cur = *reinterpret_cast<const float4 *>(B + ib);
                const float4 up = *reinterpret_cast<const float4 *>(B + ib - kAC);
                const float4 dn = *reinterpret_cast<const float4 *>(B + ib + kAC);
                const float left = B[ib - 1], right = B[ib + 4];
                float4 s4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (p.S != nullptr)
                {
                    s4 = __ldg(reinterpret_cast<const float4 *>(p.S + static_cast<int64_t>(x) * p.yDim + yb));
                }
                const float wUp = SideWeight(x - 1, p.xDim, wrapX, gw);
                const float wDn = SideWeight(x + 1, p.xDim, wrapX, gw);
                const float c[4] = {cur.x, cur.y, cur.z, cur.w};
                const float u[4] = {up.x, up.y, up.z, up.w};
                const float dd[4] = {dn.x, dn.y, dn.z, dn.w};
                const float sv[4] = {s4.x, s4.y, s4.z, s4.w};
                float o[4];
#pragma unroll
                for (int k = 0; k < 4; k++)
                {
                    const int32_t y = yb + k;
                    const float ym = (k > 0) ? c[k - 1] : left;
                    const float yp = (k < 3) ? c[k + 1] : right;
                    const float wYm = SideWeight(y - 1, p.yDim, wrapY, gw);
                    const float wYp = SideWeight(y + 1, p.yDim, wrapY, gw);
                    o[k] = (p.adv != 0) ? CellTick<true>(p, c[k], u[k], dd[k], ym, yp, wUp, wDn, wYm, wYp, sv[k])
                                        : CellTick<false>(p, c[k], u[k], dd[k], ym, yp, wUp, wDn, wYm, wYp, sv[k]);
                }
                *reinterpret_cast<float4 *>(p.out + static_cast<int64_t>(x) * p.yDim + yb) =
                    make_float4(o[0], o[1], o[2], o[3]);
            }
        }

        PFN_cuTensorMapEncodeTiled_v12000 Encoder()
        {
            // looked up once (thread-safe static initialisation)
            static const PFN_cuTensorMapEncodeTiled_v12000 s_fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
                void *fn = nullptr;
                cudaDriverEntryPointQueryResult q;
                if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                        cudaSuccess &&
                    q == cudaDriverEntryPointSuccess)
                {
                    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
                }
                return nullptr;
            }();
            return s_fn;
        }

        constexpr size_t kSmemBytes = sizeof(float) * static_cast<size_t>((kAR + kBR) * kAC);
    }

    bool MakeTickBlockTensorMap(TickBlockTensorMap &map, const float *field, int32_t xDim, int32_t yDim)
    {
        static_assert(sizeof(TickBlockTensorMap) == sizeof(CUtensorMap), "opaque tensor map size");
        PFN_cuTensorMapEncodeTiled_v12000 enc = Encoder();
        if (enc == nullptr || (yDim % 4) != 0 || (reinterpret_cast<uintptr_t>(field) & 15) != 0)
        {
            return false;
        }
        cuuint64_t gdim[2] = {static_cast<cuuint64_t>(yDim), static_cast<cuuint64_t>(xDim)};
        cuuint64_t gstride[1] = {static_cast<cuuint64_t>(yDim) * 4u};
        cuuint32_t box[2] = {static_cast<cuuint32_t>(kAC), static_cast<cuuint32_t>(kAR)};
        cuuint32_t estr[2] = {1, 1};
        CUresult r = enc(reinterpret_cast<CUtensorMap *>(&map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                         const_cast<float *>(field), gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        return r == CUDA_SUCCESS;
    }

    int PrepareTickBlocked()
    {
        static SmemLimit s_limit;
        return s_limit.Ensure(TickBlocked2, kSmemBytes, "cudaFuncSetAttribute(TickBlocked2)");
    }

    void LaunchTickBlocked2(const TickBlockParams &p, const TickBlockTensorMap &map, cudaStream_t s)
    {
        const dim3 grid(static_cast<unsigned>((p.yDim + kBY - 1) / kBY), static_cast<unsigned>((p.xDim + kBX - 1) / kBX));
        const CUtensorMap &tm = *reinterpret_cast<const CUtensorMap *>(&map);
        TickBlocked2<<<grid, kThreads, kSmemBytes, s>>>(p, tm);
    }
}
