// adi.cu -- ADI (alternating-direction implicit) diffusion on sm_103a.
//
// One ADI step (Internal::Diffusion2DADI, include/Hal/Pde/ADIequations.h:
// 306-378) is two sweeps:
//   x-sweep: for every y, solve (I - r/2 Lx) w = (I + r/2 Ly) f along x;
//   y-sweep: for every x, solve (I - r/2 Ly) v = (I + r/2 Lx) w along y,
//            then commit v (PDEGrid2D: f' = f + (v - f) - decay f + src
//            - uptake n f).
// Every line of a sweep solves the same tridiagonal matrix; adi_plan.h
// describes the partitioned Thomas solve and its FP64 precomputation.
//
// Layout.  The resident field is kept transposed ("layout B",
// index y*xDim + x) so that the x-sweep's lines are contiguous.  Each sweep
// reads contiguous lines and writes its result transposed: the x-sweep reads
// f (B) and writes w in HAL's layout ("layout A", x*yDim + y), whose y-lines
// the y-sweep reads, writing f' back in layout B.  Both sweeps therefore run
// the same kernel, AdiSweep:
//   1. stage the CTA's R lines plus the line on either side (the explicit
//      cross-axis term) into shared memory with TMA, completion on an
//      mbarrier whose wait is bounded.  When L is a multiple of 256 one 3-D
//      tensor copy (cp.async.bulk.tensor, box 32 x P x (R+2), 128-byte
//      swizzle, zero fill outside the field) stages the whole tile and the
//      kernel indexes shared memory through the same swizzle; otherwise each
//      32-element chunk is a 1-D cp.async.bulk (or plain loads for ragged
//      lines) into a 36-float slot.  Either way every later access is a
//      conflict-free 128-bit LDS/STS;
//   2. each thread solves one 32-row chunk of two lines (two interleaved
//      Thomas chains in registers), exchanges the separator right-hand sides
//      through shared memory, applies the banded reduced solve and the
//      coupling correction (and the periodic Sherman-Morrison correction);
//   3. the tile is written out transposed, four lines (16 bytes) per store,
//      with the commit terms applied on the way out.
#include "common.cuh"
#include "adi_plan.h"
#include "adi_sweep.h"
#include "adi64.h"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

namespace halcuda
{
    namespace
    {
        constexpr int M = kAdiM;
        constexpr int kCoefFloats = 3 * kCoefCount * M;
        // in shared memory each block type's coefficients start 16 bytes
        // further along the banks than the last type's, so that a warp whose
        // chunks span two types reads both in one wavefront
        constexpr int kCoefTypeStride = kCoefCount * M + 4;
        constexpr int kCoefSmemFloats = 3 * kCoefTypeStride;
        constexpr int kChunkStride = M + 4;  // floats per 32-element chunk in shared memory
        constexpr int kNL = 2;               // lines solved by one thread
        constexpr int kMaxThreads = 512;
        constexpr int kMaxR = 128;           // lines per CTA (a power of two, >= 8)
        constexpr int kGbandSmem = 2048;     // floats of G's band staged in shared memory
        // bound of the mbarrier wait (ns of %globaltimer); the staged copies
        // take microseconds, so reaching it means the copies never landed
        constexpr unsigned long long kWaitLimitNs = 2000000000ull;

        // Thomas forward elimination and back substitution of one 32-row
        // block (with the identity padding described in adi_plan.h) for all
        // kNL lines of a thread: each coefficient vector is read from shared
        // memory 16 bytes at a time, once, and applied to every line, and the
        // lines' recurrences interleave.
        __device__ __forceinline__ void BlockSolveN(float (&z)[kNL][M], const float *cf)
        {
            const float4 *fw = reinterpret_cast<const float4 *>(cf + kCoefFw * M);
            const float4 *ib = reinterpret_cast<const float4 *>(cf + kCoefIb * M);
            const float4 *cb = reinterpret_cast<const float4 *>(cf + kCoefCb * M);
#pragma unroll
            for (int j = 0; j < M / 4; j++)
            {
                const float4 w4 = fw[j];
#pragma unroll
                for (int l = 0; l < kNL; l++)
                {
                    if (j > 0)
                    {
                        z[l][4 * j] = fmaf(-w4.x, z[l][4 * j - 1], z[l][4 * j]);
                    }
                    z[l][4 * j + 1] = fmaf(-w4.y, z[l][4 * j], z[l][4 * j + 1]);
                    z[l][4 * j + 2] = fmaf(-w4.z, z[l][4 * j + 1], z[l][4 * j + 2]);
                    z[l][4 * j + 3] = fmaf(-w4.w, z[l][4 * j + 2], z[l][4 * j + 3]);
                }
            }
#pragma unroll
            for (int j = M / 4 - 1; j >= 0; j--)
            {
                const float4 i4 = ib[j];
                const float4 c4 = cb[j];
#pragma unroll
                for (int l = 0; l < kNL; l++)
                {
                    if (j == M / 4 - 1)
                    {
                        z[l][4 * j + 3] *= i4.w;
                    }
                    else
                    {
                        z[l][4 * j + 3] = fmaf(-c4.w, z[l][4 * j + 4], z[l][4 * j + 3] * i4.w);
                    }
                    z[l][4 * j + 2] = fmaf(-c4.z, z[l][4 * j + 3], z[l][4 * j + 2] * i4.z);
                    z[l][4 * j + 1] = fmaf(-c4.y, z[l][4 * j + 2], z[l][4 * j + 1] * i4.y);
                    z[l][4 * j + 0] = fmaf(-c4.x, z[l][4 * j + 1], z[l][4 * j + 0] * i4.x);
                }
            }
        }

        // The coupling correction x = z - sL p - sR q over the block, for all
        // kNL lines with one read of p and q.
        __device__ __forceinline__ void BlockCorrectN(float (&z)[kNL][M], const float *cf, const float (&sL)[kNL],
                                                      const float (&sR)[kNL])
        {
            const float4 *pv = reinterpret_cast<const float4 *>(cf + kCoefP * M);
            const float4 *qv = reinterpret_cast<const float4 *>(cf + kCoefQ * M);
#pragma unroll
            for (int j = 0; j < M / 4; j++)
            {
                const float4 p4 = pv[j];
                const float4 q4 = qv[j];
#pragma unroll
                for (int l = 0; l < kNL; l++)
                {
                    z[l][4 * j + 0] = fmaf(-sL[l], p4.x, fmaf(-sR[l], q4.x, z[l][4 * j + 0]));
                    z[l][4 * j + 1] = fmaf(-sL[l], p4.y, fmaf(-sR[l], q4.y, z[l][4 * j + 1]));
                    z[l][4 * j + 2] = fmaf(-sL[l], p4.z, fmaf(-sR[l], q4.z, z[l][4 * j + 2]));
                    z[l][4 * j + 3] = fmaf(-sL[l], p4.w, fmaf(-sR[l], q4.w, z[l][4 * j + 3]));
                }
            }
        }

        // Separators on both sides of chunk k in one pass over the exchanged
        // values s_m = xA[m] + xB[m]: sR = row k of G, sL = row k-1 (each 0
        // where that separator does not exist).  G is the banded inverse,
        // rows of 2B+1 entries, in shared or global memory.
        __device__ __forceinline__ void BandDot2(const float *G, int32_t P, int32_t B, int k, const float *xA,
                                                 const float *xB, float &sL, float &sR)
        {
            const int S = P - 1;
            const int W = 2 * B + 1;
            sL = 0.0f;
            sR = 0.0f;
            const int lo = max(0, k - 1 - B);
            const int hi = min(S - 1, k + B);
            const bool hasR = k < S, hasL = k >= 1;
            for (int m = lo; m <= hi; m++)
            {
                const float sm = xA[m] + xB[m];
                if (hasR && m >= k - B)
                {
                    sR = fmaf(G[k * W + (m - k + B)], sm, sR);
                }
                if (hasL && m <= k - 1 + B)
                {
                    sL = fmaf(G[(k - 1) * W + (m - k + 1 + B)], sm, sL);
                }
            }
        }

        // BandDot2 for a band half-width B known at compile time: the same
        // products in the same (ascending m) order, unrolled.
        template <int B>
        __device__ __forceinline__ void BandDot2Fixed(const float *G, int32_t P, int k, const float *xA,
                                                      const float *xB, float &sL, float &sR)
        {
            constexpr int W = 2 * B + 1;
            const int S = P - 1;
            sL = 0.0f;
            sR = 0.0f;
            const bool hasR = k < S, hasL = k >= 1;
#pragma unroll
            for (int t = 0; t <= 2 * B + 1; t++)
            {
                const int m = k - 1 - B + t;
                if (m < 0 || m > S - 1)
                {
                    continue;
                }
                const float sm = xA[m] + xB[m];
                if (hasR && t >= 1)
                {
                    sR = fmaf(G[k * W + (t - 1)], sm, sR);
                }
                if (hasL && t <= 2 * B)
                {
                    sL = fmaf(G[(k - 1) * W + t], sm, sL);
                }
            }
        }

        // Float offset, within the staged lines, of element i of chunk k of
        // staged line `line`.  SWZ: the TMA tensor layout with 128-byte
        // swizzle (128-byte rows row = line*P + k, 16-byte unit u stored at
        // u ^ (row & 7); the swizzled path is used only when P % 8 == 0, so
        // row & 7 == k & 7); otherwise chunks padded to kChunkStride floats
        // with line stride LS.
        template <bool SWZ>
        __device__ __forceinline__ int SOff(int line, int k, int i, int P, int LS)
        {
            if constexpr (SWZ)
            {
                // P % 8 == 0, so row & 7 == k & 7
                return (line * P + k) * M + (i ^ ((k & 7) << 2));
            }
            else
            {
                return line * LS + k * kChunkStride + i;
            }
        }

        // Float offset of the 16-byte unit q (elements 4q..4q+3) of chunk k.
        template <bool SWZ>
        __device__ __forceinline__ int SOff4(int line, int k, int q, int P, int LS)
        {
            if constexpr (SWZ)
            {
                return (line * P + k) * M + ((q ^ (k & 7)) << 2);
            }
            else
            {
                return line * LS + k * kChunkStride + 4 * q;
            }
        }

        // The same for a precomputed row (line*P + k) and swizzle term k & 7.
        template <bool SWZ>
        __device__ __forceinline__ int SOff4Row(int row, int k, int q, int sw, int P, int LS)
        {
            if constexpr (SWZ)
            {
                return row * M + ((q ^ sw) << 2);
            }
            else
            {
                return (row / P) * LS + k * kChunkStride + 4 * q;
            }
        }

        // Solution rows (both layouts).  The solve writes each chunk of a
        // line back over its staged row with the 16-byte units permuted once
        // more by SolSwz(line quad): the write-out reads the same unit of 4
        // (or 8) quads in one quarter-warp, and the extra permutation puts
        // them in different bank groups.  The permutation is within a chunk,
        // which the one thread that solved it writes whole.
        __device__ __forceinline__ int SolSwz(int ll)
        {
            const int qd = ll >> 2;
            return ((qd << 1) & 6) | ((qd >> 2) & 1);
        }

        // Float offset of unit q of chunk k of solution line ll (staged row
        // ll + 1).
        template <bool SWZ>
        __device__ __forceinline__ int SolOff4(int ll, int k, int q, int P, int LS)
        {
            if constexpr (SWZ)
            {
                return ((ll + 1) * P + k) * M + ((q ^ (k & 7) ^ SolSwz(ll)) << 2);
            }
            else
            {
                return SOff4<SWZ>(ll + 1, k, q ^ SolSwz(ll), P, LS);
            }
        }

        // Element pos of solution line ll.
        template <bool SWZ>
        __device__ __forceinline__ int SolPos(int ll, int32_t pos, int P, int LS)
        {
            const int k = pos >> 5;
            const int i = pos & 31;
            return SolOff4<SWZ>(ll, k, i >> 2, P, LS) + (i & 3);
        }

        // Element pos of a staged line.
        template <bool SWZ>
        __device__ __forceinline__ int SPos(int line, int32_t pos, int P, int LS)
        {
            return SOff<SWZ>(line, pos >> 5, pos & 31, P, LS);
        }

        __device__ __forceinline__ float4 Ld4(const float *p)
        {
            return *reinterpret_cast<const float4 *>(p);
        }

        __device__ __forceinline__ void St4(float *p, float4 v)
        {
            *reinterpret_cast<float4 *>(p) = v;
        }

        __device__ __forceinline__ uint32_t SmemAddr(const void *p)
        {
            return static_cast<uint32_t>(__cvta_generic_to_shared(p));
        }

        __device__ __forceinline__ unsigned long long GlobalTimerNs()
        {
            unsigned long long t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            return t;
        }

        // Waits for phase 0 of the mbarrier at shared address bar, suspended
        // in try_wait between polls, for at most limitNs of %globaltimer;
        // returns whether the phase completed.
        __device__ __forceinline__ bool MbarWaitBounded(uint32_t bar, unsigned long long limitNs)
        {
            const unsigned long long t0 = GlobalTimerNs();
            uint32_t done = 0;
            while (!done)
            {
                asm volatile(
                    "{ .reg .pred ok; mbarrier.try_wait.parity.shared::cta.b64 ok, [%1], 0, %2; selp.u32 %0, 1, 0, ok; }"
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

        // One CTA's tile of a sweep: lines x0 .. x0+R-1 of the grid p.  tmap
        // is the grid's line tensor map (SWZ) or null.
        // Agent counts of write-out unit u: nc[e][i] = agents binned in cell
        // (line0 + e, 4u + i), i.e. offsets[c + 1] - offsets[c] at c = (line0
        // + e) * L + 4u + i (cells in layout A); 0 for the quad's lines at or
        // past quadLines (outside the grid).  With L % 4 == 0 each line's five
        // offsets are one 16-byte load and one 4-byte load.
        __device__ __forceinline__ void UnitCounts(const int32_t *__restrict__ off, int32_t line0, int32_t quadLines,
                                                   int32_t u, int32_t L, bool vecL, int32_t (&nc)[4][4])
        {
#pragma unroll
            for (int e = 0; e < 4; e++)
            {
                const int32_t *oc = off + static_cast<int64_t>(line0 + e) * L + 4 * u;
                if (e >= quadLines)
                {
                    nc[e][0] = nc[e][1] = nc[e][2] = nc[e][3] = 0;
                }
                else if (vecL)
                {
                    const int4 a = __ldg(reinterpret_cast<const int4 *>(oc));
                    const int32_t b = __ldg(oc + 4);
                    nc[e][0] = a.y - a.x;
                    nc[e][1] = a.z - a.y;
                    nc[e][2] = a.w - a.z;
                    nc[e][3] = b - a.w;
                }
                else
                {
#pragma unroll
                    for (int i = 0; i < 4; i++)
                    {
                        nc[e][i] = (4 * u + i < L) ? __ldg(oc + i + 1) - __ldg(oc + i) : 0;
                    }
                }
            }
        }

        // UPT: the y-sweep's commit has the agent uptake term (a separate
        // instantiation, so that the uncoupled tick keeps its registers).
        template <int MODE, bool SWZ, bool UPT = false>
        __device__ __forceinline__ void SweepTile(const SweepParams &p, const CUtensorMap *tmap, const int32_t x0)
        {
            extern __shared__ __align__(1024) float smem[];
            __shared__ __align__(8) unsigned long long mbar;
            __shared__ int s_fail;
            __shared__ uint32_t s_tmaBytes;
            const int P = p.plan.P;
            const int R = p.R;
            // staged lines first, on a 1024-byte boundary (128-byte swizzle)
            // the dynamic buffer is declared 1024-byte aligned (the 128-byte
            // swizzle pattern repeats every 1024 bytes) and used directly, so
            // every access through it is a shared-memory access
            float *sLines = smem;
            float *sCoef = sLines + (R + 2) * p.LS;  // kCoefSmemFloats
            float *xA = sCoef + kCoefSmemFloats;     // R * P
            float *xB = xA + R * P;                  // R * P
            float *sG = xB + R * P;                  // kGbandSmem: G's band when it fits
            const int gCount = (P > 1) ? (P - 1) * (2 * p.plan.B + 1) : 0;
            const bool gInSmem = gCount <= kGbandSmem;
            const float *G = gInSmem ? sG : p.plan.gband;

            const int tid = threadIdx.x;
            const int nthreads = blockDim.x;
            if ((SmemAddr(smem) & 1023u) != 0u)
            {
                if (tid == 0)
                {
                    atomicExch(p.err, 2);
                }
                return;  // uniform: the address is the same for every thread
            }
            if constexpr (!SWZ)
            {
                // the chunked form also runs the batched tiles, whose shapes
                // come from a table: the tile's shape must fit its launch
                // (every line pair of every chunk has a thread, and the
                // buffers above fit the dynamic shared memory; uniform: the
                // same values for every thread)
                uint32_t dynBytes;
                asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dynBytes));
                const int64_t need = 4 * (static_cast<int64_t>(R + 2) * p.LS + kCoefSmemFloats +
                                          2 * static_cast<int64_t>(R) * P + kGbandSmem);
                if (R < 1 || R > kMaxR || (R / kNL) * P > nthreads || need > static_cast<int64_t>(dynBytes) ||
                    p.inStride < p.L || p.outStride < p.Nlines)
                {
                    if (tid == 0)
                    {
                        atomicExch(p.err, 3);
                    }
                    return;
                }
            }
            const int32_t L = p.L;
            const bool vecL = (L & 3) == 0;
            // lines padded to a multiple of 4 floats: whole 16-byte copies,
            // the padding (zeros) included
            const int32_t L4 = (L + 3) & ~3;
            const bool inPadded = p.inStride >= L4 && (p.inStride & 3) == 0;

            // ---- 1. stage lines x0-1 .. x0+R --------------------------------
            __shared__ const float *sSrc[kMaxR + 2];
            __shared__ int sTma[kMaxR + 2];
            const uint32_t bar = SmemAddr(&mbar);
            const int nStaged = R + 2;
            uint32_t tmaBytes = 0;
            if constexpr (SWZ)
            {
                // one 3-D tensor copy: 32 floats x P chunks x (R+2) lines; lines
                // outside the grid arrive as zeros
                tmaBytes = static_cast<uint32_t>(nStaged) * static_cast<uint32_t>(P) * M * 4u;
                if (tid == 0)
                {
                    s_fail = 0;
                    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
                    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(tmaBytes)
                                 : "memory");
                    asm volatile(
                        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(SmemAddr(sLines)),
                        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(0), "r"(0), "r"(x0 - 1), "r"(bar)
                        : "memory");
                }
                for (int q = tid; q < kCoefFloats / 4; q += nthreads)
                {
                    const int t = q / (kCoefCount * M / 4);
                    St4(sCoef + t * kCoefTypeStride + 4 * (q - t * (kCoefCount * M / 4)),
                        __ldg(reinterpret_cast<const float4 *>(p.plan.coef) + q));
                }
                if (gInSmem)
                {
                    for (int q = tid; q < gCount; q += nthreads)
                    {
                        sG[q] = __ldg(p.plan.gband + q);
                    }
                }
                __syncthreads();  // mbarrier initialised before anyone waits on it
            }
            else
            {
                if (tid == 0)
                {
                    s_fail = 0;
                    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
                    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
                }
                for (int rs = tid; rs < nStaged; rs += nthreads)
                {
                    // source of staged line rs: a grid line, the neighbour line
                    // beyond an edge (wrapped, a Dirichlet ghost line, or zeros);
                    // lines further out (a CTA past the last line) are never read
                    const int32_t line = x0 - 1 + rs;
                    const float *src = nullptr;
                    bool padded = false;  // the line's stride pads it to a multiple of 4 floats
                    if (line >= 0 && line < p.Nlines)
                    {
                        src = p.in + static_cast<int64_t>(line) * p.inStride;
                        padded = inPadded;
                    }
                    else if (line == -1 || line == p.Nlines)
                    {
                        if (p.wrapLines)
                        {
                            src = p.in + static_cast<int64_t>((line < 0) ? p.Nlines - 1 : 0) * p.inStride;
                            padded = inPadded;
                        }
                        else
                        {
                            src = (line < 0) ? p.ghostLo : p.ghostHi;
                        }
                    }
                    sSrc[rs] = src;
                    sTma[rs] = (src != nullptr) && (vecL || padded) && ((reinterpret_cast<uintptr_t>(src) & 15) == 0);
                }
                for (int q = tid; q < kCoefFloats / 4; q += nthreads)
                {
                    const int t = q / (kCoefCount * M / 4);
                    St4(sCoef + t * kCoefTypeStride + 4 * (q - t * (kCoefCount * M / 4)),
                        __ldg(reinterpret_cast<const float4 *>(p.plan.coef) + q));
                }
                if (gInSmem)
                {
                    for (int q = tid; q < gCount; q += nthreads)
                    {
                        sG[q] = __ldg(p.plan.gband + q);
                    }
                }
                __syncthreads();  // mbarrier initialised, line sources known
                if (tid == 0)
                {
                    for (int rr = 0; rr < nStaged; rr++)
                    {
                        tmaBytes += sTma[rr] ? static_cast<uint32_t>(L4) * 4u : 0u;
                    }
                    if (tmaBytes > 0)
                    {
                        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(tmaBytes)
                                     : "memory");
                    }
                    s_tmaBytes = tmaBytes;
                }
                __syncthreads();  // the expected byte count is in place before any copy lands
                tmaBytes = s_tmaBytes;
                {
                    // thread -> chunk kc of lines rr0, rr0 + rstride, ...
                    const int kc = tid % P;
                    const int rstride = nthreads / P;
                    const int32_t n = min(M, L - kc * M);  // elements of this chunk inside the line
                    const int32_t n4 = (n + 3) & ~3;          // the same in whole 16-byte units
                    for (int rr = tid / P; rr < nStaged && tid < rstride * P; rr += rstride)
                    {
                        const float *src = sSrc[rr];
                        float *dst = sLines + rr * p.LS + kc * kChunkStride;
                        int32_t filled = n;  // elements the copies write
                        if (sTma[rr])
                        {
                            // a padded line's last chunk takes its padding
                            // (zeros) along, to a whole 16-byte unit
                            filled = n4;
                            asm volatile(
                                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                                    SmemAddr(dst)),
                                "l"(src + kc * M), "r"(static_cast<uint32_t>(n4) * 4u), "r"(bar)
                                : "memory");
                        }
                        else if (src != nullptr)
                        {
                            // a line the bulk copy cannot take (unaligned or
                            // ragged): 4-byte asynchronous copies, all of the
                            // chunk in flight at once; the thread waits for
                            // its own copies below
                            for (int i = 0; i < n; i++)
                            {
                                asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(SmemAddr(dst + i)),
                                             "l"(src + kc * M + i)
                                             : "memory");
                            }
                        }
                        else
                        {
                            for (int i = 0; i < n; i++)
                            {
                                dst[i] = 0.0f;
                            }
                        }
                        for (int i = filled; i < M; i++)
                        {
                            dst[i] = 0.0f;  // padding past the line end (disjoint from the copy)
                        }
                    }
                    asm volatile("cp.async.wait_all;" ::: "memory");
                }
            }
            if (tmaBytes > 0)
            {
                // every thread waits for the copies' bytes, suspended in
                // try_wait between polls; bounded by kWaitLimitNs.  A wait
                // that gives up records the failure and waits once more
                // (bounded again), so that no copy is still writing into
                // this CTA's shared memory when it exits.
                if (!MbarWaitBounded(bar, kWaitLimitNs))
                {
                    s_fail = 1;
                    MbarWaitBounded(bar, kWaitLimitNs);
                }
            }
            if constexpr (SWZ)
            {
                // the lines just outside the grid: a wrapped line or a
                // Dirichlet ghost line replaces the zeros of the tensor copy
                for (int side = 0; side < 2; side++)
                {
                    const int32_t line = (side == 0) ? -1 : p.Nlines;
                    const int rr = line - (x0 - 1);
                    if (rr < 0 || rr >= nStaged)
                    {
                        continue;
                    }
                    // (the tensor-staged form runs dense lines only: inStride == L)
                    const float *src = p.wrapLines ? p.in + static_cast<int64_t>((side == 0) ? p.Nlines - 1 : 0) * L
                                                   : ((side == 0) ? p.ghostLo : p.ghostHi);
                    if (src == nullptr)
                    {
                        continue;
                    }
                    for (int32_t pos = tid; pos < L; pos += nthreads)
                    {
                        sLines[SPos<SWZ>(rr, pos, P, p.LS)] = __ldg(src + pos);
                    }
                }
            }
            __syncthreads();
            if (s_fail)
            {
                if (tid == 0)
                {
                    atomicExch(p.err, 1);
                }
                return;  // uniform: every thread saw the same flag after the barrier
            }

            // ---- 2. right-hand sides and solve: thread -> (line pair g, chunk k)
            // Each line's right-hand side (I + r/2 L_cross) is formed while
            // its chunk is loaded, from the staged lines on either side
            // (ExplicitDiffusion*2ADI, src/Pde/ADIequations.cpp:19-47), plus
            // the implicit-axis Dirichlet term ImplicitBoundarySource
            // (ADIequations.h:198-220) at positions 0 and L-1.  The staged
            // lines are only read until the exchange barrier below.
            const int g = tid / P;
            const int k = tid - g * P;
            const int type = AdiBlockType(k, P);
            const float *cf = sCoef + type * kCoefTypeStride;
            const float a = p.plan.a;
            const int ll0 = g * kNL;  // first line of the thread within the CTA
            float z[kNL][M];
            bool act[kNL];
            float wUp[kNL], wDn[kNL];
            {
                const bool hasGhost = (p.ghostLo != nullptr);
#pragma unroll
                for (int j = 0; j < kNL; j++)
                {
                    const int32_t line = x0 + ll0 + j;
                    act[j] = (ll0 + j < R) && (line < p.Nlines);
                    wUp[j] = (line >= 1 || p.wrapLines) ? 1.0f : (hasGhost ? 2.0f : 0.0f);
                    wDn[j] = (line + 1 < p.Nlines || p.wrapLines) ? 1.0f : (hasGhost ? 2.0f : 0.0f);
                }
            }
            bool unit = true;  // both lines inside the grid with unit neighbour weights
#pragma unroll
            for (int j = 0; j < kNL; j++)
            {
                unit = unit && act[j] && wUp[j] == 1.0f && wDn[j] == 1.0f;
            }
            if (unit)
            {
                // the general form below with every weight 1 and every line
                // active: the same roundings (x * 1 is exact)
#pragma unroll
                for (int q = 0; q < M / 4; q++)
                {
                    float4 rows[kNL + 2];
#pragma unroll
                    for (int r = 0; r < kNL + 2; r++)
                    {
                        rows[r] = Ld4(sLines + SOff4<SWZ>(ll0 + r, k, q, P, p.LS));
                    }
#pragma unroll
                    for (int j = 0; j < kNL; j++)
                    {
                        const float4 up = rows[j], c = rows[j + 1], dn = rows[j + 2];
                        z[j][4 * q + 0] = fmaf((dn.x - c.x) + (up.x - c.x), p.halfR, c.x);
                        z[j][4 * q + 1] = fmaf((dn.y - c.y) + (up.y - c.y), p.halfR, c.y);
                        z[j][4 * q + 2] = fmaf((dn.z - c.z) + (up.z - c.z), p.halfR, c.z);
                        z[j][4 * q + 3] = fmaf((dn.w - c.w) + (up.w - c.w), p.halfR, c.w);
                    }
                }
            }
            else
#pragma unroll
            for (int q = 0; q < M / 4; q++)
            {
                // staged rows ll0 .. ll0 + kNL + 1: line ll is staged row ll + 1
                float4 rows[kNL + 2];
#pragma unroll
                for (int r = 0; r < kNL + 2; r++)
                {
                    rows[r] = (ll0 < R) ? Ld4(sLines + SOff4<SWZ>(ll0 + r, k, q, P, p.LS))
                                        : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                }
#pragma unroll
                for (int j = 0; j < kNL; j++)
                {
                    const float4 up = rows[j], c = rows[j + 1], dn = rows[j + 2];
                    // centre + (d(+1) + d(-1)) * r / 2, the differences first
                    const float4 v = make_float4(fmaf((dn.x - c.x) * wDn[j] + (up.x - c.x) * wUp[j], p.halfR, c.x),
                                                 fmaf((dn.y - c.y) * wDn[j] + (up.y - c.y) * wUp[j], p.halfR, c.y),
                                                 fmaf((dn.z - c.z) * wDn[j] + (up.z - c.z) * wUp[j], p.halfR, c.z),
                                                 fmaf((dn.w - c.w) * wDn[j] + (up.w - c.w) * wUp[j], p.halfR, c.w));
                    z[j][4 * q + 0] = act[j] ? v.x : 0.0f;
                    z[j][4 * q + 1] = act[j] ? v.y : 0.0f;
                    z[j][4 * q + 2] = act[j] ? v.z : 0.0f;
                    z[j][4 * q + 3] = act[j] ? v.w : 0.0f;
                }
            }
            if (p.implLo != nullptr)
            {
                const int lastIdx = (L - 1) - k * M;  // position L-1 within this chunk, if here
#pragma unroll
                for (int j = 0; j < kNL; j++)
                {
                    if (!act[j])
                    {
                        continue;
                    }
                    const int32_t line = x0 + ll0 + j;
                    if (k == 0)
                    {
                        z[j][0] = fmaf(p.r, __ldg(p.implLo + line), z[j][0]);
                    }
                    if (lastIdx >= 0 && lastIdx < M)
                    {
                        const float add = p.r * __ldg(p.implHi + line);
#pragma unroll
                        for (int e = 0; e < M; e++)
                        {
                            z[j][e] += (e == lastIdx) ? add : 0.0f;
                        }
                    }
                }
            }
            BlockSolveN(z, cf);
#pragma unroll
            for (int j = 0; j < kNL; j++)
            {
                if (!act[j])
                {
                    continue;
                }
                const int ll = g * kNL + j;
                if (k < P - 1)
                {
                    xA[ll * P + k] = fmaf(-a, z[j][M - 2], z[j][M - 1]);
                }
                if (k >= 1)
                {
                    xB[ll * P + k - 1] = -a * z[j][0];
                }
            }
            __syncthreads();
            float sLs[kNL], sRs[kNL];
#pragma unroll
            for (int j = 0; j < kNL; j++)
            {
                const int ll = g * kNL + j;
                sLs[j] = 0.0f;
                sRs[j] = 0.0f;
                if (act[j] && P > 1)
                {
                    switch (p.plan.B)
                    {
                    case 1:
                        BandDot2Fixed<1>(G, P, k, xA + ll * P, xB + ll * P, sLs[j], sRs[j]);
                        break;
                    case 2:
                        BandDot2Fixed<2>(G, P, k, xA + ll * P, xB + ll * P, sLs[j], sRs[j]);
                        break;
                    default:
                        BandDot2(G, P, p.plan.B, k, xA + ll * P, xB + ll * P, sLs[j], sRs[j]);
                        break;
                    }
                }
            }
            BlockCorrectN(z, cf, sLs, sRs);
#pragma unroll
            for (int j = 0; j < kNL; j++)
            {
                if (!act[j])
                {
                    continue;
                }
                const int ll = g * kNL + j;
                if (k < P - 1)
                {
                    z[j][M - 1] = sRs[j];
                }
                // every staged-line read finished before the barrier above,
                // so the line's buffer can take the solution (SolOff4's unit
                // order)
                const int swo = (k & 7) ^ SolSwz(ll);
                const int rowo = (ll + 1) * P + k;
#pragma unroll
                for (int q = 0; q < M / 4; q++)
                {
                    const int o = SWZ ? SOff4Row<SWZ>(rowo, k, q, swo, P, p.LS)
                                      : SOff4<SWZ>(ll + 1, k, q ^ SolSwz(ll), P, p.LS);
                    St4(sLines + o, make_float4(z[j][4 * q], z[j][4 * q + 1], z[j][4 * q + 2], z[j][4 * q + 3]));
                }
            }

            // write-out mapping: thread -> group qd of 4 lines; out[pos *
            // Nlines + line].  The lanes of a quarter-warp cover whole 64-byte
            // segments of the output.
            const int Q = R >> 2;  // a power of two <= 32
            const int qd = tid & (Q - 1);
            const int uStart = tid / Q;
            const int32_t line0 = x0 + 4 * qd;
            const int step = nthreads / Q;
            // 16-byte output rows; with a padded output stride the last quad
            // of the last tile may reach into the padding, which takes zeros
            // (the tensor-staged form runs dense rows only: outStride == Nlines)
            const int32_t outRow = SWZ ? p.Nlines : p.outStride;
            const bool vecOut = (outRow & 3) == 0;
            const bool quadOk = line0 < p.Nlines;
            const int32_t quadLines = p.Nlines - line0;  // lines of the quad inside the grid (4 or more: all)
            // units of 4 positions; the chunked form also writes a last,
            // partial unit (positions past L skipped), the tensor-staged one
            // has L % 256 == 0
            const int32_t nU = SWZ ? (L >> 2) : ((L + 3) >> 2);
            // units per write-out batch: the y-sweep's commit loads two units
            // ahead of the barrier; the x-sweep only stores (1: 21.18 against
            // 21.23 us per 2048^2 tick with 2, 21.56 with 4)
            constexpr int kUB = (MODE == kSweepTick) ? 2 : 1;
            const int64_t nl = outRow;
            // the commit's f and src of this thread's first write-out units,
            // loaded before the barrier so that their latency overlaps it
            // (the tensor-staged form; the register budget of the chunked
            // form has no room for them)
            constexpr bool kPre = (MODE == kSweepTick) && SWZ;
            float4 fv0[kUB][4], sv0[kUB][4];
            if constexpr (kPre)
            {
#pragma unroll
                for (int b = 0; b < kUB; b++)
                {
                    const int32_t u = uStart + b * step;
                    const bool ok = vecOut && vecL && quadOk && u < nU;
                    const int64_t g0 = static_cast<int64_t>(4 * u) * nl + line0;
#pragma unroll
                    for (int i = 0; i < 4; i++)
                    {
                        fv0[b][i] = ok ? __ldg(reinterpret_cast<const float4 *>(p.f + g0 + i * nl))
                                       : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        sv0[b][i] = (ok && p.src != nullptr) ? __ldg(reinterpret_cast<const float4 *>(p.src + g0 + i * nl))
                                                             : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    }
                }
            }
            __syncthreads();

            // ---- 2c. periodic lines: Sherman-Morrison correction -----------
            // x = y - factor * z_sm, factor = (y_0 + y_{L-1} beta/gamma) /
            // (1 + z_sm,0 + z_sm,L-1 beta/gamma) (TdmaSolver::TDMAperiodic,
            // include/Hal/Pde/TdmaSolver.h:112-119)
            if (p.plan.periodic)
            {
                float *sFactor = xA;  // the exchange rows are free now
                for (int ll = tid; ll < R; ll += nthreads)
                {
                    const float y0 = sLines[SolPos<SWZ>(ll, 0, P, p.LS)];
                    const float yl = sLines[SolPos<SWZ>(ll, L - 1, P, p.LS)];
                    sFactor[ll] = fmaf(yl, p.plan.bog, y0) * p.plan.invDenom;
                }
                __syncthreads();
                const int nUnits = P * (M / 4);
                for (int u = tid; u < nUnits; u += nthreads)
                {
                    const int kk = u >> 3;
                    const int q = u & 7;
                    float zs[4];
#pragma unroll
                    for (int e = 0; e < 4; e++)
                    {
                        const int32_t pos = 4 * u + e;
                        zs[e] = (pos < L) ? __ldg(p.plan.zsm + pos) : 0.0f;
                    }
                    for (int ll = 0; ll < R; ll++)
                    {
                        if (x0 + ll >= p.Nlines)
                        {
                            break;
                        }
                        const float fct = sFactor[ll];
                        float *at = sLines + SolOff4<SWZ>(ll, kk, q, P, p.LS);
                        float4 v = Ld4(at);
                        v.x = fmaf(-fct, zs[0], v.x);
                        v.y = fmaf(-fct, zs[1], v.y);
                        v.z = fmaf(-fct, zs[2], v.z);
                        v.w = fmaf(-fct, zs[3], v.w);
                        St4(at, v);
                    }
                }
                __syncthreads();
            }

            // ---- 3. write out ---------------------------------------------
            if constexpr (MODE == kSweepDeltas)
            {
                for (int ll = 0; ll < R; ll++)
                {
                    const int32_t line = x0 + ll;
                    if (line >= p.Nlines)
                    {
                        break;
                    }
                    const int64_t base = static_cast<int64_t>(line) * L;
                    for (int32_t pos = tid; pos < L; pos += nthreads)
                    {
                        const double v = static_cast<double>(sLines[SolPos<SWZ>(ll, pos, P, p.LS)]);
                        p.deltas[base + pos] = p.deltas[base + pos] + (v - p.f64[base + pos]);
                    }
                }
            }
            else
            {
                if (vecOut && (vecL || !SWZ))
                {
                    // 16-byte units: 4 positions x 4 lines move as a 4x4 block
                    // (4 LDS.128, a register transpose, 4 STG.128).  UPT: the
                    // commit has an uptake term (agents coupled), with the
                    // unit's counts loaded line by line (UnitCounts); without
                    // it the commit skips the count loads and that product.
                    auto writeVec = [&]() {
                        const bool hasSrc = (p.src != nullptr);
                        (void)hasSrc;  // read by the commit of MODE kSweepTick only
                        // unit u of solution line 4qd+e sits at
                        // SolOff4(4qd, u >> 3, u & 7) + e * lineStride: the
                        // four lines of a quad share one SolSwz
                        const int lineStride = SOff4<SWZ>(1, 0, 0, P, p.LS);
                        // kUB units from u0 on; PRE: their f and src are fv0/sv0
                        auto block = [&](int32_t u0, auto preTag) {
                            constexpr bool PRE = decltype(preTag)::value;
                            (void)PRE;  // read by the commit of MODE kSweepTick only
                            float4 o[kUB][4];
                            float4 fv[kUB][4], sv[kUB][4];
#pragma unroll
                            for (int b = 0; b < kUB; b++)
                            {
                                const int32_t u = u0 + b * step;
                                const bool ok = u < nU;
                                const float *su = sLines + SolOff4<SWZ>(4 * qd, u >> 3, u & 7, P, p.LS);
                                float4 a[4];
#pragma unroll
                                for (int e = 0; e < 4; e++)
                                {
                                    a[e] = ok ? Ld4(su + e * lineStride) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                                }
                                o[b][0] = make_float4(a[0].x, a[1].x, a[2].x, a[3].x);
                                o[b][1] = make_float4(a[0].y, a[1].y, a[2].y, a[3].y);
                                o[b][2] = make_float4(a[0].z, a[1].z, a[2].z, a[3].z);
                                o[b][3] = make_float4(a[0].w, a[1].w, a[2].w, a[3].w);
#pragma unroll
                                for (int i = 0; i < 4; i++)
                                {
                                    fv[b][i] = sv[b][i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                                }
                                if constexpr (MODE == kSweepTick)
                                {
                                    if constexpr (PRE && kPre)
                                    {
#pragma unroll
                                        for (int i = 0; i < 4; i++)
                                        {
                                            fv[b][i] = fv0[b][i];
                                            sv[b][i] = sv0[b][i];
                                        }
                                    }
                                    else if (ok)
                                    {
                                        const int64_t g0 = static_cast<int64_t>(4 * u) * nl + line0;
#pragma unroll
                                        for (int i = 0; i < 4; i++)
                                        {
                                            if (!SWZ && !vecL && 4 * u + i >= L)
                                            {
                                                continue;  // past the line end: no output row
                                            }
                                            fv[b][i] = __ldg(reinterpret_cast<const float4 *>(p.f + g0 + i * nl));
                                            if (hasSrc)
                                            {
                                                sv[b][i] = __ldg(reinterpret_cast<const float4 *>(p.src + g0 + i * nl));
                                            }
                                        }
                                    }
                                }
                            }
#pragma unroll
                            for (int b = 0; b < kUB; b++)
                            {
                                const int32_t u = u0 + b * step;
                                if (u >= nU)
                                {
                                    continue;
                                }
                                float *out = p.out + static_cast<int64_t>(4 * u) * nl + line0;
                                // per-agent uptake counts of the unit's 4 lines x 4 positions
                                int32_t nc[4][4] = {};
                                (void)nc;  // read by the commit of MODE kSweepTick only
                                if constexpr (UPT)
                                {
                                    UnitCounts(p.cellOffsets, line0, quadLines, u, L, vecL, nc);
                                }
#pragma unroll
                                for (int i = 0; i < 4; i++)
                                {
                                    float4 w4 = o[b][i];
                                    if constexpr (MODE == kSweepTick)
                                    {
                                        const int32_t n0 = nc[0][i], n1 = nc[1][i], n2 = nc[2][i], n3 = nc[3][i];
                                        // f' = f + ((v - f) - decay f + src - uptake n f)
                                        auto commit = [&](float vv, float f0, float s0, int32_t nv) {
                                            float d = vv - f0;
                                            d = fmaf(f0, p.negDecay, d);
                                            d += s0;
                                            if constexpr (UPT)
                                            {
                                                d = fmaf(f0, p.negUptake * static_cast<float>(nv), d);
                                            }
                                            return f0 + d;
                                        };
                                        w4.x = commit(w4.x, fv[b][i].x, sv[b][i].x, n0);
                                        w4.y = commit(w4.y, fv[b][i].y, sv[b][i].y, n1);
                                        w4.z = commit(w4.z, fv[b][i].z, sv[b][i].z, n2);
                                        w4.w = commit(w4.w, fv[b][i].w, sv[b][i].w, n3);
                                    }
                                    if constexpr (!SWZ)
                                    {
                                        if (!vecL && 4 * u + i >= L)
                                        {
                                            continue;  // past the line end: no output row
                                        }
                                        if (quadLines < 4)
                                        {
                                            // lines past the grid: the row's padding, zeros
                                            w4.y = (quadLines > 1) ? w4.y : 0.0f;
                                            w4.z = (quadLines > 2) ? w4.z : 0.0f;
                                            w4.w = 0.0f;
                                        }
                                    }
                                    St4(out + i * nl, w4);
                                }
                            }
                        };
                        if constexpr (kPre)
                        {
                            // exactly four units per thread (the thread-capped
                            // shapes, e.g. 16 lines of 2048): a rotating
                            // pipeline whose loads run one unit ahead
                            if (quadOk && uStart + 3 * step < nU && uStart + 4 * step >= nU)
                            {
                                auto loadFS = [&](int32_t u, float4(&fo)[4], float4(&so)[4]) {
                                    const int64_t g0 = static_cast<int64_t>(4 * u) * nl + line0;
#pragma unroll
                                    for (int i = 0; i < 4; i++)
                                    {
                                        fo[i] = __ldg(reinterpret_cast<const float4 *>(p.f + g0 + i * nl));
                                        so[i] = hasSrc ? __ldg(reinterpret_cast<const float4 *>(p.src + g0 + i * nl))
                                                       : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                                    }
                                };
                                auto unitOut = [&](int32_t u, const float4(&fi)[4], const float4(&si)[4]) {
                                    const float *su = sLines + SolOff4<SWZ>(4 * qd, u >> 3, u & 7, P, p.LS);
                                    float4 a[4];
#pragma unroll
                                    for (int e = 0; e < 4; e++)
                                    {
                                        a[e] = Ld4(su + e * lineStride);
                                    }
                                    const float4 o[4] = {make_float4(a[0].x, a[1].x, a[2].x, a[3].x),
                                                         make_float4(a[0].y, a[1].y, a[2].y, a[3].y),
                                                         make_float4(a[0].z, a[1].z, a[2].z, a[3].z),
                                                         make_float4(a[0].w, a[1].w, a[2].w, a[3].w)};
                                    float *out = p.out + static_cast<int64_t>(4 * u) * nl + line0;
                                    int32_t nc[4][4] = {};
                                    if constexpr (UPT)
                                    {
                                        UnitCounts(p.cellOffsets, line0, quadLines, u, L, vecL, nc);
                                    }
#pragma unroll
                                    for (int i = 0; i < 4; i++)
                                    {
                                        const int32_t n0 = nc[0][i], n1 = nc[1][i], n2 = nc[2][i], n3 = nc[3][i];
                                        auto commit = [&](float vv, float f0, float s0, int32_t nv) {
                                            float d = vv - f0;
                                            d = fmaf(f0, p.negDecay, d);
                                            d += s0;
                                            if constexpr (UPT)
                                            {
                                                d = fmaf(f0, p.negUptake * static_cast<float>(nv), d);
                                            }
                                            return f0 + d;
                                        };
                                        float4 w4 = o[i];
                                        w4.x = commit(w4.x, fi[i].x, si[i].x, n0);
                                        w4.y = commit(w4.y, fi[i].y, si[i].y, n1);
                                        w4.z = commit(w4.z, fi[i].z, si[i].z, n2);
                                        w4.w = commit(w4.w, fi[i].w, si[i].w, n3);
                                        St4(out + i * nl, w4);
                                    }
                                };
                                float4 fC[4], sC[4], fD[4], sD[4];
                                unitOut(uStart, fv0[0], sv0[0]);
                                loadFS(uStart + 2 * step, fC, sC);
                                unitOut(uStart + step, fv0[1], sv0[1]);
                                loadFS(uStart + 3 * step, fD, sD);
                                unitOut(uStart + 2 * step, fC, sC);
                                unitOut(uStart + 3 * step, fD, sD);
                                return;
                            }
                        }
                        int32_t uFirst = uStart;
                        if constexpr (kPre)
                        {
                            if (quadOk && uStart < nU)
                            {
                                block(uStart, std::true_type{});
                            }
                            uFirst += kUB * step;
                        }
                        for (int32_t u0 = uFirst; u0 < nU && quadOk; u0 += kUB * step)
                        {
                            block(u0, std::false_type{});
                        }
                    };
                    writeVec();
                    return;
                }
                constexpr int kBatch = 2;
                for (int32_t pos0 = uStart; pos0 < L && quadOk; pos0 += kBatch * step)
                {
                    float4 v[kBatch], fv[kBatch], sv[kBatch];
                    int32_t nn[kBatch][4];
#pragma unroll
                    for (int b = 0; b < kBatch; b++)
                    {
                        const int32_t pos = pos0 + b * step;
                        v[b] = fv[b] = sv[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        nn[b][0] = nn[b][1] = nn[b][2] = nn[b][3] = 0;
                        if (pos < L)
                        {
                            v[b] = make_float4(sLines[SolPos<SWZ>(4 * qd, pos, P, p.LS)],
                                               sLines[SolPos<SWZ>(4 * qd + 1, pos, P, p.LS)],
                                               sLines[SolPos<SWZ>(4 * qd + 2, pos, P, p.LS)],
                                               sLines[SolPos<SWZ>(4 * qd + 3, pos, P, p.LS)]);
                            if constexpr (MODE == kSweepTick)
                            {
                                const int64_t gi = static_cast<int64_t>(pos) * outRow + line0;
                                if (vecOut)
                                {
                                    fv[b] = __ldg(reinterpret_cast<const float4 *>(p.f + gi));
                                    if (p.src != nullptr)
                                    {
                                        sv[b] = __ldg(reinterpret_cast<const float4 *>(p.src + gi));
                                    }
                                }
                                else
                                {
                                    float tf[4] = {0, 0, 0, 0}, ts[4] = {0, 0, 0, 0};
#pragma unroll
                                    for (int e = 0; e < 4; e++)
                                    {
                                        if (line0 + e < p.Nlines)
                                        {
                                            tf[e] = __ldg(p.f + gi + e);
                                            ts[e] = (p.src != nullptr) ? __ldg(p.src + gi + e) : 0.0f;
                                        }
                                    }
                                    fv[b] = make_float4(tf[0], tf[1], tf[2], tf[3]);
                                    sv[b] = make_float4(ts[0], ts[1], ts[2], ts[3]);
                                }
                                if (p.cellOffsets != nullptr)
                                {
#pragma unroll
                                    for (int e = 0; e < 4; e++)
                                    {
                                        if (line0 + e < p.Nlines)
                                        {
                                            const int64_t ci = static_cast<int64_t>(line0 + e) * L + pos;
                                            nn[b][e] = __ldg(p.cellOffsets + ci + 1) - __ldg(p.cellOffsets + ci);
                                        }
                                    }
                                }
                            }
                        }
                    }
#pragma unroll
                    for (int b = 0; b < kBatch; b++)
                    {
                        const int32_t pos = pos0 + b * step;
                        if (pos >= L)
                        {
                            continue;
                        }
                        float4 o = v[b];
                        if constexpr (MODE == kSweepTick)
                        {
                            auto commit = [&](float vv, float f0, float s0, int32_t n0) {
                                float d = vv - f0;
                                d = fmaf(f0, p.negDecay, d);
                                d += s0;
                                d = fmaf(f0, p.negUptake * static_cast<float>(n0), d);
                                return f0 + d;
                            };
                            o.x = commit(v[b].x, fv[b].x, sv[b].x, nn[b][0]);
                            o.y = commit(v[b].y, fv[b].y, sv[b].y, nn[b][1]);
                            o.z = commit(v[b].z, fv[b].z, sv[b].z, nn[b][2]);
                            o.w = commit(v[b].w, fv[b].w, sv[b].w, nn[b][3]);
                        }
                        const int64_t gi = static_cast<int64_t>(pos) * outRow + line0;
                        if (vecOut)
                        {
                            St4(p.out + gi, o);
                        }
                        else
                        {
                            const float t[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
                            for (int e = 0; e < 4; e++)
                            {
                                if (line0 + e < p.Nlines)
                                {
                                    p.out[gi + e] = t[e];
                                }
                            }
                        }
                    }
                }
            }
        }

        template <int MODE, bool SWZ, bool UPT = false>
        __global__ void __launch_bounds__(kMaxThreads)
            AdiSweep(SweepParams p, const __grid_constant__ CUtensorMap tmap)
        {
            SweepTile<MODE, SWZ, UPT>(p, &tmap, static_cast<int32_t>(blockIdx.x) * p.R);
        }

        // Batched form: CTA b runs tile tiles[b] = (grid, first line) of the
        // table's grids, with the 36-float chunk staging (no tensor map).
        template <int MODE>
        __global__ void __launch_bounds__(kMaxThreads)
            AdiSweepTiles(const SweepParams *__restrict__ table, const int2 *__restrict__ tiles)
        {
            const int2 t = tiles[blockIdx.x];
            SweepTile<MODE, false>(table[t.x], nullptr, t.y);
        }

        // out[c][r] = in[r][c] for an rows x cols matrix (32x32 tiles).
        template <typename TIn>
        __global__ void Transpose(const TIn *__restrict__ in, float *__restrict__ out, int32_t rows, int32_t cols,
                                  int32_t inStride, int32_t outStride)
        {
            __shared__ float tile[32][33];
            const int32_t c0 = blockIdx.x * 32;
            const int32_t r0 = blockIdx.y * 32;
            for (int j = threadIdx.y; j < 32; j += blockDim.y)
            {
                const int32_t r = r0 + j;
                const int32_t c = c0 + threadIdx.x;
                if (r < rows && c < cols)
                {
                    tile[j][threadIdx.x] = static_cast<float>(in[static_cast<int64_t>(r) * inStride + c]);
                }
            }
            __syncthreads();
            for (int j = threadIdx.y; j < 32; j += blockDim.y)
            {
                const int32_t c = c0 + j;
                const int32_t r = r0 + threadIdx.x;
                if (r < rows && c < cols)
                {
                    out[static_cast<int64_t>(c) * outStride + r] = tile[threadIdx.x][j];
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

        // Launch shape of a sweep over lines of length L: lines per CTA R (a
        // power of two >= 8, so the transposed stores cover whole 32-byte
        // sectors), threads = (R / kNL) * P.  swz: the staged lines use the
        // 128-byte-swizzled tensor layout (L % 256 == 0).
        struct SweepShape
        {
            int32_t R, threads, LS;
            size_t smem;
        };

        SweepShape ShapeFor(int32_t P, int32_t Nlines, bool swz)
        {
            SweepShape s;
            // The largest power of two (<= kMaxR, <= 1024/P threads-wise)
            // that still gives enough CTAs to cover the SMs: longer line
            // groups make the transposed stores longer contiguous segments.
            int32_t R = 8;
            while (R * 2 <= 1024 / P && R * 2 <= kMaxR && (Nlines + 2 * R - 1) / (2 * R) >= 120)
            {
                R *= 2;
            }
            s.R = R;
            s.threads = ((R / kNL) * P + 31) & ~31;
            s.LS = swz ? P * M : P * kChunkStride + 4;  // padded: lines 4 mod 32 banks apart
            s.smem = 1024 + sizeof(float) * (static_cast<size_t>(kCoefSmemFloats) + kGbandSmem + static_cast<size_t>(R + 2) * s.LS +
                                             2 * static_cast<size_t>(R) * P + 2 * static_cast<size_t>(R));
            return s;
        }

        template <int MODE, bool SWZ, bool UPT = false>
        int EnableSweepSmem(size_t bytes)
        {
            static SmemLimit s_limit;
            return s_limit.Ensure(AdiSweep<MODE, SWZ, UPT>, bytes, "cudaFuncSetAttribute(AdiSweep)");
        }

        template <int MODE>
        int EnableSweepSmemBoth(int32_t P, int32_t Nlines)
        {
            HAL_TRY((EnableSweepSmem<MODE, true>(ShapeFor(P, Nlines, true).smem)));
            HAL_TRY((EnableSweepSmem<MODE, false>(ShapeFor(P, Nlines, false).smem)));
            if constexpr (MODE == kSweepTick)
            {
                HAL_TRY((EnableSweepSmem<MODE, true, true>(ShapeFor(P, Nlines, true).smem)));
                HAL_TRY((EnableSweepSmem<MODE, false, true>(ShapeFor(P, Nlines, false).smem)));
            }
            return HAL_CUDA_OK;
        }

        // cuTensorMapEncodeTiled through the runtime's driver entry point.
        PFN_cuTensorMapEncodeTiled_v12000 TensorMapEncoder()
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

        // Tensor map over Nlines lines of L floats (L % 256 == 0) seen as
        // [line][chunk][32], box = (R+2) lines x P chunks x 32, 128-byte
        // swizzle, zero fill outside the tensor.
        bool MakeLineTensorMap(CUtensorMap &map, const float *base, int32_t L, int32_t Nlines, int32_t R)
        {
            PFN_cuTensorMapEncodeTiled_v12000 enc = TensorMapEncoder();
            if (enc == nullptr || (L % (8 * M)) != 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0)
            {
                return false;
            }
            const cuuint64_t P = static_cast<cuuint64_t>(L / M);
            cuuint64_t gdim[3] = {static_cast<cuuint64_t>(M), P, static_cast<cuuint64_t>(Nlines)};
            cuuint64_t gstride[2] = {static_cast<cuuint64_t>(M) * 4u, static_cast<cuuint64_t>(L) * 4u};
            cuuint32_t box[3] = {static_cast<cuuint32_t>(M), static_cast<cuuint32_t>(P), static_cast<cuuint32_t>(R + 2)};
            cuuint32_t estr[3] = {1, 1, 1};
            CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), gdim, gstride, box,
                             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            return r == CUDA_SUCCESS;
        }
    }
}

namespace halcuda
{
    static_assert(kSweepTileThreads == kMaxThreads, "batched sweep CTAs use the kernel's thread bound");
    static_assert(kSweepTileMaxR == kMaxR, "batched sweep tiles use the kernel's line bound");

    SweepTileShape SweepTileShapeFor(int32_t P, int32_t rCap, int32_t budget)
    {
        // as many lines as (R / kNL) * P <= budget threads allow, a power of
        // two in [8, min(rCap, kMaxR)]
        budget = std::min(budget, kSweepTileThreads);
        SweepTileShape sh;
        int32_t R = 8;
        while (R * 2 <= kMaxR && R * 2 <= rCap && (R * 2 / kNL) * P <= budget)
        {
            R *= 2;
        }
        sh.R = R;
        sh.threads = ((R / kNL) * P + 31) & ~31;
        sh.LS = P * kChunkStride + 4;
        sh.smem = 1024 + sizeof(float) * (static_cast<size_t>(kCoefSmemFloats) + kGbandSmem + static_cast<size_t>(R + 2) * sh.LS +
                                          2 * static_cast<size_t>(R) * P + 2 * static_cast<size_t>(R));
        return sh;
    }

    namespace
    {
        template <int MODE>
        int PrepareTiles(size_t smem)
        {
            static SmemLimit s_limit;
            return s_limit.Ensure(AdiSweepTiles<MODE>, smem, "cudaFuncSetAttribute(AdiSweepTiles)");
        }

        template <int MODE>
        int LaunchTiles(const SweepParams *table, const int2 *tiles, int32_t nTiles, size_t smem, int32_t threads,
                        cudaStream_t s)
        {
            AdiSweepTiles<MODE><<<static_cast<unsigned>(nTiles), static_cast<unsigned>(threads), smem, s>>>(table,
                                                                                                       tiles);
            CountLaunch();
            return LaunchStatus("AdiSweepTiles");
        }
    }

    int PrepareSweepTiles(int mode, size_t smem)
    {
        switch (mode)
        {
        case kSweepW:
            return PrepareTiles<kSweepW>(smem);
        case kSweepTick:
            return PrepareTiles<kSweepTick>(smem);
        default:
            SetError("PrepareSweepTiles: unsupported mode %d", mode);
            return HAL_CUDA_EINVAL;
        }
    }

    AdiDevicePlan::~AdiDevicePlan()
    {
        cudaFree(m_pCoef);
        cudaFree(m_pGband);
        cudaFree(m_pZsm);
    }

    int AdiDevicePlan::Build(int32_t L, double r, int ends)
    {
        AdiLinePlanHost h;
        if (!BuildAdiLinePlan(L, r, ends, h))
        {
            SetError("ADI line length %d outside [1, %d]", L, HAL_CUDA_ADI_MAX_LINE);
            return HAL_CUDA_ENOTSUP;
        }
        if (!(h.selfCheck < 1e-5))
        {
            SetError("ADI plan self-check failed (L=%d, r=%g, rel err %g)", L, r, h.selfCheck);
            return HAL_CUDA_ENOTSUP;
        }
        auto upload = [](const std::vector<float> &v, float **dst) {
            if (v.empty())
            {
                return HAL_CUDA_OK;
            }
            HAL_TRY(CudaStatus(cudaMalloc(reinterpret_cast<void **>(dst), v.size() * sizeof(float)), "cudaMalloc(plan)"));
            return CudaStatus(cudaMemcpy(*dst, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice),
                              "cudaMemcpy(plan)");
        };
        HAL_TRY(upload(h.coef, &m_pCoef));
        HAL_TRY(upload(h.gband, &m_pGband));
        HAL_TRY(upload(h.zsm, &m_pZsm));
        m_dev = {};
        m_dev.L = h.L;
        m_dev.P = h.P;
        m_dev.B = h.B;
        m_dev.periodic = (ends == kEndsPeriodic) ? 1 : 0;
        m_dev.nlast = h.L - (h.P - 1) * kAdiM;
        m_dev.a = static_cast<float>(h.offDiag);
        m_dev.coef = m_pCoef;
        m_dev.gband = m_pGband;
        m_dev.zsm = m_pZsm;
        m_dev.bog = static_cast<float>(h.betaOverGamma);
        m_dev.invDenom = static_cast<float>(h.invDenom);
        return HAL_CUDA_OK;
    }

    int LaunchTranspose(const float *in, float *out, int32_t rows, int32_t cols, cudaStream_t s)
    {
        return LaunchTransposeStrided(in, cols, out, rows, rows, cols, s);
    }

    int LaunchTransposeStrided(const float *in, int32_t inStride, float *out, int32_t outStride, int32_t rows,
                               int32_t cols, cudaStream_t s)
    {
        dim3 block(32, 8);
        dim3 grid((cols + 31) / 32, (rows + 31) / 32);
        Transpose<float><<<grid, block, 0, s>>>(in, out, rows, cols, inStride, outStride);
        CountLaunch();
        return LaunchStatus("Transpose launch");
    }

    int LaunchSweepTiles(int mode, const SweepParams *table, const int2 *tiles, int32_t nTiles, size_t smem,
                         int32_t threads, cudaStream_t s)
    {
        if (nTiles <= 0)
        {
            return HAL_CUDA_OK;
        }
        if (threads < 32 || threads > kSweepTileThreads || threads % 32 != 0)
        {
            SetError("LaunchSweepTiles: %d threads per tile CTA (a multiple of 32 up to %d)", threads,
                     kSweepTileThreads);
            return HAL_CUDA_EINVAL;
        }
        switch (mode)
        {
        case kSweepW:
            return LaunchTiles<kSweepW>(table, tiles, nTiles, smem, threads, s);
        case kSweepTick:
            return LaunchTiles<kSweepTick>(table, tiles, nTiles, smem, threads, s);
        default:
            SetError("LaunchSweepTiles: unsupported mode %d", mode);
            return HAL_CUDA_EINVAL;
        }
    }
}

namespace halcuda
{
    struct Adi
    {
        int32_t xDim = 0, yDim = 0;
        int device = 0;
        StreamSlot stream;
        DevBuf<float> field[2];  // layout B (y*xDim + x)
        int cur = 0;
        DevBuf<float> w;         // x-sweep output, layout A; also staging for uploads
        DevBuf<float> src;       // layout B
        bool hasSrc = false;
        DevBuf<float> ghost;     // ghost table (hal_cuda.h layout)
        bool hasGhost = false;
        DevBuf<double> f64, d64;
        DevBuf<float> g32;       // ghost table of the FP64 interface call, in float
        // the interface calls on lines longer than the FP32 partitioned solve
        // takes: the FP64 Thomas solve per line, with its ghost table in FP64
        std::unique_ptr<Adi64> adi64;
        DevBuf<double> g64;
        bool exact = false;      // hal_cuda_adi_set_exact: the FP64 solve at every size
        DevBuf<int32_t> err;
        // set once a bounded device wait has given up: the sweep that gave
        // up left its lines undefined, so the handle takes no further ticks
        bool stopped = false;
        const hal_cuda_agents *agents = nullptr;
        double uptake = 0.0;
        std::map<std::string, std::unique_ptr<LinePlanBuf>> plans;
        GraphCache graph[2];  // by the parity of the starting buffer
        GraphCache coupled[2];          // coupled agent + ADI ticks, by parity
        int64_t coupledLaunches[2] = {0, 0};  // kernel launches per replay
        // TMA tensor maps of the staged lines: x-sweep input field[0] /
        // field[1] (lines along x), y-sweep input w (lines along y)
        CUtensorMap tmapX[2];
        CUtensorMap tmapY;
        bool swzX = false, swzY = false;

        void ResetGraphs()
        {
            graph[0].Reset();
            graph[1].Reset();
            coupled[0].Reset();
            coupled[1].Reset();
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
            HAL_TRY(err.Alloc(1, "cudaMalloc(err)"));
            HAL_TRY(CudaStatus(cudaMemset(field[0].p, 0, n * sizeof(float)), "cudaMemset"));
            HAL_TRY(CudaStatus(cudaMemset(err.p, 0, sizeof(int32_t)), "cudaMemset"));
            std::memset(tmapX, 0, sizeof(tmapX));
            std::memset(&tmapY, 0, sizeof(tmapY));
            const int32_t Px = (xDim + M - 1) / M, Py = (yDim + M - 1) / M;
            const int32_t Rx = ShapeFor(Px, yDim, true).R, Ry = ShapeFor(Py, xDim, true).R;
            swzX = MakeLineTensorMap(tmapX[0], field[0].p, xDim, yDim, Rx) &&
                   MakeLineTensorMap(tmapX[1], field[1].p, xDim, yDim, Rx);
            swzY = MakeLineTensorMap(tmapY, w.p, yDim, xDim, Ry);
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
                    // plans captured in the cached graphs may be freed
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

        // Checks (and clears) the device error flag of the bounded waits.
        int CheckDeviceError(const char *who)
        {
            int32_t h = 0;
            HAL_TRY(CudaStatus(cudaMemcpyAsync(&h, err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, stream.Get()),
                               "cudaMemcpy(err)"));
            HAL_TRY(CudaStatus(cudaStreamSynchronize(stream.Get()), who));
            if (h != 0)
            {
                cudaMemsetAsync(err.p, 0, sizeof(int32_t), stream.Get());
                stopped = true;
                SetError(h == 2   ? "%s: the sweep's shared-memory buffer was not 1024-byte aligned"
                         : h == 3 ? "%s: a sweep tile's lines or shared memory exceed its launch (internal error)"
                                  : "%s: a staged copy did not complete within its wait limit",
                         who);
                return HAL_CUDA_ETIMEOUT;
            }
            return HAL_CUDA_OK;
        }

        // Refuses work on a handle whose device wait has given up before.
        int Usable(const char *who) const
        {
            if (stopped)
            {
                SetError("%s: the handle stopped after a sweep gave up waiting for its staged lines; its field is "
                         "undefined: destroy the handle and create a new one",
                         who);
                return HAL_CUDA_ETIMEOUT;
            }
            return HAL_CUDA_OK;
        }

        template <typename TIn>
        int TransposeTo(const TIn *in, float *out, int32_t rows, int32_t cols, cudaStream_t s)
        {
            dim3 block(32, 8);
            dim3 grid((cols + 31) / 32, (rows + 31) / 32);
            Transpose<TIn><<<grid, block, 0, s>>>(in, out, rows, cols, cols, rows);
            CountLaunch();
            return LaunchStatus("Transpose launch");
        }

        template <int MODE>
        int LaunchSweep(SweepParams &p, cudaStream_t s, const CUtensorMap *tmap)
        {
            const bool swz = (tmap != nullptr);
            // the single grid's lines and output rows are dense
            p.inStride = p.L;
            p.outStride = p.Nlines;
            SweepShape sh = ShapeFor(p.plan.P, p.Nlines, swz);
            p.R = sh.R;
            p.LS = sh.LS;
            unsigned blocks = static_cast<unsigned>((p.Nlines + sh.R - 1) / sh.R);
            auto launch = [&](auto uptTag) -> int {
                constexpr bool UPT = decltype(uptTag)::value;
                if (swz)
                {
                    HAL_TRY((EnableSweepSmem<MODE, true, UPT>(sh.smem)));
                    AdiSweep<MODE, true, UPT><<<blocks, sh.threads, sh.smem, s>>>(p, *tmap);
                }
                else
                {
                    CUtensorMap none;
                    std::memset(&none, 0, sizeof(none));
                    HAL_TRY((EnableSweepSmem<MODE, false, UPT>(sh.smem)));
                    AdiSweep<MODE, false, UPT><<<blocks, sh.threads, sh.smem, s>>>(p, none);
                }
                return HAL_CUDA_OK;
            };
            if constexpr (MODE == kSweepTick)
            {
                if (p.cellOffsets != nullptr)
                {
                    HAL_TRY(launch(std::true_type{}));
                }
                else
                {
                    HAL_TRY(launch(std::false_type{}));
                }
            }
            else
            {
                HAL_TRY(launch(std::false_type{}));
            }
            CountLaunch();
            return LaunchStatus("AdiSweep launch");
        }

        // x-sweep: lines along x (layout B input), w out in layout A.
        int LaunchX(const float *fB, double r, bool wrapX, bool wrapY, const float *ghostTab, cudaStream_t s)
        {
            HAL_TRY(Usable("ADI x-sweep"));
            const LinePlanDev *pl = nullptr;
            const int ends = wrapX ? kEndsPeriodic : (ghostTab ? kEndsDirichlet : kEndsZeroFlux);
            HAL_TRY(Plan(xDim, r, ends, &pl));
            GhostView gv = MakeGhostView(ghostTab, xDim, yDim);
            SweepParams p = {};
            p.in = fB;
            p.L = xDim;
            p.Nlines = yDim;
            p.wrapLines = wrapY;
            p.ghostLo = (!wrapY) ? gv.ylo : nullptr;  // bc(x, -1) for every x
            p.ghostHi = (!wrapY) ? gv.yhi : nullptr;
            p.implLo = (!wrapX) ? gv.xlo : nullptr;   // bc(-1, y) for every line y
            p.implHi = (!wrapX) ? gv.xhi : nullptr;
            p.halfR = static_cast<float>(r / 2.0);
            p.r = static_cast<float>(r);
            p.plan = *pl;
            p.out = w.p;
            p.err = err.p;
            const CUtensorMap *tm = nullptr;
            if (swzX)
            {
                tm = (fB == field[0].p) ? &tmapX[0] : ((fB == field[1].p) ? &tmapX[1] : nullptr);
            }
            return LaunchSweep<kSweepW>(p, s, tm);
        }

        // y-sweep: lines along y (w in layout A).
        template <int MODE>
        int LaunchY(float *outB, const float *fB, const double *f64, double *deltas, double r, double decay,
                    bool wrapX, bool wrapY, const float *ghostTab, bool extras, cudaStream_t s)
        {
            const LinePlanDev *pl = nullptr;
            const int ends = wrapY ? kEndsPeriodic : (ghostTab ? kEndsDirichlet : kEndsZeroFlux);
            HAL_TRY(Plan(yDim, r, ends, &pl));
            GhostView gv = MakeGhostView(ghostTab, xDim, yDim);
            SweepParams p = {};
            p.in = w.p;
            p.L = yDim;
            p.Nlines = xDim;
            p.wrapLines = wrapX;
            p.ghostLo = (!wrapX) ? gv.xlo : nullptr;  // bc(-1, y) for every y
            p.ghostHi = (!wrapX) ? gv.xhi : nullptr;
            p.implLo = (!wrapY) ? gv.ylo : nullptr;   // bc(x, -1) for every line x
            p.implHi = (!wrapY) ? gv.yhi : nullptr;
            p.halfR = static_cast<float>(r / 2.0);
            p.r = static_cast<float>(r);
            p.plan = *pl;
            p.out = outB;
            p.f = fB;
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
            p.f64 = f64;
            p.deltas = deltas;
            p.err = err.p;
            return LaunchSweep<MODE>(p, s, swzY ? &tmapY : nullptr);
        }

        // Sets the shared-memory limits of both sweeps before a graph
        // capture (the attribute call is not a stream operation).
        int PrepareShapes(double r, bool wrapX, bool wrapY, const float *g)
        {
            const LinePlanDev *px = nullptr, *py = nullptr;
            HAL_TRY(Plan(xDim, r, wrapX ? kEndsPeriodic : (g ? kEndsDirichlet : kEndsZeroFlux), &px));
            HAL_TRY(Plan(yDim, r, wrapY ? kEndsPeriodic : (g ? kEndsDirichlet : kEndsZeroFlux), &py));
            HAL_TRY(EnableSweepSmemBoth<kSweepW>(px->P, yDim));
            HAL_TRY(EnableSweepSmemBoth<kSweepTick>(py->P, xDim));
            HAL_TRY(EnableSweepSmemBoth<kSweepPlain>(py->P, xDim));
            return HAL_CUDA_OK;
        }

        int EnqueueTick(int c, double r, double decay, bool wrapX, bool wrapY, bool plain, cudaStream_t s)
        {
            const float *g = (!plain && hasGhost) ? ghost.p : nullptr;
            HAL_TRY(LaunchX(field[c].p, r, wrapX, wrapY, g, s));
            if (plain)
            {
                return LaunchY<kSweepPlain>(field[c ^ 1].p, field[c].p, nullptr, nullptr, r, decay, wrapX, wrapY,
                                            nullptr, false, s);
            }
            return LaunchY<kSweepTick>(field[c ^ 1].p, field[c].p, nullptr, nullptr, r, decay, wrapX, wrapY, g,
                                       true, s);
        }

        int RunTicks(int32_t ticks, double r, double decay, bool wrapX, bool wrapY, bool plain)
        {
            HAL_TRY(Usable("ADI ticks"));
            if (ticks <= 0)
            {
                return HAL_CUDA_OK;
            }
            cudaStream_t s = stream.Get();
            const float *g = (!plain && hasGhost) ? ghost.p : nullptr;
            HAL_TRY(PrepareShapes(r, wrapX, wrapY, g));
            char key[256];
            snprintf(key, sizeof(key), "%d|%a|%a|%d|%d|%d|%d|%d|%p|%p|%a", ticks, r, decay, wrapX, wrapY,
                     plain ? 1 : 0, hasSrc, hasGhost, static_cast<void *>(s), static_cast<const void *>(agents),
                     uptake);
            GraphCache &graph = this->graph[cur];
            if (graph.exec == nullptr || graph.key != key)
            {
                graph.Reset();
                cudaGraph_t gr = nullptr;
                HAL_TRY(CudaStatus(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                                   "cudaStreamBeginCapture"));
                int c = cur;
                int rc = HAL_CUDA_OK;
                for (int32_t t = 0; t < ticks && rc == HAL_CUDA_OK; t++)
                {
                    rc = EnqueueTick(c, r, decay, wrapX, wrapY, plain, s);
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

        // `ticks` coupled ticks on the handle's stream, each the agents'
        // resident step (bins, forces, move) and then the ADI tick whose
        // commit takes up the field per agent of those bins; replayed from a
        // CUDA graph cached per buffer parity.  Every replay starts from the
        // agents' precounted bins (CoupledStepBegin) and leaves them so.
        int RunCoupled(hal_cuda_agents *ag, int32_t ticks, double r, double decay, bool wrapX, bool wrapY,
                       const CoupledStep &st)
        {
            HAL_TRY(Usable("ADI coupled ticks"));
            if (ticks <= 0)
            {
                return HAL_CUDA_OK;
            }
            cudaStream_t s = stream.Get();
            const float *g = hasGhost ? ghost.p : nullptr;
            HAL_TRY(PrepareShapes(r, wrapX, wrapY, g));
            HAL_TRY(CoupledStepBegin(ag, st, s));
            char key[384];
            snprintf(key, sizeof(key), "%d|%a|%a|%d|%d|%d|%d|%p|%p|%a|%d|%a|%a|%a|%a", ticks, r, decay, wrapX, wrapY,
                     hasSrc, hasGhost, static_cast<void *>(s), static_cast<const void *>(ag), uptake,
                     CoupledAgentCount(ag), st.interactionRad, st.springConstant, st.friction, st.maxVel);
            GraphCache &gc = coupled[cur];
            if (gc.exec == nullptr || gc.key != key)
            {
                gc.Reset();
                const int64_t l0 = g_launches.load();
                cudaGraph_t gr = nullptr;
                HAL_TRY(CudaStatus(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                                   "cudaStreamBeginCapture"));
                int c = cur;
                int rc = HAL_CUDA_OK;
                for (int32_t t = 0; t < ticks && rc == HAL_CUDA_OK; t++)
                {
                    rc = CoupledStepOnce(ag, st, wrapX, wrapY, s);
                    if (rc == HAL_CUDA_OK)
                    {
                        rc = EnqueueTick(c, r, decay, wrapX, wrapY, false, s);
                    }
                    c ^= 1;
                }
                cudaError_t e = cudaStreamEndCapture(s, &gr);
                if (rc == HAL_CUDA_OK && !CoupledBinsPrecounted(ag))
                {
                    SetError("hal_cuda_adi_run_coupled: the agent steps did not leave their bins counted");
                    rc = HAL_CUDA_EDEVICE;
                }
                if (rc != HAL_CUDA_OK)
                {
                    if (gr != nullptr)
                    {
                        cudaGraphDestroy(gr);
                    }
                    return rc;
                }
                HAL_TRY(CudaStatus(e, "cudaStreamEndCapture"));
                e = cudaGraphInstantiate(&gc.exec, gr, 0);
                cudaGraphDestroy(gr);
                HAL_TRY(CudaStatus(e, "cudaGraphInstantiate"));
                gc.key = key;
                coupledLaunches[cur] = g_launches.load() - l0;  // counted at capture for this first launch
            }
            else
            {
                CountLaunch(coupledLaunches[cur]);
            }
            HAL_TRY(CudaStatus(cudaGraphLaunch(gc.exec, s), "cudaGraphLaunch"));
            cur ^= (ticks & 1);
            return CoupledStepEnd(ag, s);
        }

        // The device address of a host buffer the GPU reads and writes in
        // place (pinned: cudaHostAlloc, cudaMallocHost or cudaHostRegister), or
        // null for pageable memory.  The transposes then move the data across
        // the host link themselves: 85 us for 16.8 MB against 93 us for a copy
        // plus a device transpose (GB300, NVLink-C2C).
        static void *MappedHost(const void *host)
        {
            cudaPointerAttributes a;
            if (cudaPointerGetAttributes(&a, host) != cudaSuccess)
            {
                cudaGetLastError();  // not a pointer CUDA knows: take the copy path
                return nullptr;
            }
            return (a.type == cudaMemoryTypeHost) ? a.devicePointer : nullptr;
        }

        // Host field (layout A) -> field[cur] (layout B).
        int Upload(const float *host, cudaStream_t s)
        {
            if (const void *d = MappedHost(host))
            {
                return TransposeTo<float>(static_cast<const float *>(d), field[cur].p, xDim, yDim, s);
            }
            HAL_TRY(CudaStatus(cudaMemcpyAsync(w.p, host, Length() * sizeof(float), cudaMemcpyHostToDevice, s),
                               "cudaMemcpy(field)"));
            return TransposeTo<float>(w.p, field[cur].p, xDim, yDim, s);
        }

        // field[cur] (layout B) -> host (layout A).
        int Download(float *host, cudaStream_t s)
        {
            if (void *d = MappedHost(host))
            {
                return TransposeTo<float>(field[cur].p, static_cast<float *>(d), yDim, xDim, s);
            }
            HAL_TRY(TransposeTo<float>(field[cur].p, w.p, yDim, xDim, s));
            return CudaStatus(cudaMemcpyAsync(host, w.p, Length() * sizeof(float), cudaMemcpyDeviceToHost, s),
                              "cudaMemcpy(field)");
        }

        int UploadSource(const float *host, cudaStream_t s)
        {
            if (src.p == nullptr)
            {
                HAL_TRY(src.Alloc(Length(), "cudaMalloc(src)"));
            }
            if (const void *d = MappedHost(host))
            {
                HAL_TRY(TransposeTo<float>(static_cast<const float *>(d), src.p, xDim, yDim, s));
            }
            else
            {
                HAL_TRY(CudaStatus(cudaMemcpyAsync(w.p, host, Length() * sizeof(float), cudaMemcpyHostToDevice, s),
                                   "cudaMemcpy(src)"));
                HAL_TRY(TransposeTo<float>(w.p, src.p, xDim, yDim, s));
            }
            hasSrc = true;
            return HAL_CUDA_OK;
        }
    };
}

using halcuda::Adi;

struct hal_cuda_adi : public Adi
{
};

void halcuda::AdiDims(const hal_cuda_adi *h, int32_t *xDim, int32_t *yDim)
{
    *xDim = h->xDim;
    *yDim = h->yDim;
}

extern "C" int hal_cuda_adi_create(int32_t xDim, int32_t yDim, hal_cuda_adi **out)
{
    HAL_REQUIRE(out != nullptr, "hal_cuda_adi_create: out is NULL");
    *out = nullptr;
    HAL_REQUIRE(xDim > 0 && yDim > 0, "hal_cuda_adi_create: dimensions must be positive");
    HAL_REQUIRE(static_cast<int64_t>(xDim) * yDim < (int64_t(1) << 31),
                "hal_cuda_adi_create: xDim*yDim exceeds int32");
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
        if (h->exact || h->xDim > HAL_CUDA_ADI_MAX_LINE || h->yDim > HAL_CUDA_ADI_MAX_LINE)
        {
            // exact mode, or lines beyond the FP32 partitioned solve: the
            // FP64 Thomas solve per line, in the CPU backend's operation
            // order (bit-exact)
            if (h->adi64 == nullptr)
            {
                h->adi64.reset(new (std::nothrow) Adi64());
                if (h->adi64 == nullptr)
                {
                    SetError("%s: out of host memory", who);
                    return HAL_CUDA_ENOMEM;
                }
            }
            const double *g = nullptr;
            if (ghost != nullptr)
            {
                const size_t ng = 2 * (static_cast<size_t>(h->xDim) + h->yDim);
                if (h->g64.p == nullptr)
                {
                    HAL_TRY(h->g64.Alloc(ng, "cudaMalloc(ghost)"));
                }
                HAL_TRY(CudaStatus(cudaMemcpyAsync(h->g64.p, ghost, ng * sizeof(double), cudaMemcpyHostToDevice, s),
                                   "cudaMemcpy(ghost)"));
                g = h->g64.p;
            }
            HAL_TRY(CudaStatus(cudaMemcpyAsync(h->f64.p, field, n * sizeof(double), cudaMemcpyHostToDevice, s),
                               "cudaMemcpy(field)"));
            HAL_TRY(CudaStatus(cudaMemcpyAsync(h->d64.p, deltas, n * sizeof(double), cudaMemcpyHostToDevice, s),
                               "cudaMemcpy(deltas)"));
            HAL_TRY(h->adi64->Run(h->f64.p, h->d64.p, h->xDim, h->yDim, wrapX, wrapY, r, g, s));
            HAL_TRY(CudaStatus(cudaMemcpyAsync(deltas, h->d64.p, n * sizeof(double), cudaMemcpyDeviceToHost, s),
                               "cudaMemcpy(deltas)"));
            return CudaStatus(cudaStreamSynchronize(s), who);
        }
        const float *g = nullptr;
        if (ghost != nullptr)
        {
            size_t ng = 2 * (static_cast<size_t>(h->xDim) + h->yDim);
            std::vector<float> gf(ng);
            for (size_t i = 0; i < ng; i++)
            {
                gf[i] = static_cast<float>(ghost[i]);
            }
            HAL_TRY(CudaStatus(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
            HAL_TRY(CudaStatus(cudaMemcpy(h->g32.p, gf.data(), ng * sizeof(float), cudaMemcpyHostToDevice),
                               "cudaMemcpy(ghost)"));
            g = h->g32.p;
        }
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->f64.p, field, n * sizeof(double), cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(field)"));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->d64.p, deltas, n * sizeof(double), cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(deltas)"));
        // the field in layout B, in float, in the spare buffer of the pair
        float *fB = h->field[h->cur ^ 1].p;
        HAL_TRY(h->TransposeTo<double>(h->f64.p, fB, h->xDim, h->yDim, s));
        HAL_TRY(h->LaunchX(fB, r, wrapX != 0, wrapY != 0, g, s));
        HAL_TRY(h->LaunchY<kSweepDeltas>(nullptr, nullptr, h->f64.p, h->d64.p, r, 0.0, wrapX != 0, wrapY != 0, g,
                                          false, s));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(deltas, h->d64.p, n * sizeof(double), cudaMemcpyDeviceToHost, s),
                           "cudaMemcpy(deltas)"));
        return h->CheckDeviceError(who);
    }
}

extern "C" int hal_cuda_diffuse_adi(hal_cuda_adi *h, const double *field, int64_t fieldLen, double *deltas,
                                    int64_t deltasLen, double diffRate, int32_t xDim, int32_t yDim,
                                    int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
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
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && field != nullptr && deltas != nullptr, "hal_cuda_diffuse_adi_bc: NULL argument");
    return DiffuseAdiCommon(h, field, deltas, diffRate, wrapX, wrapY, ghost, "hal_cuda_diffuse_adi_bc");
}

extern "C" int hal_cuda_adi_set_field(hal_cuda_adi *h, const float *field, int64_t len)
{
    HAL_REQUIRE(h != nullptr && field != nullptr, "hal_cuda_adi_set_field: NULL argument");
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()), "hal_cuda_adi_set_field: field must hold xDim*yDim values");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    HAL_TRY(h->Upload(field, s));
    return halcuda::CudaStatus(cudaStreamSynchronize(s), "hal_cuda_adi_set_field");
}

extern "C" int hal_cuda_adi_get_field(hal_cuda_adi *h, float *field, int64_t len)
{
    HAL_REQUIRE(h != nullptr && field != nullptr, "hal_cuda_adi_get_field: NULL argument");
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()), "hal_cuda_adi_get_field: field must hold xDim*yDim values");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    HAL_TRY(h->Download(field, s));
    return h->CheckDeviceError("hal_cuda_adi_get_field");
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
    cudaStream_t s = h->stream.Get();
    HAL_TRY(h->UploadSource(dense, s));
    return halcuda::CudaStatus(cudaStreamSynchronize(s), "hal_cuda_adi_set_source");
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
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr, "hal_cuda_adi_run_ticks: handle is NULL");
    HAL_REQUIRE(ticks >= 0, "hal_cuda_adi_run_ticks: negative tick count");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return h->RunTicks(ticks, diffRate, decay, wrapX != 0, wrapY != 0, false);
}

extern "C" int hal_cuda_adi_run_coupled(hal_cuda_adi *h, hal_cuda_agents *agents, int32_t ticks, double diffRate,
                                        double decay, int32_t wrapX, int32_t wrapY, double interactionRad,
                                        double springConstant, double friction, double maxVel)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && agents != nullptr, "hal_cuda_adi_run_coupled: handle is NULL");
    HAL_REQUIRE(ticks >= 0, "hal_cuda_adi_run_coupled: negative tick count");
    HAL_REQUIRE(h->agents == agents,
                "hal_cuda_adi_run_coupled: the agent handle is not the one coupled by hal_cuda_adi_set_uptake");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    halcuda::CoupledStep st;
    st.interactionRad = interactionRad;
    st.springConstant = springConstant;
    st.friction = friction;
    st.maxVel = maxVel;
    return h->RunCoupled(agents, ticks, diffRate, decay, wrapX != 0, wrapY != 0, st);
}

extern "C" int hal_cuda_adi_run_steps(hal_cuda_adi *h, float *field, int64_t len, int32_t steps, double diffRate,
                                      int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
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
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && field != nullptr, "hal_cuda_adi_run_ticks_host: NULL argument");
    HAL_REQUIRE(len == static_cast<int64_t>(h->Length()),
                "hal_cuda_adi_run_ticks_host: field must hold xDim*yDim values");
    HAL_REQUIRE(ticks >= 0, "hal_cuda_adi_run_ticks_host: negative tick count");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    if (src != nullptr)
    {
        HAL_TRY(h->UploadSource(src, s));
    }
    else
    {
        h->hasSrc = false;
    }
    HAL_TRY(h->Upload(field, s));
    HAL_TRY(h->RunTicks(ticks, diffRate, decay, wrapX != 0, wrapY != 0, false));
    HAL_TRY(h->Download(field, s));
    return h->CheckDeviceError("hal_cuda_adi_run_ticks_host");
}

extern "C" int hal_cuda_adi_sync(hal_cuda_adi *h)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_adi_sync: handle is NULL");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return h->CheckDeviceError("hal_cuda_adi_sync");
}

extern "C" void *hal_cuda_adi_stream(hal_cuda_adi *h)
{
    return h ? static_cast<void *>(h->stream.Get()) : nullptr;
}

extern "C" int hal_cuda_adi_set_exact(hal_cuda_adi *h, int32_t exact)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_adi_set_exact: handle is NULL");
    h->exact = exact != 0;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_adi_set_stream(hal_cuda_adi *h, void *stream)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_adi_set_stream: handle is NULL");
    h->stream.Set(stream);
    h->ResetGraphs();
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_adi_profile_graph(hal_cuda_adi *h, int32_t iters, double diffRate, double decay,
                                          int32_t wrapX, int32_t wrapY, float *ms)
{
    HAL_REQUIRE(h != nullptr && ms != nullptr, "hal_cuda_adi_profile_graph: NULL argument");
    HAL_REQUIRE(iters > 0, "hal_cuda_adi_profile_graph: iters must be positive");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    const float *g = h->hasGhost ? h->ghost.p : nullptr;
    HAL_TRY(h->PrepareShapes(diffRate, wrapX != 0, wrapY != 0, g));
    const int c = h->cur;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    HAL_TRY(CudaStatus(cudaEventCreate(&e0), "cudaEventCreate"));
    int rc = CudaStatus(cudaEventCreate(&e1), "cudaEventCreate");
    for (int which = 0; which < 2 && rc == HAL_CUDA_OK; which++)
    {
        // `iters` back-to-back launches of one sweep on the same inputs: the
        // x-sweep rewrites w, the y-sweep rewrites the other parity's field
        rc = CudaStatus(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        int lr = HAL_CUDA_OK;
        for (int32_t t = 0; t < iters && rc == HAL_CUDA_OK && lr == HAL_CUDA_OK; t++)
        {
            lr = (which == 0) ? h->LaunchX(h->field[c].p, diffRate, wrapX != 0, wrapY != 0, g, s)
                              : h->LaunchY<kSweepTick>(h->field[c ^ 1].p, h->field[c].p, nullptr, nullptr, diffRate,
                                                       decay, wrapX != 0, wrapY != 0, g, true, s);
        }
        cudaGraph_t gr = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(s, &gr);
        if (rc == HAL_CUDA_OK)
        {
            rc = (lr != HAL_CUDA_OK) ? lr : CudaStatus(ec, "cudaStreamEndCapture");
        }
        cudaGraphExec_t ex = nullptr;
        if (rc == HAL_CUDA_OK)
        {
            rc = CudaStatus(cudaGraphInstantiate(&ex, gr, 0), "cudaGraphInstantiate");
        }
        if (gr != nullptr)
        {
            cudaGraphDestroy(gr);
        }
        if (rc == HAL_CUDA_OK)
        {
            rc = CudaStatus(cudaGraphLaunch(ex, s), "cudaGraphLaunch");  // warm-up replay
        }
        if (rc == HAL_CUDA_OK)
        {
            cudaEventRecord(e0, s);
            rc = CudaStatus(cudaGraphLaunch(ex, s), "cudaGraphLaunch");
            cudaEventRecord(e1, s);
        }
        if (rc == HAL_CUDA_OK)
        {
            rc = CudaStatus(cudaEventSynchronize(e1), "hal_cuda_adi_profile_graph");
        }
        if (rc == HAL_CUDA_OK)
        {
            float t = 0.0f;
            cudaEventElapsedTime(&t, e0, e1);
            ms[which] = t / static_cast<float>(iters);
            CountLaunch(2 * static_cast<int64_t>(iters));
        }
        if (ex != nullptr)
        {
            cudaGraphExecDestroy(ex);
        }
    }
    cudaEventDestroy(e0);
    if (e1 != nullptr)
    {
        cudaEventDestroy(e1);
    }
    HAL_TRY(rc);
    return h->CheckDeviceError("hal_cuda_adi_profile_graph");
}

extern "C" int hal_cuda_adi_profile(hal_cuda_adi *h, int32_t iters, double diffRate, double decay, int32_t wrapX,
                                    int32_t wrapY, float *ms)
{
    HAL_REQUIRE(h != nullptr && ms != nullptr, "hal_cuda_adi_profile: NULL argument");
    HAL_REQUIRE(iters > 0, "hal_cuda_adi_profile: iters must be positive");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    const float *g = h->hasGhost ? h->ghost.p : nullptr;
    HAL_TRY(h->PrepareShapes(diffRate, wrapX != 0, wrapY != 0, g));
    cudaEvent_t ev[3];
    for (auto &e : ev)
    {
        HAL_TRY(CudaStatus(cudaEventCreate(&e), "cudaEventCreate"));
    }
    double tX = 0.0, tY = 0.0;
    int rc = HAL_CUDA_OK;
    for (int32_t t = 0; t < iters && rc == HAL_CUDA_OK; t++)
    {
        int c = h->cur;
        cudaEventRecord(ev[0], s);
        rc = h->LaunchX(h->field[c].p, diffRate, wrapX != 0, wrapY != 0, g, s);
        if (rc != HAL_CUDA_OK)
        {
            break;
        }
        cudaEventRecord(ev[1], s);
        rc = h->LaunchY<kSweepTick>(h->field[c ^ 1].p, h->field[c].p, nullptr, nullptr, diffRate, decay, wrapX != 0,
                                    wrapY != 0, g, true, s);
        if (rc != HAL_CUDA_OK)
        {
            break;
        }
        cudaEventRecord(ev[2], s);
        rc = CudaStatus(cudaEventSynchronize(ev[2]), "hal_cuda_adi_profile");
        float a = 0.0f, b = 0.0f;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[1], ev[2]);
        tX += a;
        tY += b;
        h->cur ^= 1;
    }
    for (auto &e : ev)
    {
        cudaEventDestroy(e);
    }
    HAL_TRY(rc);
    HAL_TRY(h->CheckDeviceError("hal_cuda_adi_profile"));
    ms[0] = static_cast<float>(tX / iters);
    ms[1] = static_cast<float>(tY / iters);
    return HAL_CUDA_OK;
}
