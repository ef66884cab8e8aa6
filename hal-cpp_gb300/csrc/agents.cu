// agents.cu -- cell-bucket agent forces (IAgentForceBackend2D) on sm_103a.
//
// The CPU backend (src/Agents/CpuAgentForceBackend2D.cpp:66-176) runs four
// serial passes: count agents per cell, exclusive prefix into offsets, stable
// scatter of agent indices, and a per-agent scan of the surrounding cells
// summing a linear spring force.  Here each pass is data-parallel:
//   BinCount     one thread per agent: clamped cell, atomic count, arrival rank
//   scan         reduce-then-scan over the cells (three launches, no spin waits)
//   Scatter      agent -> offsets[cell] + arrival rank (order within a cell is
//                the atomic arrival order, not yet the CPU's)
//   Stabilize    one thread per arrival-order slot: its agent counts the
//                lower-indexed agents of its cell, which gives exactly the
//                CPU's slot; it writes the final bucket and a cell-sorted copy
//                of positions and radii
//   Forces       one thread per sorted slot walks the cell window x-major then
//                y, and each cell's slots in order -- the CPU's summation
//                order -- and writes the agent's velocity delta.
// The binning is integer work and matches the CPU bit for bit: the cell of a
// position is floored in the precision the caller gave it (FP64 on the
// interface path, as the CPU does; FP32 on the resident path, where the CPU
// fed the same float32 values bins identically).  The force sum runs in FP32
// on the resident path and in FP64 with IEEE round-to-nearest operations (no
// contraction) on the FP64 interface path, where positions stay FP64 end to
// end and the result matches the CPU backend bit for bit.
#include "common.cuh"
#include "agents_wells.h"

#include <cmath>
#include <type_traits>

namespace halcuda
{
    namespace
    {
        // Scan tiles of 4096 cells: 256 threads, each with 16 cells in four
        // 16-byte groups, so every thread has four loads in flight.
        constexpr int kScanThreads = 256;
        constexpr int kScanGroups = 4;
        constexpr int kScanItems = 4 * kScanGroups;
        constexpr int kScanTile = kScanThreads * kScanItems;
        // tiles whose prefix ScanApplySum forms itself (4.19M cells)
        constexpr int kScanSumTiles = 1024;

        // Position pairs in the precision of the path: float2 on the FP32
        // resident path, double2 on the FP64 interface path.
        template <typename T>
        struct Vec2;
        template <>
        struct Vec2<float>
        {
            using Type = float2;
            __device__ static float2 Make(float x, float y) { return make_float2(x, y); }
        };
        template <>
        struct Vec2<double>
        {
            using Type = double2;
            __device__ static double2 Make(double x, double y) { return make_double2(x, y); }
        };
        template <typename T>
        using V2 = typename Vec2<T>::Type;

        // AgentForceCellCoord (CpuAgentForceBackend2D.cpp:14-27): the floor is
        // taken in the precision of the positions, as the CPU takes it in FP64.
        __device__ __forceinline__ int32_t Floor32(float v) { return static_cast<int32_t>(floorf(v)); }
        __device__ __forceinline__ int32_t Floor32(double v) { return static_cast<int32_t>(floor(v)); }

        template <typename TP>
        __device__ __forceinline__ int32_t CellCoord(TP v, int32_t dim)
        {
            int32_t c = Floor32(v);
            c = (c < 0) ? 0 : c;
            c = (c >= dim) ? dim - 1 : c;
            return c;
        }

        // Programmatic dependent launch (LaunchChained): the next kernel of a
        // dispatch may be scheduled once every CTA of this one has started;
        // each kernel waits for its predecessor to complete before it touches
        // any buffer (both are no-ops in a plain launch).
        __device__ __forceinline__ void ChainEntry()
        {
            asm volatile("griddepcontrol.launch_dependents;");
            asm volatile("griddepcontrol.wait;" ::: "memory");
        }

        template <typename TP>
        __global__ void BinCount(const TP *__restrict__ pos, int32_t n, int32_t xDim, int32_t yDim,
                                 V2<TP> *__restrict__ posF, int32_t *__restrict__ cellOf,
                                 int32_t *__restrict__ arrival, int32_t *__restrict__ counts)
        {
            ChainEntry();
            int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
            if (i >= n)
            {
                return;
            }
            const TP px = pos[2 * static_cast<int64_t>(i)];
            const TP py = pos[2 * static_cast<int64_t>(i) + 1];
            if (posF != nullptr)  // null when the positions are already V2-aligned
            {
                posF[i] = Vec2<TP>::Make(px, py);
            }
            int32_t c = CellCoord(px, xDim) * yDim + CellCoord(py, yDim);
            cellOf[i] = c;
            arrival[i] = atomicAdd(counts + c, 1);
        }

        // A kernel of the agent dispatch, launched with programmatic stream
        // serialization so that its launch overlaps its predecessor's tail
        // (the kernels start with ChainEntry).
        template <typename... KArgs, typename... Args>
        void LaunchChained(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args... args)
        {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(grid);
            cfg.blockDim = dim3(block);
            cfg.dynamicSmemBytes = 0;
            cfg.stream = s;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            at[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
        }

        // Inclusive warp scan.
        __device__ __forceinline__ int32_t WarpScan(int32_t v, int lane)
        {
#pragma unroll
            for (int d = 1; d < 32; d <<= 1)
            {
                int32_t t = __shfl_up_sync(0xffffffffu, v, d);
                if (lane >= d)
                {
                    v += t;
                }
            }
            return v;
        }

        // Exclusive block scan of one value per thread; returns the block total.
        __device__ __forceinline__ int32_t BlockExclusiveScan(int32_t v, int32_t &excl)
        {
            __shared__ int32_t warpSums[32];
            const int lane = threadIdx.x & 31;
            const int warp = threadIdx.x >> 5;
            const int nwarps = blockDim.x >> 5;
            int32_t inc = WarpScan(v, lane);
            if (lane == 31)
            {
                warpSums[warp] = inc;
            }
            __syncthreads();
            if (warp == 0)
            {
                int32_t s = (lane < nwarps) ? warpSums[lane] : 0;
                int32_t si = WarpScan(s, lane);
                if (lane < nwarps)
                {
                    warpSums[lane] = si - s;  // exclusive prefix of the warp sums
                }
            }
            __syncthreads();
            excl = inc - v + warpSums[warp];
            __shared__ int32_t s_total;
            if (threadIdx.x == blockDim.x - 1)
            {
                s_total = excl + v;
            }
            __syncthreads();
            const int32_t total = s_total;
            __syncthreads();
            return total;
        }

        // Pass 1 of the scan: per-tile sums.
        // Four consecutive cells [base, base + 4): one 16-byte access when the
        // four are in range and aligned, element by element otherwise.
        __device__ __forceinline__ bool Vec4Ok(const int32_t *p, int64_t base, int64_t C)
        {
            return base + 4 <= C && ((reinterpret_cast<uintptr_t>(p + base) & 15u) == 0u);
        }

        __device__ __forceinline__ void LoadItems(const int32_t *__restrict__ p, int64_t base, int64_t C,
                                                  int32_t *v)
        {
            if (Vec4Ok(p, base, C))
            {
                const int4 t = *reinterpret_cast<const int4 *>(p + base);
                v[0] = t.x;
                v[1] = t.y;
                v[2] = t.z;
                v[3] = t.w;
                return;
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
            {
                v[q] = (base + q < C) ? p[base + q] : 0;
            }
        }

        __device__ __forceinline__ void StoreItems(int32_t *__restrict__ p, int64_t base, int64_t C, const int32_t *v)
        {
            if (Vec4Ok(p, base, C))
            {
                *reinterpret_cast<int4 *>(p + base) = make_int4(v[0], v[1], v[2], v[3]);
                return;
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
            {
                if (base + q < C)
                {
                    p[base + q] = v[q];
                }
            }
        }

        // The tile sum needs no order: group g of a thread is cells tile +
        // g * 1024 + 4 * thread, so each warp's loads are contiguous.
        __global__ void __launch_bounds__(kScanThreads) ScanReduce(const int32_t *__restrict__ counts, int64_t C,
                                                                   int32_t *__restrict__ tileSums)
        {
            ChainEntry();
            const int64_t tile0 = static_cast<int64_t>(blockIdx.x) * kScanTile;
            int32_t v[kScanItems];
#pragma unroll
            for (int g = 0; g < kScanGroups; g++)
            {
                LoadItems(counts, tile0 + g * (4 * kScanThreads) + 4 * threadIdx.x, C, v + 4 * g);
            }
            int32_t s = 0;
#pragma unroll
            for (int q = 0; q < kScanItems; q++)
            {
                s += v[q];
            }
            int32_t excl;
            int32_t total = BlockExclusiveScan(s, excl);
            if (threadIdx.x == 0)
            {
                tileSums[blockIdx.x] = total;
            }
        }

        // Pass 2: exclusive scan of the tile sums by one CTA (looping over
        // chunks of kScanThreads).
        __global__ void __launch_bounds__(kScanThreads) ScanTiles(int32_t *__restrict__ tileSums, int32_t nTiles)
        {
            ChainEntry();
            int32_t carry = 0;
            for (int32_t base = 0; base < nTiles; base += kScanThreads)
            {
                int32_t idx = base + threadIdx.x;
                int32_t v = (idx < nTiles) ? tileSums[idx] : 0;
                int32_t excl;
                int32_t total = BlockExclusiveScan(v, excl);
                if (idx < nTiles)
                {
                    tileSums[idx] = carry + excl;
                }
                carry += total;
            }
        }

        // Counts up to this many cells (in practice: all) are cleared by
        // ScanApply as it reads them, writing only the 4-cell groups that
        // hold a count; a memset before the binning clears counts not known
        // to be zero.  With every group written, clearing in the scan had
        // measured 3.5x slower than a memset at 109M cells; with only the
        // occupied groups it is faster at both measured sizes (4.19M cells,
        // 1M agents: 119.2 -> 115.0 us per dispatch; 109M cells, 5.2M
        // agents: agent pass 0.818 -> 0.772 ms).
        constexpr int64_t kClearInScanCells = int64_t(1) << 40;

        // The cells of a thread of passes 3: kScanItems consecutive cells
        // from tile + thread * kScanItems (in order, for the exclusive scan),
        // loaded as four 16-byte groups.  With `clear` the groups holding a
        // count are written back as zeros (most cells are empty, and an empty
        // group is already cleared).
        __device__ __forceinline__ void LoadThreadCells(int32_t *__restrict__ counts, int64_t base, int64_t C,
                                                        bool clear, int32_t (&v)[kScanItems])
        {
#pragma unroll
            for (int g = 0; g < kScanGroups; g++)
            {
                LoadItems(counts, base + 4 * g, C, v + 4 * g);
            }
            if (clear)
            {
#pragma unroll
                for (int g = 0; g < kScanGroups; g++)
                {
                    if ((v[4 * g] | v[4 * g + 1] | v[4 * g + 2] | v[4 * g + 3]) != 0)
                    {
                        const int32_t zeros[4] = {0, 0, 0, 0};
                        StoreItems(counts, base + 4 * g, C, zeros);
                    }
                }
            }
        }

        // The thread's exclusive offsets from its first one, stored as four
        // 16-byte groups.
        __device__ __forceinline__ void StoreThreadOffsets(int32_t *__restrict__ offsets, int64_t base, int64_t C,
                                                           int32_t first, const int32_t (&v)[kScanItems])
        {
            int32_t o[kScanItems];
            o[0] = first;
#pragma unroll
            for (int q = 1; q < kScanItems; q++)
            {
                o[q] = o[q - 1] + v[q - 1];
            }
#pragma unroll
            for (int g = 0; g < kScanGroups; g++)
            {
                StoreItems(offsets, base + 4 * g, C, o + 4 * g);
            }
        }

        // Pass 3: tile-local exclusive scan plus the tile prefix -> offsets.
        // With CLEAR it also zeroes the counts it has read (only the groups
        // holding one), so the next binning starts from zero without a memset.
        template <bool CLEAR>
        __global__ void __launch_bounds__(kScanThreads) ScanApply(int32_t *__restrict__ counts, int64_t C,
                                                                  const int32_t *__restrict__ tilePrefix,
                                                                  int32_t *__restrict__ offsets, int32_t n)
        {
            ChainEntry();
            const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
            int32_t v[kScanItems];
            LoadThreadCells(counts, base, C, CLEAR, v);
            int32_t s = 0;
#pragma unroll
            for (int q = 0; q < kScanItems; q++)
            {
                s += v[q];
            }
            int32_t excl;
            BlockExclusiveScan(s, excl);
            StoreThreadOffsets(offsets, base, C, tilePrefix[blockIdx.x] + excl, v);
            if (blockIdx.x == 0 && threadIdx.x == 0)
            {
                offsets[C] = n;
            }
        }

        // Passes 2 and 3 in one launch, for grids of at most kScanSumTiles
        // tiles: each CTA reduces the tile sums before its own (a few per
        // thread) into its tile's prefix, then runs ScanApply<true>'s tile
        // scan.  This saves the single-CTA ScanTiles launch between them.
        __global__ void __launch_bounds__(kScanThreads) ScanApplySum(int32_t *__restrict__ counts, int64_t C,
                                                                     const int32_t *__restrict__ tileSums,
                                                                     int32_t *__restrict__ offsets, int32_t n)
        {
            ChainEntry();
            int32_t before = 0;
            for (int32_t t = static_cast<int32_t>(threadIdx.x); t < static_cast<int32_t>(blockIdx.x);
                 t += kScanThreads)
            {
                before += tileSums[t];
            }
            int32_t unused;
            const int32_t prefix = BlockExclusiveScan(before, unused);  // the block total
            const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
            int32_t v[kScanItems];
            LoadThreadCells(counts, base, C, true, v);
            int32_t sum = 0;
#pragma unroll
            for (int q = 0; q < kScanItems; q++)
            {
                sum += v[q];
            }
            int32_t excl;
            BlockExclusiveScan(sum, excl);
            StoreThreadOffsets(offsets, base, C, prefix + excl, v);
            if (blockIdx.x == 0 && threadIdx.x == 0)
            {
                offsets[C] = n;
            }
        }

        __global__ void Scatter(const int32_t *__restrict__ cellOf, const int32_t *__restrict__ arrival,
                                const int32_t *__restrict__ offsets, int32_t n, int32_t *__restrict__ bucketTmp)
        {
            ChainEntry();
            int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
            if (i >= n)
            {
                return;
            }
            bucketTmp[offsets[cellOf[i]] + arrival[i]] = i;
        }

        // The CPU scatters in agent-index order (CpuAgentForceBackend2D.cpp:
        // 100-109), so an agent's slot within its cell is the number of
        // lower-indexed agents in the same cell.
        template <typename TP, typename TR>
        __global__ void Stabilize(const int32_t *__restrict__ cellOf, const int32_t *__restrict__ offsets,
                                  const int32_t *__restrict__ bucketTmp, const V2<TP> *__restrict__ posF,
                                  const TR *__restrict__ rad, int32_t n, int32_t *__restrict__ bucket,
                                  V2<TP> *__restrict__ sPos, TR *__restrict__ sRad)
        {
            ChainEntry();
            // thread -> arrival-order slot q: its agent i, then i's stable
            // slot in the same cell (neighbouring threads share a cell's
            // offsets and bucket range, and their writes land near q)
            const int32_t q = blockIdx.x * blockDim.x + threadIdx.x;
            if (q >= n)
            {
                return;
            }
            const int32_t i = bucketTmp[q];
            const int32_t c = cellOf[i];
            const int32_t s = offsets[c];
            const int32_t e = offsets[c + 1];
            int32_t rank = 0;
            for (int32_t t = s; t < e; t++)
            {
                rank += (bucketTmp[t] < i) ? 1 : 0;
            }
            const int32_t slot = s + rank;
            bucket[slot] = i;
            sPos[slot] = posF[i];
            sRad[slot] = rad[i];
        }

        // Stable order within each cell (the CPU's scatter in agent index
        // order, CpuAgentForceBackend2D.cpp:100-109), one thread per
        // arrival-order slot q: its agent i, whose position gives its cell
        // again (no cell-array gather), goes to slot s + (number of
        // lower-indexed agents of the cell).  Neighbouring threads share a
        // cell's offsets and range of arrival-ordered indices, and the writes
        // land within the cell's own slots.
        template <typename TP, typename TR>
        __global__ void StabilizeSlots(const int32_t *__restrict__ offsets, const int32_t *__restrict__ bucketTmp,
                                       const V2<TP> *__restrict__ pos, const TR *__restrict__ rad, int32_t n,
                                       int32_t xDim, int32_t yDim, int32_t *__restrict__ bucket,
                                       V2<TP> *__restrict__ sPos, TR *__restrict__ sRad)
        {
            ChainEntry();
            const int32_t q = blockIdx.x * blockDim.x + threadIdx.x;
            if (q >= n)
            {
                return;
            }
            const int32_t i = bucketTmp[q];
            const V2<TP> p = pos[i];
            const TR r = rad[i];
            const int32_t c = CellCoord(p.x, xDim) * yDim + CellCoord(p.y, yDim);
            const int32_t s = offsets[c];
            const int32_t e = offsets[c + 1];
            int32_t rank = 0;
            for (int32_t t = s; t < e; t++)
            {
                rank += (bucketTmp[t] < i) ? 1 : 0;
            }
            const int32_t slot = s + rank;
            bucket[slot] = i;
            sPos[slot] = p;
            sRad[slot] = r;
        }

        // IEEE-exact FP64 helpers (no contraction) and their FP32 twins.
        __device__ __forceinline__ double Add(double a, double b) { return __dadd_rn(a, b); }
        __device__ __forceinline__ double Sub(double a, double b) { return __dsub_rn(a, b); }
        __device__ __forceinline__ double Mul(double a, double b) { return __dmul_rn(a, b); }
        __device__ __forceinline__ double Div(double a, double b) { return __ddiv_rn(a, b); }
        __device__ __forceinline__ double Sqrt(double a) { return __dsqrt_rn(a); }
        __device__ __forceinline__ float Add(float a, float b) { return __fadd_rn(a, b); }
        __device__ __forceinline__ float Sub(float a, float b) { return __fsub_rn(a, b); }
        __device__ __forceinline__ float Mul(float a, float b) { return __fmul_rn(a, b); }
        __device__ __forceinline__ double Abs(double a) { return fabs(a); }
        __device__ __forceinline__ float Abs(float a) { return fabsf(a); }

        // AgentForceDisp (CpuAgentForceBackend2D.cpp:30-45).
        template <typename T>
        __device__ __forceinline__ T Disp(T a, T b, T dimF, bool wrap)
        {
            T d = Sub(b, a);
            if (wrap && Abs(d) > Mul(dimF, T(0.5)))
            {
                d = (a > b) ? Add(d, dimF) : Sub(d, dimF);
            }
            return d;
        }

        // The agent grid's displacement GridGeometry2D::DispX/DispY
        // (src/Grids/GridGeometry2D.cpp:132-150) of p2 seen from p1: on a
        // wrapped axis DispWrap (src/MathUtil.cpp:363-379) shifts one end by
        // the axis length before subtracting, so it rounds differently from
        // AgentForceDisp.
        template <typename T>
        __device__ __forceinline__ T DispGrid(T p1, T p2, T dimF, bool wrap)
        {
            if (wrap && Abs(Sub(p1, p2)) > Mul(dimF, T(0.5)))
            {
                return (p1 > p2) ? Sub(Add(p2, dimF), p1) : Sub(p2, Add(p1, dimF));
            }
            return Sub(p2, p1);
        }

        // Overlap force laws: the overlapFun(touchDist, other) of
        // SphericalAgent2D::SumForces (include/Hal/Agents/SphericalAgent2D.h:
        // 74-102) as a law kind and its parameters.
        constexpr int kLawLinear = HAL_CUDA_FORCE_LINEAR;
        constexpr int kLawClamped = HAL_CUDA_FORCE_LINEAR_CLAMPED;
        constexpr int kLawPower = HAL_CUDA_FORCE_POWER;

        template <typename T>
        struct LawParams
        {
            T scale;
            T exponent;
        };

        __device__ __forceinline__ double Pow(double a, double b) { return pow(a, b); }
        __device__ __forceinline__ float Pow(float a, float b) { return powf(a, b); }

        template <int LAW, typename T>
        __device__ __forceinline__ T OverlapForce(T touch, const LawParams<T> &lp)
        {
            if constexpr (LAW == kLawLinear)
            {
                // springConstant * touchDist (CpuAgentForceBackend2D.cpp:165)
                return Mul(lp.scale, touch);
            }
            else if constexpr (LAW == kLawClamped)
            {
                // no force unless overlapping, then Hooke's law
                // (examples/OffLatticeExample.cpp:147-154)
                return (touch < T(0)) ? T(0) : Mul(lp.scale, touch);
            }
            else
            {
                // pow(scale * touchDist, exponent) (examples/Chemotaxis.cpp:128-130)
                return Pow(Mul(lp.scale, touch), lp.exponent);
            }
        }

        // One neighbour's contribution (CpuAgentForceBackend2D.cpp:153-169,
        // SphericalAgent2D.h:83-98): the displacement to pj, and for
        // 0 < d < R the force law's force along it, subtracted from (vx, vy);
        // with SUM a positive force is added to sum.
        template <typename T, int LAW, bool SUM, bool GRID>
        __device__ __forceinline__ void PairStep(T px, T py, T rad, V2<T> pj, T radj, T R, const LawParams<T> &lp,
                                                 T xDimF, T yDimF, int32_t wrapX, int32_t wrapY, T &vx, T &vy,
                                                 T &sum)
        {
            T xComp, yComp;
            if constexpr (GRID)
            {
                xComp = DispGrid(px, pj.x, xDimF, wrapX != 0);
                yComp = DispGrid(py, pj.y, yDimF, wrapY != 0);
            }
            else
            {
                xComp = Disp(px, pj.x, xDimF, wrapX != 0);
                yComp = Disp(py, pj.y, yDimF, wrapY != 0);
            }
            if constexpr (std::is_same<T, double>::value)
            {
                // IEEE operations in the CPU's order: bit-exact
                const T dist = Sqrt(Add(Mul(xComp, xComp), Mul(yComp, yComp)));
                if ((dist < R) && (dist > T(0)))
                {
                    const T touchDist = Sub(Add(rad, radj), dist);
                    const T force = OverlapForce<LAW>(touchDist, lp);
                    vx = Sub(vx, Mul(Div(xComp, dist), force));
                    vy = Sub(vy, Mul(Div(yComp, dist), force));
                    if constexpr (SUM)
                    {
                        if (force > T(0))
                        {
                            sum = Add(sum, Abs(force));
                        }
                    }
                }
            }
            else
            {
                // FP32 path: 1/d from rsqrt (d^2 = 0 gives NaN, which fails
                // both tests like the CPU's d > 0)
                const T d2 = fmaf(xComp, xComp, yComp * yComp);
                const T inv = rsqrtf(d2);
                const T dist = d2 * inv;
                if ((dist < R) && (dist > T(0)))
                {
                    const T force = OverlapForce<LAW>((rad + radj) - dist, lp);
                    const T scale = inv * force;
                    vx -= xComp * scale;
                    vy -= yComp * scale;
                    if constexpr (SUM)
                    {
                        if (force > T(0))
                        {
                            sum += force;
                        }
                    }
                }
            }
        }

        // One agent's force sum: its velocity after the neighbours' forces
        // (or the deltas, from zero) and the sum of its positive forces.
        template <typename T>
        struct ForceAcc
        {
            V2<T> v;
            T sum;
        };

        // Pass 4 (CpuAgentForceBackend2D.cpp:112-175) for the agent in sorted
        // slot `slot`; offsets are the cell offsets of its grid.  Starting
        // from v0, each neighbour j within range subtracts (disp/d)*force,
        // force = LAW(touchDist); with SUM the positive forces are summed as
        // SumForces returns them.  GRID visits each cell's agents in
        // descending index order with the agent grid's displacement, which is
        // SphericalAgent2D::SumForces on an AgentGrid2D whose agents were
        // created in index order (each square's list is newest first,
        // AgentPT2D.h:200-241); otherwise the order is the CPU backend's
        // (ascending index within a cell).
        template <typename T, int LAW, bool SUM, bool GRID>
        __device__ __forceinline__ ForceAcc<T> ForceSlotLaw(const int32_t slot, const int32_t *__restrict__ offsets,
                                                            const V2<T> *__restrict__ sPos,
                                                            const T *__restrict__ sRad, double interactionRad, T R,
                                                            const LawParams<T> lp, int32_t xDim, int32_t yDim,
                                                            int32_t wrapX, int32_t wrapY, V2<T> v0)
        {
            const V2<T> pf = sPos[slot];
            const T px = pf.x;
            const T py = pf.y;
            const T rad = sRad[slot];
            // window bounds in FP64, as the CPU computes them
            int32_t xStart = static_cast<int32_t>(floor(static_cast<double>(pf.x) - interactionRad));
            int32_t xEnd = static_cast<int32_t>(ceil(static_cast<double>(pf.x) + interactionRad));
            int32_t yStart = static_cast<int32_t>(floor(static_cast<double>(pf.y) - interactionRad));
            int32_t yEnd = static_cast<int32_t>(ceil(static_cast<double>(pf.y) + interactionRad));
            // off-grid cells of a non-wrapped axis are skipped anyway
            if (!wrapX)
            {
                xStart = max(xStart, 0);
                xEnd = min(xEnd, xDim);
            }
            if (!wrapY)
            {
                yStart = max(yStart, 0);
                yEnd = min(yEnd, yDim);
            }
            const T xDimF = static_cast<T>(xDim);
            const T yDimF = static_cast<T>(yDim);
            T vx = v0.x, vy = v0.y;
            T sum = T(0);
            // one candidate slot q of the window, in the CPU's visiting order
            auto visit = [&](int32_t q) {
                if (q == slot)
                {
                    return;
                }
                PairStep<T, LAW, SUM, GRID>(px, py, rad, sPos[q], sRad[q], R, lp, xDimF, yDimF, wrapX, wrapY, vx,
                                            vy, sum);
            };
            auto result = [&]() {
                ForceAcc<T> acc;
                acc.v.x = vx;
                acc.v.y = vy;
                acc.sum = sum;
                return acc;
            };
            if constexpr (GRID)
            {
                // cell by cell, each cell's slots from last to first
                for (int32_t xSq = xStart; xSq < xEnd; xSq++)
                {
                    int32_t retX = xSq;
                    if (retX < 0 || retX >= xDim)
                    {
                        retX %= xDim;  // only reached on a wrapped axis (clamped otherwise)
                        retX = (retX < 0) ? retX + xDim : retX;
                    }
                    for (int32_t ySq = yStart; ySq < yEnd; ySq++)
                    {
                        int32_t retY = ySq;
                        if (retY < 0 || retY >= yDim)
                        {
                            retY %= yDim;
                            retY = (retY < 0) ? retY + yDim : retY;
                        }
                        const int32_t cell = retX * yDim + retY;
                        const int32_t s = __ldg(offsets + cell);
                        const int32_t e = __ldg(offsets + cell + 1);
                        for (int32_t q = e - 1; q >= s; q--)
                        {
                            visit(q);
                        }
                    }
                }
                return result();
            }
            // Common case: a window of at most four rows whose y-range does
            // not wrap, so each row is one run of cells.  All rows' offset
            // pairs are loaded before the first candidate, which shortens the
            // chain of dependent loads; the visiting order is unchanged.
            const int32_t nRows = xEnd - xStart;
            if (nRows > 0 && nRows <= 4 && yStart >= 0 && yEnd <= yDim && yEnd > yStart)
            {
                int32_t rs[4], re[4];
#pragma unroll
                for (int j = 0; j < 4; j++)
                {
                    rs[j] = 0;
                    re[j] = 0;
                    if (j < nRows)
                    {
                        int32_t retX = xStart + j;
                        if (retX < 0 || retX >= xDim)
                        {
                            retX %= xDim;  // only reached on a wrapped axis (clamped otherwise)
                            retX = (retX < 0) ? retX + xDim : retX;
                        }
                        const int32_t cell = retX * yDim + yStart;
                        rs[j] = __ldg(offsets + cell);
                        re[j] = __ldg(offsets + cell + (yEnd - yStart));
                    }
                }
                // The rows' runs, one after another, form one sequence of
                // candidates in the visiting order; it is walked in groups of
                // kGroup whose loads are issued before any of them is used, so
                // a thread waits for one round trip per group, not per
                // candidate.
                constexpr int kGroup = 4;
                const int32_t c1 = re[0] - rs[0];
                const int32_t c2 = c1 + (re[1] - rs[1]);
                const int32_t c3 = c2 + (re[2] - rs[2]);
                const int32_t total = c3 + (re[3] - rs[3]);
                for (int32_t k0 = 0; k0 < total; k0 += kGroup)
                {
                    int32_t qs[kGroup];
                    V2<T> pj[kGroup];
                    T rj[kGroup];
#pragma unroll
                    for (int u = 0; u < kGroup; u++)
                    {
                        const int32_t k = k0 + u;
                        qs[u] = (k >= total) ? -1
                                : (k < c1)   ? rs[0] + k
                                : (k < c2)   ? rs[1] + (k - c1)
                                : (k < c3)   ? rs[2] + (k - c2)
                                             : rs[3] + (k - c3);
                        if (qs[u] >= 0)
                        {
                            pj[u] = sPos[qs[u]];
                            rj[u] = sRad[qs[u]];
                        }
                    }
#pragma unroll
                    for (int u = 0; u < kGroup; u++)
                    {
                        if (qs[u] >= 0 && qs[u] != slot)
                        {
                            PairStep<T, LAW, SUM, GRID>(px, py, rad, pj[u], rj[u], R, lp, xDimF, yDimF, wrapX, wrapY,
                                                        vx, vy, sum);
                        }
                    }
                }
                return result();
            }
            for (int32_t xSq = xStart; xSq < xEnd; xSq++)
            {
                int32_t retX = xSq;
                const bool inX = (retX >= 0) && (retX < xDim);
                if (!inX)
                {
                    if (!wrapX)
                    {
                        continue;
                    }
                    retX %= xDim;
                    retX = (retX < 0) ? retX + xDim : retX;
                }
                // The cells (retX, ySq) for consecutive ySq are consecutive
                // cell indices, and their agents consecutive bucket slots, so
                // the row is walked as runs of cells that do not wrap: two
                // offset loads per run, the same visiting order as cell by
                // cell (the CPU's order).
                for (int32_t ySq = yStart; ySq < yEnd;)
                {
                    int32_t retY = ySq;
                    if (retY < 0 || retY >= yDim)
                    {
                        retY %= yDim;  // only reached on a wrapped axis (clamped otherwise)
                        retY = (retY < 0) ? retY + yDim : retY;
                    }
                    const int32_t run = min(yEnd - ySq, yDim - retY);
                    ySq += run;
                    const int32_t cell = retX * yDim + retY;
                    const int32_t s = __ldg(offsets + cell);
                    const int32_t e = __ldg(offsets + cell + run);
                    for (int32_t q = s; q < e; q++)
                    {
                        visit(q);
                    }
                }
            }
            return result();
        }

        // The CPU backend's pass 4: linear law, velocity deltas from zero.
        template <typename T>
        __device__ __forceinline__ V2<T> ForceSlot(const int32_t slot, const int32_t *__restrict__ offsets,
                                                   const V2<T> *__restrict__ sPos, const T *__restrict__ sRad,
                                                   double interactionRad, T R, T k, int32_t xDim, int32_t yDim,
                                                   int32_t wrapX, int32_t wrapY)
        {
            LawParams<T> lp;
            lp.scale = k;
            lp.exponent = T(1);
            return ForceSlotLaw<T, kLawLinear, false, false>(slot, offsets, sPos, sRad, interactionRad, R, lp, xDim,
                                                             yDim, wrapX, wrapY, Vec2<T>::Make(T(0), T(0)))
                .v;
        }

        template <typename TV, typename TVec>
        __device__ __forceinline__ void StoreDelta(TV *__restrict__ vel, int32_t i, TVec d)
        {
            vel[2 * static_cast<int64_t>(i)] = static_cast<TV>(d.x);
            vel[2 * static_cast<int64_t>(i) + 1] = static_cast<TV>(d.y);
        }

        // Pass 4 over cell-sorted slots: one thread per slot.  With velIn the
        // sum starts from the agent's velocity (SumForces adds to xVel/yVel),
        // otherwise from zero (the interface's velocity deltas); with SUM the
        // agent's sum of positive forces goes to sums.
        // WALLS: neither axis wraps (a compile-time 0 for both wrap flags, so
        // the displacement's wrap test leaves the per-candidate code).
        template <typename T, typename TV, int LAW = kLawLinear, bool SUM = false, bool GRID = false,
                  bool WALLS = false>
        __global__ void Forces(const int32_t *__restrict__ bucket, const int32_t *__restrict__ offsets,
                               const V2<T> *__restrict__ sPos, const T *__restrict__ sRad, int32_t n,
                               double interactionRad, T R, LawParams<T> lp, int32_t xDim, int32_t yDim,
                               int32_t wrapX, int32_t wrapY, TV *vel, T *__restrict__ sums, const TV *velIn)
        {
            ChainEntry();
            const int32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
            if (slot >= n)
            {
                return;
            }
            const int32_t i = bucket[slot];
            V2<T> v0 = Vec2<T>::Make(T(0), T(0));
            if (velIn != nullptr)
            {
                v0 = Vec2<T>::Make(static_cast<T>(velIn[2 * static_cast<int64_t>(i)]),
                                   static_cast<T>(velIn[2 * static_cast<int64_t>(i) + 1]));
            }
            const ForceAcc<T> acc = ForceSlotLaw<T, LAW, SUM, GRID>(slot, offsets, sPos, sRad, interactionRad, R, lp,
                                                                    xDim, yDim, WALLS ? 0 : wrapX, WALLS ? 0 : wrapY,
                                                                    v0);
            StoreDelta(vel, i, acc.v);
            if constexpr (SUM)
            {
                sums[i] = acc.sum;
            }
        }

        // SphericalAgent2D's per-tick update after its forces
        // (include/Hal/Agents/SphericalAgent2D.h:133-162) in FP32, each IEEE
        // operation rounded to nearest with no contraction:
        //   vel += delta;  CapVelocity(maxVel) when maxVel >= 0;
        //   ForceMove: MoveSafePT(pos + vel) (AgentPT2D.h:157-186): a point
        //     on the grid is taken as is; otherwise each wrapped axis wraps
        //     (Wrap, src/MathUtil.cpp:48-53) and each closed axis whose new
        //     coordinate left [0, dim) keeps the old one;
        //   ApplyFriction(friction): vel *= friction.
        struct MoveParams
        {
            float friction;
            float maxVel;  // < 0: no cap
            float xDimF, yDimF;
            int32_t wrapX, wrapY;
        };

        __device__ __forceinline__ float WrapCoord(float v, float dim)
        {
            const float m = fmodf(v, dim);
            return (m < 0.0f) ? __fadd_rn(dim, m) : m;
        }

        __device__ __forceinline__ void MoveAgent(const MoveParams &mp, float2 &p, float2 &v)
        {
            if (mp.maxVel >= 0.0f)
            {
                const float maxVelSq = __fmul_rn(mp.maxVel, mp.maxVel);
                const float normSq = __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y));
                if (normSq > maxVelSq)
                {
                    const float conv = __fdiv_rn(mp.maxVel, __fsqrt_rn(normSq));
                    v.x = __fmul_rn(v.x, conv);
                    v.y = __fmul_rn(v.y, conv);
                }
            }
            float nx = __fadd_rn(p.x, v.x);
            float ny = __fadd_rn(p.y, v.y);
            const bool in = nx >= 0.0f && nx < mp.xDimF && ny >= 0.0f && ny < mp.yDimF;
            if (!in)
            {
                if (mp.wrapX)
                {
                    nx = WrapCoord(nx, mp.xDimF);
                }
                else if (!(nx >= 0.0f && nx < mp.xDimF))
                {
                    nx = p.x;
                }
                if (mp.wrapY)
                {
                    ny = WrapCoord(ny, mp.yDimF);
                }
                else if (!(ny >= 0.0f && ny < mp.yDimF))
                {
                    ny = p.y;
                }
            }
            p.x = nx;
            p.y = ny;
            v.x = __fmul_rn(v.x, mp.friction);
            v.y = __fmul_rn(v.y, mp.friction);
        }

        // Forces of the resident step with the move fused in: the slot's
        // agent adds its delta to its velocity and moves.  Positions are read
        // from the cell-sorted copy, so writing the agent-order positions
        // here races with no other thread.  With counts set, the moved agent
        // is also counted into its new cell, BinCount's work for the next
        // tick (cell, arrival rank): this tick's scan cleared the counts, and
        // its scatter has read the previous cells and ranks.
        template <int LAW = kLawLinear, bool SUM = false, bool WALLS = false>
        __global__ void ForcesMove(const int32_t *__restrict__ bucket, const int32_t *__restrict__ offsets,
                                   const float2 *__restrict__ sPos, const float *__restrict__ sRad, int32_t n,
                                   double interactionRad, float R, LawParams<float> lp, int32_t xDim, int32_t yDim,
                                   MoveParams mp, float *__restrict__ deltas, float2 *__restrict__ pos,
                                   float2 *__restrict__ velocity, float *__restrict__ sums,
                                   int32_t *__restrict__ cellOf, int32_t *__restrict__ arrival,
                                   int32_t *__restrict__ counts)
        {
            ChainEntry();
            const int32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
            if (slot >= n)
            {
                return;
            }
            const int32_t i = bucket[slot];
            const ForceAcc<float> acc = ForceSlotLaw<float, LAW, SUM, false>(
                slot, offsets, sPos, sRad, interactionRad, R, lp, xDim, yDim, WALLS ? 0 : mp.wrapX,
                WALLS ? 0 : mp.wrapY, make_float2(0.f, 0.f));
            const V2<float> d = acc.v;
            StoreDelta(deltas, i, d);
            if constexpr (SUM)
            {
                sums[i] = acc.sum;
            }
            float2 p = sPos[slot];
            float2 v = velocity[i];
            v.x = __fadd_rn(v.x, d.x);
            v.y = __fadd_rn(v.y, d.y);
            MoveAgent(mp, p, v);
            pos[i] = p;
            velocity[i] = v;
            if (counts != nullptr)
            {
                const int32_t c = CellCoord(p.x, xDim) * yDim + CellCoord(p.y, yDim);
                cellOf[i] = c;
                arrival[i] = atomicAdd(counts + c, 1);
            }
        }

        // ---- many independent wells in one pass ------------------------------
        // Agents of all wells are concatenated, and so are the cells of the
        // wells that have agents (well w's cells start at cellBase); the
        // count, scan, scatter and stable-rank passes then run unchanged over
        // the concatenation, and each agent's window walks its own well.

        __global__ void BinCountWells(const float *__restrict__ pos, const int32_t *__restrict__ wellOf,
                                      const AgentWellDev *__restrict__ wells, int32_t n, float2 *__restrict__ posF,
                                      int32_t *__restrict__ binOf, int32_t *__restrict__ arrival,
                                      int32_t *__restrict__ counts)
        {
            ChainEntry();
            const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
            if (i >= n)
            {
                return;
            }
            const AgentWellDev wd = wells[wellOf[i]];
            const float px = pos[2 * static_cast<int64_t>(i)];
            const float py = pos[2 * static_cast<int64_t>(i) + 1];
            posF[i] = make_float2(px, py);
            const int32_t b = static_cast<int32_t>(wd.binBase) + (CellCoord(px, wd.xDim) >> wd.binShift) * wd.binsY +
                              (CellCoord(py, wd.yDim) >> wd.binShift);
            binOf[i] = b;
            arrival[i] = atomicAdd(counts + b, 1);
        }

        // The order within a coarse bin: by cell, then by agent index (the
        // per-cell binning's order for each cell).  The agent at
        // arrival-order slot q counts the agents of its bin before it.
        __global__ void StabilizeWells(const int32_t *__restrict__ binOf, const int32_t *__restrict__ offsets,
                                       const int32_t *__restrict__ bucketTmp, const float2 *__restrict__ posF,
                                       const float *__restrict__ rad, const int32_t *__restrict__ wellOf,
                                       const AgentWellDev *__restrict__ wells, int32_t n,
                                       int32_t *__restrict__ bucket, float2 *__restrict__ sPos,
                                       float *__restrict__ sRad, int32_t *__restrict__ sCell)
        {
            ChainEntry();
            const int32_t q = blockIdx.x * blockDim.x + threadIdx.x;
            if (q >= n)
            {
                return;
            }
            const int32_t i = bucketTmp[q];
            const AgentWellDev wd = wells[wellOf[i]];
            const float2 p = posF[i];
            const int32_t c = CellCoord(p.x, wd.xDim) * wd.yDim + CellCoord(p.y, wd.yDim);
            const int32_t b = binOf[i];
            const int32_t s = offsets[b];
            const int32_t e = offsets[b + 1];
            int32_t rank = 0;
            for (int32_t t = s; t < e; t++)
            {
                const int32_t j = bucketTmp[t];
                const float2 pj = posF[j];
                const int32_t cj = CellCoord(pj.x, wd.xDim) * wd.yDim + CellCoord(pj.y, wd.yDim);
                rank += (cj < c || (cj == c && j < i)) ? 1 : 0;
            }
            const int32_t slot = s + rank;
            bucket[slot] = i;
            sPos[slot] = p;
            sRad[slot] = rad[i];
            sCell[slot] = c;
        }

        // Pass 4 of one well's agent over the coarse bins: the window's cells
        // x-major then y, each cell's agents (a run of its bin, in index
        // order), so the visiting order and the sum are those of ForceSlot
        // on the well's own per-cell bins.
        __device__ __forceinline__ V2<float> ForceSlotWell(const int32_t slot, const int32_t *__restrict__ offsets,
                                                           const float2 *__restrict__ sPos,
                                                           const float *__restrict__ sRad,
                                                           const int32_t *__restrict__ sCell, double interactionRad,
                                                           float R, float k, const AgentWellDev &wd)
        {
            const float2 pf = sPos[slot];
            const float rad = sRad[slot];
            const int32_t xDim = wd.xDim, yDim = wd.yDim;
            int32_t xStart = static_cast<int32_t>(floor(static_cast<double>(pf.x) - interactionRad));
            int32_t xEnd = static_cast<int32_t>(ceil(static_cast<double>(pf.x) + interactionRad));
            int32_t yStart = static_cast<int32_t>(floor(static_cast<double>(pf.y) - interactionRad));
            int32_t yEnd = static_cast<int32_t>(ceil(static_cast<double>(pf.y) + interactionRad));
            if (!wd.wrapX)
            {
                xStart = max(xStart, 0);
                xEnd = min(xEnd, xDim);
            }
            if (!wd.wrapY)
            {
                yStart = max(yStart, 0);
                yEnd = min(yEnd, yDim);
            }
            LawParams<float> lp;
            lp.scale = k;
            lp.exponent = 1.0f;
            const float xDimF = static_cast<float>(xDim);
            const float yDimF = static_cast<float>(yDim);
            float vx = 0.0f, vy = 0.0f, sum = 0.0f;
            const int32_t sh = wd.binShift;
            const int32_t nRows = xEnd - xStart;
            if (sh == 0 && nRows > 0 && nRows <= 4 && yStart >= 0 && yEnd <= yDim && yEnd > yStart)
            {
                // One cell per bin and a window whose y-range does not wrap:
                // each window row is one run of consecutive bins, so one
                // stretch of slots.  All rows' bounds are loaded before the
                // first candidate; the rows' stretches, one after another,
                // are walked in groups of four whose loads are issued before
                // any of them is used.  The visiting order is unchanged.
                int32_t rs[4], re[4];
#pragma unroll
                for (int j = 0; j < 4; j++)
                {
                    rs[j] = 0;
                    re[j] = 0;
                    if (j < nRows)
                    {
                        int32_t retX = xStart + j;
                        if (retX < 0 || retX >= xDim)
                        {
                            retX %= xDim;  // only reached on a wrapped axis (clamped otherwise)
                            retX = (retX < 0) ? retX + xDim : retX;
                        }
                        const int32_t bin = static_cast<int32_t>(wd.binBase) + retX * wd.binsY + yStart;
                        rs[j] = __ldg(offsets + bin);
                        re[j] = __ldg(offsets + bin + (yEnd - yStart));
                    }
                }
                constexpr int kGroup = 4;
                const int32_t c1 = re[0] - rs[0];
                const int32_t c2 = c1 + (re[1] - rs[1]);
                const int32_t c3 = c2 + (re[2] - rs[2]);
                const int32_t total = c3 + (re[3] - rs[3]);
                for (int32_t k0 = 0; k0 < total; k0 += kGroup)
                {
                    int32_t qs[kGroup];
                    float2 pj[kGroup];
                    float rj[kGroup];
#pragma unroll
                    for (int u = 0; u < kGroup; u++)
                    {
                        const int32_t kk = k0 + u;
                        qs[u] = (kk >= total) ? -1
                                : (kk < c1)   ? rs[0] + kk
                                : (kk < c2)   ? rs[1] + (kk - c1)
                                : (kk < c3)   ? rs[2] + (kk - c2)
                                              : rs[3] + (kk - c3);
                        if (qs[u] >= 0)
                        {
                            pj[u] = sPos[qs[u]];
                            rj[u] = sRad[qs[u]];
                        }
                    }
#pragma unroll
                    for (int u = 0; u < kGroup; u++)
                    {
                        if (qs[u] >= 0 && qs[u] != slot)
                        {
                            PairStep<float, kLawLinear, false, false>(pf.x, pf.y, rad, pj[u], rj[u], R, lp, xDimF,
                                                                      yDimF, wd.wrapX, wd.wrapY, vx, vy, sum);
                        }
                    }
                }
                return make_float2(vx, vy);
            }
            const int32_t bs = 1 << sh;
            for (int32_t xSq = xStart; xSq < xEnd; xSq++)
            {
                int32_t retX = xSq;
                if (retX < 0 || retX >= xDim)
                {
                    retX %= xDim;  // only reached on a wrapped axis (clamped otherwise)
                    retX = (retX < 0) ? retX + xDim : retX;
                }
                const int32_t binRow = static_cast<int32_t>(wd.binBase) + (retX >> sh) * wd.binsY;
                // the row's window cells as runs that stay in one bin and do
                // not wrap: a run's cells are consecutive cell indices, so its
                // agents are one stretch of the bin's (cell, index) order
                for (int32_t ySq = yStart; ySq < yEnd;)
                {
                    int32_t retY = ySq;
                    if (retY < 0 || retY >= yDim)
                    {
                        retY %= yDim;  // only reached on a wrapped axis (clamped otherwise)
                        retY = (retY < 0) ? retY + yDim : retY;
                    }
                    const int32_t by = retY >> sh;
                    const int32_t binEnd = min((by + 1) * bs, yDim);  // first y past the bin
                    const int32_t run = min(yEnd - ySq, binEnd - retY);
                    ySq += run;
                    const int32_t cLo = retX * yDim + retY;
                    const int32_t cHi = cLo + run - 1;
                    const int32_t s = __ldg(offsets + binRow + by);
                    const int32_t e = __ldg(offsets + binRow + by + 1);
                    for (int32_t t = s; t < e; t++)
                    {
                        const int32_t ct = __ldg(sCell + t);
                        if (ct > cHi)
                        {
                            break;  // the bin is ordered by cell
                        }
                        if (ct >= cLo && t != slot)
                        {
                            PairStep<float, kLawLinear, false, false>(pf.x, pf.y, rad, sPos[t], sRad[t], R, lp, xDimF,
                                                                      yDimF, wd.wrapX, wd.wrapY, vx, vy, sum);
                        }
                    }
                }
            }
            return make_float2(vx, vy);
        }

        __global__ void ForcesWells(const int32_t *__restrict__ bucket, const int32_t *__restrict__ offsets,
                                    const float2 *__restrict__ sPos, const float *__restrict__ sRad,
                                    const int32_t *__restrict__ sCell, const int32_t *__restrict__ wellOf,
                                    const AgentWellDev *__restrict__ wells, int32_t n, double interactionRad, float R,
                                    float k, float *__restrict__ vel)
        {
            ChainEntry();
            const int32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
            if (slot >= n)
            {
                return;
            }
            const int32_t i = bucket[slot];
            const AgentWellDev wd = wells[wellOf[i]];
            StoreDelta(vel, i, ForceSlotWell(slot, offsets, sPos, sRad, sCell, interactionRad, R, k, wd));
        }

        // ForcesWells with each agent's SphericalAgent2D update fused, moved
        // within its own well (its sizes and wrap flags).
        __global__ void ForcesWellsMove(const int32_t *__restrict__ bucket, const int32_t *__restrict__ offsets,
                                        const float2 *__restrict__ sPos, const float *__restrict__ sRad,
                                        const int32_t *__restrict__ sCell, const int32_t *__restrict__ wellOf,
                                        const AgentWellDev *__restrict__ wells, int32_t n, double interactionRad,
                                        float R, float k, float friction, float maxVel, float *__restrict__ vel,
                                        float2 *__restrict__ pos, float2 *__restrict__ velocity)
        {
            ChainEntry();
            const int32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
            if (slot >= n)
            {
                return;
            }
            const int32_t i = bucket[slot];
            const AgentWellDev wd = wells[wellOf[i]];
            const V2<float> d = ForceSlotWell(slot, offsets, sPos, sRad, sCell, interactionRad, R, k, wd);
            StoreDelta(vel, i, d);
            MoveParams mp;
            mp.friction = friction;
            mp.maxVel = maxVel;
            mp.xDimF = static_cast<float>(wd.xDim);
            mp.yDimF = static_cast<float>(wd.yDim);
            mp.wrapX = wd.wrapX;
            mp.wrapY = wd.wrapY;
            float2 p = sPos[slot];
            float2 v = velocity[i];
            v.x = __fadd_rn(v.x, d.x);
            v.y = __fadd_rn(v.y, d.y);
            MoveAgent(mp, p, v);
            pos[i] = p;
            velocity[i] = v;
        }
    }

    struct ForceLawSpec
    {
        int kind = kLawLinear;
        double scale = 0.0;
        double exponent = 1.0;
        bool sums = false;  // write each agent's sum of positive forces
        bool grid = false;  // the agent grid's order and displacement (FP64)

        static ForceLawSpec Linear(double k)
        {
            ForceLawSpec l;
            l.scale = k;
            return l;
        }
    };

    struct Agents
    {
        int32_t xDim = 0, yDim = 0, maxAgents = 0;
        int64_t C = 0;
        int32_t n = 0;          // agents of the last upload
        int device = 0;
        StreamSlot stream;
        DevBuf<float> pos32, rad32, vel32;
        DevBuf<float2> velState;  // the agents' own velocities (xVel, yVel) of the resident step
        DevBuf<double> pos64, rad64, vel64;
        DevBuf<float2> sPos;
        DevBuf<double2> sPosD;  // FP64 interface path
        DevBuf<float> sRad32;
        DevBuf<double> sRad64;
        DevBuf<int32_t> cellOf, arrival, counts, offsets, tileSums, bucketTmp, bucket;
        DevBuf<float> sums32;    // per-agent sums of positive forces (FP32 path)
        DevBuf<double> sums64;   // the same, FP64 path
        bool sumsValid = false;  // sums32 holds the last dispatch's or step's sums
        int32_t nTiles = 0;
        bool countsDirty = true;  // counts not known to be zero (cleared by each scan)
        // counts, cellOf and arrival hold the binning of the current pos32,
        // counted by the last resident step's force kernel as it moved the
        // agents: the next FP32 binning skips its count pass
        bool binsPrecounted = false;

        // pos32 changed by other means than the resident step: the precounted
        // bins are stale and the counts must be cleared before a binning
        void DropPrecount()
        {
            if (binsPrecounted)
            {
                binsPrecounted = false;
                countsDirty = true;
            }
        }

        int Init(int32_t x, int32_t y, int32_t maxN)
        {
            xDim = x;
            yDim = y;
            maxAgents = maxN;
            C = static_cast<int64_t>(x) * y;
            device = CurrentDevice();
            HAL_TRY(CudaStatus(cudaSetDevice(device), "cudaSetDevice"));
            HAL_TRY(stream.Create("cudaStreamCreate"));
            size_t m = static_cast<size_t>(maxN > 0 ? maxN : 1);
            HAL_TRY(pos32.Alloc(2 * m, "cudaMalloc(agents)"));
            HAL_TRY(rad32.Alloc(m, "cudaMalloc(agents)"));
            HAL_TRY(vel32.Alloc(2 * m, "cudaMalloc(agents)"));
            HAL_TRY(velState.Alloc(m, "cudaMalloc(agents)"));
            HAL_TRY(CudaStatus(cudaMemset(velState.p, 0, m * sizeof(float2)), "cudaMemset"));
            HAL_TRY(sPos.Alloc(m, "cudaMalloc(agents)"));
            HAL_TRY(sRad32.Alloc(m, "cudaMalloc(agents)"));
            HAL_TRY(cellOf.Alloc(m, "cudaMalloc(agents)"));
            HAL_TRY(arrival.Alloc(m, "cudaMalloc(agents)"));
            HAL_TRY(bucketTmp.Alloc(m, "cudaMalloc(agents)"));
            HAL_TRY(bucket.Alloc(m, "cudaMalloc(agents)"));
            HAL_TRY(counts.Alloc(static_cast<size_t>(C), "cudaMalloc(bins)"));
            HAL_TRY(offsets.Alloc(static_cast<size_t>(C) + 1, "cudaMalloc(bins)"));
            nTiles = static_cast<int32_t>((C + kScanTile - 1) / kScanTile);
            HAL_TRY(tileSums.Alloc(static_cast<size_t>(nTiles), "cudaMalloc(bins)"));

            HAL_TRY(CudaStatus(cudaMemset(offsets.p, 0, (static_cast<size_t>(C) + 1) * sizeof(int32_t)), "cudaMemset"));
            return HAL_CUDA_OK;
        }

        V2<float> *SortedPosBuf(float) { return sPos.p; }
        V2<double> *SortedPosBuf(double) { return sPosD.p; }

        // Bins n agents (positions of type TP, interleaved x,y, in one of the
        // handle's own device buffers) and sorts radii of type TR alongside.
        // With ev != nullptr, records an event after each stage (count, scan,
        // scatter, stabilize) for profiling.
        template <typename TP, typename TR>
        int Bin(const TP *pos, const TR *rad, TR *sRad, cudaStream_t s, cudaEvent_t *ev = nullptr)
        {
            // the resident step's force kernel already counted these positions
            const bool pre = binsPrecounted && static_cast<const void *>(pos) == static_cast<const void *>(pos32.p);
            if (!pre)
            {
                DropPrecount();
            }
            binsPrecounted = false;
            if (countsDirty && !pre)
            {
                // a previous binning stopped before its scan cleared the counts
                HAL_TRY(CudaStatus(cudaMemsetAsync(counts.p, 0, static_cast<size_t>(C) * sizeof(int32_t), s),
                                   "cudaMemsetAsync(counts)"));
            }
            countsDirty = true;
            const int T = 256;
            unsigned ablocks = static_cast<unsigned>((n + T - 1) / T);
            if (n > 0 && !pre)
            {
                LaunchChained(BinCount<TP>, ablocks, T, s, pos, n, xDim, yDim, static_cast<V2<TP> *>(nullptr),
                              cellOf.p, arrival.p, counts.p);
                CountLaunch();
            }
            if (ev)
            {
                cudaEventRecord(ev[0], s);
            }
            LaunchChained(ScanReduce, nTiles, kScanThreads, s, counts.p, C, tileSums.p);
            if (nTiles <= kScanSumTiles)
            {
                LaunchChained(ScanApplySum, nTiles, kScanThreads, s, counts.p, C, tileSums.p, offsets.p, n);
                CountLaunch(2);
            }
            else
            {
                LaunchChained(ScanTiles, 1u, kScanThreads, s, tileSums.p, nTiles);
                LaunchChained(ScanApply<true>, nTiles, kScanThreads, s, counts.p, C, tileSums.p, offsets.p, n);
                CountLaunch(3);
            }
            countsDirty = (cudaPeekAtLastError() != cudaSuccess);
            if (ev)
            {
                cudaEventRecord(ev[1], s);
            }
            if (n > 0)
            {
                LaunchChained(Scatter, ablocks, T, s, cellOf.p, arrival.p, offsets.p, n, bucketTmp.p);
                CountLaunch();
            }
            if (ev)
            {
                cudaEventRecord(ev[2], s);
            }
            if (n > 0)
            {
                // pos is the handle's own device buffer (cudaMalloc'd, so
                // aligned for V2<TP>)
                LaunchChained(StabilizeSlots<TP, TR>, ablocks, T, s, offsets.p, bucketTmp.p,
                              reinterpret_cast<const V2<TP> *>(pos), rad, n, xDim, yDim, bucket.p, SortedPosBuf(TP()),
                              sRad);
                CountLaunch();
            }
            if (ev)
            {
                cudaEventRecord(ev[3], s);
            }
            return LaunchStatus("agent binning");
        }

        // Pass 4 with force law `law`: velocity deltas (from zero, or from
        // velIn) into vel, and with law.sums each agent's sum of positive
        // forces into sums.  law.grid (FP64 only) selects the agent grid's
        // visiting order and displacement.
        template <typename T, typename TV>
        int Force(const T *sRad, double R, const ForceLawSpec &law, bool wrapX, bool wrapY, TV *vel, T *sums,
                  const TV *velIn, cudaStream_t s)
        {
            if (n == 0)
            {
                return HAL_CUDA_OK;
            }
            const int T_ = 128;
            const unsigned blocks = static_cast<unsigned>((n + T_ - 1) / T_);
            LawParams<T> lp;
            lp.scale = static_cast<T>(law.scale);
            lp.exponent = static_cast<T>(law.exponent);
            auto go = [&](auto kernel) {
                LaunchChained(kernel, blocks, T_, s, bucket.p, offsets.p, SortedPosBuf(T()), sRad, n, R,
                              static_cast<T>(R), lp, xDim, yDim, static_cast<int32_t>(wrapX),
                              static_cast<int32_t>(wrapY), vel, sums, velIn);
            };
            const bool grid = std::is_same<T, double>::value && law.grid;
            switch (law.kind * 4 + (law.sums ? 2 : 0) + (grid ? 1 : 0))
            {
            case 0:
                // the interface's law on a grid with walls: the wrap tests compiled out
                if constexpr (std::is_same<T, float>::value)
                {
                    if (!wrapX && !wrapY)
                    {
                        go(Forces<T, TV, kLawLinear, false, false, true>);
                        break;
                    }
                }
                go(Forces<T, TV, kLawLinear, false, false>);
                break;
            case 1: go(Forces<T, TV, kLawLinear, false, true>); break;
            case 2: go(Forces<T, TV, kLawLinear, true, false>); break;
            case 3: go(Forces<T, TV, kLawLinear, true, true>); break;
            case 4: go(Forces<T, TV, kLawClamped, false, false>); break;
            case 5: go(Forces<T, TV, kLawClamped, false, true>); break;
            case 6: go(Forces<T, TV, kLawClamped, true, false>); break;
            case 7: go(Forces<T, TV, kLawClamped, true, true>); break;
            case 8: go(Forces<T, TV, kLawPower, false, false>); break;
            case 9: go(Forces<T, TV, kLawPower, false, true>); break;
            case 10: go(Forces<T, TV, kLawPower, true, false>); break;
            default: go(Forces<T, TV, kLawPower, true, true>); break;
            }
            CountLaunch();
            return LaunchStatus("agent forces");
        }

        // The interface's pass 4: linear law, deltas from zero.
        template <typename T, typename TV>
        int Force(const T *sRad, double R, double k, bool wrapX, bool wrapY, TV *vel, cudaStream_t s)
        {
            return Force<T, TV>(sRad, R, ForceLawSpec::Linear(k), wrapX, wrapY, vel, static_cast<T *>(nullptr),
                                static_cast<const TV *>(nullptr), s);
        }

        // Buffer of the FP32 force sums, allocated on first use.
        int SumsBuf32(float **out)
        {
            if (sums32.p == nullptr)
            {
                HAL_TRY(sums32.Alloc(static_cast<size_t>(maxAgents > 0 ? maxAgents : 1), "cudaMalloc(force sums)"));
            }
            *out = sums32.p;
            return HAL_CUDA_OK;
        }
    };

    const int32_t *AgentsCellOffsets(const hal_cuda_agents *a, int32_t *xDim, int32_t *yDim);
}

namespace
{
    // One resident tick of the agents: bin, then forces with the move fused.
    int StepOnce(halcuda::Agents &a, double R, const halcuda::ForceLawSpec &law, const halcuda::MoveParams &mp,
                 cudaStream_t s)
    {
        using namespace halcuda;
        HAL_TRY((a.Bin<float, float>(a.pos32.p, a.rad32.p, a.sRad32.p, s)));
        if (a.n == 0)
        {
            return HAL_CUDA_OK;
        }
        float *sums = nullptr;
        if (law.sums)
        {
            HAL_TRY(a.SumsBuf32(&sums));
        }
        const int T = 128;
        const unsigned blocks = static_cast<unsigned>((a.n + T - 1) / T);
        LawParams<float> lp;
        lp.scale = static_cast<float>(law.scale);
        lp.exponent = static_cast<float>(law.exponent);
        // the force kernel counts the moved agents into their new cells (the
        // next binning's count pass); this binning's scan cleared the counts
        auto go = [&](auto kernel) {
            LaunchChained(kernel, blocks, T, s, a.bucket.p, a.offsets.p, a.sPos.p, a.sRad32.p, a.n, R,
                          static_cast<float>(R), lp, a.xDim, a.yDim, mp, a.vel32.p,
                          reinterpret_cast<float2 *>(a.pos32.p), a.velState.p, sums, a.cellOf.p, a.arrival.p,
                          a.counts.p);
        };
        switch (law.kind * 2 + (law.sums ? 1 : 0))
        {
        case 0:
            if (!mp.wrapX && !mp.wrapY)
            {
                go(ForcesMove<kLawLinear, false, true>);  // walls: the wrap tests compiled out
            }
            else
            {
                go(ForcesMove<kLawLinear, false>);
            }
            break;
        case 1: go(ForcesMove<kLawLinear, true>); break;
        case 2: go(ForcesMove<kLawClamped, false>); break;
        case 3: go(ForcesMove<kLawClamped, true>); break;
        case 4: go(ForcesMove<kLawPower, false>); break;
        default: go(ForcesMove<kLawPower, true>); break;
        }
        CountLaunch();
        const int rc = LaunchStatus("agent forces and move");
        a.binsPrecounted = (rc == HAL_CUDA_OK);
        a.countsDirty = (rc != HAL_CUDA_OK);
        return rc;
    }
}

using halcuda::Agents;

struct hal_cuda_agents : public Agents
{
};

namespace halcuda
{
    AgentBinsView AgentsBins(const hal_cuda_agents *a)
    {
        AgentBinsView v;
        v.offsets = a->offsets.p;
        v.bucket = a->bucket.p;
        v.cellOf = a->cellOf.p;
        v.n = a->n;
        v.xDim = a->xDim;
        v.yDim = a->yDim;
        v.device = a->device;
        v.stream = a->stream.Get();
        return v;
    }

    const int32_t *AgentsCellOffsets(const hal_cuda_agents *a, int32_t *xDim, int32_t *yDim)
    {
        *xDim = a->xDim;
        *yDim = a->yDim;
        return a->offsets.p;
    }
}

extern "C" int hal_cuda_agents_create(int32_t xDim, int32_t yDim, int32_t maxAgents, hal_cuda_agents **out)
{
    HAL_REQUIRE(out != nullptr, "hal_cuda_agents_create: out is NULL");
    *out = nullptr;
    HAL_REQUIRE(xDim > 0 && yDim > 0, "hal_cuda_agents_create: dimensions must be positive");
    HAL_REQUIRE(static_cast<int64_t>(xDim) * yDim < (int64_t(1) << 31) - 1,
                "hal_cuda_agents_create: xDim*yDim exceeds int32");
    HAL_REQUIRE(maxAgents >= 0, "hal_cuda_agents_create: negative capacity");
    hal_cuda_agents *h = new (std::nothrow) hal_cuda_agents();
    if (h == nullptr)
    {
        halcuda::SetError("hal_cuda_agents_create: out of host memory");
        return HAL_CUDA_ENOMEM;
    }
    int rc = h->Init(xDim, yDim, maxAgents);
    if (rc != HAL_CUDA_OK)
    {
        delete h;
        return rc;
    }
    *out = h;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_agents_destroy(hal_cuda_agents *h)
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
    // The cell window spans about 2R cells per axis; a wrapped axis walks all
    // of it, so the radius is bounded to keep every launch short.
    constexpr double kMaxInteractionRad = 1048576.0;

    bool RadiusOk(double r)
    {
        return std::isfinite(r) && r >= 0.0 && r <= kMaxInteractionRad;
    }
}

namespace
{
    // A hal_cuda_force_law checked and turned into a spec; sums as given.
    int LawFrom(const hal_cuda_force_law *law, bool sums, const char *who, halcuda::ForceLawSpec *out)
    {
        HAL_REQUIRE(law != nullptr, "%s: law is NULL", who);
        HAL_REQUIRE(law->kind == HAL_CUDA_FORCE_LINEAR || law->kind == HAL_CUDA_FORCE_LINEAR_CLAMPED ||
                        law->kind == HAL_CUDA_FORCE_POWER,
                    "%s: unknown force law kind %d", who, law->kind);
        HAL_REQUIRE(std::isfinite(law->scale), "%s: the law's scale must be finite", who);
        HAL_REQUIRE(law->kind != HAL_CUDA_FORCE_POWER || std::isfinite(law->exponent),
                    "%s: the law's exponent must be finite", who);
        out->kind = law->kind;
        out->scale = law->scale;
        out->exponent = (law->kind == HAL_CUDA_FORCE_POWER) ? law->exponent : 1.0;
        out->sums = sums;
        out->grid = false;
        return HAL_CUDA_OK;
    }

    // The FP64 interface path's buffers, allocated on its first call.
    int Ensure64(hal_cuda_agents *h)
    {
        if (h->sPosD.p == nullptr)  // the last of the FP64 buffers: all or none are allocated
        {
            size_t m = static_cast<size_t>(h->maxAgents > 0 ? h->maxAgents : 1);
            HAL_TRY(h->pos64.Alloc(2 * m, "cudaMalloc(agents64)"));
            HAL_TRY(h->rad64.Alloc(m, "cudaMalloc(agents64)"));
            HAL_TRY(h->vel64.Alloc(2 * m, "cudaMalloc(agents64)"));
            HAL_TRY(h->sRad64.Alloc(m, "cudaMalloc(agents64)"));
            HAL_TRY(h->sPosD.Alloc(m, "cudaMalloc(agents64)"));
        }
        return HAL_CUDA_OK;
    }
}

extern "C" int hal_cuda_accumulate_forces(hal_cuda_agents *h, const double *positions, int64_t posLen,
                                          const double *radii, int64_t radLen, double *velocityDeltas,
                                          double interactionRad, double springConstant, int32_t xDim, int32_t yDim,
                                          int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr, "hal_cuda_accumulate_forces: handle is NULL");
    HAL_REQUIRE(xDim == h->xDim && yDim == h->yDim,
                "CudaAgentForceBackend2D::AccumulateForces called with dimensions differing from construction");
    HAL_REQUIRE(posLen == 2 * radLen && radLen >= 0,
                "CudaAgentForceBackend2D::AccumulateForces: positions must hold two values per radius");
    HAL_REQUIRE(radLen <= h->maxAgents,
                "CudaAgentForceBackend2D::AccumulateForces called with more agents than the construction-time capacity");
    HAL_REQUIRE(radLen == 0 || (positions != nullptr && radii != nullptr && velocityDeltas != nullptr),
                "hal_cuda_accumulate_forces: NULL array");
    HAL_REQUIRE(RadiusOk(interactionRad), "hal_cuda_accumulate_forces: interactionRad %g outside [0, %g]",
                interactionRad, kMaxInteractionRad);
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    HAL_TRY(Ensure64(h));
    cudaStream_t s = h->stream.Get();
    h->n = static_cast<int32_t>(radLen);
    if (h->n > 0)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->pos64.p, positions, posLen * sizeof(double), cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(positions)"));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->rad64.p, radii, radLen * sizeof(double), cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(radii)"));
    }
    HAL_TRY((h->Bin<double, double>(h->pos64.p, h->rad64.p, h->sRad64.p, s)));
    HAL_TRY((h->Force<double, double>(h->sRad64.p, interactionRad, springConstant, wrapX != 0, wrapY != 0,
                                      h->vel64.p, s)));
    if (h->n > 0)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(velocityDeltas, h->vel64.p, posLen * sizeof(double), cudaMemcpyDeviceToHost, s),
                           "cudaMemcpy(velocityDeltas)"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_accumulate_forces");
}

extern "C" int hal_cuda_sum_forces(hal_cuda_agents *h, const double *positions, const double *radii, int64_t n,
                                   const double *velocities, double *velocitiesOut, double *forceSums,
                                   double interactionRad, const hal_cuda_force_law *law, int32_t order,
                                   int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
    const char *who = "hal_cuda_sum_forces";
    HAL_REQUIRE(h != nullptr, "%s: handle is NULL", who);
    HAL_REQUIRE(xDim == h->xDim && yDim == h->yDim,
                "CudaAgentForceBackend2D::SumForces called with dimensions differing from construction");
    HAL_REQUIRE(n >= 0 && n <= h->maxAgents,
                "CudaAgentForceBackend2D::SumForces called with more agents than the construction-time capacity");
    HAL_REQUIRE(n == 0 || (positions != nullptr && radii != nullptr && velocitiesOut != nullptr),
                "%s: NULL array", who);
    HAL_REQUIRE(RadiusOk(interactionRad), "%s: interactionRad %g outside [0, %g]", who, interactionRad,
                kMaxInteractionRad);
    HAL_REQUIRE(order == HAL_CUDA_ORDER_BACKEND || order == HAL_CUDA_ORDER_AGENTGRID, "%s: unknown order %d", who,
                order);
    halcuda::ForceLawSpec spec;
    HAL_TRY(LawFrom(law, forceSums != nullptr, who, &spec));
    spec.grid = (order == HAL_CUDA_ORDER_AGENTGRID);
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    HAL_TRY(Ensure64(h));
    if (forceSums != nullptr && h->sums64.p == nullptr)
    {
        HAL_TRY(h->sums64.Alloc(static_cast<size_t>(h->maxAgents > 0 ? h->maxAgents : 1), "cudaMalloc(force sums)"));
    }
    cudaStream_t s = h->stream.Get();
    h->n = static_cast<int32_t>(n);
    h->sumsValid = false;  // the FP32 sums are not this call's
    const size_t bytes2 = 2 * static_cast<size_t>(n) * sizeof(double);
    if (n > 0)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->pos64.p, positions, bytes2, cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(positions)"));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->rad64.p, radii, static_cast<size_t>(n) * sizeof(double),
                                           cudaMemcpyHostToDevice, s), "cudaMemcpy(radii)"));
        if (velocities != nullptr)
        {
            HAL_TRY(CudaStatus(cudaMemcpyAsync(h->vel64.p, velocities, bytes2, cudaMemcpyHostToDevice, s),
                               "cudaMemcpy(velocities)"));
        }
    }
    HAL_TRY((h->Bin<double, double>(h->pos64.p, h->rad64.p, h->sRad64.p, s)));
    // velocities in place: each thread reads and writes only its own agent
    HAL_TRY((h->Force<double, double>(h->sRad64.p, interactionRad, spec, wrapX != 0, wrapY != 0, h->vel64.p,
                                      forceSums != nullptr ? h->sums64.p : nullptr,
                                      velocities != nullptr ? h->vel64.p : nullptr, s)));
    if (n > 0)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(velocitiesOut, h->vel64.p, bytes2, cudaMemcpyDeviceToHost, s),
                           "cudaMemcpy(velocities)"));
        if (forceSums != nullptr)
        {
            HAL_TRY(CudaStatus(cudaMemcpyAsync(forceSums, h->sums64.p, static_cast<size_t>(n) * sizeof(double),
                                               cudaMemcpyDeviceToHost, s), "cudaMemcpy(force sums)"));
        }
    }
    return CudaStatus(cudaStreamSynchronize(s), who);
}

extern "C" int hal_cuda_agents_upload(hal_cuda_agents *h, const float *positions, const float *radii, int32_t n)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_agents_upload: handle is NULL");
    HAL_REQUIRE(n >= 0 && n <= h->maxAgents, "AgentForceKernel2D::UploadAgents: agent count %d outside [0, %d]", n,
                h->maxAgents);
    HAL_REQUIRE(n == 0 || (positions != nullptr && radii != nullptr), "hal_cuda_agents_upload: NULL array");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    h->DropPrecount();
    h->n = n;
    if (n > 0)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->pos32.p, positions, 2 * static_cast<size_t>(n) * sizeof(float),
                                           cudaMemcpyHostToDevice, s), "cudaMemcpy(positions)"));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->rad32.p, radii, static_cast<size_t>(n) * sizeof(float),
                                           cudaMemcpyHostToDevice, s), "cudaMemcpy(radii)"));
        HAL_TRY(CudaStatus(cudaMemsetAsync(h->velState.p, 0, static_cast<size_t>(n) * sizeof(float2), s),
                           "cudaMemsetAsync(velocities)"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_agents_upload");
}

extern "C" int hal_cuda_agents_set_velocities(hal_cuda_agents *h, const float *velocities, int32_t n)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_agents_set_velocities: handle is NULL");
    HAL_REQUIRE(n == h->n, "hal_cuda_agents_set_velocities: %d agents given, %d uploaded", n, h->n);
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    if (n > 0)
    {
        const size_t bytes = static_cast<size_t>(n) * sizeof(float2);
        HAL_TRY(CudaStatus(velocities != nullptr
                               ? cudaMemcpyAsync(h->velState.p, velocities, bytes, cudaMemcpyHostToDevice, s)
                               : cudaMemsetAsync(h->velState.p, 0, bytes, s),
                           "hal_cuda_agents_set_velocities"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_agents_set_velocities");
}

extern "C" int hal_cuda_agents_get_state(hal_cuda_agents *h, float *positions, float *velocities, int32_t n)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_agents_get_state: handle is NULL");
    HAL_REQUIRE(n == h->n, "hal_cuda_agents_get_state: %d agents requested, %d uploaded", n, h->n);
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    const size_t bytes = static_cast<size_t>(n) * sizeof(float2);
    if (n > 0 && positions != nullptr)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(positions, h->pos32.p, bytes, cudaMemcpyDeviceToHost, s),
                           "cudaMemcpy(positions)"));
    }
    if (n > 0 && velocities != nullptr)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(velocities, h->velState.p, bytes, cudaMemcpyDeviceToHost, s),
                           "cudaMemcpy(velocities)"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_agents_get_state");
}

namespace halcuda
{
    // ---- resident steps inside another handle's run (hal_cuda_adi_run_coupled)

    int CoupledStepBegin(hal_cuda_agents *h, const CoupledStep &st, cudaStream_t s)
    {
        HAL_REQUIRE(h != nullptr, "hal_cuda_adi_run_coupled: agent handle is NULL");
        HAL_REQUIRE(RadiusOk(st.interactionRad), "hal_cuda_adi_run_coupled: interactionRad %g outside [0, %g]",
                    st.interactionRad, kMaxInteractionRad);
        HAL_REQUIRE(std::isfinite(st.springConstant), "hal_cuda_adi_run_coupled: springConstant must be finite");
        HAL_REQUIRE(std::isfinite(st.friction), "hal_cuda_adi_run_coupled: friction must be finite");
        HAL_REQUIRE(!std::isnan(st.maxVel), "hal_cuda_adi_run_coupled: maxVel is NaN");
        HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
        // the agent handle's own queued work comes first
        cudaStream_t own = h->stream.Get();
        if (own != s)
        {
            cudaEvent_t ev = nullptr;
            HAL_TRY(CudaStatus(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate"));
            cudaError_t e = cudaEventRecord(ev, own);
            if (e == cudaSuccess)
            {
                e = cudaStreamWaitEvent(s, ev, 0);
            }
            cudaEventDestroy(ev);
            HAL_TRY(CudaStatus(e, "hal_cuda_adi_run_coupled: stream order"));
        }
        // every replayed tick starts from counts that hold the current
        // positions' binning (the previous tick's force kernel counted them)
        if (!h->binsPrecounted && h->n > 0)
        {
            if (h->countsDirty)
            {
                HAL_TRY(CudaStatus(cudaMemsetAsync(h->counts.p, 0, static_cast<size_t>(h->C) * sizeof(int32_t), s),
                                   "cudaMemsetAsync(counts)"));
            }
            const int T = 256;
            BinCount<float><<<static_cast<unsigned>((h->n + T - 1) / T), T, 0, s>>>(
                h->pos32.p, h->n, h->xDim, h->yDim, static_cast<float2 *>(nullptr), h->cellOf.p, h->arrival.p,
                h->counts.p);
            CountLaunch();
            HAL_TRY(LaunchStatus("agent binning"));
            h->binsPrecounted = true;
            h->countsDirty = false;
        }
        h->sumsValid = false;
        return HAL_CUDA_OK;
    }

    int CoupledStepOnce(hal_cuda_agents *h, const CoupledStep &st, int32_t wrapX, int32_t wrapY, cudaStream_t s)
    {
        MoveParams mp;
        mp.friction = static_cast<float>(st.friction);
        mp.maxVel = (st.maxVel < 0 || std::isinf(st.maxVel)) ? -1.0f : static_cast<float>(st.maxVel);
        mp.xDimF = static_cast<float>(h->xDim);
        mp.yDimF = static_cast<float>(h->yDim);
        mp.wrapX = wrapX != 0;
        mp.wrapY = wrapY != 0;
        return StepOnce(*h, st.interactionRad, ForceLawSpec::Linear(st.springConstant), mp, s);
    }

    int CoupledStepEnd(hal_cuda_agents *h, cudaStream_t s)
    {
        // the agent handle's later work waits for the run
        cudaStream_t own = h->stream.Get();
        if (own == s)
        {
            return HAL_CUDA_OK;
        }
        cudaEvent_t ev = nullptr;
        HAL_TRY(CudaStatus(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate"));
        cudaError_t e = cudaEventRecord(ev, s);
        if (e == cudaSuccess)
        {
            e = cudaStreamWaitEvent(own, ev, 0);
        }
        cudaEventDestroy(ev);
        return CudaStatus(e, "hal_cuda_adi_run_coupled: stream order");
    }

    int32_t CoupledAgentCount(const hal_cuda_agents *h)
    {
        return h->n;
    }

    bool CoupledBinsPrecounted(const hal_cuda_agents *h)
    {
        return h->binsPrecounted;
    }
}

namespace
{
    int StepCommon(hal_cuda_agents *h, int32_t ticks, double interactionRad, const halcuda::ForceLawSpec &law,
                   int32_t wrapX, int32_t wrapY, double friction, double maxVel, const char *who)
    {
        HAL_REQUIRE(h != nullptr, "%s: handle is NULL", who);
        HAL_REQUIRE(ticks >= 0, "%s: ticks must be >= 0", who);
        HAL_REQUIRE(RadiusOk(interactionRad), "%s: interactionRad %g outside [0, %g]", who, interactionRad,
                    kMaxInteractionRad);
        HAL_REQUIRE(std::isfinite(friction), "%s: friction must be finite", who);
        HAL_REQUIRE(!std::isnan(maxVel), "%s: maxVel is NaN", who);
        using namespace halcuda;
        HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
        cudaStream_t s = h->stream.Get();
        MoveParams mp;
        mp.friction = static_cast<float>(friction);
        mp.maxVel = (maxVel < 0 || std::isinf(maxVel)) ? -1.0f : static_cast<float>(maxVel);
        mp.xDimF = static_cast<float>(h->xDim);
        mp.yDimF = static_cast<float>(h->yDim);
        mp.wrapX = wrapX != 0;
        mp.wrapY = wrapY != 0;
        h->sumsValid = false;
        for (int32_t t = 0; t < ticks; t++)
        {
            HAL_TRY(StepOnce(*h, interactionRad, law, mp, s));
        }
        h->sumsValid = law.sums && ticks > 0;
        return HAL_CUDA_OK;
    }

    int DispatchCommon(hal_cuda_agents *h, double interactionRad, const halcuda::ForceLawSpec &law, int32_t wrapX,
                       int32_t wrapY, const char *who)
    {
        HAL_REQUIRE(h != nullptr, "%s: handle is NULL", who);
        HAL_REQUIRE(RadiusOk(interactionRad), "%s: interactionRad %g outside [0, %g]", who, interactionRad,
                    kMaxInteractionRad);
        using namespace halcuda;
        HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
        cudaStream_t s = h->stream.Get();
        h->sumsValid = false;
        HAL_TRY((h->Bin<float, float>(h->pos32.p, h->rad32.p, h->sRad32.p, s)));
        float *sums = nullptr;
        if (law.sums)
        {
            HAL_TRY(h->SumsBuf32(&sums));
        }
        HAL_TRY((h->Force<float, float>(h->sRad32.p, interactionRad, law, wrapX != 0, wrapY != 0, h->vel32.p, sums,
                                        static_cast<const float *>(nullptr), s)));
        h->sumsValid = law.sums;
        return HAL_CUDA_OK;
    }
}

extern "C" int hal_cuda_agents_step(hal_cuda_agents *h, int32_t ticks, double interactionRad, double springConstant,
                                    int32_t wrapX, int32_t wrapY, double friction, double maxVel)
{
    HAL_TRACE();
    return StepCommon(h, ticks, interactionRad, halcuda::ForceLawSpec::Linear(springConstant), wrapX, wrapY, friction,
                      maxVel, "hal_cuda_agents_step");
}

extern "C" int hal_cuda_agents_step_law(hal_cuda_agents *h, int32_t ticks, double interactionRad,
                                        const hal_cuda_force_law *law, int32_t withSums, int32_t wrapX,
                                        int32_t wrapY, double friction, double maxVel)
{
    HAL_TRACE();
    halcuda::ForceLawSpec spec;
    HAL_TRY(LawFrom(law, withSums != 0, "hal_cuda_agents_step_law", &spec));
    return StepCommon(h, ticks, interactionRad, spec, wrapX, wrapY, friction, maxVel, "hal_cuda_agents_step_law");
}

extern "C" int hal_cuda_agents_dispatch(hal_cuda_agents *h, double interactionRad, double springConstant,
                                        int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
    return DispatchCommon(h, interactionRad, halcuda::ForceLawSpec::Linear(springConstant), wrapX, wrapY,
                          "hal_cuda_agents_dispatch");
}

extern "C" int hal_cuda_agents_dispatch_law(hal_cuda_agents *h, double interactionRad, const hal_cuda_force_law *law,
                                            int32_t withSums, int32_t wrapX, int32_t wrapY)
{
    HAL_TRACE();
    halcuda::ForceLawSpec spec;
    HAL_TRY(LawFrom(law, withSums != 0, "hal_cuda_agents_dispatch_law", &spec));
    return DispatchCommon(h, interactionRad, spec, wrapX, wrapY, "hal_cuda_agents_dispatch_law");
}

extern "C" int hal_cuda_agents_get_force_sums(hal_cuda_agents *h, float *forceSums, int32_t n)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_agents_get_force_sums: handle is NULL");
    HAL_REQUIRE(n == h->n, "hal_cuda_agents_get_force_sums: %d agents requested, %d uploaded", n, h->n);
    HAL_REQUIRE(n == 0 || forceSums != nullptr, "hal_cuda_agents_get_force_sums: NULL array");
    HAL_REQUIRE(h->sumsValid || n == 0,
                "hal_cuda_agents_get_force_sums: the last dispatch or step did not compute force sums");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    if (n > 0)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(forceSums, h->sums32.p, static_cast<size_t>(n) * sizeof(float),
                                           cudaMemcpyDeviceToHost, s), "cudaMemcpy(force sums)"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_agents_get_force_sums");
}

extern "C" int hal_cuda_agents_download(hal_cuda_agents *h, float *velocityDeltas, int32_t n)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_agents_download: handle is NULL");
    HAL_REQUIRE(n == h->n, "hal_cuda_agents_download: %d agents requested, %d uploaded", n, h->n);
    HAL_REQUIRE(n == 0 || velocityDeltas != nullptr, "hal_cuda_agents_download: NULL array");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    if (n > 0)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(velocityDeltas, h->vel32.p, 2 * static_cast<size_t>(n) * sizeof(float),
                                           cudaMemcpyDeviceToHost, s), "cudaMemcpy(velocityDeltas)"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_agents_download");
}

extern "C" int hal_cuda_agents_get_bins(hal_cuda_agents *h, int32_t *cellOffsets, int32_t *bucketAgents)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_agents_get_bins: handle is NULL");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    if (cellOffsets != nullptr)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(cellOffsets, h->offsets.p, (static_cast<size_t>(h->C) + 1) * sizeof(int32_t),
                                           cudaMemcpyDeviceToHost, s), "cudaMemcpy(offsets)"));
    }
    if (bucketAgents != nullptr && h->n > 0)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(bucketAgents, h->bucket.p, static_cast<size_t>(h->n) * sizeof(int32_t),
                                           cudaMemcpyDeviceToHost, s), "cudaMemcpy(bucket)"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_agents_get_bins");
}

extern "C" int hal_cuda_agents_sync(hal_cuda_agents *h)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_agents_sync: handle is NULL");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return halcuda::CudaStatus(cudaStreamSynchronize(h->stream.Get()), "hal_cuda_agents_sync");
}

extern "C" void *hal_cuda_agents_stream(hal_cuda_agents *h)
{
    return h ? static_cast<void *>(h->stream.Get()) : nullptr;
}

extern "C" int hal_cuda_agents_set_stream(hal_cuda_agents *h, void *stream)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_agents_set_stream: handle is NULL");
    h->stream.Set(stream);
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_agents_profile(hal_cuda_agents *h, int32_t iters, double interactionRad, double springConstant,
                                       int32_t wrapX, int32_t wrapY, float *ms)
{
    HAL_REQUIRE(h != nullptr && ms != nullptr, "hal_cuda_agents_profile: NULL argument");
    HAL_REQUIRE(iters > 0, "hal_cuda_agents_profile: iters must be positive");
    HAL_REQUIRE(RadiusOk(interactionRad), "hal_cuda_agents_profile: interactionRad out of range");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    cudaEvent_t ev[6];
    for (auto &e : ev)
    {
        HAL_TRY(CudaStatus(cudaEventCreate(&e), "cudaEventCreate"));
    }
    double acc[6] = {0, 0, 0, 0, 0, 0};
    int rc = HAL_CUDA_OK;
    for (int32_t t = 0; t < iters && rc == HAL_CUDA_OK; t++)
    {
        cudaEventRecord(ev[5], s);
        rc = h->Bin<float, float>(h->pos32.p, h->rad32.p, h->sRad32.p, s, ev);
        if (rc == HAL_CUDA_OK)
        {
            rc = h->Force<float, float>(h->sRad32.p, interactionRad, springConstant, wrapX != 0, wrapY != 0,
                                        h->vel32.p, s);
        }
        cudaEventRecord(ev[4], s);
        if (rc == HAL_CUDA_OK)
        {
            rc = CudaStatus(cudaEventSynchronize(ev[4]), "hal_cuda_agents_profile");
        }
        if (rc != HAL_CUDA_OK)
        {
            break;
        }
        float t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, tall = 0;
        cudaEventElapsedTime(&t0, ev[5], ev[0]);
        cudaEventElapsedTime(&t1, ev[0], ev[1]);
        cudaEventElapsedTime(&t2, ev[1], ev[2]);
        cudaEventElapsedTime(&t3, ev[2], ev[3]);
        cudaEventElapsedTime(&t4, ev[3], ev[4]);
        cudaEventElapsedTime(&tall, ev[5], ev[4]);
        acc[0] += t0;
        acc[1] += t1;
        acc[2] += t2;
        acc[3] += t3;
        acc[4] += t4;
        acc[5] += tall;
    }
    for (auto &e : ev)
    {
        cudaEventDestroy(e);
    }
    HAL_TRY(rc);
    for (int q = 0; q < 6; q++)
    {
        ms[q] = static_cast<float>(acc[q] / iters);
    }
    return HAL_CUDA_OK;
}

// ---------------------------------------------------------------------------
// Agent forces without allocation.
//
// Some callers cannot call cudaMalloc: a host framework that reserves its
// device memory in its own pool at start-up and forbids cudaMalloc/cudaFree in
// its step loop (both synchronise the whole device and stall the framework's
// other streams), or a plugin whose host budgets device memory and hands it
// only pointers to inputs and outputs.  For them this entry point runs the same
// binning and force kernels as hal_cuda_agents_dispatch with every piece of
// scratch taken from one file-scope device array of fixed size, so it needs no
// handle and allocates nothing.  The caller passes device pointers to the
// positions, radii and velocity deltas.
//
// The array is a static __device__ variable: every GPU that loads this library
// holds it (HAL_CUDA_NOALLOC_SCRATCH_BYTES) until the process exits.  In host
// code its name is only a host-side stand-in, so its device address is looked
// up once per device with cudaGetSymbolAddress, with that device current,
// on the first call made on that device.  All calls share it and it keeps the
// last call's contents; the cell counts, the only part that must start at
// zero, are cleared on the caller's stream at the start of each call.
// ---------------------------------------------------------------------------
#include <cuda.h>
#include <mutex>

namespace
{
    constexpr size_t kNoAllocMaxAgents = HAL_CUDA_NOALLOC_MAX_AGENTS;
    constexpr size_t kNoAllocMaxCells = HAL_CUDA_NOALLOC_MAX_CELLS;
    constexpr size_t kNoAllocMaxTiles = (kNoAllocMaxCells + halcuda::kScanTile - 1) / halcuda::kScanTile;

    constexpr size_t Round256(size_t b)
    {
        return (b + 255) / 256 * 256;
    }

    // Byte offsets of the regions of the scratch array (each 256-byte aligned).
    constexpr size_t kOffPosF = 0;
    constexpr size_t kOffSPos = kOffPosF + Round256(kNoAllocMaxAgents * sizeof(float2));
    constexpr size_t kOffSRad = kOffSPos + Round256(kNoAllocMaxAgents * sizeof(float2));
    constexpr size_t kOffCellOf = kOffSRad + Round256(kNoAllocMaxAgents * sizeof(float));
    constexpr size_t kOffArrival = kOffCellOf + Round256(kNoAllocMaxAgents * sizeof(int32_t));
    constexpr size_t kOffBucketTmp = kOffArrival + Round256(kNoAllocMaxAgents * sizeof(int32_t));
    constexpr size_t kOffBucket = kOffBucketTmp + Round256(kNoAllocMaxAgents * sizeof(int32_t));
    constexpr size_t kOffCounts = kOffBucket + Round256(kNoAllocMaxAgents * sizeof(int32_t));
    constexpr size_t kOffOffsets = kOffCounts + Round256(kNoAllocMaxCells * sizeof(int32_t));
    constexpr size_t kOffTileSums = kOffOffsets + Round256((kNoAllocMaxCells + 1) * sizeof(int32_t));
    constexpr size_t kNoAllocBytes = kOffTileSums + Round256(kNoAllocMaxTiles * sizeof(int32_t));
    static_assert(kNoAllocBytes <= HAL_CUDA_NOALLOC_SCRATCH_BYTES, "no-alloc scratch regions exceed the stated size");

    static __device__ __align__(256) unsigned char gNoAllocScratch[HAL_CUDA_NOALLOC_SCRATCH_BYTES];

    constexpr int kNoAllocMaxDevices = 64;
    std::mutex gNoAllocMutex;
    unsigned char *gNoAllocAddr[kNoAllocMaxDevices] = {};
    // The CUDA context each cached address belongs to (its unique id,
    // cuCtxGetId).  After cudaDeviceReset the runtime creates a new primary
    // context, loads this module again and the array may sit elsewhere; a
    // changed id makes the next call look the address up again.
    unsigned long long gNoAllocCtx[kNoAllocMaxDevices] = {};

    using CtxGetCurrentFn = CUresult (*)(CUcontext *);
    using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

    // Id of the calling thread's current context (0 when it cannot be read).
    unsigned long long CurrentContextId()
    {
        static CtxGetCurrentFn s_getCurrent = nullptr;
        static CtxGetIdFn s_getId = nullptr;
        static bool s_resolved = false;
        if (!s_resolved)
        {
            void *fn = nullptr;
            cudaDriverEntryPointQueryResult q;
            if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) ==
                    cudaSuccess && q == cudaDriverEntryPointSuccess)
            {
                s_getCurrent = reinterpret_cast<CtxGetCurrentFn>(fn);
            }
            fn = nullptr;
            if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
                q == cudaDriverEntryPointSuccess)
            {
                s_getId = reinterpret_cast<CtxGetIdFn>(fn);
            }
            s_resolved = true;
        }
        CUcontext ctx = nullptr;
        unsigned long long id = 0;
        if (s_getCurrent == nullptr || s_getId == nullptr || s_getCurrent(&ctx) != CUDA_SUCCESS || ctx == nullptr ||
            s_getId(ctx, &id) != CUDA_SUCCESS)
        {
            return 0;
        }
        return id;
    }

    // Device address of gNoAllocScratch on the current device `dev`; looked
    // up on the first call on that device, and again whenever the device's
    // context has changed since (a cudaDeviceReset in between).
    int NoAllocScratch(int dev, unsigned char **out)
    {
        if (dev < 0 || dev >= kNoAllocMaxDevices)
        {
            halcuda::SetError("hal_cuda_agents_forces_noalloc: device ordinal %d not supported", dev);
            return HAL_CUDA_EDEVICE;
        }
        std::lock_guard<std::mutex> lock(gNoAllocMutex);
        // an id of 0 (no context yet, or the driver cannot say) never
        // matches, so the address is looked up then
        void *p = nullptr;
        const unsigned long long ctx = CurrentContextId();
        if (gNoAllocAddr[dev] == nullptr || ctx == 0 || ctx != gNoAllocCtx[dev])
        {
            HAL_TRY(halcuda::CudaStatus(cudaGetSymbolAddress(&p, gNoAllocScratch),
                                        "cudaGetSymbolAddress(no-alloc scratch)"));
            gNoAllocAddr[dev] = static_cast<unsigned char *>(p);
            gNoAllocCtx[dev] = CurrentContextId();
        }
        *out = gNoAllocAddr[dev];
        return HAL_CUDA_OK;
    }

    // The pointer must be device (or managed) memory reachable from `dev`.
    bool OnDevice(const void *p, int dev)
    {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
        {
            cudaGetLastError();
            return false;
        }
        return a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev);
    }
}

extern "C" int hal_cuda_agents_forces_noalloc(const float *positions, const float *radii, int32_t n,
                                              float *velocityDeltas, double interactionRad, double springConstant,
                                              int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY, void *stream)
{
    HAL_REQUIRE(xDim > 0 && yDim > 0, "hal_cuda_agents_forces_noalloc: dimensions must be positive");
    HAL_REQUIRE(static_cast<int64_t>(xDim) * yDim <= static_cast<int64_t>(kNoAllocMaxCells),
                "hal_cuda_agents_forces_noalloc: grid %d x %d has more than %d cells, the no-alloc limit",
                xDim, yDim, HAL_CUDA_NOALLOC_MAX_CELLS);
    HAL_REQUIRE(n >= 0 && static_cast<size_t>(n) <= kNoAllocMaxAgents,
                "hal_cuda_agents_forces_noalloc: agent count %d outside [0, %d], the no-alloc limit", n,
                HAL_CUDA_NOALLOC_MAX_AGENTS);
    HAL_REQUIRE(RadiusOk(interactionRad), "hal_cuda_agents_forces_noalloc: interactionRad %g outside [0, %g]",
                interactionRad, kMaxInteractionRad);
    HAL_REQUIRE(n == 0 || (positions != nullptr && radii != nullptr && velocityDeltas != nullptr),
                "hal_cuda_agents_forces_noalloc: NULL array");
    using namespace halcuda;
    int dev = 0;
    HAL_TRY(CudaStatus(cudaGetDevice(&dev), "cudaGetDevice"));
    HAL_REQUIRE(n == 0 || (OnDevice(positions, dev) && OnDevice(radii, dev) && OnDevice(velocityDeltas, dev)),
                "hal_cuda_agents_forces_noalloc: positions, radii and velocityDeltas must be device memory of "
                "the current device %d", dev);
    unsigned char *base = nullptr;
    HAL_TRY(NoAllocScratch(dev, &base));
    if (n == 0)
    {
        return HAL_CUDA_OK;
    }
    float2 *posF = reinterpret_cast<float2 *>(base + kOffPosF);
    float2 *sPos = reinterpret_cast<float2 *>(base + kOffSPos);
    float *sRad = reinterpret_cast<float *>(base + kOffSRad);
    int32_t *cellOf = reinterpret_cast<int32_t *>(base + kOffCellOf);
    int32_t *arrival = reinterpret_cast<int32_t *>(base + kOffArrival);
    int32_t *bucketTmp = reinterpret_cast<int32_t *>(base + kOffBucketTmp);
    int32_t *bucket = reinterpret_cast<int32_t *>(base + kOffBucket);
    int32_t *counts = reinterpret_cast<int32_t *>(base + kOffCounts);
    int32_t *offsets = reinterpret_cast<int32_t *>(base + kOffOffsets);
    int32_t *tileSums = reinterpret_cast<int32_t *>(base + kOffTileSums);

    const int64_t C = static_cast<int64_t>(xDim) * yDim;
    const unsigned nTiles = static_cast<unsigned>((C + kScanTile - 1) / kScanTile);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    HAL_TRY(CudaStatus(cudaMemsetAsync(counts, 0, static_cast<size_t>(C) * sizeof(int32_t), s),
                       "cudaMemsetAsync(no-alloc counts)"));
    const int T = 256;
    const unsigned ablocks = static_cast<unsigned>((n + T - 1) / T);
    BinCount<float><<<ablocks, T, 0, s>>>(positions, n, xDim, yDim, posF, cellOf, arrival, counts);
    ScanReduce<<<nTiles, kScanThreads, 0, s>>>(counts, C, tileSums);
    ScanTiles<<<1, kScanThreads, 0, s>>>(tileSums, static_cast<int32_t>(nTiles));
    ScanApply<false><<<nTiles, kScanThreads, 0, s>>>(counts, C, tileSums, offsets, n);
    Scatter<<<ablocks, T, 0, s>>>(cellOf, arrival, offsets, n, bucketTmp);
    Stabilize<float, float><<<ablocks, T, 0, s>>>(cellOf, offsets, bucketTmp, posF, radii, n, bucket, sPos, sRad);
    const int TF = 128;
    LawParams<float> lp;
    lp.scale = static_cast<float>(springConstant);
    lp.exponent = 1.0f;
    Forces<float, float><<<static_cast<unsigned>((n + TF - 1) / TF), TF, 0, s>>>(
        bucket, offsets, sPos, sRad, n, interactionRad, static_cast<float>(interactionRad), lp, xDim, yDim,
        wrapX != 0, wrapY != 0, velocityDeltas, static_cast<float *>(nullptr), static_cast<const float *>(nullptr));
    CountLaunch(7);
    return LaunchStatus("hal_cuda_agents_forces_noalloc");
}

namespace halcuda
{
    int32_t AgentScanTiles(int64_t cells)
    {
        return static_cast<int32_t>((cells + kScanTile - 1) / kScanTile);
    }

    int LaunchAgentWells(const AgentWellsArgs &a, cudaStream_t s)
    {
        if (a.n <= 0)
        {
            return HAL_CUDA_OK;
        }
        // a.counts is zero here when small (allocated zeroed; every
        // ScanApply<true> clears the counts it has read); large ones are
        // cleared by a memset
        const bool clearInScan = a.cells <= kClearInScanCells;
        if (!clearInScan)
        {
            HAL_TRY(CudaStatus(cudaMemsetAsync(a.counts, 0, static_cast<size_t>(a.cells) * sizeof(int32_t), s),
                               "cudaMemsetAsync(well counts)"));
        }
        const int T = 256;
        const unsigned ablocks = static_cast<unsigned>((a.n + T - 1) / T);
        const int32_t nTiles = AgentScanTiles(a.cells);
        LaunchChained(BinCountWells, ablocks, T, s, a.pos, a.wellOf, a.wells, a.n, a.posF, a.cellOf, a.arrival,
                      a.counts);
        LaunchChained(ScanReduce, nTiles, kScanThreads, s, a.counts, a.cells, a.tileSums);
        LaunchChained(ScanTiles, 1u, kScanThreads, s, a.tileSums, nTiles);
        if (clearInScan)
        {
            LaunchChained(ScanApply<true>, nTiles, kScanThreads, s, a.counts, a.cells, a.tileSums, a.offsets, a.n);
        }
        else
        {
            LaunchChained(ScanApply<false>, nTiles, kScanThreads, s, a.counts, a.cells, a.tileSums, a.offsets, a.n);
        }
        LaunchChained(Scatter, ablocks, T, s, a.cellOf, a.arrival, a.offsets, a.n, a.bucketTmp);
        LaunchChained(StabilizeWells, ablocks, T, s, a.cellOf, a.offsets, a.bucketTmp, a.posF, a.rad, a.wellOf,
                      a.wells, a.n, a.bucket, a.sPos, a.sRad, a.sCell);
        const int TF = (a.forceThreads == 64 || a.forceThreads == 256) ? a.forceThreads : 128;
        const unsigned fblocks = static_cast<unsigned>((a.n + TF - 1) / TF);
        if (a.velState != nullptr)
        {
            LaunchChained(ForcesWellsMove, fblocks, TF, s, a.bucket, a.offsets, a.sPos, a.sRad, a.sCell, a.wellOf,
                          a.wells, a.n, a.interactionRad, a.R, a.k, a.friction, a.maxVel, a.vel, a.posOut,
                          a.velState);
        }
        else
        {
            LaunchChained(ForcesWells, fblocks, TF, s, a.bucket, a.offsets, a.sPos, a.sRad, a.sCell, a.wellOf,
                          a.wells, a.n, a.interactionRad, a.R, a.k, a.vel);
        }
        CountLaunch(7);
        return LaunchStatus("agent wells");
    }
}
