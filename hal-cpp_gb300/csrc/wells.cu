// wells.cu -- many independent wells (MultiWellExperiment) per launch.
//
// The reference advances wells one by one, or on host threads
// (include/Hal/Tools/MultiWellExperiment.h:83-103,
// include/Hal/Concurrency/MultiThread.h:19-91), each with its own PDEGrid2D
// tick.  Here a tick of every well is a handful of launches over packed
// tables:
//   - TickTiles over (well, CTA column, CTA row) tiles of the explicit wells;
//   - AdiSweepTiles (x-sweep) and AdiSweepTiles (y-sweep) over
//     (well, first line) tiles of the ADI wells;
//   - the agent pass over the concatenated agents and cells of the wells
//     that have agents.
// The kernels are the single-grid handles' kernels (diffusion.cu, adi.cu,
// agents.cu) reading their parameters from a per-well table, so each well's
// result is bit-identical to running it alone.  Tiles are ordered largest
// well first, so the block scheduler starts the long tiles early.
//
// Device memory: one arena holds every well's two field buffers, its source
// and (ADI) its x-sweep intermediate, each 256-byte aligned.  Explicit wells
// keep HAL's layout (x*yDim + y); ADI wells keep the transposed layout of the
// single-grid ADI handle (y*xDim + x).  All wells advance together, so one
// parity bit says which buffer holds the field, and the parameter tables
// exist once per parity.
#include "common.cuh"
#include "adi_plan.h"
#include "adi_sweep.h"
#include "agents_wells.h"
#include "tick_params.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <utility>
#include <vector>

namespace halcuda
{
    namespace
    {
        constexpr size_t kAlignFloats = 64;  // 256 bytes

        size_t RoundUp(size_t n)
        {
            return (n + kAlignFloats - 1) / kAlignFloats * kAlignFloats;
        }

        // interactionRad bound shared with the single-grid agent handle
        constexpr double kMaxInteractionRad = 1048576.0;
    }

    struct Wells
    {
        int device = 0;
        StreamSlot stream;
        // Graph branch of a tick: the explicit wells' tiles run on their own
        // stream beside the agent pass and the ADI sweeps (EnqueueTick).
        StreamSlot sideExplicit;
        EventSlot fork, joinExplicit;
        std::vector<hal_cuda_well_desc> desc;
        DevBuf<float> arena;
        std::vector<size_t> offF0, offF1, offSrc, offW;
        // ADI wells keep their rows padded to multiples of 4 floats: the
        // field and source (layout B, yDim rows) with stride strideF >= xDim,
        // the x-sweep's w (layout A, xDim rows) with stride strideW >= yDim.
        // The padding holds zeros (the arena starts zeroed and the sweeps
        // write zeros there), so every line stages by 16-byte copies.
        std::vector<int32_t> strideF, strideW;
        std::vector<uint8_t> hasSrc;
        int cur = 0;

        // explicit wells
        std::vector<int32_t> expIdx;     // well -> row of the tick table, or -1
        std::vector<int32_t> expWell;    // row -> well
        DevBuf<TickParams> tickTab[2];   // by parity
        DevBuf<int4> tiles4, tiles1;
        int32_t nTiles4 = 0, nTiles1 = 0;

        // ADI wells
        std::vector<int32_t> adiIdx;     // well -> row of the sweep tables, or -1
        std::vector<int32_t> adiWell;    // row -> well
        std::vector<std::unique_ptr<AdiDevicePlan>> planX, planY;
        DevBuf<SweepParams> sxTab[2], syTab[2];
        DevBuf<int2> tilesX, tilesY;
        int32_t nTilesX = 0, nTilesY = 0;
        size_t smemX = 0, smemY = 0;
        int32_t threadsX = 0, threadsY = 0;  // threads per tile CTA of each sweep
        DevBuf<int32_t> err;
        // set once a bounded device wait has given up: the wells' fields are
        // undefined from then on, so the handle takes no further ticks
        bool stopped = false;
        // Lines per sweep tile are capped at rCap, chosen by the autotuner
        // (Autotune) the first time the wells tick.
        int32_t rCap = kSweepTileMaxR;
        // Threads per tile CTA are at most tileBudget, also chosen by the
        // autotuner: smaller CTAs (fewer lines each) let several share an SM.
        int32_t tileBudget = kSweepTileThreads;
        int32_t forceThreads = 128;  // agent force kernel block size, also tuned
        bool tuned = false;
        float tunedMs = 0.0f, defaultMs = 0.0f;
        std::pair<double, double> agentsTunedFor{-1.0, 0.0};  // (R, k) the force block size was tuned for

        // agents
        std::vector<int64_t> cellBase;   // well -> first coarse agent bin in the concatenation, or -1
        int64_t agentCells = 0;          // coarse agent bins of all wells with agents
        int64_t agentCap = 0;
        int32_t nAgents = 0;
        std::vector<int32_t> counts;     // agents per well (last set_agents)
        DevBuf<AgentWellDev> agentWells;
        DevBuf<float> apos, arad, avel, sRad;
        DevBuf<float2> avelState;        // agents' own velocities, for motion
        bool motion = false;             // agents move after their forces each tick
        float friction = 1.0f, maxVel = -1.0f;
        DevBuf<float2> posF, sPos;
        DevBuf<int32_t> wellOf, cellOf, arrival, bucketTmp, bucket, sCell, binCounts, offsets, tileSums;

        GraphCache graph[2];             // one tick, by parity

        float *F(int32_t w, int c)
        {
            return arena.p + ((c == 0) ? offF0[w] : offF1[w]);
        }

        float *Src(int32_t w)
        {
            return arena.p + offSrc[w];
        }

        float *W(int32_t w)
        {
            return arena.p + offW[w];
        }

        size_t Cells(int32_t w) const
        {
            return static_cast<size_t>(desc[w].xDim) * static_cast<size_t>(desc[w].yDim);
        }

        void ResetGraphs()
        {
            graph[0].Reset();
            graph[1].Reset();
        }

        int Init(const hal_cuda_well_desc *wells, int32_t n)
        {
            device = CurrentDevice();
            HAL_TRY(CudaStatus(cudaSetDevice(device), "cudaSetDevice"));
            HAL_TRY(stream.Create("cudaStreamCreate"));
            HAL_TRY(sideExplicit.Create("cudaStreamCreate"));
            HAL_TRY(fork.Create("cudaEventCreate"));
            HAL_TRY(joinExplicit.Create("cudaEventCreate"));
            desc.assign(wells, wells + n);
            const size_t nw = static_cast<size_t>(n);
            offF0.resize(nw);
            offF1.resize(nw);
            offSrc.resize(nw);
            offW.assign(nw, 0);
            hasSrc.assign(nw, 0);
            expIdx.assign(nw, -1);
            adiIdx.assign(nw, -1);
            cellBase.assign(nw, -1);
            counts.assign(nw, 0);
            strideF.assign(nw, 0);
            strideW.assign(nw, 0);
            size_t total = 0;
            for (int32_t w = 0; w < n; w++)
            {
                const bool adi = desc[w].kind == HAL_CUDA_WELL_ADI;
                strideF[w] = adi ? (desc[w].xDim + 3) & ~3 : desc[w].xDim;
                strideW[w] = adi ? (desc[w].yDim + 3) & ~3 : desc[w].yDim;
                const size_t c = adi ? RoundUp(static_cast<size_t>(desc[w].yDim) * static_cast<size_t>(strideF[w]))
                                     : RoundUp(Cells(w));
                offF0[w] = total;
                offF1[w] = total + c;
                offSrc[w] = total + 2 * c;
                total += 3 * c;
                if (adi)
                {
                    offW[w] = total;
                    total += RoundUp(static_cast<size_t>(desc[w].xDim) * static_cast<size_t>(strideW[w]));
                    adiIdx[w] = static_cast<int32_t>(adiWell.size());
                    adiWell.push_back(w);
                }
                else
                {
                    expIdx[w] = static_cast<int32_t>(expWell.size());
                    expWell.push_back(w);
                }
                if (desc[w].maxAgents > 0)
                {
                    cellBase[w] = agentCells;
                    agentCells += WellBins(desc[w].xDim, desc[w].yDim,
                                           WellBinShift(desc[w].xDim, desc[w].yDim, desc[w].maxAgents));
                    agentCap += desc[w].maxAgents;
                }
            }
            HAL_TRY(arena.Alloc(total, "cudaMalloc(wells arena)"));
            HAL_TRY(CudaStatus(cudaMemset(arena.p, 0, total * sizeof(float)), "cudaMemset(wells arena)"));
            HAL_TRY(err.Alloc(1, "cudaMalloc(err)"));
            HAL_TRY(CudaStatus(cudaMemset(err.p, 0, sizeof(int32_t)), "cudaMemset(err)"));
            HAL_TRY(BuildExplicit());
            HAL_TRY(BuildAdi());
            HAL_TRY(BuildAgents());
            HAL_TRY(UploadTables());
            return CudaStatus(cudaDeviceSynchronize(), "wells setup");
        }

        // Tiles of the explicit wells, largest well first.
        int BuildExplicit()
        {
            std::vector<int32_t> order = expWell;
            std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return Cells(a) > Cells(b); });
            std::vector<int4> t4, t1;
            for (int32_t w : order)
            {
                const hal_cuda_well_desc &d = desc[w];
                const int vec = (d.yDim % 4 == 0) ? 4 : 1;
                const int32_t gx = (d.yDim + 32 * vec - 1) / (32 * vec);
                const int32_t gy = (d.xDim + kTickWarps * kTickRowsPerThread - 1) / (kTickWarps * kTickRowsPerThread);
                std::vector<int4> &t = (vec == 4) ? t4 : t1;
                for (int32_t by = 0; by < gy; by++)
                {
                    for (int32_t bx = 0; bx < gx; bx++)
                    {
                        t.push_back(make_int4(expIdx[w], bx, by, 0));
                    }
                }
            }
            nTiles4 = static_cast<int32_t>(t4.size());
            nTiles1 = static_cast<int32_t>(t1.size());
            HAL_TRY(Upload(tiles4, t4));
            HAL_TRY(Upload(tiles1, t1));
            for (int c = 0; c < 2; c++)
            {
                HAL_TRY(tickTab[c].Alloc(std::max<size_t>(expWell.size(), 1), "cudaMalloc(tick table)"));
            }
            return HAL_CUDA_OK;
        }

        // Line plans and tiles of the ADI wells, largest well first.
        int BuildAdi()
        {
            planX.clear();
            planY.clear();
            for (int32_t w : adiWell)
            {
                const hal_cuda_well_desc &d = desc[w];
                auto px = std::make_unique<AdiDevicePlan>();
                auto py = std::make_unique<AdiDevicePlan>();
                HAL_TRY(px->Build(d.xDim, d.diffRate, d.wrapX ? kEndsPeriodic : kEndsZeroFlux));
                HAL_TRY(py->Build(d.yDim, d.diffRate, d.wrapY ? kEndsPeriodic : kEndsZeroFlux));
                planX.push_back(std::move(px));
                planY.push_back(std::move(py));
            }
            for (int c = 0; c < 2; c++)
            {
                HAL_TRY(sxTab[c].Alloc(std::max<size_t>(adiWell.size(), 1), "cudaMalloc(sweep table)"));
                HAL_TRY(syTab[c].Alloc(std::max<size_t>(adiWell.size(), 1), "cudaMalloc(sweep table)"));
            }
            return BuildAdiTiles();
        }

        // Sweep tiles of the ADI wells at the current rCap, largest well first.
        int BuildAdiTiles()
        {
            std::vector<int32_t> order = adiWell;
            std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return Cells(a) > Cells(b); });
            std::vector<int2> tx, ty;
            smemX = smemY = 0;
            threadsX = threadsY = 32;
            for (int32_t w : order)
            {
                const int32_t a = adiIdx[w];
                const SweepTileShape sx = SweepTileShapeFor(planX[a]->Dev().P, rCap, tileBudget);
                const SweepTileShape sy = SweepTileShapeFor(planY[a]->Dev().P, rCap, tileBudget);
                smemX = std::max(smemX, sx.smem);
                smemY = std::max(smemY, sy.smem);
                threadsX = std::max(threadsX, sx.threads);
                threadsY = std::max(threadsY, sy.threads);
                for (int32_t x0 = 0; x0 < desc[w].yDim; x0 += sx.R)
                {
                    tx.push_back(make_int2(a, x0));
                }
                for (int32_t x0 = 0; x0 < desc[w].xDim; x0 += sy.R)
                {
                    ty.push_back(make_int2(a, x0));
                }
            }
            nTilesX = static_cast<int32_t>(tx.size());
            nTilesY = static_cast<int32_t>(ty.size());
            HAL_TRY(Upload(tilesX, tx));
            HAL_TRY(Upload(tilesY, ty));
            if (nTilesX > 0)
            {
                HAL_TRY(PrepareSweepTiles(kSweepW, smemX));
                HAL_TRY(PrepareSweepTiles(kSweepTick, smemY));
            }
            return HAL_CUDA_OK;
        }

        int BuildAgents()
        {
            if (agentCap == 0)
            {
                return HAL_CUDA_OK;
            }
            std::vector<AgentWellDev> wd(desc.size());
            for (size_t w = 0; w < desc.size(); w++)
            {
                wd[w].binBase = std::max<int64_t>(cellBase[w], 0);
                wd[w].xDim = desc[w].xDim;
                wd[w].yDim = desc[w].yDim;
                wd[w].wrapX = desc[w].wrapX;
                wd[w].wrapY = desc[w].wrapY;
                wd[w].binShift = WellBinShift(desc[w].xDim, desc[w].yDim, desc[w].maxAgents);
                wd[w].binsY = (desc[w].yDim + (1 << wd[w].binShift) - 1) >> wd[w].binShift;
            }
            HAL_TRY(Upload(agentWells, wd));
            const size_t m = static_cast<size_t>(agentCap);
            HAL_TRY(apos.Alloc(2 * m, "cudaMalloc(well agents)"));
            HAL_TRY(arad.Alloc(m, "cudaMalloc(well agents)"));
            HAL_TRY(avel.Alloc(2 * m, "cudaMalloc(well agents)"));
            HAL_TRY(avelState.Alloc(m, "cudaMalloc(well agents)"));
            HAL_TRY(CudaStatus(cudaMemset(avelState.p, 0, m * sizeof(float2)), "cudaMemset"));
            HAL_TRY(sRad.Alloc(m, "cudaMalloc(well agents)"));
            HAL_TRY(posF.Alloc(m, "cudaMalloc(well agents)"));
            HAL_TRY(sPos.Alloc(m, "cudaMalloc(well agents)"));
            HAL_TRY(wellOf.Alloc(m, "cudaMalloc(well agents)"));
            HAL_TRY(cellOf.Alloc(m, "cudaMalloc(well agents)"));
            HAL_TRY(arrival.Alloc(m, "cudaMalloc(well agents)"));
            HAL_TRY(bucketTmp.Alloc(m, "cudaMalloc(well agents)"));
            HAL_TRY(bucket.Alloc(m, "cudaMalloc(well agents)"));
            HAL_TRY(sCell.Alloc(m, "cudaMalloc(well agents)"));
            const size_t C = static_cast<size_t>(agentCells);
            HAL_TRY(binCounts.Alloc(C, "cudaMalloc(well bins)"));
            // zero once: every binning's scan clears the counts it read
            HAL_TRY(CudaStatus(cudaMemset(binCounts.p, 0, C * sizeof(int32_t)), "cudaMemset(well bins)"));
            HAL_TRY(offsets.Alloc(C + 1, "cudaMalloc(well bins)"));
            HAL_TRY(tileSums.Alloc(static_cast<size_t>(AgentScanTiles(agentCells)), "cudaMalloc(well bins)"));
            return HAL_CUDA_OK;
        }

        template <typename T>
        static int Upload(DevBuf<T> &buf, const std::vector<T> &v)
        {
            HAL_TRY(buf.Alloc(std::max<size_t>(v.size(), 1), "cudaMalloc(wells table)"));
            if (v.empty())
            {
                return HAL_CUDA_OK;
            }
            return CudaStatus(cudaMemcpy(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice),
                              "cudaMemcpy(wells table)");
        }

        // Parameter tables of both parities from the current sources.
        int UploadTables()
        {
            for (int c = 0; c < 2; c++)
            {
                std::vector<TickParams> tt(expWell.size());
                for (size_t e = 0; e < expWell.size(); e++)
                {
                    const int32_t w = expWell[e];
                    const hal_cuda_well_desc &d = desc[w];
                    TickParams p;
                    std::memset(&p, 0, sizeof(p));
                    p.f = F(w, c);
                    p.out = F(w, c ^ 1);
                    p.xDim = d.xDim;
                    p.yDim = d.yDim;
                    p.r = static_cast<float>(d.diffRate);
                    p.negDecay = static_cast<float>(-d.decay);
                    p.wrapX = d.wrapX;
                    p.wrapY = d.wrapY;
                    p.src = hasSrc[w] ? Src(w) : nullptr;
                    tt[e] = p;
                }
                std::vector<SweepParams> sx(adiWell.size()), sy(adiWell.size());
                for (size_t a = 0; a < adiWell.size(); a++)
                {
                    const int32_t w = adiWell[a];
                    const hal_cuda_well_desc &d = desc[w];
                    SweepParams p;
                    std::memset(&p, 0, sizeof(p));
                    p.in = F(w, c);
                    p.L = d.xDim;
                    p.Nlines = d.yDim;
                    p.wrapLines = d.wrapY;
                    p.halfR = static_cast<float>(d.diffRate / 2.0);
                    p.r = static_cast<float>(d.diffRate);
                    p.plan = planX[a]->Dev();
                    const SweepTileShape shx = SweepTileShapeFor(p.plan.P, rCap, tileBudget);
                    p.R = shx.R;
                    p.LS = shx.LS;
                    p.out = W(w);
                    p.err = err.p;
                    p.inStride = strideF[w];
                    p.outStride = strideW[w];
                    sx[a] = p;

                    SweepParams q;
                    std::memset(&q, 0, sizeof(q));
                    q.in = W(w);
                    q.L = d.yDim;
                    q.Nlines = d.xDim;
                    q.wrapLines = d.wrapX;
                    q.halfR = static_cast<float>(d.diffRate / 2.0);
                    q.r = static_cast<float>(d.diffRate);
                    q.plan = planY[a]->Dev();
                    const SweepTileShape shy = SweepTileShapeFor(q.plan.P, rCap, tileBudget);
                    q.R = shy.R;
                    q.LS = shy.LS;
                    q.out = F(w, c ^ 1);
                    q.f = F(w, c);
                    q.src = hasSrc[w] ? Src(w) : nullptr;
                    q.negDecay = static_cast<float>(-d.decay);
                    q.err = err.p;
                    q.inStride = strideW[w];
                    q.outStride = strideF[w];
                    sy[a] = q;
                }
                cudaStream_t s = stream.Get();
                if (!tt.empty())
                {
                    HAL_TRY(CudaStatus(cudaMemcpyAsync(tickTab[c].p, tt.data(), tt.size() * sizeof(TickParams),
                                                       cudaMemcpyHostToDevice, s), "cudaMemcpy(tick table)"));
                }
                if (!sx.empty())
                {
                    HAL_TRY(CudaStatus(cudaMemcpyAsync(sxTab[c].p, sx.data(), sx.size() * sizeof(SweepParams),
                                                       cudaMemcpyHostToDevice, s), "cudaMemcpy(sweep table)"));
                    HAL_TRY(CudaStatus(cudaMemcpyAsync(syTab[c].p, sy.data(), sy.size() * sizeof(SweepParams),
                                                       cudaMemcpyHostToDevice, s), "cudaMemcpy(sweep table)"));
                }
            }
            // the host vectors go out of scope: the copies must finish first
            return CudaStatus(cudaStreamSynchronize(stream.Get()), "wells tables");
        }

        // One tick of every well from parity c, enqueued on s.  With ev, the
        // stages run one after another on s and each records an event
        // (profiling).  Without, the explicit wells' tiles run on a branch
        // of their own beside the agent pass and the ADI sweeps, which stay
        // in order on s: the three read and write disjoint buffers.  The
        // bandwidth-bound explicit tiles then overlap the agent pass, a
        // chain of latency-bound gathers.  (The ADI sweep tiles hold a whole
        // SM's registers each, so a branch beside them finds no free slot.)
        int EnqueueTick(int c, double R, double k, cudaStream_t s, cudaEvent_t *ev)
        {
            if (ev == nullptr)
            {
                const bool exp = nTiles4 > 0 || nTiles1 > 0;
                if (exp)
                {
                    cudaStream_t e = sideExplicit.Get();
                    HAL_TRY(CudaStatus(cudaEventRecord(fork.e, s), "cudaEventRecord(fork)"));
                    HAL_TRY(CudaStatus(cudaStreamWaitEvent(e, fork.e, 0), "cudaStreamWaitEvent(fork)"));
                    HAL_TRY(LaunchTickTiles(tickTab[c].p, tiles4.p, nTiles4, 4, e));
                    HAL_TRY(LaunchTickTiles(tickTab[c].p, tiles1.p, nTiles1, 1, e));
                    HAL_TRY(CudaStatus(cudaEventRecord(joinExplicit.e, e), "cudaEventRecord(join)"));
                }
                if (nAgents > 0)
                {
                    HAL_TRY(LaunchAgentWells(AgentArgs(R, k), s));
                }
                HAL_TRY(LaunchSweepTiles(kSweepW, sxTab[c].p, tilesX.p, nTilesX, smemX, threadsX, s));
                HAL_TRY(LaunchSweepTiles(kSweepTick, syTab[c].p, tilesY.p, nTilesY, smemY, threadsY, s));
                if (exp)
                {
                    HAL_TRY(CudaStatus(cudaStreamWaitEvent(s, joinExplicit.e, 0), "cudaStreamWaitEvent(join)"));
                }
                return HAL_CUDA_OK;
            }
            HAL_TRY(LaunchTickTiles(tickTab[c].p, tiles4.p, nTiles4, 4, s));
            HAL_TRY(LaunchTickTiles(tickTab[c].p, tiles1.p, nTiles1, 1, s));
            if (ev)
            {
                cudaEventRecord(ev[0], s);
            }
            HAL_TRY(LaunchSweepTiles(kSweepW, sxTab[c].p, tilesX.p, nTilesX, smemX, threadsX, s));
            if (ev)
            {
                cudaEventRecord(ev[1], s);
            }
            HAL_TRY(LaunchSweepTiles(kSweepTick, syTab[c].p, tilesY.p, nTilesY, smemY, threadsY, s));
            if (ev)
            {
                cudaEventRecord(ev[2], s);
            }
            if (nAgents > 0)
            {
                HAL_TRY(LaunchAgentWells(AgentArgs(R, k), s));
            }
            if (ev)
            {
                cudaEventRecord(ev[3], s);
            }
            return HAL_CUDA_OK;
        }

        AgentWellsArgs AgentArgs(double R, double k)
        {
            AgentWellsArgs a;
            a.pos = apos.p;
            a.rad = arad.p;
            a.wellOf = wellOf.p;
            a.wells = agentWells.p;
            a.n = nAgents;
            a.cells = agentCells;
            a.posF = posF.p;
            a.sPos = sPos.p;
            a.sRad = sRad.p;
            a.cellOf = cellOf.p;
            a.arrival = arrival.p;
            a.bucketTmp = bucketTmp.p;
            a.bucket = bucket.p;
            a.sCell = sCell.p;
            a.counts = binCounts.p;
            a.offsets = offsets.p;
            a.tileSums = tileSums.p;
            a.interactionRad = R;
            a.R = static_cast<float>(R);
            a.k = static_cast<float>(k);
            a.vel = avel.p;
            a.forceThreads = forceThreads;
            a.velState = motion ? avelState.p : nullptr;
            a.posOut = reinterpret_cast<float2 *>(apos.p);
            a.friction = friction;
            a.maxVel = maxVel;
            return a;
        }

        int KernelsPerTick() const
        {
            return (nTiles4 > 0) + (nTiles1 > 0) + (nTilesX > 0) + (nTilesY > 0) + (nAgents > 0 ? 7 : 0);
        }

        // Mean device ms of one x-sweep plus one y-sweep launch over every
        // ADI well, from the live parity.  The y-sweep writes the other
        // parity's buffer and the parity is not flipped, so the wells' state
        // does not change.
        int TimeSweeps(int warm, int iters, float *ms)
        {
            cudaStream_t s = stream.Get();
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            HAL_TRY(CudaStatus(cudaEventCreate(&e0), "cudaEventCreate"));
            int rc = CudaStatus(cudaEventCreate(&e1), "cudaEventCreate");
            for (int t = 0; t < warm + iters && rc == HAL_CUDA_OK; t++)
            {
                if (t == warm)
                {
                    cudaEventRecord(e0, s);
                }
                rc = LaunchSweepTiles(kSweepW, sxTab[cur].p, tilesX.p, nTilesX, smemX, threadsX, s);
                if (rc == HAL_CUDA_OK)
                {
                    rc = LaunchSweepTiles(kSweepTick, syTab[cur].p, tilesY.p, nTilesY, smemY, threadsY, s);
                }
            }
            if (rc == HAL_CUDA_OK)
            {
                cudaEventRecord(e1, s);
                rc = CudaStatus(cudaEventSynchronize(e1), "wells autotune");
            }
            if (rc == HAL_CUDA_OK)
            {
                float t = 0.0f;
                cudaEventElapsedTime(&t, e0, e1);
                *ms = t / static_cast<float>(iters);
            }
            cudaEventDestroy(e0);
            if (e1 != nullptr)
            {
                cudaEventDestroy(e1);
            }
            return rc;
        }

        // Autotuner of the ADI sweep tiles: times the batched x- and y-sweeps
        // with the threads per tile CTA capped at 512, 256 and 128 and the
        // lines per tile capped at 128, 64, 32, 16 and 8 (settings that give
        // the same tiles as an earlier one are skipped), on the wells' own
        // data, and keeps the fastest.  Fewer lines per tile give more,
        // smaller CTAs: each tile CTA of 512 threads holds a whole SM's
        // registers, while 256- and 128-thread CTAs share an SM two and four
        // at a time and overlap one another's staging, solve and write-out.
        // More lines give longer contiguous stores.  Which wins depends on
        // the mix of well sizes.
        int Autotune()
        {
            tuned = true;
            if (nTilesX == 0)
            {
                rCap = kSweepTileMaxR;
                tileBudget = kSweepTileThreads;
                return HAL_CUDA_OK;
            }
            std::vector<std::vector<int32_t>> seen;
            float best = 0.0f;
            int32_t bestCap = kSweepTileMaxR, bestBudget = kSweepTileThreads;
            bool first = true;
            for (int32_t budget = kSweepTileThreads; budget >= 128; budget /= 2)
            {
                for (int32_t cap = kSweepTileMaxR; cap >= 8; cap /= 2)
                {
                    std::vector<int32_t> shape;
                    for (size_t a = 0; a < adiWell.size(); a++)
                    {
                        shape.push_back(SweepTileShapeFor(planX[a]->Dev().P, cap, budget).R);
                        shape.push_back(SweepTileShapeFor(planY[a]->Dev().P, cap, budget).R);
                    }
                    if (std::find(seen.begin(), seen.end(), shape) != seen.end())
                    {
                        continue;
                    }
                    seen.push_back(shape);
                    rCap = cap;
                    tileBudget = budget;
                    HAL_TRY(BuildAdiTiles());
                    HAL_TRY(UploadTables());
                    float ms = 0.0f;
                    HAL_TRY(TimeSweeps(2, 5, &ms));
                    if (first)
                    {
                        defaultMs = ms;
                    }
                    if (first || ms < best)
                    {
                        best = ms;
                        bestCap = cap;
                        bestBudget = budget;
                    }
                    first = false;
                }
            }
            rCap = bestCap;
            tileBudget = bestBudget;
            tunedMs = best;
            HAL_TRY(BuildAdiTiles());
            HAL_TRY(UploadTables());
            ResetGraphs();
            return HAL_CUDA_OK;
        }

        // Block size of the agent force kernel (64, 128 or 256 threads),
        // timed on the wells' agents with the interaction radius and spring
        // constant of the run.  The pass only rewrites its own bins and
        // deltas, so repeating it changes nothing.
        int TuneAgents(double R, double k)
        {
            agentsTunedFor = std::make_pair(R, k);
            if (nAgents == 0)
            {
                return HAL_CUDA_OK;
            }
            cudaStream_t s = stream.Get();
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            HAL_TRY(CudaStatus(cudaEventCreate(&e0), "cudaEventCreate"));
            int rc = CudaStatus(cudaEventCreate(&e1), "cudaEventCreate");
            float best = 0.0f;
            int32_t bestT = 128;
            for (int32_t t : {128, 64, 256})
            {
                forceThreads = t;
                AgentWellsArgs a = AgentArgs(R, k);
                a.velState = nullptr;  // timing runs compute forces only: the agents stay put
                for (int it = 0; it < 5 && rc == HAL_CUDA_OK; it++)
                {
                    if (it == 2)
                    {
                        cudaEventRecord(e0, s);
                    }
                    rc = LaunchAgentWells(a, s);
                }
                if (rc == HAL_CUDA_OK)
                {
                    cudaEventRecord(e1, s);
                    rc = CudaStatus(cudaEventSynchronize(e1), "wells agent autotune");
                }
                if (rc != HAL_CUDA_OK)
                {
                    break;
                }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (t == 128 || ms < best)
                {
                    best = ms;
                    bestT = t;
                }
            }
            cudaEventDestroy(e0);
            if (e1 != nullptr)
            {
                cudaEventDestroy(e1);
            }
            forceThreads = bestT;
            ResetGraphs();
            return rc;
        }

        int RunTicks(int32_t ticks, double R, double k)
        {
            if (stopped)
            {
                SetError("hal_cuda_wells_run_ticks: the handle stopped after a sweep gave up waiting for its staged "
                         "lines; the fields are undefined: destroy the handle and create a new one");
                return HAL_CUDA_ETIMEOUT;
            }
            if (!tuned)
            {
                HAL_TRY(Autotune());
            }
            if (agentsTunedFor != std::make_pair(R, k))
            {
                HAL_TRY(TuneAgents(R, k));
            }
            cudaStream_t s = stream.Get();
            char key[160];
            snprintf(key, sizeof(key), "%a|%a|%d|%d|%a|%a|%d|%p", R, k, nAgents, motion ? 1 : 0,
                     static_cast<double>(friction), static_cast<double>(maxVel), forceThreads, static_cast<void *>(s));
            for (int32_t t = 0; t < ticks; t++)
            {
                GraphCache &g = graph[cur];
                if (g.exec == nullptr || g.key != key)
                {
                    g.Reset();
                    HAL_TRY(CudaStatus(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                                       "cudaStreamBeginCapture"));
                    const int rc = EnqueueTick(cur, R, k, s, nullptr);
                    cudaGraph_t gr = nullptr;
                    const cudaError_t e = cudaStreamEndCapture(s, &gr);
                    if (rc != HAL_CUDA_OK)
                    {
                        if (gr != nullptr)
                        {
                            cudaGraphDestroy(gr);
                        }
                        return rc;
                    }
                    HAL_TRY(CudaStatus(e, "cudaStreamEndCapture"));
                    const cudaError_t ei = cudaGraphInstantiate(&g.exec, gr, 0);
                    cudaGraphDestroy(gr);
                    HAL_TRY(CudaStatus(ei, "cudaGraphInstantiate"));
                    g.key = key;
                }
                HAL_TRY(CudaStatus(cudaGraphLaunch(g.exec, s), "cudaGraphLaunch"));
                CountLaunch(KernelsPerTick());
                cur ^= 1;
            }
            return HAL_CUDA_OK;
        }

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
    };
}

using halcuda::Wells;

struct hal_cuda_wells : public Wells
{
};

namespace
{
    int CheckWell(const hal_cuda_wells *h, int32_t well, int64_t len, const char *who)
    {
        HAL_REQUIRE(h != nullptr, "%s: handle is NULL", who);
        HAL_REQUIRE(well >= 0 && well < static_cast<int32_t>(h->desc.size()), "%s: well %d outside [0, %d)", who,
                    well, static_cast<int32_t>(h->desc.size()));
        HAL_REQUIRE(len == static_cast<int64_t>(h->Cells(well)), "%s: length %lld, well %d holds %lld cells", who,
                    static_cast<long long>(len), well, static_cast<long long>(h->Cells(well)));
        return HAL_CUDA_OK;
    }
}

extern "C" int hal_cuda_wells_create(const hal_cuda_well_desc *wells, int32_t nWells, hal_cuda_wells **out)
{
    HAL_REQUIRE(out != nullptr, "hal_cuda_wells_create: out is NULL");
    *out = nullptr;
    HAL_REQUIRE(wells != nullptr && nWells > 0, "hal_cuda_wells_create: no wells");
    int64_t cells = 0, agents = 0;
    for (int32_t w = 0; w < nWells; w++)
    {
        const hal_cuda_well_desc &d = wells[w];
        HAL_REQUIRE(d.xDim >= 1 && d.yDim >= 1 && d.xDim <= HAL_CUDA_WELLS_MAX_SIDE && d.yDim <= HAL_CUDA_WELLS_MAX_SIDE,
                    "hal_cuda_wells_create: well %d is %d x %d, sides must be in [1, %d]", w, d.xDim, d.yDim,
                    HAL_CUDA_WELLS_MAX_SIDE);
        HAL_REQUIRE(d.kind == HAL_CUDA_WELL_EXPLICIT || d.kind == HAL_CUDA_WELL_ADI,
                    "hal_cuda_wells_create: well %d has unknown kind %d", w, d.kind);
        HAL_REQUIRE(std::isfinite(d.diffRate) && d.diffRate >= 0.0, "hal_cuda_wells_create: well %d rate %g", w,
                    d.diffRate);
        // PDEGrid2D::CheckDiffusionStable (PDEGrid2D.h:436-442)
        HAL_REQUIRE(d.kind != HAL_CUDA_WELL_EXPLICIT || d.diffRate <= 0.25,
                    "hal_cuda_wells_create: well %d explicit rate %g above the stable 0.25", w, d.diffRate);
        HAL_REQUIRE(std::isfinite(d.decay), "hal_cuda_wells_create: well %d decay %g", w, d.decay);
        HAL_REQUIRE(d.maxAgents >= 0, "hal_cuda_wells_create: well %d negative agent capacity", w);
        if (d.maxAgents > 0)
        {
            cells += static_cast<int64_t>(d.xDim) * d.yDim;
            agents += d.maxAgents;
        }
    }
    HAL_REQUIRE(cells < (int64_t(1) << 31) - 1 && agents < (int64_t(1) << 31) - 1,
                "hal_cuda_wells_create: agent cells or capacity exceed int32");
    hal_cuda_wells *h = new (std::nothrow) hal_cuda_wells();
    if (h == nullptr)
    {
        halcuda::SetError("hal_cuda_wells_create: out of host memory");
        return HAL_CUDA_ENOMEM;
    }
    int rc = h->Init(wells, nWells);
    if (rc != HAL_CUDA_OK)
    {
        delete h;
        return rc;
    }
    *out = h;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_wells_destroy(hal_cuda_wells *h)
{
    if (h != nullptr)
    {
        cudaSetDevice(h->device);
        cudaStreamSynchronize(h->stream.Get());
        delete h;
    }
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_wells_set_field(hal_cuda_wells *h, int32_t well, const float *field, int64_t len)
{
    HAL_TRY(CheckWell(h, well, len, "hal_cuda_wells_set_field"));
    HAL_REQUIRE(field != nullptr, "hal_cuda_wells_set_field: field is NULL");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    const hal_cuda_well_desc &d = h->desc[well];
    const size_t bytes = static_cast<size_t>(len) * sizeof(float);
    if (d.kind == HAL_CUDA_WELL_ADI)
    {
        // dense through the x-sweep scratch, then into the padded rows
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->W(well), field, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpy(field)"));
        HAL_TRY(LaunchTransposeStrided(h->W(well), d.yDim, h->F(well, h->cur), h->strideF[well], d.xDim, d.yDim, s));
    }
    else
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->F(well, h->cur), field, bytes, cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(field)"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_wells_set_field");
}

extern "C" int hal_cuda_wells_get_field(hal_cuda_wells *h, int32_t well, float *field, int64_t len)
{
    HAL_TRY(CheckWell(h, well, len, "hal_cuda_wells_get_field"));
    HAL_REQUIRE(field != nullptr, "hal_cuda_wells_get_field: field is NULL");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    HAL_TRY(h->CheckDeviceError("hal_cuda_wells_get_field"));
    cudaStream_t s = h->stream.Get();
    const hal_cuda_well_desc &d = h->desc[well];
    const size_t bytes = static_cast<size_t>(len) * sizeof(float);
    const float *from = h->F(well, h->cur);
    if (d.kind == HAL_CUDA_WELL_ADI)
    {
        HAL_TRY(LaunchTransposeStrided(from, h->strideF[well], h->W(well), d.yDim, d.yDim, d.xDim, s));
        from = h->W(well);
    }
    HAL_TRY(CudaStatus(cudaMemcpyAsync(field, from, bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpy(field)"));
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_wells_get_field");
}

extern "C" int hal_cuda_wells_set_source(hal_cuda_wells *h, int32_t well, const float *dense, int64_t len)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_wells_set_source: handle is NULL");
    using namespace halcuda;
    if (dense == nullptr)
    {
        HAL_REQUIRE(well >= 0 && well < static_cast<int32_t>(h->desc.size()), "hal_cuda_wells_set_source: bad well");
        HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
        h->hasSrc[well] = 0;
        return h->UploadTables();
    }
    HAL_TRY(CheckWell(h, well, len, "hal_cuda_wells_set_source"));
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    const hal_cuda_well_desc &d = h->desc[well];
    const size_t bytes = static_cast<size_t>(len) * sizeof(float);
    if (d.kind == HAL_CUDA_WELL_ADI)
    {
        // through the x-sweep scratch, which holds nothing between ticks
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->W(well), dense, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpy(source)"));
        HAL_TRY(LaunchTransposeStrided(h->W(well), d.yDim, h->Src(well), h->strideF[well], d.xDim, d.yDim, s));
    }
    else
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->Src(well), dense, bytes, cudaMemcpyHostToDevice, s),
                           "cudaMemcpy(source)"));
    }
    HAL_TRY(CudaStatus(cudaStreamSynchronize(s), "hal_cuda_wells_set_source"));
    if (!h->hasSrc[well])
    {
        h->hasSrc[well] = 1;
        return h->UploadTables();
    }
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_wells_set_agents(hal_cuda_wells *h, const int32_t *counts, const float *positions,
                                         const float *radii)
{
    HAL_REQUIRE(h != nullptr && counts != nullptr, "hal_cuda_wells_set_agents: NULL argument");
    int64_t n = 0;
    for (size_t w = 0; w < h->desc.size(); w++)
    {
        HAL_REQUIRE(counts[w] >= 0 && counts[w] <= h->desc[w].maxAgents,
                    "hal_cuda_wells_set_agents: well %d has %d agents, capacity %d", static_cast<int>(w), counts[w],
                    h->desc[w].maxAgents);
        n += counts[w];
    }
    HAL_REQUIRE(n == 0 || (positions != nullptr && radii != nullptr), "hal_cuda_wells_set_agents: NULL array");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    std::vector<int32_t> wellOf(static_cast<size_t>(n));
    int64_t at = 0;
    for (size_t w = 0; w < h->desc.size(); w++)
    {
        std::fill(wellOf.begin() + at, wellOf.begin() + at + counts[w], static_cast<int32_t>(w));
        at += counts[w];
    }
    if (n > 0)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->apos.p, positions, 2 * static_cast<size_t>(n) * sizeof(float),
                                           cudaMemcpyHostToDevice, s), "cudaMemcpy(positions)"));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->arad.p, radii, static_cast<size_t>(n) * sizeof(float),
                                           cudaMemcpyHostToDevice, s), "cudaMemcpy(radii)"));
        HAL_TRY(CudaStatus(cudaMemcpyAsync(h->wellOf.p, wellOf.data(), static_cast<size_t>(n) * sizeof(int32_t),
                                           cudaMemcpyHostToDevice, s), "cudaMemcpy(wellOf)"));
        HAL_TRY(CudaStatus(cudaMemsetAsync(h->avelState.p, 0, static_cast<size_t>(n) * sizeof(float2), s),
                           "cudaMemsetAsync(velocities)"));
    }
    h->counts.assign(counts, counts + h->desc.size());
    h->agentsTunedFor = std::make_pair(-1.0, 0.0);  // new agents: re-tune the force block size
    h->nAgents = static_cast<int32_t>(n);
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_wells_set_agents");
}

extern "C" int hal_cuda_wells_set_motion(hal_cuda_wells *h, int32_t enabled, double friction, double maxVel)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_wells_set_motion: handle is NULL");
    HAL_REQUIRE(std::isfinite(friction), "hal_cuda_wells_set_motion: friction must be finite");
    HAL_REQUIRE(!std::isnan(maxVel), "hal_cuda_wells_set_motion: maxVel is NaN");
    h->motion = enabled != 0;
    h->friction = static_cast<float>(friction);
    h->maxVel = (maxVel < 0 || std::isinf(maxVel)) ? -1.0f : static_cast<float>(maxVel);
    h->ResetGraphs();
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_wells_set_velocities(hal_cuda_wells *h, const float *velocities, int64_t len)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_wells_set_velocities: handle is NULL");
    HAL_REQUIRE(len == 2 * static_cast<int64_t>(h->nAgents), "hal_cuda_wells_set_velocities: %lld values for %d agents",
                static_cast<long long>(len), h->nAgents);
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    if (h->nAgents > 0)
    {
        const size_t bytes = static_cast<size_t>(h->nAgents) * sizeof(float2);
        HAL_TRY(CudaStatus(velocities != nullptr
                               ? cudaMemcpyAsync(h->avelState.p, velocities, bytes, cudaMemcpyHostToDevice, s)
                               : cudaMemsetAsync(h->avelState.p, 0, bytes, s),
                           "hal_cuda_wells_set_velocities"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_wells_set_velocities");
}

extern "C" int hal_cuda_wells_get_agents(hal_cuda_wells *h, float *positions, float *velocities, int64_t len)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_wells_get_agents: handle is NULL");
    HAL_REQUIRE(len == 2 * static_cast<int64_t>(h->nAgents), "hal_cuda_wells_get_agents: %lld values for %d agents",
                static_cast<long long>(len), h->nAgents);
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    const size_t bytes = static_cast<size_t>(len) * sizeof(float);
    if (len > 0 && positions != nullptr)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(positions, h->apos.p, bytes, cudaMemcpyDeviceToHost, s),
                           "cudaMemcpy(positions)"));
    }
    if (len > 0 && velocities != nullptr)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(velocities, h->avelState.p, bytes, cudaMemcpyDeviceToHost, s),
                           "cudaMemcpy(velocities)"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_wells_get_agents");
}

extern "C" int hal_cuda_wells_run_ticks(hal_cuda_wells *h, int32_t ticks, double interactionRad,
                                        double springConstant)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr, "hal_cuda_wells_run_ticks: handle is NULL");
    HAL_REQUIRE(ticks >= 0, "hal_cuda_wells_run_ticks: negative tick count");
    HAL_REQUIRE(std::isfinite(interactionRad) && interactionRad >= 0.0 && interactionRad <= halcuda::kMaxInteractionRad,
                "hal_cuda_wells_run_ticks: interactionRad %g outside [0, %g]", interactionRad,
                halcuda::kMaxInteractionRad);
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return h->RunTicks(ticks, interactionRad, springConstant);
}

extern "C" int hal_cuda_wells_get_forces(hal_cuda_wells *h, float *velocityDeltas, int64_t len)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_wells_get_forces: handle is NULL");
    HAL_REQUIRE(len == 2 * static_cast<int64_t>(h->nAgents), "hal_cuda_wells_get_forces: length %lld, %d agents",
                static_cast<long long>(len), h->nAgents);
    HAL_REQUIRE(len == 0 || velocityDeltas != nullptr, "hal_cuda_wells_get_forces: NULL array");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    cudaStream_t s = h->stream.Get();
    if (len > 0)
    {
        HAL_TRY(CudaStatus(cudaMemcpyAsync(velocityDeltas, h->avel.p, static_cast<size_t>(len) * sizeof(float),
                                           cudaMemcpyDeviceToHost, s), "cudaMemcpy(velocityDeltas)"));
    }
    return CudaStatus(cudaStreamSynchronize(s), "hal_cuda_wells_get_forces");
}

extern "C" int hal_cuda_wells_profile(hal_cuda_wells *h, int32_t iters, double interactionRad,
                                      double springConstant, float *ms)
{
    HAL_REQUIRE(h != nullptr && ms != nullptr, "hal_cuda_wells_profile: NULL argument");
    HAL_REQUIRE(iters > 0, "hal_cuda_wells_profile: iters must be positive");
    HAL_REQUIRE(std::isfinite(interactionRad) && interactionRad >= 0.0 && interactionRad <= halcuda::kMaxInteractionRad,
                "hal_cuda_wells_profile: interactionRad out of range");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    if (!h->tuned)
    {
        HAL_TRY(h->Autotune());
    }
    if (h->agentsTunedFor != std::make_pair(interactionRad, springConstant))
    {
        HAL_TRY(h->TuneAgents(interactionRad, springConstant));
    }
    cudaStream_t s = h->stream.Get();
    cudaEvent_t ev[5];
    for (auto &e : ev)
    {
        HAL_TRY(CudaStatus(cudaEventCreate(&e), "cudaEventCreate"));
    }
    double acc[5] = {0, 0, 0, 0, 0};
    int rc = HAL_CUDA_OK;
    for (int32_t t = 0; t < iters && rc == HAL_CUDA_OK; t++)
    {
        cudaEventRecord(ev[4], s);
        rc = h->EnqueueTick(h->cur, interactionRad, springConstant, s, ev);
        if (rc == HAL_CUDA_OK)
        {
            rc = CudaStatus(cudaEventSynchronize(ev[3]), "hal_cuda_wells_profile");
        }
        if (rc != HAL_CUDA_OK)
        {
            break;
        }
        h->cur ^= 1;
        float t0 = 0, t1 = 0, t2 = 0, t3 = 0, ta = 0;
        cudaEventElapsedTime(&t0, ev[4], ev[0]);
        cudaEventElapsedTime(&t1, ev[0], ev[1]);
        cudaEventElapsedTime(&t2, ev[1], ev[2]);
        cudaEventElapsedTime(&t3, ev[2], ev[3]);
        cudaEventElapsedTime(&ta, ev[4], ev[3]);
        acc[0] += t0;
        acc[1] += t1;
        acc[2] += t2;
        acc[3] += t3;
        acc[4] += ta;
    }
    for (auto &e : ev)
    {
        cudaEventDestroy(e);
    }
    HAL_TRY(rc);
    for (int q = 0; q < 5; q++)
    {
        ms[q] = static_cast<float>(acc[q] / iters);
    }
    return h->CheckDeviceError("hal_cuda_wells_profile");
}

extern "C" int hal_cuda_wells_autotune(hal_cuda_wells *h, int32_t *rCap, float *msTuned, float *msDefault)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_wells_autotune: handle is NULL");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    HAL_TRY(h->Autotune());
    if (rCap != nullptr)
    {
        *rCap = h->rCap;
    }
    if (msTuned != nullptr)
    {
        *msTuned = h->tunedMs;
    }
    if (msDefault != nullptr)
    {
        *msDefault = h->defaultMs;
    }
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_wells_sync(hal_cuda_wells *h)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_wells_sync: handle is NULL");
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return h->CheckDeviceError("hal_cuda_wells_sync");
}

extern "C" void *hal_cuda_wells_stream(hal_cuda_wells *h)
{
    return h ? static_cast<void *>(h->stream.Get()) : nullptr;
}

extern "C" int hal_cuda_wells_set_stream(hal_cuda_wells *h, void *stream)
{
    HAL_REQUIRE(h != nullptr, "hal_cuda_wells_set_stream: handle is NULL");
    h->stream.Set(stream);
    h->ResetGraphs();
    return HAL_CUDA_OK;
}
