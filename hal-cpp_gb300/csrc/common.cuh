// common.cuh -- shared host/device helpers of the hal_cuda library.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "hal_cuda.h"

#include <nvtx3/nvToolsExt.h>
#include "hal_cuda_measure.h"

namespace halcuda
{
    // Thread-local message of the last failed call (hal_cuda_last_error).
    void SetError(const char *fmt, ...);
    void ClearError();

    // NVTX range over one library call, in the domain "hal_cuda" (HAL_TRACE at
    // the top of the hot-path entry points): Nsight tools show the calls on
    // the timeline and can filter kernels by call, e.g. ncu --nvtx
    // --nvtx-include "hal_cuda@hal_cuda_adi_run_ticks/".  Without a tool
    // attached a range costs a call through a no-op stub.
    inline nvtxDomainHandle_t TraceDomain()
    {
        static const nvtxDomainHandle_t s_domain = nvtxDomainCreateA("hal_cuda");
        return s_domain;
    }

    class TraceRange
    {
    public:
        explicit TraceRange(const char *name)
        {
            nvtxEventAttributes_t a = {};
            a.version = NVTX_VERSION;
            a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
            a.messageType = NVTX_MESSAGE_TYPE_ASCII;
            a.message.ascii = name;
            nvtxDomainRangePushEx(TraceDomain(), &a);
        }
        ~TraceRange() { nvtxDomainRangePop(TraceDomain()); }
        TraceRange(const TraceRange &) = delete;
        TraceRange &operator=(const TraceRange &) = delete;
    };

    // Counts every kernel launch issued by the library (hal_cuda_launch_count).
    extern std::atomic<int64_t> g_launches;
    inline void CountLaunch(int64_t n = 1)
    {
        g_launches.fetch_add(n, std::memory_order_relaxed);
    }

    // Device selected for new handles on this thread.
    int CurrentDevice();

    // Grid sizes of the resident handles (for the on-disk format).
    void DiffusionDims(const hal_cuda_diffusion *h, int32_t *xDim, int32_t *yDim);
    void AdiDims(const hal_cuda_adi *h, int32_t *xDim, int32_t *yDim);

    // Device cell offsets of an agent handle's last dispatch (agents.cu) and
    // its grid: the agent count of cell i is offsets[i + 1] - offsets[i].
    const int32_t *AgentsCellOffsets(const hal_cuda_agents *a, int32_t *xDim, int32_t *yDim);

    // Resident agent steps enqueued by another handle on its stream (agents.cu;
    // hal_cuda_adi_run_coupled): Begin orders the agent handle's queued work
    // first and counts the current positions when the last step did not;
    // StepOnce is one hal_cuda_agents_step tick with the linear law; End
    // orders the agent handle's later work after the run.
    struct CoupledStep
    {
        double interactionRad, springConstant, friction, maxVel;
    };
    int CoupledStepBegin(hal_cuda_agents *a, const CoupledStep &st, cudaStream_t s);
    int CoupledStepOnce(hal_cuda_agents *a, const CoupledStep &st, int32_t wrapX, int32_t wrapY, cudaStream_t s);
    int CoupledStepEnd(hal_cuda_agents *a, cudaStream_t s);
    int32_t CoupledAgentCount(const hal_cuda_agents *a);
    bool CoupledBinsPrecounted(const hal_cuda_agents *a);

    // Maps a CUDA error to a status, recording the message.
    inline int CudaStatus(cudaError_t e, const char *what)
    {
        if (e == cudaSuccess)
        {
            return HAL_CUDA_OK;
        }
        SetError("%s: %s", what, cudaGetErrorString(e));
        return (e == cudaErrorMemoryAllocation) ? HAL_CUDA_ENOMEM : HAL_CUDA_EDEVICE;
    }

    // Checks a launch and (for synchronous calls) the stream.
    inline int LaunchStatus(const char *what)
    {
        return CudaStatus(cudaGetLastError(), what);
    }

    // A device buffer owned by a handle.
    template <typename T>
    struct DevBuf
    {
        T *p = nullptr;
        size_t n = 0;

        int Alloc(size_t count, const char *what)
        {
            Free();
            if (count == 0)
            {
                count = 1;
            }
            cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&p), count * sizeof(T));
            if (e != cudaSuccess)
            {
                p = nullptr;
                return CudaStatus(e, what);
            }
            n = count;
            return HAL_CUDA_OK;
        }

        void Free()
        {
            if (p != nullptr)
            {
                cudaFree(p);
            }
            p = nullptr;
            n = 0;
        }

        ~DevBuf()
        {
            Free();
        }
    };

    // A pinned host staging buffer, grown on demand.
    template <typename T>
    struct HostBuf
    {
        T *p = nullptr;
        size_t n = 0;

        int Reserve(size_t count, const char *what)
        {
            if (count <= n)
            {
                return HAL_CUDA_OK;
            }
            Free();
            cudaError_t e = cudaMallocHost(reinterpret_cast<void **>(&p), count * sizeof(T));
            if (e != cudaSuccess)
            {
                p = nullptr;
                return CudaStatus(e, what);
            }
            n = count;
            return HAL_CUDA_OK;
        }

        void Free()
        {
            if (p != nullptr)
            {
                cudaFreeHost(p);
            }
            p = nullptr;
            n = 0;
        }

        ~HostBuf()
        {
            Free();
        }
    };

    // The stream a handle runs on: its own, or one the caller supplied.
    struct StreamSlot
    {
        cudaStream_t own = nullptr;
        cudaStream_t user = nullptr;
        bool hasUser = false;

        // priority: CUDA's stream priority (0 is the default and the lowest;
        // cudaDeviceGetStreamPriorityRange gives the highest, a negative value)
        int Create(const char *what, int priority = 0)
        {
            return CudaStatus(cudaStreamCreateWithPriority(&own, cudaStreamNonBlocking, priority), what);
        }

        cudaStream_t Get() const
        {
            return hasUser ? user : own;
        }

        void Set(void *s)
        {
            hasUser = (s != nullptr);
            user = static_cast<cudaStream_t>(s);
        }

        ~StreamSlot()
        {
            if (own != nullptr)
            {
                cudaStreamDestroy(own);
            }
        }
    };

    // An event without timing, for ordering streams (fork and join).
    struct EventSlot
    {
        cudaEvent_t e = nullptr;

        int Create(const char *what)
        {
            return CudaStatus(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), what);
        }

        ~EventSlot()
        {
            if (e != nullptr)
            {
                cudaEventDestroy(e);
            }
        }
    };

    // Cached CUDA graph of a fixed launch sequence, re-captured when its key
    // changes.
    struct GraphCache
    {
        cudaGraphExec_t exec = nullptr;
        std::string key;

        void Reset()
        {
            if (exec != nullptr)
            {
                cudaGraphExecDestroy(exec);
            }
            exec = nullptr;
            key.clear();
        }

        ~GraphCache()
        {
            Reset();
        }
    };

    // Ghost-table offsets (see hal_cuda.h).
    struct GhostView
    {
        const float *xlo;  // bc(-1, y), yDim values
        const float *xhi;  // bc(xDim, y)
        const float *ylo;  // bc(x, -1), xDim values
        const float *yhi;  // bc(x, yDim)
    };

    // Raises a kernel's dynamic shared-memory limit on the calling thread's
    // current device, once per device and size (the attribute is per device).
    class SmemLimit
    {
    public:
        template <typename Kernel>
        int Ensure(Kernel kernel, size_t bytes, const char *what)
        {
            int dev = 0;
            cudaError_t e = cudaGetDevice(&dev);
            if (e != cudaSuccess)
            {
                return CudaStatus(e, what);
            }
            std::lock_guard<std::mutex> lock(m_mu);
            if (static_cast<size_t>(dev) >= m_enabled.size())
            {
                m_enabled.resize(static_cast<size_t>(dev) + 1, 0);
            }
            if (bytes > m_enabled[static_cast<size_t>(dev)])
            {
                e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
                if (e != cudaSuccess)
                {
                    return CudaStatus(e, what);
                }
                m_enabled[static_cast<size_t>(dev)] = bytes;
            }
            return HAL_CUDA_OK;
        }

    private:
        std::mutex m_mu;
        std::vector<size_t> m_enabled;  // by device
    };

    inline GhostView MakeGhostView(const float *g, int32_t xDim, int32_t yDim)
    {
        GhostView v;
        v.xlo = g;
        v.xhi = g ? g + yDim : nullptr;
        v.ylo = g ? g + 2 * yDim : nullptr;
        v.yhi = g ? g + 2 * yDim + xDim : nullptr;
        return v;
    }
}

#define HAL_TRY(expr)                  \
    do                                 \
    {                                  \
        int _rc = (expr);              \
        if (_rc != HAL_CUDA_OK)        \
        {                              \
            return _rc;                \
        }                              \
    } while (0)

#define HAL_REQUIRE(cond, ...)                \
    do                                        \
    {                                         \
        if (!(cond))                          \
        {                                     \
            ::halcuda::SetError(__VA_ARGS__); \
            return HAL_CUDA_EINVAL;           \
        }                                     \
    } while (0)

// Opens a TraceRange named after the enclosing entry point until it returns.
#define HAL_TRACE() ::halcuda::TraceRange halTraceRange_(__func__)
