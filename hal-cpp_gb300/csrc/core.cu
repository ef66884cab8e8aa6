// core.cu -- library-wide entry points: version, errors, device selection.
#include "common.cuh"

#include <cstring>

namespace halcuda
{
    namespace
    {
        thread_local char t_lastError[512] = {0};
        thread_local int t_device = 0;
    }

    std::atomic<int64_t> g_launches{0};

    void SetError(const char *fmt, ...)
    {
        va_list args;
        va_start(args, fmt);
        vsnprintf(t_lastError, sizeof(t_lastError), fmt, args);
        va_end(args);
    }

    void ClearError()
    {
        t_lastError[0] = '\0';
    }

    int CurrentDevice()
    {
        return t_device;
    }

    namespace
    {
        constexpr int kIssueChains = 8;
        constexpr int kIssueIters = 2048;

        // Eight independent chains of FP64 adds per thread: the issue rate of
        // the FP64 pipe (GB300 runs FP64 at a small fraction of FP32).  Each
        // thread writes one value so the chains are not removed.
        __global__ void __launch_bounds__(256) Fp64IssueKernel(double *out, double a, double b)
        {
            double r[kIssueChains];
#pragma unroll
            for (int k = 0; k < kIssueChains; k++)
            {
                r[k] = a + k + threadIdx.x;
            }
            for (int i = 0; i < kIssueIters; i++)
            {
#pragma unroll
                for (int k = 0; k < kIssueChains; k++)
                {
                    r[k] = __dadd_rn(r[k], b);
                }
            }
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < kIssueChains; k++)
            {
                s += r[k];
            }
            out[blockIdx.x * blockDim.x + threadIdx.x] = s;
        }
    }
}

extern "C" const char *hal_cuda_version(void)
{
    return "hal_cuda 0.1 (sm_103a)";
}

extern "C" const char *hal_cuda_last_error(void)
{
    return halcuda::t_lastError;
}

extern "C" int hal_cuda_device_count(int32_t *count)
{
    HAL_REQUIRE(count != nullptr, "hal_cuda_device_count: count is NULL");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess)
    {
        *count = 0;
        return halcuda::CudaStatus(e, "cudaGetDeviceCount");
    }
    *count = n;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_set_device(int32_t device)
{
    int n = 0;
    HAL_TRY(halcuda::CudaStatus(cudaGetDeviceCount(&n), "cudaGetDeviceCount"));
    HAL_REQUIRE(device >= 0 && device < n, "hal_cuda_set_device: device %d of %d", device, n);
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(device), "cudaSetDevice"));
    halcuda::t_device = device;
    return HAL_CUDA_OK;
}

extern "C" int64_t hal_cuda_launch_count(void)
{
    return halcuda::g_launches.load();
}

extern "C" int hal_cuda_fp64_issue_rate(double *opsPerSecond)
{
    HAL_REQUIRE(opsPerSecond != nullptr, "hal_cuda_fp64_issue_rate: NULL argument");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(t_device), "cudaSetDevice"));
    int sms = 0;
    HAL_TRY(CudaStatus(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, t_device), "cudaDeviceGetAttribute"));
    const unsigned blocks = static_cast<unsigned>(sms) * 8u, threads = 256u;
    double *out = nullptr;
    HAL_TRY(CudaStatus(cudaMalloc(&out, sizeof(double) * blocks * threads), "cudaMalloc(fp64 probe)"));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = CudaStatus(cudaEventCreate(&e0), "cudaEventCreate");
    if (rc == HAL_CUDA_OK)
    {
        rc = CudaStatus(cudaEventCreate(&e1), "cudaEventCreate");
    }
    float best = 0.0f;
    for (int rep = 0; rep < 4 && rc == HAL_CUDA_OK; rep++)
    {
        cudaEventRecord(e0, 0);
        Fp64IssueKernel<<<blocks, threads, 0, 0>>>(out, 1.0, 1e-9);
        CountLaunch();
        cudaEventRecord(e1, 0);
        rc = LaunchStatus("Fp64IssueKernel launch");
        if (rc == HAL_CUDA_OK)
        {
            rc = CudaStatus(cudaEventSynchronize(e1), "hal_cuda_fp64_issue_rate");
        }
        float ms = 0.0f;
        if (rc == HAL_CUDA_OK)
        {
            cudaEventElapsedTime(&ms, e0, e1);
            best = (rep == 1 || ms < best) ? ms : best;  // the first launch is warm-up
        }
    }
    if (e0 != nullptr)
    {
        cudaEventDestroy(e0);
    }
    if (e1 != nullptr)
    {
        cudaEventDestroy(e1);
    }
    cudaFree(out);
    HAL_TRY(rc);
    *opsPerSecond = static_cast<double>(blocks) * threads * kIssueIters * kIssueChains / (best * 1e-3);
    return HAL_CUDA_OK;
}
