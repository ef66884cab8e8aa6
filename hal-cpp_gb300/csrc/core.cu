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
