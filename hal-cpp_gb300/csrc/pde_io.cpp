// pde_io.cpp -- PDEGrid2D's on-disk format for the resident fields.
//
// SavePDEGrid2D / LoadPDEGrid2D (src/Grids/PDEGridSerialization.cpp:34-62)
// write, through BinaryWriter (include/Hal/IO/BinaryWriter.h:36-50), raw
// native-endian values with no padding:
//   int32 xDim, int32 yDim, bool wrapX, bool wrapY (one byte each),
//   int32 updateCt, double field[xDim*yDim], double deltas[xDim*yDim]
// (field in HAL's layout x*yDim + y).  A load fails when the read fails or
// the dimensions are invalid (Internal::CheckLoadedDims,
// src/Grids/GridSerialization.cpp:14-32).  The layout has to match the
// reference byte for byte so that either side can read the other's files.
//
// Host code only: the handle save/load calls move the FP32 device field with
// the handles' own get/set calls.
#include "common.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

namespace
{
    constexpr size_t kHeaderBytes = 4 + 4 + 1 + 1 + 4;

    struct File
    {
        std::FILE *f = nullptr;
        ~File()
        {
            if (f != nullptr)
            {
                std::fclose(f);
            }
        }
    };

    bool DimsOk(int32_t xDim, int32_t yDim)
    {
        return xDim > 0 && yDim > 0 &&
               static_cast<int64_t>(xDim) * yDim <= std::numeric_limits<int32_t>::max();
    }

    int ReadHeader(std::FILE *f, const char *path, int32_t *xDim, int32_t *yDim, int32_t *wrapX, int32_t *wrapY,
                   int32_t *updateCt)
    {
        unsigned char h[kHeaderBytes];
        if (std::fread(h, 1, kHeaderBytes, f) != kHeaderBytes)
        {
            ::halcuda::SetError("LoadPDEGrid2D: failed read or invalid dimensions in saved data (%s)", path);
            return HAL_CUDA_EINVAL;
        }
        int32_t x, y, u;
        std::memcpy(&x, h, 4);
        std::memcpy(&y, h + 4, 4);
        std::memcpy(&u, h + 10, 4);
        if (!DimsOk(x, y))
        {
            ::halcuda::SetError("LoadPDEGrid2D: failed read or invalid dimensions in saved data (%s)", path);
            return HAL_CUDA_EINVAL;
        }
        *xDim = x;
        *yDim = y;
        *wrapX = h[8] != 0;
        *wrapY = h[9] != 0;
        *updateCt = u;
        return HAL_CUDA_OK;
    }

    int Write(const char *path, int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY, int32_t updateCt,
              const double *field, const double *deltas)
    {
        File file;
        file.f = std::fopen(path, "wb");
        HAL_REQUIRE(file.f != nullptr, "BinaryWriter failed to open file for writing: %s", path);
        unsigned char h[kHeaderBytes];
        const unsigned char wx = wrapX != 0, wy = wrapY != 0;
        std::memcpy(h, &xDim, 4);
        std::memcpy(h + 4, &yDim, 4);
        h[8] = wx;
        h[9] = wy;
        std::memcpy(h + 10, &updateCt, 4);
        const size_t n = static_cast<size_t>(xDim) * static_cast<size_t>(yDim);
        bool ok = std::fwrite(h, 1, kHeaderBytes, file.f) == kHeaderBytes;
        ok = ok && std::fwrite(field, sizeof(double), n, file.f) == n;
        if (deltas != nullptr)
        {
            ok = ok && std::fwrite(deltas, sizeof(double), n, file.f) == n;
        }
        else
        {
            const std::vector<double> zeros(n, 0.0);
            ok = ok && std::fwrite(zeros.data(), sizeof(double), n, file.f) == n;
        }
        ok = (std::fclose(file.f) == 0) && ok;
        file.f = nullptr;
        if (!ok)
        {
            ::halcuda::SetError("BinaryWriter write failed: %s", path);
            return HAL_CUDA_EDEVICE;
        }
        return HAL_CUDA_OK;
    }

    // Reads a file whose grid must be xDim x yDim; deltas may be NULL (then
    // they are read and discarded).
    int Read(const char *path, int32_t xDim, int32_t yDim, double *field, double *deltas, int32_t *wrapX,
             int32_t *wrapY, int32_t *updateCt)
    {
        File file;
        file.f = std::fopen(path, "rb");
        HAL_REQUIRE(file.f != nullptr, "BinaryReader failed to open file for reading: %s", path);
        int32_t x = 0, y = 0;
        HAL_TRY(ReadHeader(file.f, path, &x, &y, wrapX, wrapY, updateCt));
        HAL_REQUIRE(x == xDim && y == yDim, "LoadPDEGrid2D: saved grid is %d x %d, the handle's %d x %d (%s)", x, y,
                    xDim, yDim, path);
        const size_t n = static_cast<size_t>(xDim) * static_cast<size_t>(yDim);
        std::vector<double> scratch;
        if (deltas == nullptr)
        {
            scratch.resize(n);
            deltas = scratch.data();
        }
        const bool ok = std::fread(field, sizeof(double), n, file.f) == n &&
                        std::fread(deltas, sizeof(double), n, file.f) == n;
        HAL_REQUIRE(ok, "LoadPDEGrid2D: failed read or invalid dimensions in saved data (%s)", path);
        return HAL_CUDA_OK;
    }

    // Save / load of a resident FP32 field through the handle's get/set calls.
    template <typename GetField>
    int SaveResident(const char *path, int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY, int32_t updateCt,
                     GetField get)
    {
        const size_t n = static_cast<size_t>(xDim) * static_cast<size_t>(yDim);
        std::vector<float> f32(n);
        HAL_TRY(get(f32.data(), static_cast<int64_t>(n)));
        std::vector<double> f64(f32.begin(), f32.end());
        return Write(path, xDim, yDim, wrapX, wrapY, updateCt, f64.data(), nullptr);
    }

    template <typename SetField>
    int LoadResident(const char *path, int32_t xDim, int32_t yDim, int32_t *wrapX, int32_t *wrapY,
                     int32_t *updateCt, SetField set)
    {
        const size_t n = static_cast<size_t>(xDim) * static_cast<size_t>(yDim);
        std::vector<double> f64(n), d64(n);
        int32_t wx = 0, wy = 0, u = 0;
        HAL_TRY(Read(path, xDim, yDim, f64.data(), d64.data(), &wx, &wy, &u));
        for (double d : d64)
        {
            if (d != 0.0)
            {
                ::halcuda::SetError("LoadPDEGrid2D: %s holds deltas pending an Update(); a resident field has none",
                                    path);
                return HAL_CUDA_ENOTSUP;
            }
        }
        std::vector<float> f32(f64.begin(), f64.end());
        HAL_TRY(set(f32.data(), static_cast<int64_t>(n)));
        if (wrapX != nullptr)
        {
            *wrapX = wx;
        }
        if (wrapY != nullptr)
        {
            *wrapY = wy;
        }
        if (updateCt != nullptr)
        {
            *updateCt = u;
        }
        return HAL_CUDA_OK;
    }
}

extern "C" int hal_cuda_pdegrid2d_write(const char *path, int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY,
                                        int32_t updateCt, const double *field, const double *deltas)
{
    HAL_REQUIRE(path != nullptr && field != nullptr, "hal_cuda_pdegrid2d_write: NULL argument");
    HAL_REQUIRE(DimsOk(xDim, yDim), "hal_cuda_pdegrid2d_write: invalid dimensions %d x %d", xDim, yDim);
    return Write(path, xDim, yDim, wrapX, wrapY, updateCt, field, deltas);
}

extern "C" int hal_cuda_pdegrid2d_read_header(const char *path, int32_t *xDim, int32_t *yDim, int32_t *wrapX,
                                              int32_t *wrapY, int32_t *updateCt)
{
    HAL_REQUIRE(path != nullptr && xDim != nullptr && yDim != nullptr && wrapX != nullptr && wrapY != nullptr &&
                    updateCt != nullptr,
                "hal_cuda_pdegrid2d_read_header: NULL argument");
    File file;
    file.f = std::fopen(path, "rb");
    HAL_REQUIRE(file.f != nullptr, "BinaryReader failed to open file for reading: %s", path);
    return ReadHeader(file.f, path, xDim, yDim, wrapX, wrapY, updateCt);
}

extern "C" int hal_cuda_pdegrid2d_read(const char *path, int32_t xDim, int32_t yDim, double *field, double *deltas)
{
    HAL_REQUIRE(path != nullptr && field != nullptr, "hal_cuda_pdegrid2d_read: NULL argument");
    int32_t wx, wy, u;
    return Read(path, xDim, yDim, field, deltas, &wx, &wy, &u);
}

extern "C" int hal_cuda_diffusion_save(hal_cuda_diffusion *h, const char *path, int32_t wrapX, int32_t wrapY,
                                       int32_t updateCt)
{
    HAL_REQUIRE(h != nullptr && path != nullptr, "hal_cuda_diffusion_save: NULL argument");
    int32_t xDim, yDim;
    halcuda::DiffusionDims(h, &xDim, &yDim);
    return SaveResident(path, xDim, yDim, wrapX, wrapY, updateCt,
                        [h](float *f, int64_t n) { return hal_cuda_diffusion_get_field(h, f, n); });
}

extern "C" int hal_cuda_diffusion_load(hal_cuda_diffusion *h, const char *path, int32_t *wrapX, int32_t *wrapY,
                                       int32_t *updateCt)
{
    HAL_REQUIRE(h != nullptr && path != nullptr, "hal_cuda_diffusion_load: NULL argument");
    int32_t xDim, yDim;
    halcuda::DiffusionDims(h, &xDim, &yDim);
    return LoadResident(path, xDim, yDim, wrapX, wrapY, updateCt,
                        [h](const float *f, int64_t n) { return hal_cuda_diffusion_set_field(h, f, n); });
}

extern "C" int hal_cuda_adi_save(hal_cuda_adi *h, const char *path, int32_t wrapX, int32_t wrapY, int32_t updateCt)
{
    HAL_REQUIRE(h != nullptr && path != nullptr, "hal_cuda_adi_save: NULL argument");
    int32_t xDim, yDim;
    halcuda::AdiDims(h, &xDim, &yDim);
    return SaveResident(path, xDim, yDim, wrapX, wrapY, updateCt,
                        [h](float *f, int64_t n) { return hal_cuda_adi_get_field(h, f, n); });
}

extern "C" int hal_cuda_adi_load(hal_cuda_adi *h, const char *path, int32_t *wrapX, int32_t *wrapY,
                                 int32_t *updateCt)
{
    HAL_REQUIRE(h != nullptr && path != nullptr, "hal_cuda_adi_load: NULL argument");
    int32_t xDim, yDim;
    halcuda::AdiDims(h, &xDim, &yDim);
    return LoadResident(path, xDim, yDim, wrapX, wrapY, updateCt,
                        [h](const float *f, int64_t n) { return hal_cuda_adi_set_field(h, f, n); });
}
