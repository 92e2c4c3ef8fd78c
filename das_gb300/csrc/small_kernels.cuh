// small_kernels.cuh -- elementwise helper kernels shared by the engine files.
#pragma once

#include <algorithm>

#include "w2d_common.cuh"

namespace w2d {

// ---- small elementwise kernels ------------------------------------------------
static __global__ void v2dt2_kernel(float* out, const float* vel, size_t n, float dt2)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float v = vel[i];
        out[i] = fmul(fmul(v, v), dt2);  // v * v * dt2 (wave2d.c:60-61)
    }
}

static __global__ void scale_kernel(float* a, size_t n, float s)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        a[i] = fmul(a[i], s);
}

static __global__ void add_kernel(float* acc, const float* x, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        acc[i] = fadd(acc[i], x[i]);
}

static __global__ void correlate_kernel(const float* src, const float* rec, float* image, size_t n,
                                 float dt)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        image[i] = fadd(image[i], fmul(fmul(src[i], rec[i]), dt));
}

static inline int grid_for(size_t n, int block = 256)
{
    size_t b = (n + block - 1) / block;
    return (int)std::min<size_t>(b, 152 * 16);
}

}  // namespace w2d
