// elastic.cu -- reference-compatible elastic_2d_step entry point.
#include <string.h>

#include <mutex>

#include "elastic_kernels.cuh"
#include "w2d_common.cuh"
#include "wave2d_cuda.h"

using namespace w2d;

namespace {

std::mutex g_mu;
float* g_buf = nullptr;
size_t g_cap = 0;
cudaStream_t g_stream = nullptr;

int legacy_elastic(float* vx, float* vz, float* sxx, float* szz, float* sxz, const float* lam,
                   const float* mu, const float* bx, const float* bz, const float* sponge, int nx,
                   int nz, float dx, float dz, float dt, int fs)
{
    W2D_CHECK_ARG(vx && vz && sxx && szz && sxz && lam && mu && bx && bz, "NULL field");
    W2D_CHECK_ARG(nx >= 5 && nz >= 5, "grid must be at least 5 x 5");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_stream && cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking)) {
        set_error("stream creation failed");
        return W2D_ECUDA;
    }
    const int ldx = pitch_for(nx);
    const size_t plane = (size_t)ldx * nz;
    if (g_cap < 10 * plane) {
        if (g_buf) cudaFree(g_buf);
        g_buf = nullptr;
        g_cap = 0;
        if (cudaMalloc(&g_buf, 10 * plane * 4) != cudaSuccess) {
            cudaGetLastError();
            set_error("device allocation failed");
            return W2D_ENOMEM;
        }
        g_cap = 10 * plane;
    }
    float* d[10];
    for (int i = 0; i < 10; ++i) d[i] = g_buf + (size_t)i * plane;
    const float* host_in[10] = {vx, vz, sxx, szz, sxz, lam, mu, bx, bz, sponge};
    const size_t hp = (size_t)nx * 4, dp = (size_t)ldx * 4;
    for (int i = 0; i < 10; ++i)
        if (host_in[i])
            W2D_CUDA_TRY(cudaMemcpy2DAsync(d[i], dp, host_in[i], hp, hp, nz,
                                           cudaMemcpyHostToDevice, g_stream));
    ElGeom g;
    g.nx = nx;
    g.nz = nz;
    g.ldx = ldx;
    g.rdx = 1.0f / dx;
    g.rdz = 1.0f / dz;
    g.dt = dt;
    g.free_surface = fs ? 1 : 0;
    g.sponge = sponge ? d[9] : nullptr;
    ElFields f{d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8]};
    launch_elastic_step(g, f, g_stream);
    W2D_CUDA_TRY(cudaGetLastError());
    float* host_out[5] = {vx, vz, sxx, szz, sxz};
    for (int i = 0; i < 5; ++i)
        W2D_CUDA_TRY(cudaMemcpy2DAsync(host_out[i], hp, d[i], dp, hp, nz, cudaMemcpyDeviceToHost,
                                       g_stream));
    W2D_CUDA_TRY(cudaStreamSynchronize(g_stream));
    return W2D_OK;
}

}  // namespace

extern "C" {

void elastic_2d_step(float* vx, float* vz, float* sxx, float* szz, float* sxz,
                     const float* lambda_, const float* mu, const float* buo_x,
                     const float* buo_z, const float* sponge, int nx, int nz, float dx, float dz,
                     float dt, int free_surface_top)
{
    legacy_elastic(vx, vz, sxx, szz, sxz, lambda_, mu, buo_x, buo_z, sponge, nx, nz, dx, dz, dt,
                   free_surface_top);
}

int w2d_elastic_2d_step_status(float* vx, float* vz, float* sxx, float* szz, float* sxz,
                               const float* lambda_, const float* mu, const float* buo_x,
                               const float* buo_z, const float* sponge, int nx, int nz, float dx,
                               float dz, float dt, int free_surface_top)
{
    return legacy_elastic(vx, vz, sxx, szz, sxz, lambda_, mu, buo_x, buo_z, sponge, nx, nz, dx,
                          dz, dt, free_surface_top);
}

}  // extern "C"
