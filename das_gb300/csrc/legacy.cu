// legacy.cu -- the reference engine's per-step C functions (wave2d.c) on the GPU.
//
// acoustic_2d_step, elastic_2d_step and correlate_imaging_condition keep the
// reference signatures: the caller passes host arrays of nz x nx floats, the
// call is synchronous.  One mutex-guarded context holds a stream, page-locked
// staging memory and pitched device buffers that grow with the largest grid
// seen; every device operation is ordered on that one stream.
#include <string.h>

#include <mutex>

#include "acoustic_kernels.cuh"
#include "elastic_kernels.cuh"
#include "small_kernels.cuh"
#include "w2d_common.cuh"
#include "wave2d_cuda.h"

using namespace w2d;

namespace {

struct LegacyCtx {
    std::mutex mu;
    cudaStream_t st = nullptr;
    float* dev = nullptr;  // device planes
    size_t dev_cap = 0;    // floats
    float* pin = nullptr;  // page-locked staging (packed nz x nx planes)
    size_t pin_cap = 0;    // floats
    int* shot = nullptr;   // {-1,-1,-1,0,-1}: no source, no receivers
    int* rec_ptr = nullptr;
    int rec_cap = 0;
    unsigned* err = nullptr;
    AcMaps tm;
    const float* tm_base = nullptr;
    int tm_nx = 0, tm_nz = 0;
};
LegacyCtx g;

int prepare(int n_planes_dev, size_t plane_dev, int n_planes_pin, size_t plane_pin, int nx)
{
    if (!g.st) W2D_CUDA_TRY(cudaStreamCreateWithFlags(&g.st, cudaStreamNonBlocking));
    if (!g.shot) {
        W2D_CUDA_TRY(cudaMalloc(&g.shot, 5 * sizeof(int)));
        W2D_CUDA_TRY(cudaMalloc(&g.err, sizeof(unsigned)));
        const int sh[5] = {-1, -1, -1, 0, -1};
        W2D_CUDA_TRY(cudaMemcpyAsync(g.shot, sh, sizeof sh, cudaMemcpyHostToDevice, g.st));
        W2D_CUDA_TRY(cudaMemsetAsync(g.err, 0, sizeof(unsigned), g.st));
        W2D_CUDA_TRY(cudaStreamSynchronize(g.st));
    }
    const size_t need_dev = (size_t)n_planes_dev * plane_dev;
    if (need_dev > g.dev_cap) {
        W2D_CUDA_TRY(cudaStreamSynchronize(g.st));
        if (g.dev) cudaFree(g.dev);
        g.dev = nullptr;
        g.dev_cap = 0;
        g.tm_base = nullptr;
        if (cudaMalloc(&g.dev, need_dev * 4) != cudaSuccess) {
            cudaGetLastError();
            set_error("device allocation failed");
            return W2D_ENOMEM;
        }
        g.dev_cap = need_dev;
    }
    const size_t need_pin = (size_t)n_planes_pin * plane_pin;
    if (need_pin > g.pin_cap) {
        if (g.pin) cudaFreeHost(g.pin);
        g.pin = nullptr;
        g.pin_cap = 0;
        W2D_CUDA_TRY(cudaMallocHost(&g.pin, need_pin * 4));
        g.pin_cap = need_pin;
    }
    if (nx + 1 > g.rec_cap) {
        if (g.rec_ptr) cudaFree(g.rec_ptr);
        g.rec_ptr = nullptr;
        W2D_CUDA_TRY(cudaMalloc(&g.rec_ptr, (nx + 1) * sizeof(int)));
        W2D_CUDA_TRY(cudaMemsetAsync(g.rec_ptr, 0, (nx + 1) * sizeof(int), g.st));
        g.rec_cap = nx + 1;
    }
    return W2D_OK;
}

// host array (nz x nx) -> staging slot k -> pitched device plane
int upload(float* dplane, int k, const float* host, int nx, int nz, int ldx)
{
    const size_t n = (size_t)nx * nz;
    float* stage = g.pin + (size_t)k * n;
    memcpy(stage, host, n * 4);
    W2D_CUDA_TRY(cudaMemcpy2DAsync(dplane, (size_t)ldx * 4, stage, (size_t)nx * 4, (size_t)nx * 4,
                                   nz, cudaMemcpyHostToDevice, g.st));
    return W2D_OK;
}

int download(float* host, int k, const float* dplane, int nx, int nz, int ldx)
{
    W2D_CUDA_TRY(cudaMemcpy2DAsync(g.pin + (size_t)k * nx * nz, (size_t)nx * 4, dplane,
                                   (size_t)ldx * 4, (size_t)nx * 4, nz, cudaMemcpyDeviceToHost,
                                   g.st));
    return W2D_OK;
}

int finish_downloads(float* const* hosts, const int* slots, int count, int nx, int nz)
{
    W2D_CUDA_TRY(cudaStreamSynchronize(g.st));
    const size_t n = (size_t)nx * nz;
    for (int i = 0; i < count; ++i) memcpy(hosts[i], g.pin + (size_t)slots[i] * n, n * 4);
    return W2D_OK;
}

int legacy_acoustic(const float* p_curr, const float* p_prev, float* p_next, const float* vel,
                    const float* sponge, int nx, int nz, float dx, float dz, float dt, int fs)
{
    W2D_CHECK_ARG(p_curr && p_prev && p_next && vel, "NULL field");
    W2D_CHECK_ARG(nx >= 5 && nz >= 5, "grid must be at least 5 x 5");
    std::lock_guard<std::mutex> lk(g.mu);
    const int ldx = pitch_for(nx);
    const size_t plane = (size_t)ldx * nz;
    int rc;
    if ((rc = prepare(6, plane, 5, (size_t)nx * nz, nx))) return rc;
    float* d = g.dev;
    float *dc = d, *dprev = d + plane, *dn = d + 2 * plane, *dv = d + 3 * plane,
          *ds = d + 4 * plane, *dvel = d + 5 * plane;
    if (g.tm_base != dc || g.tm_nx != nx || g.tm_nz != nz) {
        if ((rc = make_ac_maps(&g.tm, dc, dprev, dv, ds, nx, nz, ldx, 32))) return rc;
        g.tm_base = dc;
        g.tm_nx = nx;
        g.tm_nz = nz;
    }
    if ((rc = upload(dc, 0, p_curr, nx, nz, ldx)) || (rc = upload(dprev, 1, p_prev, nx, nz, ldx)) ||
        (rc = upload(dn, 2, p_next, nx, nz, ldx)) || (rc = upload(dvel, 3, vel, nx, nz, ldx)))
        return rc;
    if (sponge && (rc = upload(ds, 4, sponge, nx, nz, ldx))) return rc;
    v2dt2_kernel<<<grid_for(plane), 256, 0, g.st>>>(dv, dvel, plane, dt * dt);
    AcGeom geo;
    memset(&geo, 0, sizeof geo);
    geo.nx = nx;
    geo.nz = nz;
    geo.ldx = ldx;
    geo.inv_dx2 = 1.0f / (dx * dx);
    geo.inv_dz2 = 1.0f / (dz * dz);
    geo.free_surface = fs ? 1 : 0;
    geo.rec_ptr = g.rec_ptr;
    geo.rec_list = g.rec_ptr;
    geo.shot = g.shot;
    AcStep s;
    memset(&s, 0, sizeof s);
    s.p_next = dn;
    s.err = g.err;
    if (sponge)
        W2D_CUDA_TRY((launch_acoustic_step<8, 4, SPONGE_ARRAY>(g.tm, geo, s, g.st)));
    else
        W2D_CUDA_TRY((launch_acoustic_step<8, 4, SPONGE_NONE>(g.tm, geo, s, g.st)));
    if ((rc = download(p_next, 0, dn, nx, nz, ldx))) return rc;
    unsigned h = 0;
    W2D_CUDA_TRY(cudaMemcpyAsync(&h, g.err, 4, cudaMemcpyDeviceToHost, g.st));
    float* outs[1] = {p_next};
    int slots[1] = {0};
    if ((rc = finish_downloads(outs, slots, 1, nx, nz))) return rc;
    if (h) {
        cudaMemsetAsync(g.err, 0, 4, g.st);
        set_error("device wait gave up in acoustic_2d_step");
        return W2D_ETIMEOUT;
    }
    return W2D_OK;
}

int legacy_correlate(const float* src, const float* rec, float* image, int nx, int nz, float dt)
{
    W2D_CHECK_ARG(src && rec && image && nx > 0 && nz > 0, "bad arguments");
    std::lock_guard<std::mutex> lk(g.mu);
    const size_t n = (size_t)nx * nz;
    int rc;
    if ((rc = prepare(3, n, 3, n, nx))) return rc;
    float* d = g.dev;
    // flat arrays: one row of n floats each
    if ((rc = upload(d, 0, src, (int)n, 1, (int)n)) || (rc = upload(d + n, 1, rec, (int)n, 1, (int)n)) ||
        (rc = upload(d + 2 * n, 2, image, (int)n, 1, (int)n)))
        return rc;
    correlate_kernel<<<grid_for(n), 256, 0, g.st>>>(d, d + n, d + 2 * n, n, dt);
    W2D_CUDA_TRY(cudaGetLastError());
    if ((rc = download(image, 2, d + 2 * n, (int)n, 1, (int)n))) return rc;
    float* outs[1] = {image};
    int slots[1] = {2};
    return finish_downloads(outs, slots, 1, (int)n, 1);
}

int legacy_elastic(float* vx, float* vz, float* sxx, float* szz, float* sxz, const float* lam,
                   const float* mu, const float* bx, const float* bz, const float* sponge, int nx,
                   int nz, float dx, float dz, float dt, int fs)
{
    W2D_CHECK_ARG(vx && vz && sxx && szz && sxz && lam && mu && bx && bz, "NULL field");
    W2D_CHECK_ARG(nx >= 5 && nz >= 5, "grid must be at least 5 x 5");
    std::lock_guard<std::mutex> lk(g.mu);
    const int ldx = pitch_for(nx);
    const size_t plane = (size_t)ldx * nz;
    int rc;
    if ((rc = prepare(10, plane, 10, (size_t)nx * nz, nx))) return rc;
    float* d[10];
    for (int i = 0; i < 10; ++i) d[i] = g.dev + (size_t)i * plane;
    const float* in[10] = {vx, vz, sxx, szz, sxz, lam, mu, bx, bz, sponge};
    for (int i = 0; i < 10; ++i)
        if (in[i] && (rc = upload(d[i], i, in[i], nx, nz, ldx))) return rc;
    ElGeom geo;
    geo.nx = nx;
    geo.nz = nz;
    geo.ldx = ldx;
    geo.rdx = 1.0f / dx;
    geo.rdz = 1.0f / dz;
    geo.dt = dt;
    geo.free_surface = fs ? 1 : 0;
    geo.sponge = sponge ? d[9] : nullptr;
    ElMaps maps;
    if ((rc = make_el_state_map(&maps.src, d[0], nx, nz, ldx, plane))) return rc;
    maps.dst = maps.src;
    ElStep st;
    st.src = d[0];
    st.dst = d[0];
    st.plane = plane;
    st.lam = d[5];
    st.mu = d[6];
    st.bx = d[7];
    st.bz = d[8];
    st.pstride = 0;
    st.src_pos = nullptr;  // no source term
    st.wav = nullptr;
    st.nt = st.n = 0;
    st.err = g.err;
    W2D_CUDA_TRY(launch_elastic_step(geo, maps, st, g.st));
    {
        unsigned h = 0;
        W2D_CUDA_TRY(cudaMemcpyAsync(&h, g.err, 4, cudaMemcpyDeviceToHost, g.st));
        W2D_CUDA_TRY(cudaStreamSynchronize(g.st));
        if (h) {
            cudaMemsetAsync(g.err, 0, 4, g.st);
            set_error("device wait gave up in elastic_2d_step");
            return W2D_ETIMEOUT;
        }
    }
    float* outs[5] = {vx, vz, sxx, szz, sxz};
    int slots[5] = {0, 1, 2, 3, 4};
    for (int i = 0; i < 5; ++i)
        if ((rc = download(outs[i], i, d[i], nx, nz, ldx))) return rc;
    return finish_downloads(outs, slots, 5, nx, nz);
}

}  // namespace

extern "C" {

void acoustic_2d_step(const float* p_curr, const float* p_prev, float* p_next, const float* vel,
                      const float* sponge, int nx, int nz, float dx, float dz, float dt,
                      int free_surface_top)
{
    legacy_acoustic(p_curr, p_prev, p_next, vel, sponge, nx, nz, dx, dz, dt, free_surface_top);
}

int w2d_acoustic_2d_step_status(const float* p_curr, const float* p_prev, float* p_next,
                                const float* vel, const float* sponge, int nx, int nz, float dx,
                                float dz, float dt, int free_surface_top)
{
    return legacy_acoustic(p_curr, p_prev, p_next, vel, sponge, nx, nz, dx, dz, dt,
                           free_surface_top);
}

void correlate_imaging_condition(const float* src_wavefield, const float* rec_wavefield,
                                 float* image, int nx, int nz, float dt)
{
    legacy_correlate(src_wavefield, rec_wavefield, image, nx, nz, dt);
}

int w2d_correlate_status(const float* src, const float* rec, float* image, int nx, int nz,
                         float dt)
{
    return legacy_correlate(src, rec, image, nx, nz, dt);
}

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
