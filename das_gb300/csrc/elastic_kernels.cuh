// elastic_kernels.cuh -- 2D elastic velocity-stress step (Levander staggered
// grid, 4th order in space) for sm_103a.
//
// Follows tsw_rtm/c_engine/wave2d.c:95-212: a velocity phase that reads the
// stresses, then a stress phase that reads the UPDATED velocities, each on rows
// [1 if free surface else 2, nz-2) and columns [2, nx-2), each multiplied by the
// sponge; then, with the free surface, szz = sxz = 0 on row 0 and sxx on row 0
// from the free-surface relation.  The two phases are two launches (the stress
// phase needs velocities of neighbouring tiles).  Where the reference reads row
// -1 (sxz in the velocity phase, vz in the stress phase, at iz = 1) this engine
// reads zero.  Arithmetic is float32 in the reference's operation order without
// contraction into FMA.
#pragma once

#include "w2d_common.cuh"

namespace w2d {

struct ElGeom {
    int nx, nz, ldx;
    float rdx, rdz;  // 1/dx, 1/dz
    float dt;
    int free_surface;
    const float* sponge;  // pitched, or null
};

struct ElFields {
    float *vx, *vz, *sxx, *szz, *sxz;
    const float *lam, *mu, *bx, *bz;
};

// c1*(a[+s]-a[0]) + c2*(a[+2s]-a[-s])
__device__ __forceinline__ float el_dfwd(float am1, float a0, float ap1, float ap2)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return fadd(fmul(k1, fsub(ap1, a0)), fmul(k2, fsub(ap2, am1)));
}
// c1*(a[0]-a[-s]) + c2*(a[+s]-a[-2s])
__device__ __forceinline__ float el_dbwd(float am2, float am1, float a0, float ap1)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return fadd(fmul(k1, fsub(a0, am1)), fmul(k2, fsub(ap1, am2)));
}

static __global__ void __launch_bounds__(256) elastic_velocity_kernel(ElGeom g, ElFields f)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y * blockDim.y + threadIdx.y;
    const int z0 = g.free_surface ? 1 : 2;
    if (ix < 2 || ix >= g.nx - 2 || iz < z0 || iz >= g.nz - 2) return;
    const int L = g.ldx;
    const size_t c = (size_t)iz * L + ix;
    const float* sxx = f.sxx;
    const float* sxz = f.sxz;
    const float* szz = f.szz;
    const float sxz_m2z = iz >= 2 ? __ldg(sxz + c - 2 * L) : 0.0f;
    const float a = fmul(el_dfwd(__ldg(sxx + c - 1), __ldg(sxx + c), __ldg(sxx + c + 1),
                                 __ldg(sxx + c + 2)),
                         g.rdx);
    const float b = fmul(el_dbwd(sxz_m2z, __ldg(sxz + c - L), __ldg(sxz + c), __ldg(sxz + c + L)),
                         g.rdz);
    float vx = fadd(f.vx[c], fmul(fmul(g.dt, __ldg(f.bx + c)), fadd(a, b)));
    const float e = fmul(el_dbwd(__ldg(sxz + c - 2), __ldg(sxz + c - 1), __ldg(sxz + c),
                                 __ldg(sxz + c + 1)),
                         g.rdx);
    const float h = fmul(el_dfwd(__ldg(szz + c - L), __ldg(szz + c), __ldg(szz + c + L),
                                 __ldg(szz + c + 2 * L)),
                         g.rdz);
    float vz = fadd(f.vz[c], fmul(fmul(g.dt, __ldg(f.bz + c)), fadd(e, h)));
    if (g.sponge) {
        const float s = __ldg(g.sponge + c);
        vx = fmul(vx, s);
        vz = fmul(vz, s);
    }
    f.vx[c] = vx;
    f.vz[c] = vz;
}

static __global__ void __launch_bounds__(256) elastic_stress_kernel(ElGeom g, ElFields f)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y * blockDim.y + threadIdx.y;
    const int L = g.ldx;
    const float* vx = f.vx;
    const float* vz = f.vz;
    if (g.free_surface && iz == 0 && ix < g.nx) {
        // free-surface row (wave2d.c:198-211)
        f.szz[ix] = 0.0f;
        f.sxz[ix] = 0.0f;
        if (ix >= 2 && ix < g.nx - 2) {
            const float l = __ldg(f.lam + ix), m = __ldg(f.mu + ix);
            const float ex = fmul(el_dbwd(vx[ix - 2], vx[ix - 1], vx[ix], vx[ix + 1]), g.rdx);
            const float num = fmul(fmul(4.0f, m), fadd(l, m));
            const float den = fadd(fadd(l, fmul(2.0f, m)), 1e-8f);
            f.sxx[ix] = fmul(__fdiv_rn(num, den), ex);
        }
        return;
    }
    const int z0 = g.free_surface ? 1 : 2;
    if (ix < 2 || ix >= g.nx - 2 || iz < z0 || iz >= g.nz - 2) return;
    const size_t c = (size_t)iz * L + ix;
    const float vz_m2z = iz >= 2 ? vz[c - 2 * L] : 0.0f;
    const float ex = fmul(el_dbwd(vx[c - 2], vx[c - 1], vx[c], vx[c + 1]), g.rdx);
    const float ez = fmul(el_dbwd(vz_m2z, vz[c - L], vz[c], vz[c + L]), g.rdz);
    const float l = __ldg(f.lam + c), m = __ldg(f.mu + c);
    const float l2m = fadd(l, fmul(2.0f, m));
    float sxx = fadd(f.sxx[c], fmul(g.dt, fadd(fmul(l2m, ex), fmul(l, ez))));
    float szz = fadd(f.szz[c], fmul(g.dt, fadd(fmul(l, ex), fmul(l2m, ez))));
    const float gx = fmul(el_dfwd(vz[c - 1], vz[c], vz[c + 1], vz[c + 2]), g.rdx);
    const float hz = fmul(el_dfwd(vx[c - L], vx[c], vx[c + L], vx[c + 2 * L]), g.rdz);
    float sxz = fadd(f.sxz[c], fmul(fmul(g.dt, m), fadd(gx, hz)));
    if (g.sponge) {
        const float s = __ldg(g.sponge + c);
        sxx = fmul(sxx, s);
        szz = fmul(szz, s);
        sxz = fmul(sxz, s);
    }
    f.sxx[c] = sxx;
    f.szz[c] = szz;
    f.sxz[c] = sxz;
}

inline void launch_elastic_step(const ElGeom& g, const ElFields& f, cudaStream_t st)
{
    dim3 block(32, 8);
    dim3 grid((g.nx + 31) / 32, (g.nz + 7) / 8);
    elastic_velocity_kernel<<<grid, block, 0, st>>>(g, f);
    elastic_stress_kernel<<<grid, block, 0, st>>>(g, f);
}

}  // namespace w2d
