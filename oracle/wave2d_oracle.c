/*
 * wave2d_oracle.c -- CPU restatement of the 2D finite-difference engine of
 * ll23002/DAS (tsw_rtm/c_engine/wave2d.c).  TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker for the CUDA engine in das_gb300/csrc.  Only the
 * test suite, the smoke check and the CPU-baseline leg of bench.py load it.
 * The product path never calls into it.
 *
 * Two arithmetic flavours are provided for every operator:
 *   *_f32  float32, with every product and sum evaluated in the same order as
 *          the reference C source.  Built with -ffp-contract=off, so no
 *          multiply-add is fused and the results are bit-identical to the
 *          reference library compiled for x86-64 (where gcc emits no FMA).
 *   *_f64  the same stencil in float64, used to state the error of every
 *          float32 result against a double-precision run.
 *
 * Reference anchors (paths inside the reference project):
 *   acoustic step     tsw_rtm/c_engine/wave2d.c:19-82
 *   elastic step      tsw_rtm/c_engine/wave2d.c:95-212
 *   imaging condition tsw_rtm/c_engine/wave2d.c:218-231
 *   Cerjan sponge     tsw_rtm/c_engine/wave2d.c:237-265
 *
 * One deliberate definition: the reference elastic step reads row -1 of sxz
 * and vz when the free surface is on (wave2d.c:135 and :170 at iz = 1).  Here
 * row -1 reads as zero.  The parity tests give the reference library two zero
 * guard rows in front of row 0, which produces exactly that value.
 */
#include <math.h>
#include <stddef.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- acoustic: 4th-order Laplacian, 2nd-order leapfrog ------------------ */

/* c2*(a[-2s]+a[+2s]) + c1*(a[-s]+a[+s]) + c0*a[0], summed left to right. */
static inline float d2_f32(const float* a, ptrdiff_t s)
{
    const float k0 = -2.5f, k1 = 4.0f / 3.0f, k2 = -1.0f / 12.0f;
    float far_pair = a[-2 * s] + a[2 * s];
    float near_pair = a[-s] + a[s];
    float acc = k2 * far_pair;
    acc = acc + k1 * near_pair;
    return acc + k0 * a[0];
}

static inline double d2_f64(const double* a, ptrdiff_t s)
{
    const double k0 = -2.5, k1 = 4.0 / 3.0, k2 = -1.0 / 12.0;
    double far_pair = a[-2 * s] + a[2 * s];
    double near_pair = a[-s] + a[s];
    double acc = k2 * far_pair;
    acc = acc + k1 * near_pair;
    return acc + k0 * a[0];
}

/* One acoustic time step.  Same argument meaning as the reference
 * acoustic_2d_step: interior cells 2 <= iz < nz-2, 2 <= ix < nx-2 are written;
 * with the free surface, rows 0 and 1 of p_next are then set over all ix. */
void oracle_acoustic_step_f32(const float* p_curr, const float* p_prev, float* p_next,
                              const float* vel, const float* sponge, int nx, int nz,
                              float dx, float dz, float dt, int free_surface_top)
{
    const float inv_dx2 = 1.0f / (dx * dx);
    const float inv_dz2 = 1.0f / (dz * dz);
    const float dt2 = dt * dt;
    int iz;
#pragma omp parallel for schedule(static)
    for (iz = 2; iz < nz - 2; ++iz) {
        for (int ix = 2; ix < nx - 2; ++ix) {
            const ptrdiff_t c = (ptrdiff_t)iz * nx + ix;
            const float lap_x = d2_f32(p_curr + c, 1) * inv_dx2;
            const float lap_z = d2_f32(p_curr + c, nx) * inv_dz2;
            const float vv = vel[c] * vel[c] * dt2;
            float u = 2.0f * p_curr[c] - p_prev[c] + vv * (lap_x + lap_z);
            if (sponge) u *= sponge[c];
            p_next[c] = u;
        }
    }
    if (free_surface_top) {
        for (int ix = 0; ix < nx; ++ix) {
            p_next[ix] = 0.0f;
            p_next[nx + ix] = -p_next[2 * nx + ix];
        }
    }
}

void oracle_acoustic_step_f64(const double* p_curr, const double* p_prev, double* p_next,
                              const double* vel, const double* sponge, int nx, int nz,
                              double dx, double dz, double dt, int free_surface_top)
{
    const double inv_dx2 = 1.0 / (dx * dx);
    const double inv_dz2 = 1.0 / (dz * dz);
    const double dt2 = dt * dt;
    int iz;
#pragma omp parallel for schedule(static)
    for (iz = 2; iz < nz - 2; ++iz) {
        for (int ix = 2; ix < nx - 2; ++ix) {
            const ptrdiff_t c = (ptrdiff_t)iz * nx + ix;
            const double lap_x = d2_f64(p_curr + c, 1) * inv_dx2;
            const double lap_z = d2_f64(p_curr + c, nx) * inv_dz2;
            const double vv = vel[c] * vel[c] * dt2;
            double u = 2.0 * p_curr[c] - p_prev[c] + vv * (lap_x + lap_z);
            if (sponge) u *= sponge[c];
            p_next[c] = u;
        }
    }
    if (free_surface_top) {
        for (int ix = 0; ix < nx; ++ix) {
            p_next[ix] = 0.0;
            p_next[nx + ix] = -p_next[2 * nx + ix];
        }
    }
}

/* ---- elastic: Levander velocity-stress, 4th-order staggered ------------- */

/* Forward difference about the half point between a[0] and a[s]:
 * c1*(a[s]-a[0]) + c2*(a[2s]-a[-s]). */
static inline float dfwd_f32(const float* a, ptrdiff_t s)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return k1 * (a[s] - a[0]) + k2 * (a[2 * s] - a[-s]);
}
/* Backward difference about the half point between a[-s] and a[0]:
 * c1*(a[0]-a[-s]) + c2*(a[s]-a[-2s]).  `m2` is a[-2s] (row -1 reads zero). */
static inline float dbwd_f32(const float* a, ptrdiff_t s, float m2)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return k1 * (a[0] - a[-s]) + k2 * (a[s] - m2);
}
static inline double dfwd_f64(const double* a, ptrdiff_t s)
{
    const double k1 = 9.0 / 8.0, k2 = -1.0 / 24.0;
    return k1 * (a[s] - a[0]) + k2 * (a[2 * s] - a[-s]);
}
static inline double dbwd_f64(const double* a, ptrdiff_t s, double m2)
{
    const double k1 = 9.0 / 8.0, k2 = -1.0 / 24.0;
    return k1 * (a[0] - a[-s]) + k2 * (a[s] - m2);
}

void oracle_elastic_step_f32(float* vx, float* vz, float* sxx, float* szz, float* sxz,
                             const float* lam, const float* mu, const float* bx,
                             const float* bz, const float* sponge, int nx, int nz,
                             float dx, float dz, float dt, int free_surface_top)
{
    const float rdx = 1.0f / dx, rdz = 1.0f / dz;
    const int z0 = free_surface_top ? 1 : 2;
    const ptrdiff_t n = nx;
    int iz;
    /* velocity phase: stresses are only read */
#pragma omp parallel for schedule(static)
    for (iz = z0; iz < nz - 2; ++iz) {
        for (int ix = 2; ix < nx - 2; ++ix) {
            const ptrdiff_t c = (ptrdiff_t)iz * nx + ix;
            const float sxz_m2 = (iz >= 2) ? sxz[c - 2 * n] : 0.0f;
            const float a = dfwd_f32(sxx + c, 1) * rdx;
            const float b = dbwd_f32(sxz + c, n, sxz_m2) * rdz;
            vx[c] += dt * bx[c] * (a + b);
            const float e = dbwd_f32(sxz + c, 1, sxz[c - 2]) * rdx;
            const float f = dfwd_f32(szz + c, n) * rdz;
            vz[c] += dt * bz[c] * (e + f);
            if (sponge) {
                const float s = sponge[c];
                vx[c] *= s;
                vz[c] *= s;
            }
        }
    }
    /* stress phase: the updated velocities are only read */
#pragma omp parallel for schedule(static)
    for (iz = z0; iz < nz - 2; ++iz) {
        for (int ix = 2; ix < nx - 2; ++ix) {
            const ptrdiff_t c = (ptrdiff_t)iz * nx + ix;
            const float vz_m2 = (iz >= 2) ? vz[c - 2 * n] : 0.0f;
            const float ex = dbwd_f32(vx + c, 1, vx[c - 2]) * rdx;
            const float ez = dbwd_f32(vz + c, n, vz_m2) * rdz;
            const float l = lam[c], m = mu[c];
            sxx[c] += dt * ((l + 2.0f * m) * ex + l * ez);
            szz[c] += dt * (l * ex + (l + 2.0f * m) * ez);
            const float g = dfwd_f32(vz + c, 1) * rdx;
            const float h = dfwd_f32(vx + c, n) * rdz;
            sxz[c] += dt * m * (g + h);
            if (sponge) {
                const float s = sponge[c];
                sxx[c] *= s;
                szz[c] *= s;
                sxz[c] *= s;
            }
        }
    }
    if (free_surface_top) {
        for (int ix = 0; ix < nx; ++ix) {
            szz[ix] = 0.0f;
            sxz[ix] = 0.0f;
            if (ix >= 2 && ix < nx - 2) {
                const float l = lam[ix], m = mu[ix];
                const float ex = dbwd_f32(vx + ix, 1, vx[ix - 2]) * rdx;
                sxx[ix] = 4.0f * m * (l + m) / (l + 2.0f * m + 1e-8f) * ex;
            }
        }
    }
}

void oracle_elastic_step_f64(double* vx, double* vz, double* sxx, double* szz, double* sxz,
                             const double* lam, const double* mu, const double* bx,
                             const double* bz, const double* sponge, int nx, int nz,
                             double dx, double dz, double dt, int free_surface_top)
{
    const double rdx = 1.0 / dx, rdz = 1.0 / dz;
    const int z0 = free_surface_top ? 1 : 2;
    const ptrdiff_t n = nx;
    int iz;
#pragma omp parallel for schedule(static)
    for (iz = z0; iz < nz - 2; ++iz) {
        for (int ix = 2; ix < nx - 2; ++ix) {
            const ptrdiff_t c = (ptrdiff_t)iz * nx + ix;
            const double sxz_m2 = (iz >= 2) ? sxz[c - 2 * n] : 0.0;
            const double a = dfwd_f64(sxx + c, 1) * rdx;
            const double b = dbwd_f64(sxz + c, n, sxz_m2) * rdz;
            vx[c] += dt * bx[c] * (a + b);
            const double e = dbwd_f64(sxz + c, 1, sxz[c - 2]) * rdx;
            const double f = dfwd_f64(szz + c, n) * rdz;
            vz[c] += dt * bz[c] * (e + f);
            if (sponge) {
                vx[c] *= sponge[c];
                vz[c] *= sponge[c];
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (iz = z0; iz < nz - 2; ++iz) {
        for (int ix = 2; ix < nx - 2; ++ix) {
            const ptrdiff_t c = (ptrdiff_t)iz * nx + ix;
            const double vz_m2 = (iz >= 2) ? vz[c - 2 * n] : 0.0;
            const double ex = dbwd_f64(vx + c, 1, vx[c - 2]) * rdx;
            const double ez = dbwd_f64(vz + c, n, vz_m2) * rdz;
            const double l = lam[c], m = mu[c];
            sxx[c] += dt * ((l + 2.0 * m) * ex + l * ez);
            szz[c] += dt * (l * ex + (l + 2.0 * m) * ez);
            const double g = dfwd_f64(vz + c, 1) * rdx;
            const double h = dfwd_f64(vx + c, n) * rdz;
            sxz[c] += dt * m * (g + h);
            if (sponge) {
                sxx[c] *= sponge[c];
                szz[c] *= sponge[c];
                sxz[c] *= sponge[c];
            }
        }
    }
    if (free_surface_top) {
        for (int ix = 0; ix < nx; ++ix) {
            szz[ix] = 0.0;
            sxz[ix] = 0.0;
            if (ix >= 2 && ix < nx - 2) {
                const double l = lam[ix], m = mu[ix];
                const double ex = dbwd_f64(vx + ix, 1, vx[ix - 2]) * rdx;
                sxx[ix] = 4.0 * m * (l + m) / (l + 2.0 * m + 1e-8) * ex;
            }
        }
    }
}

/* ---- zero-lag imaging condition ----------------------------------------- */

void oracle_correlate_f32(const float* src, const float* rec, float* image, int nx, int nz,
                          float dt)
{
    const ptrdiff_t n = (ptrdiff_t)nx * nz;
    ptrdiff_t i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < n; ++i) image[i] += src[i] * rec[i] * dt;
}

void oracle_correlate_f64(const double* src, const double* rec, double* image, int nx, int nz,
                          double dt)
{
    const ptrdiff_t n = (ptrdiff_t)nx * nz;
    ptrdiff_t i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < n; ++i) image[i] += src[i] * rec[i] * dt;
}

/* ---- Cerjan sponge ------------------------------------------------------- */

/* Distance into the absorbing frame: the largest of n-ix, ix-(nx-1-n),
 * iz-(nz-1-n) and, without a free surface, n-iz; clamped at 0. */
static inline float sponge_distance(int ix, int iz, int nx, int nz, int n, int free_surface_top)
{
    float d = 0.0f;
    const float left = (float)(n - ix);
    const float right = (float)(ix - (nx - 1 - n));
    const float bottom = (float)(iz - (nz - 1 - n));
    if (left > d) d = left;
    if (right > d) d = right;
    if (bottom > d) d = bottom;
    if (!free_surface_top) {
        const float top = (float)(n - iz);
        if (top > d) d = top;
    }
    return d;
}

void oracle_cerjan_sponge(float* sponge, int nx, int nz, int n_sponge, float alpha,
                          int free_surface_top)
{
    for (int iz = 0; iz < nz; ++iz) {
        for (int ix = 0; ix < nx; ++ix) {
            const float d = sponge_distance(ix, iz, nx, nz, n_sponge, free_surface_top);
            sponge[(ptrdiff_t)iz * nx + ix] = (d > 0.0f) ? expf(-alpha * d * d) : 1.0f;
        }
    }
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Thread count of later parallel regions of the calling thread (the OpenMP runtime is
 * one per process, so this also sets it for the reference library loaded beside). */
void oracle_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
