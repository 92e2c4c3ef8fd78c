// elastic_adjoint_kernels.cuh -- elastic modelling pieces and the exact discrete
// adjoint of the velocity-stress step (parameter gradients for elastic RTM).
//
// Modelling (no counterpart in the reference, which only exports the step):
//   * state u_n = (vx, vz, sxx, szz, sxz); the step is elastic_kernels.cuh
//     (wave2d.c:95-212), updated cells M = rows [1 if free surface else 2, nz-2),
//     columns [2, nx-2); every other cell stays zero (zero start, sources and
//     receivers on M), so the free-surface rule reduces to zero stresses on row 0;
//   * vertical force source: vz[src] += w[n] * dt before step n;
//   * vertical-strain receivers: d_n = Dz- vz of u_{n+1} at (rec_iz, rec_ix),
//     the same 4th-order staggered difference the stress update uses.
//
// Adjoint of one step u' = S(V(u)) (V: v' = s(v + dt b G sigma); S: sigma' =
// s(sigma + dt C E v')), with the staggered operators' transposes
// D-^T = -D+ and D+^T = -D- on fields that vanish outside M:
//   K1  q = s * adj_sigma'                 (adjoint stress after S^T)
//       t = dt * C q                       (per cell, C = [[l+2m, l, 0],[l, l+2m, 0],[0,0,m]])
//   K2  adj_v += E^T t = -(Dx+ txx + Dz- txz,  Dz+ tzz + Dx- txz)
//       g_lambda += dt (exx + ezz)(qxx + qzz),  g_mu += dt (2 exx qxx + 2 ezz qzz + exz qxz),
//       with the forward strains e = E v_{n+1}
//   K3  g_bx += s dt adj_vx (Dx+ sxx_n + Dz- sxz_n), g_bz likewise (forward stresses of u_n);
//       adj_v = s adj_v;  r = dt b adj_v
//   K4  adj_sigma = q + G^T r = q - (Dx- rx,  Dz- rz,  Dz+ rx + Dx+ rz)
// K2 and K3 run as one kernel (el_adj_k23), and K1 of step n-1 runs inside K4 of
// step n (el_adj_k4), so one adjoint step is three passes.
// Receiver residuals enter as adj_vz += Dz-^T (residual) on the four cells of
// the receiver's stencil.  Float32; not bit-for-bit with anything, checked
// against finite differences.
#pragma once

#include "elastic_kernels.cuh"

namespace w2d {

struct ElState {
    float *vx, *vz, *sxx, *szz, *sxz;
};

__device__ __forceinline__ ElState el_shift(ElState s, size_t o)
{
    return ElState{s.vx + o, s.vz + o, s.sxx + o, s.szz + o, s.sxz + o};
}

// Per-shot strides (floats) of a batch: shot s of a state at + s * state, of the
// parameters at + s * param, of the four gradient planes at + s * grad.
struct ElStrides {
    size_t state, param, grad;
};

struct ElParams {
    const float *lam, *mu, *bx, *bz;
    const float* sponge;  // pitched, or null
};

// reads a[iz*L+ix] with zero outside the grid (rows/cols outside M hold zero)
__device__ __forceinline__ float el_at(const float* a, int ix, int iz, int nx, int nz, int L)
{
    return (ix >= 0 && ix < nx && iz >= 0 && iz < nz) ? a[(size_t)iz * L + ix] : 0.0f;
}

// c1*(a[+1]-a[0]) + c2*(a[+2]-a[-1]) along x or z
__device__ __forceinline__ float d_fwd_x(const float* a, int ix, int iz, int nx, int nz, int L)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return k1 * (el_at(a, ix + 1, iz, nx, nz, L) - el_at(a, ix, iz, nx, nz, L)) +
           k2 * (el_at(a, ix + 2, iz, nx, nz, L) - el_at(a, ix - 1, iz, nx, nz, L));
}
__device__ __forceinline__ float d_bwd_x(const float* a, int ix, int iz, int nx, int nz, int L)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return k1 * (el_at(a, ix, iz, nx, nz, L) - el_at(a, ix - 1, iz, nx, nz, L)) +
           k2 * (el_at(a, ix + 1, iz, nx, nz, L) - el_at(a, ix - 2, iz, nx, nz, L));
}
__device__ __forceinline__ float d_fwd_z(const float* a, int ix, int iz, int nx, int nz, int L)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return k1 * (el_at(a, ix, iz + 1, nx, nz, L) - el_at(a, ix, iz, nx, nz, L)) +
           k2 * (el_at(a, ix, iz + 2, nx, nz, L) - el_at(a, ix, iz - 1, nx, nz, L));
}
__device__ __forceinline__ float d_bwd_z(const float* a, int ix, int iz, int nx, int nz, int L)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return k1 * (el_at(a, ix, iz, nx, nz, L) - el_at(a, ix, iz - 1, nx, nz, L)) +
           k2 * (el_at(a, ix, iz + 1, nx, nz, L) - el_at(a, ix, iz - 2, nx, nz, L));
}

// one cell of M of shot blockIdx.z; c indexes the cell within a plane of that shot
#define EL_CELL                                                  \
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;        \
    const int iz = blockIdx.y * blockDim.y + threadIdx.y;        \
    if (!el_in_m(ix, iz, g.nx, g.nz, g.free_surface)) return;    \
    const int L = g.ldx;                                         \
    const size_t c = (size_t)iz * L + ix;                        \
    const size_t po_ = blockIdx.z * sd.param;                    \
    const float sp = p.sponge ? p.sponge[c] : 1.0f;              \
    const float* lam_ = p.lam + po_;                             \
    const float* mu_ = p.mu + po_;                               \
    const float* bx_ = p.bx + po_;                               \
    const float* bz_ = p.bz + po_;                               \
    (void)lam_; (void)mu_; (void)bx_; (void)bz_;

// K1
static __global__ void el_adj_k1(ElGeom g, ElParams p, ElStrides sd, ElState a, ElState t)
{
    EL_CELL
    a = el_shift(a, blockIdx.z * sd.state);
    t = el_shift(t, blockIdx.z * sd.state);
    const float qxx = sp * a.sxx[c], qzz = sp * a.szz[c], qxz = sp * a.sxz[c];
    a.sxx[c] = qxx;
    a.szz[c] = qzz;
    a.sxz[c] = qxz;
    const float l = lam_[c], m = mu_[c];
    t.sxx[c] = g.dt * ((l + 2.0f * m) * qxx + l * qzz);
    t.szz[c] = g.dt * (l * qxx + (l + 2.0f * m) * qzz);
    t.sxz[c] = g.dt * m * qxz;
}

// K2 and K3 of one step in one pass: K3 touches the adjoint velocities only at
// their own cell, right after K2 has produced them.
static __global__ void el_adj_k23(ElGeom g, ElParams p, ElStrides sd, ElState a, ElState t,
                                  ElState r, ElState f_next, ElState f_curr, float* g_lam,
                                  float* g_mu, float* g_bx, float* g_bz)
{
    EL_CELL
    const int nx = g.nx, nz = g.nz;
    const size_t so = blockIdx.z * sd.state, go = blockIdx.z * sd.grad;
    a = el_shift(a, so);
    t = el_shift(t, so);
    r = el_shift(r, so);
    f_next = el_shift(f_next, so);
    f_curr = el_shift(f_curr, so);
    g_lam += go;
    g_mu += go;
    g_bx += go;
    g_bz += go;
    // K2
    float avx = a.vx[c], avz = a.vz[c];
    avx -= d_fwd_x(t.sxx, ix, iz, nx, nz, L) * g.rdx + d_bwd_z(t.sxz, ix, iz, nx, nz, L) * g.rdz;
    avz -= d_fwd_z(t.szz, ix, iz, nx, nz, L) * g.rdz + d_bwd_x(t.sxz, ix, iz, nx, nz, L) * g.rdx;
    const float exx = d_bwd_x(f_next.vx, ix, iz, nx, nz, L) * g.rdx;
    const float ezz = d_bwd_z(f_next.vz, ix, iz, nx, nz, L) * g.rdz;
    const float exz = d_fwd_x(f_next.vz, ix, iz, nx, nz, L) * g.rdx +
                      d_fwd_z(f_next.vx, ix, iz, nx, nz, L) * g.rdz;
    const float qxx = a.sxx[c], qzz = a.szz[c], qxz = a.sxz[c];
    g_lam[c] += g.dt * (exx + ezz) * (qxx + qzz);
    g_mu[c] += g.dt * (2.0f * exx * qxx + 2.0f * ezz * qzz + exz * qxz);
    // K3
    const float gx = d_fwd_x(f_curr.sxx, ix, iz, nx, nz, L) * g.rdx +
                     d_bwd_z(f_curr.sxz, ix, iz, nx, nz, L) * g.rdz;
    const float gz = d_bwd_x(f_curr.sxz, ix, iz, nx, nz, L) * g.rdx +
                     d_fwd_z(f_curr.szz, ix, iz, nx, nz, L) * g.rdz;
    g_bx[c] += sp * g.dt * avx * gx;
    g_bz[c] += sp * g.dt * avz * gz;
    const float vx = sp * avx, vz = sp * avz;
    a.vx[c] = vx;
    a.vz[c] = vz;
    r.vx[c] = g.dt * bx_[c] * vx;
    r.vz[c] = g.dt * bz_[c] * vz;
}

// K4 of step n, followed (then_k1) by K1 of step n-1 on the same cell: K1 reads
// only this cell's adjoint stresses, which K4 has just produced, so the two fuse
// into one pass (the receiver residual added between them touches vz only).
static __global__ void el_adj_k4(ElGeom g, ElParams p, ElStrides sd, ElState a, ElState r,
                                 ElState t, int then_k1)
{
    EL_CELL
    const int nx = g.nx, nz = g.nz;
    const size_t so = blockIdx.z * sd.state;
    a = el_shift(a, so);
    r = el_shift(r, so);
    t = el_shift(t, so);
    float sxx = a.sxx[c], szz = a.szz[c], sxz = a.sxz[c];
    sxx -= d_bwd_x(r.vx, ix, iz, nx, nz, L) * g.rdx;
    szz -= d_bwd_z(r.vz, ix, iz, nx, nz, L) * g.rdz;
    sxz -= d_fwd_z(r.vx, ix, iz, nx, nz, L) * g.rdz + d_fwd_x(r.vz, ix, iz, nx, nz, L) * g.rdx;
    if (then_k1) {
        const float qxx = sp * sxx, qzz = sp * szz, qxz = sp * sxz;
        sxx = qxx;
        szz = qzz;
        sxz = qxz;
        const float l = lam_[c], m = mu_[c];
        t.sxx[c] = g.dt * ((l + 2.0f * m) * qxx + l * qzz);
        t.szz[c] = g.dt * (l * qxx + (l + 2.0f * m) * qzz);
        t.sxz[c] = g.dt * m * qxz;
    }
    a.sxx[c] = sxx;
    a.szz[c] = szz;
    a.sxz[c] = sxz;
}

// Adjoint of the sampling: adj_vz += Dz-^T (residual) at each receiver, i.e. on
// rows rec_iz (+c1), rec_iz-1 (-c1), rec_iz+1 (+c2), rec_iz-2 (-c2), cells of M only.
// One thread per column; receivers sharing a column (CSR rec_ptr / rec_list, in
// index order) add into its cells one after another, so every cell receives its
// contributions in receiver order.
static __global__ void el_adj_receivers(ElGeom g, float* adj_vz, size_t state_stride,
                                        const int* rec_ptr, const int* rec_list, int rec_iz,
                                        const float* resid, size_t resid_stride)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    if (ix >= g.nx) return;
    adj_vz += blockIdx.y * state_stride;  // shot blockIdx.y
    resid += blockIdx.y * resid_stride;
    const int k0 = rec_ptr[ix], k1 = rec_ptr[ix + 1];
    if (k0 == k1) return;
    const float c1 = 9.0f / 8.0f, c2 = -1.0f / 24.0f;
    const int dz[4] = {0, -1, 1, -2};
    const float cf[4] = {c1, -c1, c2, -c2};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int iz = rec_iz + dz[j];
        if (!el_in_m(ix, iz, g.nx, g.nz, g.free_surface)) continue;
        float* cell = adj_vz + (size_t)iz * g.ldx + ix;
        float v = *cell;
        for (int k = k0; k < k1; ++k)
            v = fadd(v, fmul(cf[j], fmul(__ldg(resid + __ldg(rec_list + k)), g.rdz)));
        *cell = v;
    }
}

}  // namespace w2d
