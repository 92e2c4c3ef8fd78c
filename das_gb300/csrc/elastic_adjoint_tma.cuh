// elastic_adjoint_tma.cuh -- TMA-tiled forms of the elastic adjoint passes
// (the scheme is in elastic_adjoint_kernels.cuh).
//
// el_adj_a (K2 + K3 of step n) and el_adj_b (K4 of step n with K1 of step n-1) on
// 128 x TZ tiles of shot blockIdx.z.  The fields a pass differentiates arrive as
// 136 x (TZ+4) TMA boxes on one mbarrier (2-row / 4-column halo; outside the grid
// the boxes read zero, the fields' value outside M): pass A takes the three
// t = dt C q planes, the forward velocities of u_{n+1} and the forward stresses of
// u_n (eight boxes); pass B the two r = dt b adj_v planes.  Each lane owns four
// consecutive x points (float4), x neighbours come by warp shuffles, z neighbours
// are read from the box rows; the fields used at one point only (adjoint fields,
// parameters, gradients) are float4 global accesses.  Arithmetic as the reference
// forms (float32, contraction allowed): these passes are checked against finite
// differences, not bit for bit.
#pragma once

#include "elastic_adjoint_kernels.cuh"

namespace w2d {

template <int WARPS, int RPW>
struct ElAdjTile {
    static constexpr int TZ = WARPS * RPW;
    static constexpr int BOX = (TZ + 4) * EL_SW;
    static constexpr int PT = TZ * EL_TX;              // one staged pointwise field
    static constexpr int A_FLOATS = 8 * BOX + 12 * PT;  // pass A
    static constexpr int B_FLOATS = 2 * BOX + 6 * PT;   // pass B
};

// c1*(a[x+1]-a[x]) + c2*(a[x+2]-a[x-1]) of point j from an el_xrow row
__device__ __forceinline__ float adj_dxp(const float e[8], int j)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return k1 * (e[j + 3] - e[j + 2]) + k2 * (e[j + 4] - e[j + 1]);
}
// c1*(a[x]-a[x-1]) + c2*(a[x+1]-a[x-2])
__device__ __forceinline__ float adj_dxm(const float e[8], int j)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return k1 * (e[j + 2] - e[j + 1]) + k2 * (e[j + 3] - e[j]);
}
// along z from four box rows (m2 = z-2, m1 = z-1, c = z, p1 = z+1, p2 = z+2)
__device__ __forceinline__ float adj_dzp(float m1, float c, float p1, float p2)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return k1 * (p1 - c) + k2 * (p2 - m1);
}
__device__ __forceinline__ float adj_dzm(float m2, float m1, float c, float p1)
{
    const float k1 = 9.0f / 8.0f, k2 = -1.0f / 24.0f;
    return k1 * (c - m1) + k2 * (p1 - m2);
}

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, const float v[4])
{
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}

// Receiver residuals pass A adds to the adjoint vz before K2 (the adjoint of the
// vertical-strain sampling, as el_adj_receivers): row n of the residual traces, shot s
// at + s * resid_stride; receivers by column (CSR ptr / list).  resid null: none.
struct ElAdjRecv {
    const float* resid;
    size_t resid_stride;
    const int* ptr;
    const int* list;
    int rec_iz;
};

struct ElAdjMaps {
    CUtensorMap tmp;     // the t / r planes (5 per shot)
    CUtensorMap f_next;  // u_{n+1}
    CUtensorMap f_curr;  // u_n
};

// K2 + K3 of step n
template <int WARPS, int RPW>
__global__ void __launch_bounds__(WARPS * 32)
    el_adj_a(const __grid_constant__ ElAdjMaps maps, const ElGeom g, const ElParams p,
             const ElStrides sd, ElState a, ElState r, float* g_lam, float* g_mu, float* g_bx,
             float* g_bz, const ElAdjRecv rv, unsigned* err)
{
    using T = ElAdjTile<WARPS, RPW>;
    extern __shared__ __align__(128) float smem[];
    float* b_txx = smem;
    float* b_txz = smem + T::BOX;
    float* b_tzz = smem + 2 * T::BOX;
    float* b_nvx = smem + 3 * T::BOX;
    float* b_nvz = smem + 4 * T::BOX;
    float* b_cxx = smem + 5 * T::BOX;
    float* b_cxz = smem + 6 * T::BOX;
    float* b_czz = smem + 7 * T::BOX;
    // staged: adj vx, vz, sxx, szz, sxz, g_lambda, g_mu, sponge, bx, bz, g_bx, g_bz
    float* pt = smem + 8 * T::BOX;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::A_FLOATS);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int x0 = blockIdx.x * EL_TX, z0 = blockIdx.y * T::TZ, sh = blockIdx.z;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    // set-up overlaps the previous kernel when launched as a programmatic dependent;
    // every thread waits before any global access
    grid_dep_launch();
    grid_dep_wait();
    if (tid == 0) {
        mbar_expect_tx(bar, 8u * T::BOX * 4u);
        const int xs = x0 - EL_HX, zs = z0 - 2, pb = 5 * sh;
        tma_load_3d(b_txx, &maps.tmp, xs, zs, pb + EL_SXX, bar);
        tma_load_3d(b_txz, &maps.tmp, xs, zs, pb + EL_SXZ, bar);
        tma_load_3d(b_tzz, &maps.tmp, xs, zs, pb + EL_SZZ, bar);
        tma_load_3d(b_nvx, &maps.f_next, xs, zs, pb + EL_VX, bar);
        tma_load_3d(b_nvz, &maps.f_next, xs, zs, pb + EL_VZ, bar);
        tma_load_3d(b_cxx, &maps.f_curr, xs, zs, pb + EL_SXX, bar);
        tma_load_3d(b_cxz, &maps.f_curr, xs, zs, pb + EL_SXZ, bar);
        tma_load_3d(b_czz, &maps.f_curr, xs, zs, pb + EL_SZZ, bar);
    }
    const int ixb = x0 + 4 * lane;
    const bool col_ok = ixb < g.ldx;
    const size_t so = (size_t)sh * sd.state, po = (size_t)sh * sd.param, go = (size_t)sh * sd.grad;
    a = el_shift(a, so);
    r = el_shift(r, so);
    g_lam += go;
    g_mu += go;
    g_bx += go;
    g_bz += go;
    const float* bxp = p.bx + po;
    const float* bzp = p.bz + po;
    const int zr0 = z0 + warp * RPW;
    const int sr0 = zr0 - (z0 - 2);
    {
        const float* f[12] = {a.vx, a.vz, a.sxx, a.szz, a.sxz, g_lam, g_mu,
                              p.sponge, bxp, bzp, g_bx, g_bz};
        el_stage_pointwise<WARPS, RPW>(pt, f, 12, zr0, ixb, lane, warp, g);
    }
    __syncthreads();
    if (__syncthreads_or(!mbar_wait_bounded(bar, 0))) {
        cp_async_wait_all();
        if (tid == 0) atomicOr(err, ERR_TMA_TIMEOUT);
        return;
    }
    cp_async_wait_all();  // this thread's staged fields (read and updated only by it)
    auto staged = [&](int f, int rr) { return el_staged<WARPS, RPW>(pt, f, warp, rr, lane); };
    if (rv.resid && col_ok && zr0 + RPW > rv.rec_iz - 2 && zr0 <= rv.rec_iz + 1) {
        // the receivers' residuals on the four rows of their strain stencil (each cell's
        // contributions in receiver order), added to this thread's staged adjoint vz
        // before the rows below read it
        const float c1 = 9.0f / 8.0f, c2 = -1.0f / 24.0f;
        const float* res = rv.resid + (size_t)sh * rv.resid_stride;
        for (int rr = 0; rr < RPW; ++rr) {
            const int iz = zr0 + rr, dzr = iz - rv.rec_iz;
            if (dzr < -2 || dzr > 1 || iz >= g.nz) continue;
            const float cf = dzr == 0 ? c1 : (dzr == -1 ? -c1 : (dzr == 1 ? c2 : -c2));
            for (int j = 0; j < 4; ++j) {
                const int ix = ixb + j;
                if (!el_in_m(ix, iz, g.nx, g.nz, g.free_surface)) continue;
                const int k0 = __ldg(rv.ptr + ix), k1 = __ldg(rv.ptr + ix + 1);
                if (k0 == k1) continue;
                float* cell = &pt[(1 * T::TZ + warp * RPW + rr) * EL_TX + 4 * lane + j];
                float v = *cell;
                for (int k = k0; k < k1; ++k)
                    v = fadd(v, fmul(cf, fmul(__ldg(res + __ldg(rv.list + k)), g.rdz)));
                *cell = v;
            }
        }
    }
    // Two phases per row (K2, then K3) so that only one phase's operands are live.
#pragma unroll 1
    for (int rr = 0; rr < RPW; ++rr) {
        const int iz = zr0 + rr, sr = sr0 + rr;
        const bool live = iz < g.nz && col_ok;
        const size_t off = (size_t)iz * g.ldx + ixb;
        bool in_m[4], all = true;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            in_m[j] = el_in_m(ixb + j, iz, g.nx, g.nz, g.free_surface);
            all &= in_m[j];
        }
        float avx[4], avz[4];
        {
            // K2: adjoint velocities and the lambda / mu gradients (forward strains of u_{n+1})
            float etxx[8], etxz[8], envx[8], envz[8];
            el_xrow(b_txx, sr, lane, etxx);
            el_xrow(b_txz, sr, lane, etxz);
            el_xrow(b_nvx, sr, lane, envx);
            el_xrow(b_nvz, sr, lane, envz);
            if (live) {
                const float4 txz_m2 = el_row4(b_txz, sr - 2, lane),
                             txz_m1 = el_row4(b_txz, sr - 1, lane),
                             txz_p1 = el_row4(b_txz, sr + 1, lane);
                const float4 tzz_m1 = el_row4(b_tzz, sr - 1, lane), tzz_c = el_row4(b_tzz, sr, lane),
                             tzz_p1 = el_row4(b_tzz, sr + 1, lane),
                             tzz_p2 = el_row4(b_tzz, sr + 2, lane);
                const float4 nvx_m1 = el_row4(b_nvx, sr - 1, lane),
                             nvx_p1 = el_row4(b_nvx, sr + 1, lane),
                             nvx_p2 = el_row4(b_nvx, sr + 2, lane);
                const float4 nvz_m2 = el_row4(b_nvz, sr - 2, lane),
                             nvz_m1 = el_row4(b_nvz, sr - 1, lane),
                             nvz_p1 = el_row4(b_nvz, sr + 1, lane);
                const float4 avx4 = staged(0, rr), avz4 = staged(1, rr);
                const float4 qxx4 = staged(2, rr), qzz4 = staged(3, rr), qxz4 = staged(4, rr);
                const float4 gl4 = staged(5, rr), gm4 = staged(6, rr);
                float o_gl[4], o_gm[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    float vx = el_c(avx4, j), vz = el_c(avz4, j);
                    vx -= adj_dxp(etxx, j) * g.rdx +
                          adj_dzm(el_c(txz_m2, j), el_c(txz_m1, j), etxz[j + 2], el_c(txz_p1, j)) *
                              g.rdz;
                    vz -= adj_dzp(el_c(tzz_m1, j), el_c(tzz_c, j), el_c(tzz_p1, j),
                                  el_c(tzz_p2, j)) * g.rdz +
                          adj_dxm(etxz, j) * g.rdx;
                    avx[j] = vx;
                    avz[j] = vz;
                    const float exx = adj_dxm(envx, j) * g.rdx;
                    const float ezz =
                        adj_dzm(el_c(nvz_m2, j), el_c(nvz_m1, j), envz[j + 2], el_c(nvz_p1, j)) *
                        g.rdz;
                    const float exz = adj_dxp(envz, j) * g.rdx +
                                      adj_dzp(el_c(nvx_m1, j), envx[j + 2], el_c(nvx_p1, j),
                                              el_c(nvx_p2, j)) * g.rdz;
                    const float qxx = el_c(qxx4, j), qzz = el_c(qzz4, j), qxz = el_c(qxz4, j);
                    o_gl[j] = el_c(gl4, j) + g.dt * (exx + ezz) * (qxx + qzz);
                    o_gm[j] = el_c(gm4, j) + g.dt * (2.0f * exx * qxx + 2.0f * ezz * qzz + exz * qxz);
                }
                if (all) {
                    st4(g_lam + off, o_gl);
                    st4(g_mu + off, o_gm);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (in_m[j]) {
                            g_lam[off + j] = o_gl[j];
                            g_mu[off + j] = o_gm[j];
                        }
                }
            }
        }
        {
            // K3: buoyancy gradients (forward stresses of u_n), sponge, r = dt b adj_v
            float ecxx[8], ecxz[8];
            el_xrow(b_cxx, sr, lane, ecxx);
            el_xrow(b_cxz, sr, lane, ecxz);
            if (live) {
                const float4 cxz_m2 = el_row4(b_cxz, sr - 2, lane),
                             cxz_m1 = el_row4(b_cxz, sr - 1, lane),
                             cxz_p1 = el_row4(b_cxz, sr + 1, lane);
                const float4 czz_m1 = el_row4(b_czz, sr - 1, lane), czz_c = el_row4(b_czz, sr, lane),
                             czz_p1 = el_row4(b_czz, sr + 1, lane),
                             czz_p2 = el_row4(b_czz, sr + 2, lane);
                const float4 sp4 = p.sponge ? staged(7, rr) : make_float4(1.f, 1.f, 1.f, 1.f);
                const float4 bx4 = staged(8, rr), bz4 = staged(9, rr);
                const float4 gbx4 = staged(10, rr), gbz4 = staged(11, rr);
                float o_gbx[4], o_gbz[4], o_rx[4], o_rz[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float gx = adj_dxp(ecxx, j) * g.rdx +
                                     adj_dzm(el_c(cxz_m2, j), el_c(cxz_m1, j), ecxz[j + 2],
                                             el_c(cxz_p1, j)) * g.rdz;
                    const float gz = adj_dxm(ecxz, j) * g.rdx +
                                     adj_dzp(el_c(czz_m1, j), el_c(czz_c, j), el_c(czz_p1, j),
                                             el_c(czz_p2, j)) * g.rdz;
                    const float sp = el_c(sp4, j);
                    o_gbx[j] = el_c(gbx4, j) + sp * g.dt * avx[j] * gx;
                    o_gbz[j] = el_c(gbz4, j) + sp * g.dt * avz[j] * gz;
                    avx[j] = sp * avx[j];
                    avz[j] = sp * avz[j];
                    o_rx[j] = g.dt * el_c(bx4, j) * avx[j];
                    o_rz[j] = g.dt * el_c(bz4, j) * avz[j];
                }
                if (all) {
                    st4(a.vx + off, avx);
                    st4(a.vz + off, avz);
                    st4(r.vx + off, o_rx);
                    st4(r.vz + off, o_rz);
                    st4(g_bx + off, o_gbx);
                    st4(g_bz + off, o_gbz);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        if (!in_m[j]) continue;
                        const size_t c = off + j;
                        a.vx[c] = avx[j];
                        a.vz[c] = avz[j];
                        r.vx[c] = o_rx[j];
                        r.vz[c] = o_rz[j];
                        g_bx[c] = o_gbx[j];
                        g_bz[c] = o_gbz[j];
                    }
                }
            }
        }
    }
}

// K4 of step n, then (then_k1) K1 of step n-1
template <int WARPS, int RPW>
__global__ void __launch_bounds__(WARPS * 32)
    el_adj_b(const __grid_constant__ ElAdjMaps maps, const ElGeom g, const ElParams p,
             const ElStrides sd, ElState a, ElState t, int then_k1, unsigned* err)
{
    using T = ElAdjTile<WARPS, RPW>;
    extern __shared__ __align__(128) float smem[];
    float* b_rx = smem;
    float* b_rz = smem + T::BOX;
    float* pt = smem + 2 * T::BOX;  // staged adj sxx, szz, sxz, sponge, lambda, mu
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::B_FLOATS);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int x0 = blockIdx.x * EL_TX, z0 = blockIdx.y * T::TZ, sh = blockIdx.z;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    grid_dep_launch();
    grid_dep_wait();  // as in pass A
    if (tid == 0) {
        mbar_expect_tx(bar, 2u * T::BOX * 4u);
        tma_load_3d(b_rx, &maps.tmp, x0 - EL_HX, z0 - 2, 5 * sh + EL_VX, bar);
        tma_load_3d(b_rz, &maps.tmp, x0 - EL_HX, z0 - 2, 5 * sh + EL_VZ, bar);
    }
    const int ixb = x0 + 4 * lane;
    const bool col_ok = ixb < g.ldx;
    const size_t so = (size_t)sh * sd.state, po = (size_t)sh * sd.param;
    a = el_shift(a, so);
    t = el_shift(t, so);
    const float* lamp = p.lam + po;
    const float* mup = p.mu + po;
    const int zr0 = z0 + warp * RPW;
    const int sr0 = zr0 - (z0 - 2);
    {
        const float* f[6] = {a.sxx, a.szz, a.sxz, then_k1 ? p.sponge : nullptr,
                             then_k1 ? lamp : nullptr, then_k1 ? mup : nullptr};
        el_stage_pointwise<WARPS, RPW>(pt, f, 6, zr0, ixb, lane, warp, g);
    }
    __syncthreads();
    if (__syncthreads_or(!mbar_wait_bounded(bar, 0))) {
        cp_async_wait_all();
        if (tid == 0) atomicOr(err, ERR_TMA_TIMEOUT);
        return;
    }
    cp_async_wait_all();  // this thread's staged fields (read only by it)
#pragma unroll
    for (int rr = 0; rr < RPW; ++rr) {
        const int iz = zr0 + rr, sr = sr0 + rr;
        float erx[8], erz[8];
        el_xrow(b_rx, sr, lane, erx);
        el_xrow(b_rz, sr, lane, erz);
        if (iz >= g.nz || !col_ok) continue;
        const float4 rx_m1 = el_row4(b_rx, sr - 1, lane), rx_p1 = el_row4(b_rx, sr + 1, lane),
                     rx_p2 = el_row4(b_rx, sr + 2, lane);
        const float4 rz_m2 = el_row4(b_rz, sr - 2, lane), rz_m1 = el_row4(b_rz, sr - 1, lane),
                     rz_p1 = el_row4(b_rz, sr + 1, lane);
        const size_t off = (size_t)iz * g.ldx + ixb;
        const float4 sxx4 = el_staged<WARPS, RPW>(pt, 0, warp, rr, lane),
                     szz4 = el_staged<WARPS, RPW>(pt, 1, warp, rr, lane),
                     sxz4 = el_staged<WARPS, RPW>(pt, 2, warp, rr, lane);
        float4 sp4 = make_float4(1.f, 1.f, 1.f, 1.f), l4 = sp4, m4 = sp4;
        if (then_k1) {
            if (p.sponge) sp4 = el_staged<WARPS, RPW>(pt, 3, warp, rr, lane);
            l4 = el_staged<WARPS, RPW>(pt, 4, warp, rr, lane);
            m4 = el_staged<WARPS, RPW>(pt, 5, warp, rr, lane);
        }
        float oxx[4], ozz[4], oxz[4], txx[4], tzz[4], txz[4];
        bool all = true;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            all &= el_in_m(ixb + j, iz, g.nx, g.nz, g.free_surface);
            float sxx = el_c(sxx4, j), szz = el_c(szz4, j), sxz = el_c(sxz4, j);
            sxx -= adj_dxm(erx, j) * g.rdx;
            szz -= adj_dzm(el_c(rz_m2, j), el_c(rz_m1, j), erz[j + 2], el_c(rz_p1, j)) * g.rdz;
            sxz -= adj_dzp(el_c(rx_m1, j), erx[j + 2], el_c(rx_p1, j), el_c(rx_p2, j)) * g.rdz +
                   adj_dxp(erz, j) * g.rdx;
            txx[j] = tzz[j] = txz[j] = 0.0f;
            if (then_k1) {
                const float sp = el_c(sp4, j);
                sxx = sp * sxx;
                szz = sp * szz;
                sxz = sp * sxz;
                const float l = el_c(l4, j), m = el_c(m4, j);
                txx[j] = g.dt * ((l + 2.0f * m) * sxx + l * szz);
                tzz[j] = g.dt * (l * sxx + (l + 2.0f * m) * szz);
                txz[j] = g.dt * m * sxz;
            }
            oxx[j] = sxx;
            ozz[j] = szz;
            oxz[j] = sxz;
        }
        if (all) {
            st4(a.sxx + off, oxx);
            st4(a.szz + off, ozz);
            st4(a.sxz + off, oxz);
            if (then_k1) {
                st4(t.sxx + off, txx);
                st4(t.szz + off, tzz);
                st4(t.sxz + off, txz);
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (!el_in_m(ixb + j, iz, g.nx, g.nz, g.free_surface)) continue;
                const size_t c = off + j;
                a.sxx[c] = oxx[j];
                a.szz[c] = ozz[j];
                a.sxz[c] = oxz[j];
                if (then_k1) {
                    t.sxx[c] = txx[j];
                    t.szz[c] = tzz[j];
                    t.sxz[c] = txz[j];
                }
            }
        }
    }
}

constexpr int EL_ADJ_WARPS = 4, EL_ADJ_RPW = 1;  // default tile: 128 x 4

inline bool el_adj_tile_supported(int warps, int rpw)
{
    return (warps == 4 && (rpw == 2 || rpw == 1)) || (warps == 8 && rpw == 1);
}

template <int WARPS, int RPW>
cudaError_t launch_el_adj_a_t(const ElAdjMaps& m, const ElGeom& g, const ElParams& p,
                              const ElStrides& sd, const ElState& a, const ElState& r, float* glam,
                              float* gmu, float* gbx, float* gbz, const ElAdjRecv& rv,
                              unsigned* err, int n_shots, cudaStream_t st, int pdl)
{
    using T = ElAdjTile<WARPS, RPW>;
    const int bytes = T::A_FLOATS * 4 + 128;
    const cudaError_t e = set_smem_once<el_adj_a<WARPS, RPW>>(bytes);
    if (e != cudaSuccess) return e;
    dim3 grid((g.nx + EL_TX - 1) / EL_TX, (g.nz + T::TZ - 1) / T::TZ, n_shots);
    return el_launch(el_adj_a<WARPS, RPW>, grid, dim3(WARPS * 32), bytes, st, pdl, m, g, p, sd, a,
                     r, glam, gmu, gbx, gbz, rv, err);
}

template <int WARPS, int RPW>
cudaError_t launch_el_adj_b_t(const ElAdjMaps& m, const ElGeom& g, const ElParams& p,
                              const ElStrides& sd, const ElState& a, const ElState& t,
                              int then_k1, unsigned* err, int n_shots, cudaStream_t st, int pdl)
{
    using T = ElAdjTile<WARPS, RPW>;
    const int bytes = T::B_FLOATS * 4 + 128;
    const cudaError_t e = set_smem_once<el_adj_b<WARPS, RPW>>(bytes);
    if (e != cudaSuccess) return e;
    dim3 grid((g.nx + EL_TX - 1) / EL_TX, (g.nz + T::TZ - 1) / T::TZ, n_shots);
    return el_launch(el_adj_b<WARPS, RPW>, grid, dim3(WARPS * 32), bytes, st, pdl, m, g, p, sd, a,
                     t, then_k1, err);
}

// Pass A / pass B on tiles of `warps` x `rpw` rows (maps with box height warps*rpw + 4).
inline cudaError_t launch_el_adj_a(const ElAdjMaps& m, const ElGeom& g, const ElParams& p,
                                   const ElStrides& sd, const ElState& a, const ElState& r,
                                   float* glam, float* gmu, float* gbx, float* gbz,
                                   const ElAdjRecv& rv, unsigned* err, int n_shots,
                                   cudaStream_t st, int warps = EL_ADJ_WARPS,
                                   int rpw = EL_ADJ_RPW, int pdl = 0)
{
    if (warps == 4 && rpw == 2)
        return launch_el_adj_a_t<4, 2>(m, g, p, sd, a, r, glam, gmu, gbx, gbz, rv, err, n_shots,
                                       st, pdl);
    if (warps == 4 && rpw == 1)
        return launch_el_adj_a_t<4, 1>(m, g, p, sd, a, r, glam, gmu, gbx, gbz, rv, err, n_shots,
                                       st, pdl);
    if (warps == 8 && rpw == 1)
        return launch_el_adj_a_t<8, 1>(m, g, p, sd, a, r, glam, gmu, gbx, gbz, rv, err, n_shots,
                                       st, pdl);
    return cudaErrorInvalidValue;
}

inline cudaError_t launch_el_adj_b(const ElAdjMaps& m, const ElGeom& g, const ElParams& p,
                                   const ElStrides& sd, const ElState& a, const ElState& t,
                                   int then_k1, unsigned* err, int n_shots, cudaStream_t st,
                                   int warps = EL_ADJ_WARPS, int rpw = EL_ADJ_RPW, int pdl = 0)
{
    if (warps == 4 && rpw == 2)
        return launch_el_adj_b_t<4, 2>(m, g, p, sd, a, t, then_k1, err, n_shots, st, pdl);
    if (warps == 4 && rpw == 1)
        return launch_el_adj_b_t<4, 1>(m, g, p, sd, a, t, then_k1, err, n_shots, st, pdl);
    if (warps == 8 && rpw == 1)
        return launch_el_adj_b_t<8, 1>(m, g, p, sd, a, t, then_k1, err, n_shots, st, pdl);
    return cudaErrorInvalidValue;
}

// 3D map over the states (5 planes per shot) of a buffer, with boxes of tile height tz.
inline int make_el_adj_map(CUtensorMap* m, const float* base, int nx, int nz, int ldx,
                           size_t plane, int n_shots, int tz = EL_ADJ_WARPS * EL_ADJ_RPW)
{
    return make_tensor_map_3d(m, base, nx, nz, 5 * n_shots, ldx, plane, EL_SW, tz + 4);
}

}  // namespace w2d
