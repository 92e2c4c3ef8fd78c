// acoustic_step2.cuh -- two time steps of the reference scheme per launch.
//
// One CTA advances a 128 x TZ tile by steps n and n+1 (tsw_rtm/c_engine/wave2d.c:19-82
// twice, with everything the Python loops do between the two calls): the first step
// is evaluated on the tile plus a 2-row / 2-column ring (the second step's stencil
// reach), kept in shared memory, then the second step on the tile.  p_curr arrives as
// one 136 x (TZ+8) TMA box (4-row / 4-column halo), p_prev, vel^2 dt^2 (and a per-cell
// sponge) as 136 x (TZ+4) boxes; each wavefield crosses HBM / L2 once per two steps.
//
// Reference semantics kept bit for bit (same float32 operations as the one-step
// kernel, acoustic_kernels.cuh):
//   * cells the reference never writes keep the value of the buffer the reference
//     would write into: for step n that is the stale p_next buffer (a fifth TMA box,
//     boundary tiles only), for step n+1 it is p_prev (already in a box);
//   * free surface (p_next[0,:] = 0, p_next[1,:] = -p_next[2,:] over every column),
//     then receiver sampling of p_next, then the next step's injections (receiver data
//     in receiver order, source), per column by one thread;
//   * snapshot / illumination / imaging of both steps' p_curr.
// The two results go to two buffers other than the three read (a neighbouring CTA may
// still be reading its halo from them); the engine renames buffers so that the three
// logical roles continue the reference's rotation.
#pragma once

#include "acoustic_kernels.cuh"

namespace w2d {

constexpr int AC2_W = AC_SW;  // 136 columns: x0-4 .. x0+131

template <int R2, int SPONGE>
struct Ac2Tile {
    static constexpr int TZ = 4 * R2;  // output rows, R2 per warp
    static constexpr int R1 = R2 + 1;  // first-step rows per warp (TZ + 4 over 4 warps)
    static constexpr int ER = TZ + 4;  // first-step rows: z0-2 .. z0+TZ+1
    static constexpr int BR = TZ + 8;  // p_curr rows: z0-4 .. z0+TZ+3
    static constexpr int B_FLOATS = BR * AC2_W;
    static constexpr int E_FLOATS = ER * AC2_W;
    static constexpr int N_BOXES = SPONGE == SPONGE_ARRAY ? 3 : 2;  // p_prev, vel (, sponge)
    // the second step's result of a boundary tile reuses the p_curr box's centre rows
    static constexpr int FLOATS = B_FLOATS + N_BOXES * E_FLOATS + E_FLOATS;
    static constexpr unsigned TX_BYTES = (B_FLOATS + N_BOXES * E_FLOATS) * 4u;
    static constexpr size_t SMEM_BYTES = FLOATS * 4u + 128;
};

struct Ac2Maps {
    CUtensorMap curr;    // box AC2_W x (TZ+8)
    CUtensorMap prev;    // box AC2_W x (TZ+4)
    CUtensorMap vel;     // box AC2_W x (TZ+4)
    CUtensorMap sponge;  // box AC2_W x (TZ+4) (SPONGE_ARRAY only)
    CUtensorMap stale;   // box AC2_W x (TZ+4): step n's p_next buffer (boundary tiles)
};

// s[0]: step n (p_curr = the curr buffer), s[1]: step n+1 (p_curr = the first result);
// their p_next fields are unused.
struct Ac2Step {
    AcStep s[2];
    float* out1;  // p_{n+1} (with step n+1's injections)
    float* out2;  // p_{n+2} (with step n+2's injections)
    int src_ix, src_iz, rec_iz;  // the values of AcGeom::shot, by value
};

__device__ __forceinline__ bool ac_written(int ix, int iz, int nx, int nz)
{
    return iz >= 2 && iz < nz - 2 && ix >= 2 && ix < nx - 2;
}

// Work classes of a tile, from the first step's region (the tile plus its 2-cell
// ring): `edge` when a cell there is one the reference never writes or lies on a
// source / receiver row (stale values, free surface, sampling, injections), `spg`
// when a cell there has a sponge factor from the table.
template <int R2, int SPONGE>
__device__ __forceinline__ void ac2_tile_class(const AcGeom& g, const Ac2Step& p, int x0, int z0,
                                               bool& edge, bool& spg)
{
    using T = Ac2Tile<R2, SPONGE>;
    const int xa = x0 - 2, xb = x0 + AC_TX + 1, za = z0 - 2, zb = z0 + T::TZ + 1;
    edge = xa < 2 || xb >= g.nx - 2 || za < 2 || zb >= g.nz - 2;
    const bool src = p.s[0].inj_w || p.s[1].inj_w;
    const bool rec = p.s[0].rec_out || p.s[0].inj_data || p.s[1].rec_out || p.s[1].inj_data;
    if (src && p.src_iz >= za && p.src_iz <= zb) edge = true;
    if (rec && p.rec_iz >= za && p.rec_iz <= zb) edge = true;
    spg = false;
    if (SPONGE == SPONGE_LUT) {
        const int n = g.n_sponge;
        spg = xa < n || xb > g.nx - 1 - n || zb > g.nz - 1 - n || (!g.free_surface && za < n);
    }
}

// Sponge factor of a written cell (LUT mode).
__device__ __forceinline__ float ac2_lut(const AcGeom& g, int ix, int iz, float u)
{
    const int d = sponge_dist(ix, iz, g.nx, g.nz, g.n_sponge, g.free_surface);
    return d > 0 ? fmul(u, __ldg(g.sponge_lut + d)) : u;
}

// Free surface, receiver sampling and next-step injections of one column of a result
// held in shared memory (rows from global row `zorg`, `rows` of them, pitch AC2_W):
// the one-step kernel's order (acoustic_kernels.cuh, general path).  own_rows:
// global rows this tile samples receivers on.
__device__ __forceinline__ void ac2_column(float* R, int zorg, int rows, int c, int ix,
                                           const AcGeom& g, const Ac2Step& p, const AcStep& s,
                                           int own_lo, int own_hi)
{
    if (g.free_surface) {
        const int r0 = 0 - zorg, r1 = 1 - zorg, r2 = 2 - zorg;
        if (r0 >= 0 && r0 < rows) R[r0 * AC2_W + c] = 0.0f;
        // p_next[1, ix] = -p_next[2, ix] before any injection
        if (r1 >= 0 && r1 < rows && r2 < rows) R[r1 * AC2_W + c] = -R[r2 * AC2_W + c];
    }
    const int src_ix = p.src_ix, src_iz = p.src_iz, rec_iz = p.rec_iz;
    if ((s.rec_out || s.inj_data) && rec_iz - zorg >= 0 && rec_iz - zorg < rows) {
        const int k0 = __ldg(g.rec_ptr + ix), k1 = __ldg(g.rec_ptr + ix + 1);
        if (k1 > k0) {
            float* cell = R + (rec_iz - zorg) * AC2_W + c;
            float val = *cell;
            if (s.rec_out && rec_iz >= own_lo && rec_iz < own_hi)
                for (int k = k0; k < k1; ++k) s.rec_out[__ldg(g.rec_list + k)] = val;
            if (s.inj_data) {
                for (int k = k0; k < k1; ++k)
                    val = fadd(val, fmul(__ldg(s.inj_data + __ldg(g.rec_list + k)), s.dt2_inj));
                *cell = val;
            }
        }
    }
    if (s.inj_w && ix == src_ix && src_iz - zorg >= 0 && src_iz - zorg < rows) {
        float* cell = R + (src_iz - zorg) * AC2_W + c;
        *cell = fadd(*cell, fmul(__ldg(s.inj_w), s.dt2_inj));
    }
}

template <int R2, int SPONGE>
__global__ void __launch_bounds__(128)
    acoustic_step2_kernel(const __grid_constant__ Ac2Maps maps, const AcGeom g,
                          const __grid_constant__ Ac2Step p)
{
    using T = Ac2Tile<R2, SPONGE>;
    extern __shared__ __align__(128) float smem[];
    float* B = smem;                  // p_curr: rows z0-4.., columns x0-4..
    float* A = B + T::B_FLOATS;       // p_prev: rows z0-2..
    float* V = A + T::E_FLOATS;       // vel^2 dt^2: rows z0-2..
    float* S = V + T::E_FLOATS;       // per-cell sponge: rows z0-2.. (SPONGE_ARRAY)
    float* E = smem + T::B_FLOATS + T::N_BOXES * T::E_FLOATS;  // step n result: rows z0-2..
    // step n+1 result of a boundary tile, rows z0..: p_curr's centre rows, each cell
    // overwritten by the thread that has just read it as that step's p_prev
    float* F = B + 4 * AC2_W;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::FLOATS);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int x0 = blockIdx.x * AC_TX, z0 = blockIdx.y * T::TZ;
    const int nx = g.nx, nz = g.nz, ldx = g.ldx;
    if (tid == 0) {
        prefetch_tensormap(&maps.curr);
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    // set-up overlaps the previous kernel's tail when launched as a programmatic
    // dependent; every thread waits before any global access
    grid_dep_launch();
    grid_dep_wait();
    bool edge, spg;
    ac2_tile_class<R2, SPONGE>(g, p, x0, z0, edge, spg);
    if (tid == 0) {
        // an edge tile also takes the stale p_next region into E, where the first
        // step leaves the cells the reference never writes untouched
        mbar_expect_tx(bar, T::TX_BYTES + (edge ? T::E_FLOATS * 4u : 0u));
        tma_load_2d(B, &maps.curr, x0 - AC_HX, z0 - 4, bar);
        tma_load_2d(A, &maps.prev, x0 - AC_HX, z0 - 2, bar);
        tma_load_2d(V, &maps.vel, x0 - AC_HX, z0 - 2, bar);
        if (SPONGE == SPONGE_ARRAY) tma_load_2d(S, &maps.sponge, x0 - AC_HX, z0 - 2, bar);
        if (edge) tma_load_2d(E, &maps.stale, x0 - AC_HX, z0 - 2, bar);
    }
    __syncthreads();
    // a CTA-uniform decision: a partial exit before the warp shuffles would be undefined
    if (__syncthreads_or(!mbar_wait_bounded(bar, 0))) {
        if (tid == 0) atomicOr(p.s[0].err, ERR_TMA_TIMEOUT);
        return;
    }
    const int sc = AC_HX + 4 * lane;  // shared-memory column of this lane's first point
    const int ixb = x0 + 4 * lane;
    auto ld4 = [&](const float* box, int row) {
        return *reinterpret_cast<const float4*>(&box[row * AC2_W + sc]);
    };
    auto x_halo = [&](const float* box, int row, float e[8]) {
        const float4 w = ld4(box, row);
        float l2 = __shfl_up_sync(0xffffffffu, w.z, 1);
        float l1 = __shfl_up_sync(0xffffffffu, w.w, 1);
        float r1 = __shfl_down_sync(0xffffffffu, w.x, 1);
        float r2 = __shfl_down_sync(0xffffffffu, w.y, 1);
        if (lane == 0) {
            l2 = box[row * AC2_W + AC_HX - 2];
            l1 = box[row * AC2_W + AC_HX - 1];
        }
        if (lane == 31) {
            r1 = box[row * AC2_W + AC_HX + AC_TX];
            r2 = box[row * AC2_W + AC_HX + AC_TX + 1];
        }
        e[0] = l2;
        e[1] = l1;
        e[2] = w.x;
        e[3] = w.y;
        e[4] = w.z;
        e[5] = w.w;
        e[6] = r1;
        e[7] = r2;
    };

    // ---- step n on rows z0-2 .. z0+TZ+1, columns x0-2 .. x0+129 -> E ----
#pragma unroll
    for (int r = 0; r < T::R1; ++r) {
        const int er = warp * T::R1 + r;  // E row; p_curr rows er .. er+4 around it
        const int iz = z0 - 2 + er;
        float e[8];
        x_halo(B, er + 2, e);
        float u[4];
        ac_row(e, ld4(B, er), ld4(B, er + 1), ld4(B, er + 3), ld4(B, er + 4), ld4(A, er),
               ld4(V, er), g.inv_dx2, g.inv_dz2, u);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (SPONGE == SPONGE_ARRAY) u[j] = fmul(u[j], S[er * AC2_W + sc + j]);
            const int ix = ixb + j;
            if (edge && !ac_written(ix, iz, nx, nz))
                u[j] = E[er * AC2_W + sc + j];  // stale value (zero outside the grid)
            else if (SPONGE == SPONGE_LUT && spg)
                u[j] = ac2_lut(g, ix, iz, u[j]);
        }
        *reinterpret_cast<float4*>(&E[er * AC2_W + sc]) = make_float4(u[0], u[1], u[2], u[3]);
    }
    // the ring columns x0-2, x0-1, x0+128, x0+129 (shared columns 2, 3, 132, 133)
    for (int t = tid; t < 4 * T::ER; t += 128) {
        const int er = t >> 2, k = t & 3;
        const int c = k < 2 ? 2 + k : AC_TX + 2 + k;
        const int ix = x0 - AC_HX + c, iz = z0 - 2 + er;
        float v;
        if (edge && !ac_written(ix, iz, nx, nz)) {
            v = E[er * AC2_W + c];  // stale value (zero outside the grid)
        } else {
            const float* b = B + (er + 2) * AC2_W;
            const float cc = b[c];
            const float lx = fmul(lap5(b[c - 2], b[c - 1], cc, b[c + 1], b[c + 2]), g.inv_dx2);
            const float lz = fmul(lap5(B[er * AC2_W + c], B[(er + 1) * AC2_W + c], cc,
                                       B[(er + 3) * AC2_W + c], B[(er + 4) * AC2_W + c]),
                                  g.inv_dz2);
            v = fadd(fsub(fmul(2.0f, cc), A[er * AC2_W + c]), fmul(V[er * AC2_W + c], fadd(lx, lz)));
            if (SPONGE == SPONGE_ARRAY) v = fmul(v, S[er * AC2_W + c]);
            if (SPONGE == SPONGE_LUT && spg) v = ac2_lut(g, ix, iz, v);
        }
        E[er * AC2_W + c] = v;
    }
    __syncthreads();
    if (edge) {
        // free surface, sampling of step n, injections of step n+1, per column
        for (int c = 2 + tid; c < AC_TX + 6; c += 128) {
            const int ix = x0 - AC_HX + c;
            if (ix < 0 || ix >= nx) continue;
            const bool own_col = c >= AC_HX && c < AC_HX + AC_TX;
            ac2_column(E, z0 - 2, T::ER, c, ix, g, p, p.s[0], own_col ? z0 : 0,
                       own_col ? z0 + T::TZ : 0);
        }
        __syncthreads();
    }

    // ---- fused pointwise work of both steps' p_curr on the tile ----
    const bool col_ok = ixb < ldx;
    const bool fused0 = p.s[0].snap_out || p.s[0].illum || p.s[0].image;
    const bool fused1 = p.s[1].snap_out || p.s[1].illum || p.s[1].image;
    if (fused0 || fused1) {
#pragma unroll
        for (int r = 0; r < R2; ++r) {
            const int cr = warp * R2 + r, iz = z0 + cr;
            if (!col_ok || iz >= nz) continue;
            const size_t off = (size_t)iz * ldx + ixb;
            if (fused0) ac_fused_row(p.s[0], off, ld4(B, cr + 4));
            if (fused1) ac_fused_row(p.s[1], off, ld4(E, cr + 2));
        }
    }

    // ---- step n+1 on the tile -> F ----
#pragma unroll
    for (int r = 0; r < R2; ++r) {
        const int cr = warp * R2 + r, iz = z0 + cr;
        float e[8];
        x_halo(E, cr + 2, e);
        float u[4];
        ac_row(e, ld4(E, cr), ld4(E, cr + 1), ld4(E, cr + 3), ld4(E, cr + 4), ld4(B, cr + 4),
               ld4(V, cr + 2), g.inv_dx2, g.inv_dz2, u);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (SPONGE == SPONGE_ARRAY) u[j] = fmul(u[j], S[(cr + 2) * AC2_W + sc + j]);
            const int ix = ixb + j;
            if (edge && (iz >= nz || ix >= nx))
                u[j] = 0.0f;
            else if (edge && !ac_written(ix, iz, nx, nz))
                u[j] = A[(cr + 2) * AC2_W + sc + j];  // the reference's p_next of step n+1
            else if (SPONGE == SPONGE_LUT && spg)
                u[j] = ac2_lut(g, ix, iz, u[j]);
        }
        if (!edge) {
            // both results of a tile away from the edges leave from registers
            if (col_ok && iz < nz) {
                const size_t off = (size_t)iz * ldx + ixb;
                *reinterpret_cast<float4*>(p.out1 + off) = make_float4(e[2], e[3], e[4], e[5]);
                *reinterpret_cast<float4*>(p.out2 + off) = make_float4(u[0], u[1], u[2], u[3]);
            }
        } else {
            *reinterpret_cast<float4*>(&F[cr * AC2_W + sc]) = make_float4(u[0], u[1], u[2], u[3]);
        }
    }
    if (!edge) return;
    __syncthreads();
    for (int c = AC_HX + tid; c < AC_HX + AC_TX; c += 128) {
        const int ix = x0 - AC_HX + c;
        if (ix >= nx) continue;
        ac2_column(F, z0, T::TZ, c, ix, g, p, p.s[1], z0, z0 + T::TZ);
    }
    __syncthreads();

    // ---- both results of an edge tile, every column up to the row pitch ----
#pragma unroll
    for (int r = 0; r < R2; ++r) {
        const int cr = warp * R2 + r, iz = z0 + cr;
        if (!col_ok || iz >= nz) continue;
        const size_t off = (size_t)iz * ldx + ixb;
        *reinterpret_cast<float4*>(p.out1 + off) = ld4(E, cr + 2);
        *reinterpret_cast<float4*>(p.out2 + off) = ld4(F, cr);
    }
}

constexpr int AC2_R2 = 3;  // default: tiles of 128 x 12 (rows per warp 2..4 supported)

template <int R2, int SPONGE>
inline cudaError_t launch_acoustic_step2_t(const Ac2Maps& m, const AcGeom& g, const Ac2Step& p,
                                           cudaStream_t st, int pdl)
{
    using T = Ac2Tile<R2, SPONGE>;
    const cudaError_t e = set_smem_once<acoustic_step2_kernel<R2, SPONGE>>((int)T::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    dim3 grid((g.nx + AC_TX - 1) / AC_TX, (g.nz + T::TZ - 1) / T::TZ);
    return launch_ex(acoustic_step2_kernel<R2, SPONGE>, grid, dim3(128), T::SMEM_BYTES, st, pdl, m,
                     g, p);
}

template <int R2>
inline cudaError_t launch_acoustic_step2_r(int sponge, const Ac2Maps& m, const AcGeom& g,
                                           const Ac2Step& p, cudaStream_t st, int pdl)
{
    if (sponge == SPONGE_LUT) return launch_acoustic_step2_t<R2, SPONGE_LUT>(m, g, p, st, pdl);
    if (sponge == SPONGE_ARRAY) return launch_acoustic_step2_t<R2, SPONGE_ARRAY>(m, g, p, st, pdl);
    return launch_acoustic_step2_t<R2, SPONGE_NONE>(m, g, p, st, pdl);
}

// rpw: rows per warp of the tile (2, 3 or 4); the maps' boxes must match it.
inline cudaError_t launch_acoustic_step2(int rpw, int sponge, const Ac2Maps& m, const AcGeom& g,
                                         const Ac2Step& p, cudaStream_t st, int pdl)
{
    if (rpw == 2) return launch_acoustic_step2_r<2>(sponge, m, g, p, st, pdl);
    if (rpw == 4) return launch_acoustic_step2_r<4>(sponge, m, g, p, st, pdl);
    return launch_acoustic_step2_r<3>(sponge, m, g, p, st, pdl);
}

// Box heights of the two-step kernel's maps for rows-per-warp rpw.
inline int ac2_curr_rows(int rpw) { return 4 * rpw + 8; }
inline int ac2_ring_rows(int rpw) { return 4 * rpw + 4; }

}  // namespace w2d
