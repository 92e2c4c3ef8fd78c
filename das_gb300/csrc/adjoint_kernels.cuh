// adjoint_kernels.cuh -- discrete adjoint of the fused acoustic step, for the
// velocity gradient of a least-squares misfit (RTM as the adjoint).
//
// Forward step (interior cells i, acoustic_kernels.cuh):
//     P[n+1]_i = s_i * (2 P[n]_i - P[n-1]_i + c_i (L P[n])_i),   c = v^2 dt^2,
// rows 0 and 1 with a free surface: P[n+1][0,:] = 0, P[n+1][1,x] = -P[n+1][2,x];
// traces d[n] = P[n+1] at the receivers (before the next injection).
//
// With residual traces r[n] (dJ/dd[n]) the adjoint of P[n] is
//     Lam[n] = S^T r[n-1] + 2 a[n+1] + L^T(c a[n+1]) - a[n+2],
// where a[n] = s * mu[n] on interior cells (zero elsewhere) and mu[n] is Lam[n]
// restricted to the interior with the free-surface fold mu[2,x] = Lam[2,x] -
// Lam[1,x].  L is the same symmetric 4th-order stencil, so L^T(c a) is the
// stencil applied to the product c*a (zero outside the interior).  The gradient
// with respect to c accumulates in the same pass:
//     dJ/dc_i = sum_n a[n+1]_i (L P[n])_i.
// Sources and receivers must sit on written cells (interior, or rows 0/1 with
// the free surface) so that the reference's never-written cells stay zero and
// the step is linear in the wavefields.
#pragma once

#include "acoustic_kernels.cuh"

namespace w2d {

struct AdjStep {
    float* a_out;            // a[n]
    float* grad;             // += a[n+1] * (L P[n]) on interior cells, or null
    const float* resid_row;  // r[n-1] (n_rec), or null
    unsigned* err;
};

struct AdjMaps {
    CUtensorMap a1;   // a[n+1], halo box
    CUtensorMap c;    // v^2 dt^2, halo box
    CUtensorMap pf;   // forward field P[n], halo box
    CUtensorMap a2;   // a[n+2], plain box
};

template <int WARPS, int RPW>
struct AdjTile {
    static constexpr int TZ = WARPS * RPW;
    static constexpr int H_FLOATS = (TZ + 4) * AC_SW;
    static constexpr int P_FLOATS = TZ * AC_TX;
    static constexpr int FLOATS = 3 * H_FLOATS + P_FLOATS;
    static constexpr unsigned TX_BYTES = FLOATS * 4u;
    static constexpr size_t SMEM_BYTES = FLOATS * 4u + 128;
};

// Laplacian (x part * inv_dx2 + z part * inv_dz2) of a halo tile at shared-memory
// row `srow`, column `scol`.
__device__ __forceinline__ float adj_lap(const float* t, int srow, int scol, float inv_dx2,
                                         float inv_dz2)
{
    const float* p = t + srow * AC_SW + scol;
    const float lx = lap5(p[-2], p[-1], p[0], p[1], p[2]);
    const float lz = lap5(p[-2 * AC_SW], p[-AC_SW], p[0], p[AC_SW], p[2 * AC_SW]);
    return lx * inv_dx2 + lz * inv_dz2;
}

// Per-cell form: one point per thread iteration, scalar shared-memory and global
// accesses.  Kept as the check of the vectorised form below (they differ only in the
// compiler's contraction choices) and selectable with w2d_fwi_set_adjoint_form.
template <int WARPS, int RPW>
__global__ void __launch_bounds__(WARPS * 32)
    acoustic_adjoint_cells_kernel(const __grid_constant__ AdjMaps maps, const AcGeom g,
                                  const AdjStep s)
{
    static_assert(RPW >= 3, "free-surface rows 0..2 must belong to one warp");
    using T = AdjTile<WARPS, RPW>;
    extern __shared__ __align__(128) float smem[];
    float* ta1 = smem;
    float* tb = smem + T::H_FLOATS;  // c, then c * a[n+1]
    float* tp = smem + 2 * T::H_FLOATS;
    float* ta2 = smem + 3 * T::H_FLOATS;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::FLOATS);
    const int x0 = blockIdx.x * AC_TX;
    const int z0 = blockIdx.y * T::TZ;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        mbar_expect_tx(bar, T::TX_BYTES);
        // the model, the forward field P[n] (recomputed before this segment's adjoint steps)
        // and a[n+2] (two launches back): issued before the dependency wait.  Each adjoint
        // step releases its dependents only after its own wait, so when this one started the
        // step before the previous one had completed.
        tma_load_2d(tb, &maps.c, x0 - AC_HX, z0 - 2, bar);
        tma_load_2d(tp, &maps.pf, x0 - AC_HX, z0 - 2, bar);
        tma_load_2d(ta2, &maps.a2, x0, z0, bar);
    }
    // a[n+1] is the previous launch's output (and the gradient it updated): after the wait
    grid_dep_wait();
    grid_dep_launch();
    if (threadIdx.x == 0) tma_load_2d(ta1, &maps.a1, x0 - AC_HX, z0 - 2, bar);
    __syncthreads();
    // a CTA-uniform decision: a partial exit before the warp shuffles would be undefined
    if (__syncthreads_or(!mbar_wait_bounded(bar, 0))) {
        if (threadIdx.x == 0) atomicOr(s.err, ERR_TMA_TIMEOUT);
        return;
    }
    for (int i = threadIdx.x; i < T::H_FLOATS; i += blockDim.x) tb[i] = tb[i] * ta1[i];
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nx = g.nx, nz = g.nz, ldx = g.ldx;
    const int ixb = x0 + 4 * lane;
    const int zr0 = z0 + warp * RPW;
    const int rec_iz = g.shot[2];
    float lam_row1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const int iz = zr0 + r;
        if (iz >= nz) break;
        const int srow = warp * RPW + r + 2;
        const bool row_interior = iz >= 2 && iz < nz - 2;
        const bool need_row = row_interior || (g.free_surface && iz == 1);
        if (!need_row) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int ix = ixb + j;
            if (ix >= nx) continue;
            const int scol = AC_HX + 4 * lane + j;
            const float a1 = ta1[srow * AC_SW + scol];
            const float a2 = ta2[(srow - 2) * AC_TX + 4 * lane + j];
            float lam = 2.0f * a1 + adj_lap(tb, srow, scol, g.inv_dx2, g.inv_dz2) - a2;
            if (s.resid_row && iz == rec_iz) {
                const int k0 = __ldg(g.rec_ptr + ix), k1 = __ldg(g.rec_ptr + ix + 1);
                for (int k = k0; k < k1; ++k) lam += __ldg(s.resid_row + __ldg(g.rec_list + k));
            }
            const bool interior = row_interior && ix >= 2 && ix < nx - 2;
            if (!interior) {
                if (iz == 1) lam_row1[j] = lam;  // free-surface row feeds the fold of row 2
                continue;
            }
            if (g.free_surface && iz == 2) lam -= lam_row1[j];
            float sp = 1.0f;
            if (g.sponge_lut) {
                const int d = sponge_dist(ix, iz, nx, nz, g.n_sponge, g.free_surface);
                if (d > 0) sp = __ldg(g.sponge_lut + d);
            }
            const size_t off = (size_t)iz * ldx + ix;
            s.a_out[off] = sp * lam;
            if (s.grad)
                s.grad[off] += a1 * adj_lap(tp, srow, scol, g.inv_dx2, g.inv_dz2);
        }
    }
}

// Vectorised form (the default): each lane owns four consecutive x points (float4
// shared-memory reads, x neighbours by warp shuffles, a five-row register window
// along z for c * a[n+1], formed as its rows are read, and for P[n]), float4 stores of a[n] and of the gradient on
// tiles away from the frame; tiles touching the frame, the receiver row or the
// sponge apply the per-point rules of the per-cell form to the same values.
template <int WARPS, int RPW>
__global__ void __launch_bounds__(WARPS * 32)
    acoustic_adjoint_kernel(const __grid_constant__ AdjMaps maps, const AcGeom g, const AdjStep s)
{
    static_assert(RPW >= 3, "free-surface rows 0..2 must belong to one warp");
    using T = AdjTile<WARPS, RPW>;
    extern __shared__ __align__(128) float smem[];
    float* ta1 = smem;
    float* tb = smem + T::H_FLOATS;  // c
    float* tp = smem + 2 * T::H_FLOATS;
    float* ta2 = smem + 3 * T::H_FLOATS;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::FLOATS);
    const int x0 = blockIdx.x * AC_TX;
    const int z0 = blockIdx.y * T::TZ;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        mbar_expect_tx(bar, T::TX_BYTES);
        // the model, the forward field P[n] and a[n+2] (two launches back): issued before
        // the dependency wait (see the per-cell form)
        tma_load_2d(tb, &maps.c, x0 - AC_HX, z0 - 2, bar);
        tma_load_2d(tp, &maps.pf, x0 - AC_HX, z0 - 2, bar);
        tma_load_2d(ta2, &maps.a2, x0, z0, bar);
    }
    grid_dep_wait();
    grid_dep_launch();
    if (threadIdx.x == 0) tma_load_2d(ta1, &maps.a1, x0 - AC_HX, z0 - 2, bar);
    __syncthreads();
    if (__syncthreads_or(!mbar_wait_bounded(bar, 0))) {
        if (threadIdx.x == 0) atomicOr(s.err, ERR_TMA_TIMEOUT);
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nx = g.nx, nz = g.nz, ldx = g.ldx;
    const int ixb = x0 + 4 * lane;
    const int zr0 = z0 + warp * RPW;
    const int sc = AC_HX + 4 * lane;  // shared-memory column of this lane's first point
    const int sr0 = warp * RPW;       // halo-box row of global row zr0 - 2
    const float idx2 = g.inv_dx2, idz2 = g.inv_dz2;
    auto ld4 = [&](const float* box, int row) {
        return *reinterpret_cast<const float4*>(&box[row * AC_SW + sc]);
    };
    // c * a[n+1] of a box row (the product is formed where it is read: no extra pass)
    auto ldb = [&](int row) {
        const float4 c = ld4(tb, row), a = ld4(ta1, row);
        return make_float4(c.x * a.x, c.y * a.y, c.z * a.z, c.w * a.w);
    };
    // box value at a shared-memory index: P[n], or c * a[n+1] when prod
    auto at = [&](const float* box, bool prod, int i) { return prod ? tb[i] * ta1[i] : box[i]; };
    auto x_halo = [&](const float* box, bool prod, const float4& w, int row, float e[8]) {
        float l2 = __shfl_up_sync(0xffffffffu, w.z, 1);
        float l1 = __shfl_up_sync(0xffffffffu, w.w, 1);
        float r1 = __shfl_down_sync(0xffffffffu, w.x, 1);
        float r2 = __shfl_down_sync(0xffffffffu, w.y, 1);
        if (lane == 0) {
            l2 = at(box, prod, row * AC_SW + AC_HX - 2);
            l1 = at(box, prod, row * AC_SW + AC_HX - 1);
        }
        if (lane == 31) {
            r1 = at(box, prod, row * AC_SW + AC_HX + AC_TX);
            r2 = at(box, prod, row * AC_SW + AC_HX + AC_TX + 1);
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
    // the same Laplacian as adj_lap: x part * inv_dx2 + z part * inv_dz2
    auto lap = [&](const float e[8], const float4& m2, const float4& m1, const float4& p1,
                   const float4& p2, int j) {
        const float lx = lap5(e[j], e[j + 1], e[j + 2], e[j + 3], e[j + 4]);
        const float lz = lap5(comp(m2, j), comp(m1, j), e[j + 2], comp(p1, j), comp(p2, j));
        return lx * idx2 + lz * idz2;
    };

    // a tile whose every point is an interior cell away from the receiver row and the
    // sponge: no per-point rule applies
    const int rec_iz = g.shot[2];
    bool plain = x0 >= 2 && x0 + AC_TX - 1 < nx - 2 && z0 >= 2 && z0 + T::TZ - 1 < nz - 2 &&
                 !(s.resid_row && rec_iz >= z0 && rec_iz < z0 + T::TZ);
    if (plain && g.sponge_lut) {
        const int n = g.n_sponge;
        plain = x0 >= n && x0 + AC_TX - 1 <= nx - 1 - n && z0 + T::TZ - 1 <= nz - 1 - n &&
                (g.free_surface || z0 >= n);
    }

    float4 b0 = ldb(sr0), b1 = ldb(sr0 + 1), b2 = ldb(sr0 + 2), b3 = ldb(sr0 + 3);
    float4 q0 = ld4(tp, sr0), q1 = ld4(tp, sr0 + 1), q2 = ld4(tp, sr0 + 2), q3 = ld4(tp, sr0 + 3);
    float lam_row1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const int iz = zr0 + r;
        const int srow = sr0 + r + 2;
        const float4 b4 = ldb(srow + 2), q4 = ld4(tp, srow + 2);
        float eb[8], eq[8];
        x_halo(tb, true, b2, srow, eb);
        x_halo(tp, false, q2, srow, eq);
        const float4 a1 = ld4(ta1, srow);
        const float4 a2 = *reinterpret_cast<const float4*>(&ta2[(sr0 + r) * AC_TX + 4 * lane]);
        float lam[4], gr[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            lam[j] = 2.0f * comp(a1, j) + lap(eb, b0, b1, b3, b4, j) - comp(a2, j);
            gr[j] = comp(a1, j) * lap(eq, q0, q1, q3, q4, j);
        }
        if (plain) {
            const size_t off = (size_t)iz * ldx + ixb;
            *reinterpret_cast<float4*>(s.a_out + off) = make_float4(lam[0], lam[1], lam[2], lam[3]);
            if (s.grad) {
                float4 gv = *reinterpret_cast<const float4*>(s.grad + off);
                gv.x += gr[0];
                gv.y += gr[1];
                gv.z += gr[2];
                gv.w += gr[3];
                *reinterpret_cast<float4*>(s.grad + off) = gv;
            }
        } else if (iz < nz) {
            const bool row_interior = iz >= 2 && iz < nz - 2;
            const bool need_row = row_interior || (g.free_surface && iz == 1);
            if (need_row) {
                const int rec_c0 = g.shot[4], n_rec = g.shot[3];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int ix = ixb + j;
                    if (ix >= nx) continue;
                    float lm = lam[j];
                    if (s.resid_row && iz == rec_iz) {
                        if (rec_c0 >= 0) {
                            const int rr = ix - rec_c0;
                            if (rr >= 0 && rr < n_rec) lm += __ldg(s.resid_row + rr);
                        } else {
                            const int k0 = __ldg(g.rec_ptr + ix), k1 = __ldg(g.rec_ptr + ix + 1);
                            for (int k = k0; k < k1; ++k)
                                lm += __ldg(s.resid_row + __ldg(g.rec_list + k));
                        }
                    }
                    const bool interior = row_interior && ix >= 2 && ix < nx - 2;
                    if (!interior) {
                        if (iz == 1) lam_row1[j] = lm;  // feeds the fold of row 2
                        continue;
                    }
                    if (g.free_surface && iz == 2) lm -= lam_row1[j];
                    float sp = 1.0f;
                    if (g.sponge_lut) {
                        const int d = sponge_dist(ix, iz, nx, nz, g.n_sponge, g.free_surface);
                        if (d > 0) sp = __ldg(g.sponge_lut + d);
                    }
                    const size_t off = (size_t)iz * ldx + ix;
                    s.a_out[off] = sp * lm;
                    if (s.grad) s.grad[off] += gr[j];
                }
            }
        }
        b0 = b1;
        b1 = b2;
        b2 = b3;
        b3 = b4;
        q0 = q1;
        q1 = q2;
        q2 = q3;
        q3 = q4;
    }
}

// pdl: a programmatic dependent of the stream's previous operation, which must then be
// an adjoint step (it releases this launch only after its own wait).
// cells: the per-cell form instead of the vectorised one.
template <int WARPS, int RPW>
inline cudaError_t launch_adjoint_step(const AdjMaps& m, const AcGeom& g, const AdjStep& s,
                                       cudaStream_t st, int pdl = 0, int cells = 0)
{
    using T = AdjTile<WARPS, RPW>;
    auto kernel = cells ? acoustic_adjoint_cells_kernel<WARPS, RPW>
                        : acoustic_adjoint_kernel<WARPS, RPW>;
    const cudaError_t e = cells
        ? set_smem_once<acoustic_adjoint_cells_kernel<WARPS, RPW>>((int)T::SMEM_BYTES)
        : set_smem_once<acoustic_adjoint_kernel<WARPS, RPW>>((int)T::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    dim3 grid((g.nx + AC_TX - 1) / AC_TX, (g.nz + T::TZ - 1) / T::TZ);
    return launch_ex(kernel, grid, dim3(WARPS * 32), T::SMEM_BYTES, st, pdl, m, g, s);
}

}  // namespace w2d
