// acoustic_kernels.cuh -- fused 2D acoustic time-step kernels for sm_103a.
//
// One launch advances one wavefield by one step of the reference scheme
// (tsw_rtm/c_engine/wave2d.c:19-82): 4th-order Laplacian in x and z,
// second-order leapfrog, Cerjan sponge multiply on the interior, free-surface
// rows 0 and 1 rewritten after the interior.  Everything else the reference
// does around that call in Python (tsw_rtm/wave_solver.py:157-183 and
// :210-242) is fused into the same pass so each wavefield is read once:
//   * receiver sampling of p_next (forward, wave_solver.py:177),
//   * source injection of the NEXT step into p_next (forward, :159),
//   * receiver-data injection of the NEXT step into p_next (backward, :212-213),
//   * snapshot copy of p_curr (forward, :179-180),
//   * illumination accumulation sum(p_curr^2) (rtm_engine.py:89),
//   * zero-lag imaging image += fwd * p_curr * dt (wave2d.c:218-231 at :230-240).
//
// Tiling: a CTA owns a 128 (x) by WARPS*RPW (z) tile.  p_curr arrives through
// one TMA 2D box load with a 2-row / 4-column halo into shared memory; each lane
// owns four consecutive x points (float4) and each warp walks RPW rows keeping
// a five-row register window along z; the x halo comes from the neighbouring
// lanes through warp shuffles (shared memory only at the warp's two ends).
// p_prev and the velocity term are streamed with float4 loads issued before
// the TMA wait.
//
// Cells the reference never writes (ix < 2, ix >= nx-2, iz >= nz-2, and iz < 2
// without a free surface) keep their value in the p_next buffer; sampling or
// injecting there reads that stale value, exactly as the reference's 3-buffer
// rotation does.
#pragma once

#include "w2d_common.cuh"

namespace w2d {

// Geometry and per-shot constants of one acoustic propagation.
struct AcGeom {
    int nx, nz, ldx;
    float inv_dx2, inv_dz2;  // 1/(dx*dx), 1/(dz*dz) in float32, as the reference
    int free_surface;
    int n_sponge;
    const float* sponge_lut;  // n_sponge+1 values by integer frame distance, or null
    const float* sponge_arr;  // full pitched sponge array, or null (then LUT or none)
    const int* rec_ptr;       // CSR over columns: receivers of column ix are
    const int* rec_list;      //   rec_list[rec_ptr[ix] .. rec_ptr[ix+1])
    const int* shot;          // device ints {src_ix, src_iz, rec_iz}
};

// Per-launch pointers (all optional ones may be null).
struct AcStep {
    const float* p_prev;
    float* p_next;
    const float* v2dt2;      // vel*vel*dt2 per cell (pitched)
    float* snap_out;         // forward: copy of p_curr
    float* illum;            // forward: += p_curr^2
    float* rec_out;          // forward: samples of p_next at the receivers, one row
    const float* snap_in;    // backward: forward snapshot of this step
    float* image;            // backward: += snap_in * p_curr * img_dt
    float img_dt;
    const float* inj_w;      // forward: wavelet sample of the next step
    const float* inj_data;   // backward: receiver-data row of the next step
    float dt2_inj;           // float32(dt**2) as the Python drivers compute it
    unsigned* err;
};

constexpr int AC_TX = 128;  // tile width in x (32 lanes x float4)
constexpr int AC_HX = 4;    // x halo kept in shared memory (2 used; 4 keeps TMA x aligned)
constexpr int AC_SW = AC_TX + 2 * AC_HX;

__device__ __forceinline__ float lap5(float m2, float m1, float c, float p1, float p2)
{
    // ((c2*(m2+p2)) + (c1*(m1+p1))) + (c0*c), the reference order (wave2d.c:50-57)
    const float k0 = -2.5f, k1 = 4.0f / 3.0f, k2 = -1.0f / 12.0f;
    float acc = fmul(k2, fadd(m2, p2));
    acc = fadd(acc, fmul(k1, fadd(m1, p1)));
    return fadd(acc, fmul(k0, c));
}

__device__ __forceinline__ float comp(const float4& v, int j)
{
    return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

__device__ __forceinline__ int sponge_dist(int ix, int iz, int nx, int nz, int n, int fs)
{
    int d = 0;
    d = max(d, n - ix);
    d = max(d, ix - (nx - 1 - n));
    d = max(d, iz - (nz - 1 - n));
    if (!fs) d = max(d, n - iz);
    return d;
}

template <int WARPS, int RPW>
struct AcTile {
    static constexpr int TZ = WARPS * RPW;
    static constexpr int SH = TZ + 4;
    static constexpr int SMEM_FLOATS = SH * AC_SW;
    static constexpr unsigned TX_BYTES = SMEM_FLOATS * 4u;
};

// Pointwise operands of one tile, loaded before the TMA box is waited for.
template <int RPW>
struct AcPoint {
    float4 pp[RPW], vv[RPW], sp[RPW];
};

template <int WARPS, int RPW>
__device__ __forceinline__ void ac_load_pointwise(const AcGeom& g, const AcStep& s, int x0, int z0,
                                                  AcPoint<RPW>& P)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int ixb = x0 + 4 * lane;
    const int zr0 = z0 + warp * RPW;
    const bool col_ok = ixb < g.ldx;
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const int iz = zr0 + r;
        P.pp[r] = P.vv[r] = P.sp[r] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (col_ok && iz < g.nz) {
            const size_t off = (size_t)iz * g.ldx + ixb;
            P.pp[r] = __ldg(reinterpret_cast<const float4*>(s.p_prev + off));
            P.vv[r] = __ldg(reinterpret_cast<const float4*>(s.v2dt2 + off));
            if (g.sponge_arr) P.sp[r] = __ldg(reinterpret_cast<const float4*>(g.sponge_arr + off));
        }
    }
}

// Stencil, fused pointwise work and stores of one tile whose p_curr box (with
// halo) is in shared memory.  Called by every thread of the CTA.
template <int WARPS, int RPW>
__device__ __forceinline__ void ac_tile_body(const float* tile, const AcGeom& g, const AcStep& s,
                                             int x0, int z0, const AcPoint<RPW>& P)
{
    static_assert(RPW >= 3, "free-surface rows 0..2 must belong to one warp");
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nx = g.nx, nz = g.nz, ldx = g.ldx;
    const int ixb = x0 + 4 * lane;
    const int zr0 = z0 + warp * RPW;
    const bool col_ok = ixb < ldx;
    const float4* pp = P.pp;
    const float4* vv = P.vv;
    const float4* sp = P.sp;

    const int sc = AC_HX + 4 * lane;  // shared-memory column of this lane's first point
    const int sr0 = warp * RPW;       // shared-memory row of global row zr0 - 2
    auto lds4 = [&](int srow) {
        return *reinterpret_cast<const float4*>(&tile[srow * AC_SW + sc]);
    };

    float out[RPW][4];
    float4 w0 = lds4(sr0 + 0), w1 = lds4(sr0 + 1), w2 = lds4(sr0 + 2), w3 = lds4(sr0 + 3);
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const float4 w4 = lds4(sr0 + r + 4);
        const int srow = sr0 + r + 2;
        float l2 = __shfl_up_sync(0xffffffffu, w2.z, 1);
        float l1 = __shfl_up_sync(0xffffffffu, w2.w, 1);
        float r1 = __shfl_down_sync(0xffffffffu, w2.x, 1);
        float r2 = __shfl_down_sync(0xffffffffu, w2.y, 1);
        if (lane == 0) {
            l2 = tile[srow * AC_SW + AC_HX - 2];
            l1 = tile[srow * AC_SW + AC_HX - 1];
        }
        if (lane == 31) {
            r1 = tile[srow * AC_SW + AC_HX + AC_TX];
            r2 = tile[srow * AC_SW + AC_HX + AC_TX + 1];
        }
        const float e[8] = {l2, l1, w2.x, w2.y, w2.z, w2.w, r1, r2};
        const int iz = zr0 + r;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float c = e[j + 2];
            const float lx = fmul(lap5(e[j], e[j + 1], c, e[j + 3], e[j + 4]), g.inv_dx2);
            const float lz = fmul(lap5(comp(w0, j), comp(w1, j), c, comp(w3, j), comp(w4, j)),
                                  g.inv_dz2);
            float u = fadd(fsub(fmul(2.0f, c), comp(pp[r], j)), fmul(comp(vv[r], j), fadd(lx, lz)));
            if (g.sponge_arr) {
                u = fmul(u, comp(sp[r], j));
            } else if (g.sponge_lut) {
                const int d = sponge_dist(ixb + j, iz, nx, nz, g.n_sponge, g.free_surface);
                if (d > 0) u = fmul(u, __ldg(g.sponge_lut + d));
            }
            out[r][j] = u;
        }
        w0 = w1;
        w1 = w2;
        w2 = w3;
        w3 = w4;
    }

    // ---- fused pointwise work on p_curr (snapshot / illumination / imaging) ----
    if (s.snap_out || s.illum || s.image) {
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
            const int iz = zr0 + r;
            if (!col_ok || iz >= nz) continue;
            const float4 c = lds4(sr0 + r + 2);
            const size_t off = (size_t)iz * ldx + ixb;
            if (s.snap_out) __stcs(reinterpret_cast<float4*>(s.snap_out + off), c);
            if (s.illum) {
                float4 a = *reinterpret_cast<float4*>(s.illum + off);
                a.x = fadd(a.x, fmul(c.x, c.x));
                a.y = fadd(a.y, fmul(c.y, c.y));
                a.z = fadd(a.z, fmul(c.z, c.z));
                a.w = fadd(a.w, fmul(c.w, c.w));
                *reinterpret_cast<float4*>(s.illum + off) = a;
            }
            if (s.image) {
                const float4 f = __ldcs(reinterpret_cast<const float4*>(s.snap_in + off));
                float4 a = *reinterpret_cast<float4*>(s.image + off);
                a.x = fadd(a.x, fmul(fmul(f.x, c.x), s.img_dt));
                a.y = fadd(a.y, fmul(fmul(f.y, c.y), s.img_dt));
                a.z = fadd(a.z, fmul(fmul(f.z, c.z), s.img_dt));
                a.w = fadd(a.w, fmul(fmul(f.w, c.w), s.img_dt));
                *reinterpret_cast<float4*>(s.image + off) = a;
            }
        }
    }

    // ---- stores, boundary rows, receivers and next-step injection ----
    const int src_ix = g.shot[0], src_iz = g.shot[1], rec_iz = g.shot[2];
    const bool rec_active = (s.rec_out != nullptr) || (s.inj_data != nullptr);
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const int iz = zr0 + r;
        if (!col_ok || iz >= nz) continue;
        const bool row_interior = (iz >= 2) && (iz < nz - 2);
        const bool special = (rec_active && iz == rec_iz) || (s.inj_w && iz == src_iz) ||
                             (g.free_surface && iz < 2);
        float* row_next = s.p_next + (size_t)iz * ldx;
        if (!special && row_interior && ixb >= 2 && ixb + 3 < nx - 2) {
            *reinterpret_cast<float4*>(row_next + ixb) =
                make_float4(out[r][0], out[r][1], out[r][2], out[r][3]);
            continue;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int ix = ixb + j;
            if (ix >= nx) continue;
            bool wr = row_interior && ix >= 2 && ix < nx - 2;
            float val = out[r][j];
            if (g.free_surface && iz == 0) {
                val = 0.0f;
                wr = true;
            } else if (g.free_surface && iz == 1) {
                // p_next[1,:] = -p_next[2,:] over every column (wave2d.c:75-80); row 2 is
                // this thread's register row 2 (zr0 == 0 here) or a never-written cell.
                float row2 = 0.0f;
                const bool row2_interior = (2 < nz - 2) && ix >= 2 && ix < nx - 2;
                if (row2_interior) {
                    if (zr0 == 0) row2 = out[2][j];
                } else {
                    row2 = s.p_next[(size_t)2 * ldx + ix];
                }
                val = -row2;
                wr = true;
            }
            const bool at_rec = rec_active && iz == rec_iz;
            const bool at_src = s.inj_w && iz == src_iz && ix == src_ix;
            if (!wr && (at_rec || at_src)) val = row_next[ix];
            if (at_rec) {
                const int k0 = __ldg(g.rec_ptr + ix), k1 = __ldg(g.rec_ptr + ix + 1);
                if (s.rec_out)
                    for (int k = k0; k < k1; ++k) s.rec_out[__ldg(g.rec_list + k)] = val;
                if (s.inj_data && k1 > k0) {
                    for (int k = k0; k < k1; ++k)
                        val = fadd(val, fmul(__ldg(s.inj_data + __ldg(g.rec_list + k)), s.dt2_inj));
                    wr = true;
                }
            }
            if (at_src) {
                val = fadd(val, fmul(__ldg(s.inj_w), s.dt2_inj));
                wr = true;
            }
            if (wr) row_next[ix] = val;
        }
    }
}

template <int WARPS, int RPW>
__global__ void __launch_bounds__(WARPS * 32)
    acoustic_step_kernel(const __grid_constant__ CUtensorMap tm_curr, const AcGeom g, const AcStep s)
{
    using T = AcTile<WARPS, RPW>;
    __shared__ __align__(128) float tile[T::SMEM_FLOATS];
    __shared__ __align__(8) uint64_t bar;
    const int x0 = blockIdx.x * AC_TX;
    const int z0 = blockIdx.y * T::TZ;
    if (threadIdx.x == 0) {
        prefetch_tensormap(&tm_curr);
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, T::TX_BYTES);
        tma_load_2d(tile, &tm_curr, x0 - AC_HX, z0 - 2, &bar);
    }
    AcPoint<RPW> P;
    ac_load_pointwise<WARPS, RPW>(g, s, x0, z0, P);
    if (!mbar_wait_bounded(&bar, 0)) {
        if ((threadIdx.x & 31) == 0) atomicOr(s.err, ERR_TMA_TIMEOUT);
        return;
    }
    ac_tile_body<WARPS, RPW>(tile, g, s, x0, z0, P);
}

template <int WARPS, int RPW>
inline void launch_acoustic_step(const CUtensorMap& tm, const AcGeom& g, const AcStep& s,
                                 cudaStream_t st)
{
    dim3 grid((g.nx + AC_TX - 1) / AC_TX, (g.nz + WARPS * RPW - 1) / (WARPS * RPW));
    acoustic_step_kernel<WARPS, RPW><<<grid, WARPS * 32, 0, st>>>(tm, g, s);
}

// Injection into a field before the first step of a pass (forward: the source
// sample w[0]; backward: receiver row nt-1).  One thread per column, receivers
// of a column added in index order so repeated indices accumulate as the
// reference's per-receiver Python loop does.
static __global__ void inject_kernel(float* p, AcGeom g, const float* w, const float* data_row,
                              float dt2_inj)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    if (ix >= g.nx) return;
    const int src_ix = g.shot[0], src_iz = g.shot[1], rec_iz = g.shot[2];
    if (w && ix == src_ix) {
        float* q = p + (size_t)src_iz * g.ldx + ix;
        *q = fadd(*q, fmul(*w, dt2_inj));
    }
    if (data_row) {
        const int k0 = g.rec_ptr[ix], k1 = g.rec_ptr[ix + 1];
        if (k1 > k0) {
            float* q = p + (size_t)rec_iz * g.ldx + ix;
            float v = *q;
            for (int k = k0; k < k1; ++k) v = fadd(v, fmul(data_row[g.rec_list[k]], dt2_inj));
            *q = v;
        }
    }
}

}  // namespace w2d
