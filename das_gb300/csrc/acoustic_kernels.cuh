// acoustic_kernels.cuh -- fused 2D acoustic time-step kernels for sm_103a.
//
// One tile-step advances a 128 (x) by TZ (z) tile of one wavefield by one step of
// the reference scheme (tsw_rtm/c_engine/wave2d.c:19-82): 4th-order Laplacian in
// x and z, second-order leapfrog, Cerjan sponge multiply on the interior,
// free-surface rows 0 and 1 rewritten after the interior.  Everything else the
// reference does around that call in Python (tsw_rtm/wave_solver.py:157-183 and
// :210-242) is fused into the same pass so each wavefield is read once:
//   * receiver sampling of p_next (forward, wave_solver.py:177),
//   * source injection of the NEXT step into p_next (forward, :159),
//   * receiver-data injection of the NEXT step into p_next (backward, :212-213),
//   * snapshot copy of p_curr (forward, :179-180),
//   * illumination accumulation sum(p_curr^2) (rtm_engine.py:89),
//   * zero-lag imaging image += fwd * p_curr * dt (wave2d.c:218-231 at :230-240).
//
// Data movement: three 2D TMA boxes per tile land in shared memory on one
// mbarrier -- p_curr with a 2-row / 4-column halo (136 x (TZ+4); the 4-column
// halo keeps the box's x start 16-byte aligned), p_prev and vel^2 dt^2 (128 x TZ
// each), plus the sponge when it is a per-cell array.  No register holds an
// operand while the copies are in flight.  Each lane owns four consecutive x
// points (float4); each warp walks RPW rows keeping a five-row register window
// along z; the x halo comes from the neighbouring lanes through warp shuffles
// (shared memory only at the warp's two ends).  p_next leaves with float4
// stores.
//
// Tiles that touch no boundary row/column, no sponge cell, no source and no
// receiver row take a straight path (stencil + float4 store per row).  Other
// tiles take the general path: cells the reference never writes (ix < 2,
// ix >= nx-2, iz >= nz-2, and iz < 2 without a free surface) keep their value
// in the p_next buffer; sampling or injecting there reads that stale value,
// exactly as the reference's 3-buffer rotation does.
#pragma once

#include "w2d_common.cuh"

namespace w2d {

enum SpongeMode { SPONGE_NONE = 0, SPONGE_LUT = 1, SPONGE_ARRAY = 2 };

// Geometry and per-shot constants of one acoustic propagation.
struct AcGeom {
    int nx, nz, ldx;
    float inv_dx2, inv_dz2;  // 1/(dx*dx), 1/(dz*dz) in float32, as the reference
    int free_surface;
    int n_sponge;
    const float* sponge_lut;  // n_sponge+1 values by integer frame distance (LUT mode)
    const int* rec_ptr;       // CSR over columns: receivers of column ix are
    const int* rec_list;      //   rec_list[rec_ptr[ix] .. rec_ptr[ix+1])
    const int* shot;          // device ints {src_ix, src_iz, rec_iz, n_rec, rec_c0}: rec_c0
                              //   is the column of receiver 0 when receiver r sits at
                              //   column rec_c0 + r for every r, else -1
    int l2_hints;             // 1: keep p_curr, vel^2 dt^2 and p_next in L2 (evict-last),
                              //    stream p_prev (evict-first)
};

// rec_c0 of the shot ints: the column of receiver 0 when receiver r sits at column
// rec_c0 + r for every r (then each column holds at most one receiver and its index
// follows from the column), else -1.
inline int receivers_consecutive_c0(const int* rec_ix, int n_rec)
{
    if (n_rec <= 0) return -1;
    for (int r = 1; r < n_rec; ++r)
        if (rec_ix[r] != rec_ix[0] + r) return -1;
    return rec_ix[0];
}

// Per-launch pointers (all optional ones may be null).
struct AcStep {
    float* p_next;
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
    int early;               // p_prev and the model may be read before the dependency
                             // wait (acoustic_step_kernel): nothing still running writes them
};

// The TMA descriptors of one tile-step.
struct AcMaps {
    CUtensorMap curr;    // p_curr, box AC_SW x (TZ+4)
    CUtensorMap prev;    // p_prev, box AC_TX x TZ
    CUtensorMap vel;     // vel^2 dt^2, box AC_TX x TZ
    CUtensorMap sponge;  // per-cell sponge, box AC_TX x TZ (SPONGE_ARRAY only)
};

constexpr int AC_TX = 128;  // tile width in x (32 lanes x float4)
constexpr int AC_HX = 4;    // x halo kept in shared memory (2 used; 4 keeps TMA x aligned)
constexpr int AC_SW = AC_TX + 2 * AC_HX;

template <int WARPS, int RPW, int SPONGE>
struct AcTile {
    static constexpr int TZ = WARPS * RPW;
    static constexpr int C_FLOATS = (TZ + 4) * AC_SW;
    static constexpr int P_FLOATS = TZ * AC_TX;
    static constexpr int S_FLOATS = SPONGE == SPONGE_ARRAY ? TZ * AC_TX : 0;
    static constexpr int FLOATS = C_FLOATS + 2 * P_FLOATS + S_FLOATS;
    static constexpr unsigned TX_BYTES = FLOATS * 4u;
    static constexpr size_t SMEM_BYTES = FLOATS * 4u + 128;  // + mbarrier slot
};

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

// Issue the TMA boxes of a tile at (x0, z0) onto `bar` (one elected thread).
template <int WARPS, int RPW, int SPONGE>
__device__ __forceinline__ void ac_issue_loads(float* smem, const AcMaps* m, int x0, int z0,
                                               uint64_t* bar, int l2_hints = 0)
{
    using T = AcTile<WARPS, RPW, SPONGE>;
    mbar_expect_tx(bar, T::TX_BYTES);
    if (l2_hints) {
        // p_curr is re-read next step as p_prev and vel^2 dt^2 every step; p_prev's
        // plane is overwritten next step
        const uint64_t keep = policy_evict_last(), drop = policy_evict_first();
        tma_load_2d_hint(smem, &m->curr, x0 - AC_HX, z0 - 2, bar, keep);
        tma_load_2d_hint(smem + T::C_FLOATS, &m->prev, x0, z0, bar, drop);
        tma_load_2d_hint(smem + T::C_FLOATS + T::P_FLOATS, &m->vel, x0, z0, bar, keep);
    } else {
        tma_load_2d(smem, &m->curr, x0 - AC_HX, z0 - 2, bar);
        tma_load_2d(smem + T::C_FLOATS, &m->prev, x0, z0, bar);
        tma_load_2d(smem + T::C_FLOATS + T::P_FLOATS, &m->vel, x0, z0, bar);
    }
    if (SPONGE == SPONGE_ARRAY)
        tma_load_2d(smem + T::C_FLOATS + 2 * T::P_FLOATS, &m->sponge, x0, z0, bar);
}

// The boxes of a tile that only earlier steps wrote (p_prev, v^2 dt^2, the sponge
// array), expecting the whole tile's bytes on `bar`; then the p_curr box with its halo.
template <int WARPS, int RPW, int SPONGE>
__device__ __forceinline__ void ac_issue_own(float* smem, const AcMaps* m, int x0, int z0,
                                             uint64_t* bar, int l2_hints)
{
    using T = AcTile<WARPS, RPW, SPONGE>;
    mbar_expect_tx(bar, T::TX_BYTES);
    if (l2_hints) {
        tma_load_2d_hint(smem + T::C_FLOATS, &m->prev, x0, z0, bar, policy_evict_first());
        tma_load_2d_hint(smem + T::C_FLOATS + T::P_FLOATS, &m->vel, x0, z0, bar,
                         policy_evict_last());
    } else {
        tma_load_2d(smem + T::C_FLOATS, &m->prev, x0, z0, bar);
        tma_load_2d(smem + T::C_FLOATS + T::P_FLOATS, &m->vel, x0, z0, bar);
    }
    if (SPONGE == SPONGE_ARRAY)
        tma_load_2d(smem + T::C_FLOATS + 2 * T::P_FLOATS, &m->sponge, x0, z0, bar);
}

template <int WARPS, int RPW, int SPONGE>
__device__ __forceinline__ void ac_issue_curr(float* smem, const AcMaps* m, int x0, int z0,
                                              uint64_t* bar, int l2_hints)
{
    if (l2_hints)
        tma_load_2d_hint(smem, &m->curr, x0 - AC_HX, z0 - 2, bar, policy_evict_last());
    else
        tma_load_2d(smem, &m->curr, x0 - AC_HX, z0 - 2, bar);
}

// True when no cell of the tile needs boundary, sponge, source or receiver work.
template <int WARPS, int RPW, int SPONGE>
__device__ __forceinline__ bool ac_tile_is_plain(const AcGeom& g, const AcStep& s, int x0, int z0)
{
    constexpr int TZ = WARPS * RPW;
    const int x1 = x0 + AC_TX - 1, z1 = z0 + TZ - 1;
    if (x0 < 2 || x1 >= g.nx - 2 || z0 < 2 || z1 >= g.nz - 2) return false;
    if (SPONGE == SPONGE_LUT) {
        const int n = g.n_sponge;
        if (x0 < n || x1 > g.nx - 1 - n || z1 > g.nz - 1 - n || (!g.free_surface && z0 < n))
            return false;
    }
    if (s.inj_w || s.rec_out || s.inj_data) {
        const int src_iz = g.shot[1], rec_iz = g.shot[2];
        if (s.inj_w && src_iz >= z0 && src_iz <= z1) return false;
        if ((s.rec_out || s.inj_data) && rec_iz >= z0 && rec_iz <= z1) return false;
    }
    return true;
}

// Stencil of one row of four points: reference operation order, no contraction.
__device__ __forceinline__ void ac_row(const float e[8], const float4& w0, const float4& w1,
                                       const float4& w3, const float4& w4, const float4& pp,
                                       const float4& vv, float inv_dx2, float inv_dz2,
                                       float u[4])
{
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float c = e[j + 2];
        const float lx = fmul(lap5(e[j], e[j + 1], c, e[j + 3], e[j + 4]), inv_dx2);
        const float lz = fmul(lap5(comp(w0, j), comp(w1, j), c, comp(w3, j), comp(w4, j)), inv_dz2);
        u[j] = fadd(fsub(fmul(2.0f, c), comp(pp, j)), fmul(comp(vv, j), fadd(lx, lz)));
    }
}

// Snapshot / illumination / imaging of one row of p_curr (fused pointwise work).
__device__ __forceinline__ void ac_fused_row(const AcStep& s, size_t off, const float4& c)
{
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

// Stencil, fused pointwise work and stores of one tile whose boxes are in shared
// memory.  Called by every thread of the CTA.
template <int WARPS, int RPW, int SPONGE>
__device__ __forceinline__ void ac_tile_body(const float* smem, const AcGeom& g, const AcStep& s,
                                             int x0, int z0)
{
    static_assert(RPW >= 3, "free-surface rows 0..2 must belong to one warp");
    using T = AcTile<WARPS, RPW, SPONGE>;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nx = g.nx, nz = g.nz, ldx = g.ldx;
    const int ixb = x0 + 4 * lane;
    const int zr0 = z0 + warp * RPW;
    const bool col_ok = ixb < ldx;
    const float* tile = smem;
    const float* tp = smem + T::C_FLOATS;
    const float* tv = tp + T::P_FLOATS;
    const float* ts = tv + T::P_FLOATS;

    const int sc = AC_HX + 4 * lane;  // shared-memory column of this lane's first point
    const int sr0 = warp * RPW;       // shared-memory row of global row zr0 - 2
    auto lds4 = [&](int srow) {
        return *reinterpret_cast<const float4*>(&tile[srow * AC_SW + sc]);
    };
    auto pw4 = [&](const float* base, int r) {
        return *reinterpret_cast<const float4*>(&base[(sr0 + r) * AC_TX + 4 * lane]);
    };
    auto x_halo = [&](const float4& w2, int srow, float e[8]) {
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
        e[0] = l2;
        e[1] = l1;
        e[2] = w2.x;
        e[3] = w2.y;
        e[4] = w2.z;
        e[5] = w2.w;
        e[6] = r1;
        e[7] = r2;
    };
    const bool fused = s.snap_out || s.illum || s.image;

    if (ac_tile_is_plain<WARPS, RPW, SPONGE>(g, s, x0, z0)) {
        // ---- straight path: every cell of the tile is an interior cell ----
        float4 w0 = lds4(sr0 + 0), w1 = lds4(sr0 + 1), w2 = lds4(sr0 + 2), w3 = lds4(sr0 + 3);
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
            const float4 w4 = lds4(sr0 + r + 4);
            float e[8];
            x_halo(w2, sr0 + r + 2, e);
            float u[4];
            ac_row(e, w0, w1, w3, w4, pw4(tp, r), pw4(tv, r), g.inv_dx2, g.inv_dz2, u);
            if (SPONGE == SPONGE_ARRAY) {
                const float4 sp = pw4(ts, r);
                u[0] = fmul(u[0], sp.x);
                u[1] = fmul(u[1], sp.y);
                u[2] = fmul(u[2], sp.z);
                u[3] = fmul(u[3], sp.w);
            }
            const size_t off = (size_t)(zr0 + r) * ldx + ixb;
            if (g.l2_hints)  // read next step as p_curr
                st_hint_v4(s.p_next + off, make_float4(u[0], u[1], u[2], u[3]), policy_evict_last());
            else
                *reinterpret_cast<float4*>(s.p_next + off) = make_float4(u[0], u[1], u[2], u[3]);
            if (fused) ac_fused_row(s, off, w2);
            w0 = w1;
            w1 = w2;
            w2 = w3;
            w3 = w4;
        }
        return;
    }

    // ---- general path ----
    float out[RPW][4];
    {
        float4 w0 = lds4(sr0 + 0), w1 = lds4(sr0 + 1), w2 = lds4(sr0 + 2), w3 = lds4(sr0 + 3);
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
            const float4 w4 = lds4(sr0 + r + 4);
            float e[8];
            x_halo(w2, sr0 + r + 2, e);
            float u[4];
            ac_row(e, w0, w1, w3, w4, pw4(tp, r), pw4(tv, r), g.inv_dx2, g.inv_dz2, u);
            const int iz = zr0 + r;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (SPONGE == SPONGE_ARRAY) {
                    u[j] = fmul(u[j], comp(pw4(ts, r), j));
                } else if (SPONGE == SPONGE_LUT) {
                    const int d = sponge_dist(ixb + j, iz, nx, nz, g.n_sponge, g.free_surface);
                    if (d > 0) u[j] = fmul(u[j], __ldg(g.sponge_lut + d));
                }
                out[r][j] = u[j];
            }
            w0 = w1;
            w1 = w2;
            w2 = w3;
            w3 = w4;
        }
    }

    if (fused) {
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
            const int iz = zr0 + r;
            if (!col_ok || iz >= nz) continue;
            ac_fused_row(s, (size_t)iz * ldx + ixb, lds4(sr0 + r + 2));
        }
    }

    // stores, boundary rows, receivers and next-step injection
    const int src_ix = g.shot[0], src_iz = g.shot[1], rec_iz = g.shot[2];
    const bool rec_active = (s.rec_out != nullptr) || (s.inj_data != nullptr);
    // The receiver row's lookups for this lane's four columns.  Receivers on consecutive
    // columns in index order (rec_c0 >= 0, the usual surface line): receiver ix - rec_c0,
    // one round of loads (the data samples).  Otherwise three rounds of independent loads
    // (CSR bounds, first receiver index, its data sample) rather than one dependent chain
    // per column.  The first receiver of column ixb+j is rk[j] (-1: none); further ones
    // (CSR only, rare) are read in the loop below.
    int kb[4] = {0, 0, 0, 0}, ke[4] = {0, 0, 0, 0}, rk[4] = {-1, -1, -1, -1};
    float rd[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const bool warp_rec = rec_active && col_ok && rec_iz >= zr0 && rec_iz < zr0 + RPW &&
                          rec_iz < nz;
    if (warp_rec) {
        const int rec_c0 = g.shot[4], n_rec = g.shot[3];
        if (rec_c0 >= 0) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int r = ixb + j - rec_c0;
                rk[j] = (ixb + j < nx && r >= 0 && r < n_rec) ? r : -1;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const bool in = ixb + j < nx;
                kb[j] = in ? __ldg(g.rec_ptr + ixb + j) : 0;
                ke[j] = in ? __ldg(g.rec_ptr + ixb + j + 1) : 0;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) rk[j] = ke[j] > kb[j] ? __ldg(g.rec_list + kb[j]) : -1;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            rd[j] = (s.inj_data && rk[j] >= 0) ? __ldg(s.inj_data + rk[j]) : 0.0f;
    }
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
            if (at_rec && rk[j] >= 0) {
                // receivers of the column in index order (the reference's per-receiver
                // loop): sampling sees the value before any injection
                const int k0 = kb[j], k1 = ke[j];
                if (s.rec_out) {
                    s.rec_out[rk[j]] = val;
                    for (int k = k0 + 1; k < k1; ++k) s.rec_out[__ldg(g.rec_list + k)] = val;
                }
                if (s.inj_data) {
                    val = fadd(val, fmul(rd[j], s.dt2_inj));
                    for (int k = k0 + 1; k < k1; ++k)
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

// One tile per CTA, one launch per time step.
template <int WARPS, int RPW, int SPONGE>
__global__ void __launch_bounds__(WARPS * 32)
    acoustic_step_kernel(const __grid_constant__ AcMaps maps, const AcGeom g, const AcStep s)
{
    using T = AcTile<WARPS, RPW, SPONGE>;
    extern __shared__ __align__(128) float smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::FLOATS);
    const int x0 = blockIdx.x * AC_TX;
    const int z0 = blockIdx.y * T::TZ;
    if (threadIdx.x == 0) {
        prefetch_tensormap(&maps.curr);
        mbar_init(bar, 1);
        fence_mbar_init();
        // Early: p_prev was written by the step before the previous one and the model
        // long before.  Each step kernel triggers its dependents only after its own
        // dependency wait (below), so this kernel started after that step had completed:
        // these boxes go out while the previous step still drains.
        if (s.early) ac_issue_own<WARPS, RPW, SPONGE>(smem, &maps, x0, z0, bar, g.l2_hints);
    }
    if (s.snap_in && threadIdx.x < T::TZ && z0 + (int)threadIdx.x < g.nz) {
        // imaging steps read the forward snapshot (written in the forward pass) from HBM
        // after the stencil: bring the tile's rows into L2 now (one row per thread,
        // within the row pitch).  (Prefetching the next imaging step's rows one step
        // ahead as well measured no better.)
        const int row = z0 + threadIdx.x;
        prefetch_l2_bulk(s.snap_in + (size_t)row * g.ldx + x0,
                         (uint32_t)min(AC_TX, g.ldx - x0) * 4u);
    }
    // p_curr is the previous step's output: read only after the wait.  The dependents
    // are released after it, so the next step cannot start before this one's
    // predecessor has completed (what makes the next step's early boxes safe).
    grid_dep_wait();
    grid_dep_launch();
    if (threadIdx.x == 0) {
        if (!s.early) ac_issue_own<WARPS, RPW, SPONGE>(smem, &maps, x0, z0, bar, g.l2_hints);
        ac_issue_curr<WARPS, RPW, SPONGE>(smem, &maps, x0, z0, bar, g.l2_hints);
    }
    __syncthreads();
    // a CTA-uniform decision: a partial exit before the warp shuffles would be undefined
    if (__syncthreads_or(!mbar_wait_bounded(bar, 0))) {
        if (threadIdx.x == 0) atomicOr(s.err, ERR_TMA_TIMEOUT);
        return;
    }
    ac_tile_body<WARPS, RPW, SPONGE>(smem, g, s, x0, z0);
}

// Persistent form of the same tile-step: a grid sized to the resident capacity,
// tiles handed out by an atomic counter, and the next tile's TMA boxes loading
// into a second shared-memory stage while the current tile is computed.
//
// The counter is never reset between launches: every CTA takes tiles until it
// draws an index past the last tile, so one launch draws exactly ntiles + gridDim.x
// indices and the next launch starts at base + ntiles + gridDim.x.
template <int WARPS, int RPW, int SPONGE>
__global__ void __launch_bounds__(WARPS * 32)
    acoustic_step_persistent(const __grid_constant__ AcMaps maps, const AcGeom g, const AcStep s,
                             unsigned* counter, unsigned base, int tiles_x, int ntiles)
{
    using T = AcTile<WARPS, RPW, SPONGE>;
    extern __shared__ __align__(128) float smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * T::FLOATS);
    __shared__ int s_tile[2];
    const int tid = threadIdx.x;
    if (tid == 0) {
        prefetch_tensormap(&maps.curr);
        prefetch_tensormap(&maps.prev);
        prefetch_tensormap(&maps.vel);
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
        fence_mbar_init();
    }
    grid_dep_launch();
    grid_dep_wait();
    auto issue = [&](int t, int stage) {
        const int x0 = (t % tiles_x) * AC_TX, z0 = (t / tiles_x) * T::TZ;
        ac_issue_loads<WARPS, RPW, SPONGE>(smem + stage * T::FLOATS, &maps, x0, z0, bar + stage,
                                           g.l2_hints);
    };
    // an index outside [0, ntiles) ends the CTA's work
    auto draw = [&]() {
        const unsigned u = atomicAdd(counter, 1u) - base;
        return u < (unsigned)ntiles ? (int)u : ntiles;
    };
    if (tid == 0) {
        const int t = draw();
        s_tile[0] = t;
        if (t < ntiles) issue(t, 0);
    }
    __syncthreads();
    for (int i = 0;; ++i) {
        const int st = i & 1;
        const int t = s_tile[st];
        if (t >= ntiles) break;
        bool next_issued = false;
        if (tid == 0) {
            // the other stage was released by the barrier that ended the previous tile
            const int tn = draw();
            s_tile[st ^ 1] = tn;
            if (tn < ntiles) {
                fence_proxy_async_shared();
                issue(tn, st ^ 1);
                next_issued = true;
            }
        }
        const bool got = mbar_wait_bounded(bar + st, (unsigned)(i >> 1) & 1u);
        if (__syncthreads_or(!got)) {
            if (tid == 0) {
                atomicOr(s.err, ERR_TMA_TIMEOUT);
                // let the copy in flight into the other stage land before leaving
                if (next_issued) mbar_wait_bounded(bar + (st ^ 1), (unsigned)((i + 1) >> 1) & 1u);
            }
            return;
        }
        const int x0 = (t % tiles_x) * AC_TX, z0 = (t / tiles_x) * T::TZ;
        ac_tile_body<WARPS, RPW, SPONGE>(smem + st * T::FLOATS, g, s, x0, z0);
        __syncthreads();
    }
}

// Launch with optional programmatic stream serialization (the kernel may begin
// while the previous kernel of the stream drains).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_ex(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                             cudaStream_t st, int pdl, Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <int WARPS, int RPW, int SPONGE>
inline cudaError_t launch_acoustic_step(const AcMaps& m, const AcGeom& g, const AcStep& s,
                                        cudaStream_t st, int pdl = 0)
{
    using T = AcTile<WARPS, RPW, SPONGE>;
    const cudaError_t e =
        set_smem_once<acoustic_step_kernel<WARPS, RPW, SPONGE>>((int)T::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    dim3 grid((g.nx + AC_TX - 1) / AC_TX, (g.nz + T::TZ - 1) / T::TZ);
    if (!pdl) {
        acoustic_step_kernel<WARPS, RPW, SPONGE><<<grid, WARPS * 32, T::SMEM_BYTES, st>>>(m, g, s);
        return cudaGetLastError();
    }
    return launch_ex(acoustic_step_kernel<WARPS, RPW, SPONGE>, grid, dim3(WARPS * 32),
                     T::SMEM_BYTES, st, pdl, m, g, s);
}

// Shared memory of the persistent form: two stages and their barriers.
template <int WARPS, int RPW, int SPONGE>
constexpr size_t persistent_smem_bytes()
{
    return 2 * AcTile<WARPS, RPW, SPONGE>::FLOATS * 4u + 128;
}

// Resident CTAs of the persistent form on the current device (0 on error): one query
// per instantiation and device, safe when several host threads ask.
template <int WARPS, int RPW, int SPONGE>
inline int persistent_capacity()
{
    auto query = [](int dev) {
        const int smem = (int)persistent_smem_bytes<WARPS, RPW, SPONGE>();
        if (set_smem_once<acoustic_step_persistent<WARPS, RPW, SPONGE>>(smem) != cudaSuccess)
            return 0;
        int per_sm = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, acoustic_step_persistent<WARPS, RPW, SPONGE>, WARPS * 32, smem) !=
                cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return 0;
        return per_sm * sms;
    };
    static std::once_flag once[W2D_MAX_DEVICES];
    static int cap[W2D_MAX_DEVICES];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (dev < 0 || dev >= W2D_MAX_DEVICES) return query(dev);
    std::call_once(once[dev], [&query, dev] { cap[dev] = query(dev); });
    return cap[dev];
}

// One persistent launch; *base is advanced by the indices the launch draws.
template <int WARPS, int RPW, int SPONGE>
inline cudaError_t launch_acoustic_persistent(const AcMaps& m, const AcGeom& g, const AcStep& s,
                                              cudaStream_t st, int pdl, unsigned* counter,
                                              unsigned* base)
{
    using T = AcTile<WARPS, RPW, SPONGE>;
    const int cap = persistent_capacity<WARPS, RPW, SPONGE>();
    if (cap <= 0) return cudaErrorInvalidConfiguration;
    const int tiles_x = (g.nx + AC_TX - 1) / AC_TX;
    const int ntiles = tiles_x * ((g.nz + T::TZ - 1) / T::TZ);
    const int grid = cap < ntiles ? cap : ntiles;
    const unsigned b = *base;
    const cudaError_t e =
        launch_ex(acoustic_step_persistent<WARPS, RPW, SPONGE>, dim3(grid), dim3(WARPS * 32),
                  persistent_smem_bytes<WARPS, RPW, SPONGE>(), st, pdl, m, g, s, counter, b,
                  tiles_x, ntiles);
    if (e == cudaSuccess) *base = b + (unsigned)(ntiles + grid);
    return e;
}

// Encode the TMA descriptors of one tile-step over pitched fields.
inline int make_ac_maps(AcMaps* m, const float* curr, const float* prev, const float* vel,
                        const float* sponge, int nx, int nz, int ldx, int tz)
{
    int rc;
    if ((rc = make_tensor_map_2d(&m->curr, curr, nx, nz, ldx, AC_SW, tz + 4))) return rc;
    if ((rc = make_tensor_map_2d(&m->prev, prev, nx, nz, ldx, AC_TX, tz))) return rc;
    if ((rc = make_tensor_map_2d(&m->vel, vel, nx, nz, ldx, AC_TX, tz))) return rc;
    if (sponge && (rc = make_tensor_map_2d(&m->sponge, sponge, nx, nz, ldx, AC_TX, tz))) return rc;
    if (!sponge) m->sponge = m->vel;
    return W2D_OK;
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
