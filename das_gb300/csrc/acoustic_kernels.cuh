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
    const int* shot;          // device ints {src_ix, src_iz, rec_iz}
    int l2_hints;             // 1: keep p_curr, vel^2 dt^2 and p_next in L2 (evict-last),
                              //    stream p_prev (evict-first)
};

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
    }
    // the set-up above overlaps the previous step's tail when launched as a
    // programmatic dependent; nothing of the previous step is read before the wait
    grid_dep_launch();
    grid_dep_wait();
    if (threadIdx.x == 0) ac_issue_loads<WARPS, RPW, SPONGE>(smem, &maps, x0, z0, bar, g.l2_hints);
    if (s.snap_in && threadIdx.x < T::TZ && z0 + (int)threadIdx.x < g.nz) {
        // imaging steps read the forward snapshot from HBM after the stencil: start
        // bringing the tile's rows into L2 now, beside the boxes (one row per thread,
        // within the row pitch).  (Prefetching the next imaging step's rows one step
        // ahead as well measured no better.)
        const int row = z0 + threadIdx.x;
        prefetch_l2_bulk(s.snap_in + (size_t)row * g.ldx + x0,
                         (uint32_t)min(AC_TX, g.ldx - x0) * 4u);
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

// ---------------------------------------------------------------------------------
// Time-persistent form: one cooperative launch advances S consecutive steps of a pass.
//
// Each resident CTA owns a static set of tiles (CTA b: tiles b, b + G, b + 2G, ...) and
// walks them in step order: all of its tiles at step j, then at step j + 1.  A tile
// starts step j once its 3 x 3 neighbour tiles have published step j - 1 (per-tile
// counters `done`, st.release after the tile's stores, ld.acquire before the halo box is
// loaded), so there is no launch, grid-wide barrier or memory flush between steps.  The
// p_prev and v^2 dt^2 boxes read only what this tile itself wrote (or the model) and are
// issued before the wait; only the p_curr box, whose halo neighbours wrote, waits.
//
// Why the neighbour dependency suffices: step j writes p_next into the plane that held
// the field of step j - 2 (p_curr at step j - 2, read by the 3 x 3 neighbourhood through
// the halo; p_prev at step j - 1, read by the tile itself), and reads what the
// neighbourhood wrote at step j - 1.  Why it cannot deadlock: all CTAs are resident
// (cooperative launch), each walks its tiles in step order, so every tile-step a CTA
// waits for belongs to an earlier step of a CTA that reaches it.  Every wait is bounded;
// a timeout sets ERR_DEP_TIMEOUT | ERR_ABORT and all CTAs stop.  The tile body is the
// one every other form runs: results are bit-identical to one launch per step.
struct AcPlan {
    AcMaps maps[3];      // TMA descriptors of local step j use maps[j % 3]
    float* next[3];      // and p_next = next[j % 3]
    int dir;             // +1 forward pass (it = it0 + j), -1 backward pass (it = it0 - j)
    int it0, S;          // reference step of local step 0; steps in this launch
    int nt, interval, n_rec;
    unsigned j0;         // steps of this sequence completed before the launch
    int tiles_x, tiles_z, ntiles;
    size_t plane;        // floats per pitched plane
    float dt2_inj, img_dt;
    // forward pass
    const float* wavelet;  // source sample of step it + 1 injected by step it
    float* rec_out;        // (nt, n_rec) samples of p_next, or null
    float* snaps;          // snapshot it / interval - slot0 on it % interval == 0, or null
    float* illum;          // += p_curr^2 on snapshot steps, or null
    // backward pass
    const float* data;     // receiver row it - 1 injected by step it, or null
    const float* snap_in;  // forward snapshot k - slot0 of imaging steps, or null
    float* image;
    int slot0, n_snaps_valid;
    unsigned* done;        // per tile: steps of this sequence completed
    unsigned* err;
};

// Bounded wait until *p >= target (acquire).  Gives up early when another CTA has set
// ERR_ABORT; on timeout sets ERR_DEP_TIMEOUT | ERR_ABORT so that every CTA stops.
__device__ __forceinline__ bool wait_done(const unsigned* p, unsigned target, unsigned* err)
{
    for (unsigned i = 0; i < (1u << 24); ++i) {
        if (ld_acquire_u32(p) >= target) return true;
        if (i > 64) __nanosleep(128);
        if ((i & 1023) == 1023 && (*reinterpret_cast<volatile unsigned*>(err) & ERR_ABORT))
            return false;
    }
    atomicOr(err, ERR_DEP_TIMEOUT | ERR_ABORT);
    return false;
}

// The AcStep of local step j (the per-step options of the host loops, step for step).
__device__ __forceinline__ void ac_plan_step(const AcPlan& p, int j, AcStep& s)
{
    const int it = p.it0 + p.dir * j;
    s.p_next = p.next[j % 3];
    s.snap_out = nullptr;
    s.illum = nullptr;
    s.rec_out = nullptr;
    s.snap_in = nullptr;
    s.image = nullptr;
    s.img_dt = p.img_dt;
    s.inj_w = nullptr;
    s.inj_data = nullptr;
    s.dt2_inj = p.dt2_inj;
    s.err = p.err;
    if (p.dir > 0) {
        if (it + 1 < p.nt) s.inj_w = p.wavelet + it + 1;
        if (p.rec_out) s.rec_out = p.rec_out + (size_t)it * p.n_rec;
        if (it % p.interval == 0) {
            if (p.snaps) s.snap_out = p.snaps + (size_t)(it / p.interval - p.slot0) * p.plane;
            if (p.illum) s.illum = p.illum;
        }
    } else {
        if (it >= 1 && p.n_rec > 0 && p.data) s.inj_data = p.data + (size_t)(it - 1) * p.n_rec;
        if (p.snap_in && it % p.interval == 0) {
            const int k = it / p.interval;
            if (k >= 0 && k < p.n_snaps_valid) {
                s.snap_in = p.snap_in + (size_t)(k - p.slot0) * p.plane;
                s.image = p.image;
            }
        }
    }
}

// Registers held to what the shared memory allows resident: 8 CTAs of a 128 x 16 tile,
// 4 of a 128 x 32 tile per SM.
template <int WARPS, int RPW, int SPONGE>
__global__ void __launch_bounds__(WARPS * 32, 128 / (WARPS * RPW))
    acoustic_steps_coop(const __grid_constant__ AcPlan p, const AcGeom g)
{
    using T = AcTile<WARPS, RPW, SPONGE>;
    extern __shared__ __align__(128) float smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::FLOATS);
    __shared__ int s_ok;
    const int tid = threadIdx.x;
    const int G = gridDim.x;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        s_ok = 1;
    }
    __syncthreads();
    unsigned phase = 0;
    for (int j = 0; j < p.S; ++j) {
        AcStep s;
        ac_plan_step(p, j, s);
        const AcMaps& m = p.maps[j % 3];
        const unsigned need = p.j0 + (unsigned)j;  // neighbours have completed step j - 1
        for (int t = blockIdx.x; t < p.ntiles; t += G) {
            const int tx = t % p.tiles_x, tz = t / p.tiles_x;
            const int x0 = tx * AC_TX, z0 = tz * T::TZ;
            if (tid == 0) {
                // this tile's own planes: what it wrote before (ordered by the barrier
                // that ended its previous tile-step) and the model
                fence_proxy_async_global();
                fence_proxy_async_shared();
                mbar_expect_tx(bar, T::TX_BYTES);
                tma_load_2d(smem + T::C_FLOATS, &m.prev, x0, z0, bar);
                tma_load_2d(smem + T::C_FLOATS + T::P_FLOATS, &m.vel, x0, z0, bar);
                if (SPONGE == SPONGE_ARRAY)
                    tma_load_2d(smem + T::C_FLOATS + 2 * T::P_FLOATS, &m.sponge, x0, z0, bar);
            }
            if (s.snap_in && tid < T::TZ && z0 + tid < g.nz)
                prefetch_l2_bulk(s.snap_in + (size_t)(z0 + tid) * g.ldx + x0,
                                 (uint32_t)min(AC_TX, g.ldx - x0) * 4u);
            if (tid < 9 && need > 0) {
                const int ux = tx + tid % 3 - 1, uz = tz + tid / 3 - 1;
                if (ux >= 0 && ux < p.tiles_x && uz >= 0 && uz < p.tiles_z)
                    if (!wait_done(p.done + uz * p.tiles_x + ux, need, p.err)) s_ok = 0;
            }
            __syncthreads();
            const int ok = s_ok;
            if (tid == 0) {
                // issued also when a wait failed (the CTA then discards the box): the
                // barrier completes and no copy lands after the CTA has left
                fence_proxy_async_global();  // the neighbours' stores, acquired above
                tma_load_2d(smem, &m.curr, x0 - AC_HX, z0 - 2, bar);
            }
            const bool got = mbar_wait_bounded(bar, phase);
            phase ^= 1u;
            if (__syncthreads_or(!got || !ok)) {
                if (tid == 0 && !got) atomicOr(p.err, ERR_TMA_TIMEOUT | ERR_ABORT);
                return;
            }
            ac_tile_body<WARPS, RPW, SPONGE>(smem, g, s, x0, z0);
            __syncthreads();
            if (tid == 0) {
                __threadfence();
                st_release_u32(p.done + t, need + 1u);
            }
        }
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

// Resident CTAs of the time-persistent form on the current device (0 on error): the
// cooperative launch requires the whole grid to be resident at once.
template <int WARPS, int RPW, int SPONGE>
inline int coop_capacity()
{
    auto query = [](int dev) {
        using T = AcTile<WARPS, RPW, SPONGE>;
        if (set_smem_once<acoustic_steps_coop<WARPS, RPW, SPONGE>>((int)T::SMEM_BYTES) !=
            cudaSuccess)
            return 0;
        int per_sm = 0, sms = 0, coop = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, acoustic_steps_coop<WARPS, RPW, SPONGE>, WARPS * 32,
                (int)T::SMEM_BYTES) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
            !coop)
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

// One cooperative launch of the time-persistent form over p.S steps.
template <int WARPS, int RPW, int SPONGE>
inline cudaError_t launch_acoustic_coop(const AcPlan& p, const AcGeom& g, cudaStream_t st)
{
    using T = AcTile<WARPS, RPW, SPONGE>;
    const int cap = coop_capacity<WARPS, RPW, SPONGE>();
    if (cap <= 0) return cudaErrorCooperativeLaunchTooLarge;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cap < p.ntiles ? cap : p.ntiles);
    cfg.blockDim = dim3(WARPS * 32);
    cfg.dynamicSmemBytes = T::SMEM_BYTES;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, acoustic_steps_coop<WARPS, RPW, SPONGE>, p, g);
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
