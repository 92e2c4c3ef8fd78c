// elastic_kernels.cuh -- 2D elastic velocity-stress step (Levander staggered
// grid, 4th order in space) for sm_103a.
//
// Follows tsw_rtm/c_engine/wave2d.c:95-212: a velocity phase that reads the
// stresses, then a stress phase that reads the UPDATED velocities, each on rows
// [1 if free surface else 2, nz-2) and columns [2, nx-2) (the set M), each
// multiplied by the sponge; then, with the free surface, szz = sxz = 0 on row 0
// and sxx on row 0 from the free-surface relation.  The two phases are two
// launches (the stress phase needs velocities of neighbouring tiles).  Where the
// reference reads row -1 (sxz in the velocity phase, vz in the stress phase, at
// iz = 1) this engine reads zero.  Arithmetic is float32 in the reference's
// operation order without contraction into FMA.
//
// Data movement.  A state is five consecutive pitched planes (vx, vz, sxx, szz,
// sxz) described by one 3D tensor map (x, row, plane).  Each CTA owns a 128 x TZ
// tile; the fields a phase differentiates arrive as TMA boxes of 136 x (TZ+4)
// (2-row and 4-column halo; the 4 keeps the box's x start 16-byte aligned; cells
// outside the grid read as zero) on one mbarrier: sxx, sxz, szz for the velocity
// phase, the new vx, vz for the stress phase.  Each lane owns four consecutive
// x points (float4) and each warp walks RPW rows with a four-row register window
// per field along z; x neighbours come from the adjacent lanes by warp shuffles
// (shared memory only at the warp's two ends).  Fields used at one point only
// (the velocities or stresses being updated, the parameters, the sponge) are
// float4 loads from global memory.
//
// A step may run in place (src == dst) or out of place (dst receives every cell
// of the tile: updated cells in M, copies of src elsewhere, and the free-surface
// row).  The velocity phase can add a source term vz += w * dt at one cell of M
// before the update (the modelling source of the elastic engine).
#pragma once

#include <utility>

#include "w2d_common.cuh"

namespace w2d {

struct ElGeom {
    int nx, nz, ldx;
    float rdx, rdz;  // 1/dx, 1/dz
    float dt;
    int free_surface;
    const float* sponge;  // pitched, or null
};

// One launch of a phase over n_shots shots (blockIdx.z): source and destination
// states (5 planes each, plane stride `plane` floats; shot s at + s * 5 * plane),
// parameters (pitched planes; shot s at + s * pstride), optional source term.
struct ElStep {
    const float* src;
    float* dst;
    size_t plane;
    const float *lam, *mu, *bx, *bz;
    size_t pstride;
    // velocity phase: vz[src_pos[2s+1], src_pos[2s]] += wav[s*nt + n] * dt first
    // (src_pos null: no source term)
    const int* src_pos;
    const float* wav;
    int nt, n;
    unsigned* err;
    // stress phase: the vertical strain Dz- vz of the new velocities at row rec_iz for
    // every receiver (receivers by column: CSR rec_ptr / rec_list), into trace[k] of
    // shot s at + s * trace_stride (null: no sampling)
    float* trace = nullptr;
    const int* rec_ptr = nullptr;
    const int* rec_list = nullptr;
    int rec_iz = 0;
    size_t trace_stride = 0;
    // the pointwise fields may be staged before the dependency wait: the launch two back
    // wrote them (or nothing running does), see the phases' kernels
    int early = 0;
};

struct ElMaps {
    CUtensorMap src;  // 3D map over the source state's planes
    CUtensorMap dst;  // 3D map over the destination state's planes
};

constexpr int EL_TX = 128;
constexpr int EL_HX = 4;
constexpr int EL_SW = EL_TX + 2 * EL_HX;
enum { EL_VX = 0, EL_VZ = 1, EL_SXX = 2, EL_SZZ = 3, EL_SXZ = 4 };

template <int WARPS, int RPW>
struct ElTile {
    static constexpr int TZ = WARPS * RPW;
    static constexpr int BOX = (TZ + 4) * EL_SW;  // floats per halo box
    static constexpr int PT = TZ * EL_TX;         // floats per pointwise field of the tile
    static constexpr int V_FLOATS = 3 * BOX + 5 * PT;  // velocity phase
    static constexpr int S_FLOATS = 2 * BOX + 6 * PT;  // stress phase
};

// Each thread stages the float4s of the pointwise fields it will use (its warp's rows,
// its four columns) into shared memory with asynchronous copies issued at entry, so
// their latency overlaps the halo boxes' instead of following it.
template <int WARPS, int RPW>
__device__ __forceinline__ void el_stage_pointwise(float* pt, const float* const* fields,
                                                   int n_fields, int zr0, int ixb, int lane,
                                                   int warp, const ElGeom& g)
{
    using T = ElTile<WARPS, RPW>;
    if (ixb >= g.ldx) return;
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const int iz = zr0 + r;
        if (iz >= g.nz) continue;
        const size_t off = (size_t)iz * g.ldx + ixb;
        const int lr = warp * RPW + r;
        for (int f = 0; f < n_fields; ++f)
            if (fields[f]) cp_async16(&pt[(f * T::TZ + lr) * EL_TX + 4 * lane], fields[f] + off);
    }
}

// The float4 a thread staged for field f, row r of its warp.
template <int WARPS, int RPW>
__device__ __forceinline__ float4 el_staged(const float* pt, int f, int warp, int r, int lane)
{
    using T = ElTile<WARPS, RPW>;
    return *reinterpret_cast<const float4*>(&pt[(f * T::TZ + warp * RPW + r) * EL_TX + 4 * lane]);
}

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

__device__ __forceinline__ float el_c(const float4& v, int j)
{
    return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

// Row `srow` of a box as this lane's float4 plus the x neighbours it needs:
// e[0..1] = x-2, x-1 of the first point; e[2..5] the four points; e[6..7] = x+4, x+5.
__device__ __forceinline__ void el_xrow(const float* box, int srow, int lane, float e[8])
{
    const float4 w = *reinterpret_cast<const float4*>(&box[srow * EL_SW + EL_HX + 4 * lane]);
    float l2 = __shfl_up_sync(0xffffffffu, w.z, 1);
    float l1 = __shfl_up_sync(0xffffffffu, w.w, 1);
    float r1 = __shfl_down_sync(0xffffffffu, w.x, 1);
    float r2 = __shfl_down_sync(0xffffffffu, w.y, 1);
    if (lane == 0) {
        l2 = box[srow * EL_SW + EL_HX - 2];
        l1 = box[srow * EL_SW + EL_HX - 1];
    }
    if (lane == 31) {
        r1 = box[srow * EL_SW + EL_HX + EL_TX];
        r2 = box[srow * EL_SW + EL_HX + EL_TX + 1];
    }
    e[0] = l2;
    e[1] = l1;
    e[2] = w.x;
    e[3] = w.y;
    e[4] = w.z;
    e[5] = w.w;
    e[6] = r1;
    e[7] = r2;
}

__device__ __forceinline__ float4 el_row4(const float* box, int srow, int lane)
{
    return *reinterpret_cast<const float4*>(&box[srow * EL_SW + EL_HX + 4 * lane]);
}

__device__ __forceinline__ bool el_in_m(int ix, int iz, int nx, int nz, int fs)
{
    return iz >= (fs ? 1 : 2) && iz < nz - 2 && ix >= 2 && ix < nx - 2;
}

// Store four values of one row: float4 when all four go out, else per point.
__device__ __forceinline__ void el_store_row(float* dst, const float* src, size_t off, int ixb,
                                             int iz, const ElGeom& g, const float u[4],
                                             bool in_place)
{
    bool all = true;
#pragma unroll
    for (int j = 0; j < 4; ++j) all &= el_in_m(ixb + j, iz, g.nx, g.nz, g.free_surface);
    if (all) {
        *reinterpret_cast<float4*>(dst + off) = make_float4(u[0], u[1], u[2], u[3]);
        return;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (ixb + j >= g.ldx) continue;
        if (el_in_m(ixb + j, iz, g.nx, g.nz, g.free_surface)) dst[off + j] = u[j];
        else if (!in_place) dst[off + j] = src[off + j];
    }
}

template <int WARPS, int RPW>
__global__ void __launch_bounds__(WARPS * 32)
    elastic_velocity_kernel(const __grid_constant__ ElMaps maps, const ElGeom g, const ElStep s)
{
    using T = ElTile<WARPS, RPW>;
    extern __shared__ __align__(128) float smem[];
    float* bxx = smem;             // sxx box
    float* bxz = smem + T::BOX;    // sxz box
    float* bzz = smem + 2 * T::BOX;  // szz box
    float* pt = smem + 3 * T::BOX;   // staged vx, vz, bx, bz, sponge
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::V_FLOATS);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int x0 = blockIdx.x * EL_TX, z0 = blockIdx.y * T::TZ, sh = blockIdx.z;
    if (tid == 0) {
        prefetch_tensormap(&maps.src);
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    // every lane takes part in the shuffles; lanes past the row pitch only skip
    // their loads and stores
    const int ixb = x0 + 4 * lane;
    const bool col_ok = ixb < g.ldx;
    const bool in_place = s.src == s.dst;
    const size_t so = (size_t)sh * 5 * s.plane, po = (size_t)sh * s.pstride;
    const float* vx_s = s.src + so + (size_t)EL_VX * s.plane;
    const float* vz_s = s.src + so + (size_t)EL_VZ * s.plane;
    float* vx_d = s.dst + so + (size_t)EL_VX * s.plane;
    float* vz_d = s.dst + so + (size_t)EL_VZ * s.plane;
    const float* bxp = s.bx + po;
    const float* bzp = s.bz + po;
    const int zr0 = z0 + warp * RPW;
    const float* f[5] = {vx_s, vz_s, bxp, bzp, g.sponge};
    // Early: the velocities were written by the velocity phase of the previous step
    // (two launches back) and the buoyancies and sponge are constant.  Each phase
    // releases its dependents only after its own wait, so this launch started after that
    // one had completed, and the stress phase still running only reads velocities.
    if (s.early) el_stage_pointwise<WARPS, RPW>(pt, f, 5, zr0, ixb, lane, warp, g);
    // the stresses are the previous launch's output: after the wait
    grid_dep_wait();
    grid_dep_launch();
    if (tid == 0) {
        mbar_expect_tx(bar, 3u * T::BOX * 4u);
        tma_load_3d(bxx, &maps.src, x0 - EL_HX, z0 - 2, 5 * sh + EL_SXX, bar);
        tma_load_3d(bxz, &maps.src, x0 - EL_HX, z0 - 2, 5 * sh + EL_SXZ, bar);
        tma_load_3d(bzz, &maps.src, x0 - EL_HX, z0 - 2, 5 * sh + EL_SZZ, bar);
    }
    if (!s.early) el_stage_pointwise<WARPS, RPW>(pt, f, 5, zr0, ixb, lane, warp, g);
    __syncthreads();
    // a CTA-uniform decision: a partial exit before the warp shuffles would be undefined
    if (__syncthreads_or(!mbar_wait_bounded(bar, 0))) {
        cp_async_wait_all();
        if (tid == 0) atomicOr(s.err, ERR_TMA_TIMEOUT);
        return;
    }
    cp_async_wait_all();  // this thread's staged fields (read only by this thread)
    int inj_ix = -1, inj_iz = -1;
    float inj = 0.0f;
    if (s.src_pos) {
        inj_ix = __ldg(s.src_pos + 2 * sh);
        inj_iz = __ldg(s.src_pos + 2 * sh + 1);
        inj = fmul(__ldg(s.wav + (size_t)sh * s.nt + s.n), g.dt);
    }
    const int sr = zr0 - (z0 - 2);  // box row of global row zr0
    // z windows: sxz rows z-2..z+1, szz rows z-1..z+2
    float4 xz0 = el_row4(bxz, sr - 2, lane), xz1 = el_row4(bxz, sr - 1, lane),
           xz2 = el_row4(bxz, sr, lane);
    float4 zz0 = el_row4(bzz, sr - 1, lane), zz1 = el_row4(bzz, sr, lane),
           zz2 = el_row4(bzz, sr + 1, lane);
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const int iz = zr0 + r;
        const float4 xz3 = el_row4(bxz, sr + r + 1, lane);
        const float4 zz3 = el_row4(bzz, sr + r + 2, lane);
        float exx[8], exz[8];
        el_xrow(bxx, sr + r, lane, exx);
        el_xrow(bxz, sr + r, lane, exz);
        if (iz < g.nz && col_ok) {
            const size_t off = (size_t)iz * g.ldx + ixb;
            const float4 vx4 = el_staged<WARPS, RPW>(pt, 0, warp, r, lane);
            float4 vz4 = el_staged<WARPS, RPW>(pt, 1, warp, r, lane);
            const float4 bx4 = el_staged<WARPS, RPW>(pt, 2, warp, r, lane);
            const float4 bz4 = el_staged<WARPS, RPW>(pt, 3, warp, r, lane);
            const float4 sp4 = g.sponge ? el_staged<WARPS, RPW>(pt, 4, warp, r, lane)
                                        : make_float4(1.f, 1.f, 1.f, 1.f);
            float ux[4], uz[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float vz_in = el_c(vz4, j);
                if (iz == inj_iz && ixb + j == inj_ix) vz_in = fadd(vz_in, inj);
                const float a = fmul(el_dfwd(exx[j + 1], exx[j + 2], exx[j + 3], exx[j + 4]), g.rdx);
                const float b = fmul(el_dbwd(el_c(xz0, j), el_c(xz1, j), el_c(xz2, j), el_c(xz3, j)),
                                     g.rdz);
                float vx = fadd(el_c(vx4, j), fmul(fmul(g.dt, el_c(bx4, j)), fadd(a, b)));
                const float e = fmul(el_dbwd(exz[j], exz[j + 1], exz[j + 2], exz[j + 3]), g.rdx);
                const float h = fmul(el_dfwd(el_c(zz0, j), el_c(zz1, j), el_c(zz2, j), el_c(zz3, j)),
                                     g.rdz);
                float vz = fadd(vz_in, fmul(fmul(g.dt, el_c(bz4, j)), fadd(e, h)));
                if (g.sponge) {
                    vx = fmul(vx, el_c(sp4, j));
                    vz = fmul(vz, el_c(sp4, j));
                }
                ux[j] = vx;
                uz[j] = vz;
            }
            // (the source term is only used on cells of M)
            el_store_row(vx_d, vx_s, off, ixb, iz, g, ux, in_place);
            el_store_row(vz_d, vz_s, off, ixb, iz, g, uz, in_place);
        }
        xz0 = xz1;
        xz1 = xz2;
        xz2 = xz3;
        zz0 = zz1;
        zz1 = zz2;
        zz2 = zz3;
    }
}

template <int WARPS, int RPW>
__global__ void __launch_bounds__(WARPS * 32)
    elastic_stress_kernel(const __grid_constant__ ElMaps maps, const ElGeom g, const ElStep s)
{
    using T = ElTile<WARPS, RPW>;
    extern __shared__ __align__(128) float smem[];
    float* bvx = smem;
    float* bvz = smem + T::BOX;
    float* pt = smem + 2 * T::BOX;  // staged lambda, mu, sxx, szz, sxz, sponge
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::S_FLOATS);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int x0 = blockIdx.x * EL_TX, z0 = blockIdx.y * T::TZ, sh = blockIdx.z;
    if (tid == 0) {
        prefetch_tensormap(&maps.dst);
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    const int ixb = x0 + 4 * lane;
    const bool col_ok = ixb < g.ldx;  // see the velocity phase
    const bool in_place = s.src == s.dst;
    const size_t so = (size_t)sh * 5 * s.plane, po = (size_t)sh * s.pstride;
    const float* sxx_s = s.src + so + (size_t)EL_SXX * s.plane;
    const float* szz_s = s.src + so + (size_t)EL_SZZ * s.plane;
    const float* sxz_s = s.src + so + (size_t)EL_SXZ * s.plane;
    float* sxx_d = s.dst + so + (size_t)EL_SXX * s.plane;
    float* szz_d = s.dst + so + (size_t)EL_SZZ * s.plane;
    float* sxz_d = s.dst + so + (size_t)EL_SXZ * s.plane;
    const float* lamp = s.lam + po;
    const float* mup = s.mu + po;
    const int zr0 = z0 + warp * RPW;
    const float* f[6] = {lamp, mup, sxx_s, szz_s, sxz_s, g.sponge};
    // Early: the stresses were written by the stress phase of the previous step (two
    // launches back), lambda, mu and the sponge are constant; the velocity phase still
    // running only reads stresses.
    if (s.early) el_stage_pointwise<WARPS, RPW>(pt, f, 6, zr0, ixb, lane, warp, g);
    // the new velocities are the previous launch's output: after the wait
    grid_dep_wait();
    grid_dep_launch();
    if (tid == 0) {
        mbar_expect_tx(bar, 2u * T::BOX * 4u);
        tma_load_3d(bvx, &maps.dst, x0 - EL_HX, z0 - 2, 5 * sh + EL_VX, bar);
        tma_load_3d(bvz, &maps.dst, x0 - EL_HX, z0 - 2, 5 * sh + EL_VZ, bar);
    }
    if (!s.early) el_stage_pointwise<WARPS, RPW>(pt, f, 6, zr0, ixb, lane, warp, g);
    __syncthreads();
    // a CTA-uniform decision: a partial exit before the warp shuffles would be undefined
    if (__syncthreads_or(!mbar_wait_bounded(bar, 0))) {
        cp_async_wait_all();
        if (tid == 0) atomicOr(s.err, ERR_TMA_TIMEOUT);
        return;
    }
    cp_async_wait_all();  // this thread's staged fields (read only by this thread)
    const int sr = zr0 - (z0 - 2);
    // z windows: vx rows z-1..z+2, vz rows z-2..z+1
    float4 x0w = el_row4(bvx, sr - 1, lane), x1w = el_row4(bvx, sr, lane),
           x2w = el_row4(bvx, sr + 1, lane);
    float4 z0w = el_row4(bvz, sr - 2, lane), z1w = el_row4(bvz, sr - 1, lane),
           z2w = el_row4(bvz, sr, lane);
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const int iz = zr0 + r;
        const float4 x3w = el_row4(bvx, sr + r + 2, lane);
        const float4 z3w = el_row4(bvz, sr + r + 1, lane);
        float evx[8], evz[8];
        el_xrow(bvx, sr + r, lane, evx);
        el_xrow(bvz, sr + r, lane, evz);
        if (iz < g.nz && col_ok) {
            const size_t off = (size_t)iz * g.ldx + ixb;
            const float4 lam4 = el_staged<WARPS, RPW>(pt, 0, warp, r, lane);
            const float4 mu4 = el_staged<WARPS, RPW>(pt, 1, warp, r, lane);
            const float4 sxx4 = el_staged<WARPS, RPW>(pt, 2, warp, r, lane);
            const float4 szz4 = el_staged<WARPS, RPW>(pt, 3, warp, r, lane);
            const float4 sxz4 = el_staged<WARPS, RPW>(pt, 4, warp, r, lane);
            const float4 sp4 = g.sponge ? el_staged<WARPS, RPW>(pt, 5, warp, r, lane)
                                        : make_float4(1.f, 1.f, 1.f, 1.f);
            float uxx[4], uzz[4], uxz[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int ix = ixb + j;
                const float l = el_c(lam4, j), m = el_c(mu4, j);
                const float ex = fmul(el_dbwd(evx[j], evx[j + 1], evx[j + 2], evx[j + 3]), g.rdx);
                uxx[j] = el_c(sxx4, j);
                uzz[j] = el_c(szz4, j);
                uxz[j] = el_c(sxz4, j);
                if (g.free_surface && iz == 0) {
                    // free-surface row (wave2d.c:198-211)
                    uzz[j] = 0.0f;
                    uxz[j] = 0.0f;
                    if (ix >= 2 && ix < g.nx - 2) {
                        const float num = fmul(fmul(4.0f, m), fadd(l, m));
                        const float den = fadd(fadd(l, fmul(2.0f, m)), 1e-8f);
                        uxx[j] = fmul(__fdiv_rn(num, den), ex);
                    }
                    continue;
                }
                if (!el_in_m(ix, iz, g.nx, g.nz, g.free_surface)) continue;
                const float ez = fmul(el_dbwd(el_c(z0w, j), el_c(z1w, j), el_c(z2w, j), el_c(z3w, j)),
                                      g.rdz);
                const float l2m = fadd(l, fmul(2.0f, m));
                float sxx = fadd(uxx[j], fmul(g.dt, fadd(fmul(l2m, ex), fmul(l, ez))));
                float szz = fadd(uzz[j], fmul(g.dt, fadd(fmul(l, ex), fmul(l2m, ez))));
                const float gx = fmul(el_dfwd(evz[j + 1], evz[j + 2], evz[j + 3], evz[j + 4]), g.rdx);
                const float hz = fmul(el_dfwd(el_c(x0w, j), el_c(x1w, j), el_c(x2w, j), el_c(x3w, j)),
                                      g.rdz);
                float sxz = fadd(uxz[j], fmul(fmul(g.dt, m), fadd(gx, hz)));
                if (g.sponge) {
                    const float sp = el_c(sp4, j);
                    sxx = fmul(sxx, sp);
                    szz = fmul(szz, sp);
                    sxz = fmul(sxz, sp);
                }
                uxx[j] = sxx;
                uzz[j] = szz;
                uxz[j] = sxz;
            }
            bool all = true;
#pragma unroll
            for (int j = 0; j < 4; ++j) all &= el_in_m(ixb + j, iz, g.nx, g.nz, g.free_surface);
            if (all) {
                *reinterpret_cast<float4*>(sxx_d + off) = make_float4(uxx[0], uxx[1], uxx[2], uxx[3]);
                *reinterpret_cast<float4*>(szz_d + off) = make_float4(uzz[0], uzz[1], uzz[2], uzz[3]);
                *reinterpret_cast<float4*>(sxz_d + off) = make_float4(uxz[0], uxz[1], uxz[2], uxz[3]);
            } else {
                const bool fs_row = g.free_surface && iz == 0;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int ix = ixb + j;
                    if (ix >= g.ldx) continue;
                    // written: M, the free-surface row inside the grid, and (out of
                    // place) every other cell as a copy
                    const bool w = el_in_m(ix, iz, g.nx, g.nz, g.free_surface) ||
                                   (fs_row && ix < g.nx) || !in_place;
                    if (!w) continue;
                    sxx_d[off + j] = uxx[j];
                    szz_d[off + j] = uzz[j];
                    sxz_d[off + j] = uxz[j];
                }
            }
        }
        if (s.trace && iz == s.rec_iz && col_ok) {
            // receivers on this row: the strain the stress update itself uses (ez)
            float* tr = s.trace + (size_t)sh * s.trace_stride;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int ix = ixb + j;
                if (ix >= g.nx) continue;
                const int k0 = __ldg(s.rec_ptr + ix), k1 = __ldg(s.rec_ptr + ix + 1);
                if (k0 == k1) continue;
                const float d = fmul(
                    el_dbwd(el_c(z0w, j), el_c(z1w, j), el_c(z2w, j), el_c(z3w, j)), g.rdz);
                for (int k = k0; k < k1; ++k) tr[__ldg(s.rec_list + k)] = d;
            }
        }
        x0w = x1w;
        x1w = x2w;
        x2w = x3w;
        z0w = z1w;
        z1w = z2w;
        z2w = z3w;
    }
}

constexpr int EL_WARPS = 4, EL_RPW = 2;  // default tile: 4 warps x 2 rows (128 x 8)

// Tile shapes the step kernels are built for (warps per CTA x rows per warp).
inline bool el_tile_supported(int warps, int rpw)
{
    return (warps == 4 && (rpw == 4 || rpw == 2)) || (warps == 8 && (rpw == 2 || rpw == 1));
}

// The 3D tensor map of the 5-plane states of n_shots shots stored one after another,
// with boxes of tile height tz (+ 4 halo rows).
inline int make_el_state_map(CUtensorMap* m, const float* base, int nx, int nz, int ldx,
                             size_t plane, int n_shots = 1, int tz = EL_WARPS * EL_RPW)
{
    return make_tensor_map_3d(m, base, nx, nz, 5 * n_shots, ldx, plane, EL_SW, tz + 4);
}

// One launch with an optional programmatic-dependent attribute (the kernel runs its
// set-up while the previous kernel of the stream finishes, then waits for it).
template <typename... KArgs, typename... Args>
inline cudaError_t el_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
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

template <int WARPS, int RPW>
cudaError_t launch_elastic_step_t(const ElGeom& g, const ElMaps& maps, const ElStep& s,
                                  cudaStream_t st, int n_shots, int pdl)
{
    using T = ElTile<WARPS, RPW>;
    const int vbytes = T::V_FLOATS * 4 + 128, sbytes = T::S_FLOATS * 4 + 128;
    cudaError_t e = set_smem_once<elastic_velocity_kernel<WARPS, RPW>>(vbytes);
    if (e == cudaSuccess) e = set_smem_once<elastic_stress_kernel<WARPS, RPW>>(sbytes);
    if (e != cudaSuccess) return e;
    dim3 grid((g.nx + EL_TX - 1) / EL_TX, (g.nz + T::TZ - 1) / T::TZ, n_shots);
    e = el_launch(elastic_velocity_kernel<WARPS, RPW>, grid, dim3(WARPS * 32), vbytes, st, pdl,
                  maps, g, s);
    if (e != cudaSuccess) return e;
    ElStep s2 = s;
    s2.src_pos = nullptr;
    s2.early = 1;  // after the velocity kernel, which releases it only after its own wait
    // the stress phase always follows the velocity kernel directly
    return el_launch(elastic_stress_kernel<WARPS, RPW>, grid, dim3(WARPS * 32), sbytes, st, 1,
                     maps, g, s2);
}

// Velocity then stress phase of one step of n_shots shots (src -> dst; src == dst
// updates in place), on tiles of `warps` x `rpw` rows; the maps' box height must be
// warps * rpw + 4.  pdl: the velocity kernel is a programmatic dependent of the
// stream's previous operation, which must then be one of this file's or the tiled
// adjoint's kernels (each waits for its predecessor before any global access).
inline cudaError_t launch_elastic_step(const ElGeom& g, const ElMaps& maps, const ElStep& s,
                                       cudaStream_t st, int n_shots = 1, int warps = EL_WARPS,
                                       int rpw = EL_RPW, int pdl = 0)
{
    if (warps == 4 && rpw == 4) return launch_elastic_step_t<4, 4>(g, maps, s, st, n_shots, pdl);
    if (warps == 4 && rpw == 2) return launch_elastic_step_t<4, 2>(g, maps, s, st, n_shots, pdl);
    if (warps == 8 && rpw == 2) return launch_elastic_step_t<8, 2>(g, maps, s, st, n_shots, pdl);
    if (warps == 8 && rpw == 1) return launch_elastic_step_t<8, 1>(g, maps, s, st, n_shots, pdl);
    return cudaErrorInvalidValue;
}

}  // namespace w2d
