// batch_kernels.cuh -- multi-shot RTM kernels: one launch per phase step over all
// active shots (grid form), or a persistent kernel over a (step, shot, tile) work
// queue (queue form).
//
// Grid form (acoustic_batch_step_kernel): every launch advances each active shot
// by one phase step, one CTA per (shot, tile), launches chained as programmatic
// dependents.  Queue form (acoustic_batch_kernel), described below.
//
// Many shots of different grid sizes and lengths advance together.  One launch
// (a "chunk") covers S consecutive phase steps of every active shot; a shot's
// phase step k is forward step k for k < nt and backward step 2*nt-1-k after
// that, so a shot runs its whole forward-then-backward migration as one sequence
// of 2*nt tile-steps.  Work items are numbered step-major (local step j, then
// shot, then tile) and handed out with one atomic counter; a CTA processes an
// item as soon as the 3 x 3 neighbouring tiles of the same shot have completed
// phase step k-1 (per-tile counters with release/acquire), so steps overlap
// across the grid instead of meeting at a kernel boundary.  Because items are
// taken in increasing order, every item an item waits for was taken earlier by
// a running CTA: the waits cannot deadlock.  Every wait is bounded; on timeout
// the CTA raises an error bit that makes all CTAs stop.
//
// Why the dependency suffices: the plane written at step k (p_next) was p_prev
// at step k-1 (read only by the same tile) and p_curr at step k-2 (read by the
// tile and its neighbours through the halo); all of those reads belong to items
// the 3 x 3 neighbourhood completed before it finished step k-1.
#pragma once

#include "acoustic_kernels.cuh"

namespace w2d {

// Device-resident descriptor of one shot of a batch.
struct BShot {
    AcGeom g;           // g.shot points at shot_ints of this descriptor
    int shot_ints[5];   // src_ix, src_iz, rec_iz, n_rec, rec_c0 (AcGeom::shot)
    int nt, interval, n_rec;
    int tiles_x, tiles_z, ntiles;
    int k_end;          // 2 * nt phase steps
    int k0;             // phase step at which the current chunk starts
    int maps_index;     // index into the BMaps table
    int pad_;
    float* wave[6];     // forward triple, backward triple
    float* snaps;       // ceil(nt/interval) snapshot planes
    float* illum;
    float* image;
    const float* wavelet;
    const float* data;
    float dt2_inj, img_dt;
    unsigned* done;     // per tile: phase steps completed
    int mode;           // 0: migration (forward + backward); 1: forward modelling only
    float* traces;      // mode 1: (nt, n_rec) receiver samples
};

// TMA descriptors of one shot (global memory; CUtensorMap carries its own alignment).
struct BMaps {
    CUtensorMap curr[6];
    CUtensorMap prev[6];
    CUtensorMap vel[2];
};

struct BatchArgs {
    BShot* shots;
    const BMaps* maps;
    const int* active;       // indices of active shots
    const int* tile_prefix;  // prefix sums of their tile counts (n_active + 1)
    const int* n_active;     // device scalar
    int S;                   // phase steps per launch
    unsigned* head;          // work counter (zeroed before each launch)
    unsigned* err;
};

__device__ __forceinline__ bool wait_counter(const unsigned* p, unsigned target, unsigned* err)
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

// The AcStep and TMA-descriptor indices of phase step k of one shot.
__device__ __forceinline__ void batch_phase(const BShot* sh, int k, unsigned* err, AcStep& s,
                                            int& ci, int& pi, int& vi)
{
    const int nt = sh->nt, interval = sh->interval;
    s.snap_out = nullptr;
    s.illum = nullptr;
    s.rec_out = nullptr;
    s.snap_in = nullptr;
    s.image = nullptr;
    s.img_dt = sh->img_dt;
    s.inj_w = nullptr;
    s.inj_data = nullptr;
    s.dt2_inj = sh->dt2_inj;
    s.err = err;
    if (k < nt) {
        const int it = k;
        pi = it % 3;
        ci = (it + 1) % 3;
        s.p_next = sh->wave[(it + 2) % 3];
        vi = 0;
        if (it + 1 < nt) s.inj_w = sh->wavelet + it + 1;
        if (sh->mode == 1) {
            s.rec_out = sh->traces + (size_t)it * sh->n_rec;
        } else if (it % interval == 0) {
            s.snap_out = sh->snaps + (size_t)(it / interval) * sh->g.ldx * sh->g.nz;
            s.illum = sh->illum;
        }
    } else {
        const int m = k - nt, it = nt - 1 - m;
        pi = 3 + m % 3;
        ci = 3 + (m + 1) % 3;
        s.p_next = sh->wave[3 + (m + 2) % 3];
        vi = 1;
        if (it >= 1 && sh->n_rec > 0) s.inj_data = sh->data + (size_t)(it - 1) * sh->n_rec;
        if (it % interval == 0) {
            s.snap_in = sh->snaps + (size_t)(it / interval) * sh->g.ldx * sh->g.nz;
            s.image = sh->image;
        }
    }
}

// Registers capped so that four 256-thread (or eight 128-thread) CTAs fit per SM.
template <int WARPS, int RPW>
__global__ void __launch_bounds__(WARPS * 32, RPW == 4 ? 1024 / (WARPS * 32) : 1)
    acoustic_batch_kernel(const BatchArgs a)
{
    using T = AcTile<WARPS, RPW, SPONGE_LUT>;
    extern __shared__ __align__(128) float smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::FLOATS);
    __shared__ int s_item;
    __shared__ int s_ok;
    const int tid = threadIdx.x;
    const int n_act = *a.n_active;
    if (n_act <= 0) return;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        s_item = (int)atomicAdd(a.head, 1u);
    }
    const int T_all = a.tile_prefix[n_act];
    const long long total = (long long)a.S * T_all;
    unsigned phase = 0;
    // The next queue index is taken while the current item is processed, which
    // hides the atomic's round trip.  Items are still processed in increasing
    // order per CTA, so every awaited item is held by a CTA that reaches it.
    int next = 0;
    for (;;) {
        if (tid == 0) s_ok = (*reinterpret_cast<volatile unsigned*>(a.err) & ERR_ABORT) ? 0 : 1;
        __syncthreads();
        const long long item = s_item;
        if (item >= total || !s_ok) break;
        if (tid == 0) next = (int)atomicAdd(a.head, 1u);
        const int j = (int)(item / T_all);
        const int r = (int)(item - (long long)j * T_all);
        int lo = 0, hi = n_act - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(a.tile_prefix + mid) <= r) lo = mid;
            else hi = mid - 1;
        }
        BShot* sh = a.shots + __ldg(a.active + lo);
        const int t = r - __ldg(a.tile_prefix + lo);
        const int k = sh->k0 + j;
        if (k >= sh->k_end) {
            __syncthreads();
            if (tid == 0) s_item = next;
            continue;
        }
        const int tiles_x = sh->tiles_x, tiles_z = sh->tiles_z;
        const int tx = t % tiles_x, tz = t / tiles_x;
        if (tid < 9 && k > 0) {
            const int nx_ = tx + tid % 3 - 1, nz_ = tz + tid / 3 - 1;
            if (nx_ >= 0 && nx_ < tiles_x && nz_ >= 0 && nz_ < tiles_z)
                if (!wait_counter(sh->done + nz_ * tiles_x + nx_, (unsigned)k, a.err)) s_ok = 0;
        }
        __syncthreads();
        if (!s_ok) break;

        // the tile-step of phase step k
        const BMaps* mp = a.maps + sh->maps_index;
        AcStep s;
        int ci, pi, vi;
        batch_phase(sh, k, a.err, s, ci, pi, vi);
        const int x0 = tx * AC_TX, z0 = tz * T::TZ;
        if (tid == 0) {
            fence_proxy_async_global();
            fence_proxy_async_shared();
            mbar_expect_tx(bar, T::TX_BYTES);
            tma_load_2d(smem, &mp->curr[ci], x0 - AC_HX, z0 - 2, bar);
            tma_load_2d(smem + T::C_FLOATS, &mp->prev[pi], x0, z0, bar);
            tma_load_2d(smem + T::C_FLOATS + T::P_FLOATS, &mp->vel[vi], x0, z0, bar);
        }
        const bool got = mbar_wait_bounded(bar, phase);
        if (__syncthreads_or(!got)) {
            if (tid == 0) atomicOr(a.err, ERR_TMA_TIMEOUT | ERR_ABORT);
            break;
        }
        phase ^= 1u;
        ac_tile_body<WARPS, RPW, SPONGE_LUT>(smem, sh->g, s, x0, z0);
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            st_release_u32(sh->done + t, (unsigned)(k + 1));
            s_item = next;
        }
    }
}

struct BatchStepArgs {
    BShot* shots;
    const BMaps* maps;
    const int2* items;       // per CTA: {shot slot, tile}, the active shots' tiles in order
    int n_active;
    int max_shots;           // size of the shot table (range check of active entries)
    int j;                   // phase step k0 + j of every active shot
    unsigned* err;
};

// Grid form: one launch advances every active shot by one phase step, one CTA
// per (shot, tile); the launches after the first of a replay are programmatic
// dependents of the one before, so a launch's set-up overlaps the previous one's
// last wave (the first waits normally for the active-list copies and admission
// events before it).  No waits between CTAs.  4-row tiles are held to 64 registers
// so that 8 CTAs of 4 warps fit an SM (the shared memory of a 128 x 16 tile allows it).
template <int WARPS, int RPW>
__global__ void __launch_bounds__(WARPS * 32, RPW <= 4 ? 1024 / (WARPS * 32) : 1)
    acoustic_batch_step_kernel(const BatchStepArgs a)
{
    using T = AcTile<WARPS, RPW, SPONGE_LUT>;
    extern __shared__ __align__(128) float smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::FLOATS);
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    // The work table and the shots' descriptors do not change during a replay (they are
    // written before its first launch, which waits for the stream normally; the progress
    // k0 moves only in the progress kernel that ends a replay): read them while the
    // previous launch drains.
    const int2 it = __ldg(a.items + blockIdx.x);
    const int slot = it.x, t = it.y;
    if (slot < 0 || slot >= a.max_shots || t < 0) {  // inconsistent work table: skip, report
        grid_dep_wait();
        if (tid == 0) atomicOr(a.err, ERR_BAD_ITEM);
        return;
    }
    const BShot* sh = a.shots + slot;
    const int ntiles = sh->ntiles, k_end = sh->k_end;
    const int k = sh->k0 + a.j;
    if (t >= ntiles || k >= k_end) return;  // an exited CTA counts as released
    AcStep s;
    int ci, pi, vi;
    batch_phase(sh, k, a.err, s, ci, pi, vi);
    const BMaps* mp = a.maps + sh->maps_index;
    const int x0 = (t % sh->tiles_x) * AC_TX, z0 = (t / sh->tiles_x) * T::TZ;
    if (tid == 0) {
        // p_prev is the output of the launch before the previous one (or older), the model
        // older still.  Every launch releases its dependents only after its own wait, so
        // this one started after that launch had completed: these boxes go out now.
        mbar_expect_tx(bar, T::TX_BYTES);
        tma_load_2d(smem + T::C_FLOATS, &mp->prev[pi], x0, z0, bar);
        tma_load_2d(smem + T::C_FLOATS + T::P_FLOATS, &mp->vel[vi], x0, z0, bar);
    }
    // p_curr is the previous launch's output: after the wait
    grid_dep_wait();
    grid_dep_launch();
    if (tid == 0) tma_load_2d(smem, &mp->curr[ci], x0 - AC_HX, z0 - 2, bar);
    if ((s.snap_in || s.image || s.illum) && tid < 3 * T::TZ) {
        // the fused pointwise work reads these planes from HBM after the stencil (a
        // batch's planes do not stay in L2): bring the tile's rows into L2 beside the
        // boxes, one row per thread, within the row pitch
        const int r = tid % T::TZ, f = tid / T::TZ;
        const float* src = f == 0 ? s.snap_in : (f == 1 ? s.image : s.illum);
        const int ldx = sh->g.ldx;
        if (src && z0 + r < sh->g.nz)
            prefetch_l2_bulk(src + (size_t)(z0 + r) * ldx + x0,
                             (uint32_t)min(AC_TX, ldx - x0) * 4u);
    }
    __syncthreads();
    // a CTA-uniform decision: a partial exit before the warp shuffles would be undefined
    if (__syncthreads_or(!mbar_wait_bounded(bar, 0))) {
        if (tid == 0) atomicOr(a.err, ERR_TMA_TIMEOUT);
        return;
    }
    ac_tile_body<WARPS, RPW, SPONGE_LUT>(smem, sh->g, s, x0, z0);
}

// After each chunk: every active shot moves S phase steps on.
static __global__ void batch_advance_kernel(BShot* shots, const int* active, const int* n_active,
                                            int S)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *n_active) shots[active[i]].k0 += S;
}

}  // namespace w2d
