// engine.cu -- whole-loop acoustic engine: device-resident wavefields, fused
// step launches for forward modelling, backward propagation with imaging, and
// forward+backward migration of a shot with full snapshot storage or
// checkpointed recomputation.  Also the reference-compatible per-step
// acoustic_2d_step / correlate_imaging_condition entry points.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "acoustic_step2.cuh"
#include "adjoint_kernels.cuh"
#include "small_kernels.cuh"
#include "w2d_common.cuh"
#include "wave2d_cuda.h"

namespace w2d {

float cerjan_value(int d, float alpha);

// ---- tile-shape dispatch ------------------------------------------------------
struct TileShape {
    int warps, rpw;
    int tz() const { return warps * rpw; }
};

static bool tile_supported(int warps, int rpw)
{
    return (warps == 8 && rpw == 4) || (warps == 4 && rpw == 8) || (warps == 8 && rpw == 8) ||
           (warps == 4 && rpw == 4);
}

// How the step kernels are launched: one CTA per tile or persistent CTAs over a
// tile counter, each optionally as a programmatic dependent of the previous step.
struct LaunchMode {
    int persistent = 0, pdl = 0;
    unsigned* counter = nullptr;  // persistent: tile counter
    unsigned* base = nullptr;     //   and the host copy of its launch base
};

template <int W, int R, int SP>
static cudaError_t launch_one(const LaunchMode& lm, const AcMaps& m, const AcGeom& g,
                              const AcStep& s, cudaStream_t st)
{
    if (lm.persistent)
        return launch_acoustic_persistent<W, R, SP>(m, g, s, st, lm.pdl, lm.counter, lm.base);
    return launch_acoustic_step<W, R, SP>(m, g, s, st, lm.pdl);
}

template <int W, int R>
static cudaError_t launch_sp(int sponge_mode, const LaunchMode& lm, const AcMaps& m,
                             const AcGeom& g, const AcStep& s, cudaStream_t st)
{
    if (sponge_mode == SPONGE_LUT) return launch_one<W, R, SPONGE_LUT>(lm, m, g, s, st);
    if (sponge_mode == SPONGE_ARRAY) return launch_one<W, R, SPONGE_ARRAY>(lm, m, g, s, st);
    return launch_one<W, R, SPONGE_NONE>(lm, m, g, s, st);
}

static cudaError_t launch_step(TileShape t, int sponge_mode, const LaunchMode& lm,
                               const AcMaps& m, const AcGeom& g, const AcStep& s, cudaStream_t st)
{
    if (t.warps == 4 && t.rpw == 8) return launch_sp<4, 8>(sponge_mode, lm, m, g, s, st);
    if (t.warps == 8 && t.rpw == 8) return launch_sp<8, 8>(sponge_mode, lm, m, g, s, st);
    if (t.warps == 4 && t.rpw == 4) return launch_sp<4, 4>(sponge_mode, lm, m, g, s, st);
    return launch_sp<8, 4>(sponge_mode, lm, m, g, s, st);
}

// ---- device buffer helper -------------------------------------------------------
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;  // elements
    int ensure(size_t n)
    {
        if (n <= cap) return W2D_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (n == 0) return W2D_OK;
        cudaError_t e = cudaMalloc(&p, n * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error(std::string("device allocation failed: ") + cudaGetErrorString(e));
            return W2D_ENOMEM;
        }
        cap = n;
        return W2D_OK;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

}  // namespace w2d

using namespace w2d;

struct w2d_engine {
    int device = 0;  // CUDA device current at creation: every call on the handle runs there
    int nx = 0, nz = 0, ldx = 0, fs = 1;
    float dx = 0, dz = 0, dt = 0;  // dt as the float the reference C code receives
    double dt_d = 0;               // dt as the Python float the reference drivers hold
    float inv_dx2 = 0, inv_dz2 = 0, dt2 = 0;
    size_t plane = 0;  // floats per pitched field
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    TileShape tile{4, 4};
    int l2_hints = 0;
    int persistent = 0, pdl = 1;  // step launch mode (measured fastest: one CTA per tile + PDL)
    int fwi_seg = 0;  // differentiable path: steps per checkpoint segment (0: sqrt(3 nt))
    int adj_cells = 0;  // differentiable path: the per-cell adjoint kernel instead of the vectorised one
    bool chain = false;  // the last operation on the stream is a step kernel launched by step()
    bool last_step1 = false;  // ... and it was the one-step kernel (one CTA per tile)
    DevBuf<unsigned> tile_counter;
    unsigned counter_base = 0;

    int n_sponge = 0;
    DevBuf<float> sponge_lut, sponge_arr;
    bool use_lut = false, use_arr = false;

    // 10 physical wave planes: the forward pass's three logical planes (roles by
    // step, the reference's rotation) plus two spares, the same for the backward pass.
    // A two-step launch writes its results into the spares and renames: perm maps the
    // six logical planes (0..2 forward, 3..5 backward) to physical ones.
    DevBuf<float> waves;
    int perm[6] = {0, 1, 2, 5, 6, 7};
    int spare[2][2] = {{3, 4}, {8, 9}};
    // two time steps per launch where the loop allows (grid launch mode): 0 off (the
    // default: measured slower than one step per launch on the sponge-framed production
    // grids), else the tile's rows per warp (2..4); map2_rpw: the shape the two-step
    // maps were made for
    int two_step = 0, map2_rpw = -1;
    // TMA descriptors per physical plane for the current tile height: each wave plane
    // as p_curr (halo box) and as p_prev, each v^2 dt^2 slot, and the per-cell sponge;
    // and the two-step kernel's boxes
    CUtensorMap map_curr[10], map_prev[10], map_vel[2], map_sponge;
    CUtensorMap map2_curr[10], map2_prev[10], map2_vel[2], map2_sponge;
    int tm_tz = -1;
    DevBuf<float> v2dt2;  // 2 planes (slot 0 forward model, slot 1 backward model)
    bool vel_set[2] = {false, false};
    DevBuf<float> staging;  // one plane, pitched upload area

    DevBuf<int> shot;  // {src_ix, src_iz, rec_iz}
    int h_shot[3] = {-1, -1, -1};  // host copy of the same
    DevBuf<int> rec_ptr, rec_list;
    DevBuf<float> wavelet, data, rec_out;
    DevBuf<float> snaps, ckpt;
    DevBuf<float> image, illum, stack_img, stack_ill;
    DevBuf<unsigned> err;
    DevBuf<unsigned> scratch;  // small reductions (post-stack maximum)
    unsigned long long budget = 0;
    // inputs of the pass being run (engine buffers or a staged slot)
    const float* cur_w = nullptr;
    const float* cur_data = nullptr;
    // staged shot inputs (device-resident before a timed region)
    std::vector<DevBuf<float>> st_w, st_d;
    std::vector<int> st_nt, st_nrec;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    // receiver data of a migration uploads on its own stream beside the forward pass
    // (which does not read it); the backward pass waits for data_ready
    cudaStream_t up = nullptr;
    cudaEvent_t up_after = nullptr, data_ready = nullptr;
    // end of a migration's forward pass: its illumination is final and downloads on the
    // upload stream while the backward pass runs
    cudaEvent_t fwd_done = nullptr;
    bool data_pending = false;

    // stats of the last call
    int last_storage = 0;
    long long last_launches = 0, last_recompute = 0;
    float last_ms = 0.f;

    struct w2d_fwi_state* fwi = nullptr;  // differentiable-path state (checkpoints, gradient)

    // A migration's forward pass and backward pass, each captured once as a CUDA graph
    // and replayed for every later shot with the same launch sequence (the key: sizes,
    // modes, tile and every buffer address the launches hold).  One graph launch per
    // pass instead of one host launch per step: no host stall can drain the stream
    // between steps.  Default launch mode only (the two-step and counter modes carry
    // host-side state from launch to launch).
    struct PassGraph {
        std::vector<uintptr_t> key;
        cudaGraphExec_t exec = nullptr;
        long long launches = 0, recompute = 0;
        void reset()
        {
            if (exec) cudaGraphExecDestroy(exec);
            exec = nullptr;
            key.clear();
        }
    };
    PassGraph g_fwd, g_bwd;    // a migration's two passes
    PassGraph g_model, g_bcorr;  // forward modelling, backward propagation with imaging
    int use_graphs = 1;

    float* wave(int i) { return waves.p + (size_t)perm[i] * plane; }  // logical plane i
    float* phys(int k) { return waves.p + (size_t)k * plane; }
    const CUtensorMap& mcurr(int i) const { return map_curr[perm[i]]; }
    const CUtensorMap& mprev(int i) const { return map_prev[perm[i]]; }
};

namespace {

int upload_field(w2d_engine* e, float* dst_pitched, const float* host)
{
    W2D_CUDA_TRY(cudaMemcpy2DAsync(dst_pitched, (size_t)e->ldx * 4, host, (size_t)e->nx * 4,
                                   (size_t)e->nx * 4, e->nz, cudaMemcpyHostToDevice, e->stream));
    return W2D_OK;
}

// A contiguous (nz, nx) field that may be host memory or device memory of the engine's
// device (a device-resident model): into a pitched plane.
int upload_field_any(w2d_engine* e, float* dst_pitched, const float* src)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, src) != cudaSuccess) {
        cudaGetLastError();  // not a CUDA pointer: pageable host memory
        return upload_field(e, dst_pitched, src);
    }
    if (a.type == cudaMemoryTypeDevice && a.device != e->device) {
        set_error("velocity model is on device " + std::to_string(a.device) + ", the engine on " +
                  std::to_string(e->device));
        return W2D_EINVAL;
    }
    const cudaMemcpyKind kind = (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
                                    ? cudaMemcpyDeviceToDevice
                                    : cudaMemcpyHostToDevice;
    W2D_CUDA_TRY(cudaMemcpy2DAsync(dst_pitched, (size_t)e->ldx * 4, src, (size_t)e->nx * 4,
                                   (size_t)e->nx * 4, e->nz, kind, e->stream));
    return W2D_OK;
}

int download_field(w2d_engine* e, float* host, const float* src_pitched)
{
    W2D_CUDA_TRY(cudaMemcpy2DAsync(host, (size_t)e->nx * 4, src_pitched, (size_t)e->ldx * 4,
                                   (size_t)e->nx * 4, e->nz, cudaMemcpyDeviceToHost, e->stream));
    return W2D_OK;
}

// The two-step kernel's maps for the current rows-per-warp setting.
int ensure_step2_maps(w2d_engine* e)
{
    int rc;
    const int rpw = e->two_step ? e->two_step : AC2_R2;
    if (e->map2_rpw == rpw) return W2D_OK;
    const int cr = ac2_curr_rows(rpw), rr = ac2_ring_rows(rpw);
    for (int k = 0; k < 10; ++k)
        if ((rc = make_tensor_map_2d(&e->map2_curr[k], e->phys(k), e->nx, e->nz, e->ldx, AC2_W,
                                     cr)) ||
            (rc = make_tensor_map_2d(&e->map2_prev[k], e->phys(k), e->nx, e->nz, e->ldx, AC2_W,
                                     rr)))
            return rc;
    for (int i = 0; i < 2; ++i)
        if ((rc = make_tensor_map_2d(&e->map2_vel[i], e->v2dt2.p + (size_t)i * e->plane, e->nx,
                                     e->nz, e->ldx, AC2_W, rr)))
            return rc;
    e->map2_sponge = e->map2_vel[0];
    if (e->use_arr && (rc = make_tensor_map_2d(&e->map2_sponge, e->sponge_arr.p, e->nx, e->nz,
                                               e->ldx, AC2_W, rr)))
        return rc;
    e->map2_rpw = rpw;
    return W2D_OK;
}

int ensure_tensor_maps(w2d_engine* e)
{
    const int tz = e->tile.tz();
    if (e->tm_tz == tz) return ensure_step2_maps(e);
    int rc;
    for (int k = 0; k < 10; ++k) {
        if ((rc = make_tensor_map_2d(&e->map_curr[k], e->phys(k), e->nx, e->nz, e->ldx, AC_SW,
                                     tz + 4)) ||
            (rc = make_tensor_map_2d(&e->map_prev[k], e->phys(k), e->nx, e->nz, e->ldx, AC_TX, tz)))
            return rc;
    }
    for (int i = 0; i < 2; ++i)
        if ((rc = make_tensor_map_2d(&e->map_vel[i], e->v2dt2.p + (size_t)i * e->plane, e->nx,
                                     e->nz, e->ldx, AC_TX, tz)))
            return rc;
    e->map_sponge = e->map_vel[0];
    if (e->use_arr && (rc = make_tensor_map_2d(&e->map_sponge, e->sponge_arr.p, e->nx, e->nz,
                                               e->ldx, AC_TX, tz)))
        return rc;
    e->tm_tz = tz;
    return ensure_step2_maps(e);
}

int sponge_mode(const w2d_engine* e)
{
    return e->use_arr ? SPONGE_ARRAY : (e->use_lut ? SPONGE_LUT : SPONGE_NONE);
}

// One fused step launch: curr/prev are wave-plane indices, slot the velocity model.
int step(w2d_engine* e, int curr, int prev, int slot, const AcGeom& g, const AcStep& s)
{
    AcMaps m;
    m.curr = e->mcurr(curr);
    m.prev = e->mprev(prev);
    m.vel = e->map_vel[slot];
    m.sponge = e->map_sponge;
    LaunchMode lm;
    lm.persistent = e->persistent;
    // a programmatic dependent only of a step kernel: after any other operation
    // (copies, memsets, set-up kernels) the launch waits for the stream normally
    lm.pdl = e->pdl && e->chain;
    lm.counter = e->tile_counter.p;
    lm.base = &e->counter_base;
    // early reads of p_prev and the model: safe after a one-step kernel of the chain
    // (it releases this launch only after its own wait) or without a dependency at all;
    // not after a two-step launch, which wrote p_prev itself
    AcStep se = s;
    se.early = (!lm.pdl || e->last_step1) ? 1 : 0;
    e->chain = false;
    W2D_CUDA_TRY(launch_step(e->tile, sponge_mode(e), lm, m, g, se, e->stream));
    e->chain = true;
    e->last_step1 = !e->persistent;
    e->last_launches++;
    return W2D_OK;
}

// Two steps in one launch: logical planes curr / prev / next of the first step (next:
// the stale buffer the reference would write); results into the pass's spares, which
// then take over the logical roles (p_{n+1} -> next, p_{n+2} -> prev).  pass: 0
// forward, 1 backward.
int step2(w2d_engine* e, int pass, int curr, int prev, int next, int slot, const AcGeom& g,
          Ac2Step& p)
{
    int* sp = e->spare[pass];
    Ac2Maps m;
    m.curr = e->map2_curr[e->perm[curr]];
    m.prev = e->map2_prev[e->perm[prev]];
    m.vel = e->map2_vel[slot];
    m.sponge = e->map2_sponge;
    m.stale = e->map2_prev[e->perm[next]];
    p.src_ix = e->h_shot[0];
    p.src_iz = e->h_shot[1];
    p.rec_iz = e->h_shot[2];
    p.out1 = e->phys(sp[0]);
    p.out2 = e->phys(sp[1]);
    const int pdl = e->pdl && e->chain;
    e->chain = false;
    W2D_CUDA_TRY(launch_acoustic_step2(e->two_step, sponge_mode(e), m, g, p, e->stream, pdl));
    e->chain = true;
    e->last_step1 = false;  // it wrote the next step's p_prev itself
    e->last_launches++;
    const int old_next = e->perm[next], old_prev = e->perm[prev];
    e->perm[next] = sp[0];
    e->perm[prev] = sp[1];
    sp[0] = old_next;
    sp[1] = old_prev;
    return W2D_OK;
}

// Zero the three logical planes of a pass (0 forward, 1 backward).
int zero_pass(w2d_engine* e, int pass)
{
    for (int i = 0; i < 3; ++i)
        W2D_CUDA_TRY(cudaMemsetAsync(e->wave(3 * pass + i), 0, e->plane * 4, e->stream));
    return W2D_OK;
}

AcGeom geom(w2d_engine* e)
{
    AcGeom g;
    g.nx = e->nx;
    g.nz = e->nz;
    g.ldx = e->ldx;
    g.inv_dx2 = e->inv_dx2;
    g.inv_dz2 = e->inv_dz2;
    g.free_surface = e->fs;
    g.n_sponge = e->n_sponge;
    g.sponge_lut = e->use_lut ? e->sponge_lut.p : nullptr;
    g.rec_ptr = e->rec_ptr.p;
    g.rec_list = e->rec_list.p;
    g.shot = e->shot.p;
    g.l2_hints = e->l2_hints;
    return g;
}

// Receivers: CSR by column, receivers of a column in index order.
int set_shot(w2d_engine* e, int src_ix, int src_iz, const int* rec_ix, int n_rec, int rec_iz)
{
    W2D_CHECK_ARG(n_rec >= 0, "n_rec < 0");
    W2D_CHECK_ARG(n_rec == 0 || rec_ix, "rec_ix is NULL");
    W2D_CHECK_ARG(rec_iz >= 0 && rec_iz < e->nz, "receiver_iz out of range");
    std::vector<int> ptr(e->nx + 1, 0), list(std::max(n_rec, 1));
    for (int r = 0; r < n_rec; ++r) {
        W2D_CHECK_ARG(rec_ix[r] >= 0 && rec_ix[r] < e->nx, "receiver_ix out of range");
        ptr[rec_ix[r] + 1]++;
    }
    for (int i = 0; i < e->nx; ++i) ptr[i + 1] += ptr[i];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int r = 0; r < n_rec; ++r) list[fill[rec_ix[r]]++] = r;
    int rc;
    if ((rc = e->rec_ptr.ensure(e->nx + 1)) || (rc = e->rec_list.ensure(list.size())) ||
        (rc = e->shot.ensure(5)))
        return rc;
    int sh[5] = {src_ix, src_iz, rec_iz, n_rec, receivers_consecutive_c0(rec_ix, n_rec)};
    e->h_shot[0] = src_ix;
    e->h_shot[1] = src_iz;
    e->h_shot[2] = rec_iz;
    W2D_CUDA_TRY(cudaMemcpyAsync(e->rec_ptr.p, ptr.data(), ptr.size() * 4, cudaMemcpyHostToDevice,
                                 e->stream));
    W2D_CUDA_TRY(cudaMemcpyAsync(e->rec_list.p, list.data(), list.size() * 4,
                                 cudaMemcpyHostToDevice, e->stream));
    W2D_CUDA_TRY(cudaMemcpyAsync(e->shot.p, sh, sizeof sh, cudaMemcpyHostToDevice, e->stream));
    // the host vectors die at return: wait for the copies
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));
    return W2D_OK;
}

AcStep base_step(w2d_engine* e)
{
    AcStep s;
    memset(&s, 0, sizeof s);
    s.dt2_inj = (float)(e->dt_d * e->dt_d);
    s.err = e->err.p;
    return s;
}

// Forward steps [it0, it1) on the forward triple (roles by it % 3).
struct FwdOpts {
    int nt = 0, interval = 1, n_rec = 0;
    float* rec_out = nullptr;    // (nt, n_rec) device
    float* snaps = nullptr;      // snapshot slots, slot index = it/interval - slot0
    int slot0 = 0;
    bool illum = false;
    float* ckpt = nullptr;       // save state every ckpt_every steps (3 planes per checkpoint)
    int ckpt_every = 0;
};

int run_forward_steps(w2d_engine* e, int slot, const FwdOpts& o, int it0, int it1, double dt2inj,
                      float dt2inj_f)
{
    const AcGeom g = geom(e);
    e->chain = false;  // the caller may have enqueued anything before these steps
    auto fwd_opts = [&](AcStep& s, int it) {
        s = base_step(e);
        s.dt2_inj = dt2inj_f;
        if (it + 1 < o.nt) s.inj_w = e->cur_w + it + 1;
        if (o.rec_out) s.rec_out = o.rec_out + (size_t)it * o.n_rec;
        if (it % o.interval == 0) {
            if (o.snaps) s.snap_out = o.snaps + (size_t)(it / o.interval - o.slot0) * e->plane;
            if (o.illum) s.illum = e->illum.p;
        }
    };
    for (int it = it0; it < it1;) {
        if (o.ckpt && o.ckpt_every > 0 && it % o.ckpt_every == 0) {
            e->chain = false;
            float* c = o.ckpt + (size_t)(it / o.ckpt_every) * 3 * e->plane;
            W2D_CUDA_TRY(cudaMemcpyAsync(c, e->wave(it % 3), e->plane * 4,
                                         cudaMemcpyDeviceToDevice, e->stream));
            W2D_CUDA_TRY(cudaMemcpyAsync(c + e->plane, e->wave((it + 1) % 3), e->plane * 4,
                                         cudaMemcpyDeviceToDevice, e->stream));
            W2D_CUDA_TRY(cudaMemcpyAsync(c + 2 * e->plane, e->wave((it + 2) % 3), e->plane * 4,
                                         cudaMemcpyDeviceToDevice, e->stream));
        }
        // two steps in one launch unless a checkpoint falls between them
        const bool pair = e->two_step && !e->persistent && it + 1 < it1 &&
                          !(o.ckpt && o.ckpt_every > 0 && (it + 1) % o.ckpt_every == 0);
        int rc;
        if (pair) {
            Ac2Step p;
            memset(&p, 0, sizeof p);
            fwd_opts(p.s[0], it);
            fwd_opts(p.s[1], it + 1);
            rc = step2(e, 0, (it + 1) % 3, it % 3, (it + 2) % 3, slot, g, p);
            it += 2;
        } else {
            AcStep s;
            fwd_opts(s, it);
            s.p_next = e->wave((it + 2) % 3);
            rc = step(e, (it + 1) % 3, it % 3, slot, g, s);
            it += 1;
        }
        if (rc) return rc;
    }
    (void)dt2inj;
    return W2D_OK;
}

int forward_begin(w2d_engine* e, float dt2inj_f)
{
    int rc;
    if ((rc = zero_pass(e, 0))) return rc;
    const AcGeom g = geom(e);
    inject_kernel<<<(e->nx + 255) / 256, 256, 0, e->stream>>>(e->wave(1), g, e->cur_w, nullptr,
                                                              dt2inj_f);
    e->last_launches++;
    W2D_CUDA_TRY(cudaGetLastError());
    return W2D_OK;
}

// Backward steps for it in [it_lo, it_hi] descending; m = nt-1-it picks roles
// on the backward triple.  snaps: slot of step it = it/interval - slot0.
int run_backward_steps(w2d_engine* e, int slot, int nt, int interval, int n_rec, int it_hi,
                       int it_lo, const float* snaps, int slot0, int n_snaps_valid,
                       float img_dt, float dt2inj_f)
{
    const AcGeom g = geom(e);
    e->chain = false;  // the caller may have enqueued anything before these steps
    auto bwd_opts = [&](AcStep& s, int it) {
        s = base_step(e);
        s.dt2_inj = dt2inj_f;
        if (it >= 1 && n_rec > 0) s.inj_data = e->cur_data + (size_t)(it - 1) * n_rec;
        if (snaps && it % interval == 0) {
            const int k = it / interval;
            if (k >= 0 && k < n_snaps_valid) {
                s.snap_in = snaps + (size_t)(k - slot0) * e->plane;
                s.image = e->image.p;
                s.img_dt = img_dt;
            }
        }
    };
    for (int it = it_hi; it >= it_lo;) {
        const int m = nt - 1 - it;
        int rc;
        if (e->two_step && !e->persistent && it - 1 >= it_lo) {
            Ac2Step p;
            memset(&p, 0, sizeof p);
            bwd_opts(p.s[0], it);
            bwd_opts(p.s[1], it - 1);
            rc = step2(e, 1, 3 + (m + 1) % 3, 3 + m % 3, 3 + (m + 2) % 3, slot, g, p);
            it -= 2;
        } else {
            AcStep s;
            bwd_opts(s, it);
            s.p_next = e->wave(3 + (m + 2) % 3);
            rc = step(e, 3 + (m + 1) % 3, 3 + m % 3, slot, g, s);
            it -= 1;
        }
        if (rc) return rc;
    }
    return W2D_OK;
}

int backward_begin(w2d_engine* e, int nt, int n_rec, float dt2inj_f)
{
    int rc;
    if ((rc = zero_pass(e, 1))) return rc;
    const AcGeom g = geom(e);
    inject_kernel<<<(e->nx + 255) / 256, 256, 0, e->stream>>>(
        e->wave(4), g, nullptr, e->cur_data + (size_t)(nt - 1) * n_rec, dt2inj_f);
    e->last_launches++;
    W2D_CUDA_TRY(cudaGetLastError());
    return W2D_OK;
}

// Everything a pass's launches hold: when it matches a cached graph, replaying the
// graph issues exactly the launches the host code would.
std::vector<uintptr_t> pass_key(const w2d_engine* e, int pass, int nt, int interval, int mode,
                                int seg, int n_rec)
{
    std::vector<uintptr_t> k = {
        (uintptr_t)pass, (uintptr_t)nt, (uintptr_t)interval, (uintptr_t)mode, (uintptr_t)seg,
        (uintptr_t)n_rec, (uintptr_t)e->tile.warps, (uintptr_t)e->tile.rpw, (uintptr_t)e->pdl,
        (uintptr_t)e->l2_hints, (uintptr_t)e->use_lut, (uintptr_t)e->use_arr,
        (uintptr_t)e->tm_tz, (uintptr_t)e->waves.p, (uintptr_t)e->snaps.p, (uintptr_t)e->ckpt.p,
        (uintptr_t)e->v2dt2.p, (uintptr_t)e->image.p, (uintptr_t)e->illum.p,
        (uintptr_t)e->cur_w, (uintptr_t)e->cur_data, (uintptr_t)e->rec_ptr.p,
        (uintptr_t)e->rec_list.p, (uintptr_t)e->shot.p, (uintptr_t)e->err.p,
        (uintptr_t)e->sponge_lut.p, (uintptr_t)e->sponge_arr.p, (uintptr_t)e->rec_out.p};
    for (int i = 0; i < 6; ++i) k.push_back((uintptr_t)e->perm[i]);
    return k;
}

// Run one pass: replay its cached graph when the key matches, else capture the pass
// from `body` (the host code that launches it), instantiate and launch the graph.  With
// graphs off, or in a launch mode that keeps host-side state, `body` runs directly.  A
// capture the runtime refuses turns graphs off for this engine and runs `body`.
template <typename F>
int run_pass(w2d_engine* e, w2d_engine::PassGraph& pg, std::vector<uintptr_t> key, F&& body)
{
    if (!e->use_graphs || e->two_step || e->persistent) return body();
    if (pg.exec && pg.key == key) {
        W2D_CUDA_TRY(cudaGraphLaunch(pg.exec, e->stream));
        e->last_launches += pg.launches;
        e->last_recompute += pg.recompute;
        return W2D_OK;
    }
    pg.reset();
    const long long l0 = e->last_launches, r0 = e->last_recompute;
    W2D_CUDA_TRY(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = body();
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(e->stream, &graph);
    if (rc || ce != cudaSuccess || !graph) {
        // Nothing captured has run.  Whatever refused the capture (the pass's own
        // launches are checked again below), run this and later passes as direct
        // launches on this engine.
        cudaGetLastError();
        if (graph) cudaGraphDestroy(graph);
        e->use_graphs = 0;
        e->last_launches = l0;
        e->last_recompute = r0;
        return body();
    }
    const cudaError_t ie = cudaGraphInstantiate(&pg.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        // as above: nothing has run; launch directly from now on
        cudaGetLastError();
        pg.exec = nullptr;
        e->use_graphs = 0;
        e->last_launches = l0;
        e->last_recompute = r0;
        return body();
    }
    pg.key = std::move(key);
    pg.launches = e->last_launches - l0;
    pg.recompute = e->last_recompute - r0;
    W2D_CUDA_TRY(cudaGraphLaunch(pg.exec, e->stream));
    return W2D_OK;
}

int check_err(w2d_engine* e)
{
    unsigned h = 0;
    W2D_CUDA_TRY(cudaMemcpyAsync(&h, e->err.p, 4, cudaMemcpyDeviceToHost, e->stream));
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));
    if (h) {
        char buf[96];
        snprintf(buf, sizeof buf, "device wait gave up (error bits 0x%x)", h);
        set_error(buf);
        W2D_CUDA_TRY(cudaMemsetAsync(e->err.p, 0, 4, e->stream));
        // a CTA that stopped early drew fewer tile indices than the launch accounts for
        W2D_CUDA_TRY(cudaMemsetAsync(e->tile_counter.p, 0, 4, e->stream));
        e->counter_base = 0;
        return W2D_ETIMEOUT;
    }
    return W2D_OK;
}

int common_checks(w2d_engine* e, int nt, int interval)
{
    W2D_CHECK_ARG(e, "engine is NULL");
    W2D_CHECK_ARG(nt > 0, "nt must be positive");
    W2D_CHECK_ARG(interval > 0, "snapshot_interval must be positive");
    return W2D_OK;
}

size_t free_budget(w2d_engine* e)
{
    if (e->budget) return (size_t)e->budget;
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    return (size_t)(fr * 0.8);
}

}  // namespace

extern "C" {

int w2d_engine_create(w2d_engine** out, int nx, int nz, float dx, float dz, double dt,
                      const float* sponge, int free_surface_top)
{
    W2D_CHECK_ARG(out, "out is NULL");
    *out = nullptr;
    W2D_CHECK_ARG(nx >= 5 && nz >= 5, "grid must be at least 5 x 5");
    W2D_CHECK_ARG(dx > 0 && dz > 0 && dt > 0, "dx, dz, dt must be positive");
    w2d_engine* e = new w2d_engine();
    e->device = current_device();
    e->nx = nx;
    e->nz = nz;
    e->ldx = pitch_for(nx);
    e->plane = (size_t)e->ldx * nz;
    e->dx = dx;
    e->dz = dz;
    e->dt = (float)dt;
    e->dt_d = dt;
    e->fs = free_surface_top ? 1 : 0;
    e->inv_dx2 = 1.0f / (dx * dx);
    e->inv_dz2 = 1.0f / (dz * dz);
    e->dt2 = e->dt * e->dt;
    int rc = W2D_OK;
    auto fail = [&](int code) {
        w2d_engine_destroy(e);
        return code;
    };
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess ||
        cudaStreamCreateWithFlags(&e->up, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->up_after, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->data_ready, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->fwd_done, cudaEventDisableTiming) != cudaSuccess) {
        set_error("stream/event creation failed");
        return fail(W2D_ECUDA);
    }
    if ((rc = e->waves.ensure(10 * e->plane)) || (rc = e->v2dt2.ensure(2 * e->plane)) ||
        (rc = e->staging.ensure(e->plane)) || (rc = e->image.ensure(e->plane)) ||
        (rc = e->illum.ensure(e->plane)) || (rc = e->err.ensure(1)) ||
        (rc = e->tile_counter.ensure(1)))
        return fail(rc);
    if (cudaMemset(e->err.p, 0, 4) != cudaSuccess || cudaMemset(e->tile_counter.p, 0, 4) ||
        cudaMemset(e->waves.p, 0, 10 * e->plane * 4) ||
        cudaMemset(e->v2dt2.p, 0, 2 * e->plane * 4)) {
        set_error("memset failed");
        return fail(W2D_ECUDA);
    }
    // Sponge: a Cerjan table when the array is one, else the array itself.
    if (sponge) {
        // recover (n, alpha) candidates from the array: n is the largest frame
        // distance with a value != 1; alpha from the value at distance 1 is not
        // needed, the table is rebuilt from the array's own values and verified.
        int nmax = std::max(nx, nz);
        std::vector<float> lut(nmax + 2, 1.0f);
        std::vector<char> seen(nmax + 2, 0);
        bool ok = true;
        int n_est = -1;
        // distances with respect to every candidate n are not known yet; probe along
        // row nz/2 from the left edge: d = n - ix for ix < n.
        const float* mid = sponge + (size_t)(nz / 2) * nx;
        for (int ix = 0; ix < nx && mid[ix] != 1.0f; ++ix) n_est = ix + 1;
        // n_est: count of non-unit cells from the left; d = n - ix > 0 for ix < n.
        const int n = n_est < 0 ? 0 : n_est;
        for (int iz = 0; iz < nz && ok; ++iz)
            for (int ix = 0; ix < nx; ++ix) {
                int d = 0;
                d = std::max(d, n - ix);
                d = std::max(d, ix - (nx - 1 - n));
                d = std::max(d, iz - (nz - 1 - n));
                if (!free_surface_top) d = std::max(d, n - iz);
                const float v = sponge[(size_t)iz * nx + ix];
                if (d == 0) {
                    if (v != 1.0f) { ok = false; break; }
                } else if (!seen[d]) {
                    seen[d] = 1;
                    lut[d] = v;
                } else if (lut[d] != v) {
                    ok = false;
                    break;
                }
            }
        if (ok) {
            e->n_sponge = n;
            lut[0] = 1.0f;
            if ((rc = e->sponge_lut.ensure(n + 1))) return fail(rc);
            cudaMemcpy(e->sponge_lut.p, lut.data(), (n + 1) * 4, cudaMemcpyHostToDevice);
            e->use_lut = true;
        } else {
            if ((rc = e->sponge_arr.ensure(e->plane))) return fail(rc);
            cudaMemset(e->sponge_arr.p, 0, e->plane * 4);
            cudaMemcpy2D(e->sponge_arr.p, (size_t)e->ldx * 4, sponge, (size_t)nx * 4,
                         (size_t)nx * 4, nz, cudaMemcpyHostToDevice);
            e->use_arr = true;
        }
    }
    if ((rc = e->shot.ensure(5)) || (rc = e->rec_ptr.ensure(nx + 1)) ||
        (rc = e->rec_list.ensure(1)))
        return fail(rc);
    int sh[5] = {-1, -1, -1, 0, -1};
    cudaMemcpy(e->shot.p, sh, sizeof sh, cudaMemcpyHostToDevice);
    cudaMemset(e->rec_ptr.p, 0, (nx + 1) * 4);
    if ((rc = ensure_tensor_maps(e))) return fail(rc);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        set_error("engine set-up failed");
        return fail(W2D_ECUDA);
    }
    *out = e;
    return W2D_OK;
}

void w2d_engine_destroy(w2d_engine* e)
{
    W2D_ON_DEVICE_OF(e);
    if (!e) return;
    if (e->stream) cudaStreamSynchronize(e->stream);
    e->g_fwd.reset();
    e->g_bwd.reset();
    e->g_model.reset();
    e->g_bcorr.reset();
    for (DevBuf<float>* b : {&e->sponge_lut, &e->sponge_arr, &e->waves, &e->v2dt2, &e->staging,
                             &e->wavelet, &e->data, &e->rec_out, &e->snaps, &e->ckpt, &e->image,
                             &e->illum, &e->stack_img, &e->stack_ill})
        b->release();
    e->shot.release();
    e->rec_ptr.release();
    e->rec_list.release();
    e->err.release();
    e->scratch.release();
    e->tile_counter.release();
    for (auto& b : e->st_w) b.release();
    for (auto& b : e->st_d) b.release();
    if (e->t0) cudaEventDestroy(e->t0);
    if (e->t1) cudaEventDestroy(e->t1);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->ev1) cudaEventDestroy(e->ev1);
    if (e->up) cudaStreamSynchronize(e->up);
    if (e->up_after) cudaEventDestroy(e->up_after);
    if (e->data_ready) cudaEventDestroy(e->data_ready);
    if (e->fwd_done) cudaEventDestroy(e->fwd_done);
    if (e->up) cudaStreamDestroy(e->up);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

int w2d_engine_set_tile(w2d_engine* e, int warps, int rows_per_warp)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    if (warps == 0 && rows_per_warp == 0) {
        warps = 4;
        rows_per_warp = 4;
    }
    W2D_CHECK_ARG(tile_supported(warps, rows_per_warp), "unsupported tile shape");
    e->tile = TileShape{warps, rows_per_warp};
    return ensure_tensor_maps(e);
}

int w2d_engine_set_launch(w2d_engine* e, int persistent, int pdl)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->persistent = persistent ? 1 : 0;
    e->pdl = pdl ? 1 : 0;
    return W2D_OK;
}

int w2d_engine_set_graphs(w2d_engine* e, int on)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->use_graphs = on ? 1 : 0;
    e->g_fwd.reset();
    e->g_bwd.reset();
    e->g_model.reset();
    e->g_bcorr.reset();
    return W2D_OK;
}

int w2d_engine_set_two_step(w2d_engine* e, int rows_per_warp)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    W2D_CHECK_ARG(rows_per_warp == 0 || rows_per_warp == 1 ||
                      (rows_per_warp >= 2 && rows_per_warp <= 4),
                  "rows_per_warp must be 0 (off), 1 (default shape) or 2..4");
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));  // the maps may be in use
    e->two_step = rows_per_warp == 1 ? AC2_R2 : rows_per_warp;
    return ensure_step2_maps(e);
}

int w2d_engine_set_l2_hints(w2d_engine* e, int on)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    e->l2_hints = on ? 1 : 0;
    return W2D_OK;
}

int w2d_engine_set_memory_budget(w2d_engine* e, unsigned long long bytes)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    e->budget = bytes;
    return W2D_OK;
}

int w2d_engine_set_velocity(w2d_engine* e, int slot, const float* vel)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && vel, "NULL argument");
    W2D_CHECK_ARG(slot == 0 || slot == 1, "velocity slot must be 0 or 1");
    int rc;
    W2D_CUDA_TRY(cudaMemsetAsync(e->staging.p, 0, e->plane * 4, e->stream));
    if ((rc = upload_field_any(e, e->staging.p, vel))) return rc;
    v2dt2_kernel<<<grid_for(e->plane), 256, 0, e->stream>>>(e->v2dt2.p + (size_t)slot * e->plane,
                                                            e->staging.p, e->plane, e->dt2);
    W2D_CUDA_TRY(cudaGetLastError());
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->vel_set[slot] = true;
    return W2D_OK;
}

int w2d_forward(w2d_engine* e, int vel_slot, const float* wavelet, int nt, int src_ix, int src_iz,
                const int* rec_ix, int n_rec, int rec_iz, float* rec_out, float* snaps_out,
                int snapshot_interval)
{
    W2D_ON_DEVICE_OF(e);
    int rc;
    if ((rc = common_checks(e, nt, snapshot_interval))) return rc;
    W2D_CHECK_ARG(vel_slot == 0 || vel_slot == 1, "bad velocity slot");
    W2D_CHECK_ARG(e->vel_set[vel_slot], "velocity model not set");
    W2D_CHECK_ARG(wavelet, "wavelet is NULL");
    W2D_CHECK_ARG(src_ix >= 0 && src_ix < e->nx && src_iz >= 0 && src_iz < e->nz,
                  "source index out of range");
    if ((rc = set_shot(e, src_ix, src_iz, rec_ix, n_rec, rec_iz))) return rc;
    const int n_snaps = snaps_out ? (nt - 1) / snapshot_interval + 1 : 0;
    if ((rc = e->wavelet.ensure(nt)) || (rc = e->rec_out.ensure((size_t)nt * std::max(n_rec, 1))))
        return rc;
    if (snaps_out) {
        const size_t need = (size_t)n_snaps * e->plane;
        if (need * 4 > free_budget(e) + e->snaps.cap * 4) {
            set_error("snapshot storage exceeds the device memory budget");
            return W2D_ENOMEM;
        }
        if ((rc = e->snaps.ensure(need))) return rc;
    }
    W2D_CUDA_TRY(cudaMemcpyAsync(e->wavelet.p, wavelet, (size_t)nt * 4, cudaMemcpyHostToDevice,
                                 e->stream));
    e->cur_w = e->wavelet.p;
    e->last_launches = 0;
    e->last_recompute = 0;
    e->last_storage = 0;
    const float dt2inj = (float)(e->dt_d * e->dt_d);
    cudaEventRecord(e->ev0, e->stream);
    auto pass = [&]() -> int {
        int r;
        if ((r = forward_begin(e, dt2inj))) return r;
        FwdOpts o;
        o.nt = nt;
        o.interval = snapshot_interval;
        o.n_rec = n_rec;
        o.rec_out = n_rec > 0 ? e->rec_out.p : nullptr;
        o.snaps = snaps_out ? e->snaps.p : nullptr;
        return run_forward_steps(e, vel_slot, o, 0, nt, 0.0, dt2inj);
    };
    const int kind = (vel_slot << 2) | (snaps_out ? 1 : 0) | (n_rec > 0 ? 2 : 0);
    if ((rc = run_pass(e, e->g_model, pass_key(e, 2, nt, snapshot_interval, kind, 0, n_rec),
                       pass)))
        return rc;
    cudaEventRecord(e->ev1, e->stream);
    if (n_rec > 0)
        W2D_CUDA_TRY(cudaMemcpyAsync(rec_out, e->rec_out.p, (size_t)nt * n_rec * 4,
                                     cudaMemcpyDeviceToHost, e->stream));
    for (int k = 0; k < n_snaps; ++k)
        if ((rc = download_field(e, snaps_out + (size_t)k * e->nx * e->nz,
                                 e->snaps.p + (size_t)k * e->plane)))
            return rc;
    if ((rc = check_err(e))) return rc;
    cudaEventElapsedTime(&e->last_ms, e->ev0, e->ev1);
    return W2D_OK;
}

int w2d_backward_correlate(w2d_engine* e, int vel_slot, const float* data, int nt,
                           const int* rec_ix, int n_rec, int rec_iz, const float* fwd_snaps,
                           int n_snaps, float* image, int snapshot_interval)
{
    W2D_ON_DEVICE_OF(e);
    int rc;
    if ((rc = common_checks(e, nt, snapshot_interval))) return rc;
    W2D_CHECK_ARG(vel_slot == 0 || vel_slot == 1, "bad velocity slot");
    W2D_CHECK_ARG(e->vel_set[vel_slot], "velocity model not set");
    W2D_CHECK_ARG(image, "image is NULL");
    W2D_CHECK_ARG(n_rec == 0 || data, "data is NULL");
    W2D_CHECK_ARG(n_snaps >= 0 && (n_snaps == 0 || fwd_snaps), "bad forward wavefields");
    if ((rc = set_shot(e, -1, -1, rec_ix, n_rec, rec_iz))) return rc;
    // The reference correlates only while its snapshot counter, which starts at
    // (nt-1)/interval, indexes an existing snapshot (wave_solver.py:204,230): with
    // fewer snapshots it never correlates.
    if (n_snaps <= (nt - 1) / snapshot_interval) n_snaps = 0;
    if ((rc = e->data.ensure((size_t)nt * std::max(n_rec, 1)))) return rc;
    if (n_rec > 0)
        W2D_CUDA_TRY(cudaMemcpyAsync(e->data.p, data, (size_t)nt * n_rec * 4,
                                     cudaMemcpyHostToDevice, e->stream));
    if (n_snaps > 0) {
        const size_t need = (size_t)n_snaps * e->plane;
        if (need * 4 > free_budget(e) + e->snaps.cap * 4) {
            set_error("forward wavefields exceed the device memory budget");
            return W2D_ENOMEM;
        }
        if ((rc = e->snaps.ensure(need))) return rc;
        W2D_CUDA_TRY(cudaMemsetAsync(e->snaps.p, 0, need * 4, e->stream));
        for (int k = 0; k < n_snaps; ++k)
            if ((rc = upload_field(e, e->snaps.p + (size_t)k * e->plane,
                                   fwd_snaps + (size_t)k * e->nx * e->nz)))
                return rc;
    }
    W2D_CUDA_TRY(cudaMemsetAsync(e->image.p, 0, e->plane * 4, e->stream));
    if ((rc = upload_field(e, e->image.p, image))) return rc;
    e->cur_data = e->data.p;
    e->last_launches = 0;
    e->last_recompute = 0;
    const float dt2inj = (float)(e->dt_d * e->dt_d);
    const float img_dt = (float)(e->dt_d * (double)snapshot_interval);
    cudaEventRecord(e->ev0, e->stream);
    auto pass = [&]() -> int {
        int r;
        if (n_rec > 0) {
            if ((r = backward_begin(e, nt, n_rec, dt2inj))) return r;
        } else {
            if ((r = zero_pass(e, 1))) return r;
        }
        return run_backward_steps(e, vel_slot, nt, snapshot_interval, n_rec, nt - 1, 0,
                                  n_snaps > 0 ? e->snaps.p : nullptr, 0, n_snaps, img_dt,
                                  dt2inj);
    };
    if ((rc = run_pass(e, e->g_bcorr,
                       pass_key(e, 3, nt, snapshot_interval, vel_slot, n_snaps, n_rec), pass)))
        return rc;
    cudaEventRecord(e->ev1, e->stream);
    if ((rc = download_field(e, image, e->image.p))) return rc;
    if ((rc = check_err(e))) return rc;
    cudaEventElapsedTime(&e->last_ms, e->ev0, e->ev1);
    return W2D_OK;
}

}  // extern "C"

namespace {

// Forward + backward migration of one shot whose wavelet and data are already
// on the device (e->cur_w, e->cur_data) and whose geometry is set.
int migrate_core(w2d_engine* e, int nt, int n_rec, int snapshot_interval, int storage,
                 float* image_out, float* illum_out)
{
    int rc;
    const int interval = snapshot_interval;
    const int n_snaps = (nt - 1) / interval + 1;
    const size_t plane_b = e->plane * 4;

    // storage decision
    const size_t full_bytes = (size_t)n_snaps * plane_b;
    const size_t budget = free_budget(e) + e->snaps.cap * 4 + e->ckpt.cap * 4;
    int mode = storage;
    if (mode == W2D_STORE_AUTO) mode = full_bytes <= budget ? W2D_STORE_ALL : W2D_STORE_CHECKPOINT;
    W2D_CHECK_ARG(mode == W2D_STORE_ALL || mode == W2D_STORE_CHECKPOINT, "bad storage mode");
    int seg = 0, n_seg = 0;
    if (mode == W2D_STORE_ALL) {
        if (full_bytes > budget) {
            set_error("full snapshot storage exceeds the device memory budget");
            return W2D_ENOMEM;
        }
        if ((rc = e->snaps.ensure((size_t)n_snaps * e->plane))) return rc;
    } else {
        // segment length: about sqrt(3 * nt * interval) steps, rounded to the interval,
        // balancing 3-plane checkpoints against the snapshots of one segment.
        seg = (int)std::max(1.0, std::sqrt(3.0 * nt * interval));
        seg = std::max(interval, (seg / interval) * interval);
        n_seg = (nt + seg - 1) / seg;
        const int seg_snaps = seg / interval + 1;
        const size_t need = ((size_t)n_seg * 3 + seg_snaps) * plane_b;
        if (need > budget) {
            set_error("checkpoint storage exceeds the device memory budget");
            return W2D_ENOMEM;
        }
        if ((rc = e->ckpt.ensure((size_t)n_seg * 3 * e->plane)) ||
            (rc = e->snaps.ensure((size_t)seg_snaps * e->plane)))
            return rc;
    }
    e->last_launches = 0;
    e->last_recompute = 0;
    e->last_storage = mode;
    const float dt2inj = (float)(e->dt_d * e->dt_d);
    const float img_dt = (float)(e->dt_d * (double)interval);
    cudaEventRecord(e->ev0, e->stream);

    // 1. forward pass in slot 0 with illumination
    auto forward = [&]() -> int {
        int r;
        W2D_CUDA_TRY(cudaMemsetAsync(e->illum.p, 0, plane_b, e->stream));
        W2D_CUDA_TRY(cudaMemsetAsync(e->image.p, 0, plane_b, e->stream));
        if ((r = forward_begin(e, dt2inj))) return r;
        FwdOpts o;
        o.nt = nt;
        o.interval = interval;
        o.illum = true;
        if (mode == W2D_STORE_ALL) {
            o.snaps = e->snaps.p;
        } else {
            o.ckpt = e->ckpt.p;
            o.ckpt_every = seg;
        }
        if ((r = run_forward_steps(e, 0, o, 0, nt, 0.0, dt2inj))) return r;
        scale_kernel<<<grid_for(e->plane), 256, 0, e->stream>>>(e->illum.p, e->plane, img_dt);
        e->last_launches++;
        W2D_CUDA_TRY(cudaGetLastError());
        return W2D_OK;
    };
    if ((rc = run_pass(e, e->g_fwd, pass_key(e, 0, nt, interval, mode, seg, n_rec), forward)))
        return rc;
    if (image_out) W2D_CUDA_TRY(cudaEventRecord(e->fwd_done, e->stream));

    // 2. backward pass in slot 1 with imaging
    if (e->data_pending) {  // the receiver data uploaded beside the forward pass
        W2D_CUDA_TRY(cudaStreamWaitEvent(e->stream, e->data_ready, 0));
        e->data_pending = false;
    }
    auto backward = [&]() -> int {
        int rb;
        if (n_rec > 0) {
            if ((rb = backward_begin(e, nt, n_rec, dt2inj))) return rb;
        } else {
            if ((rb = zero_pass(e, 1))) return rb;
        }
        if (mode == W2D_STORE_ALL)
            return run_backward_steps(e, 1, nt, interval, n_rec, nt - 1, 0, e->snaps.p, 0,
                                      n_snaps, img_dt, dt2inj);
        for (int sgi = n_seg - 1; sgi >= 0; --sgi) {
            const int a = sgi * seg, b = std::min(nt, a + seg);
            // restore the forward state at step a and recompute [a, b) with snapshots
            const float* c = e->ckpt.p + (size_t)sgi * 3 * e->plane;
            W2D_CUDA_TRY(cudaMemcpyAsync(e->wave(a % 3), c, plane_b, cudaMemcpyDeviceToDevice,
                                         e->stream));
            W2D_CUDA_TRY(cudaMemcpyAsync(e->wave((a + 1) % 3), c + e->plane, plane_b,
                                         cudaMemcpyDeviceToDevice, e->stream));
            W2D_CUDA_TRY(cudaMemcpyAsync(e->wave((a + 2) % 3), c + 2 * e->plane, plane_b,
                                         cudaMemcpyDeviceToDevice, e->stream));
            FwdOpts r;
            r.nt = nt;
            r.interval = interval;
            r.snaps = e->snaps.p;
            r.slot0 = (a + interval - 1) / interval;  // first snapshot index in [a, b)
            int q;
            if ((q = run_forward_steps(e, 0, r, a, b, 0.0, dt2inj))) return q;
            e->last_recompute += b - a;
            if ((q = run_backward_steps(e, 1, nt, interval, n_rec, b - 1, a, e->snaps.p, r.slot0,
                                        n_snaps, img_dt, dt2inj)))
                return q;
        }
        return W2D_OK;
    };
    if ((rc = run_pass(e, e->g_bwd, pass_key(e, 1, nt, interval, mode, seg, n_rec), backward)))
        return rc;
    cudaEventRecord(e->ev1, e->stream);
    if (image_out) {
        // the illumination (final since the forward pass) comes back on the upload stream
        // beside the backward pass; the image after it
        cudaError_t ce = cudaStreamWaitEvent(e->up, e->fwd_done, 0);
        if (ce == cudaSuccess)
            ce = cudaMemcpy2DAsync(illum_out, (size_t)e->nx * 4, e->illum.p, (size_t)e->ldx * 4,
                                   (size_t)e->nx * 4, e->nz, cudaMemcpyDeviceToHost, e->up);
        const int rc_img = download_field(e, image_out, e->image.p);
        const cudaError_t se = cudaStreamSynchronize(e->up);
        W2D_CUDA_TRY(ce);
        if (rc_img) return rc_img;
        W2D_CUDA_TRY(se);
    } else {
        if ((rc = e->stack_img.ensure(e->plane)) || (rc = e->stack_ill.ensure(e->plane))) return rc;
        add_kernel<<<grid_for(e->plane), 256, 0, e->stream>>>(e->stack_img.p, e->image.p, e->plane);
        add_kernel<<<grid_for(e->plane), 256, 0, e->stream>>>(e->stack_ill.p, e->illum.p, e->plane);
        e->last_launches += 2;
        W2D_CUDA_TRY(cudaGetLastError());
    }
    if ((rc = check_err(e))) return rc;
    cudaEventElapsedTime(&e->last_ms, e->ev0, e->ev1);
    return W2D_OK;
}

int migrate_checks(w2d_engine* e, int nt, int interval, int src_ix, int src_iz, int n_rec,
                   float* image_out, float* illum_out)
{
    int rc;
    if ((rc = common_checks(e, nt, interval))) return rc;
    W2D_CHECK_ARG(e->vel_set[0] && e->vel_set[1], "velocity models not set");
    W2D_CHECK_ARG(n_rec >= 0, "n_rec < 0");
    W2D_CHECK_ARG(src_ix >= 0 && src_ix < e->nx && src_iz >= 0 && src_iz < e->nz,
                  "source index out of range");
    W2D_CHECK_ARG((image_out == nullptr) == (illum_out == nullptr),
                  "image_out and illum_out must both be set or both be NULL");
    return W2D_OK;
}

}  // namespace

extern "C" {

int w2d_migrate_shot(w2d_engine* e, const float* wavelet, int nt, int src_ix, int src_iz,
                     const float* data, const int* rec_ix, int n_rec, int rec_iz,
                     int snapshot_interval, int storage, float* image_out, float* illum_out)
{
    W2D_ON_DEVICE_OF(e);
    int rc;
    if ((rc = migrate_checks(e, nt, snapshot_interval, src_ix, src_iz, n_rec, image_out,
                             illum_out)))
        return rc;
    W2D_CHECK_ARG(wavelet, "wavelet is NULL");
    W2D_CHECK_ARG(n_rec == 0 || data, "data is NULL");
    if ((rc = set_shot(e, src_ix, src_iz, rec_ix, n_rec, rec_iz))) return rc;
    if ((rc = e->wavelet.ensure(nt)) || (rc = e->data.ensure((size_t)nt * std::max(n_rec, 1))))
        return rc;
    W2D_CUDA_TRY(cudaMemcpyAsync(e->wavelet.p, wavelet, (size_t)nt * 4, cudaMemcpyHostToDevice,
                                 e->stream));
    if (n_rec > 0) {
        // after everything already on the engine stream (an earlier pass may still read
        // the data buffer), beside the forward pass of this one
        W2D_CUDA_TRY(cudaEventRecord(e->up_after, e->stream));
        W2D_CUDA_TRY(cudaStreamWaitEvent(e->up, e->up_after, 0));
        W2D_CUDA_TRY(cudaMemcpyAsync(e->data.p, data, (size_t)nt * n_rec * 4,
                                     cudaMemcpyHostToDevice, e->up));
        W2D_CUDA_TRY(cudaEventRecord(e->data_ready, e->up));
        e->data_pending = true;
    }
    e->cur_w = e->wavelet.p;
    e->cur_data = e->data.p;
    const int rc2 = migrate_core(e, nt, n_rec, snapshot_interval, storage, image_out, illum_out);
    if (e->data_pending) {  // an early return before the backward pass: settle the copy
        cudaStreamSynchronize(e->up);
        e->data_pending = false;
    }
    return rc2;
}

int w2d_shot_stage(w2d_engine* e, int slot, const float* wavelet, int nt, const float* data,
                   int n_rec)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && wavelet && nt > 0 && slot >= 0 && slot < 4096, "bad arguments");
    W2D_CHECK_ARG(n_rec >= 0 && (n_rec == 0 || data), "bad data");
    if ((int)e->st_w.size() <= slot) {
        e->st_w.resize(slot + 1);
        e->st_d.resize(slot + 1);
        e->st_nt.resize(slot + 1, 0);
        e->st_nrec.resize(slot + 1, 0);
    }
    int rc;
    if ((rc = e->st_w[slot].ensure(nt)) ||
        (rc = e->st_d[slot].ensure((size_t)nt * std::max(n_rec, 1))))
        return rc;
    W2D_CUDA_TRY(cudaMemcpyAsync(e->st_w[slot].p, wavelet, (size_t)nt * 4, cudaMemcpyHostToDevice,
                                 e->stream));
    if (n_rec > 0)
        W2D_CUDA_TRY(cudaMemcpyAsync(e->st_d[slot].p, data, (size_t)nt * n_rec * 4,
                                     cudaMemcpyHostToDevice, e->stream));
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->st_nt[slot] = nt;
    e->st_nrec[slot] = n_rec;
    return W2D_OK;
}

int w2d_migrate_staged(w2d_engine* e, int slot, int src_ix, int src_iz, const int* rec_ix,
                       int n_rec, int rec_iz, int snapshot_interval, int storage,
                       float* image_out, float* illum_out)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && slot >= 0 && slot < (int)e->st_nt.size() && e->st_nt[slot] > 0,
                  "slot not staged");
    W2D_CHECK_ARG(n_rec == e->st_nrec[slot], "n_rec differs from the staged data");
    const int nt = e->st_nt[slot];
    int rc;
    if ((rc = migrate_checks(e, nt, snapshot_interval, src_ix, src_iz, n_rec, image_out,
                             illum_out)))
        return rc;
    if ((rc = set_shot(e, src_ix, src_iz, rec_ix, n_rec, rec_iz))) return rc;
    // the staged inputs move into the engine's own input buffers (a device-to-device copy
    // of a few hundred microseconds at most), so every shot's passes hold the same
    // addresses and replay the same captured graphs
    if ((rc = e->wavelet.ensure(nt)) || (rc = e->data.ensure((size_t)nt * std::max(n_rec, 1))))
        return rc;
    W2D_CUDA_TRY(cudaMemcpyAsync(e->wavelet.p, e->st_w[slot].p, (size_t)nt * 4,
                                 cudaMemcpyDeviceToDevice, e->stream));
    if (n_rec > 0)
        W2D_CUDA_TRY(cudaMemcpyAsync(e->data.p, e->st_d[slot].p, (size_t)nt * n_rec * 4,
                                     cudaMemcpyDeviceToDevice, e->stream));
    e->cur_w = e->wavelet.p;
    e->cur_data = e->data.p;
    return migrate_core(e, nt, n_rec, snapshot_interval, storage, image_out, illum_out);
}

int w2d_engine_timer_start(w2d_engine* e)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    if (!e->t0 && (cudaEventCreate(&e->t0) != cudaSuccess || cudaEventCreate(&e->t1) != cudaSuccess)) {
        set_error("event creation failed");
        return W2D_ECUDA;
    }
    W2D_CUDA_TRY(cudaEventRecord(e->t0, e->stream));
    return W2D_OK;
}

int w2d_engine_timer_stop(w2d_engine* e, float* ms)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && e->t0 && ms, "timer not started");
    W2D_CUDA_TRY(cudaEventRecord(e->t1, e->stream));
    W2D_CUDA_TRY(cudaEventSynchronize(e->t1));
    W2D_CUDA_TRY(cudaEventElapsedTime(ms, e->t0, e->t1));
    return W2D_OK;
}

int w2d_host_alloc(void** out, unsigned long long bytes)
{
    W2D_CHECK_ARG(out, "out is NULL");
    W2D_CUDA_TRY(cudaMallocHost(out, (size_t)bytes));
    return W2D_OK;
}

void w2d_host_free(void* p)
{
    if (p) cudaFreeHost(p);
}

int w2d_device_memory(unsigned long long* free_bytes, unsigned long long* total_bytes)
{
    W2D_CHECK_ARG(free_bytes && total_bytes, "NULL argument");
    size_t f = 0, t = 0;
    W2D_CUDA_TRY(cudaMemGetInfo(&f, &t));
    *free_bytes = f;
    *total_bytes = t;
    return W2D_OK;
}

int w2d_stack_reset(w2d_engine* e)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    int rc;
    if ((rc = e->stack_img.ensure(e->plane)) || (rc = e->stack_ill.ensure(e->plane))) return rc;
    W2D_CUDA_TRY(cudaMemsetAsync(e->stack_img.p, 0, e->plane * 4, e->stream));
    W2D_CUDA_TRY(cudaMemsetAsync(e->stack_ill.p, 0, e->plane * 4, e->stream));
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));
    return W2D_OK;
}

int w2d_stack_add(w2d_engine* e, const float* image, const float* illum)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && image && illum, "NULL argument");
    W2D_CHECK_ARG(e->stack_img.p, "stack is empty (call w2d_stack_reset first)");
    int rc;
    if ((rc = e->image.ensure(e->plane)) || (rc = e->illum.ensure(e->plane))) return rc;
    if ((rc = upload_field(e, e->image.p, image)) || (rc = upload_field(e, e->illum.p, illum)))
        return rc;
    add_kernel<<<grid_for(e->plane), 256, 0, e->stream>>>(e->stack_img.p, e->image.p, e->plane);
    add_kernel<<<grid_for(e->plane), 256, 0, e->stream>>>(e->stack_ill.p, e->illum.p, e->plane);
    W2D_CUDA_TRY(cudaGetLastError());
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));  // the caller's arrays are free to go
    return W2D_OK;
}

int w2d_stack_read(w2d_engine* e, float* image_out, float* illum_out)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && image_out && illum_out, "NULL argument");
    W2D_CHECK_ARG(e->stack_img.p, "stack is empty (call w2d_stack_reset first)");
    int rc;
    if ((rc = download_field(e, image_out, e->stack_img.p)) ||
        (rc = download_field(e, illum_out, e->stack_ill.p)))
        return rc;
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));
    return W2D_OK;
}

}  // extern "C"

// ---- post-stack on the device (rtm_engine.py:145-158) ---------------------------
namespace {

__device__ __forceinline__ float ps_sponge(const AcGeom& g, const float* arr, int ix, int iz)
{
    if (arr) return arr[(size_t)iz * g.ldx + ix];
    if (g.sponge_lut) {
        const int d = sponge_dist(ix, iz, g.nx, g.nz, g.n_sponge, g.free_surface);
        return d > 0 ? g.sponge_lut[d] : 1.0f;
    }
    return 1.0f;
}

// muted copies of the stack and the largest illumination (as ordered bits: >= 0)
__global__ void ps_mute_kernel(AcGeom g, const float* arr, int mute, const float* img,
                               const float* ill, float* img_out, float* ill_out, unsigned* maxbits)
{
    const size_t n = (size_t)g.ldx * g.nz;
    unsigned local = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int iz = (int)(i / g.ldx), ix = (int)(i % g.ldx);
        float a = img[i], b = ill[i];
        if (ix >= g.nx || (mute && ps_sponge(g, arr, ix, iz) < 0.99f)) {
            a = 0.0f;
            b = 0.0f;
        }
        img_out[i] = a;
        ill_out[i] = b;
        local = max(local, __float_as_uint(b));
    }
    atomicMax(maxbits, local);
}

// normalized = stacked / (sqrt(illum) + eps), eps = float32(1e-4) * max or 1e-12
__global__ void ps_normalize_kernel(AcGeom g, const float* img, const float* ill,
                                    const unsigned* maxbits, float* out)
{
    const float mx = __uint_as_float(*maxbits);
    const float eps = mx > 0.0f ? fmul(1e-4f, mx) : 1e-12f;
    const size_t n = (size_t)g.ldx * g.nz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        out[i] = __fdiv_rn(img[i], fadd(__fsqrt_rn(ill[i]), eps));
}

// 3x3 Laplacian, 'same' size, symmetric boundary (edge sample repeated), then mute
__global__ void ps_laplacian_kernel(AcGeom g, const float* arr, int mute, const float* img,
                                    float kx, float kz, float kc, float* out)
{
    const size_t n = (size_t)g.ldx * g.nz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int iz = (int)(i / g.ldx), ix = (int)(i % g.ldx);
        if (ix >= g.nx) {
            out[i] = 0.0f;
            continue;
        }
        const int xm = ix > 0 ? ix - 1 : 0, xp = ix < g.nx - 1 ? ix + 1 : g.nx - 1;
        const int zm = iz > 0 ? iz - 1 : 0, zp = iz < g.nz - 1 ? iz + 1 : g.nz - 1;
        const float* r = img + (size_t)iz * g.ldx;
        float v = kz * img[(size_t)zm * g.ldx + ix] + kx * r[xm] + kc * r[ix] + kx * r[xp] +
                  kz * img[(size_t)zp * g.ldx + ix];
        if (mute && ps_sponge(g, arr, ix, iz) < 0.99f) v = 0.0f;
        out[i] = v;
    }
}

}  // namespace

extern "C" {

int w2d_post_stack(w2d_engine* e, int mute_sponge, float* raw_out, float* laplacian_out,
                   float* normalized_out)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && raw_out && laplacian_out && normalized_out, "NULL argument");
    W2D_CHECK_ARG(e->stack_img.p, "stack is empty (call w2d_stack_reset first)");
    int rc;
    if ((rc = e->snaps.ensure(2 * e->plane)) || (rc = e->scratch.ensure(1))) return rc;
    unsigned* maxbits = e->scratch.p;
    float* lap = e->snaps.p;
    float* nrm = e->snaps.p + e->plane;
    const AcGeom g = geom(e);
    const float* arr = e->use_arr ? e->sponge_arr.p : nullptr;
    W2D_CUDA_TRY(cudaMemsetAsync(maxbits, 0, 4, e->stream));
    ps_mute_kernel<<<grid_for(e->plane), 256, 0, e->stream>>>(g, arr, mute_sponge, e->stack_img.p,
                                                             e->stack_ill.p, e->image.p,
                                                             e->illum.p, maxbits);
    ps_normalize_kernel<<<grid_for(e->plane), 256, 0, e->stream>>>(g, e->image.p, e->illum.p,
                                                                  maxbits, nrm);
    const double ix2 = 1.0 / ((double)e->dx * e->dx), iz2 = 1.0 / ((double)e->dz * e->dz);
    ps_laplacian_kernel<<<grid_for(e->plane), 256, 0, e->stream>>>(
        g, arr, mute_sponge, e->image.p, (float)ix2, (float)iz2, (float)(-2.0 * ix2 - 2.0 * iz2),
        lap);
    W2D_CUDA_TRY(cudaGetLastError());
    if ((rc = download_field(e, raw_out, e->image.p)) ||
        (rc = download_field(e, laplacian_out, lap)) ||
        (rc = download_field(e, normalized_out, nrm)))
        return rc;
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));
    return W2D_OK;
}

int w2d_engine_last_stats(w2d_engine* e, int* storage_used, long long* step_launches,
                          long long* recomputed_steps, float* device_ms)
{
    W2D_CHECK_ARG(e, "engine is NULL");
    if (storage_used) *storage_used = e->last_storage;
    if (step_launches) *step_launches = e->last_launches;
    if (recomputed_steps) *recomputed_steps = e->last_recompute;
    if (device_ms) *device_ms = e->last_ms;
    return W2D_OK;
}

}  // extern "C"

// ---- differentiable forward modelling and its adjoint (velocity gradient) -----

namespace {

// contiguous (nz, nx) velocity on the device -> pitched vel and vel^2 dt^2
__global__ void fwi_model_kernel(float* v2dt2, float* vel_p, const float* vel, int nx, int nz,
                                 int ldx, float dt2)
{
    const size_t n = (size_t)ldx * nz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int iz = (int)(i / ldx), ix = (int)(i % ldx);
        const float v = ix < nx ? vel[(size_t)iz * nx + ix] : 0.0f;
        vel_p[i] = v;
        v2dt2[i] = fmul(fmul(v, v), dt2);
    }
}

// dJ/dv = dJ/dc * 2 v dt^2, pitched -> contiguous
__global__ void fwi_chain_kernel(float* grad_v, const float* grad_c, const float* vel_p, int nx,
                                 int nz, int ldx, float dt2)
{
    const size_t n = (size_t)nx * nz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int iz = (int)(i / nx), ix = (int)(i % nx);
        const size_t o = (size_t)iz * ldx + ix;
        grad_v[i] = grad_c[o] * 2.0f * vel_p[o] * dt2;
    }
}

bool written_cell(const w2d_engine* e, int iz, int ix)
{
    const bool interior = iz >= 2 && iz < e->nz - 2 && ix >= 2 && ix < e->nx - 2;
    return interior || (e->fs && iz >= 0 && iz < 2 && ix >= 0 && ix < e->nx);
}

}  // namespace

struct w2d_fwi_state {
    int nt = 0, n_rec = 0, seg = 0, n_seg = 0;
    bool stored = false;  // one segment of every forward state, written by the forward pass
    DevBuf<float> vel_p, grad_c, zero, segbuf;
    std::vector<CUtensorMap> seg_maps;
    CUtensorMap map_c_halo, map_zero;
};

extern "C" {

int w2d_fwi_forward(w2d_engine* e, const float* vel_dev, const float* wavelet, int nt, int src_ix,
                    int src_iz, const int* rec_ix, int n_rec, int rec_iz, float* traces_dev)
{
    W2D_ON_DEVICE_OF(e);
    int rc;
    if ((rc = common_checks(e, nt, 1))) return rc;
    W2D_CHECK_ARG(vel_dev && wavelet && traces_dev, "NULL argument");
    W2D_CHECK_DEVICE_PTR(vel_dev, e->device);
    W2D_CHECK_DEVICE_PTR(traces_dev, e->device);
    W2D_CHECK_ARG(n_rec > 0 && rec_ix, "receivers required");
    W2D_CHECK_ARG(e->tile.rpw == 4 && (e->tile.warps == 4 || e->tile.warps == 8),
                  "the adjoint path runs with 4x4 or 8x4 tiles");
    W2D_CHECK_ARG(src_ix >= 0 && src_ix < e->nx && src_iz >= 0 && src_iz < e->nz &&
                      written_cell(e, src_iz, src_ix),
                  "the source must sit on a written cell (interior or free-surface rows)");
    for (int r = 0; r < n_rec; ++r)
        W2D_CHECK_ARG(rec_ix[r] >= 0 && rec_ix[r] < e->nx && written_cell(e, rec_iz, rec_ix[r]),
                      "receivers must sit on written cells (interior or free-surface rows)");
    if (!e->fwi) e->fwi = new w2d_fwi_state();
    w2d_fwi_state* f = e->fwi;
    if ((rc = set_shot(e, src_ix, src_iz, rec_ix, n_rec, rec_iz))) return rc;
    f->nt = nt;
    f->n_rec = n_rec;
    f->seg = e->fwi_seg > 0 ? std::min(e->fwi_seg, nt) : std::max(1, (int)std::sqrt(3.0 * nt));
    f->n_seg = (nt + f->seg - 1) / f->seg;
    if ((rc = f->vel_p.ensure(e->plane)) || (rc = f->grad_c.ensure(e->plane)) ||
        (rc = f->zero.ensure(e->plane)) || (rc = f->segbuf.ensure((size_t)f->seg * e->plane)) ||
        (rc = e->ckpt.ensure((size_t)f->n_seg * 3 * e->plane)) || (rc = e->wavelet.ensure(nt)) ||
        (rc = e->rec_out.ensure((size_t)nt * n_rec)) || (rc = e->data.ensure((size_t)nt * n_rec)))
        return rc;
    W2D_CUDA_TRY(cudaMemsetAsync(f->zero.p, 0, e->plane * 4, e->stream));
    W2D_CUDA_TRY(cudaMemcpyAsync(e->wavelet.p, wavelet, (size_t)nt * 4, cudaMemcpyHostToDevice,
                                 e->stream));
    fwi_model_kernel<<<grid_for(e->plane), 256, 0, e->stream>>>(e->v2dt2.p, f->vel_p.p, vel_dev,
                                                               e->nx, e->nz, e->ldx, e->dt2);
    W2D_CUDA_TRY(cudaGetLastError());
    e->vel_set[0] = true;
    e->cur_w = e->wavelet.p;
    e->last_launches = 0;
    e->last_recompute = 0;
    const float dt2inj = (float)(e->dt_d * e->dt_d);
    if ((rc = forward_begin(e, dt2inj))) return rc;
    FwdOpts o;
    o.nt = nt;
    o.n_rec = n_rec;
    o.rec_out = e->rec_out.p;
    f->stored = f->seg >= nt;
    if (f->stored) {
        // every forward state kept as it is computed: the gradient recomputes nothing
        o.snaps = f->segbuf.p;
        o.interval = 1;
        o.slot0 = 0;
    } else {
        o.ckpt = e->ckpt.p;
        o.ckpt_every = f->seg;
    }
    if ((rc = run_forward_steps(e, 0, o, 0, nt, 0.0, dt2inj))) return rc;
    W2D_CUDA_TRY(cudaMemcpyAsync(traces_dev, e->rec_out.p, (size_t)nt * n_rec * 4,
                                 cudaMemcpyDeviceToDevice, e->stream));
    return check_err(e);
}

int w2d_fwi_set_segment(w2d_engine* e, int steps)
{
    W2D_CHECK_ARG(e, "engine is NULL");
    W2D_CHECK_ARG(steps >= 0, "segment length must be >= 0");
    e->fwi_seg = steps;
    return W2D_OK;
}

int w2d_fwi_set_adjoint_form(w2d_engine* e, int cells)
{
    W2D_CHECK_ARG(e, "engine is NULL");
    e->adj_cells = cells ? 1 : 0;
    return W2D_OK;
}

int w2d_fwi_gradient(w2d_engine* e, const float* resid_dev, float* grad_dev)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && e->fwi && e->fwi->nt > 0, "call w2d_fwi_forward first");
    W2D_CHECK_ARG(resid_dev && grad_dev, "NULL argument");
    W2D_CHECK_DEVICE_PTR(resid_dev, e->device);
    W2D_CHECK_DEVICE_PTR(grad_dev, e->device);
    w2d_fwi_state* f = e->fwi;
    const int nt = f->nt, n_rec = f->n_rec, seg = f->seg;
    const size_t plane_b = e->plane * 4;
    int rc;
    W2D_CUDA_TRY(cudaMemcpyAsync(e->data.p, resid_dev, (size_t)nt * n_rec * 4,
                                 cudaMemcpyDeviceToDevice, e->stream));
    if ((rc = zero_pass(e, 1))) return rc;
    W2D_CUDA_TRY(cudaMemsetAsync(f->grad_c.p, 0, plane_b, e->stream));
    const int hz = e->tile.tz() + 4;
    if ((rc = make_tensor_map_2d(&f->map_c_halo, e->v2dt2.p, e->nx, e->nz, e->ldx, AC_SW, hz)) ||
        (rc = make_tensor_map_2d(&f->map_zero, f->zero.p, e->nx, e->nz, e->ldx, AC_SW, hz)))
        return rc;
    f->seg_maps.resize(seg);
    for (int k = 0; k < seg; ++k)
        if ((rc = make_tensor_map_2d(&f->seg_maps[k], f->segbuf.p + (size_t)k * e->plane, e->nx,
                                     e->nz, e->ldx, AC_SW, hz)))
            return rc;
    const AcGeom g = geom(e);
    bool adj_chain = false;  // the stream's last operation is an adjoint step
    auto adj = [&](int n, const CUtensorMap& pf) -> int {
        AdjMaps m;
        m.a1 = e->mcurr(3 + (n + 1) % 3);
        m.a2 = e->mprev(3 + (n + 2) % 3);
        m.c = f->map_c_halo;
        m.pf = pf;
        AdjStep s;
        s.a_out = e->wave(3 + n % 3);
        s.grad = f->grad_c.p;
        s.resid_row = n >= 1 ? e->data.p + (size_t)(n - 1) * n_rec : nullptr;
        s.err = e->err.p;
        const int pdl = e->pdl && adj_chain;
        cudaError_t ce = e->tile.warps == 4
                             ? launch_adjoint_step<4, 4>(m, g, s, e->stream, pdl, e->adj_cells)
                             : launch_adjoint_step<8, 4>(m, g, s, e->stream, pdl, e->adj_cells);
        W2D_CUDA_TRY(ce);
        adj_chain = true;
        e->last_launches++;
        return W2D_OK;
    };
    e->last_launches = 0;
    e->last_recompute = 0;
    if ((rc = adj(nt, f->map_zero))) return rc;
    const float dt2inj = (float)(e->dt_d * e->dt_d);
    for (int sgi = f->n_seg - 1; sgi >= 0; --sgi) {
        const int a = sgi * seg, b = std::min(nt, a + seg);
        if (!f->stored) {
            const float* c = e->ckpt.p + (size_t)sgi * 3 * e->plane;
            W2D_CUDA_TRY(cudaMemcpyAsync(e->wave(a % 3), c, plane_b, cudaMemcpyDeviceToDevice,
                                         e->stream));
            W2D_CUDA_TRY(cudaMemcpyAsync(e->wave((a + 1) % 3), c + e->plane, plane_b,
                                         cudaMemcpyDeviceToDevice, e->stream));
            W2D_CUDA_TRY(cudaMemcpyAsync(e->wave((a + 2) % 3), c + 2 * e->plane, plane_b,
                                         cudaMemcpyDeviceToDevice, e->stream));
            FwdOpts r;
            r.nt = nt;
            r.interval = 1;
            r.snaps = f->segbuf.p;
            r.slot0 = a;
            if ((rc = run_forward_steps(e, 0, r, a, b, 0.0, dt2inj))) return rc;
            e->last_recompute += b - a;
            adj_chain = false;  // the segment's first adjoint step waits for the stream
        }
        for (int n = b - 1; n >= a; --n)
            if ((rc = adj(n, f->seg_maps[n - a]))) return rc;
    }
    fwi_chain_kernel<<<grid_for((size_t)e->nx * e->nz), 256, 0, e->stream>>>(
        grad_dev, f->grad_c.p, f->vel_p.p, e->nx, e->nz, e->ldx, e->dt2);
    W2D_CUDA_TRY(cudaGetLastError());
    return check_err(e);
}

int w2d_engine_synchronize(w2d_engine* e)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    W2D_CUDA_TRY(cudaStreamSynchronize(e->stream));
    return W2D_OK;
}

}  // extern "C"
