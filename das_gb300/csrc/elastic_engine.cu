// elastic_engine.cu -- elastic modelling with vertical-strain receivers and its
// adjoint (gradients with respect to lambda, mu and the buoyancies), forward state
// recovered from checkpoints.  See elastic_adjoint_kernels.cuh for the scheme.
//
// A call runs a batch of shots on one grid: every kernel launch covers all shots of
// the batch (grid z = shot), each shot with its own parameters, source position,
// wavelet and traces, the receivers shared.  Small grids, whose single-shot launches
// would leave most of the GPU idle, fill it this way.
//
// Device layout (pitched planes of ldx * nz floats):
//   sponge                    1 plane (shared)
//   params                    shot-major, 4 planes per shot (lambda, mu, bx, bz)
//   state, adj, tmp           shot-major, 5 planes per shot (vx, vz, sxx, szz, sxz)
//   grad                      shot-major, 4 planes per shot
//   ckpt                      segment-major, then shot, 5 planes
//   seg                       slot-major (seg_len + 1 slots), then shot, 5 planes
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "elastic_adjoint_tma.cuh"
#include "small_kernels.cuh"
#include "w2d_common.cuh"
#include "wave2d_cuda.h"

using namespace w2d;

struct w2d_elastic {
    int device = 0;  // CUDA device current at creation: every call on the handle runs there
    int nx = 0, nz = 0, ldx = 0, fs = 1;
    float dx = 0, dz = 0, dt = 0;
    size_t plane = 0;
    cudaStream_t st = nullptr;
    float* sponge = nullptr;  // 1 plane
    float* params = nullptr;  // S x 4 planes
    size_t params_cap = 0;
    float* state = nullptr;   // S x 5 planes
    float* adj = nullptr;     // S x 5 planes
    float* tmp = nullptr;     // S x 5 planes (t: 3 stress-like, r: 2 velocity-like)
    float* grad = nullptr;    // S x 4 planes
    size_t state_cap = 0, adj_cap = 0, tmp_cap = 0, grad_cap = 0;
    float* ckpt = nullptr;
    size_t ckpt_cap = 0;
    float* seg = nullptr;
    size_t seg_cap = 0;
    float* wav = nullptr;     // S x nt
    size_t wav_cap = 0;
    int* src_pos = nullptr;   // S x {ix, iz}
    size_t pos_cap = 0;
    int* rec = nullptr;
    int* rec_ptr = nullptr;   // receivers by column (CSR, index order within a column)
    int* rec_list = nullptr;
    size_t rec_cap = 0, rp_cap = 0, rl_cap = 0;
    float* traces = nullptr;  // S x nt x n_rec
    size_t tr_cap = 0;
    int S = 0, nt = 0, n_rec = 0, seg_len = 0, n_seg = 0, rec_iz = 0;
    bool have_forward = false;
    unsigned* err = nullptr;                // device error word of the step kernels
    CUtensorMap map_state;                  // 3D map over the S x 5 planes of `state`
    std::vector<CUtensorMap> seg_maps;      // one per slot of `seg`
    int adj_form = 1;                       // 1: TMA-tiled adjoint passes, 0: per-cell kernels
    // every shot of the next batch has the same model: its parameters are stored once and
    // read by every shot (parameter stride 0), so a tile's parameters come from L2 for
    // all but the first shot to touch them
    int shared_next = 0;
    size_t pstride = 0;                     // parameter stride per shot of the current batch
    int fwd_warps = EL_WARPS, fwd_rpw = EL_RPW;          // step kernels' tile
    int adj_warps = EL_ADJ_WARPS, adj_rpw = EL_ADJ_RPW;  // adjoint passes' tile
    // the tiles the current maps were made for (a change applies at the next forward)
    int map_fwd_warps = EL_WARPS, map_fwd_rpw = EL_RPW, map_adj_warps = EL_ADJ_WARPS,
        map_adj_rpw = EL_ADJ_RPW;
    // programmatic dependent launches: on/off, and whether the stream's last operation
    // is a kernel of the step / tiled-adjoint chain (a launch may depend on it only then)
    int pdl = 1;
    bool chain = false;
    bool last_stress = false;  // ... and that kernel was a stress phase
    CUtensorMap adj_map_tmp;                // the adjoint passes' maps (their own box height)
    std::vector<CUtensorMap> adj_seg_maps;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float last_ms = 0.f;

    size_t SS() const { return 5 * plane; }  // state stride per shot
    float* P(int shot, int i) { return params + ((size_t)shot * 4 + i) * plane; }
    ElState S0(float* base)
    {
        return ElState{base, base + plane, base + 2 * plane, base + 3 * plane, base + 4 * plane};
    }
    float* slot(int i) { return seg + (size_t)i * S * SS(); }
};

namespace {

template <typename T>
int grow(T** p, size_t n, size_t* cap)
{
    if (n <= *cap) return W2D_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    if (cudaMalloc(p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation failed");
        return W2D_ENOMEM;
    }
    *cap = n;
    return W2D_OK;
}

ElGeom egeom(w2d_elastic* e)
{
    ElGeom g;
    g.nx = e->nx;
    g.nz = e->nz;
    g.ldx = e->ldx;
    g.rdx = 1.0f / e->dx;
    g.rdz = 1.0f / e->dz;
    g.dt = e->dt;
    g.free_surface = e->fs;
    g.sponge = e->sponge;
    return g;
}

ElParams eparams(w2d_elastic* e)
{
    return ElParams{e->P(0, 0), e->P(0, 1), e->P(0, 2), e->P(0, 3), e->sponge};
}

ElStrides estrides(w2d_elastic* e)
{
    return ElStrides{e->SS(), e->pstride, 4 * e->plane};
}

// Step n of every shot from the states at src to the states at dst (same pointer:
// in place), the source term w[n] * dt added to vz at each shot's source first.
int fwd_step(w2d_elastic* e, const CUtensorMap& msrc, const CUtensorMap& mdst, const float* src,
             float* dst, int n, float* trace_row = nullptr)
{
    ElMaps m;
    m.src = msrc;
    m.dst = mdst;
    ElStep st;
    st.src = src;
    st.dst = dst;
    st.plane = e->plane;
    st.lam = e->P(0, 0);
    st.mu = e->P(0, 1);
    st.bx = e->P(0, 2);
    st.bz = e->P(0, 3);
    st.pstride = e->pstride;
    st.src_pos = e->src_pos;
    st.wav = e->wav;
    st.nt = e->nt;
    st.n = n;
    st.err = e->err;
    if (trace_row) {  // receivers sampled by the stress phase
        st.trace = trace_row;
        st.rec_ptr = e->rec_ptr;
        st.rec_list = e->rec_list;
        st.rec_iz = e->rec_iz;
        st.trace_stride = (size_t)e->nt * e->n_rec;
    }
    // the velocity phase stages its fields early after a stress phase of the chain (it
    // releases its dependents only after its own wait) or with no dependency at all
    const int pdl = e->pdl && e->chain;
    st.early = (!pdl || e->last_stress) ? 1 : 0;
    W2D_CUDA_TRY(launch_elastic_step(egeom(e), m, st, e->st, e->S, e->map_fwd_warps,
                                     e->map_fwd_rpw, pdl));
    e->chain = true;
    e->last_stress = true;
    return W2D_OK;
}

int check_el_err(w2d_elastic* e)
{
    unsigned h = 0;
    W2D_CUDA_TRY(cudaMemcpyAsync(&h, e->err, 4, cudaMemcpyDeviceToHost, e->st));
    W2D_CUDA_TRY(cudaStreamSynchronize(e->st));
    if (h) {
        cudaMemsetAsync(e->err, 0, 4, e->st);
        set_error("elastic step: a tile load did not complete");
        return W2D_ETIMEOUT;
    }
    return W2D_OK;
}

bool on_m(const w2d_elastic* e, int iz, int ix)
{
    return iz >= (e->fs ? 1 : 2) && iz < e->nz - 2 && ix >= 2 && ix < e->nx - 2;
}

// checkpoint segments: about sqrt(3 nt) steps each
void plan_segments(int nt, int* seg_len, int* n_seg)
{
    *seg_len = std::max(1, (int)sqrt(3.0 * nt));
    *n_seg = (nt + *seg_len - 1) / *seg_len;
}

}  // namespace

extern "C" {

int w2d_elastic_create(w2d_elastic** out, int nx, int nz, float dx, float dz, double dt,
                       int n_sponge, float sponge_alpha, int free_surface_top)
{
    W2D_CHECK_ARG(out && nx >= 5 && nz >= 5 && dx > 0 && dz > 0 && dt > 0, "bad arguments");
    *out = nullptr;
    w2d_elastic* e = new w2d_elastic();
    e->device = current_device();
    e->nx = nx;
    e->nz = nz;
    e->ldx = pitch_for(nx);
    e->plane = (size_t)e->ldx * nz;
    e->dx = dx;
    e->dz = dz;
    e->dt = (float)dt;
    e->fs = free_surface_top ? 1 : 0;
    auto fail = [&](int rc) {
        w2d_elastic_destroy(e);
        return rc;
    };
    const size_t pb = e->plane * 4;
    if (cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) ||
        cudaEventCreate(&e->e0) || cudaEventCreate(&e->e1) || cudaMalloc(&e->sponge, pb) ||
        cudaMalloc(&e->err, sizeof(unsigned))) {
        cudaGetLastError();
        set_error("elastic engine allocation failed");
        return fail(W2D_ENOMEM);
    }
    std::vector<float> sp((size_t)nx * nz);
    build_cerjan_sponge(sp.data(), nx, nz, n_sponge, sponge_alpha, e->fs);
    if (cudaMemset(e->sponge, 0, pb) || cudaMemset(e->err, 0, sizeof(unsigned)) ||
        cudaMemcpy2D(e->sponge, (size_t)e->ldx * 4, sp.data(), (size_t)nx * 4, (size_t)nx * 4, nz,
                     cudaMemcpyHostToDevice)) {
        set_error("elastic engine set-up failed");
        return fail(W2D_ECUDA);
    }
    *out = e;
    return W2D_OK;
}

void w2d_elastic_destroy(w2d_elastic* e)
{
    W2D_ON_DEVICE_OF(e);
    if (!e) return;
    if (e->st) cudaStreamSynchronize(e->st);
    for (void* p : {(void*)e->sponge, (void*)e->params, (void*)e->state, (void*)e->adj,
                    (void*)e->tmp, (void*)e->grad, (void*)e->ckpt, (void*)e->seg, (void*)e->wav,
                    (void*)e->src_pos, (void*)e->rec, (void*)e->rec_ptr, (void*)e->rec_list,
                    (void*)e->traces, (void*)e->err})
        if (p) cudaFree(p);
    if (e->e0) cudaEventDestroy(e->e0);
    if (e->e1) cudaEventDestroy(e->e1);
    if (e->st) cudaStreamDestroy(e->st);
    delete e;
}

unsigned long long w2d_elastic_shot_bytes(int nx, int nz, int nt, int n_rec)
{
    if (nx < 5 || nz < 5 || nt <= 0) return 0;
    int seg_len = 0, n_seg = 0;
    plan_segments(nt, &seg_len, &n_seg);
    const size_t plane = (size_t)pitch_for(nx) * nz;
    // params 4, state 5, adj 5, tmp 5, grad 4, checkpoints, one segment of states
    const size_t planes = 4 + 5 + 5 + 5 + 4 + (size_t)n_seg * 5 + (size_t)(seg_len + 1) * 5;
    return (unsigned long long)(planes * plane * 4 + (size_t)nt * 4 +
                                (size_t)nt * std::max(n_rec, 1) * 4 + 64);
}

// lam, mu, bx, bz: DEVICE arrays, n_shots x (nz, nx) contiguous.  wavelets: HOST
// (n_shots, nt); src_ix, src_iz: HOST n_shots each; rec_ix: HOST n_rec (shared).
// traces_dev: DEVICE (n_shots, nt, n_rec) vertical strain.  Keeps checkpoints.
int w2d_elastic_forward_batch(w2d_elastic* e, int n_shots, const float* lam, const float* mu,
                              const float* bx, const float* bz, const float* wavelets, int nt,
                              const int* src_ix, const int* src_iz, const int* rec_ix, int n_rec,
                              int rec_iz, float* traces_dev)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && lam && mu && bx && bz && wavelets && traces_dev && nt > 0, "bad arguments");
    W2D_CHECK_ARG(n_shots >= 1 && n_shots <= 65535 && src_ix && src_iz, "bad shot count");
    W2D_CHECK_ARG(n_rec > 0 && rec_ix, "receivers required");
    W2D_CHECK_DEVICE_PTR(lam, e->device);
    W2D_CHECK_DEVICE_PTR(mu, e->device);
    W2D_CHECK_DEVICE_PTR(bx, e->device);
    W2D_CHECK_DEVICE_PTR(bz, e->device);
    W2D_CHECK_DEVICE_PTR(traces_dev, e->device);
    for (int s = 0; s < n_shots; ++s)
        W2D_CHECK_ARG(src_ix[s] >= 0 && src_ix[s] < e->nx && src_iz[s] >= 0 && src_iz[s] < e->nz &&
                          on_m(e, src_iz[s], src_ix[s]),
                      "the source must sit on an updated cell");
    W2D_CHECK_ARG(rec_iz >= 0 && rec_iz < e->nz, "receiver_iz out of range");
    for (int k = 0; k < n_rec; ++k)
        W2D_CHECK_ARG(rec_ix[k] >= 2 && rec_ix[k] < e->nx - 2, "receiver_ix must be in [2, nx-2)");
    int rc;
    const int S = n_shots;
    e->have_forward = false;
    e->S = S;
    e->nt = nt;
    e->n_rec = n_rec;
    e->rec_iz = rec_iz;
    plan_segments(nt, &e->seg_len, &e->n_seg);
    const size_t P = e->plane, SS = e->SS();
    if ((rc = grow(&e->params, (size_t)S * 4 * P, &e->params_cap)) ||
        (rc = grow(&e->state, (size_t)S * SS, &e->state_cap)) ||
        (rc = grow(&e->adj, (size_t)S * SS, &e->adj_cap)) ||
        (rc = grow(&e->tmp, (size_t)S * SS, &e->tmp_cap)) ||
        (rc = grow(&e->grad, (size_t)S * 4 * P, &e->grad_cap)) ||
        (rc = grow(&e->wav, (size_t)S * nt, &e->wav_cap)) ||
        (rc = grow(&e->src_pos, (size_t)S * 2, &e->pos_cap)) ||
        (rc = grow(&e->rec, (size_t)n_rec, &e->rec_cap)) ||
        (rc = grow(&e->traces, (size_t)S * nt * n_rec, &e->tr_cap)) ||
        (rc = grow(&e->rec_ptr, (size_t)e->nx + 1, &e->rp_cap)) ||
        (rc = grow(&e->rec_list, (size_t)n_rec, &e->rl_cap)) ||
        (rc = grow(&e->ckpt, (size_t)e->n_seg * S * SS, &e->ckpt_cap)) ||
        (rc = grow(&e->seg, (size_t)(e->seg_len + 1) * S * SS, &e->seg_cap)))
        return rc;
    e->map_fwd_warps = e->fwd_warps;
    e->map_fwd_rpw = e->fwd_rpw;
    e->map_adj_warps = e->adj_warps;
    e->map_adj_rpw = e->adj_rpw;
    const int ftz = e->fwd_warps * e->fwd_rpw, atz = e->adj_warps * e->adj_rpw;
    if ((rc = make_el_state_map(&e->map_state, e->state, e->nx, e->nz, e->ldx, P, S, ftz)))
        return rc;
    e->seg_maps.resize(e->seg_len + 1);
    for (int i = 0; i <= e->seg_len; ++i)
        if ((rc = make_el_state_map(&e->seg_maps[i], e->slot(i), e->nx, e->nz, e->ldx, P, S, ftz)))
            return rc;
    if ((rc = make_el_adj_map(&e->adj_map_tmp, e->tmp, e->nx, e->nz, e->ldx, P, S, atz)))
        return rc;
    e->adj_seg_maps.resize(e->seg_len + 1);
    for (int i = 0; i <= e->seg_len; ++i)
        if ((rc = make_el_adj_map(&e->adj_seg_maps[i], e->slot(i), e->nx, e->nz, e->ldx, P, S,
                                  atz)))
            return rc;
    const size_t hp = (size_t)e->nx * 4, dp = (size_t)e->ldx * 4, np = (size_t)e->nx * e->nz;
    const float* src[4] = {lam, mu, bx, bz};
    const int n_models = e->shared_next ? 1 : S;
    e->pstride = e->shared_next ? 0 : 4 * P;
    e->shared_next = 0;  // one batch only
    for (int s = 0; s < n_models; ++s)
        for (int i = 0; i < 4; ++i)
            W2D_CUDA_TRY(cudaMemcpy2DAsync(e->P(s, i), dp, src[i] + (size_t)s * np, hp, hp, e->nz,
                                           cudaMemcpyDeviceToDevice, e->st));
    W2D_CUDA_TRY(cudaMemcpyAsync(e->wav, wavelets, (size_t)S * nt * 4, cudaMemcpyHostToDevice,
                                 e->st));
    W2D_CUDA_TRY(cudaMemcpyAsync(e->rec, rec_ix, (size_t)n_rec * 4, cudaMemcpyHostToDevice, e->st));
    {
        std::vector<int> pos(2 * S);
        for (int s = 0; s < S; ++s) {
            pos[2 * s] = src_ix[s];
            pos[2 * s + 1] = src_iz[s];
        }
        // receivers by column for the adjoint of the sampling
        std::vector<int> ptr(e->nx + 1, 0), list(n_rec);
        for (int k = 0; k < n_rec; ++k) ptr[rec_ix[k] + 1]++;
        for (int i = 0; i < e->nx; ++i) ptr[i + 1] += ptr[i];
        std::vector<int> fill(ptr.begin(), ptr.end() - 1);
        for (int k = 0; k < n_rec; ++k) list[fill[rec_ix[k]]++] = k;
        W2D_CUDA_TRY(cudaMemcpyAsync(e->src_pos, pos.data(), pos.size() * 4,
                                     cudaMemcpyHostToDevice, e->st));
        W2D_CUDA_TRY(cudaMemcpyAsync(e->rec_ptr, ptr.data(), ptr.size() * 4,
                                     cudaMemcpyHostToDevice, e->st));
        W2D_CUDA_TRY(cudaMemcpyAsync(e->rec_list, list.data(), list.size() * 4,
                                     cudaMemcpyHostToDevice, e->st));
        W2D_CUDA_TRY(cudaStreamSynchronize(e->st));  // the host tables die here
    }
    W2D_CUDA_TRY(cudaMemsetAsync(e->state, 0, (size_t)S * SS * 4, e->st));
    W2D_CUDA_TRY(cudaEventRecord(e->e0, e->st));
    e->chain = false;
    for (int n = 0; n < nt; ++n) {
        if (n % e->seg_len == 0) {
            W2D_CUDA_TRY(cudaMemcpyAsync(e->ckpt + (size_t)(n / e->seg_len) * S * SS, e->state,
                                         (size_t)S * SS * 4, cudaMemcpyDeviceToDevice, e->st));
            e->chain = false;
        }
        if ((rc = fwd_step(e, e->map_state, e->map_state, e->state, e->state, n,
                           e->traces + (size_t)n * n_rec)))
            return rc;
    }
    e->chain = false;
    W2D_CUDA_TRY(cudaGetLastError());
    W2D_CUDA_TRY(cudaEventRecord(e->e1, e->st));
    W2D_CUDA_TRY(cudaMemcpyAsync(traces_dev, e->traces, (size_t)S * nt * n_rec * 4,
                                 cudaMemcpyDeviceToDevice, e->st));
    W2D_CUDA_TRY(cudaStreamSynchronize(e->st));
    if ((rc = check_el_err(e))) return rc;
    cudaEventElapsedTime(&e->last_ms, e->e0, e->e1);
    e->have_forward = true;
    return W2D_OK;
}

int w2d_elastic_forward(w2d_elastic* e, const float* lam, const float* mu, const float* bx,
                        const float* bz, const float* wavelet, int nt, int src_ix, int src_iz,
                        const int* rec_ix, int n_rec, int rec_iz, float* traces_dev)
{
    W2D_ON_DEVICE_OF(e);
    return w2d_elastic_forward_batch(e, 1, lam, mu, bx, bz, wavelet, nt, &src_ix, &src_iz, rec_ix,
                                     n_rec, rec_iz, traces_dev);
}

// resid_dev: DEVICE (n_shots, nt, n_rec) = dJ/d(traces) of the last forward batch.
// Gradients: DEVICE n_shots x (nz, nx) contiguous, one per shot (any may be NULL).
int w2d_elastic_gradient_batch(w2d_elastic* e, const float* resid_dev, float* g_lam, float* g_mu,
                               float* g_bx, float* g_bz)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && e->have_forward && resid_dev, "call w2d_elastic_forward first");
    W2D_CHECK_DEVICE_PTR(resid_dev, e->device);
    W2D_CHECK_DEVICE_PTR(g_lam, e->device);
    W2D_CHECK_DEVICE_PTR(g_mu, e->device);
    W2D_CHECK_DEVICE_PTR(g_bx, e->device);
    W2D_CHECK_DEVICE_PTR(g_bz, e->device);
    const int nt = e->nt, n_rec = e->n_rec, S = e->S;
    const size_t P = e->plane, pb = P * 4, SS = e->SS();
    const size_t tr_stride = (size_t)nt * n_rec;
    W2D_CUDA_TRY(cudaMemcpyAsync(e->traces, resid_dev, (size_t)S * tr_stride * 4,
                                 cudaMemcpyDeviceToDevice, e->st));
    W2D_CUDA_TRY(cudaMemsetAsync(e->adj, 0, (size_t)S * SS * 4, e->st));
    W2D_CUDA_TRY(cudaMemsetAsync(e->tmp, 0, (size_t)S * SS * 4, e->st));
    W2D_CUDA_TRY(cudaMemsetAsync(e->grad, 0, (size_t)S * 4 * pb, e->st));
    W2D_CUDA_TRY(cudaEventRecord(e->e0, e->st));
    const ElGeom g = egeom(e);
    const ElParams prm = eparams(e);
    const ElStrides sd = estrides(e);
    ElState a = e->S0(e->adj);
    ElState t{e->tmp, e->tmp, e->tmp + 2 * P, e->tmp + 3 * P, e->tmp + 4 * P};  // sxx,szz,sxz used
    ElState r{e->tmp, e->tmp + P, nullptr, nullptr, nullptr};                     // vx,vz used
    float *glam = e->grad, *gmu = e->grad + P, *gbx = e->grad + 2 * P, *gbz = e->grad + 3 * P;
    dim3 blk(32, 8), grd((e->nx + 31) / 32, (e->nz + 7) / 8, S);
    const dim3 rgrid((e->nx + 127) / 128, S);
    // adjoint of u_nt: residual of the last trace row (the tiled pass A adds each
    // step's row itself)
    if (e->adj_form != 1)
        el_adj_receivers<<<rgrid, 128, 0, e->st>>>(g, a.vz, SS, e->rec_ptr, e->rec_list,
                                                   e->rec_iz, e->traces + (size_t)(nt - 1) * n_rec,
                                                   tr_stride);
    // K1 of the last step; every later K1 runs inside the K4 of the step after it
    el_adj_k1<<<grd, blk, 0, e->st>>>(g, prm, sd, a, t);
    for (int sgi = e->n_seg - 1; sgi >= 0; --sgi) {
        const int a0 = sgi * e->seg_len, b0 = std::min(nt, a0 + e->seg_len);
        // recompute u_a0 .. u_b0 into the segment slots
        W2D_CUDA_TRY(cudaMemcpyAsync(e->slot(0), e->ckpt + (size_t)sgi * S * SS, (size_t)S * SS * 4,
                                     cudaMemcpyDeviceToDevice, e->st));
        e->chain = false;
        // out of place: slot n - a0 keeps u_n (without the w[n] source term)
        for (int n = a0; n < b0; ++n) {
            const int i = n - a0;
            int rc;
            if ((rc = fwd_step(e, e->seg_maps[i], e->seg_maps[i + 1], e->slot(i), e->slot(i + 1),
                               n)))
                return rc;
        }
        for (int n = b0 - 1; n >= a0; --n) {
            if (e->adj_form == 1) {
                ElAdjMaps m;
                m.tmp = e->adj_map_tmp;
                m.f_next = e->adj_seg_maps[n + 1 - a0];
                m.f_curr = e->adj_seg_maps[n - a0];
                const ElAdjRecv rv{e->traces + (size_t)n * n_rec, tr_stride, e->rec_ptr,
                                   e->rec_list, e->rec_iz};
                W2D_CUDA_TRY(launch_el_adj_a(m, g, prm, sd, a, r, glam, gmu, gbx, gbz, rv, e->err,
                                             S, e->st, e->map_adj_warps, e->map_adj_rpw,
                                             e->pdl && e->chain));
                W2D_CUDA_TRY(launch_el_adj_b(m, g, prm, sd, a, t, n >= 1 ? 1 : 0, e->err, S,
                                             e->st, e->map_adj_warps, e->map_adj_rpw, e->pdl));
                e->chain = true;
                e->last_stress = false;
            } else {
                e->chain = false;
                ElState f_next = e->S0(e->slot(n + 1 - a0));  // u_{n+1}
                ElState f_curr = e->S0(e->slot(n - a0));      // u_n
                el_adj_k23<<<grd, blk, 0, e->st>>>(g, prm, sd, a, t, r, f_next, f_curr, glam, gmu,
                                                   gbx, gbz);
                el_adj_k4<<<grd, blk, 0, e->st>>>(g, prm, sd, a, r, t, n >= 1 ? 1 : 0);
                if (n >= 1)
                    el_adj_receivers<<<rgrid, 128, 0, e->st>>>(
                        g, a.vz, SS, e->rec_ptr, e->rec_list, e->rec_iz,
                        e->traces + (size_t)(n - 1) * n_rec, tr_stride);
            }
        }
    }
    e->chain = false;
    W2D_CUDA_TRY(cudaGetLastError());
    W2D_CUDA_TRY(cudaEventRecord(e->e1, e->st));
    float* outs[4] = {g_lam, g_mu, g_bx, g_bz};
    const size_t hp = (size_t)e->nx * 4, dp = (size_t)e->ldx * 4, np = (size_t)e->nx * e->nz;
    for (int s = 0; s < S; ++s)
        for (int i = 0; i < 4; ++i)
            if (outs[i])
                W2D_CUDA_TRY(cudaMemcpy2DAsync(outs[i] + (size_t)s * np, hp,
                                               e->grad + ((size_t)s * 4 + i) * P, dp, hp, e->nz,
                                               cudaMemcpyDeviceToDevice, e->st));
    W2D_CUDA_TRY(cudaStreamSynchronize(e->st));
    int rc;
    if ((rc = check_el_err(e))) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e->e0, e->e1);
    e->last_ms = ms;
    return W2D_OK;
}

int w2d_elastic_gradient(w2d_elastic* e, const float* resid_dev, float* g_lam, float* g_mu,
                         float* g_bx, float* g_bz)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && e->S == 1, "the last forward call was a batch: use the batch gradient");
    return w2d_elastic_gradient_batch(e, resid_dev, g_lam, g_mu, g_bx, g_bz);
}

int w2d_elastic_set_adjoint(w2d_elastic* e, int form)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e && (form == 0 || form == 1), "form must be 0 (per-cell) or 1 (tiled)");
    e->adj_form = form;
    return W2D_OK;
}

int w2d_elastic_share_model(w2d_elastic* e, int on)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    e->shared_next = on ? 1 : 0;
    return W2D_OK;
}

int w2d_elastic_set_pdl(w2d_elastic* e, int on)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    e->pdl = on ? 1 : 0;
    return W2D_OK;
}

int w2d_elastic_set_tiles(w2d_elastic* e, int step_warps, int step_rows_per_warp,
                          int adjoint_warps, int adjoint_rows_per_warp)
{
    W2D_ON_DEVICE_OF(e);
    W2D_CHECK_ARG(e, "engine is NULL");
    W2D_CHECK_ARG(el_tile_supported(step_warps, step_rows_per_warp),
                  "step tile must be 4x4, 4x2, 8x2 or 8x1 (warps x rows per warp)");
    W2D_CHECK_ARG(el_adj_tile_supported(adjoint_warps, adjoint_rows_per_warp),
                  "adjoint tile must be 4x2, 4x1 or 8x1 (warps x rows per warp)");
    e->fwd_warps = step_warps;
    e->fwd_rpw = step_rows_per_warp;
    e->adj_warps = adjoint_warps;
    e->adj_rpw = adjoint_rows_per_warp;
    return W2D_OK;
}

float w2d_elastic_last_ms(w2d_elastic* e) { return e ? e->last_ms : 0.f; }

}  // extern "C"
