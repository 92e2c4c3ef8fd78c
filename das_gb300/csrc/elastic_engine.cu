// elastic_engine.cu -- elastic modelling with vertical-strain receivers and its
// adjoint (gradients with respect to lambda, mu and the buoyancies), forward state
// recovered from checkpoints.  See elastic_adjoint_kernels.cuh for the scheme.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "elastic_adjoint_kernels.cuh"
#include "small_kernels.cuh"
#include "w2d_common.cuh"
#include "wave2d_cuda.h"

using namespace w2d;

struct w2d_elastic {
    int nx = 0, nz = 0, ldx = 0, fs = 1;
    float dx = 0, dz = 0, dt = 0;
    size_t plane = 0;
    cudaStream_t st = nullptr;
    float* params = nullptr;  // lam, mu, bx, bz, sponge (5 planes)
    float* state = nullptr;   // 5 planes
    float* adj = nullptr;     // 5 planes
    float* tmp = nullptr;     // 5 planes (t: 3 stress-like, r: 2 velocity-like)
    float* grad = nullptr;    // 4 planes
    float* ckpt = nullptr;
    size_t ckpt_planes = 0;
    float* seg = nullptr;
    size_t seg_planes = 0;
    float* wavelet = nullptr;
    int w_cap = 0;
    int* rec = nullptr;
    int* rec_ptr = nullptr;   // receivers by column (CSR, index order within a column)
    int* rec_list = nullptr;
    int rec_cap = 0;
    float* traces = nullptr;
    size_t tr_cap = 0;
    size_t rp_cap = 0, rl_cap = 0;
    int nt = 0, n_rec = 0, seg_len = 0, n_seg = 0, src_ix = 0, src_iz = 0, rec_iz = 0;
    bool have_forward = false;
    unsigned* err = nullptr;                // device error word of the step kernels
    CUtensorMap map_state;                  // 3D map over the 5 planes of `state`
    std::vector<CUtensorMap> seg_maps;      // one per state slot of `seg`
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float last_ms = 0.f;

    float* P(int i) { return params + (size_t)i * plane; }
    ElState S(float* base)
    {
        return ElState{base, base + plane, base + 2 * plane, base + 3 * plane, base + 4 * plane};
    }
};

namespace {

template <typename T>
int grow(T** p, size_t n, size_t* cap)
{
    if (n <= *cap) return W2D_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    if (cudaMalloc(p, n * sizeof(T)) != cudaSuccess) {
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
    g.sponge = e->P(4);
    return g;
}

// Step n from the state at src to the state at dst (same pointer: in place), with
// the source term w[n] * dt added to vz at the source cell first.
int fwd_step(w2d_elastic* e, const CUtensorMap& msrc, const CUtensorMap& mdst, const float* src,
             float* dst, int n)
{
    ElMaps m;
    m.src = msrc;
    m.dst = mdst;
    ElStep st;
    st.src = src;
    st.dst = dst;
    st.plane = e->plane;
    st.lam = e->P(0);
    st.mu = e->P(1);
    st.bx = e->P(2);
    st.bz = e->P(3);
    st.inj_ix = e->src_ix;
    st.inj_iz = e->src_iz;
    st.inj_w = e->wavelet + n;
    st.err = e->err;
    W2D_CUDA_TRY(launch_elastic_step(egeom(e), m, st, e->st));
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


}  // namespace

extern "C" {

int w2d_elastic_create(w2d_elastic** out, int nx, int nz, float dx, float dz, double dt,
                       int n_sponge, float sponge_alpha, int free_surface_top)
{
    W2D_CHECK_ARG(out && nx >= 5 && nz >= 5 && dx > 0 && dz > 0 && dt > 0, "bad arguments");
    *out = nullptr;
    w2d_elastic* e = new w2d_elastic();
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
        cudaEventCreate(&e->e0) || cudaEventCreate(&e->e1) ||
        cudaMalloc(&e->params, 5 * pb) || cudaMalloc(&e->state, 5 * pb) ||
        cudaMalloc(&e->adj, 5 * pb) || cudaMalloc(&e->tmp, 5 * pb) ||
        cudaMalloc(&e->grad, 4 * pb) || cudaMalloc(&e->err, sizeof(unsigned))) {
        cudaGetLastError();
        set_error("elastic engine allocation failed");
        return fail(W2D_ENOMEM);
    }
    std::vector<float> sp((size_t)nx * nz);
    build_cerjan_sponge(sp.data(), nx, nz, n_sponge, sponge_alpha, e->fs);
    if (cudaMemset(e->params, 0, 5 * pb) || cudaMemset(e->err, 0, sizeof(unsigned)) ||
        cudaMemcpy2D(e->P(4), (size_t)e->ldx * 4, sp.data(), (size_t)nx * 4, (size_t)nx * 4, nz,
                     cudaMemcpyHostToDevice)) {
        set_error("elastic engine set-up failed");
        return fail(W2D_ECUDA);
    }
    int rc;
    if ((rc = make_el_state_map(&e->map_state, e->state, nx, nz, e->ldx, e->plane)))
        return fail(rc);
    *out = e;
    return W2D_OK;
}

void w2d_elastic_destroy(w2d_elastic* e)
{
    if (!e) return;
    if (e->st) cudaStreamSynchronize(e->st);
    for (void* p : {(void*)e->params, (void*)e->state, (void*)e->adj, (void*)e->tmp,
                    (void*)e->grad, (void*)e->ckpt, (void*)e->seg, (void*)e->wavelet,
                    (void*)e->rec, (void*)e->rec_ptr, (void*)e->rec_list, (void*)e->traces,
                    (void*)e->err})
        if (p) cudaFree(p);
    if (e->e0) cudaEventDestroy(e->e0);
    if (e->e1) cudaEventDestroy(e->e1);
    if (e->st) cudaStreamDestroy(e->st);
    delete e;
}

// lam, mu, bx, bz: DEVICE arrays, contiguous (nz, nx).  wavelet, rec_ix: HOST.
// traces_dev: DEVICE (nt, n_rec) vertical strain.  Keeps checkpoints for the gradient.
int w2d_elastic_forward(w2d_elastic* e, const float* lam, const float* mu, const float* bx,
                        const float* bz, const float* wavelet, int nt, int src_ix, int src_iz,
                        const int* rec_ix, int n_rec, int rec_iz, float* traces_dev)
{
    W2D_CHECK_ARG(e && lam && mu && bx && bz && wavelet && traces_dev && nt > 0, "bad arguments");
    W2D_CHECK_ARG(n_rec > 0 && rec_ix, "receivers required");
    W2D_CHECK_ARG(src_ix >= 0 && src_ix < e->nx && src_iz >= 0 && src_iz < e->nz &&
                      on_m(e, src_iz, src_ix),
                  "the source must sit on an updated cell");
    W2D_CHECK_ARG(rec_iz >= 0 && rec_iz < e->nz, "receiver_iz out of range");
    for (int k = 0; k < n_rec; ++k)
        W2D_CHECK_ARG(rec_ix[k] >= 2 && rec_ix[k] < e->nx - 2, "receiver_ix must be in [2, nx-2)");
    int rc;
    e->nt = nt;
    e->n_rec = n_rec;
    e->src_ix = src_ix;
    e->src_iz = src_iz;
    e->rec_iz = rec_iz;
    e->seg_len = std::max(1, (int)sqrt(3.0 * nt));
    e->n_seg = (nt + e->seg_len - 1) / e->seg_len;
    size_t wc = e->w_cap, rcap = e->rec_cap;
    if ((rc = grow(&e->wavelet, (size_t)nt, &wc)) || (rc = grow(&e->rec, (size_t)n_rec, &rcap)) ||
        (rc = grow(&e->traces, (size_t)nt * n_rec, &e->tr_cap)) ||
        (rc = grow(&e->rec_ptr, (size_t)e->nx + 1, &e->rp_cap)) ||
        (rc = grow(&e->rec_list, (size_t)n_rec, &e->rl_cap)) ||
        (rc = grow(&e->ckpt, (size_t)e->n_seg * 5 * e->plane, &e->ckpt_planes)) ||
        (rc = grow(&e->seg, (size_t)(e->seg_len + 1) * 5 * e->plane, &e->seg_planes)))
        return rc;
    e->w_cap = (int)wc;
    e->rec_cap = (int)rcap;
    e->seg_maps.resize(e->seg_len + 1);
    for (int i = 0; i <= e->seg_len; ++i)
        if ((rc = make_el_state_map(&e->seg_maps[i], e->seg + (size_t)i * 5 * e->plane, e->nx,
                                    e->nz, e->ldx, e->plane)))
            return rc;
    const size_t hp = (size_t)e->nx * 4, dp = (size_t)e->ldx * 4;
    const float* src[4] = {lam, mu, bx, bz};
    for (int i = 0; i < 4; ++i)
        W2D_CUDA_TRY(cudaMemcpy2DAsync(e->P(i), dp, src[i], hp, hp, e->nz, cudaMemcpyDeviceToDevice,
                                       e->st));
    W2D_CUDA_TRY(cudaMemcpyAsync(e->wavelet, wavelet, (size_t)nt * 4, cudaMemcpyHostToDevice, e->st));
    W2D_CUDA_TRY(cudaMemcpyAsync(e->rec, rec_ix, (size_t)n_rec * 4, cudaMemcpyHostToDevice, e->st));
    {
        // receivers by column for the adjoint of the sampling
        std::vector<int> ptr(e->nx + 1, 0), list(n_rec);
        for (int k = 0; k < n_rec; ++k) ptr[rec_ix[k] + 1]++;
        for (int i = 0; i < e->nx; ++i) ptr[i + 1] += ptr[i];
        std::vector<int> fill(ptr.begin(), ptr.end() - 1);
        for (int k = 0; k < n_rec; ++k) list[fill[rec_ix[k]]++] = k;
        W2D_CUDA_TRY(cudaMemcpyAsync(e->rec_ptr, ptr.data(), ptr.size() * 4,
                                     cudaMemcpyHostToDevice, e->st));
        W2D_CUDA_TRY(cudaMemcpyAsync(e->rec_list, list.data(), list.size() * 4,
                                     cudaMemcpyHostToDevice, e->st));
        W2D_CUDA_TRY(cudaStreamSynchronize(e->st));  // the host tables die here
    }
    W2D_CUDA_TRY(cudaMemsetAsync(e->state, 0, 5 * e->plane * 4, e->st));
    W2D_CUDA_TRY(cudaEventRecord(e->e0, e->st));
    const ElGeom g = egeom(e);
    const ElState s = e->S(e->state);
    for (int n = 0; n < nt; ++n) {
        if (n % e->seg_len == 0)
            W2D_CUDA_TRY(cudaMemcpyAsync(e->ckpt + (size_t)(n / e->seg_len) * 5 * e->plane, e->state,
                                         5 * e->plane * 4, cudaMemcpyDeviceToDevice, e->st));
        if ((rc = fwd_step(e, e->map_state, e->map_state, e->state, e->state, n))) return rc;
        el_sample_kernel<<<(n_rec + 127) / 128, 128, 0, e->st>>>(g, s.vz, e->rec, n_rec, rec_iz,
                                                                 e->traces + (size_t)n * n_rec);
    }
    W2D_CUDA_TRY(cudaGetLastError());
    W2D_CUDA_TRY(cudaEventRecord(e->e1, e->st));
    W2D_CUDA_TRY(cudaMemcpyAsync(traces_dev, e->traces, (size_t)nt * n_rec * 4,
                                 cudaMemcpyDeviceToDevice, e->st));
    W2D_CUDA_TRY(cudaStreamSynchronize(e->st));
    if ((rc = check_el_err(e))) return rc;
    cudaEventElapsedTime(&e->last_ms, e->e0, e->e1);
    e->have_forward = true;
    return W2D_OK;
}

// resid_dev: DEVICE (nt, n_rec) = dJ/d(traces).  Gradients: DEVICE (nz, nx) contiguous
// (any may be NULL).
int w2d_elastic_gradient(w2d_elastic* e, const float* resid_dev, float* g_lam, float* g_mu,
                         float* g_bx, float* g_bz)
{
    W2D_CHECK_ARG(e && e->have_forward && resid_dev, "call w2d_elastic_forward first");
    const int nt = e->nt, n_rec = e->n_rec;
    const size_t P = e->plane, pb = P * 4;
    W2D_CUDA_TRY(cudaMemcpyAsync(e->traces, resid_dev, (size_t)nt * n_rec * 4,
                                 cudaMemcpyDeviceToDevice, e->st));
    W2D_CUDA_TRY(cudaMemsetAsync(e->adj, 0, 5 * pb, e->st));
    W2D_CUDA_TRY(cudaMemsetAsync(e->tmp, 0, 5 * pb, e->st));
    W2D_CUDA_TRY(cudaMemsetAsync(e->grad, 0, 4 * pb, e->st));
    W2D_CUDA_TRY(cudaEventRecord(e->e0, e->st));
    const ElGeom g = egeom(e);
    ElParams prm{e->P(0), e->P(1), e->P(2), e->P(3), e->P(4)};
    ElState a = e->S(e->adj);
    ElState t{e->tmp, e->tmp, e->tmp + 2 * P, e->tmp + 3 * P, e->tmp + 4 * P};  // sxx,szz,sxz used
    ElState r{e->tmp, e->tmp + P, nullptr, nullptr, nullptr};                     // vx,vz used
    float *glam = e->grad, *gmu = e->grad + P, *gbx = e->grad + 2 * P, *gbz = e->grad + 3 * P;
    dim3 blk(32, 8), grd((e->nx + 31) / 32, (e->nz + 7) / 8);
    // adjoint of u_nt: residual of the last trace row
    const int rb = (e->nx + 127) / 128;
    el_adj_receivers<<<rb, 128, 0, e->st>>>(g, a.vz, e->rec_ptr, e->rec_list, e->rec_iz,
                                            e->traces + (size_t)(nt - 1) * n_rec);
    // K1 of the last step; every later K1 runs inside the K4 of the step after it
    el_adj_k1<<<grd, blk, 0, e->st>>>(g, prm, a, t);
    for (int sgi = e->n_seg - 1; sgi >= 0; --sgi) {
        const int a0 = sgi * e->seg_len, b0 = std::min(nt, a0 + e->seg_len);
        // recompute u_a0 .. u_b0 into the segment buffer
        float* slot0 = e->seg;
        W2D_CUDA_TRY(cudaMemcpyAsync(slot0, e->ckpt + (size_t)sgi * 5 * P, 5 * pb,
                                     cudaMemcpyDeviceToDevice, e->st));
        // out of place: slot n - a0 keeps u_n (without the w[n] source term)
        for (int n = a0; n < b0; ++n) {
            const int i = n - a0;
            int rc;
            if ((rc = fwd_step(e, e->seg_maps[i], e->seg_maps[i + 1], e->seg + (size_t)i * 5 * P,
                               e->seg + (size_t)(i + 1) * 5 * P, n)))
                return rc;
        }
        for (int n = b0 - 1; n >= a0; --n) {
            ElState f_next = e->S(e->seg + (size_t)(n + 1 - a0) * 5 * P);  // u_{n+1}
            ElState f_curr = e->S(e->seg + (size_t)(n - a0) * 5 * P);      // u_n
            el_adj_k23<<<grd, blk, 0, e->st>>>(g, prm, a, t, r, f_next, f_curr, glam, gmu, gbx,
                                               gbz);
            el_adj_k4<<<grd, blk, 0, e->st>>>(g, prm, a, r, t, n >= 1 ? 1 : 0);
            if (n >= 1)
                el_adj_receivers<<<rb, 128, 0, e->st>>>(g, a.vz, e->rec_ptr, e->rec_list,
                                                        e->rec_iz,
                                                        e->traces + (size_t)(n - 1) * n_rec);
        }
    }
    W2D_CUDA_TRY(cudaGetLastError());
    W2D_CUDA_TRY(cudaEventRecord(e->e1, e->st));
    float* outs[4] = {g_lam, g_mu, g_bx, g_bz};
    const size_t hp = (size_t)e->nx * 4, dp = (size_t)e->ldx * 4;
    for (int i = 0; i < 4; ++i)
        if (outs[i])
            W2D_CUDA_TRY(cudaMemcpy2DAsync(outs[i], hp, e->grad + (size_t)i * P, dp, hp, e->nz,
                                           cudaMemcpyDeviceToDevice, e->st));
    W2D_CUDA_TRY(cudaStreamSynchronize(e->st));
    int rc;
    if ((rc = check_el_err(e))) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e->e0, e->e1);
    e->last_ms = ms;
    return W2D_OK;
}

float w2d_elastic_last_ms(w2d_elastic* e) { return e ? e->last_ms : 0.f; }

}  // extern "C"
