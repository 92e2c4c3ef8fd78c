// batch.cu -- batched / continuously fed RTM engine on one GPU.
//
// Shots of different grid sizes and lengths are admitted into a device memory
// arena (admission by memory budget: a shot is taken when its wavefields,
// snapshot store, models and inputs fit), advanced together by the kernels of
// batch_kernels.cuh, and retired as soon as their last phase step ends.  One
// "replay" advances every active shot by S * chunks phase steps: in the grid form
// (default) as S * chunks launches of one phase step each over all active shots'
// tiles, chained as programmatic dependents, plus one progress advance; in the
// queue form as a CUDA graph of `chunks` persistent launches of S phase steps each
// (plus the counter reset and the per-chunk advance).  Shots join or leave between
// two replays; the active list lives in device memory.
#include <string.h>

#include <algorithm>
#include <map>
#include <vector>

#include "arena.h"
#include "batch_kernels.cuh"
#include "small_kernels.cuh"
#include "w2d_common.cuh"
#include "wave2d_cuda.h"

using namespace w2d;

namespace w2d {
float cerjan_value(int d, float alpha);
}

namespace {

constexpr size_t kAlign = 256;

struct HostShot {
    bool used = false, finished = false;
    size_t off = 0, bytes = 0;  // arena block
    long long model_key = 0;    // nonzero: the models live in a shared model block
    int nx = 0, nz = 0, ldx = 0;
    size_t plane = 0;
    int k0 = 0, k_end = 0;
    float img_dt = 0.f;
    float* image = nullptr;
    float* illum = nullptr;
    double counted_pts = 0;  // grid points x phase steps
    int mode = 0;            // 0: migration, 1: forward modelling
    int nt = 0, n_rec = 0;
    float* traces = nullptr;  // mode 1: (nt, n_rec)
};

// Device copy of models shared by the shots submitted with one model key.
struct ModelBlock {
    size_t off = 0, bytes = 0;
    int refs = 0;
    int nx = 0, nz = 0, n_models = 0;
    double dt = 0;
};

}  // namespace

struct w2d_batch {
    int device = 0;  // CUDA device current at creation: every call on the handle runs there
    cudaStream_t st = nullptr;     // replays of the captured time loop
    cudaStream_t st_up = nullptr;  // shot admission (uploads, set-up kernels)
    char* arena = nullptr;
    size_t arena_bytes = 0;
    ArenaFreeList free_list{kAlign};  // the arena's free blocks
    int max_shots = 0;
    BShot* d_shots = nullptr;
    BMaps* d_maps = nullptr;
    int* d_active = nullptr;
    int* d_prefix = nullptr;
    int* d_nact = nullptr;
    int2* d_items = nullptr;  // grid form: per CTA {slot, tile} of the active shots
    size_t items_cap = 0;
    unsigned* d_head = nullptr;
    unsigned* d_err = nullptr;
    std::vector<BShot> h_shots;
    std::vector<HostShot> hs;
    std::map<long long, ModelBlock> models;  // by model key
    std::vector<int> active;
    bool active_dirty = true;
    int warps = 8, rpw = 4, S = 16, chunks = 8;
    int grid = 0;
    int form = 1;    // 1: one launch per phase step over all shots (grid form); 0: queue form
    int t_all = 0;   // tiles of the active shots (grid form launch size)
    cudaGraphExec_t gexec = nullptr;
    // grid form: the replay's launches as a graph, re-captured when the active set
    // (grid size, shot count) or the configuration changes
    cudaGraphExec_t gexec_grid = nullptr;
    long long grid_key = -1;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<cudaEvent_t> ready;  // per slot: admission work finished
    std::vector<int> joining;        // admitted shots that join at the next launch
    bool in_flight = false;
    float last_ms = 0.f;
    double last_pts = 0;
    long long last_launches = 0;
};

namespace {

bool arena_alloc(w2d_batch* b, size_t bytes, size_t* off) { return b->free_list.alloc(bytes, off); }

void arena_free(w2d_batch* b, size_t off, size_t bytes) { b->free_list.free(off, bytes); }

size_t largest_free(const w2d_batch* b) { return b->free_list.largest(); }

template <int W, int R>
cudaError_t set_attr_and_occ(int* grid)
{
    using T = AcTile<W, R, SPONGE_LUT>;
    cudaError_t e = cudaFuncSetAttribute(acoustic_batch_kernel<W, R>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)T::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    int per_sm = 0, dev = 0, sms = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, acoustic_batch_kernel<W, R>,
                                                           W * 32, T::SMEM_BYTES)) != cudaSuccess)
        return e;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    *grid = std::max(1, per_sm) * sms;
    return cudaSuccess;
}

template <int W, int R>
cudaError_t batch_step_attr()
{
    using T = AcTile<W, R, SPONGE_LUT>;
    return set_smem_once<acoustic_batch_step_kernel<W, R>>((int)T::SMEM_BYTES);
}

cudaError_t batch_step_attr_cfg(const w2d_batch* b)
{
    if (b->warps == 4 && b->rpw == 4) return batch_step_attr<4, 4>();
    if (b->warps == 4 && b->rpw == 8) return batch_step_attr<4, 8>();
    if (b->warps == 8 && b->rpw == 8) return batch_step_attr<8, 8>();
    return batch_step_attr<8, 4>();
}

template <int W, int R>
cudaError_t launch_batch_step(const BatchStepArgs& a, int grid, cudaStream_t st, int pdl)
{
    using T = AcTile<W, R, SPONGE_LUT>;
    return launch_ex(acoustic_batch_step_kernel<W, R>, dim3(grid), dim3(W * 32), T::SMEM_BYTES,
                     st, pdl, a);
}

// pdl: launch as a programmatic dependent of the previous kernel; only when the
// previous operation of the stream is that kernel.
cudaError_t launch_step_cfg(w2d_batch* b, const BatchStepArgs& a, int pdl)
{
    if (b->warps == 4 && b->rpw == 4) return launch_batch_step<4, 4>(a, b->t_all, b->st, pdl);
    if (b->warps == 4 && b->rpw == 8) return launch_batch_step<4, 8>(a, b->t_all, b->st, pdl);
    if (b->warps == 8 && b->rpw == 8) return launch_batch_step<8, 8>(a, b->t_all, b->st, pdl);
    return launch_batch_step<8, 4>(a, b->t_all, b->st, pdl);
}

template <int W, int R>
void launch_batch(const BatchArgs& a, int grid, cudaStream_t st)
{
    using T = AcTile<W, R, SPONGE_LUT>;
    acoustic_batch_kernel<W, R><<<grid, W * 32, T::SMEM_BYTES, st>>>(a);
}

cudaError_t prepare_config(w2d_batch* b)
{
    if (b->warps == 4 && b->rpw == 4) return set_attr_and_occ<4, 4>(&b->grid);
    if (b->warps == 4 && b->rpw == 8) return set_attr_and_occ<4, 8>(&b->grid);
    if (b->warps == 8 && b->rpw == 8) return set_attr_and_occ<8, 8>(&b->grid);
    return set_attr_and_occ<8, 4>(&b->grid);
}

void launch_cfg(w2d_batch* b, const BatchArgs& a)
{
    if (b->warps == 4 && b->rpw == 4) launch_batch<4, 4>(a, b->grid, b->st);
    else if (b->warps == 4 && b->rpw == 8) launch_batch<4, 8>(a, b->grid, b->st);
    else if (b->warps == 8 && b->rpw == 8) launch_batch<8, 8>(a, b->grid, b->st);
    else launch_batch<8, 4>(a, b->grid, b->st);
}

// Capture the grid form's replay: `steps` launches (the first waits for the stream
// normally, the others are programmatic dependents of the one before) and the
// progress advance.  An existing executable graph is updated in place when the
// topology allows, else replaced.
int capture_grid_replay(w2d_batch* b, int steps)
{
    BatchStepArgs a;
    a.shots = b->d_shots;
    a.maps = b->d_maps;
    a.items = b->d_items;
    a.n_active = (int)b->active.size();
    a.max_shots = b->max_shots;
    a.err = b->d_err;
    cudaGraph_t g = nullptr;
    W2D_CUDA_TRY(batch_step_attr_cfg(b));  // outside the capture
    W2D_CUDA_TRY(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaSuccess;
    for (int j = 0; j < steps && ce == cudaSuccess; ++j) {
        a.j = j;
        ce = launch_step_cfg(b, a, j > 0 ? 1 : 0);
    }
    if (ce == cudaSuccess) {
        batch_advance_kernel<<<(b->max_shots + 127) / 128, 128, 0, b->st>>>(b->d_shots, b->d_active,
                                                                             b->d_nact, steps);
        ce = cudaGetLastError();
    }
    const cudaError_t ee = cudaStreamEndCapture(b->st, &g);
    if (ce != cudaSuccess || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        set_error(std::string("replay capture failed: ") +
                  cudaGetErrorString(ce != cudaSuccess ? ce : ee));
        return W2D_ECUDA;
    }
    if (b->gexec_grid) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(b->gexec_grid, g, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(b->gexec_grid);
            b->gexec_grid = nullptr;
        }
    }
    if (!b->gexec_grid) {
        ce = cudaGraphInstantiate(&b->gexec_grid, g, 0);
        if (ce != cudaSuccess) {
            cudaGraphDestroy(g);
            set_error(std::string("replay instantiation failed: ") + cudaGetErrorString(ce));
            return W2D_ECUDA;
        }
    }
    cudaGraphDestroy(g);
    return W2D_OK;
}

int build_graph(w2d_batch* b)
{
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    W2D_CUDA_TRY(prepare_config(b));
    BatchArgs a;
    a.shots = b->d_shots;
    a.maps = b->d_maps;
    a.active = b->d_active;
    a.tile_prefix = b->d_prefix;
    a.n_active = b->d_nact;
    a.S = b->S;
    a.head = b->d_head;
    a.err = b->d_err;
    cudaGraph_t g = nullptr;
    W2D_CUDA_TRY(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    for (int c = 0; c < b->chunks; ++c) {
        cudaMemsetAsync(b->d_head, 0, sizeof(unsigned), b->st);
        launch_cfg(b, a);
        batch_advance_kernel<<<(b->max_shots + 127) / 128, 128, 0, b->st>>>(b->d_shots, b->d_active,
                                                                             b->d_nact, b->S);
    }
    cudaError_t ce = cudaStreamEndCapture(b->st, &g);
    if (ce != cudaSuccess) {
        set_error(std::string("graph capture failed: ") + cudaGetErrorString(ce));
        return W2D_ECUDA;
    }
    ce = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
        set_error(std::string("graph instantiation failed: ") + cudaGetErrorString(ce));
        return W2D_ECUDA;
    }
    return W2D_OK;
}

}  // namespace

extern "C" {

int w2d_batch_create(w2d_batch** out, unsigned long long arena_bytes, int max_shots)
{
    W2D_CHECK_ARG(out && max_shots > 0 && max_shots <= 65536, "bad arguments");
    *out = nullptr;
    w2d_batch* b = new w2d_batch();
    b->device = current_device();
    b->max_shots = max_shots;
    auto fail = [&](int rc) {
        w2d_batch_destroy(b);
        return rc;
    };
    if (arena_bytes == 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        arena_bytes = (unsigned long long)(fr * 0.8);
    }
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->st_up, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess) {
        set_error("stream/event creation failed");
        return fail(W2D_ECUDA);
    }
    if (cudaMalloc(&b->arena, arena_bytes) != cudaSuccess) {
        cudaGetLastError();
        set_error("arena allocation failed");
        return fail(W2D_ENOMEM);
    }
    b->arena_bytes = arena_bytes;
    b->free_list.reset((size_t)arena_bytes);
    if (cudaMalloc(&b->d_shots, sizeof(BShot) * max_shots) != cudaSuccess ||
        cudaMalloc(&b->d_maps, sizeof(BMaps) * max_shots) != cudaSuccess ||
        cudaMalloc(&b->d_active, sizeof(int) * max_shots) != cudaSuccess ||
        cudaMalloc(&b->d_prefix, sizeof(int) * (max_shots + 1)) != cudaSuccess ||
        cudaMalloc(&b->d_nact, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&b->d_head, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&b->d_err, sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        set_error("table allocation failed");
        return fail(W2D_ENOMEM);
    }
    cudaMemset(b->d_nact, 0, sizeof(int));
    cudaMemset(b->d_err, 0, sizeof(unsigned));
    cudaMemset(b->d_prefix, 0, sizeof(int) * (max_shots + 1));
    b->h_shots.resize(max_shots);
    b->hs.resize(max_shots);
    b->ready.assign(max_shots, nullptr);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        set_error("batch set-up failed");
        return fail(W2D_ECUDA);
    }
    *out = b;
    return W2D_OK;
}

void w2d_batch_destroy(w2d_batch* b)
{
    W2D_ON_DEVICE_OF(b);
    if (!b) return;
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->gexec_grid) cudaGraphExecDestroy(b->gexec_grid);
    for (void* p : {(void*)b->arena, (void*)b->d_shots, (void*)b->d_maps, (void*)b->d_active,
                    (void*)b->d_prefix, (void*)b->d_nact, (void*)b->d_head, (void*)b->d_err,
                    (void*)b->d_items})
        if (p) cudaFree(p);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->st_up) cudaStreamSynchronize(b->st_up);
    for (cudaEvent_t ev : b->ready)
        if (ev) cudaEventDestroy(ev);
    if (b->st_up) cudaStreamDestroy(b->st_up);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
}

int w2d_batch_set_config(w2d_batch* b, int warps, int rows_per_warp, int steps_per_launch,
                         int launches_per_graph)
{
    W2D_ON_DEVICE_OF(b);
    W2D_CHECK_ARG(b, "batch is NULL");
    W2D_CHECK_ARG((warps == 8 && rows_per_warp == 4) || (warps == 4 && rows_per_warp == 4) ||
                      (warps == 4 && rows_per_warp == 8) || (warps == 8 && rows_per_warp == 8),
                  "unsupported tile shape");
    W2D_CHECK_ARG(steps_per_launch >= 1 && steps_per_launch <= 4096, "bad steps per launch");
    W2D_CHECK_ARG(launches_per_graph >= 1 && launches_per_graph <= 1024, "bad launches per graph");
    const int old_tz = b->warps * b->rpw;
    for (int i = 0; i < b->max_shots; ++i)
        W2D_CHECK_ARG(!b->hs[i].used || b->hs[i].finished || old_tz == warps * rows_per_warp,
                      "tile height cannot change while shots are active");
    b->warps = warps;
    b->rpw = rows_per_warp;
    b->S = steps_per_launch;
    b->chunks = launches_per_graph;
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if (b->gexec_grid) {
        cudaGraphExecDestroy(b->gexec_grid);
        b->gexec_grid = nullptr;
    }
    b->grid_key = -1;
    return W2D_OK;
}

int w2d_batch_set_form(w2d_batch* b, int form)
{
    W2D_ON_DEVICE_OF(b);
    W2D_CHECK_ARG(b, "batch is NULL");
    W2D_CHECK_ARG(form == 0 || form == 1, "form must be 0 (queue) or 1 (grid)");
    W2D_CHECK_ARG(!b->in_flight, "change the form between replays only");
    if (form != b->form) {
        b->active_dirty = true;  // the grid form's work table is built with the active list
        b->grid_key = -1;
    }
    b->form = form;
    return W2D_OK;
}

unsigned long long w2d_batch_free_bytes(w2d_batch* b) { return b ? largest_free(b) : 0ull; }

}  // extern "C"

namespace {

// Arena bytes of one job: an upper bound that holds for every supported tile shape
// (the smallest tile height is 16 rows).
unsigned long long job_bytes(const w2d_shot_desc* d, int mode)
{
    if (!d || d->nx < 5 || d->nz < 5 || d->nt <= 0) return 0;
    if (mode == 0 && d->snapshot_interval <= 0) return 0;
    const size_t ldx = (size_t)pitch_for(d->nx);
    const size_t plane = ldx * d->nz;
    const size_t n_snaps = mode == 0 ? (size_t)(d->nt - 1) / d->snapshot_interval + 1 : 0;
    const size_t planes = mode == 0 ? 10 + n_snaps : 4;  // waves, models, image, illum, snaps
    const size_t ntiles = (size_t)((d->nx + AC_TX - 1) / AC_TX) * ((d->nz + 15) / 16);
    size_t f = planes * plane + (size_t)d->nt + (size_t)d->nt * std::max(d->n_rec, 1) +
               (size_t)std::max(d->n_sponge, 0) + 1 + (size_t)d->nx + 1 +
               (size_t)std::max(d->n_rec, 1) + ntiles + 64;
    return (unsigned long long)(f * 4 + 16 * kAlign);
}

// Admission of one job.  mode 0: migration (forward with snapshots and
// illumination, then backward with imaging; 2 * nt phase steps).  mode 1: forward
// modelling only, receivers sampled every step into an (nt, n_rec) gather.
int submit_job(w2d_batch* b, const w2d_shot_desc* d, int mode, int* slot_out)
{
    W2D_CHECK_ARG(b && d && slot_out, "NULL argument");
    W2D_CHECK_ARG(d->nx >= 5 && d->nz >= 5, "grid must be at least 5 x 5");
    W2D_CHECK_ARG(d->dx > 0 && d->dz > 0 && d->dt > 0, "dx, dz, dt must be positive");
    W2D_CHECK_ARG(d->nt > 0 && (mode == 1 || d->snapshot_interval > 0),
                  "nt and interval must be positive");
    W2D_CHECK_ARG(d->vel_fwd && (mode == 1 || d->vel_bwd) && d->wavelet, "NULL model or wavelet");
    W2D_CHECK_ARG(d->n_rec >= 0 && (d->n_rec == 0 || ((mode == 1 || d->data) && d->rec_ix)),
                  "bad receivers");
    W2D_CHECK_ARG(d->src_ix >= 0 && d->src_ix < d->nx && d->src_iz >= 0 && d->src_iz < d->nz,
                  "source index out of range");
    W2D_CHECK_ARG(d->rec_iz >= 0 && d->rec_iz < d->nz, "receiver_iz out of range");
    for (int r = 0; r < d->n_rec; ++r)
        W2D_CHECK_ARG(d->rec_ix[r] >= 0 && d->rec_ix[r] < d->nx, "receiver_ix out of range");
    int slot = -1;
    for (int i = 0; i < b->max_shots; ++i)
        if (!b->hs[i].used) {
            slot = i;
            break;
        }
    if (slot < 0) {
        set_error("no free shot slot");
        return W2D_ENOMEM;
    }
    const int nx = d->nx, nz = d->nz, ldx = pitch_for(nx), nt = d->nt, n_rec = d->n_rec;
    const size_t plane = (size_t)ldx * nz;
    const int interval = mode == 0 ? d->snapshot_interval : 1;
    const size_t n_snaps = mode == 0 ? (size_t)(nt - 1) / interval + 1 : 0;
    const int n_waves = mode == 0 ? 6 : 3, n_models = mode == 0 ? 2 : 1;
    const size_t n_img = mode == 0 ? 1 : 0;
    const int tz = b->warps * b->rpw;
    const int tiles_x = (nx + AC_TX - 1) / AC_TX, tiles_z = (nz + tz - 1) / tz;
    const int n_sp = std::max(d->n_sponge, 0);
    // layout of the shot's block (each piece 256-byte aligned); in mode 1 the
    // data block holds the output gather
    size_t cur = 0;
    auto take = [&](size_t bytes) {
        const size_t o = cur;
        cur += (bytes + kAlign - 1) / kAlign * kAlign;
        return o;
    };
    const long long key = d->model_key;
    ModelBlock* shared = nullptr;
    if (key) {
        auto it = b->models.find(key);
        if (it != b->models.end()) {
            const ModelBlock& m = it->second;
            W2D_CHECK_ARG(m.nx == nx && m.nz == nz && m.n_models == n_models && m.dt == d->dt,
                          "a model key given to jobs of different grids, steps or kinds");
            shared = &it->second;
        }
    }
    const size_t o_wave = take(n_waves * plane * 4), o_vel = take(key ? 0 : n_models * plane * 4),
                 o_img = take(n_img * plane * 4), o_ill = take(n_img * plane * 4),
                 o_snap = take(n_snaps * plane * 4), o_w = take((size_t)nt * 4),
                 o_data = take((size_t)nt * std::max(n_rec, 1) * 4), o_lut = take((n_sp + 1) * 4),
                 o_ptr = take((nx + 1) * 4), o_list = take(std::max(n_rec, 1) * 4),
                 o_done = take((size_t)tiles_x * tiles_z * 4);
    size_t off = 0, moff = 0;
    const size_t mbytes = (size_t)n_models * plane * 4;
    if (!arena_alloc(b, cur, &off)) {
        set_error("not enough arena memory for this shot now");
        return W2D_ENOMEM;
    }
    if (key && !shared && !arena_alloc(b, mbytes, &moff)) {  // the key's first shot
        arena_free(b, off, cur);
        set_error("not enough arena memory for this shot now");
        return W2D_ENOMEM;
    }
    const bool own_model_block = key && !shared;
    char* base = b->arena + off;
    float* wave = reinterpret_cast<float*>(base + o_wave);
    float* vel = key ? reinterpret_cast<float*>(b->arena + (shared ? shared->off : moff))
                     : reinterpret_cast<float*>(base + o_vel);
    float* img = reinterpret_cast<float*>(base + o_img);
    float* ill = reinterpret_cast<float*>(base + o_ill);
    float* snaps = reinterpret_cast<float*>(base + o_snap);
    float* wdev = reinterpret_cast<float*>(base + o_w);
    float* ddev = reinterpret_cast<float*>(base + o_data);
    float* lut = reinterpret_cast<float*>(base + o_lut);
    int* rptr = reinterpret_cast<int*>(base + o_ptr);
    int* rlist = reinterpret_cast<int*>(base + o_list);
    unsigned* done = reinterpret_cast<unsigned*>(base + o_done);
    cudaStream_t st = b->st_up;
    const float dtf = (float)d->dt;
    const float dt2 = dtf * dtf;
    int rc = W2D_OK;
    auto undo = [&](int code) {
        arena_free(b, off, cur);
        if (own_model_block) arena_free(b, moff, mbytes);
        return code;
    };
    // host-side tables
    std::vector<int> ptr(nx + 1, 0), list(std::max(n_rec, 1), 0);
    for (int r = 0; r < n_rec; ++r) ptr[d->rec_ix[r] + 1]++;
    for (int i = 0; i < nx; ++i) ptr[i + 1] += ptr[i];
    {
        std::vector<int> fill(ptr.begin(), ptr.end() - 1);
        for (int r = 0; r < n_rec; ++r) list[fill[d->rec_ix[r]]++] = r;
    }
    std::vector<float> hlut(n_sp + 1, 1.0f);
    for (int k = 1; k <= n_sp; ++k) hlut[k] = cerjan_value(k, d->sponge_alpha);
    // uploads: the models pass through a pitched staging plane (the image plane,
    // or in mode 1 the last wavefield plane), which is cleared again afterwards
    float* stage = mode == 0 ? img : wave + 2 * plane;
    // zero what is read before it is written: the wavefields, image and illumination
    // (and the staging plane among them), the per-tile progress counters; the
    // snapshot store, models, inputs and tables are written in full first
    if (cudaMemsetAsync(base + o_wave, 0, o_vel - o_wave, st) != cudaSuccess ||
        cudaMemsetAsync(base + o_img, 0, o_snap - o_img, st) != cudaSuccess ||
        cudaMemsetAsync(base + o_done, 0, cur - o_done, st) != cudaSuccess)
        return undo(W2D_ECUDA);
    for (int m = 0; m < (shared ? 0 : n_models); ++m) {  // a shared copy is there already
        const float* hv = m == 0 ? d->vel_fwd : d->vel_bwd;
        if (cudaMemcpy2DAsync(stage, (size_t)ldx * 4, hv, (size_t)nx * 4, (size_t)nx * 4, nz,
                              cudaMemcpyHostToDevice, st) != cudaSuccess)
            return undo(W2D_ECUDA);
        v2dt2_kernel<<<grid_for(plane), 256, 0, st>>>(vel + m * plane, stage, plane, dt2);
    }
    if (cudaMemsetAsync(stage, 0, plane * 4, st) != cudaSuccess ||
        cudaMemcpyAsync(wdev, d->wavelet, (size_t)nt * 4, cudaMemcpyHostToDevice, st) ||
        (mode == 0 && n_rec > 0 &&
         cudaMemcpyAsync(ddev, d->data, (size_t)nt * n_rec * 4, cudaMemcpyHostToDevice, st)) ||
        cudaMemcpyAsync(lut, hlut.data(), hlut.size() * 4, cudaMemcpyHostToDevice, st) ||
        cudaMemcpyAsync(rptr, ptr.data(), ptr.size() * 4, cudaMemcpyHostToDevice, st) ||
        cudaMemcpyAsync(rlist, list.data(), list.size() * 4, cudaMemcpyHostToDevice, st))
        return undo(W2D_ECUDA);
    // descriptor
    BShot& h = b->h_shots[slot];
    memset(&h, 0, sizeof h);
    h.g.nx = nx;
    h.g.nz = nz;
    h.g.ldx = ldx;
    h.g.inv_dx2 = 1.0f / (d->dx * d->dx);
    h.g.inv_dz2 = 1.0f / (d->dz * d->dz);
    h.g.free_surface = d->free_surface ? 1 : 0;
    h.g.n_sponge = d->n_sponge;
    h.g.sponge_lut = lut;
    h.g.rec_ptr = rptr;
    h.g.rec_list = rlist;
    h.g.shot = reinterpret_cast<const int*>(reinterpret_cast<const char*>(b->d_shots + slot) +
                                            offsetof(BShot, shot_ints));
    h.shot_ints[0] = d->src_ix;
    h.shot_ints[1] = d->src_iz;
    h.shot_ints[2] = d->rec_iz;
    h.shot_ints[3] = n_rec;
    h.shot_ints[4] = receivers_consecutive_c0(d->rec_ix, n_rec);
    h.nt = nt;
    h.interval = interval;
    h.n_rec = n_rec;
    h.tiles_x = tiles_x;
    h.tiles_z = tiles_z;
    h.ntiles = tiles_x * tiles_z;
    h.k_end = mode == 0 ? 2 * nt : nt;
    h.k0 = 0;
    h.maps_index = slot;
    for (int i = 0; i < n_waves; ++i) h.wave[i] = wave + (size_t)i * plane;
    h.snaps = mode == 0 ? snaps : nullptr;
    h.illum = mode == 0 ? ill : nullptr;
    h.image = mode == 0 ? img : nullptr;
    h.wavelet = wdev;
    h.data = mode == 0 ? ddev : nullptr;
    h.dt2_inj = (float)(d->dt * d->dt);
    h.img_dt = (float)(d->dt * (double)interval);
    h.done = done;
    h.mode = mode;
    h.traces = mode == 1 ? ddev : nullptr;
    BMaps maps;
    memset(&maps, 0, sizeof maps);
    for (int i = 0; i < n_waves; ++i) {
        if ((rc = make_tensor_map_2d(&maps.curr[i], h.wave[i], nx, nz, ldx, AC_SW, tz + 4)) ||
            (rc = make_tensor_map_2d(&maps.prev[i], h.wave[i], nx, nz, ldx, AC_TX, tz)))
            return undo(rc);
    }
    for (int i = 0; i < n_models; ++i)
        if ((rc = make_tensor_map_2d(&maps.vel[i], vel + i * plane, nx, nz, ldx, AC_TX, tz)))
            return undo(rc);
    if (cudaMemcpyAsync(b->d_shots + slot, &h, sizeof h, cudaMemcpyHostToDevice, st) ||
        cudaMemcpyAsync(b->d_maps + slot, &maps, sizeof maps, cudaMemcpyHostToDevice, st))
        return undo(W2D_ECUDA);
    // first injections: w[0] into the forward p_curr, data row nt-1 into the backward p_curr
    inject_kernel<<<(nx + 255) / 256, 256, 0, st>>>(h.wave[1], h.g, wdev, nullptr, h.dt2_inj);
    if (mode == 0 && n_rec > 0)
        inject_kernel<<<(nx + 255) / 256, 256, 0, st>>>(h.wave[4], h.g, nullptr,
                                                        ddev + (size_t)(nt - 1) * n_rec, h.dt2_inj);
    if (!b->ready[slot] && cudaEventCreateWithFlags(&b->ready[slot], cudaEventDisableTiming)) {
        set_error("event creation failed");
        return undo(W2D_ECUDA);
    }
    // the admission work runs on its own stream, overlapping a replay in flight;
    // the next launch waits for this event before the shot joins
    if (cudaGetLastError() != cudaSuccess || cudaEventRecord(b->ready[slot], st) != cudaSuccess) {
        set_error("shot admission failed on the device");
        return undo(W2D_ECUDA);
    }
    if (key) {
        if (shared) {
            shared->refs++;
        } else {
            ModelBlock m;
            m.off = moff;
            m.bytes = mbytes;
            m.refs = 1;
            m.nx = nx;
            m.nz = nz;
            m.n_models = n_models;
            m.dt = d->dt;
            b->models[key] = m;
        }
    }
    HostShot& hsh = b->hs[slot];
    hsh = HostShot();
    hsh.used = true;
    hsh.off = off;
    hsh.bytes = cur;
    hsh.model_key = key;
    hsh.nx = nx;
    hsh.nz = nz;
    hsh.ldx = ldx;
    hsh.plane = plane;
    hsh.k_end = h.k_end;
    hsh.img_dt = h.img_dt;
    hsh.image = h.image;
    hsh.illum = h.illum;
    hsh.counted_pts = (double)h.k_end * nx * nz;
    hsh.mode = mode;
    hsh.nt = nt;
    hsh.n_rec = n_rec;
    hsh.traces = h.traces;
    b->joining.push_back(slot);
    *slot_out = slot;
    return W2D_OK;
}

}  // namespace

extern "C" {

unsigned long long w2d_batch_shot_bytes(const w2d_shot_desc* d) { return job_bytes(d, 0); }

unsigned long long w2d_batch_model_bytes(const w2d_shot_desc* d) { return job_bytes(d, 1); }

int w2d_batch_submit(w2d_batch* b, const w2d_shot_desc* d, int* slot_out)
{
    W2D_ON_DEVICE_OF(b);
    return submit_job(b, d, 0, slot_out);
}

int w2d_batch_submit_modelling(w2d_batch* b, const w2d_shot_desc* d, int* slot_out)
{
    W2D_ON_DEVICE_OF(b);
    return submit_job(b, d, 1, slot_out);
}

int w2d_batch_launch(w2d_batch* b)
{
    W2D_ON_DEVICE_OF(b);
    W2D_CHECK_ARG(b, "batch is NULL");
    W2D_CHECK_ARG(!b->in_flight, "a replay is already in flight");
    b->last_ms = 0.f;
    b->last_pts = 0;
    b->last_launches = 0;
    for (int s : b->joining) {
        W2D_CUDA_TRY(cudaStreamWaitEvent(b->st, b->ready[s], 0));
        b->active.push_back(s);
        b->active_dirty = true;
    }
    b->joining.clear();
    if (b->active.empty()) return W2D_OK;
    int rc;
    if (b->active_dirty) {
        std::vector<int> prefix(b->active.size() + 1, 0);
        for (size_t i = 0; i < b->active.size(); ++i)
            prefix[i + 1] = prefix[i] + b->h_shots[b->active[i]].ntiles;
        const int n = (int)b->active.size();
        // pageable sources: the copies are staged before these calls return
        W2D_CUDA_TRY(cudaMemcpyAsync(b->d_active, b->active.data(), n * 4, cudaMemcpyHostToDevice,
                                     b->st));
        W2D_CUDA_TRY(cudaMemcpyAsync(b->d_prefix, prefix.data(), (n + 1) * 4,
                                     cudaMemcpyHostToDevice, b->st));
        W2D_CUDA_TRY(cudaMemcpyAsync(b->d_nact, &n, 4, cudaMemcpyHostToDevice, b->st));
        b->t_all = prefix[n];
        if (b->form == 1) {
            // the grid form's work table: CTA r takes tile r - prefix[i] of active shot i
            if ((size_t)b->t_all > b->items_cap) {
                if (b->d_items) {
                    W2D_CUDA_TRY(cudaStreamSynchronize(b->st));  // the last replay read it
                    cudaFree(b->d_items);
                    b->d_items = nullptr;
                    b->items_cap = 0;
                }
                const size_t cap = std::max<size_t>(1024, 2 * (size_t)b->t_all);
                W2D_CUDA_TRY(cudaMalloc(&b->d_items, cap * sizeof(int2)));
                b->items_cap = cap;
                b->grid_key = -1;  // the captured replay holds the old table's address
            }
            std::vector<int2> items(b->t_all);
            for (int i = 0; i < n; ++i)
                for (int t = 0; t < prefix[i + 1] - prefix[i]; ++t)
                    items[prefix[i] + t] = make_int2(b->active[i], t);
            W2D_CUDA_TRY(cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(int2),
                                         cudaMemcpyHostToDevice, b->st));
        }
        b->active_dirty = false;
    }
    if (b->form == 1) {
        // grid form: S * chunks launches, one phase step of every active shot each,
        // then one advance of the shots' progress, replayed as one captured graph
        const int steps = b->S * b->chunks;
        const long long key =
            (((long long)b->t_all * 65536 + (long long)b->active.size()) * 4096 + steps) * 256 +
            b->warps * 16 + b->rpw;
        if (b->grid_key != key || !b->gexec_grid) {
            if ((rc = capture_grid_replay(b, steps))) return rc;
            b->grid_key = key;
        }
        W2D_CUDA_TRY(cudaEventRecord(b->e0, b->st));
        W2D_CUDA_TRY(cudaGraphLaunch(b->gexec_grid, b->st));
        W2D_CUDA_TRY(cudaEventRecord(b->e1, b->st));
        b->last_launches = steps + 1;
        b->in_flight = true;
        return W2D_OK;
    }
    if (!b->gexec && (rc = build_graph(b))) return rc;
    W2D_CUDA_TRY(cudaEventRecord(b->e0, b->st));
    W2D_CUDA_TRY(cudaGraphLaunch(b->gexec, b->st));
    W2D_CUDA_TRY(cudaEventRecord(b->e1, b->st));
    b->last_launches = 2LL * b->chunks;
    b->in_flight = true;
    return W2D_OK;
}

int w2d_batch_wait(w2d_batch* b, int* n_finished)
{
    W2D_ON_DEVICE_OF(b);
    W2D_CHECK_ARG(b, "batch is NULL");
    if (n_finished) *n_finished = 0;
    if (!b->in_flight) return W2D_OK;
    b->in_flight = false;
    unsigned herr = 0;
    W2D_CUDA_TRY(cudaMemcpyAsync(&herr, b->d_err, 4, cudaMemcpyDeviceToHost, b->st));
    W2D_CUDA_TRY(cudaStreamSynchronize(b->st));
    cudaEventElapsedTime(&b->last_ms, b->e0, b->e1);
    if (herr) {
        char buf[96];
        snprintf(buf, sizeof buf, "persistent kernel stopped (error bits 0x%x)", herr);
        set_error(buf);
        cudaMemsetAsync(b->d_err, 0, 4, b->st);
        return W2D_ETIMEOUT;
    }
    // host mirror of the device-side progress; retire finished shots
    const int adv = b->S * b->chunks;
    std::vector<int> still;
    int fin = 0;
    for (int s : b->active) {
        HostShot& h = b->hs[s];
        const int k1 = std::min(h.k0 + adv, h.k_end);
        b->last_pts += (double)(k1 - h.k0) * h.nx * h.nz;
        h.k0 += adv;
        if (h.k0 >= h.k_end) {
            if (h.mode == 0)
                scale_kernel<<<grid_for(h.plane), 256, 0, b->st>>>(h.illum, h.plane, h.img_dt);
            h.finished = true;
            ++fin;
        } else {
            still.push_back(s);
        }
    }
    if (fin) {
        W2D_CUDA_TRY(cudaGetLastError());
        W2D_CUDA_TRY(cudaStreamSynchronize(b->st));
        b->active.swap(still);
        b->active_dirty = true;
    }
    if (n_finished) *n_finished = fin;
    return W2D_OK;
}

int w2d_batch_step(w2d_batch* b, int* n_finished)
{
    W2D_ON_DEVICE_OF(b);
    int rc;
    if ((rc = w2d_batch_launch(b))) return rc;
    return w2d_batch_wait(b, n_finished);
}

int w2d_batch_is_finished(w2d_batch* b, int slot)
{
    W2D_ON_DEVICE_OF(b);
    if (!b || slot < 0 || slot >= b->max_shots || !b->hs[slot].used) return -1;
    return b->hs[slot].finished ? 1 : 0;
}

// Give a retired shot's memory back: its block, and its shared models once no admitted
// shot uses them.
static void release_shot(w2d_batch* b, int slot)
{
    HostShot& h = b->hs[slot];
    arena_free(b, h.off, h.bytes);
    if (h.model_key) {
        auto it = b->models.find(h.model_key);
        if (it != b->models.end() && --it->second.refs == 0) {
            arena_free(b, it->second.off, it->second.bytes);
            b->models.erase(it);
        }
    }
    h = HostShot();
}

int w2d_batch_fetch(w2d_batch* b, int slot, float* image_out, float* illum_out)
{
    W2D_ON_DEVICE_OF(b);
    W2D_CHECK_ARG(b && slot >= 0 && slot < b->max_shots && b->hs[slot].used, "bad slot");
    HostShot& h = b->hs[slot];
    W2D_CHECK_ARG(h.finished, "shot not finished");
    W2D_CHECK_ARG(h.mode == 0, "a modelling job: fetch its gather with w2d_batch_fetch_traces");
    // on the admission stream: a finished shot's results are complete (w2d_batch_wait
    // synchronised the replay stream), and the next replay may already be running
    const size_t hp = (size_t)h.nx * 4, dp = (size_t)h.ldx * 4;
    if (image_out)
        W2D_CUDA_TRY(cudaMemcpy2DAsync(image_out, hp, h.image, dp, hp, h.nz,
                                       cudaMemcpyDeviceToHost, b->st_up));
    if (illum_out)
        W2D_CUDA_TRY(cudaMemcpy2DAsync(illum_out, hp, h.illum, dp, hp, h.nz,
                                       cudaMemcpyDeviceToHost, b->st_up));
    W2D_CUDA_TRY(cudaStreamSynchronize(b->st_up));
    release_shot(b, slot);
    return W2D_OK;
}

int w2d_batch_fetch_traces(w2d_batch* b, int slot, float* traces_out)
{
    W2D_ON_DEVICE_OF(b);
    W2D_CHECK_ARG(b && slot >= 0 && slot < b->max_shots && b->hs[slot].used, "bad slot");
    HostShot& h = b->hs[slot];
    W2D_CHECK_ARG(h.finished, "shot not finished");
    W2D_CHECK_ARG(h.mode == 1, "a migration job: fetch its image with w2d_batch_fetch");
    if (traces_out && h.n_rec > 0)
        W2D_CUDA_TRY(cudaMemcpyAsync(traces_out, h.traces, (size_t)h.nt * h.n_rec * 4,
                                     cudaMemcpyDeviceToHost, b->st_up));
    W2D_CUDA_TRY(cudaStreamSynchronize(b->st_up));
    release_shot(b, slot);
    return W2D_OK;
}

int w2d_batch_cancel(w2d_batch* b, int slot)
{
    W2D_ON_DEVICE_OF(b);
    W2D_CHECK_ARG(b && slot >= 0 && slot < b->max_shots && b->hs[slot].used, "bad slot");
    W2D_CHECK_ARG(!b->in_flight, "cancel between replays only");
    auto it = std::find(b->active.begin(), b->active.end(), slot);
    if (it != b->active.end()) {
        b->active.erase(it);
        b->active_dirty = true;
    }
    auto jt = std::find(b->joining.begin(), b->joining.end(), slot);
    if (jt != b->joining.end()) b->joining.erase(jt);
    W2D_CUDA_TRY(cudaStreamSynchronize(b->st_up));
    W2D_CUDA_TRY(cudaStreamSynchronize(b->st));
    release_shot(b, slot);
    return W2D_OK;
}

int w2d_batch_stats(w2d_batch* b, int* n_active, float* last_ms, double* last_points,
                    long long* last_launches)
{
    W2D_ON_DEVICE_OF(b);
    W2D_CHECK_ARG(b, "batch is NULL");
    if (n_active) *n_active = (int)b->active.size();
    if (last_ms) *last_ms = b->last_ms;
    if (last_points) *last_points = b->last_pts;
    if (last_launches) *last_launches = b->last_launches;
    return W2D_OK;
}

}  // extern "C"
