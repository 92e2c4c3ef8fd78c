// noalloc.cu -- forward modelling that allocates nothing.
//
// Some callers cannot allocate device memory: code running inside a host
// application that owns every allocation through its own pool, a plugin whose
// host forbids cudaMalloc/cudaFree (they synchronise the device and fragment a
// shared memory budget), or a caller that must not change the device's memory
// footprint between two measurements.  For them this file offers one entry point
// that takes the caller's device buffers for inputs and outputs and keeps every
// scratch buffer it needs -- three wavefield planes, the vel^2 dt^2 plane, the
// receiver table, the sponge table, the source/receiver rows and an error word --
// in ONE file-scope __device__ array of fixed size (W2D_NOALLOC_SCRATCH_BYTES).
//
// When the array occupies device memory: with the CUDA runtime's default lazy
// module loading the module holding the array is loaded on a device at the first
// launch or symbol lookup there, so the array is mapped by the first call of this
// entry point on that device (or when the library is loaded, under
// CUDA_MODULE_LOADING=EAGER) and stays until the process exits.  A caller that
// needs a fixed footprint makes one warm-up call per device before the region it
// measures.  That first call can fail with W2D_ECUDA (out of memory) if the
// device has no room for the array.
//
// Host code must not use the array's name as a device address: on the host the
// name is only a stand-in.  At the first call on a device (with that device
// current) the entry point asks the runtime for the array's device address with
// cudaGetSymbolAddress and caches it per device id; that first call should come
// before any stream capture.  cudaDeviceReset invalidates the cached address and
// is not supported between calls.  Each call is synchronous: it waits for its
// copies and kernels with cudaStreamSynchronize, on error paths too.  All calls
// share the array and it keeps the last call's contents: each call clears the
// wavefield planes and the error word it relies on.  Calls whose work overlaps on
// the GPU (two host threads, or two streams) would race on the array; the entry
// point serialises host callers with a mutex and finishes its work before
// returning.
#include <string.h>

#include <mutex>

#include "acoustic_kernels.cuh"
#include "small_kernels.cuh"
#include "w2d_common.cuh"
#include "wave2d_cuda.h"
#include "wave2d_noalloc.h"

using namespace w2d;

namespace w2d {
float cerjan_value(int d, float alpha);
}

namespace {

constexpr size_t kPlaneMax = W2D_NOALLOC_MAX_POINTS;  // pitched floats per plane
constexpr int kNxMax = W2D_NOALLOC_MAX_NX;
constexpr int kRecMax = W2D_NOALLOC_MAX_RECEIVERS;
constexpr int kSpongeMax = W2D_NOALLOC_MAX_SPONGE;

// scratch layout (in floats / ints from the start of the array)
constexpr size_t kOffWave = 0;                          // 3 planes
constexpr size_t kOffVel = 3 * kPlaneMax;               // 1 plane
constexpr size_t kOffLut = 4 * kPlaneMax;               // kSpongeMax + 1 floats
constexpr size_t kOffPtr = kOffLut + kSpongeMax + 64;   // kNxMax + 1 ints
constexpr size_t kOffList = kOffPtr + kNxMax + 64;      // kRecMax ints
constexpr size_t kOffShot = kOffList + kRecMax + 64;    // 5 ints
constexpr size_t kOffErr = kOffShot + 64;               // 1 unsigned
constexpr size_t kWords = kOffErr + 64;
static_assert(kWords * 4 <= W2D_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the array");

__device__ __align__(256) unsigned char g_noalloc_scratch[W2D_NOALLOC_SCRATCH_BYTES];

std::mutex g_mu;
void* g_addr[64] = {nullptr};  // device address of the array, per device id

// Host-side tables (static: no host allocation per call either).
int g_ptr[kNxMax + 1];
int g_cursor[kNxMax];
int g_list[kRecMax];
float g_lut[kSpongeMax + 1];

// contiguous (nz, nx) device velocity -> pitched vel^2 dt^2
__global__ void noalloc_model_kernel(float* v2dt2, const float* vel, int nx, int nz, int ldx,
                                     float dt2)
{
    const size_t n = (size_t)ldx * nz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int iz = (int)(i / ldx), ix = (int)(i % ldx);
        const float v = ix < nx ? vel[(size_t)iz * nx + ix] : 0.0f;
        v2dt2[i] = fmul(fmul(v, v), dt2);
    }
}

}  // namespace

extern "C" {

int w2d_forward_noalloc(const float* vel_dev, const float* wavelet_dev, int nt, int nx, int nz,
                        float dx, float dz, double dt, int n_sponge, float sponge_alpha,
                        int free_surface_top, int src_ix, int src_iz, const int* rec_ix,
                        int n_rec, int rec_iz, float* traces_dev, void* stream)
{
    W2D_CHECK_ARG(vel_dev && wavelet_dev && traces_dev, "NULL device buffer");
    W2D_CHECK_ARG(nt > 0 && nx >= 5 && nz >= 5 && dx > 0 && dz > 0 && dt > 0, "bad grid");
    const int ldx = pitch_for(nx);
    W2D_CHECK_ARG(nx <= kNxMax && (size_t)ldx * nz <= kPlaneMax,
                  "grid exceeds the fixed scratch of the no-allocation entry point "
                  "(W2D_NOALLOC_MAX_NX columns, W2D_NOALLOC_MAX_POINTS pitched cells)");
    W2D_CHECK_ARG(n_rec >= 1 && n_rec <= kRecMax && rec_ix,
                  "1..W2D_NOALLOC_MAX_RECEIVERS receivers required");
    W2D_CHECK_ARG(n_sponge <= kSpongeMax, "n_sponge exceeds W2D_NOALLOC_MAX_SPONGE");
    W2D_CHECK_ARG(src_ix >= 0 && src_ix < nx && src_iz >= 0 && src_iz < nz,
                  "source index out of range");
    W2D_CHECK_ARG(rec_iz >= 0 && rec_iz < nz, "receiver_iz out of range");
    for (int r = 0; r < n_rec; ++r)
        W2D_CHECK_ARG(rec_ix[r] >= 0 && rec_ix[r] < nx, "receiver_ix out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    int dev = 0;
    W2D_CUDA_TRY(cudaGetDevice(&dev));
    W2D_CHECK_ARG(dev >= 0 && dev < 64, "device id out of range");
    // the caller's buffers must be device memory of the current device
    W2D_CHECK_DEVICE_PTR(vel_dev, dev);
    W2D_CHECK_DEVICE_PTR(wavelet_dev, dev);
    W2D_CHECK_DEVICE_PTR(traces_dev, dev);
    if (!g_addr[dev]) {
        // once per device, with that device current: the array's device address
        void* p = nullptr;
        W2D_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_addr[dev] = p;
    }
    float* base = static_cast<float*>(g_addr[dev]);
    float* wave = base + kOffWave;
    float* vel = base + kOffVel;
    float* lut = base + kOffLut;
    int* rptr = reinterpret_cast<int*>(base + kOffPtr);
    int* rlist = reinterpret_cast<int*>(base + kOffList);
    int* shot = reinterpret_cast<int*>(base + kOffShot);
    unsigned* err = reinterpret_cast<unsigned*>(base + kOffErr);
    const size_t plane = (size_t)ldx * nz;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // receiver table (columns -> receivers in index order) in static host storage
    for (int i = 0; i <= nx; ++i) g_ptr[i] = 0;
    for (int r = 0; r < n_rec; ++r) g_ptr[rec_ix[r] + 1]++;
    for (int i = 0; i < nx; ++i) g_ptr[i + 1] += g_ptr[i];
    for (int i = 0; i < nx; ++i) g_cursor[i] = g_ptr[i];
    for (int r = 0; r < n_rec; ++r) g_list[g_cursor[rec_ix[r]]++] = r;
    const int n_lut = n_sponge > 0 ? n_sponge : 0;
    g_lut[0] = 1.0f;
    for (int d = 1; d <= n_lut; ++d) g_lut[d] = cerjan_value(d, sponge_alpha);
    const int sh[5] = {src_ix, src_iz, rec_iz, n_rec, receivers_consecutive_c0(rec_ix, n_rec)};

    // tensor maps are host-side encodings of the scratch planes: build them before any
    // work is queued, so that a failure here leaves nothing running
    AcMaps maps[3];
    for (int i = 0; i < 3; ++i) {
        const int rc = make_ac_maps(&maps[i], wave + (size_t)((i + 1) % 3) * plane,
                                    wave + (size_t)i * plane, vel, nullptr, nx, nz, ldx, 16);
        if (rc) return rc;
    }

    // From here on work is queued on st.  Every failure waits for what is already
    // queued before returning, so that no kernel of this call still writes the shared
    // scratch when the next call (perhaps on another stream) starts.
#define NA_TRY(expr)                                                                   \
    do {                                                                               \
        cudaError_t _e = (expr);                                                       \
        if (_e != cudaSuccess) {                                                       \
            set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));             \
            cudaStreamSynchronize(st);                                                 \
            return W2D_ECUDA;                                                          \
        }                                                                              \
    } while (0)
    NA_TRY(cudaMemsetAsync(wave, 0, 3 * plane * 4, st));
    NA_TRY(cudaMemsetAsync(err, 0, 4, st));
    NA_TRY(cudaMemcpyAsync(rptr, g_ptr, (nx + 1) * 4, cudaMemcpyHostToDevice, st));
    NA_TRY(cudaMemcpyAsync(rlist, g_list, n_rec * 4, cudaMemcpyHostToDevice, st));
    NA_TRY(cudaMemcpyAsync(lut, g_lut, (n_lut + 1) * 4, cudaMemcpyHostToDevice, st));
    NA_TRY(cudaMemcpyAsync(shot, sh, sizeof sh, cudaMemcpyHostToDevice, st));
    // the host tables are reused by the next call: finish the copies first
    NA_TRY(cudaStreamSynchronize(st));

    const float dtf = (float)dt;
    noalloc_model_kernel<<<grid_for(plane), 256, 0, st>>>(vel, vel_dev, nx, nz, ldx, dtf * dtf);
    AcGeom g;
    memset(&g, 0, sizeof g);
    g.nx = nx;
    g.nz = nz;
    g.ldx = ldx;
    g.inv_dx2 = 1.0f / (dx * dx);
    g.inv_dz2 = 1.0f / (dz * dz);
    g.free_surface = free_surface_top ? 1 : 0;
    g.n_sponge = n_lut;
    g.sponge_lut = lut;
    g.rec_ptr = rptr;
    g.rec_list = rlist;
    g.shot = shot;
    const float dt2inj = (float)(dt * dt);
    inject_kernel<<<(nx + 255) / 256, 256, 0, st>>>(wave + plane, g, wavelet_dev, nullptr, dt2inj);
    NA_TRY(cudaGetLastError());
    for (int it = 0; it < nt; ++it) {
        AcStep s;
        memset(&s, 0, sizeof s);
        s.p_next = wave + (size_t)((it + 2) % 3) * plane;
        s.rec_out = traces_dev + (size_t)it * n_rec;
        if (it + 1 < nt) s.inj_w = wavelet_dev + it + 1;
        s.dt2_inj = dt2inj;
        s.err = err;
        // maps[i]: p_curr = plane (i+1)%3, p_prev = plane i, for it % 3 == i
        NA_TRY((launch_acoustic_step<4, 4, SPONGE_LUT>(maps[it % 3], g, s, st)));
    }
    unsigned h = 0;
    NA_TRY(cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, st));
    NA_TRY(cudaStreamSynchronize(st));
#undef NA_TRY
    if (h) {
        set_error("device wait gave up in w2d_forward_noalloc");
        return W2D_ETIMEOUT;
    }
    return W2D_OK;
}

}  // extern "C"
