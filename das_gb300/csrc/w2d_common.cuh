// w2d_common.cuh -- shared device/host helpers for the GB300 wave engine.
//
// Device memory layout used by every kernel in this library: a wavefield of
// nz rows by nx columns is stored row-major with a row pitch `ldx` (floats) that
// is a multiple of 32, so that every row starts on a 128-byte boundary, every
// float4 of a row is 16-byte aligned, and a TMA tensor map can describe the
// array (strides must be multiples of 16 bytes).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "wave2d_cuda.h"

namespace w2d {

// Status codes returned across the C ABI are the W2D_* values of wave2d_cuda.h.

void set_error(const std::string& msg);
const char* last_error();

#define W2D_CUDA_TRY(expr)                                                             \
    do {                                                                               \
        cudaError_t _e = (expr);                                                       \
        if (_e != cudaSuccess) {                                                       \
            ::w2d::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));      \
            return W2D_ECUDA;                                                   \
        }                                                                              \
    } while (0)

#define W2D_CHECK_ARG(cond, msg)                                                       \
    do {                                                                               \
        if (!(cond)) {                                                                 \
            ::w2d::set_error(msg);                                                     \
            return W2D_EINVAL;                                                  \
        }                                                                              \
    } while (0)

// Makes `device` the calling thread's current device for the scope of one entry point
// and restores the caller's device at its end.  Every handle (engine, batch, elastic
// engine, correlation stack) records the device current when it was created; the
// device is per host thread, so a handle made on one device and called from another
// thread, or after w2d_set_device chose another device, still runs on its own.
// device < 0 (a NULL handle) does nothing: the entry point reports the bad handle.
class DeviceScope {
  public:
    explicit DeviceScope(int device)
    {
        int cur = -1;
        if (device >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != device &&
            cudaSetDevice(device) == cudaSuccess)
            prev_ = cur;
    }
    ~DeviceScope()
    {
        if (prev_ >= 0) cudaSetDevice(prev_);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;

  private:
    int prev_ = -1;
};

// The device current on the calling thread (0 when none can be read).
inline int current_device()
{
    int d = 0;
    return cudaGetDevice(&d) == cudaSuccess ? d : 0;
}

#define W2D_ON_DEVICE_OF(h) ::w2d::DeviceScope _w2d_device_scope((h) ? (h)->device : -1)

// A caller's DEVICE pointer must be device (or managed) memory of the handle's device: a
// host pointer, or memory of another GPU, is refused here with W2D_EINVAL instead of
// reaching a kernel.  NULL passes (the entry points check NULL themselves).
inline int check_device_ptr(const void* p, int device, const char* what)
{
    if (!p) return W2D_OK;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // the query's error is not sticky: clear it for later checks
        set_error(std::string(what) + " is not a CUDA pointer");
        return W2D_EINVAL;
    }
    if (a.type == cudaMemoryTypeManaged) return W2D_OK;
    if (a.type != cudaMemoryTypeDevice) {
        set_error(std::string(what) + " is not device memory");
        return W2D_EINVAL;
    }
    if (a.device != device) {
        set_error(std::string(what) + " is on device " + std::to_string(a.device) +
                  ", the handle on device " + std::to_string(device));
        return W2D_EINVAL;
    }
    return W2D_OK;
}

#define W2D_CHECK_DEVICE_PTR(p, dev)                                                   \
    do {                                                                               \
        const int _rc = ::w2d::check_device_ptr((p), (dev), #p);                       \
        if (_rc) return _rc;                                                           \
    } while (0)

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }
inline int pitch_for(int nx) { return round_up(nx, 32); }

// Device error-flag bits (written by kernels, read by the host after a pass).
enum ErrBits : unsigned {
    ERR_TMA_TIMEOUT = 1u,
    ERR_DEP_TIMEOUT = 2u,  // a persistent CTA waited too long for a neighbour tile
    ERR_ABORT = 4u,        // set with any error: persistent CTAs stop taking work
    ERR_BAD_ITEM = 8u,     // a batch CTA found an active-list entry out of range
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Order this thread's generic-proxy view of global / shared memory before its
// subsequent async-proxy (TMA) operations.
__device__ __forceinline__ void fence_proxy_async_global()
{
    asm volatile("fence.proxy.async.global;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_shared()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- PTX helpers (sm_100+ family; compiled for sm_103a) ---------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase.  Returns false (and the caller records an
// error bit) if the phase did not complete within `max_polls` polls; every
// try_wait suspends the thread for a hardware-defined slice, so the bound is a
// time bound of well under a second for the sizes used here.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint32_t max_polls = (1u << 22))
{
    for (uint32_t i = 0; i < max_polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 2D tiled TMA load of one box into shared memory, completion signalled on `bar`.
// The innermost coordinate x must be a multiple of 4 floats (16 bytes).
__device__ __forceinline__ void tma_load_2d(void* smem_dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Bulk prefetch of a contiguous global range into L2 (16-byte aligned address, size a
// multiple of 16 bytes); no registers or shared memory involved.
__device__ __forceinline__ void prefetch_l2_bulk(const void* p, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Per-thread asynchronous 16-byte copy global -> shared (L2 only), its commit and the
// wait for all of this thread's copies.  Both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem_dst)), "l"(gsrc)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// 3D tiled TMA load (x, row, plane) of one box into shared memory.
__device__ __forceinline__ void tma_load_3d(void* smem_dst, const CUtensorMap* map, int x, int y,
                                            int z, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// L2 eviction-priority policies for cache-hinted loads and stores.
__device__ __forceinline__ uint64_t policy_evict_last()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t policy_evict_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// tma_load_2d with an L2 eviction-priority hint.
__device__ __forceinline__ void tma_load_2d_hint(void* smem_dst, const CUtensorMap* map, int x,
                                                 int y, uint64_t* bar, uint64_t policy)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        ".L2::cache_hint [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

// float4 global store with an L2 eviction-priority hint.
__device__ __forceinline__ void st_hint_v4(float* p, float4 v, uint64_t policy)
{
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p),
                 "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "l"(policy)
                 : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Programmatic dependent launch.  launch_dependents lets the next kernel of the
// stream (launched with programmatic stream serialization) be scheduled once every
// CTA of this grid has issued it; wait blocks until the previous kernel of the
// stream has completed and its memory operations are visible.  Both are no-ops
// for a kernel launched without the attribute.
__device__ __forceinline__ void grid_dep_launch()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ void grid_dep_wait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Device ordinals covered by the per-device caches below; a device beyond them has
// its attributes set on every call instead.
constexpr int W2D_MAX_DEVICES = 64;

// Raise a kernel's dynamic shared-memory limit once per device (the attribute belongs
// to the kernel as loaded on one device, and one process may drive several devices
// through w2d_set_device): one flag per kernel (the template argument) and device,
// safe when several host threads launch it.  bytes is fixed per kernel.
template <auto Kernel>
inline cudaError_t set_smem_once(int bytes)
{
    static std::once_flag once[W2D_MAX_DEVICES];
    static cudaError_t err[W2D_MAX_DEVICES];  // zero-initialised: cudaSuccess
    int dev = 0;
    const cudaError_t ge = cudaGetDevice(&dev);
    if (ge != cudaSuccess) return ge;
    if (dev < 0 || dev >= W2D_MAX_DEVICES)
        return cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    std::call_once(once[dev], [bytes, dev] {
        err[dev] = cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        bytes);
    });
    return err[dev];
}

// IEEE single-precision arithmetic with no contraction into FMA: the engine
// evaluates every stencil in the reference's operation order so that float32
// results are bit-identical to the reference C engine built without FMA.
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

// Host: encode a 2D fp32 tensor map over a pitched array (nz rows of nx valid
// floats, row pitch ldx floats) with a box of box_x by box_z elements.  Reads
// outside [0,nx) x [0,nz) return zero.
int make_tensor_map_2d(CUtensorMap* out, const float* base, int nx, int nz, int ldx, int box_x,
                       int box_z);
// Tensor map over n_planes consecutive pitched planes (plane stride in floats):
// dims (nx, nz, n_planes), box (box_x, box_z, 1).
int make_tensor_map_3d(CUtensorMap* out, const float* base, int nx, int nz, int n_planes, int ldx,
                       size_t plane_stride, int box_x, int box_z);

}  // namespace w2d
