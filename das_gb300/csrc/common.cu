// common.cu -- error reporting, TMA descriptor encoding and the host-side
// Cerjan sponge (exported under the reference's own name).
#include <cudaTypedefs.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>

#include "w2d_common.cuh"
#include "wave2d_cuda.h"

namespace w2d {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;

int make_tensor_map_2d(CUtensorMap* out, const float* base, int nx, int nz, int ldx, int box_x,
                       int box_z)
{
    std::call_once(g_encode_once, [] {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    if (!g_encode) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return W2D_ECUDA;
    }
    if ((reinterpret_cast<uintptr_t>(base) & 15) || (ldx % 4) || box_x > 256 || box_z > 256) {
        set_error("tensor map: base/pitch not 16-byte aligned or box too large");
        return W2D_EINVAL;
    }
    cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)nz};
    cuuint64_t strides[1] = {(cuuint64_t)ldx * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)box_x, (cuuint32_t)box_z};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims,
                          strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char buf[128];
        snprintf(buf, sizeof buf, "cuTensorMapEncodeTiled failed (CUresult %d)", (int)r);
        set_error(buf);
        return W2D_ECUDA;
    }
    return W2D_OK;
}

int make_tensor_map_3d(CUtensorMap* out, const float* base, int nx, int nz, int n_planes, int ldx,
                       size_t plane_stride, int box_x, int box_z)
{
    CUtensorMap probe;
    int rc = make_tensor_map_2d(&probe, base, nx, nz, ldx, box_x, box_z);  // loads the encoder
    if (rc) return rc;
    if ((plane_stride * sizeof(float)) % 16 || n_planes < 1) {
        set_error("tensor map: plane stride not a multiple of 16 bytes");
        return W2D_EINVAL;
    }
    cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)nz, (cuuint64_t)n_planes};
    cuuint64_t strides[2] = {(cuuint64_t)ldx * sizeof(float), (cuuint64_t)plane_stride * sizeof(float)};
    cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_z, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = g_encode(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims,
                          strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char buf[128];
        snprintf(buf, sizeof buf, "cuTensorMapEncodeTiled (3D) failed (CUresult %d)", (int)r);
        set_error(buf);
        return W2D_ECUDA;
    }
    return W2D_OK;
}

// Frame distance of a cell, as float, exactly as the reference computes it
// (tsw_rtm/c_engine/wave2d.c:246-256).
static float frame_distance(int ix, int iz, int nx, int nz, int n, int fs)
{
    float d = 0.0f;
    float c[4] = {(float)(n - ix), (float)(ix - (nx - 1 - n)), (float)(iz - (nz - 1 - n)),
                  fs ? -1.0f : (float)(n - iz)};
    for (int k = 0; k < 4; ++k)
        if (c[k] > d) d = c[k];
    return d;
}

// Cerjan taper value for an integer frame distance d (d > 0), with host expf
// on the same float expression as the reference so the table is bitwise equal
// to its array.
float cerjan_value(int d, float alpha)
{
    const float df = (float)d;
    return expf(-alpha * df * df);
}

}  // namespace w2d

using namespace w2d;

extern "C" {

const char* w2d_last_error(void) { return last_error(); }

int w2d_version(void) { return W2D_ABI_VERSION; }

int w2d_set_device(int device)
{
    W2D_CUDA_TRY(cudaSetDevice(device));
    return W2D_OK;
}

int w2d_device_pci_bus_id(char* buf, int len)
{
    W2D_CHECK_ARG(buf && len > 0, "bad buffer");
    int dev = 0;
    W2D_CUDA_TRY(cudaGetDevice(&dev));
    W2D_CUDA_TRY(cudaDeviceGetPCIBusId(buf, len, dev));
    return W2D_OK;
}

void build_cerjan_sponge(float* sponge, int nx, int nz, int n_sponge, float alpha,
                         int free_surface_top)
{
    if (!sponge || nx <= 0 || nz <= 0) {
        set_error("build_cerjan_sponge: bad arguments");
        return;
    }
    for (int iz = 0; iz < nz; ++iz)
        for (int ix = 0; ix < nx; ++ix) {
            const float d = frame_distance(ix, iz, nx, nz, n_sponge, free_surface_top);
            sponge[(size_t)iz * nx + ix] = d > 0.0f ? expf(-alpha * d * d) : 1.0f;
        }
}

int w2d_sponge_lut(float* lut, int n_sponge, float alpha)
{
    if (!lut || n_sponge < 0) {
        set_error("w2d_sponge_lut: bad arguments");
        return W2D_EINVAL;
    }
    lut[0] = 1.0f;
    for (int d = 1; d <= n_sponge; ++d) lut[d] = cerjan_value(d, alpha);
    return W2D_OK;
}

}  // extern "C"
