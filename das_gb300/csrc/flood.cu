// flood.cu -- velocity-flood models built on the device from a resident base model.
//
// The reference builds the two flood models of TSW-RTM on the host
// (tsw_rtm/velocity_flood.py:24-94): the sediment flood keeps the base model's
// columns on the sediment side of its flood line and repeats the column at the
// line across the rest; the rock flood does the same from the rock side; then
// each is scaled by (1 + perturbation) when that is non-zero.  Here one pass over
// the grid writes both models from a base model already in device memory, so a
// server holding a job's base model on the GPU never ships flood models over the
// host link.  Every output cell is a copy of one base cell, optionally times
// float32(1 + p): the same float32 values the reference produces from a float32
// base model (NumPy 2 multiplies a float32 array by a Python float in float32).
#include <algorithm>

#include "small_kernels.cuh"
#include "w2d_common.cuh"
#include "wave2d_cuda.h"

using namespace w2d;

namespace {

struct FloodCols {
    int left;        // sediments on the left of the fault (x < fault)
    int ls, lr;      // the flood lines as computed (may be negative: Python indexing)
    int ws, wr;      // the same lines as column indices in [0, nx)
    int ps, pr;      // perturb the sediment / rock flood
    float ss, sr;    // float32(1 + perturbation)
};

__global__ void flood_kernel(const float* __restrict__ base, int nz, int nx, FloodCols c,
                             float* __restrict__ sed, float* __restrict__ rock)
{
    const size_t n = (size_t)nz * nx;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % nx);
        const size_t row = i - ix;
        // sediment side kept up to the line, the line's column repeated beyond it
        // (velocity_flood.py:54-57 and :67-70); rock side likewise (:60-63, :73-76)
        const int cs = c.left ? (ix < c.ls ? ix : c.ws) : (ix >= c.ls ? ix : c.ws);
        const int cr = c.left ? (ix >= c.lr ? ix : c.wr) : (ix < c.lr ? ix : c.wr);
        float vs = base[row + cs], vr = base[row + cr];
        if (c.ps) vs = fmul(vs, c.ss);
        if (c.pr) vr = fmul(vr, c.sr);
        sed[i] = vs;
        rock[i] = vr;
    }
}

}  // namespace

extern "C" {

int w2d_flood_models(const float* base_dev, int nz, int nx, int fault_x_idx, int sediment_is_left,
                     int flood_offset_cells, double perturb_sediment, double perturb_rock,
                     float* sed_dev, float* rock_dev, int* flood_lines, void* stream)
{
    W2D_CHECK_ARG(base_dev && sed_dev && rock_dev, "NULL device buffer");
    W2D_CHECK_ARG(nz > 0 && nx > 0, "bad grid");
    int dev = 0;
    W2D_CUDA_TRY(cudaGetDevice(&dev));
    W2D_CHECK_DEVICE_PTR(base_dev, dev);
    W2D_CHECK_DEVICE_PTR(sed_dev, dev);
    W2D_CHECK_DEVICE_PTR(rock_dev, dev);
    FloodCols c{};
    c.left = sediment_is_left ? 1 : 0;
    // the lines as the reference computes them (velocity_flood.py:51-52, :64-65)
    if (c.left) {
        c.ls = std::min(nx - 1, fault_x_idx - flood_offset_cells);
        c.lr = std::max(0, fault_x_idx + flood_offset_cells);
    } else {
        c.ls = std::max(0, fault_x_idx + flood_offset_cells);
        c.lr = std::min(nx - 1, fault_x_idx - flood_offset_cells);
    }
    // the column each line reads: Python indexing wraps a negative index once; past
    // either end the reference raises IndexError
    c.ws = c.ls < 0 ? c.ls + nx : c.ls;
    c.wr = c.lr < 0 ? c.lr + nx : c.lr;
    W2D_CHECK_ARG(c.ws >= 0 && c.ws < nx && c.wr >= 0 && c.wr < nx,
                  "flood line out of range of the model's columns");
    c.ps = perturb_sediment != 0.0;
    c.pr = perturb_rock != 0.0;
    c.ss = (float)(1.0 + perturb_sediment);
    c.sr = (float)(1.0 + perturb_rock);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    flood_kernel<<<grid_for((size_t)nz * nx), 256, 0, st>>>(base_dev, nz, nx, c, sed_dev,
                                                             rock_dev);
    W2D_CUDA_TRY(cudaGetLastError());
    if (flood_lines) {
        flood_lines[0] = c.ls;
        flood_lines[1] = c.lr;
    }
    return W2D_OK;
}

}  // extern "C"
