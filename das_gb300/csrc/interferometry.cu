// interferometry.cu -- virtual-source gather generation on the GPU: ambient-noise
// cross-correlation with stacking over data windows, time derivative of the
// correlations (empirical Green's function), causal / anticausal / symmetric
// branch, and linear resampling of a gather to the simulation step.
//
// Reference: tsw_rtm/interferometry.py:26-163 and run_das_pipeline.py:48-55,
// :202-213, :248-250.
//
// Cross-correlation.  The reference evaluates c(l) = sum_t s[t] r[t + l] through a
// zero-padded FFT at the data's precision (float32 under NumPy 2) and keeps rows
// [n_fft/2 - n_lags, n_fft/2 + n_lags] of the fftshifted result with Python slice
// semantics.  Here the same rows come from the direct sum: float32 samples, every
// product split exactly into two floats and accumulated in double-float
// arithmetic (about 44 bits), rounded once to float32: the result is the
// correlation rounded to float32 up to rare ties; the reference's float32 FFT
// differs from it by a few 1e-8 in relative L2.  Each window's correlations are
// added to a float32 stack in window order (the first window is copied), and the
// stack is divided by float32(number of windows) on request, as the pipeline does.
//
// Kernel layout.  One CTA per (source, 16 lags, 32 receivers); a thread owns one
// receiver and 8 consecutive lags and walks a quarter of every chunk of t with an
// 8-sample window of its receiver trace in registers (the trace is stored
// zero-padded, so no bounds tests in the loop); four warps share a lag group, one per
// quarter, and their sums are added in quarter order in double-float arithmetic
// (four times the threads of one warp per lag group: the GPU's FP32 pipes stay fed).
// The source trace is staged in shared memory in chunks; receiver-trace loads are
// coalesced across the 32 receivers of a warp.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "w2d_common.cuh"
#include "wave2d_cuda.h"

using namespace w2d;

namespace {

constexpr int XC_RX = 32;       // receivers per CTA (one per lane)
constexpr int XC_LG = 8;        // lags per thread
constexpr int XC_WY = 8;        // warps per CTA
constexpr int XC_TP = 4;        // warps sharing one lag group, each over a quarter of t
constexpr int XC_LAGS = XC_LG * (XC_WY / XC_TP);  // lags per CTA
constexpr int XC_CHUNK = 1024;  // source samples staged per shared-memory chunk
constexpr int XC_PART = XC_CHUNK / XC_TP;  // samples of a chunk per warp
static_assert(XC_WY % XC_TP == 0 && XC_PART % XC_LG == 0,
              "every warp's part of a chunk holds whole rounds of the register ring");

// Gather the source traces (n_src, nt) and the zero-padded receiver traces
// (nt + 2*pad, n_rec) out of one (nt, n_ch) data window.
__global__ void xc_gather_kernel(const float* __restrict__ data, int nt, int n_ch,
                                 const int* __restrict__ src, int n_src,
                                 const int* __restrict__ rec, int n_rec, int pad,
                                 float* __restrict__ s_out, float* __restrict__ r_out)
{
    const long long n_r = (long long)nt * n_rec, n_s = (long long)nt * n_src;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_r + n_s;
         i += (long long)gridDim.x * blockDim.x) {
        if (i < n_r) {
            const int t = (int)(i / n_rec), r = (int)(i - (long long)t * n_rec);
            r_out[(size_t)(t + pad) * n_rec + r] = data[(size_t)t * n_ch + rec[r]];
        } else {
            const long long j = i - n_r;
            const int s = (int)(j / nt), t = (int)(j - (long long)s * nt);
            s_out[(size_t)s * nt + t] = data[(size_t)t * n_ch + src[s]];
        }
    }
}

// stack[s][row][r] (+)= float32(sum_t S[s][t] * R[t + lag0 + row][r])
__global__ void __launch_bounds__(XC_RX * XC_WY)
    xc_kernel(const float* __restrict__ S, const float* __restrict__ Rp, int nt, int n_rec,
              int pad, int lag0, int n_rows, float* __restrict__ stack, int first)
{
    __shared__ float s_src[XC_CHUNK];
    __shared__ float s_part[XC_WY][2][XC_LG][XC_RX];  // the parts' (hi, lo) sums
    const int r = blockIdx.x * XC_RX + threadIdx.x;
    const int grp = threadIdx.y % (XC_WY / XC_TP), part = threadIdx.y / (XC_WY / XC_TP);
    const int row0 = blockIdx.y * XC_LAGS + grp * XC_LG;
    const int s = blockIdx.z;
    const float* Ss = S + (size_t)s * nt;
    const int rr = min(r, n_rec - 1);  // lanes past the last receiver compute a copy
    // row of Rp holding R[t + lag0 + row0] at t = 0
    const long long base = (long long)pad + lag0 + row0;
    // Double-float accumulation: each product is split exactly into p + e
    // (p = fl(a*b), e = fma(a, b, -p)), p is added to hi with Knuth's two-sum
    // (the rounding error goes to lo), and e joins lo.  The pair (hi, lo) carries
    // about 44 significant bits, enough for the sum to round correctly to float32 in
    // all but rare ties; it costs ten float32 operations per product, several times
    // less than one float64 fused multiply-add on this GPU.
    float hi[XC_LG], lo[XC_LG];
    float w[XC_LG];
#pragma unroll
    for (int j = 0; j < XC_LG; ++j) {
        hi[j] = 0.0f;
        lo[j] = 0.0f;
    }
    // The window is a ring of XC_LG registers: sample t's lag j sits in slot
    // (t + j) % XC_LG, and the slot of R[t] takes R[t + XC_LG] once t is done; the
    // sample loop is unrolled by XC_LG so every slot index is a constant (no register
    // moves).  The last chunk is padded with zero source samples to a multiple of
    // XC_LG: their products are exact zeros and leave the sums unchanged (the rows of
    // Rp they read lie inside its zero padding).
    for (int t0 = 0; t0 < nt; t0 += XC_CHUNK) {
        const int len = min(XC_CHUNK, nt - t0);
        const int len_r = (len + XC_LG - 1) / XC_LG * XC_LG;
        __syncthreads();
        for (int i = threadIdx.y * XC_RX + threadIdx.x; i < len_r; i += XC_RX * XC_WY)
            s_src[i] = i < len ? Ss[t0 + i] : 0.0f;
        __syncthreads();
        // this warp's part of the chunk: samples [a, b), its window loaded afresh
        const int a = part * XC_PART, b = min(len_r, a + XC_PART);
        if (a < b) {
#pragma unroll
            for (int j = 0; j < XC_LG; ++j) w[j] = Rp[(size_t)(base + t0 + a + j) * n_rec + rr];
        }
        for (int i0 = a; i0 < b; i0 += XC_LG) {
#pragma unroll
            for (int u = 0; u < XC_LG; ++u) {
                const float sv = s_src[i0 + u];
#pragma unroll
                for (int j = 0; j < XC_LG; ++j) {
                    const float wv = w[(u + j) % XC_LG];
                    const float p = __fmul_rn(sv, wv);
                    const float e = __fmaf_rn(sv, wv, -p);
                    const float t = __fadd_rn(hi[j], p);
                    const float bp = __fsub_rn(t, hi[j]);
                    const float err =
                        __fadd_rn(__fsub_rn(hi[j], __fsub_rn(t, bp)), __fsub_rn(p, bp));
                    hi[j] = t;
                    lo[j] = __fadd_rn(lo[j], __fadd_rn(err, e));
                }
                w[u] = Rp[(size_t)(base + t0 + i0 + u + XC_LG) * n_rec + rr];
            }
        }
    }
    // the parts of one lag group add up in part order, in double-float arithmetic
#pragma unroll
    for (int j = 0; j < XC_LG; ++j) {
        s_part[threadIdx.y][0][j][threadIdx.x] = hi[j];
        s_part[threadIdx.y][1][j][threadIdx.x] = lo[j];
    }
    __syncthreads();
    if (part != 0 || r >= n_rec) return;
#pragma unroll
    for (int j = 0; j < XC_LG; ++j) {
        float h = hi[j], l = lo[j];
        for (int q = 1; q < XC_TP; ++q) {
            const int wy = q * (XC_WY / XC_TP) + grp;
            const float ph = s_part[wy][0][j][threadIdx.x], pl = s_part[wy][1][j][threadIdx.x];
            const float t = __fadd_rn(h, ph);
            const float bp = __fsub_rn(t, h);
            const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(t, bp)), __fsub_rn(ph, bp));
            h = t;
            l = __fadd_rn(l, __fadd_rn(err, pl));
        }
        const int row = row0 + j;
        if (row >= n_rows) break;
        float* o = stack + ((size_t)s * n_rows + row) * n_rec + r;
        const float c = __fadd_rn(h, l);
        *o = first ? c : __fadd_rn(*o, c);
    }
}

__global__ void xc_divide_kernel(const float* in, float* out, size_t n, float d)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        out[i] = __fdiv_rn(in[i], d);
}

// np.gradient(c, dt, axis=0) of a float32 (n, nc) array, n >= 2.
__global__ void grad_central_kernel(const float* __restrict__ c, int n, int nc, float two_dt,
                                    float dt, float* __restrict__ out)
{
    const size_t total = (size_t)n * nc;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const int row = (int)(i / nc), col = (int)(i - (size_t)row * nc);
        float v;
        if (row == 0)
            v = __fdiv_rn(__fsub_rn(c[(size_t)nc + col], c[col]), dt);
        else if (row == n - 1)
            v = __fdiv_rn(__fsub_rn(c[i], c[i - nc]), dt);
        else
            v = __fdiv_rn(__fsub_rn(c[i + nc], c[i - nc]), two_dt);
        out[i] = v;
    }
}

// i*omega*C(omega) derivative at N = 2^ceil(log2(n)) points, by direct DFT in
// float64: spectrum C_k for k = 1..N/2-1 (DC and Nyquist terms vanish: omega_0 = 0
// and the Nyquist term is purely imaginary), then d[t] = (2/N) sum_k
// -omega_k Im(C_k e^{2 pi i k t / N}).  One CTA per column.
__global__ void grad_freq_kernel(const float* __restrict__ c, int n, int nc, int N, double dt,
                                 double* __restrict__ spec, float* __restrict__ out)
{
    const int col = blockIdx.x;
    double* re = spec + (size_t)col * N;  // N/2 complex values per column
    double* im = re + N / 2;
    for (int k = 1 + threadIdx.x; k < N / 2; k += blockDim.x) {
        double a = 0.0, b = 0.0;
        for (int t = 0; t < n; ++t) {
            const long long m = ((long long)k * t) % N;
            double sn, cs;
            sincospi(2.0 * (double)m / (double)N, &sn, &cs);
            const double x = (double)c[(size_t)t * nc + col];
            a += x * cs;
            b -= x * sn;
        }
        re[k] = a;
        im[k] = b;
    }
    __syncthreads();
    const double two_pi_over = 2.0 * M_PI / ((double)N * dt);
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        double acc = 0.0;
        for (int k = 1; k < N / 2; ++k) {
            const long long m = ((long long)k * t) % N;
            double sn, cs;
            sincospi(2.0 * (double)m / (double)N, &sn, &cs);
            // Im((re + i im)(cs + i sn)) = re*sn + im*cs
            acc += -(two_pi_over * k) * (re[k] * sn + im[k] * cs);
        }
        out[(size_t)t * nc + col] = (float)(2.0 * acc / (double)N);
    }
}

// Causal (rows from zero_idx), anticausal (rows zero_idx..0), symmetric
// (0.5 * (causal + anticausal) over the shorter length).
__global__ void branch_kernel(const float* __restrict__ in, int nc, int zero_idx, int which,
                              int n_out, float* __restrict__ out)
{
    const size_t total = (size_t)n_out * nc;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const int row = (int)(i / nc), col = (int)(i - (size_t)row * nc);
        // causal reads rows zero_idx.., anticausal rows ..zero_idx; n_out keeps both in range
        if (which == 0) {
            out[i] = in[(size_t)(zero_idx + row) * nc + col];
        } else if (which == 1) {
            out[i] = in[(size_t)(zero_idx - row) * nc + col];
        } else {
            const float pos = in[(size_t)(zero_idx + row) * nc + col];
            const float neg = in[(size_t)(zero_idx - row) * nc + col];
            out[i] = __fmul_rn(0.5f, __fadd_rn(pos, neg));
        }
    }
}

// Linear interpolation from t_i = i*dt_orig to t_j = j*dt_sim with the arithmetic
// of scipy's interp1d(kind='linear'): float64 weights, w_hi*y_hi + w_lo*y_lo,
// zero outside [t_0, t_{n-1}].
__global__ void resample_kernel(const float* __restrict__ y, int n, int nc, double dt_orig,
                                double dt_sim, int target_nt, float* __restrict__ out)
{
    const size_t total = (size_t)target_nt * nc;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(i / nc), col = (int)(i - (size_t)j * nc);
        const double xn = __dmul_rn((double)j, dt_sim);
        const double x_last = __dmul_rn((double)(n - 1), dt_orig);
        if (xn < 0.0 || xn > x_last) {
            out[i] = 0.0f;
            continue;
        }
        // first i with x_i >= xn (searchsorted, side left), clipped to [1, n-1]
        int lo = 0, hi = n;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__dmul_rn((double)mid, dt_orig) < xn) lo = mid + 1;
            else hi = mid;
        }
        const int h = min(max(lo, 1), n - 1), l = h - 1;
        const double xl = __dmul_rn((double)l, dt_orig), xh = __dmul_rn((double)h, dt_orig);
        const double span = __dsub_rn(xh, xl);
        const double w_hi = __ddiv_rn(__dsub_rn(xn, xl), span);
        const double w_lo = __ddiv_rn(__dsub_rn(xh, xn), span);
        const double v = __dadd_rn(__dmul_rn(w_hi, (double)y[(size_t)h * nc + col]),
                                   __dmul_rn(w_lo, (double)y[(size_t)l * nc + col]));
        out[i] = __double2float_rn(v);
    }
}

int grid_1d(size_t n)
{
    return (int)std::min<size_t>((n + 255) / 256, 152 * 16);
}

// Scratch for the one-call helpers (grown on demand, one user at a time).
struct Scratch {
    std::mutex mu;
    float* a = nullptr;
    size_t a_cap = 0;
    float* b = nullptr;
    size_t b_cap = 0;
    double* d = nullptr;
    size_t d_cap = 0;
    cudaStream_t st = nullptr;
};
Scratch g_scr;

template <typename T>
int grow(T** p, size_t* cap, size_t n)
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

int scratch_stream()
{
    if (!g_scr.st && cudaStreamCreateWithFlags(&g_scr.st, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("stream creation failed");
        return W2D_ECUDA;
    }
    return W2D_OK;
}

}  // namespace

struct w2d_xcorr {
    int device = 0;  // CUDA device current at creation: every call on the handle runs there
    int nt = 0, n_ch = 0, n_src = 0, n_rec = 0, lag0 = 0, n_rows = 0, pad = 0, n_added = 0;
    int n_lags = 0;
    size_t r_rows = 0;  // rows of the zero-padded receiver buffer
    int last_nt = 0;    // samples of the previous window (its rows must be cleared)
    int* d_src = nullptr;
    int* d_rec = nullptr;
    float* d_data[2] = {nullptr, nullptr};  // host windows land here, alternately
    cudaEvent_t gathered[2] = {nullptr, nullptr};  // the gather that read d_data[i] is done
    cudaStream_t st_copy = nullptr;
    float* d_s = nullptr;     // (n_src, nt)
    float* d_r = nullptr;     // (nt + 2*pad, n_rec), zero-padded
    float* d_stack = nullptr; // (n_src, n_rows, n_rec)
    float* d_out = nullptr;   // read-back staging
    cudaStream_t st = nullptr;
};

extern "C" {

int w2d_xcorr_rows(int nt, int n_lags, int* lag0, int* n_rows)
{
    W2D_CHECK_ARG(nt > 0 && n_lags >= 0 && lag0 && n_rows, "bad arguments");
    long long n_fft = 1;
    while (n_fft < 2LL * nt - 1) n_fft <<= 1;
    const long long center = n_fft / 2;
    // Python slice [center - n_lags : center + n_lags + 1] of range(n_fft)
    long long start = center - n_lags, end = center + n_lags + 1;
    if (start < 0) start += n_fft;
    if (start < 0) start = 0;
    if (end > n_fft) end = n_fft;
    *lag0 = (int)(start - center);
    *n_rows = (int)std::max(0LL, end - start);
    return W2D_OK;
}

int w2d_xcorr_create(w2d_xcorr** out, int nt, int n_ch, const int* src_ch, int n_src,
                     const int* rec_ch, int n_rec, int n_lags)
{
    W2D_CHECK_ARG(out && src_ch && rec_ch, "NULL argument");
    W2D_CHECK_ARG(nt >= 1 && n_ch >= 1 && n_src >= 1 && n_rec >= 1 && n_lags >= 0,
                  "bad sizes");
    for (int i = 0; i < n_src; ++i)
        W2D_CHECK_ARG(src_ch[i] >= 0 && src_ch[i] < n_ch, "source channel out of range");
    for (int i = 0; i < n_rec; ++i)
        W2D_CHECK_ARG(rec_ch[i] >= 0 && rec_ch[i] < n_ch, "receiver channel out of range");
    *out = nullptr;
    w2d_xcorr* x = new w2d_xcorr();
    x->device = current_device();
    x->nt = nt;
    x->n_ch = n_ch;
    x->n_src = n_src;
    x->n_rec = n_rec;
    x->n_lags = n_lags;
    w2d_xcorr_rows(nt, n_lags, &x->lag0, &x->n_rows);
    // rows of Rp read by the kernel: t + lag0 + row + j for t in [0, nt], row + j in
    // [0, rows rounded up to the CTA's lags + XC_LG]; padding keeps them inside
    const int rows_pad = (x->n_rows + XC_LAGS - 1) / XC_LAGS * XC_LAGS;
    x->pad = std::max(0, -x->lag0) + 1;
    const long long hi_row = (long long)x->pad + x->lag0 + rows_pad + XC_LG + nt;
    const long long r_rows = std::max<long long>(hi_row + 1, nt + 2LL * x->pad);
    auto fail = [&](int rc) {
        w2d_xcorr_destroy(x);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&x->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&x->st_copy, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->gathered[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->gathered[1], cudaEventDisableTiming) != cudaSuccess) {
        set_error("stream/event creation failed");
        return fail(W2D_ECUDA);
    }
    size_t c0 = 0, c1 = 0, c2 = 0, c2b = 0, c3 = 0, c4 = 0, c5 = 0, c6 = 0;
    int rc;
    if ((rc = grow(&x->d_src, &c0, n_src)) || (rc = grow(&x->d_rec, &c1, n_rec)) ||
        (rc = grow(&x->d_data[0], &c2, (size_t)nt * n_ch)) ||
        (rc = grow(&x->d_data[1], &c2b, (size_t)nt * n_ch)) ||
        (rc = grow(&x->d_s, &c3, (size_t)n_src * nt)) ||
        (rc = grow(&x->d_r, &c4, (size_t)r_rows * n_rec)) ||
        (rc = grow(&x->d_stack, &c5, (size_t)n_src * std::max(1, x->n_rows) * n_rec)) ||
        (rc = grow(&x->d_out, &c6, (size_t)n_src * std::max(1, x->n_rows) * n_rec)))
        return fail(rc);
    if (cudaMemcpy(x->d_src, src_ch, n_src * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(x->d_rec, rec_ch, n_rec * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(x->d_r, 0, (size_t)r_rows * n_rec * 4) != cudaSuccess ||
        cudaMemset(x->d_stack, 0, (size_t)n_src * std::max(1, x->n_rows) * n_rec * 4) !=
            cudaSuccess) {
        set_error("cross-correlation set-up failed");
        return fail(W2D_ECUDA);
    }
    x->r_rows = (size_t)r_rows;
    *out = x;
    return W2D_OK;
}

void w2d_xcorr_destroy(w2d_xcorr* x)
{
    W2D_ON_DEVICE_OF(x);
    if (!x) return;
    if (x->st) cudaStreamSynchronize(x->st);
    if (x->st_copy) cudaStreamSynchronize(x->st_copy);
    for (void* p : {(void*)x->d_src, (void*)x->d_rec, (void*)x->d_data[0], (void*)x->d_data[1],
                    (void*)x->d_s, (void*)x->d_r, (void*)x->d_stack, (void*)x->d_out})
        if (p) cudaFree(p);
    for (cudaEvent_t ev : x->gathered)
        if (ev) cudaEventDestroy(ev);
    if (x->st_copy) cudaStreamDestroy(x->st_copy);
    if (x->st) cudaStreamDestroy(x->st);
    delete x;
}

int w2d_xcorr_shape(w2d_xcorr* x, int* lag0, int* n_rows)
{
    W2D_CHECK_ARG(x, "NULL handle");
    if (lag0) *lag0 = x->lag0;
    if (n_rows) *n_rows = x->n_rows;
    return W2D_OK;
}

int w2d_xcorr_add_device(w2d_xcorr* x, const float* data_dev, int nt)
{
    W2D_ON_DEVICE_OF(x);
    W2D_CHECK_ARG(x && data_dev, "NULL argument");
    W2D_CHECK_DEVICE_PTR(data_dev, x->device);
    W2D_CHECK_ARG(nt >= 1 && nt <= x->nt, "window longer than the stack was created for");
    int lag0 = 0, n_rows = 0;
    w2d_xcorr_rows(nt, x->n_lags, &lag0, &n_rows);
    // the reference's stack (ndarray +=) needs every window's correlation rows to agree
    W2D_CHECK_ARG(lag0 == x->lag0 && n_rows == x->n_rows,
                  "this window's correlation rows differ from the stack's");
    W2D_CHECK_ARG((x->n_rows + XC_LAGS - 1) / XC_LAGS <= 65535 && x->n_src <= 65535,
                  "too many lags or sources for one launch");
    if (x->n_rows > 0) {
        if (x->last_nt > nt)  // rows of a longer previous window must read as zero again
            W2D_CUDA_TRY(cudaMemsetAsync(x->d_r + (size_t)(x->pad + nt) * x->n_rec, 0,
                                         (size_t)(x->last_nt - nt) * x->n_rec * 4, x->st));
        xc_gather_kernel<<<grid_1d((size_t)nt * (x->n_rec + x->n_src)), 256, 0, x->st>>>(
            data_dev, nt, x->n_ch, x->d_src, x->n_src, x->d_rec, x->n_rec, x->pad, x->d_s,
            x->d_r);
        dim3 grid((x->n_rec + XC_RX - 1) / XC_RX, (x->n_rows + XC_LAGS - 1) / XC_LAGS, x->n_src);
        xc_kernel<<<grid, dim3(XC_RX, XC_WY), 0, x->st>>>(x->d_s, x->d_r, nt, x->n_rec, x->pad,
                                                          x->lag0, x->n_rows, x->d_stack,
                                                          x->n_added == 0 ? 1 : 0);
        W2D_CUDA_TRY(cudaGetLastError());
    }
    x->last_nt = nt;
    x->n_added++;
    return W2D_OK;
}

// The host window is copied on a second stream into one of two device buffers and
// the call returns once that copy is done (the caller may reuse its array at
// once); the correlation of the previous window keeps running meanwhile.
int w2d_xcorr_add(w2d_xcorr* x, const float* data_host, int nt)
{
    W2D_ON_DEVICE_OF(x);
    W2D_CHECK_ARG(x && data_host, "NULL argument");
    W2D_CHECK_ARG(nt >= 1 && nt <= x->nt, "window longer than the stack was created for");
    const int b = x->n_added & 1;
    W2D_CUDA_TRY(cudaStreamWaitEvent(x->st_copy, x->gathered[b], 0));
    W2D_CUDA_TRY(cudaMemcpyAsync(x->d_data[b], data_host, (size_t)nt * x->n_ch * 4,
                                 cudaMemcpyHostToDevice, x->st_copy));
    W2D_CUDA_TRY(cudaStreamSynchronize(x->st_copy));
    int rc = w2d_xcorr_add_device(x, x->d_data[b], nt);
    if (rc) return rc;
    W2D_CUDA_TRY(cudaEventRecord(x->gathered[b], x->st));
    return W2D_OK;
}

int w2d_xcorr_read(w2d_xcorr* x, float* out_host, int divide)
{
    W2D_ON_DEVICE_OF(x);
    W2D_CHECK_ARG(x && out_host, "NULL argument");
    W2D_CHECK_ARG(x->n_added > 0, "no window added");
    const size_t n = (size_t)x->n_src * x->n_rows * x->n_rec;
    if (n) {
        const float* src = x->d_stack;
        if (divide) {
            xc_divide_kernel<<<grid_1d(n), 256, 0, x->st>>>(x->d_stack, x->d_out, n,
                                                            (float)x->n_added);
            W2D_CUDA_TRY(cudaGetLastError());
            src = x->d_out;
        }
        W2D_CUDA_TRY(cudaMemcpyAsync(out_host, src, n * 4, cudaMemcpyDeviceToHost, x->st));
    }
    W2D_CUDA_TRY(cudaStreamSynchronize(x->st));
    return W2D_OK;
}

int w2d_time_derivative(const float* in, int n, int nc, double dt, int scheme, float* out)
{
    W2D_CHECK_ARG(in && out && nc >= 1 && dt > 0, "bad arguments");
    W2D_CHECK_ARG(n >= 2, "at least two samples are needed for a derivative");
    W2D_CHECK_ARG(scheme == 0 || scheme == 1, "scheme must be 0 (central) or 1 (frequency)");
    std::lock_guard<std::mutex> lock(g_scr.mu);
    int rc;
    const size_t total = (size_t)n * nc;
    int N = 1;
    while (N < n) N <<= 1;
    if ((rc = scratch_stream()) || (rc = grow(&g_scr.a, &g_scr.a_cap, total)) ||
        (rc = grow(&g_scr.b, &g_scr.b_cap, total)) ||
        (scheme == 1 && (rc = grow(&g_scr.d, &g_scr.d_cap, (size_t)nc * N))))
        return rc;
    cudaStream_t st = g_scr.st;
    W2D_CUDA_TRY(cudaMemcpyAsync(g_scr.a, in, total * 4, cudaMemcpyHostToDevice, st));
    if (scheme == 0) {
        grad_central_kernel<<<grid_1d(total), 256, 0, st>>>(g_scr.a, n, nc, (float)(2.0 * dt),
                                                           (float)dt, g_scr.b);
    } else {
        grad_freq_kernel<<<nc, 256, 0, st>>>(g_scr.a, n, nc, N, dt, g_scr.d, g_scr.b);
    }
    W2D_CUDA_TRY(cudaGetLastError());
    W2D_CUDA_TRY(cudaMemcpyAsync(out, g_scr.b, total * 4, cudaMemcpyDeviceToHost, st));
    W2D_CUDA_TRY(cudaStreamSynchronize(st));
    return W2D_OK;
}

int w2d_virtual_branch(const float* in, int n, int nc, int zero_idx, int which, float* out,
                       int* n_out)
{
    W2D_CHECK_ARG(in && out && n_out && n >= 1 && nc >= 1, "bad arguments");
    W2D_CHECK_ARG(zero_idx >= 0 && zero_idx < n, "zero index out of range");
    W2D_CHECK_ARG(which >= 0 && which <= 2, "branch must be 0 causal, 1 anticausal, 2 symmetric");
    const int n_pos = n - zero_idx, n_neg = zero_idx + 1;
    const int m = which == 0 ? n_pos : (which == 1 ? n_neg : std::min(n_pos, n_neg));
    std::lock_guard<std::mutex> lock(g_scr.mu);
    int rc;
    const size_t total = (size_t)n * nc;
    if ((rc = scratch_stream()) || (rc = grow(&g_scr.a, &g_scr.a_cap, total)) ||
        (rc = grow(&g_scr.b, &g_scr.b_cap, (size_t)m * nc)))
        return rc;
    cudaStream_t st = g_scr.st;
    W2D_CUDA_TRY(cudaMemcpyAsync(g_scr.a, in, total * 4, cudaMemcpyHostToDevice, st));
    branch_kernel<<<grid_1d((size_t)m * nc), 256, 0, st>>>(g_scr.a, nc, zero_idx, which, m,
                                                           g_scr.b);
    W2D_CUDA_TRY(cudaGetLastError());
    W2D_CUDA_TRY(cudaMemcpyAsync(out, g_scr.b, (size_t)m * nc * 4, cudaMemcpyDeviceToHost, st));
    W2D_CUDA_TRY(cudaStreamSynchronize(st));
    *n_out = m;
    return W2D_OK;
}

int w2d_resample_linear(const float* in, int n, int nc, double dt_orig, double dt_sim,
                        int target_nt, float* out)
{
    W2D_CHECK_ARG(in && out && nc >= 1 && target_nt >= 0, "bad arguments");
    W2D_CHECK_ARG(n >= 2, "linear interpolation needs at least two samples");
    W2D_CHECK_ARG(dt_orig > 0 && dt_sim > 0, "time steps must be positive");
    if (target_nt == 0) return W2D_OK;
    std::lock_guard<std::mutex> lock(g_scr.mu);
    int rc;
    const size_t total_in = (size_t)n * nc, total_out = (size_t)target_nt * nc;
    if ((rc = scratch_stream()) || (rc = grow(&g_scr.a, &g_scr.a_cap, total_in)) ||
        (rc = grow(&g_scr.b, &g_scr.b_cap, total_out)))
        return rc;
    cudaStream_t st = g_scr.st;
    W2D_CUDA_TRY(cudaMemcpyAsync(g_scr.a, in, total_in * 4, cudaMemcpyHostToDevice, st));
    resample_kernel<<<grid_1d(total_out), 256, 0, st>>>(g_scr.a, n, nc, dt_orig, dt_sim,
                                                        target_nt, g_scr.b);
    W2D_CUDA_TRY(cudaGetLastError());
    W2D_CUDA_TRY(cudaMemcpyAsync(out, g_scr.b, total_out * 4, cudaMemcpyDeviceToHost, st));
    W2D_CUDA_TRY(cudaStreamSynchronize(st));
    return W2D_OK;
}

}  // extern "C"
