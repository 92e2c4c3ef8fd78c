/*
 * wave2d_noalloc.h -- forward modelling with no device allocation.
 *
 * No counterpart in the reference (ll23002/DAS allocates nothing on a GPU).
 * For callers that cannot allocate device memory -- a host application that
 * owns all allocations through its own pool, a plugin whose host forbids
 * cudaMalloc/cudaFree (they synchronise the device and fragment a shared
 * budget), code that must keep the device footprint fixed -- this entry point
 * runs the same fused forward modelling as w2d_forward on the caller's device
 * buffers, with all of its scratch in one fixed-size file-scope device array
 * (W2D_NOALLOC_SCRATCH_BYTES, held by every GPU that loads the library until
 * the process exits).
 *
 * Limits: at most W2D_NOALLOC_MAX_POINTS pitched cells per field (pitch = nx
 * rounded up to 32), W2D_NOALLOC_MAX_NX columns, W2D_NOALLOC_MAX_RECEIVERS
 * receivers, W2D_NOALLOC_MAX_SPONGE sponge cells; larger requests return
 * W2D_EINVAL with a message.
 *
 * The scratch array is mapped on a device when the library's module is loaded
 * there: at the first call on that device under the runtime's default lazy
 * module loading (or at library load with CUDA_MODULE_LOADING=EAGER).  That
 * first call, made with the device current, also looks up the array's device
 * address (cudaGetSymbolAddress) and caches it per device id; a caller that
 * needs a fixed device footprint makes it once as a warm-up, outside the
 * region it measures, and before any stream capture.  cudaDeviceReset between
 * calls is not supported (the cached address would be stale).  Every call is
 * synchronous: it waits for its own work before returning, on error paths
 * too.  Calls share the scratch and it keeps the last call's
 * contents; every call clears what it relies on.  Calls whose GPU work would
 * overlap (other threads or streams) would race on the scratch: host callers
 * are serialised by a mutex and each call finishes its work before returning.
 * vel_dev, wavelet_dev and traces_dev must be device memory of the current
 * device; host memory or another GPU's memory is refused with W2D_EINVAL.
 */
#ifndef WAVE2D_NOALLOC_H
#define WAVE2D_NOALLOC_H

#ifdef __cplusplus
extern "C" {
#endif

#define W2D_NOALLOC_MAX_POINTS (1u << 20)
#define W2D_NOALLOC_MAX_NX 4096
#define W2D_NOALLOC_MAX_RECEIVERS 4096
#define W2D_NOALLOC_MAX_SPONGE 1024
#define W2D_NOALLOC_SCRATCH_BYTES (4u * (4u * W2D_NOALLOC_MAX_POINTS + 16384u))

/* Forward modelling without snapshots -- the same traces this library's
 * w2d_forward returns for the same arguments -- in velocity vel_dev (DEVICE,
 * contiguous nz x nx) with the Cerjan sponge (n_sponge, sponge_alpha) the
 * solver would build; wavelet_dev (DEVICE,
 * nt); receiver columns rec_ix (HOST, n_rec); traces_dev (DEVICE, nt x n_rec)
 * receives the traces.  stream: a cudaStream_t, or NULL for the default stream.
 * Synchronous.  Returns W2D_OK or a W2D_E* code (w2d_last_error()). */
int w2d_forward_noalloc(const float* vel_dev, const float* wavelet_dev, int nt, int nx, int nz,
                        float dx, float dz, double dt, int n_sponge, float sponge_alpha,
                        int free_surface_top, int src_ix, int src_iz, const int* rec_ix,
                        int n_rec, int rec_iz, float* traces_dev, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* WAVE2D_NOALLOC_H */
