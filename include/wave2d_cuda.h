/*
 * wave2d_cuda.h -- C ABI of the GB300 (sm_103a) 2D wave / RTM engine.
 *
 * Library: das_gb300/libwave2d_cuda.so.  Arrays are C-contiguous float32
 * (nz rows of nx) in HOST memory unless a name says otherwise; the library
 * moves them to and from the device itself.  Integer status: 0 = success,
 * otherwise a W2D_E* code with a message from w2d_last_error().
 *
 * Part 1 repeats the four exported functions of the reference engine
 * (ll23002/DAS tsw_rtm/c_engine/wave2d.c) with identical signatures, so the
 * reference's ctypes binding (tsw_rtm/wave_solver.py:19-71) can load this
 * library in place of libwave2d.so.  They are synchronous and, like the
 * reference, return nothing; failures are reported through w2d_last_error().
 *
 * Part 2 is the whole-loop engine that the Python layer (das_gb300.wave_solver,
 * das_gb300.rtm_engine) drives: one call runs an entire forward propagation,
 * backward propagation with imaging, or forward+backward migration of a shot,
 * with every time step, injection, sampling and imaging on the device.
 *
 * Part 3 is the batched engine (many shots advanced together, continuous
 * admission), Part 4 the virtual-source gather generation upstream of migration
 * (tsw_rtm/interferometry.py).
 */
#ifndef WAVE2D_CUDA_H
#define WAVE2D_CUDA_H

#ifdef __cplusplus
extern "C" {
#endif

#define W2D_ABI_VERSION 1

enum {
    W2D_OK = 0,
    W2D_EINVAL = 1,
    W2D_ECUDA = 2,
    W2D_ENOMEM = 3,
    W2D_ETIMEOUT = 4,
    W2D_EUNSUPPORTED = 5
};

/* ---- Part 1: reference-compatible per-step functions ------------------------ */

/* Replaces acoustic_2d_step, wave2d.c:19-31.  One acoustic step; p_next's cells
 * outside the updated interior keep their incoming values.  sponge may be NULL. */
void acoustic_2d_step(const float* p_curr, const float* p_prev, float* p_next, const float* vel,
                      const float* sponge, int nx, int nz, float dx, float dz, float dt,
                      int free_surface_top);

/* Replaces elastic_2d_step, wave2d.c:95-112.  Fields updated in place.  Where
 * the reference reads row -1 (free surface on), this library reads zero. */
void elastic_2d_step(float* vx, float* vz, float* sxx, float* szz, float* sxz,
                     const float* lambda_, const float* mu, const float* buo_x,
                     const float* buo_z, const float* sponge, int nx, int nz, float dx, float dz,
                     float dt, int free_surface_top);

/* Replaces correlate_imaging_condition, wave2d.c:218-225: image += src*rec*dt. */
void correlate_imaging_condition(const float* src_wavefield, const float* rec_wavefield,
                                 float* image, int nx, int nz, float dt);

/* Replaces build_cerjan_sponge, wave2d.c:237-244 (host computation, host expf). */
void build_cerjan_sponge(float* sponge, int nx, int nz, int n_sponge, float alpha,
                         int free_surface_top);

/* The same three operations with an int status (no counterpart in the reference,
 * whose functions return void). */
int w2d_acoustic_2d_step_status(const float* p_curr, const float* p_prev, float* p_next,
                                const float* vel, const float* sponge, int nx, int nz, float dx,
                                float dz, float dt, int free_surface_top);
int w2d_elastic_2d_step_status(float* vx, float* vz, float* sxx, float* szz, float* sxz,
                               const float* lambda_, const float* mu, const float* buo_x,
                               const float* buo_z, const float* sponge, int nx, int nz, float dx,
                               float dz, float dt, int free_surface_top);
int w2d_correlate_status(const float* src, const float* rec, float* image, int nx, int nz,
                         float dt);

/* ---- Part 2: whole-loop engine ------------------------------------------------ */

const char* w2d_last_error(void);
int w2d_version(void);

/* Sponge values by integer frame distance 0..n_sponge (lut[0] = 1). */
int w2d_sponge_lut(float* lut, int n_sponge, float alpha);

typedef struct w2d_engine w2d_engine;

/* One propagation grid (WaveSolver2D.__init__, wave_solver.py:89-117).
 * sponge: the (nz, nx) array the solver holds, or NULL for no sponge.  A sponge
 * equal to the Cerjan table of some (n_sponge, alpha) is applied from a
 * per-distance table; any other array is read per cell. */
int w2d_engine_create(w2d_engine** out, int nx, int nz, float dx, float dz, double dt,
                      const float* sponge, int free_surface_top);
void w2d_engine_destroy(w2d_engine* e);

/* Velocity model for slot 0 (forward / sediment flood) or 1 (backward / rock flood):
 * contiguous nz x nx float32 in host memory, or in device memory of the engine's
 * device (a device-resident model, copied device to device; memory of another GPU
 * returns W2D_EINVAL).  Synchronous. */
int w2d_engine_set_velocity(w2d_engine* e, int slot, const float* vel);

/* Kernel tile shape (warps per CTA, rows per warp); 0,0 restores the default. */
int w2d_engine_set_tile(w2d_engine* e, int warps, int rows_per_warp);
/* L2 residency hints in the step kernel (keep p_curr, v^2 dt^2, p_next; stream p_prev). */
int w2d_engine_set_l2_hints(w2d_engine* e, int on);
/* Step launch mode (results are bit-identical in every mode): persistent = 0 one
 * CTA per tile, 1 CTAs resident for the whole step taking tiles from a counter
 * with the next tile's boxes loading while the current one is computed; pdl = 1
 * launches each step as a programmatic dependent of the previous one, so its
 * set-up overlaps the previous step's tail.  Default: persistent 0, pdl 1. */
int w2d_engine_set_launch(w2d_engine* e, int persistent, int pdl);
/* CUDA graphs for migrations (on = 1, the default): the forward pass and the backward
 * pass of w2d_migrate_shot / w2d_migrate_staged are each captured once as a graph and
 * replayed for later shots with the same sizes, modes and buffers, one graph launch
 * per pass instead of one host launch per step (default launch mode only; the
 * two-step and counter modes launch directly).  Bit-identical either way.  on = 0
 * launches every step from the host and drops the cached graphs. */
int w2d_engine_set_graphs(w2d_engine* e, int on);
/* Two time steps per launch (one-CTA-per-tile mode only): each 128 x (4 *
 * rows_per_warp) tile evaluates step n on itself plus a 2-cell ring in shared memory,
 * then step n+1, so every wavefield crosses memory once per two steps; bit-identical
 * to one step per launch.  Checkpoint boundaries fall back to single steps.
 * rows_per_warp: 0 off (the default), 1 the default shape (3), 2..4. */
int w2d_engine_set_two_step(w2d_engine* e, int rows_per_warp);

/* forward_propagate_acoustic, wave_solver.py:128-186.  rec_out: (nt, n_rec);
 * snaps_out: (ceil(nt/interval), nz, nx) or NULL.  Indices already in range. */
int w2d_forward(w2d_engine* e, int vel_slot, const float* wavelet, int nt, int src_ix,
                int src_iz, const int* rec_ix, int n_rec, int rec_iz, float* rec_out,
                float* snaps_out, int snapshot_interval);

/* backward_propagate_and_correlate, wave_solver.py:188-242.  data: (nt, n_rec);
 * fwd_snaps: (n_snaps, nz, nx); image: (nz, nx), accumulated in place. */
int w2d_backward_correlate(w2d_engine* e, int vel_slot, const float* data, int nt,
                           const int* rec_ix, int n_rec, int rec_iz, const float* fwd_snaps,
                           int n_snaps, float* image, int snapshot_interval);

/* Storage of the forward wavefield during migration. */
enum { W2D_STORE_AUTO = 0, W2D_STORE_ALL = 1, W2D_STORE_CHECKPOINT = 2 };

/* TSWRTMEngine.migrate_shot, rtm_engine.py:49-104, entirely on the device:
 * forward in velocity slot 0 with illumination, backward in slot 1 with imaging.
 * If image_out / illum_out are NULL the shot is added to the device stack
 * instead (see w2d_stack_*).  storage picks full snapshot storage or
 * checkpointed recomputation (AUTO: full storage when it fits the budget). */
int w2d_migrate_shot(w2d_engine* e, const float* wavelet, int nt, int src_ix, int src_iz,
                     const float* data, const int* rec_ix, int n_rec, int rec_iz,
                     int snapshot_interval, int storage, float* image_out, float* illum_out);

/* Device stack of migrated shots (rtm_engine.py:142-143). */
int w2d_stack_reset(w2d_engine* e);
int w2d_stack_read(w2d_engine* e, float* image_out, float* illum_out);
/* Add one shot's (image, illumination), HOST (nz, nx) arrays, to the device stack
 * (float32 adds in call order, as rtm_engine.py:142-143 stacks). */
int w2d_stack_add(w2d_engine* e, const float* image, const float* illum);
/* Post-stack of the device stack (rtm_engine.py:145-158) on the device: mute where the
 * sponge is below 0.99, illumination normalisation with eps = 1e-4 * max, 3x3
 * Laplacian with symmetric edges; the three (nz, nx) images are copied out. */
int w2d_post_stack(w2d_engine* e, int mute_sponge, float* raw_out, float* laplacian_out,
                   float* normalized_out);

/* Device-resident shot inputs: stage a shot's wavelet (nt) and data (nt, n_rec)
 * into engine-owned device memory under an integer slot, then migrate it with
 * no host-to-device traffic in the call (used for device-timed benchmarks and
 * by callers that prefetch shots). */
int w2d_shot_stage(w2d_engine* e, int slot, const float* wavelet, int nt, const float* data,
                   int n_rec);
int w2d_migrate_staged(w2d_engine* e, int slot, int src_ix, int src_iz, const int* rec_ix,
                       int n_rec, int rec_iz, int snapshot_interval, int storage,
                       float* image_out, float* illum_out);

/* CUDA-event timer on the engine's stream (device milliseconds between the calls). */
int w2d_engine_timer_start(w2d_engine* e);
int w2d_engine_timer_stop(w2d_engine* e, float* ms);

/* Select the CUDA device used by engines created afterwards on this host thread.
 * Every handle (engine, batch, elastic engine, correlation stack) keeps the device
 * that was current when it was created: calls on it run there, from any host thread,
 * and leave the calling thread's current device as they found it. */
int w2d_set_device(int device);
/* PCI bus id ("0000:xx:00.0") of the current device, for per-GPU monitoring. */
int w2d_device_pci_bus_id(char* buf, int len);

/* Free and total device memory of the current device, in bytes. */
int w2d_device_memory(unsigned long long* free_bytes, unsigned long long* total_bytes);

/* Velocity-flood models on the device (generate_velocity_flood_models,
 * tsw_rtm/velocity_flood.py:24-94): from base_dev (DEVICE, contiguous nz x nx
 * float32) write the sediment flood to sed_dev and the rock flood to rock_dev
 * (DEVICE, nz x nx), with the reference's flood lines (returned in
 * flood_lines[0..1] when not NULL) and its float32 perturbation arithmetic.
 * Asynchronous on `stream` (a cudaStream_t, NULL: the default stream).  A flood
 * line outside the model's columns (the reference raises IndexError) returns
 * W2D_EINVAL. */
int w2d_flood_models(const float* base_dev, int nz, int nx, int fault_x_idx, int sediment_is_left,
                     int flood_offset_cells, double perturb_sediment, double perturb_rock,
                     float* sed_dev, float* rock_dev, int* flood_lines, void* stream);

/* Page-locked host memory for fast host<->device copies of shot inputs/outputs. */
int w2d_host_alloc(void** out, unsigned long long bytes);
void w2d_host_free(void* p);

/* ---- Differentiable modelling (no reference counterpart: RTM as the adjoint) ----
 * Forward modelling in velocity vel_dev (DEVICE, contiguous nz x nx float32),
 * traces written to traces_dev (DEVICE, nt x n_rec), checkpoints of the forward
 * state kept in the engine.  Source and receivers must sit on written cells
 * (interior, or rows 0/1 with the free surface). */
int w2d_fwi_forward(w2d_engine* e, const float* vel_dev, const float* wavelet, int nt, int src_ix,
                    int src_iz, const int* rec_ix, int n_rec, int rec_iz, float* traces_dev);
/* Gradient of sum(resid * traces) with respect to the velocity of the last
 * w2d_fwi_forward on this engine: resid_dev (DEVICE, nt x n_rec), grad_dev
 * (DEVICE, nz x nx, overwritten).  Hand-written adjoint kernel; the forward
 * wavefield is recomputed segment by segment from the checkpoints. */
int w2d_fwi_gradient(w2d_engine* e, const float* resid_dev, float* grad_dev);
/* Steps per checkpoint segment of the next w2d_fwi_forward: 0 (the default) picks
 * sqrt(3 nt), the segment length that balances checkpoint and segment storage;
 * nt or more keeps every forward state of the run (no recomputation, nt planes
 * of device memory).  The gradient is the same bit for bit either way. */
int w2d_fwi_set_segment(w2d_engine* e, int steps);
/* Form of the adjoint kernel of w2d_fwi_gradient: 0 (the default) the vectorised
 * kernel, 1 the per-cell kernel it is checked against.  The two agree to float32
 * rounding (they differ only in the compiler's contraction choices). */
int w2d_fwi_set_adjoint_form(w2d_engine* e, int cells);
int w2d_engine_synchronize(w2d_engine* e);

/* ---- Elastic modelling and gradient (no reference counterpart: the reference only
 * exports the step, wave2d.c:95-212, which these calls advance) ----
 * Vertical force source vz[src] += w[n]*dt before step n; vertical-strain
 * receivers (Dz- vz after each step) at row rec_iz, columns in [2, nx-2); the
 * Cerjan sponge of (n_sponge, alpha).  Parameters and outputs are DEVICE arrays,
 * contiguous (nz, nx); wavelet and rec_ix are HOST arrays. */
typedef struct w2d_elastic w2d_elastic;
int w2d_elastic_create(w2d_elastic** out, int nx, int nz, float dx, float dz, double dt,
                       int n_sponge, float sponge_alpha, int free_surface_top);
void w2d_elastic_destroy(w2d_elastic* e);
int w2d_elastic_forward(w2d_elastic* e, const float* lam, const float* mu, const float* bx,
                        const float* bz, const float* wavelet, int nt, int src_ix, int src_iz,
                        const int* rec_ix, int n_rec, int rec_iz, float* traces_dev);
/* Gradients of sum(resid * traces) with respect to lambda, mu, buo_x, buo_z (any
 * output may be NULL); exact adjoint of the discrete step, forward states
 * recomputed from checkpoints. */
int w2d_elastic_gradient(w2d_elastic* e, const float* resid_dev, float* g_lam, float* g_mu,
                         float* g_bx, float* g_bz);
float w2d_elastic_last_ms(w2d_elastic* e);
/* The same for a batch of n_shots shots on this grid, advanced together (every
 * launch covers all shots): lam, mu, bx, bz DEVICE n_shots x (nz, nx) contiguous
 * (each shot its own model), wavelets HOST (n_shots, nt), src_ix / src_iz HOST
 * n_shots each, receivers shared, traces_dev DEVICE (n_shots, nt, n_rec); the
 * gradient of the last batch returns one gradient per shot (n_shots x (nz, nx)). */
int w2d_elastic_forward_batch(w2d_elastic* e, int n_shots, const float* lam, const float* mu,
                              const float* bx, const float* bz, const float* wavelets, int nt,
                              const int* src_ix, const int* src_iz, const int* rec_ix, int n_rec,
                              int rec_iz, float* traces_dev);
int w2d_elastic_gradient_batch(w2d_elastic* e, const float* resid_dev, float* g_lam, float* g_mu,
                               float* g_bx, float* g_bz);
/* How the adjoint passes run: 1 (default) TMA-tiled passes, 0 per-cell kernels.
 * The two agree to float32 rounding (contraction differs); both are exact adjoints. */
int w2d_elastic_set_adjoint(w2d_elastic* e, int form);
/* Tile shapes (warps per CTA x rows per warp, 128 columns wide) of the step kernels
 * (4x2 default, 4x4, 8x2, 8x1) and of the tiled adjoint passes (4x1 default, 4x2,
 * 8x1); applies from the next forward call.  Results do not depend on the tiles. */
int w2d_elastic_set_tiles(w2d_elastic* e, int step_warps, int step_rows_per_warp,
                          int adjoint_warps, int adjoint_rows_per_warp);
/* Programmatic dependent launches between consecutive step / tiled-adjoint kernels
 * (on by default; each kernel's set-up overlaps its predecessor's tail, and it waits
 * for the predecessor before any global access).  Results are identical either way. */
int w2d_elastic_set_pdl(w2d_elastic* e, int on);
/* The next w2d_elastic_forward_batch's shots all have the same model (the caller has
 * checked): only the first shot's lam, mu, bx, bz are read and stored, and every shot
 * reads them (their tiles then come from L2 for all but the first shot).  Gradients
 * stay per shot.  Applies to that one call. */
int w2d_elastic_share_model(w2d_elastic* e, int on);
/* Device bytes one shot of a batch holds (checkpoints, one recomputed segment, fields). */
unsigned long long w2d_elastic_shot_bytes(int nx, int nz, int nt, int n_rec);

/* ---- Part 3: batched / continuously fed migration (no reference counterpart:
 * the reference migrates shots one after another, rtm_engine.py:125-143) ----- */

/* One shot's migration job: grid, Cerjan sponge parameters (n_sponge < 0: no
 * sponge), models (vel_fwd = sediment flood, vel_bwd = rock flood), wavelet (nt),
 * data (nt, n_rec), receiver columns; host arrays, copied at submission.
 * model_key: 0, or a key the caller gives every shot whose models are identical (the
 * shots of one job): while any shot with the key is admitted, later shots with the
 * same key (same grid, dt and job kind) use its device copy of the models instead of
 * their own, so one job's shots read one model. */
typedef struct {
    int nx, nz;
    float dx, dz;
    double dt;
    int free_surface;
    int n_sponge;
    float sponge_alpha;
    int nt, snapshot_interval, n_rec;
    int src_ix, src_iz, rec_iz;
    const float* vel_fwd;
    const float* vel_bwd;
    const float* wavelet;
    const float* data;
    const int* rec_ix;
    long long model_key;
} w2d_shot_desc;

typedef struct w2d_batch w2d_batch;

/* arena_bytes: device memory for admitted shots (0 = 80 % of free memory). */
int w2d_batch_create(w2d_batch** out, unsigned long long arena_bytes, int max_shots);
void w2d_batch_destroy(w2d_batch* b);
/* Tile shape of the persistent kernel, phase steps per launch, launches per graph. */
int w2d_batch_set_config(w2d_batch* b, int warps, int rows_per_warp, int steps_per_launch,
                         int launches_per_graph);
/* How a replay advances the shots: form 1 (default) one launch per phase step over
 * every active shot's tiles; form 0 a persistent kernel over a (step, shot, tile)
 * queue with per-tile dependency counters.  Results are identical. */
int w2d_batch_set_form(w2d_batch* b, int form);
/* Device bytes one shot needs (upper bound) and the largest free arena block. */
unsigned long long w2d_batch_shot_bytes(const w2d_shot_desc* d);
unsigned long long w2d_batch_free_bytes(w2d_batch* b);
/* Admit a shot; W2D_ENOMEM when it does not fit now (retry after a fetch). */
int w2d_batch_submit(w2d_batch* b, const w2d_shot_desc* d, int* slot_out);
/* Forward-modelling job in the same batch (the many-shot form of
 * wave_solver.py:128-186 forward_propagate_acoustic without snapshots): vel_fwd is the
 * model, vel_bwd, data and snapshot_interval are ignored, and the receivers'
 * p_next samples of every step form an (nt, n_rec) gather, read back with
 * w2d_batch_fetch_traces.  Modelling and migration jobs share one replay. */
unsigned long long w2d_batch_model_bytes(const w2d_shot_desc* d);
int w2d_batch_submit_modelling(w2d_batch* b, const w2d_shot_desc* d, int* slot_out);
int w2d_batch_fetch_traces(w2d_batch* b, int slot, float* traces_out);
/* Replay the captured time loop once over all active shots (launch + wait). */
int w2d_batch_step(w2d_batch* b, int* n_finished);
/* The two halves of w2d_batch_step: launch returns at once (shots submitted while
 * a replay is in flight upload on a second stream and join the next launch);
 * wait finishes the replay and retires shots that reached the end. */
int w2d_batch_launch(w2d_batch* b);
int w2d_batch_wait(w2d_batch* b, int* n_finished);
/* 1 finished, 0 running, -1 unused slot. */
int w2d_batch_is_finished(w2d_batch* b, int slot);
/* Copy a finished shot's image and illumination (nz, nx) out and free its memory;
 * runs beside a replay in flight (launch the next replay first, then fetch). */
int w2d_batch_fetch(w2d_batch* b, int slot, float* image_out, float* illum_out);
int w2d_batch_cancel(w2d_batch* b, int slot);
/* Active shots, device ms / counted point-updates / launches of the last step call. */
int w2d_batch_stats(w2d_batch* b, int* n_active, float* last_ms, double* last_points,
                    long long* last_launches);

/* Bytes of device memory the engine may use for snapshots/checkpoints (0 = 80 %
 * of free memory at the time of the call). */
int w2d_engine_set_memory_budget(w2d_engine* e, unsigned long long bytes);

/* Statistics of the last whole-loop call: storage mode used (1 all, 2 checkpoint),
 * number of step kernels launched, recomputed forward steps, device ms. */
int w2d_engine_last_stats(w2d_engine* e, int* storage_used, long long* step_launches,
                          long long* recomputed_steps, float* device_ms);

/* ---- Part 4: virtual-source gathers (the step upstream of migration) ---------- */

/* Rows the reference keeps of an FFT cross-correlation of nt-sample traces with
 * n_lags = round(max_lag / dt) (interferometry.py:50-74): the Python slice
 * [n_fft/2 - n_lags, n_fft/2 + n_lags + 1) of the fftshifted correlation,
 * n_fft = 2^ceil(log2(2 nt - 1)); row i holds lag lag0 + i (in samples). */
int w2d_xcorr_rows(int nt, int n_lags, int* lag0, int* n_rows);

typedef struct w2d_xcorr w2d_xcorr;

/* Cross-correlation stack of (nt, n_ch) data windows: for every source channel,
 * c(l) = sum_t data[t, src] * data[t + l, rec] over the rows above and every
 * receiver channel (compute_cross_correlation, interferometry.py:26-79, without
 * the FFT: exact products summed in double-float, rounded to float32), added to a float32
 * stack in window order (run_das_pipeline.py:202-213). */
int w2d_xcorr_create(w2d_xcorr** out, int nt, int n_ch, const int* src_ch, int n_src,
                     const int* rec_ch, int n_rec, int n_lags);
void w2d_xcorr_destroy(w2d_xcorr* x);
int w2d_xcorr_shape(w2d_xcorr* x, int* lag0, int* n_rows);
/* Add one window of nt samples (nt no larger than the nt the stack was created for,
 * and giving the same correlation rows): host (nt, n_ch) float32, or a device pointer. */
int w2d_xcorr_add(w2d_xcorr* x, const float* data_host, int nt);
int w2d_xcorr_add_device(w2d_xcorr* x, const float* data_dev, int nt);
/* Stack (n_src, n_rows, n_rec) to host memory; divide = 1 divides by
 * float32(number of windows added) as run_das_pipeline.py:248-250 does. */
int w2d_xcorr_read(w2d_xcorr* x, float* out_host, int divide);

/* time_derivative_greens (interferometry.py:82-102) of an (n, nc) float32 array:
 * scheme 0 = np.gradient(c, dt, axis=0) (bit-exact), 1 = i*omega*C(omega) at
 * 2^ceil(log2(n)) points (float64 DFT). */
int w2d_time_derivative(const float* in, int n, int nc, double dt, int scheme, float* out);

/* Branch of build_virtual_shot_gather (interferometry.py:132-148): which = 0 causal
 * (rows zero_idx..), 1 anticausal (rows zero_idx..0), 2 symmetric (float32 mean of
 * the two over the shorter length).  *n_out = rows written. */
int w2d_virtual_branch(const float* in, int n, int nc, int zero_idx, int which, float* out,
                       int* n_out);

/* resample_gather_to_sim_dt (run_das_pipeline.py:48-55): linear interpolation of each
 * column from t = i*dt_orig to t = j*dt_sim, j < target_nt, zero outside the data. */
int w2d_resample_linear(const float* in, int n, int nc, double dt_orig, double dt_sim,
                        int target_nt, float* out);

#ifdef __cplusplus
}
#endif

#endif /* WAVE2D_CUDA_H */
