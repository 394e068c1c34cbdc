/* sfwi_gb300.h — C ABI of the GB300 shot-gradient engine.
 *
 * The entry points replace the per-shot engine of the SFWI elastic FWI code:
 * the class FD2DGPU_ELASTIC and the free functions of sfwi-stage{1,2}/FD2DGPU.cuh
 * that sfwi-stage{1,2}/main.cpp calls.  A handle stands for one
 * FD2DGPU_ELASTIC object; the public fields the driver writes before
 * IMAGE_SINGLESHOT (isx, isz, igz, ngx_left, delta_left, record_left_in_v, ntr)
 * are set through sfwi_set_shot_geometry.  All buffers are caller-owned host
 * arrays with the reference's layouts:
 *   models, gradients, illumination  float [allnx][allnz]  (z fastest)
 *   records                          float [ntr][nt]       (time fastest)
 *   receiver coordinates             int   [ntr]
 * Every function returns 0 on success and a negative SFWI_E* code on failure;
 * sfwi_last_error() gives a message for the calling thread's last failure.
 * A handle is used by one host thread at a time; different handles are
 * independent.
 *
 * Beyond the reference's one-shot-at-a-time calls, sfwi_enqueue_shot /
 * sfwi_run advance many shots (each with its own window width) in the same
 * kernel launches, and sfwi_ot* compute the 1D optimal-transport misfit the
 * reference only declares.
 */
#ifndef SFWI_GB300_H
#define SFWI_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sfwi_handle sfwi_handle;

enum {
    SFWI_OK = 0,
    SFWI_E_ARG = -1,      /* invalid argument (size, pointer, geometry outside the model) */
    SFWI_E_CUDA = -2,     /* CUDA runtime error (message in sfwi_last_error) */
    SFWI_E_NOMEM = -3,    /* device or host allocation failed */
    SFWI_E_STATE = -4,    /* call out of order (e.g. no model uploaded) */
    SFWI_E_NODEVICE = -5  /* no CUDA device */
};

/* misfit functions for the adjoint source */
enum {
    SFWI_MISFIT_L2 = 0,        /* sum r^2, adjoint source r (the reference's live misfit) */
    SFWI_MISFIT_OT = 1,        /* 1D W2, exponential positivity transform, per-trace scale */
    SFWI_MISFIT_OT_POWER = 2,  /* 1D W2, squared-amplitude transform */
    SFWI_MISFIT_OT_ALLTRACE = 3 /* 1D W2, exponential transform, gather-wide scale */
};

/* Constructor: FD2DGPU_ELASTIC(sou, dx, dz, dt, nxpml, nzpml, allnx, allnz,
 * scale, pml, nt, nop, ntr), sfwi-stage1/FD2DGPU.cuh:152-153.  Copies sou[nt].
 * stage selects the reference program whose IMAGE_SINGLESHOT is reproduced:
 *   1  sfwi-stage1: background forward, residual syn-obs, adjoint direction +1
 *   2  sfwi-stage2: background + Born forward, residual (du-obs)+u0,
 *      adjoint direction -1, density forced to 2000 kg/m^3
 * nop must be 4 (the 8th-order stencil of FD2DGPU.cuh:16). */
int sfwi_create(sfwi_handle **out, int stage, const float *sou, float dx, float dz, float dt, int nxpml, int nzpml,
                int allnx, int allnz, int scale, int pml, int nt, int nop, int ntr);
int sfwi_destroy(sfwi_handle *h);

/* GPUbufferVPVS(vp_all, vs_all, rho_all), sfwi-stage1/FD2DGPU.cuh:296
 * (stage 2's two-argument form: pass rho_all = NULL). */
int sfwi_gpu_buffer_vpvs(sfwi_handle *h, const float *vp_all, const float *vs_all, const float *rho_all);
/* GPUbufferM(dvp, dvs), sfwi-stage1/FD2DGPU.cuh:237: the stage-2 model perturbation. */
int sfwi_gpu_buffer_m(sfwi_handle *h, const float *dvp_all, const float *dvs_all);
/* bufferVpVsHtoD(ngx_min), FD2DGPU.cu:1348: window start column of the next shot. */
int sfwi_buffer_vpvs_htod(sfwi_handle *h, int ngx_min);
/* record_copytoGPU(record_z, record_x, gc), FD2DGPU.cu:3507-3533: observed
 * records [ntr][nt] and receiver coordinates of the next shot. */
int sfwi_record_copy_to_gpu(sfwi_handle *h, const float *rec_z, const float *rec_x, const int *gc);
/* The public fields main.cpp:619-625 writes before IMAGE_SINGLESHOT. */
int sfwi_set_shot_geometry(sfwi_handle *h, int isx, int isz, int igz, int ngx_left, int delta_left,
                           int record_left_in_v, int ntr);
/* misfit function used by the following gradient calls (default L2) */
int sfwi_set_misfit(sfwi_handle *h, int misfit_kind);

/* IMAGE_SINGLESHOT, sfwi-stage1/FD2DGPU.cuh:466-467 / sfwi-stage2/FD2DGPU.cuh:455:
 * one shot-gradient.  misfit += this shot's misfit; the Vp/Vs gradients and
 * the illumination accumulate on the device until sfwi_imagebuffer_resettozero. */
int sfwi_image_singleshot(sfwi_handle *h, double *misfit);

/* imagebuffer_resettozero(grad_pp, grad_ps, illum, b1, b2, b3, b4),
 * FD2DGPU.cu:3646-3673: copy the accumulated gradients out and zero them.
 * b1..b4 receive the reference's scattering-term buffers, which its live path
 * leaves at zero; any of the seven pointers may be NULL. */
int sfwi_imagebuffer_resettozero(sfwi_handle *h, float *grad_pp, float *grad_ps, float *illum, float *b1, float *b2,
                                 float *b3, float *b4);
/* FP64 copy of the accumulated gradients (no reset) */
int sfwi_read_gradients_f64(sfwi_handle *h, double *grad_pp, double *grad_ps, double *illum);

/* Density gradient.  No reference counterpart: the reference images Vp and Vs
 * only (doimage_gradient, FD2DGPU.cu:3350-3382).  When switched on, every
 * later gradient run also accumulates the density kernel
 *     G_rho += -sum_t v_adj(t) . (v(t) - v(t-1)) / dt
 * over the interior cells, with v(t) - v(t-1) the velocity step of the
 * background reconstruction and v_adj the adjoint velocity, into an FP64
 * [allnx][allnz] buffer.  sfwi_read_density_gradient_f64 copies it out (no
 * reset); sfwi_imagebuffer_resettozero zeroes it with the others. */
int sfwi_set_density_gradient(sfwi_handle *h, int on);

/* Snapshot imaging.  No reference counterpart: the reference reconstructs
 * the forward wavefield backwards in time from saved edge strips.  With
 * every = k > 0, later gradient runs instead keep the background vx, vz after
 * every k-th forward step (format SFWI_SNAP_F32, or SFWI_SNAP_F16 /
 * SFWI_SNAP_BF16 as 16-bit values scaled by the snapshot's max |v| over the
 * shot) and the backward pass runs the adjoint only, imaging at the snapshot
 * steps with weight k (strains of the snapshot by the reconstruction's
 * stencils; illumination k |v|^2).  every = 0 restores the reconstruction.
 * Device memory: ceil(nt/k) x 2 x packed cells x 4 (FP32) or 2 bytes, in
 * place of the edge strips; at most 512 shots per run; excludes the density
 * kernel. */
#define SFWI_SNAP_F32 1
#define SFWI_SNAP_F16 2
#define SFWI_SNAP_BF16 3
int sfwi_set_snapshots(sfwi_handle *h, int every, int format);

/* Edge strips in host memory: IMAGE_SINGLESHOT's cpu_mem and ntt
 * (sfwi-stage1/FD2DGPU.cuh:466-467; the buffers of FD2DGPU.cu:4382-4421 and
 * the copies of :4548-4561, :4600-4622).  With cpu_mem set, later gradient
 * runs keep on the device a ring of two chunks of ntt steps of strips instead
 * of all nt steps; every full chunk but the last two goes to pinned host
 * memory during the forward sweeps and comes back during the backward
 * sweeps, copied on a second stream while the step kernels run, so the
 * results are the same bits as with the strips on the device.  When 2 ntt >= nt
 * the ring would hold every step and the strips stay on the device.
 * cpu_mem = 0 restores device strips; cpu_mem != 0 needs ntt >= 1. */
int sfwi_set_cpu_mem(sfwi_handle *h, int cpu_mem, int ntt);
/* strip bytes of the last run: on the device, and in pinned host memory */
int sfwi_strip_bytes(sfwi_handle *h, size_t *device_bytes, size_t *host_bytes);
/* Pinned host memory released by handles (their host-held strips) is kept,
 * up to `bytes` in all, in a process-wide cache and reused by the next
 * handle whose strips fit in a cached block, instead of being page-locked
 * again.  0 (the default) keeps nothing; lowering the limit frees cached
 * blocks at once.  No reference counterpart. */
int sfwi_set_pinned_cache(size_t bytes);
int sfwi_read_density_gradient_f64(sfwi_handle *h, double *grad_rho);

/* Records of the last shot-gradient call(s): forward records (stage 1:
 * background; stage 2: scattered), stage-2 background records and the adjoint
 * source, each [ntr][nt] of shot `i` of the last run (0 for the one-shot call).
 * Any pointer may be NULL. */
int sfwi_read_records(sfwi_handle *h, int i, float *syn_z, float *syn_x, float *syn2_z, float *syn2_x, float *res_z,
                      float *res_x);

/* ---- batched shots: many shots per kernel launch ---- */
typedef struct {
    int nx;               /* window width in nodes (may differ between shots) */
    int isx, isz, igz;    /* as sfwi_set_shot_geometry */
    int ngx_left, delta_left, record_left_in_v;
    int ntr;
    const int *gc;        /* [ntr] receiver coordinates */
    const float *rec_z;   /* [ntr][nt] observed records (read when the shot is run) */
    const float *rec_x;
} sfwi_shot_desc;

/* queue a shot; its arrays must stay valid until sfwi_run returns */
int sfwi_enqueue_shot(sfwi_handle *h, const sfwi_shot_desc *shot);
/* drop the queued shots without running them */
int sfwi_clear_queue(sfwi_handle *h);
/* advance every queued shot together (forward, residual, backward, imaging)
 * and clear the queue; misfit += the sum over the shots (in queue order);
 * per_shot_misfit (may be NULL) receives each shot's misfit. */
int sfwi_run(sfwi_handle *h, double *misfit, double *per_shot_misfit);
/* forward modelling only of the queued shots: records are read back with
 * sfwi_read_records; clears the queue */
int sfwi_run_forward(sfwi_handle *h);

/* ---- the Born operator and its exact adjoint (stage 2) ----
 * The Born modelling operator L maps a model perturbation (dVp, dVs) to the
 * scattered records: sfwi_gpu_buffer_m(h, dvp, dvs) then sfwi_run_forward
 * (scattered records in syn_z/syn_x of sfwi_read_records).
 * sfwi_born_adjoint applies its exact transpose to the queued shots' records
 * d (sfwi_enqueue_shot rec_z/rec_x, [ntr][nt]): img_vp, img_vs (host
 * [allnx][allnz], FP64) += L^T d, with <L m, d> = <m, L^T d> to rounding,
 * about the uploaded background model.  It is the transpose of the forward
 * sweeps this library runs (split-field PML included), not of the
 * continuous adjoint equations the gradient path uses
 * (GPUcalculate_elastic_*_back, sfwi-stage1/born.cu:504-603), so
 * L^T L m is the Gauss-Newton Hessian-vector product of the reference's
 * ELSRTM_CALCULATE_Hessian_vector (sfwi-stage1/FD2DGPU.cu:5236-5774) for the
 * discrete operator.  Device memory: 4 nt bytes per packed cell for the
 * background velocities of every step, plus 88 bytes per packed cell.
 * Clears the queue. */
int sfwi_born_adjoint(sfwi_handle *h, double *img_vp, double *img_vs);
/* Gauss-Newton Hessian-vector product of the queued shots (stage 2):
 * hv_vp, hv_vs (host [allnx][allnz], FP64) += L^T L m for m = (dvp, dvs)
 * (host [allnx][allnz]), the counterpart of ELSRTM_CALCULATE_Hessian_vector
 * (sfwi-stage1/FD2DGPU.cuh:477-478, FD2DGPU.cu:5236-5379: a Born forward of
 * the vector, its scattered records propagated back and imaged) with the
 * exact adjoint above, so the product is symmetric and <m, H m> = |L m|^2.
 * It is sfwi_gpu_buffer_m(h, dvp, dvs), sfwi_run_forward, and
 * sfwi_born_adjoint of the scattered records: the uploaded perturbation is
 * replaced by m.  Shots run the handle's nt.  Clears the queue. */
int sfwi_hessian_vector(sfwi_handle *h, const float *dvp, const float *dvs, double *hv_vp, double *hv_vs);

/* ---- shots on several models in one run (request batching) ----
 * No reference counterpart: the reference runs one model per MPI job.  Each
 * model has its own grid (allnx x allnz, with allnz + 2*pml at most the
 * handle's nzpml) and its own number of time steps (nt at most the handle's
 * nt; the wavelet is the first nt samples of the handle's).  Spacing, dt,
 * PML width and stage are the handle's.  A shot's window is cut from its
 * model, so its nx, delta_left and receivers refer to that model. */
typedef struct {
    int allnx, allnz, nt;
    const float *vp, *vs, *rho;  /* host [allnx][allnz]; rho needed in stage 1, ignored in stage 2 */
    const float *dvp, *dvs;      /* stage-2 perturbation, or both NULL (zero) */
} sfwi_model_desc;
/* One gradient run of every queued shot (sfwi_enqueue_shot; records [ntr][the
 * model's nt]), shot i on models[shot_model[i]]: all shots advance in the
 * same kernel launches, a shot only for its model's nt steps.  Outputs, each
 * may be NULL: per_shot_misfit[queue index]; the FP64 gradients and
 * illumination of every model, concatenated in model order (model k at
 * offset sum_{j<k} allnx_j allnz_j), computed afresh (the handle's own
 * accumulated gradients are not touched); grad_rho when the density gradient
 * is on.  A shot's results do not depend on the other shots of the run: they
 * equal a run of that model's shots alone, bit for bit.  When the models'
 * nt differ the misfit must be L2 and snapshots off.  sfwi_read_records(h,
 * i, ...) afterwards takes the queue index and gives [ntr][handle nt] with
 * zeros after the model's nt.  Clears the queue. */
int sfwi_run_models(sfwi_handle *h, int nmodels, const sfwi_model_desc *models, const int *shot_model,
                    double *per_shot_misfit, double *grad_pp, double *grad_ps, double *illum, double *grad_rho);

/* ---- line searches ----
 * CALCULATE_ALPHA_parabola_mb (sfwi-stage1/FD2DGPU.cu:4819-5036, stage 1):
 * the L2 misfit of the current shot at the trial models vp - s grad_pp,
 * vs - s grad_ps for s = 0, step1, step2 (background forward only; rho
 * unchanged), added to *misfit_step0..2.  grad_* are [allnx][allnz] host
 * arrays; the uploaded model is left as it was. */
int sfwi_calculate_alpha_parabola_mb(sfwi_handle *h, const float *grad_pp, const float *grad_ps, float step1,
                                     float step2, double *misfit_step0, double *misfit_step1, double *misfit_step2);
/* CALCULATE_ALPHA (sfwi-stage2/FD2DGPU.cu:4576-4722, stage 2): Born runs of
 * the current shot with the model perturbation image_pp/ps (giving the
 * residual r = (du - d) + u0) and with the search direction cg_pp/ps (giving
 * its scattered records q); *fenzi += sum q.r, *fenmu += sum q.q. */
int sfwi_calculate_alpha(sfwi_handle *h, const float *image_pp, const float *image_ps, const float *cg_pp,
                         const float *cg_ps, double *fenzi, double *fenmu);
/* The same two searches over every queued shot at once: all shots and all
 * trial models advance in the same forward launches.  misfit3[k] += the
 * misfit at step k; per_shot3 (may be NULL) receives [shot][3];
 * per_shot2 (may be NULL) receives [shot][fenzi, fenmu].  Clear the queue. */
int sfwi_line_search_parabola(sfwi_handle *h, const float *grad_pp, const float *grad_ps, float step1, float step2,
                              double *misfit3, double *per_shot3);
int sfwi_line_search_exact(sfwi_handle *h, const float *image_pp, const float *image_ps, const float *cg_pp,
                           const float *cg_ps, double *fenzi, double *fenmu, double *per_shot2);

/* ---- optimal-transport misfit (declared, not implemented, in the reference:
 *      OT / OT_power / OT_alltrace, sfwi-stage1/FD2DGPU.cuh:21-25) ----
 * obs/cal/res are host [tracenum][length]; misfit += W2 over traces and both
 * components; res = (1/2) dW2/dcal (the scaling of the L2 residual). */
int sfwi_ot(const float *obs_x, const float *obs_z, const float *cal_x, const float *cal_z, float *res_x, float *res_z,
            int length, int tracenum, float dt, double *misfit);
int sfwi_ot_power(const float *obs_x, const float *obs_z, const float *cal_x, const float *cal_z, float *res_x,
                  float *res_z, int length, int tracenum, float dt, double *misfit);
int sfwi_ot_alltrace(const float *obs_x, const float *obs_z, const float *cal_x, const float *cal_z, float *res_x,
                     float *res_z, int length, int tracenum, float dt, double *misfit);
/* Allocation-free OT on device buffers.  No counterpart in the reference.
 * For callers that cannot allocate device memory: host programs whose own
 * allocator reserves every device byte up front, and inner loops where a
 * cudaMalloc/cudaFree could synchronise the device and stall the work of
 * other streams.  obs/cal/res are DEVICE pointers [tracenum][length] on the
 * current device; kind is SFWI_MISFIT_OT, SFWI_MISFIT_OT_POWER or
 * SFWI_MISFIT_OT_ALLTRACE; misfit (host) += W2; stream may be NULL (default
 * stream).  The call enqueues its kernels on `stream`, then waits for that
 * stream to reach the misfit read-back.  tracenum = 0 adds nothing and
 * returns SFWI_OK, as sfwi_ot does.
 * Working memory is a fixed 256 KB array that every device loading the
 * library keeps until the process exits: at most 8192 traces per call (larger
 * calls fail with SFWI_E_ARG before any device work) and length <= 7160.
 * The first call in a CUDA context looks up that array's device address
 * (cudaGetSymbolAddress), so make it before any stream capture.  All calls
 * on a device share the array and each call overwrites what the last one
 * left there: calls that overlap on the GPU (other streams or threads at the
 * same time) race on it and must be serialised by the caller. */
int sfwi_ot_noalloc(int kind, const float *obs_x, const float *obs_z, const float *cal_x, const float *cal_z,
                    float *res_x, float *res_z, int length, int tracenum, float dt, double *misfit, void *stream);
/* normalize(matrix, length, tracenum), sfwi-stage1/main.cpp:24-32: divide by
 * the gather's largest absolute value (host code, as in the reference). */
int sfwi_normalize(float *matrix, int length, int tracenum);

/* ---- diagnostics ---- */
const char *sfwi_last_error(void);
/* kernels launched by this handle so far (time-step, set-up and misfit kernels) */
long long sfwi_kernel_launches(sfwi_handle *h);
/* device-side durations (ms, CUDA events on the handle's stream) of the last
 * run: forward loop, backward loop, misfit/adjoint-source kernels, and the
 * whole run from the set-up kernel to the final gradient reduction */
int sfwi_last_timing(sfwi_handle *h, float *fwd_ms, float *bwd_ms, float *other_ms, float *total_ms);
/* average device duration (ms) of one launch of each time-step kernel on the
 * last run's batch: out_ms[0..3] = forward velocity sweep, forward stress
 * sweep, backward stress sweep, backward velocity sweep; each is launched
 * `reps` times back to back between CUDA events on the handle's stream.  The
 * launches overwrite the wavefields of the last run (its records and
 * gradients, already read or accumulated, are untouched). */
int sfwi_time_kernels(sfwi_handle *h, int reps, float *out_ms);

/* Debugging: the packed [X][P] arrays of the batch on the device (X packed
 * rows: the shots' padded widths in enqueue order; P the padded depth
 * rounded up to 4).  Arrays 0 .. nstate-1 are the wavefields, PML memory
 * variables and imaging accumulators (zeroed per run), the rest the
 * coefficients.  sfwi_debug_read_grid copies X*P floats of one array. */
int sfwi_debug_grid_shape(sfwi_handle *h, int *X, int *P, int *narrays, int *nstate);
/* Debugging, host only (no device use): the tile grid a batch of shots with
 * padded widths nxpml[0..nshots-1] and padded depth nzpml gets on tx x tz
 * tiles.  z_start is the batch's first tile column (NOP - 8k), x_start[s]
 * each shot's first tile row (at most NOP); tiles[s] and frame_tiles[s]
 * (optional) count each shot's tiles and those holding PML cells. */
int sfwi_debug_tile_grid(int pml, int nzpml, int tx, int tz, const int *nxpml, int nshots, int *z_start,
                         int *x_start, int *tiles, int *frame_tiles);
int sfwi_debug_read_grid(sfwi_handle *h, int array, float *dst);

/* Failure path of the device-side waits, without a fault: runs the tile
 * pipeline of the last batch with a producer that stages nothing and a wait
 * bound of `tries` (1..2^24) mbarrier tries, so the consumers' and the
 * producer's waits run out.  The kernel sets the device error flag and
 * returns, and the call reports it as a run does: SFWI_E_CUDA with "a
 * device-side pipeline wait timed out".  The flag is cleared afterwards and
 * the handle stays usable. */
int sfwi_wait_selftest(sfwi_handle *h, unsigned tries);

/* Source of the forward sweeps.  SFWI_SOURCE_TXX_TZZ (default) is the
 * reference's: sou[it] added to txx and tzz at the source cell ahead of the
 * velocity sweep (sfwi-stage1/FD2DGPU.cu:2104-2114).  SFWI_SOURCE_VZ_FORCE is
 * a vertical force with no reference counterpart: sou[it] added to vz at the
 * source cell after the velocity sweep.  Both go into the total field only,
 * so the next sweep of that field rebuilds it from its split parts. */
#define SFWI_SOURCE_TXX_TZZ 0
#define SFWI_SOURCE_VZ_FORCE 1
int sfwi_set_source(sfwi_handle *h, int kind);

/* Tile shapes of the step kernels (cells of a tile's core, x by z; CTAs per
 * SM; cells per compute thread): each is compiled as its own set of kernels.
 *   16x32           two CTAs per SM, two pipeline stages each, 4 cells a thread
 *   32x32, 16x64    one CTA (two stages fill the shared memory), less halo
 *   8x32_3CTA       three CTAs of half-height tiles
 *   16x32_2CELL     16x32 with 2 cells a thread: twice the warps, fewer registers
 *   8x32_2CELL_3STAGE  half-height tiles, 2 cells a thread, three stages: the
 *                   most tiles in flight, for small batches */
#define SFWI_TILE_16x32 0
#define SFWI_TILE_32x32 1
#define SFWI_TILE_16x64 2
#define SFWI_TILE_8x32_3CTA 3
#define SFWI_TILE_16x32_2CELL 4
#define SFWI_TILE_8x32_2CELL_3STAGE 5
#define SFWI_NUM_TILE_SHAPES 6

/* Select the tile shape for this handle's runs.  Until one is selected (here
 * or by sfwi_autotune) each batch gets SFWI_TILE_16x32, or
 * SFWI_TILE_8x32_2CELL_3STAGE when its 16x32 tiles would give fewer than four
 * to each of the device's CTA slots (small batches).  A batch already on
 * the device is re-tiled.  Results do not depend on the shape: they are
 * bit-identical, since every cell takes the same update (split where the cell
 * is damped, plain elsewhere, whatever its tile holds), reads the same values
 * and rounds in the same order. */
int sfwi_set_tile_shape(sfwi_handle *h, int shape);
/* Launch the time-step kernels with programmatic dependent launch (default
 * on): each may be scheduled while the previous one drains and waits for its
 * results on the device, which hides the launch gap between the sweeps.
 * Results do not depend on it. */
int sfwi_set_launch_overlap(sfwi_handle *h, int on);
/* Tile order of the time-step sweeps: bit k set (k = 0 forward velocity, 1
 * forward stress, 2 backward stress, 3 backward velocity sweep) draws that
 * sweep's tiles in reverse table order.  The default, bits 1 and 3, makes
 * each sweep start where the one before it ended (its freshest outputs are
 * still in L2).  Results do not depend on it. */
int sfwi_set_tile_order(sfwi_handle *h, unsigned reverse_bits);
int sfwi_get_tile_shape(sfwi_handle *h, int *shape, int *tx, int *tz);

/* Autotuner: after a gradient run (sfwi_run or sfwi_image_singleshot), time one
 * step of the four step kernels for every tile shape on the resident batch
 * (reps steps each, as sfwi_time_kernels) and keep the fastest.  *choice gets
 * its SFWI_TILE_* index, out_ms (optional, SFWI_NUM_TILE_SHAPES floats) the
 * per-step time of each shape.  Like sfwi_time_kernels it overwrites the
 * last run's wavefields; its gradients, already accumulated, are untouched. */
int sfwi_autotune(sfwi_handle *h, int reps, int *choice, float *out_ms);
/* page-locked host buffers (cudaMallocHost) for records that are copied every
 * iteration; free with sfwi_host_free */
int sfwi_host_alloc(size_t bytes, void **ptr);
int sfwi_host_free(void *ptr);
/* library version string */
const char *sfwi_version(void);

#ifdef __cplusplus
}
#endif
#endif
