/* sfwi_oracle.h — call interface shared by the CPU oracle (sfwi_oracle.c) and
 * the CPU build of the reference's own kernels (ref_harness.cpp).
 *
 * TEST INFRASTRUCTURE ONLY.  These entry points are the checker for the CUDA
 * path: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load them, and nothing in sfwi_gb300/ links or calls them.
 *
 * One call runs one shot-gradient the way the reference's IMAGE_SINGLESHOT
 * does (sfwi-stage1/FD2DGPU.cu:4321-4695, sfwi-stage2/FD2DGPU.cu:3978-4570),
 * including the per-shot set-up the caller does before it
 * (sfwi-stage1/main.cpp:585-625: record upload, model window cut, geometry).
 *
 * Layouts follow the reference: models and gradients are [allnx][allnz]
 * (z fastest), records are [ntr][nt] (time fastest).
 */
#ifndef SFWI_ORACLE_H
#define SFWI_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int stage;            /* 1: background forward, L2 residual syn-obs, adjoint dir +1
                             2: background+Born forward, residual (du-obs)+u0, dir -1, rho=2000 */
    int allnx, allnz;     /* global model size */
    int nx;               /* window width in nodes (interior, without PML) */
    int pml, nop, nt, ntr;
    float dx, dz, dt;
    int isx, isz, igz;    /* padded-grid source column/row and receiver row */
    int ngx_left;         /* leftmost coordinate of the shot (same unit as gc) */
    int delta_left;       /* window start column in the global model */
    int record_left_in_v; /* added to delta_left for the window and the gradient */
    int forward_only;     /* 1: stop after the forward loop (records only) */
    int misfit_kind;      /* 0: L2 as the reference; 1: 1D optimal transport (oracle only) */
    int nthreads;         /* OpenMP threads for the emulated launches / loops (<=0: all) */
    int snap_every;       /* oracle only: 0 = reconstruction (as the reference); k > 0 = image
                             from exact forward snapshots of vx, vz every k-th step, weight k */
    int src_kind;         /* oracle only: 0 = sou[it] added to txx and tzz before the velocity
                             sweep (as the reference); 1 = vertical force, sou[it] added to vz
                             after the velocity sweep */
} sfwi_oracle_shot;

typedef struct {
    const float *vp_all, *vs_all, *rho_all;   /* [allnx][allnz]; rho ignored by stage 2 */
    const float *dvp_all, *dvs_all;           /* stage 2 model perturbation [allnx][allnz] */
    const float *sou;                         /* [nt] source wavelet */
    const float *obs_z, *obs_x;               /* [ntr][nt] observed records */
    const int *gc;                            /* [ntr] receiver coordinates */
    /* outputs; any may be NULL */
    double *syn_z, *syn_x;    /* [ntr][nt] recorded: stage 1 background, stage 2 scattered */
    double *syn2_z, *syn2_x;  /* [ntr][nt] stage 2 background records */
    double *res_z, *res_x;    /* [ntr][nt] adjoint source (residual) */
    double *grad_pp, *grad_ps, *illum; /* [allnx][allnz], accumulated (+=) */
    double *grad_rho;         /* [allnx][allnz] density kernel (oracle only; += ) */
    double *misfit;           /* += */
} sfwi_oracle_io;

#ifdef __cplusplus
}
#endif
#endif
