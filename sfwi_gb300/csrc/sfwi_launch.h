// sfwi_launch.h — host-side launch interface of the kernels (one definition
// of each argument block, shared by the kernel files and the engine).
#pragma once
#include <cuda.h>  // CUtensorMap (types only; the driver is reached through cudaGetDriverEntryPoint)

#include "sfwi_common.cuh"

namespace sfwi {

// sfwi_kernels.cu
// TMA descriptors of the packed grid, 3-D [array][row][column]: box[k] and
// core[k] fetch k+1 consecutive arrays per instruction as (TX+2*HALO) x
// (TZ+2*HALO) halo boxes or TX x TZ core tiles (one TMA instruction costs the
// issuing warp about the same whatever its size, so arrays read together are
// fetched together)
struct TmaMaps {
    CUtensorMap box[3], core[3];
    CUtensorMap tb, lr;  // edge strips (top/bottom, left/right layouts)
    CUtensorMap rs;      // residual source per packed row [X][2 nt]
    CUtensorMap snap;    // forward snapshots [snapshot * 2 + comp][X][PS], vx and vz per box (depth 2)
};
// One build of the step kernels for one tile shape (sfwi_kernels.cu is
// compiled once per shape): tx x tz cells per tile, `ctas` persistent CTAs
// per SM.  launch runs one kernel of a time step: 0 fwd v, 1 fwd s, 2 bwd s,
// 3 bwd v.
struct TileVariant {
    int tx, tz, halo, ctas, stages;
    const char *name;
    cudaError_t (*configure)();
    void (*launch)(int which, const Params &p, const TmaMaps &tm, int it, bool born, float adj_dir, cudaStream_t st);
    void (*wait_probe)(const Params &p, cudaStream_t st);
};
const TileVariant *tile_variant_16x32();
const TileVariant *tile_variant_32x32();
const TileVariant *tile_variant_16x64();
const TileVariant *tile_variant_8x32x3();
const TileVariant *tile_variant_16x32c2();
const TileVariant *tile_variant_8x32c2s3();

// sfwi_aux.cu
struct SetupArgs {
    int X, P, nzpml, pml, allnz, stage, born_lo;
    float dt;
    const float *vp_all, *vs_all, *rho_all, *dvp_all, *dvs_all;
    size_t vslot, mslot;  // floats between model slots of vp/vs and of dvp/dvs (0: one model)
    float *ib, *lam, *mu, *dampx, *dampz, *bp, *bs, *vp, *vs, *rho;
    const ShotGeo *geo;
    // batches of shots on several models (sfwi_run_models): each shot's model
    // at aux[s].moff in the concatenated model arrays, with its own grid;
    // null: every shot cuts its window from the model slots above
    const ShotAux *aux;
};
void launch_setup(const SetupArgs &a, int nshots, int max_nxpml, cudaStream_t st);
// tlen (may be null): samples of each trace; later samples are written as zeros
void launch_record_gather(const float *rrow, const int *trow, const int *tlen, int nt, int nrc, int X, int ntr,
                          float *out, size_t cstride, cudaStream_t st);
void launch_recv_source(const float *res_z, const float *res_x, const int *rtr, int nt, int X, int rsp, float *rs,
                        cudaStream_t st);
void launch_residual_l2(int stage, int nt, int ntr_tot, const float *syn_z, const float *syn_x, const float *syn2_z,
                        const float *syn2_x, const float *obs_z, const float *obs_x, float *res_z, float *res_x,
                        double *trace_misfit, cudaStream_t st);
struct FinalArgs {
    int allnx, allnz, P, pml, nshots;
    const ShotGeo *geo;
    const float *glam, *gmu, *illum, *vp, *vs, *rho;
    double *gpp, *gps, *gil;
    const float *grho;  // density kernel per cell, or null
    double *grh;
};
void launch_finalize(const FinalArgs &a, cudaStream_t st);
// out[k] = base[k] - step[k] * g (k < nslot; no fused multiply-add, as the
// reference forms its trial models on the host)
void launch_trial_models(const float *base, const float *g, const float *steps, int nslot, size_t n, float *out,
                         cudaStream_t st);
// per trace tr < ntr: sum_t (a.b) and sum_t (a.a) over the z and x components
// of trace-major records, each term formed in float and summed in double
void launch_trace_dots(const float *az, const float *ax, const float *bz, const float *bx, int nt, int ntr,
                       double *ab, double *aa, cudaStream_t st);

// sfwi_ot.cu
// floor of the per-trace OT scale, relative to the gather's max |obs|
constexpr double OT_SIGMA_FLOOR = 1e-3;
struct OtArgs {
    int kind, nt, ntr, stage;
    double dt;
    const float *cal_z, *cal_x;    // [ntr][nt] prediction (stage 2: scattered part)
    const float *cal2_z, *cal2_x;  // stage 2: background part added to cal (may be null)
    const float *obs_z, *obs_x;
    float *res_z, *res_x;
    const double *sigma;          // [ntr][2] (z, x)
    double *trace_misfit;         // [ntr][2]
    double *scratch;              // traces longer than ot_max_nt(): ot_scratch_doubles(nt, ntr) doubles
};
cudaError_t launch_ot(const OtArgs &a, cudaStream_t st);
size_t ot_smem_bytes(int nt);
// longest trace held in shared memory; longer ones need the global scratch
int ot_max_nt();
size_t ot_scratch_doubles(int nt, int ntr);
// OT scales of a batch on the device: max |obs| per (trace, component),
// floored per shot (sigma: 2 doubles per trace; geo: the batch's shots)
void launch_ot_scales(const float *obs_z, const float *obs_x, int nt, int ntr, const ShotGeo *geo, int nshots,
                      int all, double *sigma, cudaStream_t st);

// sfwi_adjoint.cu: the exact adjoint of the Born modelling operator
struct AdjArgs {
    int X, P, PS, pml, nt, born_lo;
    float dt, dtdx, dtdz, idx, idz;
    const ShotGeo *geo;
    const int *rowshot;  // [X]: the shot of each packed row
    const float *ib, *lam, *mu, *dampx, *dampz;
    // adjoint state (velocities, stresses and their x-parts) and the fields
    // the transposed stencils gather, each [X][P]
    float *avx, *avz, *amx, *amz, *atxx, *atzz, *atxz, *amxx, *amzz, *amxz;
    float *gax, *gbz, *gcz, *gdx, *hax, *hbz, *hdx, *hcz;
    double *dbp, *dbs;   // adjoints of 2 rho vp dVp and 2 rho vs dVs per window cell
    const float *snap;   // background vx, vz after each step's velocity sweep, [2 it + comp][X][PS]
    const float *dz, *dx;  // the data (records' adjoint), trace-major [ntr][nt]
    const int *rstart, *rtr;  // per packed row: the traces recorded there, rtr[rstart[row] .. rstart[row+1])
};
void launch_adjoint_step(const AdjArgs &a, int it, cudaStream_t st);
struct ImageArgs {
    int allnx, allnz, P, pml, nshots;
    const ShotGeo *geo;
    const double *dbp, *dbs;
    const float *vp, *vs, *rho;
    double *img_vp, *img_vs;
};
void launch_born_image(const ImageArgs &a, cudaStream_t st);

// sfwi_engine.cu: set the calling thread's sfwi_last_error() message; returns code
int record_error(int code, const char *fmt, ...);

}  // namespace sfwi
