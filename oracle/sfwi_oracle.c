/* sfwi_oracle.c — CPU restatement of the reference's per-shot gradient path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle the CUDA path is checked
 * against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it; the product (sfwi_gb300/) never links or calls it.
 *
 * The file is compiled twice: -DORC_REAL=double gives the FP64 oracle
 * (symbols orc64_*), -DORC_REAL=float the single-threaded FP32 transliteration
 * timed as the CPU baseline (symbols orc32_*).  In the FP32 build every
 * expression keeps the reference's own literal types, so the places where the
 * reference promotes to double (1.0/rho in the velocity updates) promote here
 * too.
 *
 * State follows the reference exactly: every field carries its split PML
 * memory variables over the whole padded grid, the source and the adjoint
 * source are written into the total fields only, and the edge strips of vx/vz
 * are restored into the total fields only (sfwi-stage1/FD2DGPU.cu:3873-3899).
 * Each function cites the reference code it restates.
 *
 * Additions with no reference counterpart (parity unpinned):
 *   - misfit_kind 1..3: per-trace 1D quadratic-Wasserstein misfit and its
 *     adjoint source (orc*_ot_trace below);
 *   - grad_rho: a density kernel -sum_t v_adj . dv/dt, with dv the velocity
 *     step of the reconstruction (the reference computes no density
 *     gradient);
 *   - snap_every = k > 0: no reconstruction and no edge strips; the forward
 *     vx, vz are kept (exactly) after every k-th step, and the backward pass
 *     images at those steps only, with strains taken from the kept velocities
 *     by the reconstruction's own stencils (update_s) and weight k; the
 *     illumination is k * |v|^2 of the kept velocities.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "sfwi_oracle.h"

#ifndef ORC_REAL
#define ORC_REAL double
#endif
#ifndef ORC_PREFIX
#define ORC_PREFIX orc64_
#endif
typedef ORC_REAL real;
#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(ORC_PREFIX, name)

#ifdef _OPENMP
#include <omp.h>
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

/* 8th-order staggered first-derivative weights, sfwi-stage1/FD2DGPU.cuh:16 */
static const real C8[5] = {0, (real)(1225.0 / 1024.0), (real)(-245.0 / 3072.0), (real)(49.0 / 5120.0),
                           (real)(-5.0 / 7168.0)};

typedef struct {
    int nxpml, nzpml, nx, nz, pml, nop;
    real dx, dz, dt;
} grid_t;

#define IDX(ix, iz) ((size_t)(ix) * g->nzpml + (iz))

/* Ricker wavelet, sfwi-stage1/main.cpp:251-260 */
void FN(ricker)(float *w, int nt, float dt, float fm) {
    /* ricker_wave, sfwi-stage1/main.cpp:251-260: PI is a double literal
     * (main.cpp:8), Nk is stored as float, the exponent is a float product */
    const double PI_ = 3.14159265358979;
    const float Nk = (float)(PI_ * PI_ * fm * fm * dt * dt);
    const int t0 = (int)ceil(1.0 / (fm * dt));
    for (int t = 0; t < nt; t++)
        w[t] = (float)((1.0 - 2.0 * Nk * (t - t0) * (t - t0)) * exp(-Nk * (t - t0) * (t - t0)));
}

/* Window cut + PML edge replication: copyvelocityHtoD, copypmlVz, copypmlVx
 * (sfwi-stage1/FD2DGPU.cu:112-123, 233-249).  z-edges first, then x-edges
 * copy whole columns, so the corners take the z-extended values. */
static void window_model(const grid_t *g, const float *all, int allnz, int ngx_min, real *out) {
    for (int ix = 0; ix < g->nx; ix++)
        for (int iz = 0; iz < g->nz; iz++) out[IDX(ix + g->pml, iz + g->pml)] = all[(size_t)(ngx_min + ix) * allnz + iz];
    for (int ix = 0; ix < g->nxpml; ix++)
        for (int iz = 0; iz < g->pml; iz++) {
            out[IDX(ix, iz)] = out[IDX(ix, g->pml)];
            out[IDX(ix, g->nzpml - g->pml + iz)] = out[IDX(ix, g->nzpml - g->pml - 1)];
        }
    for (int ix = 0; ix < g->pml; ix++)
        for (int iz = 0; iz < g->nzpml; iz++) {
            out[IDX(ix, iz)] = out[IDX(g->pml, iz)];
            out[IDX(g->nxpml - g->pml + ix, iz)] = out[IDX(g->nxpml - g->pml - 1, iz)];
        }
}

/* PML profiles, dampX/dampZ (sfwi-stage1/FD2DGPU.cu:443-493) with rr = 1e-3
 * (:1310).  Left/top strips cover i < pml, right/bottom strips i > n-pml. */
static void damping(const grid_t *g, const real *vp, real *dampx, real *dampz) {
    const float rr = 0.001f;
    const float l10 = log10f(1 / rr);
    const int pml = g->pml;
    for (int ix = 0; ix < g->nxpml; ix++)
        for (int iz = 0; iz < g->nzpml; iz++) {
            size_t i = IDX(ix, iz);
            real p = vp[i];
            dampx[i] = 0;
            dampz[i] = 0;
            if (ix < pml) dampx[i] = (real)(l10 * (5.0 * p / (2.0 * pml)) * powf((float)(1.0 * (pml - ix) / pml), 4.0f));
            if (ix > g->nxpml - pml)
                dampx[i] = (real)(l10 * (5.0 * p / (2.0 * pml)) * powf((float)(1.0 * (ix - (g->nxpml - pml)) / pml), 4.0f));
            if (iz < pml) dampz[i] = (real)(l10 * (5.0 * p / (2.0 * pml)) * powf((float)(1.0 * (pml - iz) / pml), 4.0f));
            if (iz > g->nzpml - pml)
                dampz[i] = (real)(l10 * (5.0 * p / (2.0 * pml)) * powf((float)(1.0 * (iz - (g->nzpml - pml)) / pml), 4.0f));
        }
}

/* update_vx_vz, sfwi-stage1/born.cu:355-394 */
static void update_v(const grid_t *g, const real *txx, const real *tzz, const real *txz, real *vx, real *vx_x,
                     real *vx_z, real *vz, real *vz_x, real *vz_z, const real *rho, const real *dampx,
                     const real *dampz, int direction) {
    const int nop = g->nop;
    const real dt = g->dt, dx = g->dx, dz = g->dz;
    const int nz = g->nzpml;
    OMP_FOR
    for (int ix = nop; ix < g->nxpml - nop; ix++)
        for (int iz = nop; iz < g->nzpml - nop; iz++) {
            size_t i = (size_t)ix * nz + iz;
            real damp1 = 1 - dt * dampx[i] / 2, damp2 = 1 + dt * dampx[i] / 2;
            real damp3 = 1 - dt * dampz[i] / 2, damp4 = 1 + dt * dampz[i] / 2;
            real a = 0, b = 0, c = 0, d = 0;
            for (int k = 1; k <= nop; k++) {
                a += C8[k] * (txx[(size_t)(ix + k) * nz + iz] - txx[(size_t)(ix - k + 1) * nz + iz]);
                b += C8[k] * (txz[(size_t)ix * nz + iz + k - 1] - txz[(size_t)ix * nz + iz - k]);
                c += C8[k] * (tzz[(size_t)ix * nz + iz + k] - tzz[(size_t)ix * nz + iz - k + 1]);
                d += C8[k] * (txz[(size_t)(ix + k - 1) * nz + iz] - txz[(size_t)(ix - k) * nz + iz]);
            }
            vx_x[i] = (real)((damp1 * vx_x[i] + direction * (1.0 / rho[i]) * (dt / dx) * a) / damp2);
            vx_z[i] = (real)((damp3 * vx_z[i] + direction * (1.0 / rho[i]) * (dt / dz) * b) / damp4);
            vz_x[i] = (real)((damp1 * vz_x[i] + direction * (1.0 / rho[i]) * (dt / dx) * d) / damp2);
            vz_z[i] = (real)((damp3 * vz_z[i] + direction * (1.0 / rho[i]) * (dt / dz) * c) / damp4);
            vx[i] = vx_x[i] + vx_z[i];
            vz[i] = vz_x[i] + vz_z[i];
        }
}

/* update_txx_tzz_txz (born.cu:399-440); with strains != NULL it is
 * update_txx_tzz_txz_grad (born.cu:451-499), which also stores dv/dx, dv/dz. */
static void update_s(const grid_t *g, real *txx, real *tzz, real *txx_x, real *txx_z, real *tzz_x, real *tzz_z,
                     real *txz, real *txz_x, real *txz_z, const real *vx, const real *vz, const real *lam,
                     const real *mu, const real *dampx, const real *dampz, int direction, real *vx_gx, real *vz_gz,
                     real *vx_gz, real *vz_gx) {
    const int nop = g->nop;
    const real dt = g->dt, dx = g->dx, dz = g->dz;
    const int nz = g->nzpml;
    OMP_FOR
    for (int ix = nop; ix < g->nxpml - nop; ix++)
        for (int iz = nop; iz < g->nzpml - nop; iz++) {
            size_t i = (size_t)ix * nz + iz;
            real damp1 = 1 - dt * dampx[i] / 2, damp2 = 1 + dt * dampx[i] / 2;
            real damp3 = 1 - dt * dampz[i] / 2, damp4 = 1 + dt * dampz[i] / 2;
            real a = 0, b = 0, c = 0, d = 0; /* vx_x, vz_z, vx_z, vz_x */
            for (int k = 1; k <= nop; k++) {
                a += C8[k] * (vx[(size_t)(ix + k - 1) * nz + iz] - vx[(size_t)(ix - k) * nz + iz]);
                b += C8[k] * (vz[(size_t)ix * nz + iz + k - 1] - vz[(size_t)ix * nz + iz - k]);
                c += C8[k] * (vx[(size_t)ix * nz + iz + k] - vx[(size_t)ix * nz + iz - k + 1]);
                d += C8[k] * (vz[(size_t)(ix + k) * nz + iz] - vz[(size_t)(ix - k + 1) * nz + iz]);
            }
            txx_x[i] = (damp1 * txx_x[i] + direction * (lam[i] + 2 * mu[i]) * (dt / dx) * a) / damp2;
            txx_z[i] = (damp3 * txx_z[i] + direction * lam[i] * (dt / dz) * b) / damp4;
            tzz_x[i] = (damp1 * tzz_x[i] + direction * lam[i] * (dt / dx) * a) / damp2;
            tzz_z[i] = (damp3 * tzz_z[i] + direction * (lam[i] + 2 * mu[i]) * (dt / dz) * b) / damp4;
            txz_x[i] = (damp1 * txz_x[i] + direction * (dt / dx) * mu[i] * d) / damp2;
            txz_z[i] = (damp3 * txz_z[i] + direction * (dt / dz) * mu[i] * c) / damp4;
            txx[i] = txx_x[i] + txx_z[i];
            tzz[i] = tzz_x[i] + tzz_z[i];
            txz[i] = txz_x[i] + txz_z[i];
            if (vx_gx) {
                vx_gx[i] = a / dx;
                vz_gz[i] = b / dz;
                vx_gz[i] = c / dz;
                vz_gx[i] = d / dx;
            }
        }
}

/* the strains update_s forms (vx_x, vz_z, vx_z, vz_x), from given velocities */
static void strains(const grid_t *g, const real *vx, const real *vz, real *gxx, real *gzz, real *gxz, real *gzx) {
    const int nop = g->nop, nz = g->nzpml;
    const real dx = g->dx, dz = g->dz;
    OMP_FOR
    for (int ix = nop; ix < g->nxpml - nop; ix++)
        for (int iz = nop; iz < g->nzpml - nop; iz++) {
            size_t i = (size_t)ix * nz + iz;
            real a = 0, b = 0, c = 0, d = 0;
            for (int k = 1; k <= nop; k++) {
                a += C8[k] * (vx[(size_t)(ix + k - 1) * nz + iz] - vx[(size_t)(ix - k) * nz + iz]);
                b += C8[k] * (vz[(size_t)ix * nz + iz + k - 1] - vz[(size_t)ix * nz + iz - k]);
                c += C8[k] * (vx[(size_t)ix * nz + iz + k] - vx[(size_t)ix * nz + iz - k + 1]);
                d += C8[k] * (vz[(size_t)(ix + k) * nz + iz] - vz[(size_t)(ix - k + 1) * nz + iz]);
            }
            gxx[i] = a / dx;
            gzz[i] = b / dz;
            gxz[i] = c / dz;
            gzx[i] = d / dx;
        }
}

/* GPUcalculate_elastic_txx_tzz_txz_back, born.cu:565-603 */
static void back_s(const grid_t *g, real *txx, real *tzz, real *txx_x, real *tzz_z, real *txz, real *txz_x,
                   real *txz_z, const real *vx, const real *vz, const real *dampx, const real *dampz, int direction) {
    const int nop = g->nop;
    const real dt = g->dt, dx = g->dx, dz = g->dz;
    const int nz = g->nzpml;
    OMP_FOR
    for (int ix = nop; ix < g->nxpml - nop; ix++)
        for (int iz = nop; iz < g->nzpml - nop; iz++) {
            size_t i = (size_t)ix * nz + iz;
            real damp1 = 1 - dt * dampx[i] / 2, damp2 = 1 + dt * dampx[i] / 2;
            real damp3 = 1 - dt * dampz[i] / 2, damp4 = 1 + dt * dampz[i] / 2;
            real a = 0, b = 0, c = 0, d = 0;
            for (int k = 1; k <= nop; k++) {
                a += C8[k] * (vx[(size_t)(ix + k - 1) * nz + iz] - vx[(size_t)(ix - k) * nz + iz]);
                b += C8[k] * (vz[(size_t)ix * nz + iz + k - 1] - vz[(size_t)ix * nz + iz - k]);
                c += C8[k] * (vx[(size_t)ix * nz + iz + k] - vx[(size_t)ix * nz + iz - k + 1]);
                d += C8[k] * (vz[(size_t)(ix + k) * nz + iz] - vz[(size_t)(ix - k + 1) * nz + iz]);
            }
            txx_x[i] = (damp1 * txx_x[i] + direction * (dt / dx) * a) / damp2;
            tzz_z[i] = (damp3 * tzz_z[i] + direction * (dt / dz) * b) / damp4;
            txz_x[i] = (damp1 * txz_x[i] + direction * (dt / dx) * d) / damp2;
            txz_z[i] = (damp3 * txz_z[i] + direction * (dt / dz) * c) / damp4;
            txx[i] = txx_x[i];
            tzz[i] = tzz_z[i];
            txz[i] = txz_x[i] + txz_z[i];
        }
}

/* GPUcalculate_elastic_vx_vz_back, born.cu:504-562 (Lame factors inside the
 * derivative) */
static void back_v(const grid_t *g, const real *txx, const real *tzz, const real *txz, real *vx, real *vx_x,
                   real *vx_z, real *vz, real *vz_x, real *vz_z, const real *lam, const real *mu, const real *rho,
                   const real *dampx, const real *dampz, int direction) {
    const int nop = g->nop;
    const real dt = g->dt, dx = g->dx, dz = g->dz;
    const int nz = g->nzpml;
#define L2M(j) (lam[j] + 2 * mu[j])
    OMP_FOR
    for (int ix = nop; ix < g->nxpml - nop; ix++)
        for (int iz = nop; iz < g->nzpml - nop; iz++) {
            size_t i = (size_t)ix * nz + iz;
            real damp1 = 1 - dt * dampx[i] / 2, damp2 = 1 + dt * dampx[i] / 2;
            real damp3 = 1 - dt * dampz[i] / 2, damp4 = 1 + dt * dampz[i] / 2;
            real txx_x = 0, txz_z = 0, tzz_x = 0, tzz_z = 0, txz_x = 0, txx_z = 0;
            for (int k = 1; k <= nop; k++) {
                size_t xp = (size_t)(ix + k) * nz + iz, xm = (size_t)(ix - k + 1) * nz + iz;
                size_t xp1 = (size_t)(ix + k - 1) * nz + iz, xm1 = (size_t)(ix - k) * nz + iz;
                size_t zp = (size_t)ix * nz + iz + k, zm = (size_t)ix * nz + iz - k + 1;
                size_t zp1 = (size_t)ix * nz + iz + k - 1, zm1 = (size_t)ix * nz + iz - k;
                txx_x += C8[k] * (L2M(xp) * txx[xp] - L2M(xm) * txx[xm]);
                txz_z += C8[k] * (mu[zp1] * txz[zp1] - mu[zm1] * txz[zm1]);
                tzz_x += C8[k] * (lam[xp] * tzz[xp] - lam[xm] * tzz[xm]);
                tzz_z += C8[k] * (L2M(zp) * tzz[zp] - L2M(zm) * tzz[zm]);
                txz_x += C8[k] * (mu[xp1] * txz[xp1] - mu[xm1] * txz[xm1]);
                txx_z += C8[k] * (lam[zp] * txx[zp] - lam[zm] * txx[zm]);
            }
            vx_x[i] = (real)((damp1 * vx_x[i] + direction * (1.0 / rho[i]) * (dt / dx) * txx_x +
                              direction * (1.0 / rho[i]) * (dt / dx) * tzz_x) / damp2);
            vx_z[i] = (real)((damp3 * vx_z[i] + direction * (1.0 / rho[i]) * (dt / dz) * txz_z) / damp4);
            vz_x[i] = (real)((damp1 * vz_x[i] + direction * (1.0 / rho[i]) * (dt / dx) * txz_x) / damp2);
            vz_z[i] = (real)((damp3 * vz_z[i] + direction * (1.0 / rho[i]) * (dt / dz) * tzz_z +
                              direction * (1.0 / rho[i]) * (dt / dz) * txx_z) / damp4);
            vz[i] = vz_x[i] + vz_z[i];
            vx[i] = vx_x[i] + vx_z[i];
        }
#undef L2M
}

/* add_born_source_components: stage 2 version (sfwi-stage2/born.cu:749-801,
 * region [nop, n-nop)); stage 1 version (sfwi-stage1/born.cu:830-882) uses
 * [pml, n-pml).  Adds dt * (delta-Vp/Vs Born source) into the scattered split
 * stresses. */
static void born_source(const grid_t *g, int lo, const real *vx, const real *vz, real *bxx_x, real *bxx_z,
                        real *bzz_x, real *bzz_z, real *bxz_x, real *bxz_z, const real *dmp, const real *dms,
                        const real *rho, const real *vp, const real *vs, int direction) {
    const int nop = g->nop;
    const real dt = g->dt, dx = g->dx, dz = g->dz;
    const int nz = g->nzpml;
    OMP_FOR
    for (int ix = lo; ix < g->nxpml - lo; ix++)
        for (int iz = lo; iz < g->nzpml - lo; iz++) {
            size_t i = (size_t)ix * nz + iz;
            real a = 0, b = 0, c = 0, d = 0;
            for (int k = 1; k <= nop; k++) {
                a += C8[k] * (vx[(size_t)(ix + k - 1) * nz + iz] - vx[(size_t)(ix - k) * nz + iz]);
                b += C8[k] * (vz[(size_t)ix * nz + iz + k - 1] - vz[(size_t)ix * nz + iz - k]);
                c += C8[k] * (vx[(size_t)ix * nz + iz + k] - vx[(size_t)ix * nz + iz - k + 1]);
                d += C8[k] * (vz[(size_t)(ix + k) * nz + iz] - vz[(size_t)(ix - k + 1) * nz + iz]);
            }
            bxx_x[i] = bxx_x[i] + direction * dt * (2 * (rho[i] * vp[i]) * (dmp[i]) * (a) / dx);
            bxx_z[i] = bxx_z[i] + direction * dt * ((2 * (rho[i] * vp[i]) * (dmp[i]) - 4 * (rho[i] * vs[i]) * (dms[i])) * (b) / dz);
            bzz_x[i] = bzz_x[i] + direction * dt * ((2 * (rho[i] * vp[i]) * (dmp[i]) - 4 * (rho[i] * vs[i]) * (dms[i])) * (a) / dx);
            bzz_z[i] = bzz_z[i] + direction * dt * (2 * (rho[i] * vp[i]) * (dmp[i]) * (b) / dz);
            bxz_x[i] = bxz_x[i] + direction * dt * ((2 * (rho[i] * vs[i]) * (dms[i])) * ((d) / dx));
            bxz_z[i] = bxz_z[i] + direction * dt * ((2 * (rho[i] * vs[i]) * (dms[i])) * ((c) / dz));
        }
}

/* receiver column, GPUrecord_scatterwavefield (sfwi-stage1/FD2DGPU.cu:3161);
 * stage 2 passes dx as an int (sfwi-stage2/FD2DGPU.cu:3109) */
static int receiver_ix(int stage, int pml, int gc, int ngx_left, float dx) {
    if (stage == 2) return pml + (int)((float)(gc - ngx_left) / (int)dx);
    return pml + (int)((float)(gc - ngx_left) / dx);
}

/* column where the residual of a trace is injected,
 * GPUapplysource_backward_from_record: dx stays a float in both stages
 * (sfwi-stage1/FD2DGPU.cu:3425-3441, sfwi-stage2/FD2DGPU.cu:3357-3370), so in
 * stage 2 it differs from the recording column when dx is not a whole number */
static int injection_ix(int pml, int gc, int ngx_left, float dx) { return pml + (int)((float)(gc - ngx_left) / dx); }

/* edge strips of vx/vz: record_edge_wavefield / load_edge_wavefield
 * (sfwi-stage1/FD2DGPU.cu:3842-3899).  save=1 copies field -> strip. */
static void edge_strips(const grid_t *g, real *vx, real *vz, real *up_x, real *up_z, real *dn_x, real *dn_z,
                        real *lf_x, real *lf_z, real *rt_x, real *rt_z, int it, int save) {
    const int pml = g->pml, N = g->nop, nx = g->nx, nz = g->nz, nxpml = g->nxpml, nzpml = g->nzpml;
#define MOVE(field, strip) \
    do {                   \
        if (save)          \
            (strip) = (field); \
        else               \
            (field) = (strip); \
    } while (0)
    for (int ix = pml; ix < nxpml - pml; ix++)
        for (int iz = pml - N; iz < pml + N; iz++) {
            size_t s = (size_t)it * nx * 2 * N + (size_t)(ix - pml) * 2 * N + (iz - (pml - N));
            MOVE(vx[IDX(ix, iz)], up_x[s]);
            MOVE(vz[IDX(ix, iz)], up_z[s]);
        }
    for (int ix = pml; ix < nxpml - pml; ix++)
        for (int iz = nzpml - pml - N; iz < nzpml - pml + N; iz++) {
            size_t s = (size_t)it * nx * 2 * N + (size_t)(ix - pml) * 2 * N + (iz - (nzpml - pml - N));
            MOVE(vx[IDX(ix, iz)], dn_x[s]);
            MOVE(vz[IDX(ix, iz)], dn_z[s]);
        }
    for (int ix = pml - N; ix < pml + N; ix++)
        for (int iz = pml; iz < nzpml - pml; iz++) {
            size_t s = (size_t)it * 2 * N * nz + (size_t)(ix - (pml - N)) * nz + (iz - pml);
            MOVE(vx[IDX(ix, iz)], lf_x[s]);
            MOVE(vz[IDX(ix, iz)], lf_z[s]);
        }
    for (int ix = nxpml - pml - N; ix < nxpml - pml + N; ix++)
        for (int iz = pml; iz < nzpml - pml; iz++) {
            size_t s = (size_t)it * 2 * N * nz + (size_t)(ix - (nxpml - pml - N)) * nz + (iz - pml);
            MOVE(vx[IDX(ix, iz)], rt_x[s]);
            MOVE(vz[IDX(ix, iz)], rt_z[s]);
        }
#undef MOVE
}

/* ------------------------------------------------------------------------
 * 1D quadratic-Wasserstein misfit of one trace (no reference counterpart;
 * the reference only declares OT/OT_power/OT_alltrace, FD2DGPU.cuh:21-25).
 *
 * Transform to positive weights, kind 1/3: p(u) = exp((u-max u)/sigma), kind 2:
 * p(u) = u^2 + 1e-3 sigma^2, with sigma = max|obs| of the trace, floored at
 * 1e-3 max|obs| of the gather (kind 1, 2), or of the whole gather (kind 3).  f = p(syn)/sum p(syn), g likewise for obs,
 * F, G their running sums (the CDF at the right end of sample k), and
 * T_k = G^-1(F_k) by linear interpolation inside the containing sample:
 *   T = dt * (m + (F_k - G_{m-1}) / g_m),  G_{m-1} <= F_k < G_m.
 * Misfit W = sum_k (t_k - T_k)^2 f_k with t_k = (k+1) dt.  The adjoint source
 * written to res is (1/2) dW/dsyn, the same scaling as the L2 residual
 * (misfit sum r^2, adjoint source r):
 *   A_j  = (t_j - T_j)^2 - 2 sum_{k>=j} (t_k - T_k) f_k dt / g_m(k)
 *   dW/dp_i = (A_i - sum_j f_j A_j) / sum p,   dW/dsyn_i = dW/dp_i * p'(syn_i).
 * All of it runs in double precision.
 * ---------------------------------------------------------------------- */
#define OT_SIGMA_FLOOR 1e-3 /* per-trace scale floor, relative to the gather's max |obs| */

static double ot_trace(int kind, int n, double dt, double sigma, const float *syn, const float *obs, double *res,
                       double *work) {
    double *f = work, *F = work + n, *g = work + 2 * n, *G = work + 3 * n, *A = work + 4 * n, *T = work + 5 * n;
    int *mk = (int *)(work + 6 * n);
    if (!(sigma > 0)) sigma = 1.0;
    /* the exponential weights are shifted by the trace maximum; the shift
     * cancels in f and g and keeps exp() in range */
    double smax = -HUGE_VAL, omax = -HUGE_VAL;
    for (int k = 0; k < n; k++) {
        if (syn[k] > smax) smax = syn[k];
        if (obs[k] > omax) omax = obs[k];
    }
    double sf = 0, sg = 0;
    for (int k = 0; k < n; k++) {
        double s = syn[k], o = obs[k];
        double pf = kind == 2 ? s * s + 1e-3 * sigma * sigma : exp((s - smax) / sigma);
        double pg = kind == 2 ? o * o + 1e-3 * sigma * sigma : exp((o - omax) / sigma);
        f[k] = pf;
        g[k] = pg;
        sf += pf;
        sg += pg;
    }
    double acc = 0, accg = 0;
    for (int k = 0; k < n; k++) {
        f[k] /= sf;
        g[k] /= sg;
        acc += f[k];
        accg += g[k];
        F[k] = acc;
        G[k] = accg;
    }
    double W = 0;
    for (int k = 0; k < n; k++) {
        double y = F[k];
        /* first m with G[m] > y (clamped to n-1) */
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (G[mid] > y)
                hi = mid;
            else
                lo = mid + 1;
        }
        int m = lo;
        double Gm1 = m > 0 ? G[m - 1] : 0.0;
        T[k] = dt * (m + (y - Gm1) / g[m]);
        mk[k] = m;
        double r = (k + 1) * dt - T[k];
        W += r * r * f[k];
    }
    double suffix = 0;
    for (int j = n - 1; j >= 0; j--) {
        double r = (j + 1) * dt - T[j];
        suffix += r * f[j] * dt / g[mk[j]];
        A[j] = r * r - 2.0 * suffix;
    }
    double fa = 0;
    for (int j = 0; j < n; j++) fa += f[j] * A[j];
    for (int i = 0; i < n; i++) {
        double dWdp = (A[i] - fa) / sf;
        double s = syn[i];
        double dp = kind == 2 ? 2.0 * s : exp((s - smax) / sigma) / sigma;
        res[i] = 0.5 * dWdp * dp;
    }
    return W;
}

/* trace-gather form of the OT entry points (FD2DGPU.cuh:23-25 argument
 * order: obs_x, obs_z, cal_x, cal_z, res_x, res_z, length, tracenum, misfit) */
void FN(ot_gather)(int kind, float dt, const float *obs_x, const float *obs_z, const float *cal_x,
                   const float *cal_z, double *res_x, double *res_z, int length, int tracenum, double *misfit) {
    double *work = (double *)malloc(sizeof(double) * 7 * (size_t)length + sizeof(int) * (size_t)length + 64);
    double gmax_x = 0, gmax_z = 0;
    for (size_t i = 0; i < (size_t)length * tracenum; i++) {
        if (fabs(obs_x[i]) > gmax_x) gmax_x = fabs(obs_x[i]);
        if (fabs(obs_z[i]) > gmax_z) gmax_z = fabs(obs_z[i]);
    }
    double W = 0;
    for (int tr = 0; tr < tracenum; tr++) {
        size_t o = (size_t)tr * length;
        double sx = gmax_x, sz = gmax_z;
        if (kind != 3) {
            /* the trace's own max |obs|, floored at a fraction of the gather's
             * so that a trace the wave has not reached (|obs| ~ 0) does not
             * blow the transform up */
            sx = 0;
            sz = 0;
            for (int k = 0; k < length; k++) {
                if (fabs(obs_x[o + k]) > sx) sx = fabs(obs_x[o + k]);
                if (fabs(obs_z[o + k]) > sz) sz = fabs(obs_z[o + k]);
            }
            if (sx < OT_SIGMA_FLOOR * gmax_x) sx = OT_SIGMA_FLOOR * gmax_x;
            if (sz < OT_SIGMA_FLOOR * gmax_z) sz = OT_SIGMA_FLOOR * gmax_z;
        }
        W += ot_trace(kind, length, dt, sz, cal_z + o, obs_z + o, res_z + o, work);
        W += ot_trace(kind, length, dt, sx, cal_x + o, obs_x + o, res_x + o, work);
    }
    free(work);
    *misfit += W;
}

/* ------------------------------------------------------------------------
 * One shot-gradient: IMAGE_SINGLESHOT (sfwi-stage1/FD2DGPU.cu:4321-4695,
 * sfwi-stage2/FD2DGPU.cu:3978-4570) with the caller's set-up
 * (sfwi-stage1/main.cpp:585-625).
 * ---------------------------------------------------------------------- */
int FN(image_singleshot)(const sfwi_oracle_shot *sp, const sfwi_oracle_io *io) {
    const sfwi_oracle_shot s = *sp;
    if (s.stage != 1 && s.stage != 2) return -1;
#ifdef _OPENMP
    if (s.nthreads > 0) omp_set_num_threads(s.nthreads);
#endif
    grid_t G0;
    grid_t *g = &G0;
    g->pml = s.pml;
    g->nop = s.nop;
    g->nx = s.nx;
    g->nz = s.allnz;
    g->nxpml = s.nx + 2 * s.pml;
    g->nzpml = s.allnz + 2 * s.pml;
    g->dx = s.dx;
    g->dz = s.dz;
    g->dt = s.dt;
    const int nt = s.nt, ntr = s.ntr, pml = s.pml;
    const size_t nD = (size_t)g->nxpml * g->nzpml, nrec = (size_t)ntr * nt;

    enum {
        VP, VS, RHO, LAM, MU, DX_, DZ_, DMP, DMS,
        VX, VZ, VXX, VXZ, VZX, VZZ, TXX, TZZ, TXZ, TXXX, TXXZ, TZZX, TZZZ, TXZX, TXZZ,
        BVX, BVZ, BVXX, BVXZ, BVZX, BVZZ, BTXX, BTZZ, BTXZ, BTXXX, BTXXZ, BTZZX, BTZZZ, BTXZX, BTXZZ,
        AVX, AVZ, AVXX, AVXZ, AVZX, AVZZ, ATXX, ATZZ, ATXZ, ATXXX, ATZZZ, ATXZX, ATXZZ,
        GXX, GZZ, GXZ, GZX, VPREV_X, VPREV_Z, NFIELD
    };
    real *mem = (real *)calloc(nD * NFIELD, sizeof(real));
    if (!mem) return -3;
#define F_(k) (mem + (size_t)(k) * nD)
    real *rec = (real *)calloc(nrec * 4, sizeof(real));
    const size_t nud = (size_t)2 * g->nop * g->nx * nt, nlr = (size_t)2 * g->nz * g->nop * nt;
    const int snap = s.snap_every > 0 && !s.forward_only;
    const int nsnap = snap ? (nt + s.snap_every - 1) / s.snap_every : 0;
    real *strips = s.forward_only || snap ? NULL : (real *)calloc(4 * nud + 4 * nlr, sizeof(real));
    real *snaps = snap ? (real *)malloc(sizeof(real) * 2 * nD * (size_t)nsnap) : NULL;
    if (!rec || (!s.forward_only && !snap && !strips) || (snap && !snaps)) {
        free(mem);
        free(rec);
        free(strips);
        free(snaps);
        return -3;
    }
    real *syn_z = rec, *syn_x = rec + nrec, *syn2_z = rec + 2 * nrec, *syn2_x = rec + 3 * nrec;

    /* bufferVpVsHtoD / buffer_image_extrapolation */
    const int ngx_min = s.delta_left + s.record_left_in_v;
    window_model(g, io->vp_all, s.allnz, ngx_min, F_(VP));
    window_model(g, io->vs_all, s.allnz, ngx_min, F_(VS));
    if (s.stage == 1) {
        window_model(g, io->rho_all, s.allnz, ngx_min, F_(RHO));
    } else {
        for (size_t i = 0; i < nD; i++) F_(RHO)[i] = 2000; /* sfwi-stage2/FD2DGPU.cu:1111 */
        if (io->dvp_all) window_model(g, io->dvp_all, s.allnz, ngx_min, F_(DMP));
        if (io->dvs_all) window_model(g, io->dvs_all, s.allnz, ngx_min, F_(DMS));
    }
    /* calculate_elastic_damp_C: damping and Lame parameters
     * (GPUcalculate_elastic_rho_C, FD2DGPU.cu:1116-1124) */
    damping(g, F_(VP), F_(DX_), F_(DZ_));
    for (size_t i = 0; i < nD; i++) {
        real r = F_(RHO)[i], p = F_(VP)[i], q = F_(VS)[i];
        F_(LAM)[i] = r * (p * p - 2 * q * q);
        F_(MU)[i] = r * q * q;
    }

    int *rix = (int *)malloc(sizeof(int) * 2 * (ntr > 0 ? ntr : 1));
    int *iix = rix + (ntr > 0 ? ntr : 1);
    for (int tr = 0; tr < ntr; tr++) {
        rix[tr] = receiver_ix(s.stage, pml, io->gc[tr], s.ngx_left, s.dx);
        iix[tr] = injection_ix(pml, io->gc[tr], s.ngx_left, s.dx);
    }
    const int isx = s.isx, isz = s.isz, igz = s.igz;
    const int born_lo = s.stage == 2 ? g->nop : pml;
    const int adj_dir = s.stage == 1 ? 1 : -1;

    real *up_x = strips, *up_z = strips ? strips + nud : NULL, *dn_x = strips ? strips + 2 * nud : NULL,
         *dn_z = strips ? strips + 3 * nud : NULL;
    real *lf_x = strips ? strips + 4 * nud : NULL, *lf_z = strips ? strips + 4 * nud + nlr : NULL,
         *rt_x = strips ? strips + 4 * nud + 2 * nlr : NULL, *rt_z = strips ? strips + 4 * nud + 3 * nlr : NULL;

    /* ---------------- forward ---------------- */
    for (int it = 0; it < nt; it++) {
        size_t si = IDX(isx, isz);
        if (s.src_kind == 0) {
            F_(TXX)[si] += io->sou[it]; /* GPUapplysource on txx and tzz, FD2DGPU.cu:2104-2114 */
            F_(TZZ)[si] += io->sou[it];
        }
        update_v(g, F_(TXX), F_(TZZ), F_(TXZ), F_(VX), F_(VXX), F_(VXZ), F_(VZ), F_(VZX), F_(VZZ), F_(RHO), F_(DX_),
                 F_(DZ_), 1);
        /* vertical force (no reference counterpart): like the reference's
         * stress source it goes into the total field only, here vz after the
         * velocity sweep, so the stress sweep, the records, the edge strips
         * and the snapshots of this step see it and the next velocity sweep
         * (which rebuilds vz from its split parts) does not */
        if (s.src_kind == 1) F_(VZ)[si] += io->sou[it];
        update_s(g, F_(TXX), F_(TZZ), F_(TXXX), F_(TXXZ), F_(TZZX), F_(TZZZ), F_(TXZ), F_(TXZX), F_(TXZZ), F_(VX),
                 F_(VZ), F_(LAM), F_(MU), F_(DX_), F_(DZ_), 1, NULL, NULL, NULL, NULL);
        if (s.stage == 2) { /* born_modeling(+1, 1), sfwi-stage2/FD2DGPU.cu:1818-1843 */
            update_v(g, F_(BTXX), F_(BTZZ), F_(BTXZ), F_(BVX), F_(BVXX), F_(BVXZ), F_(BVZ), F_(BVZX), F_(BVZZ),
                     F_(RHO), F_(DX_), F_(DZ_), 1);
            born_source(g, born_lo, F_(VX), F_(VZ), F_(BTXXX), F_(BTXXZ), F_(BTZZX), F_(BTZZZ), F_(BTXZX),
                        F_(BTXZZ), F_(DMP), F_(DMS), F_(RHO), F_(VP), F_(VS), 1);
            update_s(g, F_(BTXX), F_(BTZZ), F_(BTXXX), F_(BTXXZ), F_(BTZZX), F_(BTZZZ), F_(BTXZ), F_(BTXZX),
                     F_(BTXZZ), F_(BVX), F_(BVZ), F_(LAM), F_(MU), F_(DX_), F_(DZ_), 1, NULL, NULL, NULL, NULL);
            for (int tr = 0; tr < ntr; tr++) { /* record_scatter(it, true) */
                size_t c = IDX(rix[tr], igz);
                syn_z[(size_t)tr * nt + it] = F_(BVZ)[c];
                syn_x[(size_t)tr * nt + it] = F_(BVX)[c];
                syn2_z[(size_t)tr * nt + it] = F_(VZ)[c];
                syn2_x[(size_t)tr * nt + it] = F_(VX)[c];
            }
        } else {
            for (int tr = 0; tr < ntr; tr++) { /* record_background_wave(it) */
                size_t c = IDX(rix[tr], igz);
                syn_z[(size_t)tr * nt + it] = F_(VZ)[c];
                syn_x[(size_t)tr * nt + it] = F_(VX)[c];
            }
        }
        if (snap) {
            if (it % s.snap_every == 0) {
                memcpy(snaps + (size_t)(it / s.snap_every) * 2 * nD, F_(VX), nD * sizeof(real));
                memcpy(snaps + (size_t)(it / s.snap_every) * 2 * nD + nD, F_(VZ), nD * sizeof(real));
            }
        } else if (!s.forward_only) {
            edge_strips(g, F_(VX), F_(VZ), up_x, up_z, dn_x, dn_z, lf_x, lf_z, rt_x, rt_z, it, 1);
        }
    }
    for (size_t i = 0; i < nrec; i++) {
        if (io->syn_z) io->syn_z[i] = syn_z[i];
        if (io->syn_x) io->syn_x[i] = syn_x[i];
        if (s.stage == 2 && io->syn2_z) io->syn2_z[i] = syn2_z[i];
        if (s.stage == 2 && io->syn2_x) io->syn2_x[i] = syn2_x[i];
    }
    if (s.forward_only) {
        free(mem);
        free(rec);
        free(strips);
        free(snaps);
        free(rix);
        return 0;
    }

    /* ---------------- residual (adjoint source) and misfit ---------------- */
    real *res_z = syn_z, *res_x = syn_x; /* in place, as GPU_subtract does */
    if (s.misfit_kind == 0) {
        double misfit = 0;
        for (size_t i = 0; i < nrec; i++) {
            if (s.stage == 1) { /* GPU_subtract alpha=1, sfwi-stage1/FD2DGPU.cu:3181-3195 */
                res_z[i] = (real)1.0f * syn_z[i] - io->obs_z[i];
                res_x[i] = (real)1.0f * syn_x[i] - io->obs_x[i];
            } else { /* GPU_subtract then GPU_add, sfwi-stage2/FD2DGPU.cu:3119-3158 */
                res_z[i] = syn_z[i] - io->obs_z[i];
                res_x[i] = syn_x[i] - io->obs_x[i];
                res_z[i] = (real)1.0f * res_z[i] + syn2_z[i];
                res_x[i] = (real)1.0f * res_x[i] + syn2_x[i];
            }
            misfit += (res_z[i] * res_z[i] + res_x[i] * res_x[i]); /* FD2DGPU.cu:4586-4589 */
        }
        if (io->misfit) *io->misfit += misfit;
    } else {
        /* OT: the predicted record is syn (stage 1) or du+u0 (stage 2) */
        float *pz = (float *)malloc(sizeof(float) * nrec * 2);
        double *rz = (double *)malloc(sizeof(double) * nrec * 2);
        for (size_t i = 0; i < nrec; i++) {
            pz[i] = (float)(s.stage == 2 ? syn_z[i] + syn2_z[i] : syn_z[i]);
            pz[nrec + i] = (float)(s.stage == 2 ? syn_x[i] + syn2_x[i] : syn_x[i]);
        }
        double m = 0;
        FN(ot_gather)(s.misfit_kind, s.dt, io->obs_x, io->obs_z, pz + nrec, pz, rz + nrec, rz, nt, ntr, &m);
        for (size_t i = 0; i < nrec; i++) {
            res_z[i] = (real)rz[i];
            res_x[i] = (real)rz[nrec + i];
        }
        if (io->misfit) *io->misfit += m;
        free(pz);
        free(rz);
    }
    for (size_t i = 0; i < nrec; i++) {
        if (io->res_z) io->res_z[i] = res_z[i];
        if (io->res_x) io->res_x[i] = res_x[i];
    }

    /* ---------------- backward ---------------- */
    const int nx = g->nx, nz = g->nz;
    real *gpp = (real *)calloc((size_t)s.allnx * s.allnz * 4, sizeof(real));
    real *gps = gpp + (size_t)s.allnx * s.allnz, *gil = gps + (size_t)s.allnx * s.allnz,
         *grh = gil + (size_t)s.allnx * s.allnz;
    const int off = s.delta_left + s.record_left_in_v;
    for (int it = nt - 1; it >= 0; it--) {
        /* density kernel: the velocity step of the reconstruction itself,
         * taken before the edge strips are restored into the totals (the
         * restore is not part of the step: update_v rebuilds the totals from
         * the split parts) */
        if (io->grad_rho && !snap) {
            memcpy(F_(VPREV_X), F_(VX), nD * sizeof(real));
            memcpy(F_(VPREV_Z), F_(VZ), nD * sizeof(real));
        }
        real w = 1; /* imaging weight of this step */
        if (snap) {
            if (it % s.snap_every == 0) {
                const real *sv = snaps + (size_t)(it / s.snap_every) * 2 * nD;
                memcpy(F_(VX), sv, nD * sizeof(real));
                memcpy(F_(VZ), sv + nD, nD * sizeof(real));
                strains(g, F_(VX), F_(VZ), F_(GXX), F_(GZZ), F_(GXZ), F_(GZX));
                w = (real)s.snap_every;
            } else {
                w = 0;
            }
        } else {
            edge_strips(g, F_(VX), F_(VZ), up_x, up_z, dn_x, dn_z, lf_x, lf_z, rt_x, rt_z, it, 0);
            /* born_modeling(-1, 6): reconstruct sigma (with strains) then v */
            update_s(g, F_(TXX), F_(TZZ), F_(TXXX), F_(TXXZ), F_(TZZX), F_(TZZZ), F_(TXZ), F_(TXZX), F_(TXZZ), F_(VX),
                     F_(VZ), F_(LAM), F_(MU), F_(DX_), F_(DZ_), -1, F_(GXX), F_(GZZ), F_(GXZ), F_(GZX));
            update_v(g, F_(TXX), F_(TZZ), F_(TXZ), F_(VX), F_(VXX), F_(VXZ), F_(VZ), F_(VZX), F_(VZZ), F_(RHO),
                     F_(DX_), F_(DZ_), -1);
        }
        /* elastic_rotation_addS_bac: assign (stack=false), FD2DGPU.cu:3425-3441 */
        for (int tr = 0; tr < ntr; tr++) {
            if (iix[tr] < 0 || iix[tr] >= g->nxpml) continue; /* outside the grid: nothing to inject */
            size_t c = IDX(iix[tr], igz);
            F_(AVZ)[c] = res_z[(size_t)tr * nt + it];
            F_(AVX)[c] = res_x[(size_t)tr * nt + it];
        }
        /* born_modeling(adj_dir, 8) */
        back_s(g, F_(ATXX), F_(ATZZ), F_(ATXXX), F_(ATZZZ), F_(ATXZ), F_(ATXZX), F_(ATXZZ), F_(AVX), F_(AVZ),
               F_(DX_), F_(DZ_), adj_dir);
        back_v(g, F_(ATXX), F_(ATZZ), F_(ATXZ), F_(AVX), F_(AVXX), F_(AVXZ), F_(AVZ), F_(AVZX), F_(AVZZ), F_(LAM),
               F_(MU), F_(RHO), F_(DX_), F_(DZ_), adj_dir);
        /* image_gradient: doimage_gradient + doimage_illum, FD2DGPU.cu:3324-3382 */
        if (w != 0)
        for (int ix = 0; ix < nx; ix++)
            for (int iz = 0; iz < nz; iz++) {
                size_t c = IDX(ix + pml, iz + pml);
                size_t o = (size_t)(off + ix) * nz + iz;
                real lg = -((F_(GXX)[c] + F_(GZZ)[c]) * (F_(ATXX)[c] + F_(ATZZ)[c]));
                real mg = -2 * (F_(GXX)[c] * F_(ATXX)[c] + F_(GZZ)[c] * F_(ATZZ)[c]) -
                          (F_(GXZ)[c] + F_(GZX)[c]) * F_(ATXZ)[c];
                real cpp = 2 * F_(VP)[c] * F_(RHO)[c] * lg;
                real cps = -4 * F_(VS)[c] * F_(RHO)[c] * lg + 2 * F_(VS)[c] * F_(RHO)[c] * mg;
                gpp[o] += w * cpp;
                gps[o] += w * cps;
                gil[o] += w * (F_(VX)[c] * F_(VX)[c] + F_(VZ)[c] * F_(VZ)[c]);
                if (io->grad_rho && !snap) {
                    /* v_adj . dv/dt with the reconstructed step v(it) -> v(it-1) */
                    real dvx = (F_(VPREV_X)[c] - F_(VX)[c]) / g->dt, dvz = (F_(VPREV_Z)[c] - F_(VZ)[c]) / g->dt;
                    grh[o] += -(F_(AVX)[c] * dvx + F_(AVZ)[c] * dvz);
                }
            }
    }
    for (size_t i = 0; i < (size_t)s.allnx * s.allnz; i++) {
        if (io->grad_pp) io->grad_pp[i] += gpp[i];
        if (io->grad_ps) io->grad_ps[i] += gps[i];
        if (io->illum) io->illum[i] += gil[i];
        if (io->grad_rho) io->grad_rho[i] += grh[i];
    }
    free(gpp);
    free(mem);
    free(rec);
    free(strips);
    free(snaps);
    free(rix);
#undef F_
    return 0;
}
