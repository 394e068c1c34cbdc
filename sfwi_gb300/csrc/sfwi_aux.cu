// sfwi_aux.cu — per-batch set-up, record transposes, misfits and the final
// gradient reduction.
#include <cfloat>

#include "sfwi_launch.h"

namespace sfwi {

// Window cut with PML edge replication (copyvelocityHtoD + copypmlVz +
// copypmlVx, sfwi-stage1/FD2DGPU.cu:112-123, 233-249: the two edge passes give
// every PML cell the value of the nearest interior cell, corners included),
// PML profiles (dampX/dampZ, FD2DGPU.cu:443-493, rr = 1e-3), Lame parameters
// (GPUcalculate_elastic_rho_C, FD2DGPU.cu:1116-1124; stage 2 forces rho=2000,
// sfwi-stage2/FD2DGPU.cu:1111) and the Born coefficients 2 rho vp dvp,
// 2 rho vs dvs (zero outside [born_lo, n-born_lo)).
__global__ void k_setup(SetupArgs a) {
    const int s = blockIdx.y;
    const ShotGeo g = a.geo[s];
    const int nzpml = g.nzpml;
    // the shot's model: a slot of the uploaded model arrays, or (several
    // models in one batch) its own grid in the concatenated model arrays
    const size_t mbase = a.aux ? (size_t)a.aux[s].moff : 0;
    const int allnz = a.aux ? a.aux[s].allnz : a.allnz;
    const long long n = (long long)g.nxpml * a.P;
    const float l10 = log10f(1 / 0.001f);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int lx = (int)(i / a.P), lz = (int)(i - (long long)lx * a.P);
        const size_t o = (size_t)(g.row0 + lx) * a.P + lz;
        float vp = 0.f, vs = 0.f, rho = 0.f, dmp = 0.f, dms = 0.f, dx = 0.f, dz = 0.f;
        if (lz < nzpml) {
            const int cx = min(max(lx, a.pml), g.nxpml - a.pml - 1) - a.pml;
            const int cz = min(max(lz, a.pml), nzpml - a.pml - 1) - a.pml;
            const size_t go = mbase + (size_t)(g.win0 + cx) * allnz + cz;
            const size_t gv = go + (size_t)g.model * a.vslot, gm = go + (size_t)g.model * a.mslot;
            vp = a.vp_all[gv];
            vs = a.vs_all[gv];
            rho = a.stage == 2 ? 2000.f : a.rho_all[go];
            if (a.dvp_all) dmp = a.dvp_all[gm];
            if (a.dvs_all) dms = a.dvs_all[gm];
            const int pml = a.pml;
            if (lx < pml) dx = (float)(l10 * (5.0 * vp / (2.0 * pml)) * powf((float)(1.0 * (pml - lx) / pml), 4.0f));
            if (lx > g.nxpml - pml)
                dx = (float)(l10 * (5.0 * vp / (2.0 * pml)) * powf((float)(1.0 * (lx - (g.nxpml - pml)) / pml), 4.0f));
            if (lz < pml) dz = (float)(l10 * (5.0 * vp / (2.0 * pml)) * powf((float)(1.0 * (pml - lz) / pml), 4.0f));
            if (lz > nzpml - pml)
                dz = (float)(l10 * (5.0 * vp / (2.0 * pml)) * powf((float)(1.0 * (lz - (nzpml - pml)) / pml), 4.0f));
        }
        a.vp[o] = vp;
        a.vs[o] = vs;
        a.rho[o] = rho;
        a.dampx[o] = dx;
        a.dampz[o] = dz;
        a.lam[o] = rho * (vp * vp - 2 * vs * vs);
        a.mu[o] = rho * vs * vs;
        a.ib[o] = rho != 0.f ? 1.0f / rho : 0.f;
        const bool born = lx >= a.born_lo && lx < g.nxpml - a.born_lo && lz >= a.born_lo && lz < nzpml - a.born_lo;
        a.bp[o] = born ? 2 * (rho * vp) * dmp : 0.f;
        a.bs[o] = born ? 2 * (rho * vs) * dms : 0.f;
    }
}

void launch_setup(const SetupArgs &a, int nshots, int max_nxpml, cudaStream_t st) {
    const long long n = (long long)max_nxpml * a.P;
    int bx = (int)((n + 255) / 256);
    if (bx > 1024) bx = 1024;
    k_setup<<<dim3(bx, nshots), 256, 0, st>>>(a);
}

// Receiver-row records [nt][nrc][X] -> trace-major records [nrc][ntr][nt]:
// trace tr reads packed row trow[tr] (-1: a cell outside the update region,
// which the reference records as zero).  A trace of a shot that runs fewer
// steps than the batch (tlen) gets zeros after its last step.  32 traces x 32
// steps per block, transposed through shared memory so both sides are
// coalesced.
__global__ void k_record_gather(const float *__restrict__ rrow, const int *__restrict__ trow,
                                const int *__restrict__ tlen, int nt, int nrc, int X, int ntr, float *__restrict__ out,
                                size_t cstride) {
    __shared__ float tile[32][33];
    const int c = blockIdx.z, r0 = blockIdx.x * 32, t0 = blockIdx.y * 32;
    const int tr = r0 + threadIdx.x;
    const int row = tr < ntr ? trow[tr] : -1;
    const int len = tr < ntr && tlen ? tlen[tr] : nt;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int t = t0 + k;
        tile[k][threadIdx.x] = (row >= 0 && t < len) ? rrow[((size_t)t * nrc + c) * X + row] : 0.f;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = r0 + k, t = t0 + threadIdx.x;
        if (r < ntr && t < nt) out[c * cstride + (size_t)r * nt + t] = tile[threadIdx.x][k];
    }
}

void launch_record_gather(const float *rrow, const int *trow, const int *tlen, int nt, int nrc, int X, int ntr,
                          float *out, size_t cstride, cudaStream_t st) {
    dim3 grid((ntr + 31) / 32, (nt + 31) / 32, nrc), block(32, 8);
    k_record_gather<<<grid, block, 0, st>>>(rrow, trow, tlen, nt, nrc, X, ntr, out, cstride);
}

// Residual source per packed row: rs[row][2 it + 0|1] = res_z|res_x of the
// trace rtr[row] at step it, or the all-ones pattern where no trace injects
// (and in the padding past 2 nt).  One block per row.
__global__ void k_recv_source(const float *__restrict__ res_z, const float *__restrict__ res_x,
                              const int *__restrict__ rtr, int nt, int rsp, float *__restrict__ rs) {
    const int row = blockIdx.x;
    const int tr = rtr[row];
    float *o = rs + (size_t)row * rsp;
    for (int i = threadIdx.x; i < rsp; i += blockDim.x) {
        const int t = i >> 1;
        float v = __uint_as_float(0xFFFFFFFFu);
        if (tr >= 0 && t < nt) v = (i & 1) ? res_x[(size_t)tr * nt + t] : res_z[(size_t)tr * nt + t];
        o[i] = v;
    }
}

void launch_recv_source(const float *res_z, const float *res_x, const int *rtr, int nt, int X, int rsp, float *rs,
                        cudaStream_t st) {
    if (X > 0) k_recv_source<<<X, 256, 0, st>>>(res_z, res_x, rtr, nt, rsp, rs);
}

__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
    __syncthreads();
    return t;  // valid in thread 0
}

// L2 residual and misfit per trace.  stage 1: r = 1*syn - obs
// (GPU_subtract, sfwi-stage1/FD2DGPU.cu:3181-3195); stage 2: r = (syn-obs),
// then r = 1*r + syn2 (GPU_subtract + GPU_add, sfwi-stage2/FD2DGPU.cu:3119-3158).
// misfit of the trace = sum (rz*rz + rx*rx), each term in float as the host
// loop of IMAGE_SINGLESHOT forms it (FD2DGPU.cu:4586-4589), summed in double.
__global__ void k_residual_l2(int stage, int nt, const float *syn_z, const float *syn_x, const float *syn2_z,
                              const float *syn2_x, const float *obs_z, const float *obs_x, float *res_z, float *res_x,
                              double *trace_misfit) {
    __shared__ double red[32];
    const size_t o = (size_t)blockIdx.x * nt;
    double acc = 0.0;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        float rz, rx;
        if (stage == 2) {
            rz = syn_z[o + t] - obs_z[o + t];
            rx = syn_x[o + t] - obs_x[o + t];
            rz = 1.0f * rz + syn2_z[o + t];
            rx = 1.0f * rx + syn2_x[o + t];
        } else {
            rz = 1.0f * syn_z[o + t] - obs_z[o + t];
            rx = 1.0f * syn_x[o + t] - obs_x[o + t];
        }
        res_z[o + t] = rz;
        res_x[o + t] = rx;
        acc += (double)__fadd_rn(__fmul_rn(rz, rz), __fmul_rn(rx, rx));
    }
    const double s = block_sum(acc, red);
    if (threadIdx.x == 0) trace_misfit[blockIdx.x] = s;
}

void launch_residual_l2(int stage, int nt, int ntr_tot, const float *syn_z, const float *syn_x, const float *syn2_z,
                        const float *syn2_x, const float *obs_z, const float *obs_x, float *res_z, float *res_x,
                        double *trace_misfit, cudaStream_t st) {
    k_residual_l2<<<ntr_tot, 256, 0, st>>>(stage, nt, syn_z, syn_x, syn2_z, syn2_x, obs_z, obs_x, res_z, res_x,
                                           trace_misfit);
}

// Final reduction of the per-shot imaging accumulators into the global
// gradients, in FP64 and in shot order (deterministic).  The chain rule of
// doimage_gradient (FD2DGPU.cu:3372-3373) is applied here once:
//   g_vp += 2 vp rho G_lambda,  g_vs += -4 vs rho G_lambda + 2 vs rho G_mu
// with G_* the time sums of the lambda and mu kernels.  When requested the
// density kernel G_rho = -sum_t v_adj . dv/dt is reduced the same way, as is.

__global__ void k_finalize(FinalArgs a) {
    const long long n = (long long)a.allnx * a.allnz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int gx = (int)(i / a.allnz), gz = (int)(i - (long long)gx * a.allnz);
        // running sums start from the accumulated totals and add one rounded
        // term per shot (no fused multiply-add into the sum), so a batch of
        // shots gives bit-for-bit the totals of the same shots run one by one
        double pp = a.gpp[i], ps = a.gps[i], il = a.gil[i], rh = a.grho ? a.grh[i] : 0.0;
        bool any = false;
        for (int s = 0; s < a.nshots; s++) {
            const ShotGeo g = a.geo[s];
            if (gx < g.win0 || gx >= g.win0 + g.nx) continue;
            const size_t o = (size_t)(g.row0 + a.pml + gx - g.win0) * a.P + a.pml + gz;
            const double vp = a.vp[o], vs = a.vs[o], rho = a.rho[o];
            const double gl = a.glam[o], gm = a.gmu[o];
            const double tpp = __dmul_rn(__dmul_rn(__dmul_rn(2.0, vp), rho), gl);
            const double tps = __dadd_rn(__dmul_rn(__dmul_rn(__dmul_rn(-4.0, vs), rho), gl),
                                         __dmul_rn(__dmul_rn(__dmul_rn(2.0, vs), rho), gm));
            pp = __dadd_rn(pp, tpp);
            ps = __dadd_rn(ps, tps);
            il = __dadd_rn(il, (double)a.illum[o]);
            if (a.grho) rh = __dadd_rn(rh, (double)a.grho[o]);
            any = true;
        }
        if (any) {
            a.gpp[i] = pp;
            a.gps[i] = ps;
            a.gil[i] = il;
            if (a.grho) a.grh[i] = rh;
        }
    }
}

__global__ void k_trial_models(const float *__restrict__ base, const float *__restrict__ g,
                               const float *__restrict__ steps, int nslot, size_t n, float *__restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float b = base[i], gi = g[i];
        for (int k = 0; k < nslot; k++) out[(size_t)k * n + i] = __fsub_rn(b, __fmul_rn(steps[k], gi));
    }
}

void launch_trial_models(const float *base, const float *g, const float *steps, int nslot, size_t n, float *out,
                         cudaStream_t st) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    k_trial_models<<<blocks, 256, 0, st>>>(base, g, steps, nslot, n, out);
}

// the sums of CALCULATE_ALPHA (sfwi-stage2/FD2DGPU.cu:4705-4710): per sample
// (a_z b_z + a_x b_x) and (a_z a_z + a_x a_x) in float, summed in double
__global__ void k_trace_dots(const float *az, const float *ax, const float *bz, const float *bx, int nt, double *ab,
                             double *aa) {
    __shared__ double red[32];
    const size_t o = (size_t)blockIdx.x * nt;
    double sab = 0.0, saa = 0.0;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        const float z = az[o + t], x = ax[o + t];
        sab += (double)__fadd_rn(__fmul_rn(z, bz[o + t]), __fmul_rn(x, bx[o + t]));
        saa += (double)__fadd_rn(__fmul_rn(z, z), __fmul_rn(x, x));
    }
    const double tab = block_sum(sab, red);
    const double taa = block_sum(saa, red);
    if (threadIdx.x == 0) {
        ab[blockIdx.x] = tab;
        aa[blockIdx.x] = taa;
    }
}

void launch_trace_dots(const float *az, const float *ax, const float *bz, const float *bx, int nt, int ntr,
                       double *ab, double *aa, cudaStream_t st) {
    if (ntr > 0) k_trace_dots<<<ntr, 256, 0, st>>>(az, ax, bz, bx, nt, ab, aa);
}

void launch_finalize(const FinalArgs &a, cudaStream_t st) {
    const long long n = (long long)a.allnx * a.allnz;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    k_finalize<<<blocks, 256, 0, st>>>(a);
}

}  // namespace sfwi
