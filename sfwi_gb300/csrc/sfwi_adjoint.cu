// sfwi_adjoint.cu — the exact discrete adjoint of the Born modelling operator.
//
// The stage-2 forward (sfwi-stage2/FD2DGPU.cu:1814-1843, born.cu:749-801) maps
// a model perturbation (dVp, dVs) linearly to the scattered records: each
// time step runs the scattered velocity sweep, records the scattered
// velocities, then adds the Born virtual source (dt * 2 rho vp dVp, 2 rho vs
// dVs times strains of the background velocity) to the split parts of the
// scattered stresses inside the stress sweep.  The reference's Hessian
// products (ELSRTM_CALCULATE_Hessian_vector*, sfwi-stage1/FD2DGPU.cu:
// 5236-5774, with add_born_source_adjoint_components, born.cu:886-958)
// approximate its transpose with the continuous adjoint equations.  The
// kernels here are the transpose of the forward sweeps this library runs
// (k_fwd_v, k_fwd_s: the same stencils, the same split-field PML update in
// damped cells and plain update elsewhere, the same update region), so
// <L m, d> = <m, L^T d> holds to rounding: reverse-mode differentiation of
// one time step, run backwards from the last step.
//
// Per reverse step `it` (forward step: V' = V-sweep(V, S); record V';
// S' = S-sweep(S, V', born(m, background V'))):
//   k_adj_stress    own-cell transpose of the stress sweep: the adjoint of
//                   S (and its x-parts), the fields G to be scattered into
//                   the adjoint of V', and the Born-source adjoint folded
//                   into per-cell accumulators of d(2 rho vp dVp) and
//                   d(2 rho vs dVs) with the background strains of step it
//   k_adj_velocity  adjoint of V': gathers of G (transposed stencils: the
//                   transpose of D+ is -D-), the records' data at the
//                   receiver cells, then the own-cell transpose of the
//                   velocity sweep: the adjoint of V and the fields H
//   k_adj_gather    the adjoint of S gathers H
// The transposed stencil gathers read G/H of the cells up to 4 away, which
// are zero outside the update region [4, n-4), so they stay within a shot.
#include "sfwi_launch.h"

namespace sfwi {

namespace {

constexpr float AK1 = (float)(1225.0 / 1024.0);
constexpr float AK2 = (float)(-245.0 / 3072.0);
constexpr float AK3 = (float)(49.0 / 5120.0);
constexpr float AK4 = (float)(-5.0 / 7168.0);
__device__ __forceinline__ float kk(int k) { return k == 1 ? AK1 : k == 2 ? AK2 : k == 3 ? AK3 : AK4; }

// staggered first derivatives of a packed array at index i; `s` is the
// stride of the derivative's axis (row pitch for x, 1 for z)
__device__ __forceinline__ float dp(const float *f, size_t i, long long s) {  // sum K_k (f[+k] - f[-k+1])
    float a = 0.f;
#pragma unroll
    for (int k = 1; k <= NOP; k++) a += kk(k) * (f[i + k * s] - f[i - (k - 1) * s]);
    return a;
}
__device__ __forceinline__ float dm(const float *f, size_t i, long long s) {  // sum K_k (f[+k-1] - f[-k])
    float a = 0.f;
#pragma unroll
    for (int k = 1; k <= NOP; k++) a += kk(k) * (f[i + (k - 1) * s] - f[i - k * s]);
    return a;
}

struct CellInfo {
    bool live, damped, born;
    int lx, lz, igz;
    size_t i;   // packed index in [X][P]
    int row;
};

__device__ __forceinline__ CellInfo cell_at(const AdjArgs &a, long long idx) {
    CellInfo c;
    c.row = (int)(idx / a.P);
    c.lz = (int)(idx - (long long)c.row * a.P);
    c.i = (size_t)idx;
    const ShotGeo g = a.geo[a.rowshot[c.row]];
    c.lx = c.row - g.row0;
    c.igz = g.igz;
    const int nx = g.nxpml, nz = g.nzpml, pml = a.pml;
    c.live = c.lx >= NOP && c.lx < nx - NOP && c.lz >= NOP && c.lz < nz - NOP;
    c.damped = c.live && (c.lx < pml || c.lx > nx - pml || c.lz < pml || c.lz > nz - pml);
    c.born = c.lx >= a.born_lo && c.lx < nx - a.born_lo && c.lz >= a.born_lo && c.lz < nz - a.born_lo;
    return c;
}

// the PML factors of the forward update: 1 - dt d / 2 and 1 / (1 + dt d / 2)
struct Fac {
    float d1, r2, d3, r4;
};
__device__ __forceinline__ Fac damp_factors(const AdjArgs &a, size_t i) {
    const float tx = a.dt * a.dampx[i], tz = a.dt * a.dampz[i];
    return Fac{fmaf(tx, -0.5f, 1.f), __frcp_rn(fmaf(tx, 0.5f, 1.f)), fmaf(tz, -0.5f, 1.f),
               __frcp_rn(fmaf(tz, 0.5f, 1.f))};
}

__global__ void k_adj_stress(AdjArgs a, int it) {
    const long long n = (long long)a.X * a.P;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const CellInfo c = cell_at(a, idx);
        if (!c.live) continue;
        const size_t i = c.i;
        const float Axx = a.atxx[i], Azz = a.atzz[i], Axz = a.atxz[i];
        const float l = a.lam[i], u = a.mu[i], l2m = l + 2.f * u;
        float gb[6], gax, gbz, gcz, gdx;
        if (c.damped) {
            const Fac f = damp_factors(a, i);
            const float Bxx = a.amxx[i] + Axx, Bzz = a.amzz[i] + Azz, Bxz = a.amxz[i] + Axz;
            a.amxx[i] = f.r2 * f.d1 * Bxx - f.r4 * f.d3 * Axx;
            a.amzz[i] = f.r2 * f.d1 * Bzz - f.r4 * f.d3 * Azz;
            a.amxz[i] = f.r2 * f.d1 * Bxz - f.r4 * f.d3 * Axz;
            a.atxx[i] = f.r4 * f.d3 * Axx;
            a.atzz[i] = f.r4 * f.d3 * Azz;
            a.atxz[i] = f.r4 * f.d3 * Axz;
            gb[0] = f.r2 * f.d1 * Bxx;
            gb[1] = f.r4 * f.d3 * Axx;
            gb[2] = f.r2 * f.d1 * Bzz;
            gb[3] = f.r4 * f.d3 * Azz;
            gb[4] = f.r2 * f.d1 * Bxz;
            gb[5] = f.r4 * f.d3 * Axz;
            gax = f.r2 * (l2m * Bxx + l * Bzz);
            gbz = f.r4 * (l * Axx + l2m * Azz);
            gdx = f.r2 * u * Bxz;
            gcz = f.r4 * u * Axz;
        } else {
            gb[0] = gb[1] = Axx;
            gb[2] = gb[3] = Azz;
            gb[4] = gb[5] = Axz;
            gax = l2m * Axx + l * Azz;
            gbz = l * Axx + l2m * Azz;
            gdx = gcz = u * Axz;
        }
        a.gax[i] = gax;
        a.gbz[i] = gbz;
        a.gcz[i] = gcz;
        a.gdx[i] = gdx;
        if (c.born) {
            // strains of the background velocity after the velocity sweep of
            // step it (the Born source's: Dx- vx, Dz- vz, Dx+ vz, Dz+ vx)
            const size_t so = (size_t)c.row * a.PS + c.lz;
            const float *svx = a.snap + (size_t)(2 * it) * a.X * a.PS, *svz = svx + (size_t)a.X * a.PS;
            const float AX = dm(svx, so, a.PS) * a.idx, BZ = dm(svz, so, 1) * a.idz;
            const float DX = dp(svz, so, a.PS) * a.idx, CZ = dp(svx, so, 1) * a.idz;
            const double dt = a.dt;
            const double gmix = dt * ((double)BZ * gb[1] + (double)AX * gb[2]);
            a.dbp[i] += dt * ((double)AX * gb[0] + (double)BZ * gb[3]) + gmix;
            a.dbs[i] += dt * ((double)DX * gb[4] + (double)CZ * gb[5]) - 2.0 * gmix;
        }
    }
}

__global__ void k_adj_velocity(AdjArgs a, int it) {
    const long long n = (long long)a.X * a.P;
    const long long P = a.P;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const CellInfo c = cell_at(a, idx);
        if (!c.live) continue;
        const size_t i = c.i;
        // the stress sweep read V' through tx Dx- vx, tz Dz+ vx, tz Dz- vz, tx Dx+ vz
        float AX = a.avx[i] - a.dtdx * dp(a.gax, i, P) - a.dtdz * dm(a.gcz, i, 1);
        float AZ = a.avz[i] - a.dtdz * dp(a.gbz, i, 1) - a.dtdx * dm(a.gdx, i, P);
        // the records of step it read V' at the receiver cells (every trace
        // recorded there, in trace order)
        if (c.lz == c.igz)
            for (int k = a.rstart[c.row]; k < a.rstart[c.row + 1]; k++) {
                const size_t o = (size_t)a.rtr[k] * a.nt + it;
                AZ += a.dz[o];
                AX += a.dx[o];
            }
        const float ib = a.ib[i], cx = ib * a.dtdx, cz = ib * a.dtdz;
        if (c.damped) {
            const Fac f = damp_factors(a, i);
            const float Bx = a.amx[i] + AX, Bz = a.amz[i] + AZ;
            a.amx[i] = f.r2 * f.d1 * Bx - f.r4 * f.d3 * AX;
            a.amz[i] = f.r2 * f.d1 * Bz - f.r4 * f.d3 * AZ;
            a.avx[i] = f.r4 * f.d3 * AX;
            a.avz[i] = f.r4 * f.d3 * AZ;
            a.hax[i] = f.r2 * cx * Bx;
            a.hbz[i] = f.r4 * cz * AX;
            a.hdx[i] = f.r2 * cx * Bz;
            a.hcz[i] = f.r4 * cz * AZ;
        } else {
            a.avx[i] = AX;
            a.avz[i] = AZ;
            a.hax[i] = cx * AX;
            a.hbz[i] = cz * AX;
            a.hdx[i] = cx * AZ;
            a.hcz[i] = cz * AZ;
        }
    }
}

__global__ void k_adj_gather(AdjArgs a) {
    const long long n = (long long)a.X * a.P;
    const long long P = a.P;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const CellInfo c = cell_at(a, idx);
        if (!c.live) continue;
        const size_t i = c.i;
        // the velocity sweep read S through Dx+ txx, Dz- txz, Dx- txz, Dz+ tzz
        a.atxx[i] -= dm(a.hax, i, P);
        a.atxz[i] -= dp(a.hbz, i, 1) + dp(a.hdx, i, P);
        a.atzz[i] -= dm(a.hcz, i, 1);
    }
}

int grid_blocks(long long n) {
    long long b = (n + 255) / 256;
    return (int)(b < 8192 ? (b > 0 ? b : 1) : 8192);
}

}  // namespace

void launch_adjoint_step(const AdjArgs &a, int it, cudaStream_t st) {
    const int b = grid_blocks((long long)a.X * a.P);
    k_adj_stress<<<b, 256, 0, st>>>(a, it);
    k_adj_velocity<<<b, 256, 0, st>>>(a, it);
    k_adj_gather<<<b, 256, 0, st>>>(a);
}

// L^T d on the global model: each window cell's accumulated d(2 rho vp dVp),
// d(2 rho vs dVs) times 2 rho vp, 2 rho vs goes to the model cell it was cut
// from (k_setup cuts the window with the PML cells taking the nearest edge
// value, so an edge model cell collects the PML cells beyond it), shots in
// order, FP64.
__global__ void k_born_image(ImageArgs a) {
    const long long n = (long long)a.allnx * a.allnz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int gx = (int)(i / a.allnz), gz = (int)(i - (long long)gx * a.allnz);
        double sp = a.img_vp[i], ss = a.img_vs[i];
        for (int s = 0; s < a.nshots; s++) {
            const ShotGeo g = a.geo[s];
            if (gx < g.win0 || gx >= g.win0 + g.nx) continue;
            const int cx = gx - g.win0, nzm = g.nzpml - 2 * a.pml;
            if (gz >= nzm) continue;
            const int x0 = cx == 0 ? 0 : a.pml + cx, x1 = cx == g.nx - 1 ? g.nxpml - 1 : a.pml + cx;
            const int z0 = gz == 0 ? 0 : a.pml + gz, z1 = gz == nzm - 1 ? g.nzpml - 1 : a.pml + gz;
            for (int lx = x0; lx <= x1; lx++)
                for (int lz = z0; lz <= z1; lz++) {
                    const size_t o = (size_t)(g.row0 + lx) * a.P + lz;
                    const double rho = a.rho[o];
                    sp += 2.0 * (rho * a.vp[o]) * a.dbp[o];
                    ss += 2.0 * (rho * a.vs[o]) * a.dbs[o];
                }
        }
        a.img_vp[i] = sp;
        a.img_vs[i] = ss;
    }
}

void launch_born_image(const ImageArgs &a, cudaStream_t st) {
    k_born_image<<<grid_blocks((long long)a.allnx * a.allnz), 256, 0, st>>>(a);
}

}  // namespace sfwi
