// sfwi_kernels.cu — the time-step kernels of the shot-gradient path.
//
// One launch advances every shot of a batch by one sweep.  The work is cut
// into TX x TZ tiles of one shot; this file is compiled once per tile shape
// (SFWI_TILE_X, SFWI_TILE_Z, SFWI_CTAS, SFWI_STAGES, SFWI_CPT) into its own
// namespace, and the engine picks a shape per batch.  Each kernel is
// persistent: CTAS_PER_SM CTAs per SM walk the tile list (dynamic draws from
// a per-launch counter), and an NSTAGE-stage TMA pipeline (cp.async.bulk.tensor
// into shared memory, completion on an mbarrier) loads the next tiles while
// one is computed.  Per tile the pipeline stages
//   - the fields read by the stencils as (TX+8) x (TZ+8) boxes (4-cell halo;
//     cells outside the packed arrays arrive as zeros), and
//   - the cell's own state and coefficients as TX x TZ core tiles,
// and each compute thread updates CPT consecutive cells (float4 or float2
// accesses, FP32x2 arithmetic) and writes them with one vector store.  A
// single 3-D tensor map [array][row][column] over the packed grid addresses
// every array (sfwi_common.cuh).
//
//   k_fwd_v   forward velocity sweep  (update_vx_vz, sfwi-stage1/born.cu:355-394)
//             of the background and, for the Born forward, the scattered field
//   k_fwd_s   forward stress sweep (update_txx_tzz_txz, born.cu:399-440), the Born
//             virtual source (add_born_source_components, sfwi-stage2/born.cu:749-801)
//             and the scattered stress sweep; receiver capture
//             (GPUrecord_scatterwavefield, FD2DGPU.cu:3158-3166) and edge-strip save
//             (record_edge_wavefield, FD2DGPU.cu:3842-3869)
//   k_bwd_s   reconstruction stress sweep with strains (update_txx_tzz_txz_grad,
//             born.cu:451-499), adjoint stress sweep
//             (GPUcalculate_elastic_txx_tzz_txz_back, born.cu:565-603) and the
//             zero-lag imaging condition (doimage_gradient, FD2DGPU.cu:3350-3382)
//   k_bwd_v   reconstruction velocity sweep (update_vx_vz, direction -1),
//             illumination (doimage_illum, FD2DGPU.cu:3324-3331) and adjoint
//             velocity sweep (GPUcalculate_elastic_vx_vz_back, born.cu:504-562)
//
// State representation.  In the reference every field carries two PML split
// parts over the whole grid and the total is their sum.  Here the total is the
// state everywhere and only cells of the PML frame (where dampx or dampz is
// nonzero) also keep the x-part; the z-part is total minus x-part.  Away from
// the frame the split update reduces to total += dir*coef*(Dx + Dz).
//
// Which update a cell takes depends on the cell alone (split where damped,
// plain elsewhere), never on the tile that holds it, and this file builds
// with -fmad=false with every fused multiply-add written as an intrinsic, so
// no product is fused in one tile shape and not in another: every tile shape
// and tile-grid origin gives the same bits.
//
// Three writes of the reference touch only the total field, never the split
// parts, so the next split update discards them: the source added to txx/tzz
// (GPUapplysource, FD2DGPU.cu:2104-2114), the residual assigned into the
// adjoint velocity (GPUapplysource_backward_from_record, FD2DGPU.cu:3425-3441)
// and the edge strips restored into vx/vz (load_edge_wavefield,
// FD2DGPU.cu:3873-3899).  Each is seen by exactly one stencil sweep, so here
// each is applied to the staged shared-memory box of that sweep only and the
// stored state is left untouched — the same arithmetic with no extra kernel.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "sfwi_launch.h"

#ifndef SFWI_VARIANT_NS
#define SFWI_VARIANT_NS v16x32
#define SFWI_VARIANT_FN tile_variant_16x32
#endif

namespace sfwi {
namespace SFWI_VARIANT_NS {

// 8th-order staggered first-derivative weights, sfwi-stage1/FD2DGPU.cuh:16
constexpr float K1 = (float)(1225.0 / 1024.0);
constexpr float K2 = (float)(-245.0 / 3072.0);
constexpr float K3 = (float)(49.0 / 5120.0);
constexpr float K4 = (float)(-5.0 / 7168.0);

#ifndef SFWI_STAGES
#define SFWI_STAGES 2
#endif
// shared-memory pipeline stages per CTA; with one stage the consumers'
// early release (all inputs in registers before the arithmetic) still lets
// the next tile's loads overlap this tile's arithmetic
constexpr int NSTAGE = SFWI_STAGES;
constexpr size_t SMEM_ALIGN_SLACK = 1024;
// dynamic shared memory of a kernel with nst stages of `stage` floats
constexpr size_t stage_bytes(int stage, int nst) { return (size_t)nst * stage * sizeof(float) + SMEM_ALIGN_SLACK; }
// CTAS_PER_SM CTAs of that kernel fit the SM's 228 KB of shared memory (227
// KB at most per CTA, 1 KB of it reserved per resident CTA; `extra` bytes of
// static shared memory per CTA)
constexpr bool fits_stages(int stage, int nst, size_t extra) {
    return stage_bytes(stage, nst) + extra <= 227 * 1024 &&
           CTAS_PER_SM * (stage_bytes(stage, nst) + extra + 1024) <= 228 * 1024;
}
// the most stages from NSTAGE up to `most` that still fit: kernels with
// small stages keep more tiles in flight
constexpr int deep_stages(int stage, int most, size_t extra) {
    int n = NSTAGE;
    for (int k = NSTAGE + 1; k <= most; k++)
        if (fits_stages(stage, k, extra)) n = k;
    return n;
}
constexpr int CORE = TX * TZ;  // floats of a core tile
constexpr uint32_t BOX_BYTES = BOX * 4u, CORE_BYTES = CORE * 4u;

// ----------------------------------------------------------------------------
// TMA / mbarrier primitives
// ----------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Programmatic dependent launch: the step kernels are launched so that the
// next one may start while this one drains.  griddep_wait blocks until the
// previous kernel of the stream has completed and its writes are visible
// (at once when there is no such kernel); every read of data another kernel
// wrote, and every write, comes after it.  griddep_launch lets the next
// kernel's CTAs be scheduled onto SMs this kernel's CTAs leave.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// barrier 1 over the NTHREADS consumer threads (the producer warp is not in it)
__device__ __forceinline__ void consumer_sync() { asm volatile("bar.sync 1, %0;" ::"n"(NTHREADS) : "memory"); }
__device__ __forceinline__ bool consumer_any(bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(NTHREADS)
        : "memory");
    return r != 0;
}
// bounded wait: false when the phase did not complete within `limit` tries
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// 3-D tiled bulk tensor load global -> shared, completion counted on `bar`
__device__ __forceinline__ void tma_load(float *dst, const CUtensorMap *map, int col, int row, int arr,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(col), "r"(row), "r"(arr), "r"(smem_u32(bar))
        : "memory");
}

// 2-D tiled bulk tensor load global -> shared (x = innermost coordinate)
__device__ __forceinline__ void tma_load_2d(float *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// ----------------------------------------------------------------------------
// stencils on staged boxes (row pitch BZ)
// ----------------------------------------------------------------------------
struct VC {
    float v[CPT];
};

// this thread's CPT consecutive cells of a staged row or core tile (one
// float4 or float2 shared-memory access) and of a global array (one vector
// store); `p` is 4*CPT-byte aligned
__device__ __forceinline__ void ldc(const float *p, float o[CPT]) {
    if constexpr (CPT == 4) {
        const float4 a = *reinterpret_cast<const float4 *>(p);
        o[0] = a.x, o[1] = a.y, o[2] = a.z, o[3] = a.w;
    } else {
        const float2 a = *reinterpret_cast<const float2 *>(p);
        o[0] = a.x, o[1] = a.y;
    }
}
__device__ __forceinline__ void stc(float *p, const float o[CPT]) {
    if constexpr (CPT == 4)
        *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
    else
        *reinterpret_cast<float2 *>(p) = make_float2(o[0], o[1]);
}

// a += k*(p - m) on this thread's cells as packed FP32x2 pairs; p - m is
// formed as fma(m, -1, p), which rounds exactly like a subtraction
__device__ __forceinline__ void accc(VC &a, float k, const float *pp, const float *mp) {
    float pv[CPT], mv[CPT];
    ldc(pp, pv);
    ldc(mp, mv);
    const float2 kk = make_float2(k, k), neg = make_float2(-1.f, -1.f);
#pragma unroll
    for (int h = 0; h < NP; h++) {
        const float2 d = __ffma2_rn(make_float2(mv[2 * h], mv[2 * h + 1]), neg, make_float2(pv[2 * h], pv[2 * h + 1]));
        const float2 r = __ffma2_rn(kk, d, make_float2(a.v[2 * h], a.v[2 * h + 1]));
        a.v[2 * h] = r.x;
        a.v[2 * h + 1] = r.y;
    }
}
__device__ __forceinline__ VC zero_cells() {
    VC a;
#pragma unroll
    for (int j = 0; j < CPT; j++) a.v[j] = 0.f;
    return a;
}
// D+x: sum_k K_k (f[r+k] - f[r-k+1])   (txx in update_vx, vz in txz update)
__device__ __forceinline__ VC dxp(const float *f, int r, int c) {
    const float *q = f + r * BZ + c;
    VC a = zero_cells();
    accc(a, K1, q + 1 * BZ, q);
    accc(a, K2, q + 2 * BZ, q - 1 * BZ);
    accc(a, K3, q + 3 * BZ, q - 2 * BZ);
    accc(a, K4, q + 4 * BZ, q - 3 * BZ);
    return a;
}
// D-x: sum_k K_k (f[r+k-1] - f[r-k])   (txz in update_vz, vx in txx update)
__device__ __forceinline__ VC dxm(const float *f, int r, int c) {
    const float *q = f + r * BZ + c;
    VC a = zero_cells();
    accc(a, K1, q, q - 1 * BZ);
    accc(a, K2, q + 1 * BZ, q - 2 * BZ);
    accc(a, K3, q + 2 * BZ, q - 3 * BZ);
    accc(a, K4, q + 3 * BZ, q - 4 * BZ);
    return a;
}
// the row window of the z stencils: this thread's cells and 4 on each side
struct WC {
    float w[CPT + 8];
};
__device__ __forceinline__ WC loadw(const float *f, int r, int c) {
    const float *q = f + r * BZ + c;
    WC o;
    if constexpr (CPT == 4) {
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float4 v = ld4(q - 4 + 4 * i);
            o.w[4 * i] = v.x;
            o.w[4 * i + 1] = v.y;
            o.w[4 * i + 2] = v.z;
            o.w[4 * i + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < (CPT + 8) / 2; i++) {
            const float2 v = *reinterpret_cast<const float2 *>(q - 4 + 2 * i);
            o.w[2 * i] = v.x;
            o.w[2 * i + 1] = v.y;
        }
    }
    return o;
}
__device__ __forceinline__ float2 pr(const WC &s, int i) { return make_float2(s.w[i], s.w[i + 1]); }
// k*(p - q) + a on a pair
__device__ __forceinline__ float2 kdiff2(float k, float2 p, float2 q, float2 a) {
    const float2 d = __ffma2_rn(q, make_float2(-1.f, -1.f), p);
    return __ffma2_rn(make_float2(k, k), d, a);
}
// D+z: sum_k K_k (f[c+k] - f[c-k+1]) on the cell pairs as FP32x2
__device__ __forceinline__ VC dzp(const WC &s) {
    VC a;
#pragma unroll
    for (int h = 0; h < NP; h++) {
        const int c = 4 + 2 * h;  // first cell of the pair
        float2 t = make_float2(0.f, 0.f);
        t = kdiff2(K1, pr(s, c + 1), pr(s, c), t);
        t = kdiff2(K2, pr(s, c + 2), pr(s, c - 1), t);
        t = kdiff2(K3, pr(s, c + 3), pr(s, c - 2), t);
        t = kdiff2(K4, pr(s, c + 4), pr(s, c - 3), t);
        a.v[2 * h] = t.x;
        a.v[2 * h + 1] = t.y;
    }
    return a;
}
// D-z: sum_k K_k (f[c+k-1] - f[c-k])
__device__ __forceinline__ VC dzm(const WC &s) {
    VC a;
#pragma unroll
    for (int h = 0; h < NP; h++) {
        const int c = 4 + 2 * h;
        float2 t = make_float2(0.f, 0.f);
        t = kdiff2(K1, pr(s, c), pr(s, c - 1), t);
        t = kdiff2(K2, pr(s, c + 1), pr(s, c - 2), t);
        t = kdiff2(K3, pr(s, c + 2), pr(s, c - 3), t);
        t = kdiff2(K4, pr(s, c + 3), pr(s, c - 4), t);
        a.v[2 * h] = t.x;
        a.v[2 * h + 1] = t.y;
    }
    return a;
}

__device__ __forceinline__ void f4_to(const float4 &a, float o[4]) {
    o[0] = a.x;
    o[1] = a.y;
    o[2] = a.z;
    o[3] = a.w;
}
__device__ __forceinline__ float4 to_f4(const float o[4]) { return make_float4(o[0], o[1], o[2], o[3]); }

// thread -> cells: TZ/CPT groups of CPT consecutive cells per row x TX rows
struct CellMap {
    int r, c;     // box coordinates of the first of the thread's cells
    int ci;       // core-tile index of the first cell
    int lx, lz;   // local row / column of the first cell
    size_t gi;    // packed index of the first cell
    bool live;    // the row is updated and the first cell's column < nzpml-NOP
    bool ok[CPT];     // cell inside the update region
    bool image[CPT];  // inside the imaging interior [pml, n-pml)
    bool split[CPT];  // updated cell with PML damping: the split update
    bool any_split;   // one of the thread's cells has the split update
};

__device__ __forceinline__ CellMap cell_map(const Params &p, const Tile &t, const ShotGeo &g) {
    CellMap m;
    const int tz = threadIdx.x % (TZ / CPT), tr = threadIdx.x / (TZ / CPT);
    m.r = tr + HALO;
    m.c = CPT * tz + HALO;
    m.ci = tr * TZ + CPT * tz;
    m.lx = t.x0 + tr;
    m.lz = t.z0 + CPT * tz;
    m.gi = (size_t)(g.row0 + m.lx) * p.P + m.lz;
    const bool row_ok = m.lx >= NOP && m.lx < g.nxpml - NOP;
    // lz is a multiple of CPT, as are NOP and P: the thread's cells lie wholly
    // before NOP (a tile grid may start there; not live) or at or after it,
    // and lz+CPT-1 < P
    m.live = row_ok && m.lz >= NOP && m.lz < g.nzpml - NOP;
    const int pml = p.pml, nzpml = g.nzpml, nxpml = g.nxpml;
    const bool xi = m.lx >= pml && m.lx < nxpml - pml;
    // damping is non-zero exactly for lx < pml, lx > nxpml-pml, lz < pml or
    // lz > nzpml-pml (k_setup); every other cell takes the plain update in
    // any tile, so results do not depend on how the grid is tiled
    const bool xd = m.lx < pml || m.lx > nxpml - pml;
    m.any_split = false;
#pragma unroll
    for (int j = 0; j < CPT; j++) {
        const int z = m.lz + j;
        m.ok[j] = row_ok && z >= NOP && z < nzpml - NOP;
        m.image[j] = m.ok[j] && xi && z >= pml && z < nzpml - pml;
        m.split[j] = m.ok[j] && (xd || z < pml || z > nzpml - pml);
        m.any_split |= m.split[j];
    }
    return m;
}

__device__ __forceinline__ void core4(const float *core, int slot, int ci, float o[CPT]) { ldc(core + slot * CORE + ci, o); }

// PML factors of a frame cell: the split update (d1*m + c*D)/d2 is evaluated
// as (d1*m + c*D) * (1/d2) with a correctly rounded reciprocal, one rounding
// more than a division
struct Damp {
    float d1[CPT], r2[CPT], d3[CPT], r4[CPT];
};
__device__ __forceinline__ Damp make_damp(const Params &p, const float x[CPT], const float z[CPT]) {
    Damp d;
#pragma unroll
    for (int j = 0; j < CPT; j++) {
        // 1 -+ (dt d)/2: halving is exact, so one fused step rounds once
        const float tx = p.dt * x[j], tz = p.dt * z[j];
        d.d1[j] = fmaf(tx, -0.5f, 1.f);
        d.r2[j] = __frcp_rn(fmaf(tx, 0.5f, 1.f));
        d.d3[j] = fmaf(tz, -0.5f, 1.f);
        d.r4[j] = __frcp_rn(fmaf(tz, 0.5f, 1.f));
    }
    return d;
}

struct VState {
    float vx[CPT], vz[CPT], mx[CPT], mz[CPT];
};
struct SState {
    float xx[CPT], zz[CPT], xz[CPT], mxx[CPT], mzz[CPT], mxz[CPT];
};

// FP32x2 helpers on the cells (2h, 2h+1) of a four-cell group
__device__ __forceinline__ float2 P2(const float v[CPT], int h) { return make_float2(v[2 * h], v[2 * h + 1]); }
__device__ __forceinline__ void S2(float v[CPT], int h, float2 x) {
    v[2 * h] = x.x;
    v[2 * h + 1] = x.y;
}
__device__ __forceinline__ float2 B2(float x) { return make_float2(x, x); }
// store a packed pair into cells 2h, 2h+1 of v where the cell is updated
__device__ __forceinline__ void sel2(float v[CPT], int h, float2 x, const bool ok[CPT]) {
    if (ok[2 * h]) v[2 * h] = x.x;
    if (ok[2 * h + 1]) v[2 * h + 1] = x.y;
}
// in a tile with PML cells: the split result where the cell is damped, the
// plain one in the other updated cells
__device__ __forceinline__ void pick2(float v[CPT], int h, float2 split, float2 plain, const CellMap &m) {
    if (m.ok[2 * h]) v[2 * h] = m.split[2 * h] ? split.x : plain.x;
    if (m.ok[2 * h + 1]) v[2 * h + 1] = m.split[2 * h + 1] ? split.y : plain.y;
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// velocity update of one field set on this thread's four cells:
//   vx += dir*ib*(dtdx*ax + dtdz*bz),  vz += dir*ib*(dtdx*dx_ + dtdz*cz)
// with the split form in frame cells; stores the new state.
template <bool FRAME>
__device__ __forceinline__ void v_apply(const Params &p, const CellMap &m, const FieldSet &f, VState &s,
                                        const float ib[CPT], const Damp &d, float dir, const VC &ax, const VC &bz,
                                        const VC &dx_, const VC &cz) {
    if (!FRAME) {
        // tile without PML cells: all four cells are updated (FP32x2)
        const float2 tx = B2(dir * p.dtdx), tz = B2(dir * p.dtdz);
#pragma unroll
        for (int h = 0; h < NP; h++) {
            const float2 i2 = P2(ib, h);
            const float2 cx = mul2(i2, tx), cz2 = mul2(i2, tz);
            S2(s.vx, h, add2(P2(s.vx, h), fma2(cx, P2(ax.v, h), mul2(cz2, P2(bz.v, h)))));
            S2(s.vz, h, add2(P2(s.vz, h), fma2(cx, P2(dx_.v, h), mul2(cz2, P2(cz.v, h)))));
        }
        stc(f.vx + m.gi, s.vx);
        stc(f.vz + m.gi, s.vz);
        return;
    }
    // tile with PML cells: the split update of the reference in damped cells,
    //   v_x = (d1 v_x + c_x D_x) r2,  v_z = (d3 v_z + c_z D_z) r4,  v = v_x + v_z,
    // with the x-part kept in mx and the z-part = v - mx; the plain update
    // above in the tile's other cells; cells outside the update region keep
    // their values
    {
        const float2 tx = B2(dir * p.dtdx), tz = B2(dir * p.dtdz), neg = B2(-1.f);
#pragma unroll
        for (int h = 0; h < NP; h++) {
            const float2 i2 = P2(ib, h);
            const float2 cx = mul2(i2, tx), cz2 = mul2(i2, tz);
            const float2 px = add2(P2(s.vx, h), fma2(cx, P2(ax.v, h), mul2(cz2, P2(bz.v, h))));
            const float2 pz = add2(P2(s.vz, h), fma2(cx, P2(dx_.v, h), mul2(cz2, P2(cz.v, h))));
            const float2 d1 = P2(d.d1, h), r2 = P2(d.r2, h), d3 = P2(d.d3, h), r4 = P2(d.r4, h);
            const float2 mx = P2(s.mx, h), mz = P2(s.mz, h);
            const float2 xx = mul2(fma2(d1, mx, mul2(cx, P2(ax.v, h))), r2);
            const float2 xz = mul2(fma2(d3, fma2(mx, neg, P2(s.vx, h)), mul2(cz2, P2(bz.v, h))), r4);
            const float2 zx = mul2(fma2(d1, mz, mul2(cx, P2(dx_.v, h))), r2);
            const float2 zz = mul2(fma2(d3, fma2(mz, neg, P2(s.vz, h)), mul2(cz2, P2(cz.v, h))), r4);
            sel2(s.mx, h, xx, m.split);
            sel2(s.mz, h, zx, m.split);
            pick2(s.vx, h, add2(xx, xz), px, m);
            pick2(s.vz, h, add2(zx, zz), pz, m);
        }
    }
    stc(f.vx + m.gi, s.vx);
    stc(f.vz + m.gi, s.vz);
    if (m.any_split) {
        stc(f.mvx + m.gi, s.mx);
        stc(f.mvz + m.gi, s.mz);
    }
}

// stress update of one field set from velocity derivatives
//   a = D-x vx, b = D-z vz, c = D+z vx, d = D+x vz
// with optional Born terms added to the split parts first (born != nullptr).
template <bool FRAME>
__device__ __forceinline__ void s_apply(const Params &p, const CellMap &m, const FieldSet &f, SState &s,
                                        const float lam[CPT], const float mu[CPT], const Damp &dm, float dir, const VC &a,
                                        const VC &b, const VC &c, const VC &d, const float (*born)[CPT]) {
    if (!FRAME) {
        // tile without PML cells: all four cells are updated (FP32x2)
        const float2 tx = B2(dir * p.dtdx), tz = B2(dir * p.dtdz);
#pragma unroll
        for (int h = 0; h < NP; h++) {
            const float2 l = P2(lam, h), u = P2(mu, h);
            const float2 l2m = fma2(u, B2(2.f), l);
            const float2 ax = mul2(tx, P2(a.v, h)), bz = mul2(tz, P2(b.v, h));
            const float2 cz = mul2(tz, P2(c.v, h)), dx_ = mul2(tx, P2(d.v, h));
            float2 xx = P2(s.xx, h), zz = P2(s.zz, h), xz = P2(s.xz, h);
            if (born) {
                xx = add2(xx, add2(P2(born[0], h), P2(born[1], h)));
                zz = add2(zz, add2(P2(born[2], h), P2(born[3], h)));
                xz = add2(xz, add2(P2(born[4], h), P2(born[5], h)));
            }
            S2(s.xx, h, add2(xx, fma2(l2m, ax, mul2(l, bz))));
            S2(s.zz, h, add2(zz, fma2(l, ax, mul2(l2m, bz))));
            S2(s.xz, h, fma2(u, fma2(tz, P2(c.v, h), dx_), xz));
        }
        stc(f.txx + m.gi, s.xx);
        stc(f.tzz + m.gi, s.zz);
        stc(f.txz + m.gi, s.xz);
        return;
    }
    // tile with PML cells: the split updates of the reference in damped cells
    // (x-parts in mxx, mzz, mxz; z-part = total - x-part), Born increments
    // added to the split parts before the damping; the plain update above in
    // the tile's other cells
    {
        const float2 tx = B2(dir * p.dtdx), tz = B2(dir * p.dtdz), neg = B2(-1.f);
#pragma unroll
        for (int h = 0; h < NP; h++) {
            const float2 l = P2(lam, h), u = P2(mu, h);
            const float2 l2m = fma2(u, B2(2.f), l);
            const float2 ax = mul2(tx, P2(a.v, h)), bz = mul2(tz, P2(b.v, h));
            const float2 cz = mul2(tz, P2(c.v, h)), dx_ = mul2(tx, P2(d.v, h));
            float2 pxx = P2(s.xx, h), pzz = P2(s.zz, h), pxz = P2(s.xz, h);
            if (born) {
                pxx = add2(pxx, add2(P2(born[0], h), P2(born[1], h)));
                pzz = add2(pzz, add2(P2(born[2], h), P2(born[3], h)));
                pxz = add2(pxz, add2(P2(born[4], h), P2(born[5], h)));
            }
            pxx = add2(pxx, fma2(l2m, ax, mul2(l, bz)));
            pzz = add2(pzz, fma2(l, ax, mul2(l2m, bz)));
            pxz = fma2(u, fma2(tz, P2(c.v, h), dx_), pxz);
            const float2 d1 = P2(dm.d1, h), r2 = P2(dm.r2, h), d3 = P2(dm.d3, h), r4 = P2(dm.r4, h);
            float2 mxx = P2(s.mxx, h), mzz = P2(s.mzz, h), mxz = P2(s.mxz, h);
            float2 zxx = fma2(mxx, neg, P2(s.xx, h)), zzz = fma2(mzz, neg, P2(s.zz, h));
            float2 zxz = fma2(mxz, neg, P2(s.xz, h));
            if (born) {
                mxx = add2(mxx, P2(born[0], h));
                zxx = add2(zxx, P2(born[1], h));
                mzz = add2(mzz, P2(born[2], h));
                zzz = add2(zzz, P2(born[3], h));
                mxz = add2(mxz, P2(born[4], h));
                zxz = add2(zxz, P2(born[5], h));
            }
            const float2 nxx_x = mul2(fma2(d1, mxx, mul2(l2m, ax)), r2);
            const float2 nxx_z = mul2(fma2(d3, zxx, mul2(l, bz)), r4);
            const float2 nzz_x = mul2(fma2(d1, mzz, mul2(l, ax)), r2);
            const float2 nzz_z = mul2(fma2(d3, zzz, mul2(l2m, bz)), r4);
            const float2 nxz_x = mul2(fma2(d1, mxz, mul2(u, dx_)), r2);
            const float2 nxz_z = mul2(fma2(d3, zxz, mul2(u, cz)), r4);
            sel2(s.mxx, h, nxx_x, m.split);
            sel2(s.mzz, h, nzz_x, m.split);
            sel2(s.mxz, h, nxz_x, m.split);
            pick2(s.xx, h, add2(nxx_x, nxx_z), pxx, m);
            pick2(s.zz, h, add2(nzz_x, nzz_z), pzz, m);
            pick2(s.xz, h, add2(nxz_x, nxz_z), pxz, m);
        }
    }
    stc(f.txx + m.gi, s.xx);
    stc(f.tzz + m.gi, s.zz);
    stc(f.txz + m.gi, s.xz);
    if (m.any_split) {
        stc(f.mtxx + m.gi, s.mxx);
        stc(f.mtzz + m.gi, s.mzz);
        stc(f.mtxz + m.gi, s.mxz);
    }
}

// ----------------------------------------------------------------------------
// the tile pipeline shared by the four kernels
// ----------------------------------------------------------------------------
// Shared-memory stage: NB halo boxes followed by NC core tiles.
__device__ __forceinline__ float *smem_base() {
    extern __shared__ __align__(1024) unsigned char sfwi_smem[];
    return reinterpret_cast<float *>(sfwi_smem);
}

struct TileCtx {
    Tile t;
    ShotGeo g;
    int brow, bcol;  // packed row / column of box element (0,0)
    int crow, ccol;  // packed row / column of core element (0,0)
};
__device__ __forceinline__ TileCtx tile_ctx(const Params &p, int ti) {
    TileCtx c;
    // one 64-byte record: four independent 16-byte loads
    const int4 *src = reinterpret_cast<const int4 *>(p.tiles + ti);
    int4 w[4];
#pragma unroll
    for (int i = 0; i < 4; i++) w[i] = __ldg(src + i);
    const TileRec *r = reinterpret_cast<const TileRec *>(w);
    c.t = r->t;
    c.g = r->g;
    c.brow = c.g.row0 + c.t.x0 - HALO;
    c.bcol = c.t.z0 - HALO;
    c.crow = c.g.row0 + c.t.x0;
    c.ccol = c.t.z0;
    return c;
}

// n (1..3) consecutive grid arrays from `arr` in one instruction: the halo
// boxes (or core tiles) of the tile land in n consecutive shared-memory slots
__device__ __forceinline__ void load_boxes(float *dst, const TmaMaps &tm, const TileCtx &c, int arr, int n,
                                           uint64_t *bar) {
    tma_load(dst, &tm.box[n - 1], c.bcol, c.brow, arr, bar);
}
__device__ __forceinline__ void load_cores(float *dst, const TmaMaps &tm, const TileCtx &c, int arr, int n,
                                           uint64_t *bar) {
    tma_load(dst, &tm.core[n - 1], c.ccol, c.crow, arr, bar);
}

// Warp-specialised tile pipeline.  Warp NTHREADS/32 is the producer: its lane
// 0 draws tile indices from this launch's counter (atomicAdd, one tile ahead;
// SMs that drew cheap tiles take more of them), reads each tile's 64-byte
// record, stores the tile's context in shared memory, and starts the tile's
// TMA loads on full[stage] once the consumers have released that stage
// (empty[stage]).  The NTHREADS consumer threads wait on full[stage], run
// body(ctx, stage_ptr), and release the stage one arrival per thread.  Every
// wait is bounded by p.wait_limit tries; a wait that gives up sets the error
// flag and the CTA winds down without leaving a copy in flight.
//   issue(ctx, stage_ptr, bar):    producer lane 0, arms `bar` with expect_tx first
//   body(ctx, stage_ptr, release): consumers; may use consumer_sync(); calls
//                                  release() once its reads of the stage are
//                                  done, so the refill overlaps its arithmetic
//                                  and stores (run_tiles releases after the
//                                  body for a thread that did not)
// Kernel `kid` (0..3: k_fwd_v, k_fwd_s, k_bwd_s, k_bwd_v) draws its tiles
// in reverse table order (the k-th drawn index takes entry ntiles-1-k) when
// bit kid of p.reverse_tiles is set.  A time loop reverses the second sweep
// of each step (k_fwd_s, k_bwd_v): consecutive sweeps then meet where one
// ended, and the first tiles a sweep stages are the ones whose outputs the
// sweep before wrote last, most of them still in L2.  Each tile's arithmetic
// does not depend on the order.
constexpr int PRODUCER_WARP = NTHREADS / 32;
constexpr int BLOCK_THREADS = NTHREADS + 32;

// one consumer thread's release of a stage (idempotent)
struct StageRelease {
    uint64_t *bar;
    bool done;
    __device__ __forceinline__ void operator()() {
        if (!done) {
            // this thread's generic-proxy reads of the stage come before the
            // asynchronous-proxy writes that refill it
            fence_proxy_async();
            mbar_arrive(bar);
            done = true;
        }
    }
};

template <int STAGE_FLOATS, int NST, class Issue, class Body>
__device__ __forceinline__ void run_tiles(const Params &p, int *counter, Issue issue, Body body, int kid) {
    const bool reverse = (p.reverse_tiles >> kid) & 1;
    __shared__ uint64_t full[NST], empty[NST];
    __shared__ TileCtx s_ctx[NST];
    __shared__ int s_tile[NST];
    float *sm = smem_base();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], NTHREADS);
        }
        fence_mbar_init();
    }
    __syncthreads();
    griddep_launch();
    if (warp == PRODUCER_WARP) {
        if (lane != 0) return;
        // the next tile's index and table entries are fetched before the wait
        // for a free stage, so their global round trips overlap that wait
        // (the counters and the tile table are written before the time loop,
        // so these reads may also precede the wait for the previous kernel)
        // tile indices are drawn one tile ahead, so each draw's round trip
        // overlaps the staging of the tile before it
        int t = atomicAdd(counter, 1);
        int t_next = atomicAdd(counter, 1);
        TileCtx ctx;
        if (t < p.ntiles) ctx = tile_ctx(p, reverse ? p.ntiles - 1 - t : t);
        griddep_wait();
        for (int k = 0;; k++) {
            const int s = k % NST;
            if (k >= NST && !mbar_wait(&empty[s], (uint32_t)((k / NST - 1) & 1), p.wait_limit)) {
                atomicExch(p.err, 2);
                return;  // consumers give up on full[s] the same way
            }
            s_tile[s] = t;
            if (t >= p.ntiles) {
                mbar_arrive(&full[s]);  // no tile: complete the phase with no bytes
                return;
            }
            s_ctx[s] = ctx;
            issue(ctx, sm + s * STAGE_FLOATS, &full[s]);
            // indices only grow: once one is past the end, so are all later ones
            t = t_next;
            if (t < p.ntiles) {
                ctx = tile_ctx(p, reverse ? p.ntiles - 1 - t : t);
                t_next = atomicAdd(counter, 1);
            }
        }
    }
    griddep_wait();
    for (int k = 0;; k++) {
        const int s = k % NST;
        const bool ok = mbar_wait(&full[s], (uint32_t)((k / NST) & 1), p.wait_limit);
        if (consumer_any(!ok)) {
            if (threadIdx.x == 0) {
                atomicExch(p.err, 1);
                // the other stages may still be loading: let them land (bounded)
                for (int j = 1; j < NST; j++)
                    mbar_wait(&full[(k + j) % NST], (uint32_t)(((k + j) / NST) & 1), p.wait_limit);
            }
            return;
        }
        if (s_tile[s] >= p.ntiles) return;
        const TileCtx ctx = s_ctx[s];  // the producer rewrites s_ctx[s] after the release
        StageRelease release{&empty[s], false};
        body(ctx, sm + s * STAGE_FLOATS, release);
        release();
    }
}

// ---------------------------------------------------------------------------
// forward snapshots
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ bool snap_step(const Params &p, int it) {
    return p.snap != nullptr && it % p.snap_every == 0;
}
inline bool snap_step_host(const Params &p, int it) { return snap_step(p, it); }
// per-shot scales of snapshot k into shared memory (every thread of the CTA
// takes part; ends with __syncthreads)
__device__ __forceinline__ void load_snap_scales(const Params &p, int k, float *s_sc) {
    const int n = 2 * min(p.nshots, SNAP_MAX_SHOTS);
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        s_sc[i] = p.sscale[((size_t)(i >> 1) * p.nsnap + k) * 2 + (i & 1)];
    __syncthreads();
}
__device__ __forceinline__ uint32_t to16(float v, int fmt) {
    return fmt == SNAP_F16 ? (uint32_t)__half_as_ushort(__float2half_rn(v))
                           : (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v));
}
__device__ __forceinline__ float from16(uint16_t u, int fmt) {
    return fmt == SNAP_F16 ? __half2float(__ushort_as_half(u)) : __bfloat162float(__ushort_as_bfloat16(u));
}
// this thread's consecutive cells (read from the staged box at `src`) of
// one component of snapshot k
__device__ __forceinline__ void store_snapc(const Params &p, int k, int comp, size_t cell, const float *src,
                                            float scale) {
    const size_t o = ((size_t)(2 * k + comp) * p.X) * p.PS + cell;
    float v[CPT];
    ldc(src, v);
    if (p.snap_fmt == SNAP_F32) {
        stc(reinterpret_cast<float *>(p.snap) + o, v);
    } else {
        const float inv = scale > 0.f ? 1.0f / scale : 0.f;
        uint32_t w[NP];
#pragma unroll
        for (int h = 0; h < NP; h++)
            w[h] = to16(v[2 * h] * inv, p.snap_fmt) | (to16(v[2 * h + 1] * inv, p.snap_fmt) << 16);
        uint16_t *dst = reinterpret_cast<uint16_t *>(p.snap) + o;
        if constexpr (CPT == 4)
            *reinterpret_cast<uint2 *>(dst) = make_uint2(w[0], w[1]);
        else
            *reinterpret_cast<uint32_t *>(dst) = w[0];
    }
}

// ---------------------------------------------------------------------------
// forward velocity sweep
// ---------------------------------------------------------------------------
template <bool BORN>
struct FwdV {
    static constexpr int NB = BORN ? 6 : 3;
    // core slots: 0 ib, 1 vx, 2 vz, 3 dampx, 4 dampz, 5 mvx, 6 mvz, [7 svx, 8 svz, 9 smvx, 10 smvz]
    static constexpr int NC = BORN ? 11 : 7;
    static constexpr int STAGE = NB * BOX + NC * CORE;
    // without the scattered field the stage is small enough for more stages
    static constexpr int NST = BORN ? NSTAGE : deep_stages(STAGE, NSTAGE + 2, 1024);
};

// SNAP: the run stores forward snapshots (p.snap set); without them the
// snapshot code is compiled out
template <bool BORN, bool SNAP>
__global__ void __launch_bounds__(BLOCK_THREADS, CTAS_PER_SM)
    k_fwd_v(const Params p, const __grid_constant__ TmaMaps tm, int it) {
    using S = FwdV<BORN>;
    auto issue = [&](const TileCtx &c, float *s, uint64_t *bar) {
        const bool frame = c.t.flags & TILE_FRAME;
        uint32_t bytes = S::NB * BOX_BYTES + (BORN ? 5 : 3) * CORE_BYTES;
        if (frame) bytes += (BORN ? 6 : 4) * CORE_BYTES;
        mbar_expect_tx(bar, bytes);
        float *core = s + S::NB * BOX;
        load_boxes(s, tm, c, BG_TXX, 3, bar);  // txx, tzz, txz
        load_cores(core + 0 * CORE, tm, c, C_IB, 1, bar);
        load_cores(core + 1 * CORE, tm, c, BG_VX, 2, bar);  // vx, vz
        if (frame) {
            load_cores(core + 3 * CORE, tm, c, C_DX, 2, bar);    // dampx, dampz
            load_cores(core + 5 * CORE, tm, c, BG_MVX, 2, bar);  // x-parts of vx, vz
        }
        if (BORN) {
            load_boxes(s + 3 * BOX, tm, c, SC_TXX, 3, bar);
            load_cores(core + 7 * CORE, tm, c, SC_VX, 2, bar);
            if (frame) load_cores(core + 9 * CORE, tm, c, SC_MVX, 2, bar);
        }
    };
    auto body = [&](const TileCtx &c, float *s, StageRelease &release) {
        float *s_xx = s, *s_zz = s + BOX, *s_xz = s + 2 * BOX;
        const float *core = s + S::NB * BOX;
        // (tile flags are the same for every consumer thread, so the barrier
        // below is taken by all of them or by none)
        if (p.src_kind == SRC_TXX_TZZ && (c.t.flags & TILE_SOURCE)) {
            if (threadIdx.x == 0) {
                // explosive source into the total txx and tzz (seen by this sweep only)
                const int r = c.g.isx - (c.t.x0 - HALO), cc = c.g.isz - c.bcol;
                const float sv = p.sou[it];
                s_xx[r * BZ + cc] += sv;
                s_zz[r * BZ + cc] += sv;
            }
            consumer_sync();
        }
        const CellMap m = cell_map(p, c.t, c.g);
        if (!m.live) return;
        const bool frame = c.t.flags & TILE_FRAME;
        // everything this thread needs from the stage, then release it
        float ib[CPT], ex[CPT], ez[CPT];
        core4(core, 0, m.ci, ib);
        if (frame) {
            core4(core, 3, m.ci, ex);
            core4(core, 4, m.ci, ez);
        }
        VState bg, sc;
        core4(core, 1, m.ci, bg.vx);
        core4(core, 2, m.ci, bg.vz);
        if (frame) {
            core4(core, 5, m.ci, bg.mx);
            core4(core, 6, m.ci, bg.mz);
        }
        const VC ax = dxp(s_xx, m.r, m.c);
        const VC bz = dzm(loadw(s_xz, m.r, m.c));
        const VC dx_ = dxm(s_xz, m.r, m.c);
        const VC cz = dzp(loadw(s_zz, m.r, m.c));
        VC sax, sbz, sdx, scz;
        if (BORN) {
            const float *b_xx = s + 3 * BOX, *b_zz = s + 4 * BOX, *b_xz = s + 5 * BOX;
            core4(core, 7, m.ci, sc.vx);
            core4(core, 8, m.ci, sc.vz);
            if (frame) {
                core4(core, 9, m.ci, sc.mx);
                core4(core, 10, m.ci, sc.mz);
            }
            sax = dxp(b_xx, m.r, m.c);
            sbz = dzm(loadw(b_xz, m.r, m.c));
            sdx = dxm(b_xz, m.r, m.c);
            scz = dzp(loadw(b_zz, m.r, m.c));
        }
        release();
        if (frame) {
            const Damp d = make_damp(p, ex, ez);
            v_apply<true>(p, m, p.bg, bg, ib, d, 1.f, ax, bz, dx_, cz);
            if (BORN) v_apply<true>(p, m, p.sc, sc, ib, d, 1.f, sax, sbz, sdx, scz);
        } else {
            const Damp d{};
            v_apply<false>(p, m, p.bg, bg, ib, d, 1.f, ax, bz, dx_, cz);
            if (BORN) v_apply<false>(p, m, p.sc, sc, ib, d, 1.f, sax, sbz, sdx, scz);
        }
        if (SNAP && snap_step(p, it) && p.snap_fmt != SNAP_F32) {
            // scale of this step's snapshot: max |v| over the shot (the bits of
            // non-negative floats order as unsigned integers)
            float mx = 0.f, mz = 0.f;
            // a vertical force enters vz after this sweep: the source cell's
            // snapshot value includes it
            const bool fsrc = p.src_kind == SRC_VZ_FORCE && (c.t.flags & TILE_SOURCE) && m.lx == c.g.isx;
#pragma unroll
            for (int j = 0; j < CPT; j++)
                if (m.ok[j]) {
                    mx = fmaxf(mx, fabsf(bg.vx[j]));
                    mz = fmaxf(mz, fabsf(fsrc && m.lz + j == c.g.isz ? bg.vz[j] + p.sou[it] : bg.vz[j]));
                }
            const unsigned am = __activemask();
            const unsigned rx = __reduce_max_sync(am, __float_as_uint(mx));
            const unsigned rz = __reduce_max_sync(am, __float_as_uint(mz));
            if ((threadIdx.x & 31) == __ffs(am) - 1) {
                unsigned *sc = reinterpret_cast<unsigned *>(p.sscale) + ((size_t)c.t.shot * p.nsnap + it / p.snap_every) * 2;
                atomicMax(sc, rx);
                atomicMax(sc + 1, rz);
            }
        }
    };
    run_tiles<S::STAGE, S::NST>(p, p.counters + 4 * it + 0, issue, body, 0);
}

// ---------------------------------------------------------------------------
// forward stress sweep (+ Born source + scattered stress), records, strips
// ---------------------------------------------------------------------------
template <bool BORN>
struct FwdS {
    static constexpr int NB = BORN ? 4 : 2;
    // core: 0 lam, 1 mu, 2 txx, 3 tzz, 4 txz, 5 dampx, 6 dampz, 7 mtxx, 8 mtzz, 9 mtxz,
    //       [10 bp, 11 bs, 12 stxx, 13 stzz, 14 stxz, 15 smtxx, 16 smtzz, 17 smtxz]
    static constexpr int NC = BORN ? 18 : 10;
    static constexpr int STAGE = NB * BOX + NC * CORE;
    static constexpr int NST = BORN ? NSTAGE : deep_stages(STAGE, NSTAGE + 2, 5120);  // + s_sc
};

template <bool BORN, bool SNAP>
__global__ void __launch_bounds__(BLOCK_THREADS, CTAS_PER_SM)
    k_fwd_s(const Params p, const __grid_constant__ TmaMaps tm, int it) {
    using S = FwdS<BORN>;
    const int sit = it % p.strip_steps;  // row block of this step in the strip arrays
    __shared__ float s_sc[2 * SNAP_MAX_SHOTS];  // snapshot scales of this step (16-bit formats)
    auto issue = [&](const TileCtx &c, float *s, uint64_t *bar) {
        const bool frame = c.t.flags & TILE_FRAME;
        uint32_t bytes = S::NB * BOX_BYTES + (BORN ? 10 : 5) * CORE_BYTES;
        if (frame) bytes += (BORN ? 8 : 5) * CORE_BYTES;
        mbar_expect_tx(bar, bytes);
        float *core = s + S::NB * BOX;
        load_boxes(s, tm, c, BG_VX, 2, bar);  // vx, vz
        load_cores(core + 0 * CORE, tm, c, C_LAM, 2, bar);   // lam, mu
        load_cores(core + 2 * CORE, tm, c, BG_TXX, 3, bar);  // txx, tzz, txz
        if (frame) {
            load_cores(core + 5 * CORE, tm, c, C_DX, 2, bar);
            load_cores(core + 7 * CORE, tm, c, BG_MTXX, 3, bar);
        }
        if (BORN) {
            load_boxes(s + 2 * BOX, tm, c, SC_VX, 2, bar);
            load_cores(core + 10 * CORE, tm, c, C_BP, 2, bar);  // bp, bs
            load_cores(core + 12 * CORE, tm, c, SC_TXX, 3, bar);
            if (frame) load_cores(core + 15 * CORE, tm, c, SC_MTXX, 3, bar);
        }
    };
    auto body = [&](const TileCtx &c, float *s, StageRelease &release) {
        const float *s_vx = s, *s_vz = s + BOX;
        const float *b_vx = s + 2 * BOX, *b_vz = s + 3 * BOX;
        const float *core = s + S::NB * BOX;
        if (p.src_kind == SRC_VZ_FORCE && (c.t.flags & TILE_SOURCE)) {
            // vertical force into the total vz: this sweep, the records, the
            // strips and the snapshot of this step see it
            if (threadIdx.x == 0) s[BOX + (c.g.isx - (c.t.x0 - HALO)) * BZ + (c.g.isz - c.bcol)] += p.sou[it];
            consumer_sync();
        }
        const CellMap m = cell_map(p, c.t, c.g);
        const bool frame = c.t.flags & TILE_FRAME;
        // receiver row: the velocities at column igz of this tile's core rows,
        // time-major per packed row (gathered into trace order after the loop)
        if ((c.t.flags & TILE_RECV) && threadIdx.x < TX) {
            const int lx = c.t.x0 + threadIdx.x;
            const int zc = c.g.igz - c.t.z0;
            if (lx >= NOP && lx < c.g.nxpml - NOP && zc >= 0 && zc < TZ) {
                const int bi = (threadIdx.x + HALO) * BZ + zc + HALO;
                float *rr = p.rrow + (size_t)it * p.nrc * p.X + c.g.row0 + lx;
                if (BORN) {
                    rr[0] = b_vz[bi];
                    rr[(size_t)p.X] = b_vx[bi];
                    rr[2 * (size_t)p.X] = s_vz[bi];
                    rr[3 * (size_t)p.X] = s_vx[bi];
                } else {
                    rr[0] = s_vz[bi];
                    rr[(size_t)p.X] = s_vx[bi];
                }
            }
        }
        // edge strips of the background velocity after this step: the core
        // cells of this tile inside each of the four bands
        if ((c.t.flags & TILE_STRIP) && p.tb) {
            const int pml = p.pml, nxpml = c.g.nxpml, nzpml = c.g.nzpml;
            for (int band = 0; band < 4; band++) {
                const Band bb = band_rect(band, pml, nxpml, nzpml);
                if (max(bb.x0, c.t.x0) >= min(bb.x1, c.t.x0 + TX) || max(bb.z0, c.t.z0) >= min(bb.z1, c.t.z0 + TZ))
                    continue;
                // top/bottom: core rows x the band's 8 columns; left/right: the
                // band's 8 rows x core columns
                const int n = band < 2 ? TX * 2 * NOP : 2 * NOP * TZ;
                for (int i = threadIdx.x; i < n; i += NTHREADS) {
                    int lx, lz;
                    if (band < 2) {
                        lx = c.t.x0 + i / (2 * NOP);
                        lz = bb.z0 + i % (2 * NOP);
                    } else {
                        lx = bb.x0 + i / TZ;
                        lz = c.t.z0 + i % TZ;
                    }
                    if (lx < bb.x0 || lx >= bb.x1 || lz < bb.z0 || lz >= bb.z1) continue;
                    if (lx < c.t.x0 || lx >= c.t.x0 + TX || lz < c.t.z0 || lz >= c.t.z0 + TZ) continue;
                    const int bi = (lx - c.t.x0 + HALO) * BZ + (lz - c.t.z0 + HALO);
                    if (band < 2) {
                        const long long o = c.g.row0 + lx;
                        p.tb[tb_row(sit, 0, band, p.X, (int)o) * 8 + (lz - bb.z0)] = s_vx[bi];
                        p.tb[tb_row(sit, 1, band, p.X, (int)o) * 8 + (lz - bb.z0)] = s_vz[bi];
                    } else {
                        const int r = lx - bb.x0;
                        p.lr[lr_row(sit, 0, band - 2, p.nshots, c.t.shot, r) * p.P + lz] = s_vx[bi];
                        p.lr[lr_row(sit, 1, band - 2, p.nshots, c.t.shot, r) * p.P + lz] = s_vz[bi];
                    }
                }
            }
        }
        // snapshot of the background velocity after this step (the staged box
        // holds it): the tile's core cells of this shot's rows and of the
        // row pitch (a tile's last columns can reach past it)
        if (SNAP && snap_step(p, it) && m.lx >= 0 && m.lx < c.g.nxpml && m.lz >= 0 && m.lz < p.PS) {
            const int k = it / p.snap_every;
            const size_t cell = (size_t)(c.g.row0 + m.lx) * p.PS + m.lz;
            const float *sc = s_sc + 2 * min(c.t.shot, SNAP_MAX_SHOTS - 1);
            store_snapc(p, k, 0, cell, s_vx + m.r * BZ + m.c, sc[0]);
            store_snapc(p, k, 1, cell, s_vz + m.r * BZ + m.c, sc[1]);
        }
        if (!m.live) return;
        // everything this thread needs from the stage, then release it
        float lam[CPT], mu[CPT], ex[CPT], ez[CPT];
        core4(core, 0, m.ci, lam);
        core4(core, 1, m.ci, mu);
        if (frame) {
            core4(core, 5, m.ci, ex);
            core4(core, 6, m.ci, ez);
        }
        const VC a = dxm(s_vx, m.r, m.c);
        const VC cc = dzp(loadw(s_vx, m.r, m.c));
        const VC b = dzm(loadw(s_vz, m.r, m.c));
        const VC d = dxp(s_vz, m.r, m.c);
        SState bg, sc;
        core4(core, 2, m.ci, bg.xx);
        core4(core, 3, m.ci, bg.zz);
        core4(core, 4, m.ci, bg.xz);
        if (frame) {
            core4(core, 7, m.ci, bg.mxx);
            core4(core, 8, m.ci, bg.mzz);
            core4(core, 9, m.ci, bg.mxz);
        }
        float bp[CPT], bs[CPT];
        VC as, cs, bs_, ds;
        if (BORN) {
            core4(core, 10, m.ci, bp);
            core4(core, 11, m.ci, bs);
            as = dxm(b_vx, m.r, m.c);
            cs = dzp(loadw(b_vx, m.r, m.c));
            bs_ = dzm(loadw(b_vz, m.r, m.c));
            ds = dxp(b_vz, m.r, m.c);
            core4(core, 12, m.ci, sc.xx);
            core4(core, 13, m.ci, sc.zz);
            core4(core, 14, m.ci, sc.xz);
            if (frame) {
                core4(core, 15, m.ci, sc.mxx);
                core4(core, 16, m.ci, sc.mzz);
                core4(core, 17, m.ci, sc.mxz);
            }
        }
        release();
        Damp dm{};
        if (frame) dm = make_damp(p, ex, ez);
        if (frame)
            s_apply<true>(p, m, p.bg, bg, lam, mu, dm, 1.f, a, b, cc, d, nullptr);
        else
            s_apply<false>(p, m, p.bg, bg, lam, mu, dm, 1.f, a, b, cc, d, nullptr);
        if (BORN) {
            // Born virtual source from the updated background velocity
            // (add_born_source_components, sfwi-stage2/born.cu:788-798); bp/bs
            // are zero outside the Born region
            float born[6][CPT];
#pragma unroll
            for (int h = 0; h < NP; h++) {
                const float2 bp2 = P2(bp, h), bs2 = P2(bs, h);
                const float2 mix = fma2(bs2, B2(-2.f), bp2);
                const float2 ax = mul2(P2(a.v, h), B2(p.idx)), bz = mul2(P2(b.v, h), B2(p.idz));
                const float2 dx_ = mul2(P2(d.v, h), B2(p.idx)), cz = mul2(P2(cc.v, h), B2(p.idz));
                const float2 dt2 = B2(p.dt);
                S2(born[0], h, mul2(dt2, mul2(bp2, ax)));
                S2(born[1], h, mul2(dt2, mul2(mix, bz)));
                S2(born[2], h, mul2(dt2, mul2(mix, ax)));
                S2(born[3], h, mul2(dt2, mul2(bp2, bz)));
                S2(born[4], h, mul2(dt2, mul2(bs2, dx_)));
                S2(born[5], h, mul2(dt2, mul2(bs2, cz)));
            }
            if (frame)
                s_apply<true>(p, m, p.sc, sc, lam, mu, dm, 1.f, as, bs_, cs, ds, born);
            else
                s_apply<false>(p, m, p.sc, sc, lam, mu, dm, 1.f, as, bs_, cs, ds, born);
        }
    };
    if (SNAP && snap_step(p, it) && p.snap_fmt != SNAP_F32) {
        griddep_wait();  // the scales come from the velocity sweep just before
        load_snap_scales(p, it / p.snap_every, s_sc);
    }
    run_tiles<S::STAGE, S::NST>(p, p.counters + 4 * it + 1, issue, body, 1);
}

// ---------------------------------------------------------------------------
// backward stress sweeps + imaging
// ---------------------------------------------------------------------------
// adjoint stress update of the four cells (txx' keeps only an x-part and
// tzz' only a z-part; txz' is split, its x-part in amxz) and its stores
__device__ __forceinline__ void adjoint_stress(const Params &p, const CellMap &m, bool frame, const Damp &dm,
                                               float adj_dir, const VC &aa, const VC &ba, const VC &ca, const VC &da,
                                               float axx[CPT], float azz[CPT], float axz[CPT], float amxz[CPT]) {
    if (!frame) {
        const float2 tx = B2(adj_dir * p.dtdx), tz = B2(adj_dir * p.dtdz);
#pragma unroll
        for (int h = 0; h < NP; h++) {
            S2(axx, h, fma2(tx, P2(aa.v, h), P2(axx, h)));
            S2(azz, h, fma2(tz, P2(ba.v, h), P2(azz, h)));
            S2(axz, h, add2(P2(axz, h), fma2(tx, P2(da.v, h), mul2(tz, P2(ca.v, h)))));
        }
    } else {
        // tile with PML cells: the split update in damped cells, the plain
        // one above in the others
        const float2 tx = B2(adj_dir * p.dtdx), tz = B2(adj_dir * p.dtdz), neg = B2(-1.f);
#pragma unroll
        for (int h = 0; h < NP; h++) {
            const float2 pxx = fma2(tx, P2(aa.v, h), P2(axx, h));
            const float2 pzz = fma2(tz, P2(ba.v, h), P2(azz, h));
            const float2 pxz = add2(P2(axz, h), fma2(tx, P2(da.v, h), mul2(tz, P2(ca.v, h))));
            const float2 d1 = P2(dm.d1, h), r2 = P2(dm.r2, h), d3 = P2(dm.d3, h), r4 = P2(dm.r4, h);
            const float2 nxx = mul2(fma2(d1, P2(axx, h), mul2(tx, P2(aa.v, h))), r2);
            const float2 nzz = mul2(fma2(d3, P2(azz, h), mul2(tz, P2(ba.v, h))), r4);
            const float2 nx_ = mul2(fma2(d1, P2(amxz, h), mul2(tx, P2(da.v, h))), r2);
            const float2 nz_ = mul2(fma2(d3, fma2(P2(amxz, h), neg, P2(axz, h)), mul2(tz, P2(ca.v, h))), r4);
            pick2(axx, h, nxx, pxx, m);
            pick2(azz, h, nzz, pzz, m);
            sel2(amxz, h, nx_, m.split);
            pick2(axz, h, add2(nx_, nz_), pxz, m);
        }
    }
    stc(p.ad.txx + m.gi, axx);
    stc(p.ad.tzz + m.gi, azz);
    stc(p.ad.txz + m.gi, axz);
    if (frame && m.any_split) stc(p.ad.mtxz + m.gi, amxz);
}

// zero-lag imaging of the lambda and mu kernels (doimage_gradient,
// FD2DGPU.cu:3350-3382) on the imaging cells, weight w:
//   G_lam += w * -(gxx + gzz)(txx' + tzz')
//   G_mu  += w * (-2 (gxx txx' + gzz tzz') - (gxz + gzx) txz')
// with the forward strains gxx = a/dx, gzz = b/dz, gxz = c/dz, gzx = d/dx
__device__ __forceinline__ void image_lam_mu(const Params &p, const CellMap &m, float w, const VC &a, const VC &b,
                                             const VC &cc, const VC &d, const float axx[CPT], const float azz[CPT],
                                             const float axz[CPT], float gl[CPT], float gm[CPT]) {
#pragma unroll
    for (int h = 0; h < NP; h++) {
        const float2 gxx = mul2(P2(a.v, h), B2(p.idx)), gzz = mul2(P2(b.v, h), B2(p.idz));
        const float2 gxz = mul2(P2(cc.v, h), B2(p.idz)), gzx = mul2(P2(d.v, h), B2(p.idx));
        const float2 x2 = P2(axx, h), z2 = P2(azz, h);
        // the increments are -lg and -mg (negation is exact)
        const float2 lg = mul2(add2(gxx, gzz), add2(x2, z2));
        const float2 mg = fma2(B2(2.f), fma2(gxx, x2, mul2(gzz, z2)), mul2(add2(gxz, gzx), P2(axz, h)));
        float2 ngl, ngm;
        if (w == 1.f) {
            ngl = fma2(B2(-1.f), lg, P2(gl, h));
            ngm = fma2(B2(-1.f), mg, P2(gm, h));
        } else {
            ngl = add2(P2(gl, h), mul2(B2(-w), lg));
            ngm = add2(P2(gm, h), mul2(B2(-w), mg));
        }
        if (m.image[2 * h]) {
            gl[2 * h] = ngl.x;
            gm[2 * h] = ngm.x;
        }
        if (m.image[2 * h + 1]) {
            gl[2 * h + 1] = ngl.y;
            gm[2 * h + 1] = ngm.y;
        }
    }
}

struct BwdS {
    static constexpr int NB = 4;  // vx, vz, avx, avz
    // core: 0 lam, 1 mu, 2 txx, 3 tzz, 4 txz, 5 atxx, 6 atzz, 7 atxz,
    //       8 dampx, 9 dampz, 10 mtxx, 11 mtzz, 12 mtxz, 13 amtxz, 14 glam, 15 gmu
    static constexpr int NC = 16;
    // edge strips of step `it` inside the box: one top/bottom band (vx, vz:
    // BX rows x 8) and one left/right band (vx, vz: 8 rows x BZ); the
    // residual source of step `it` for the box rows (BX rows x 4 columns)
    static constexpr int TBF = BX * 2 * NOP, LRF = 2 * NOP * BZ, RSF = BX * 4;
    static constexpr int STRIPS = NB * BOX + NC * CORE;
    static constexpr int RS = STRIPS + 2 * TBF + 2 * LRF;
    static constexpr int STAGE = RS + RSF;
    static constexpr int NST = NSTAGE;
};
// every TMA destination of a stage starts on a 128-byte boundary
static_assert((BOX * 4) % 128 == 0 && (CORE * 4) % 128 == 0, "box/core alignment");
static_assert((BwdS::TBF * 4) % 128 == 0 && (BwdS::LRF * 4) % 128 == 0 && (BwdS::RSF * 4) % 128 == 0,
              "strip/residual slot alignment");

// the top/bottom and the left/right band whose part inside the tile's box the
// producer stages by TMA (-1: none); a second band of the same kind (only on
// grids a box spans from edge to edge) is read from global memory instead
struct StripPick {
    int tb, lr;
};
__device__ __forceinline__ bool band_hits_box(const Band &b, int bx, int bz) {
    return max(b.x0, bx) < min(b.x1, bx + BX) && max(b.z0, bz) < min(b.z1, bz + BZ);
}
__device__ __forceinline__ StripPick strip_pick(const TileCtx &c, int pml, int nzpml) {
    StripPick sp{-1, -1};
    const int bx = c.t.x0 - HALO, bz = c.bcol, nxpml = c.g.nxpml;
    for (int b = 0; b < 2 && sp.tb < 0; b++)
        if (band_hits_box(band_rect(b, pml, nxpml, nzpml), bx, bz)) sp.tb = b;
    for (int b = 0; b < 2 && sp.lr < 0; b++)
        if (band_hits_box(band_rect(b + 2, pml, nxpml, nzpml), bx, bz)) sp.lr = b;
    return sp;
}
// bit pattern marking a packed row without a receiver in the residual source
constexpr uint32_t NO_RECEIVER = 0xFFFFFFFFu;

// the residual of step `it` replaces the adjoint velocity at the receivers
// in this sweep's view of the adjoint boxes (rs: the staged residual-source
// box; rows without a receiver carry the NO_RECEIVER pattern)
__device__ __forceinline__ void patch_residual(const TileCtx &c, const float *rs_box, int it, float *a_vx,
                                               float *a_vz) {
    if (threadIdx.x >= BX) return;
    const int lx = c.t.x0 - HALO + threadIdx.x;
    const int zc = c.g.igz - c.bcol;
    if (lx >= 0 && lx < c.g.nxpml && zc >= 0 && zc < BZ) {
        const float *rs = rs_box + threadIdx.x * 4 + (2 * it - ((2 * it) & ~3));
        if (__float_as_uint(rs[0]) != NO_RECEIVER) {
            a_vz[threadIdx.x * BZ + zc] = rs[0];
            a_vx[threadIdx.x * BZ + zc] = rs[1];
        }
    }
}

__global__ void __launch_bounds__(BLOCK_THREADS, CTAS_PER_SM)
    k_bwd_s(const Params p, const __grid_constant__ TmaMaps tm, int it, float adj_dir) {
    using S = BwdS;
    const int sit = it % p.strip_steps;  // row block of this step in the strip arrays
    auto issue = [&](const TileCtx &c, float *s, uint64_t *bar) {
        const bool frame = c.t.flags & TILE_FRAME, image = c.t.flags & TILE_IMAGE;
        const bool strip = c.t.flags & TILE_STRIP, recv = c.t.flags & TILE_RECV;
        const StripPick sp = strip ? strip_pick(c, p.pml, c.g.nzpml) : StripPick{-1, -1};
        const uint32_t bytes = S::NB * BOX_BYTES + (8 + (frame ? 6 : 0) + (image ? 2 : 0)) * CORE_BYTES +
                               (sp.tb >= 0 ? 2 * S::TBF * 4 : 0) + (sp.lr >= 0 ? 2 * S::LRF * 4 : 0) +
                               (recv ? S::RSF * 4 : 0);
        mbar_expect_tx(bar, bytes);
        float *core = s + S::NB * BOX;
        load_boxes(s, tm, c, BG_VX, 2, bar);            // vx, vz
        load_boxes(s + 2 * BOX, tm, c, AD_VX, 2, bar);  // adjoint vx, vz
        load_cores(core + 0 * CORE, tm, c, C_LAM, 2, bar);
        load_cores(core + 2 * CORE, tm, c, BG_TXX, 3, bar);
        load_cores(core + 5 * CORE, tm, c, AD_TXX, 3, bar);
        if (frame) {
            load_cores(core + 8 * CORE, tm, c, C_DX, 2, bar);
            load_cores(core + 10 * CORE, tm, c, BG_MTXX, 3, bar);
            load_cores(core + 13 * CORE, tm, c, AD_MTXZ, 1, bar);
        }
        if (image) load_cores(core + 14 * CORE, tm, c, G_LAM, 2, bar);  // G_lam, G_mu
        // rows of the strip arrays are addressed by (step, component, band,
        // row); a box row before a shot's first row reads either the fill
        // (negative coordinate) or rows no band cell maps to
        for (int comp = 0; comp < 2; comp++) {
            if (sp.tb >= 0)
                tma_load_2d(s + S::STRIPS + comp * S::TBF, &tm.tb, 0, (int)tb_row(sit, comp, sp.tb, p.X, c.brow), bar);
            if (sp.lr >= 0)
                tma_load_2d(s + S::STRIPS + 2 * S::TBF + comp * S::LRF, &tm.lr, c.bcol,
                            (int)lr_row(sit, comp, sp.lr, p.nshots, c.t.shot, 0), bar);
        }
        if (recv) tma_load_2d(s + S::RS, &tm.rs, (2 * it) & ~3, c.brow, bar);
    };
    auto body = [&](const TileCtx &c, float *s, StageRelease &release) {
        float *s_vx = s, *s_vz = s + BOX, *a_vx = s + 2 * BOX, *a_vz = s + 3 * BOX;
        const float *core = s + S::NB * BOX;
        const int pml = p.pml, nxpml = c.g.nxpml, nzpml = c.g.nzpml;
        if (c.t.flags & TILE_STRIP) {
            // the saved strips of step `it` replace vx, vz in this sweep's view:
            // the box cells inside each band (a cell in two bands holds the
            // same value in both), from the staged slots or, for a second band
            // of one kind, from global memory
            const StripPick sp = strip_pick(c, pml, nzpml);
            const float *tbs = s + S::STRIPS, *lrs = s + S::STRIPS + 2 * S::TBF;
            const int bx = c.t.x0 - HALO, bz = c.bcol;
            for (int band = 0; band < 4; band++) {
                const Band bb = band_rect(band, pml, nxpml, nzpml);
                if (!band_hits_box(bb, bx, bz)) continue;
                const bool staged = band < 2 ? band == sp.tb : band - 2 == sp.lr;
                // top/bottom: box rows x the band's 8 columns; left/right: the
                // band's 8 rows x box columns (fixed shapes, no division)
                const int n = band < 2 ? BX * 2 * NOP : 2 * NOP * BZ;
                for (int i = threadIdx.x; i < n; i += NTHREADS) {
                    int lx, lz;
                    if (band < 2) {
                        lx = bx + i / (2 * NOP);
                        lz = bb.z0 + i % (2 * NOP);
                    } else {
                        lx = bb.x0 + i / BZ;
                        lz = bz + i % BZ;
                    }
                    if (lx < bb.x0 || lx >= bb.x1 || lz < bb.z0 || lz >= bb.z1) continue;
                    if (lx < bx || lx >= bx + BX || lz < bz || lz >= bz + BZ) continue;
                    float vx, vz;
                    if (band < 2) {
                        if (staged) {
                            vx = tbs[i];  // slot (lx - bx) * 8 + (lz - z0)
                            vz = tbs[S::TBF + i];
                        } else {
                            const int prow = c.g.row0 + lx;
                            vx = p.tb[tb_row(sit, 0, band, p.X, prow) * 8 + (lz - bb.z0)];
                            vz = p.tb[tb_row(sit, 1, band, p.X, prow) * 8 + (lz - bb.z0)];
                        }
                    } else {
                        if (staged) {
                            vx = lrs[i];  // slot (lx - x0) * BZ + (lz - bz)
                            vz = lrs[S::LRF + i];
                        } else {
                            vx = p.lr[lr_row(sit, 0, band - 2, p.nshots, c.t.shot, lx - bb.x0) * p.P + lz];
                            vz = p.lr[lr_row(sit, 1, band - 2, p.nshots, c.t.shot, lx - bb.x0) * p.P + lz];
                        }
                    }
                    const int bi = (lx - bx) * BZ + (lz - bz);
                    s_vx[bi] = vx;
                    s_vz[bi] = vz;
                }
            }
        }
        if (c.t.flags & TILE_RECV) patch_residual(c, s + S::RS, it, a_vx, a_vz);
        // the views were patched: every consumer thread (same flags) waits
        if (c.t.flags & (TILE_STRIP | TILE_RECV)) consumer_sync();
        const CellMap m = cell_map(p, c.t, c.g);
        if (!m.live) return;
        const bool frame = c.t.flags & TILE_FRAME, image = c.t.flags & TILE_IMAGE;
        // everything this thread needs from the stage, then release it
        float lam[CPT], mu[CPT], ex[CPT], ez[CPT];
        core4(core, 0, m.ci, lam);
        core4(core, 1, m.ci, mu);
        if (frame) {
            core4(core, 8, m.ci, ex);
            core4(core, 9, m.ci, ez);
        }
        // reconstruction (direction -1) with strains
        const VC a = dxm(s_vx, m.r, m.c);
        const VC cc = dzp(loadw(s_vx, m.r, m.c));
        const VC b = dzm(loadw(s_vz, m.r, m.c));
        const VC d = dxp(s_vz, m.r, m.c);
        SState st;
        core4(core, 2, m.ci, st.xx);
        core4(core, 3, m.ci, st.zz);
        core4(core, 4, m.ci, st.xz);
        if (frame) {
            core4(core, 10, m.ci, st.mxx);
            core4(core, 11, m.ci, st.mzz);
            core4(core, 12, m.ci, st.mxz);
        }
        // adjoint stresses: txx' = x-part only, tzz' = z-part only, txz split
        float axx[CPT], azz[CPT], axz[CPT], amxz[CPT];
        core4(core, 5, m.ci, axx);
        core4(core, 6, m.ci, azz);
        core4(core, 7, m.ci, axz);
        if (frame) core4(core, 13, m.ci, amxz);
        const VC aa = dxm(a_vx, m.r, m.c);
        const VC ca = dzp(loadw(a_vx, m.r, m.c));
        const VC ba = dzm(loadw(a_vz, m.r, m.c));
        const VC da = dxp(a_vz, m.r, m.c);
        float gl[CPT], gm[CPT];
        if (image) {
            core4(core, 14, m.ci, gl);
            core4(core, 15, m.ci, gm);
        }
        release();
        Damp dm{};
        if (frame) dm = make_damp(p, ex, ez);
        if (frame)
            s_apply<true>(p, m, p.bg, st, lam, mu, dm, -1.f, a, b, cc, d, nullptr);
        else
            s_apply<false>(p, m, p.bg, st, lam, mu, dm, -1.f, a, b, cc, d, nullptr);
        adjoint_stress(p, m, frame, dm, adj_dir, aa, ba, ca, da, axx, azz, axz, amxz);
        // zero-lag imaging of the lambda and mu kernels (interior cells)
        if (image) {
            image_lam_mu(p, m, 1.f, a, b, cc, d, axx, azz, axz, gl, gm);
            stc(p.glam + m.gi, gl);
            stc(p.gmu + m.gi, gm);
        }
    };
    run_tiles<S::STAGE, S::NST>(p, p.counters + 4 * it + 2, issue, body, 2);
}

// Lame-weighted adjoint stresses of a staged box, in place (consumers):
//   P = (l+2m) txx + l tzz,  Q = l txx + (l+2m) tzz,  R = m txz
__device__ __forceinline__ void lame_weight(float *s_P, float *s_Q, float *s_R, const float *s_l, const float *s_u) {
    for (int i = threadIdx.x; i < BOX / 4; i += NTHREADS) {
        // four box cells per iteration whatever the cells per thread
        float xx[4], zz[4], xz[4], l[4], u[4], P_[4], Q_[4], R_[4];
        f4_to(ld4(s_P + 4 * i), xx);
        f4_to(ld4(s_Q + 4 * i), zz);
        f4_to(ld4(s_R + 4 * i), xz);
        f4_to(ld4(s_l + 4 * i), l);
        f4_to(ld4(s_u + 4 * i), u);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float l2m = fmaf(2.f, u[j], l[j]);
            P_[j] = fmaf(l2m, xx[j], l[j] * zz[j]);
            Q_[j] = fmaf(l[j], xx[j], l2m * zz[j]);
            R_[j] = u[j] * xz[j];
        }
        st4(s_P + 4 * i, to_f4(P_));
        st4(s_Q + 4 * i, to_f4(Q_));
        st4(s_R + 4 * i, to_f4(R_));
    }
}

// ---------------------------------------------------------------------------
// backward velocity sweeps + illumination
// ---------------------------------------------------------------------------
struct BwdV {
    static constexpr int NB = 8;  // txx, tzz, txz, atxx->P, atzz->Q, atxz->R, lam, mu
    // core: 0 ib, 1 vx, 2 vz, 3 avx, 4 avz, 5 dampx, 6 dampz, 7 mvx, 8 mvz, 9 amvx, 10 amvz, 11 illum
    static constexpr int NC = 12;
    static constexpr int STAGE = NB * BOX + NC * CORE;
    static constexpr int NST = NSTAGE;
};

// RHO: the run accumulates the density kernel (p.grho set); without it the
// density code is compiled out
template <bool RHO>
__global__ void __launch_bounds__(BLOCK_THREADS, CTAS_PER_SM)
    k_bwd_v(const Params p, const __grid_constant__ TmaMaps tm, int it, float adj_dir) {
    using S = BwdV;
    auto issue = [&](const TileCtx &c, float *s, uint64_t *bar) {
        const bool frame = c.t.flags & TILE_FRAME, image = c.t.flags & TILE_IMAGE;
        const uint32_t bytes = S::NB * BOX_BYTES + (5 + (frame ? 6 : 0) + (image ? 1 : 0)) * CORE_BYTES;
        mbar_expect_tx(bar, bytes);
        float *core = s + S::NB * BOX;
        load_boxes(s, tm, c, BG_TXX, 3, bar);            // txx, tzz, txz
        load_boxes(s + 3 * BOX, tm, c, AD_TXX, 3, bar);  // adjoint txx, tzz, txz
        load_boxes(s + 6 * BOX, tm, c, C_LAM, 2, bar);   // lam, mu
        load_cores(core + 0 * CORE, tm, c, C_IB, 1, bar);
        load_cores(core + 1 * CORE, tm, c, BG_VX, 2, bar);
        load_cores(core + 3 * CORE, tm, c, AD_VX, 2, bar);
        if (frame) {
            load_cores(core + 5 * CORE, tm, c, C_DX, 2, bar);
            load_cores(core + 7 * CORE, tm, c, BG_MVX, 2, bar);
            load_cores(core + 9 * CORE, tm, c, AD_MVX, 2, bar);
        }
        if (image) load_cores(core + 11 * CORE, tm, c, G_ILL, 1, bar);
    };
    auto body = [&](const TileCtx &c, float *s, StageRelease &release) {
        const float *s_xx = s, *s_zz = s + BOX, *s_xz = s + 2 * BOX;
        float *s_P = s + 3 * BOX, *s_Q = s + 4 * BOX, *s_R = s + 5 * BOX;
        const float *s_l = s + 6 * BOX, *s_u = s + 7 * BOX;
        const float *core = s + S::NB * BOX;
        lame_weight(s_P, s_Q, s_R, s_l, s_u);
        consumer_sync();
        const CellMap m = cell_map(p, c.t, c.g);
        if (!m.live) return;
        const bool frame = c.t.flags & TILE_FRAME, image = c.t.flags & TILE_IMAGE;
        // the density accumulator (when requested) is read from global memory
        // here, so that its round trip overlaps the stencils below (it does
        // not alias the arrays they store to)
        const bool rho_img = RHO && p.grho != nullptr && image;
        float gr[CPT];
        if (rho_img) ldc(p.grho + m.gi, gr);
        // everything this thread needs from the stage, then release it
        float ib[CPT], ex[CPT], ez[CPT], il[CPT];
        core4(core, 0, m.ci, ib);
        if (frame) {
            core4(core, 5, m.ci, ex);
            core4(core, 6, m.ci, ez);
        }
        VState bg, ad;
        core4(core, 1, m.ci, bg.vx);
        core4(core, 2, m.ci, bg.vz);
        if (frame) {
            core4(core, 7, m.ci, bg.mx);
            core4(core, 8, m.ci, bg.mz);
        }
        const VC ax = dxp(s_xx, m.r, m.c);
        const VC bz = dzm(loadw(s_xz, m.r, m.c));
        const VC dx_ = dxm(s_xz, m.r, m.c);
        const VC cz = dzp(loadw(s_zz, m.r, m.c));
        if (image) core4(core, 11, m.ci, il);
        core4(core, 3, m.ci, ad.vx);
        core4(core, 4, m.ci, ad.vz);
        if (frame) {
            core4(core, 9, m.ci, ad.mx);
            core4(core, 10, m.ci, ad.mz);
        }
        const VC aax = dxp(s_P, m.r, m.c);
        const VC abz = dzm(loadw(s_R, m.r, m.c));
        const VC adx = dxm(s_R, m.r, m.c);
        const VC acz = dzp(loadw(s_Q, m.r, m.c));
        release();
        Damp dm{};
        if (frame) dm = make_damp(p, ex, ez);
        // density kernel (when requested) needs the velocity step of this
        // sweep, (v(it) - v(it-1)) / dt.  Imaging cells lie outside the PML,
        // where the reconstruction (direction -1) subtracts dt (1/rho) D sigma,
        // so the step is formed from that increment directly rather than as a
        // difference of two nearly equal velocities.
        float gvx[CPT], gvz[CPT];
        if (rho_img) {
#pragma unroll
            for (int j = 0; j < CPT; j++) {
                gvx[j] = ib[j] * fmaf(ax.v[j], p.idx, bz.v[j] * p.idz);
                gvz[j] = ib[j] * fmaf(dx_.v[j], p.idx, cz.v[j] * p.idz);
            }
        }
        if (frame)
            v_apply<true>(p, m, p.bg, bg, ib, dm, -1.f, ax, bz, dx_, cz);
        else
            v_apply<false>(p, m, p.bg, bg, ib, dm, -1.f, ax, bz, dx_, cz);
        if (image) {
#pragma unroll
            for (int j = 0; j < CPT; j++)
                if (m.image[j]) il[j] += fmaf(bg.vx[j], bg.vx[j], bg.vz[j] * bg.vz[j]);
            stc(p.illum + m.gi, il);
        }
        if (frame)
            v_apply<true>(p, m, p.ad, ad, ib, dm, adj_dir, aax, abz, adx, acz);
        else
            v_apply<false>(p, m, p.ad, ad, ib, dm, adj_dir, aax, abz, adx, acz);
        if (rho_img) {
            // G_rho -= v_adj . (v(it) - v(it-1)) / dt

#pragma unroll
            for (int j = 0; j < CPT; j++)
                if (m.image[j]) gr[j] -= fmaf(ad.vx[j], gvx[j], ad.vz[j] * gvz[j]);
            stc(p.grho + m.gi, gr);
        }
    };
    run_tiles<S::STAGE, S::NST>(p, p.counters + 4 * it + 3, issue, body, 3);
}

// ---------------------------------------------------------------------------
// backward sweeps from forward snapshots (no reconstruction, no edge strips)
// ---------------------------------------------------------------------------
// k_bwd_s_snap: the adjoint stress update of k_bwd_s; at snapshot steps the
// imaging takes the forward strains from the snapshot box (vx, vz with their
// halo, decompressed in shared memory) with the reconstruction's stencils,
// weighted by the snapshot interval, and the illumination from the
// snapshot's own cells.  k_bwd_v_snap: the adjoint velocity update only.
// IMG: a snapshot step (imaging); the other steps' stages hold no snapshot
// boxes or accumulators, so those launches keep more tiles in flight
template <int FMT, bool IMG>
struct BwdSSnap {
    static constexpr int NB = 2;  // adjoint vx, vz
    // core: 0 atxx, 1 atzz, 2 atxz, 3 dampx, 4 dampz, 5 amtxz, [6 glam, 7 gmu, 8 illum]
    static constexpr int NC = IMG ? 9 : 6;
    static constexpr int SNAPF = NB * BOX + NC * CORE;         // snapshot vx, vz boxes as floats
    static constexpr int RAW = SNAPF + (IMG ? 2 * BOX : 0);    // 16-bit snapshot boxes as loaded
    static constexpr int RS = RAW + (IMG && FMT != SNAP_F32 ? BOX : 0);
    static constexpr int STAGE = RS + BX * 4;
    static constexpr int NST = IMG ? NSTAGE : deep_stages(STAGE, NSTAGE + 2, 8192);
};

// launched with IMG = snap_step(p, it)
template <int FMT, bool IMG>
__global__ void __launch_bounds__(BLOCK_THREADS, CTAS_PER_SM)
    k_bwd_s_snap(const Params p, const __grid_constant__ TmaMaps tm, int it, float adj_dir) {
    using S = BwdSSnap<FMT, IMG>;
    __shared__ float s_sc[IMG ? 2 * SNAP_MAX_SHOTS : 1];
    const bool sstep = IMG;
    const int k = it / p.snap_every;
    const float w = (float)p.snap_every;
    auto issue = [&](const TileCtx &c, float *s, uint64_t *bar) {
        const bool frame = c.t.flags & TILE_FRAME, img = sstep && (c.t.flags & TILE_IMAGE);
        const bool recv = c.t.flags & TILE_RECV;
        const uint32_t bytes = S::NB * BOX_BYTES + (3 + (frame ? 3 : 0) + (img ? 3 : 0)) * CORE_BYTES +
                               (img ? 2u * BOX * (FMT == SNAP_F32 ? 4u : 2u) : 0u) + (recv ? BX * 4u * 4u : 0u);
        mbar_expect_tx(bar, bytes);
        float *core = s + S::NB * BOX;
        load_boxes(s, tm, c, AD_VX, 2, bar);
        load_cores(core + 0 * CORE, tm, c, AD_TXX, 3, bar);
        if (frame) {
            load_cores(core + 3 * CORE, tm, c, C_DX, 2, bar);
            load_cores(core + 5 * CORE, tm, c, AD_MTXZ, 1, bar);
        }
        if (img) {
            load_cores(core + 6 * CORE, tm, c, G_LAM, 3, bar);  // G_lam, G_mu, illumination
            tma_load(s + (FMT == SNAP_F32 ? S::SNAPF : S::RAW), &tm.snap, c.bcol, c.brow, 2 * k, bar);
        }
        if (recv) tma_load_2d(s + S::RS, &tm.rs, (2 * it) & ~3, c.brow, bar);
    };
    auto body = [&](const TileCtx &c, float *s, StageRelease &release) {
        float *a_vx = s, *a_vz = s + BOX;
        const float *core = s + S::NB * BOX;
        float *sv = s + S::SNAPF;  // snapshot vx box, then vz box
        const bool img = sstep && (c.t.flags & TILE_IMAGE);
        if (c.t.flags & TILE_RECV) patch_residual(c, s + S::RS, it, a_vx, a_vz);
        if (FMT != SNAP_F32 && img) {
            const uint16_t *raw = reinterpret_cast<const uint16_t *>(s + S::RAW);
            const float *sc = s_sc + 2 * min(c.t.shot, SNAP_MAX_SHOTS - 1);
            for (int i = threadIdx.x; i < 2 * BOX; i += NTHREADS) sv[i] = from16(raw[i], FMT) * sc[i >= BOX];
        }
        // views written by other threads: every consumer thread (same flags) waits
        if ((c.t.flags & TILE_RECV) || (FMT != SNAP_F32 && img)) consumer_sync();
        const CellMap m = cell_map(p, c.t, c.g);
        if (!m.live) return;
        const bool frame = c.t.flags & TILE_FRAME;
        // everything this thread needs from the stage, then release it
        float ex[CPT], ez[CPT], axx[CPT], azz[CPT], axz[CPT], amxz[CPT], gl[CPT], gm[CPT], il[CPT], vx[CPT], vz[CPT];
        core4(core, 0, m.ci, axx);
        core4(core, 1, m.ci, azz);
        core4(core, 2, m.ci, axz);
        if (frame) {
            core4(core, 3, m.ci, ex);
            core4(core, 4, m.ci, ez);
            core4(core, 5, m.ci, amxz);
        }
        const VC aa = dxm(a_vx, m.r, m.c);
        const VC ca = dzp(loadw(a_vx, m.r, m.c));
        const VC ba = dzm(loadw(a_vz, m.r, m.c));
        const VC da = dxp(a_vz, m.r, m.c);
        VC a{}, b{}, cc{}, d{};
        if (img) {
            core4(core, 6, m.ci, gl);
            core4(core, 7, m.ci, gm);
            core4(core, 8, m.ci, il);
            a = dxm(sv, m.r, m.c);
            cc = dzp(loadw(sv, m.r, m.c));
            b = dzm(loadw(sv + BOX, m.r, m.c));
            d = dxp(sv + BOX, m.r, m.c);
            ldc(sv + m.r * BZ + m.c, vx);
            ldc(sv + BOX + m.r * BZ + m.c, vz);
        }
        release();
        Damp dm{};
        if (frame) dm = make_damp(p, ex, ez);
        adjoint_stress(p, m, frame, dm, adj_dir, aa, ba, ca, da, axx, azz, axz, amxz);
        if (img) {
            image_lam_mu(p, m, w, a, b, cc, d, axx, azz, axz, gl, gm);
#pragma unroll
            for (int j = 0; j < CPT; j++)
                if (m.image[j]) il[j] = fmaf(w, fmaf(vx[j], vx[j], vz[j] * vz[j]), il[j]);
            stc(p.glam + m.gi, gl);
            stc(p.gmu + m.gi, gm);
            stc(p.illum + m.gi, il);
        }
    };
    if (IMG && FMT != SNAP_F32) {
        griddep_wait();
        load_snap_scales(p, k, s_sc);
    }
    run_tiles<S::STAGE, S::NST>(p, p.counters + 4 * it + 2, issue, body, 2);
}

struct BwdVSnap {
    static constexpr int NB = 5;  // atxx->P, atzz->Q, atxz->R, lam, mu
    // core: 0 ib, 1 avx, 2 avz, 3 dampx, 4 dampz, 5 amvx, 6 amvz
    static constexpr int NC = 7;
    static constexpr int STAGE = NB * BOX + NC * CORE;
    static constexpr int NST = deep_stages(STAGE, NSTAGE + 1, 1024);
};

__global__ void __launch_bounds__(BLOCK_THREADS, CTAS_PER_SM)
    k_bwd_v_snap(const Params p, const __grid_constant__ TmaMaps tm, int it, float adj_dir) {
    using S = BwdVSnap;
    auto issue = [&](const TileCtx &c, float *s, uint64_t *bar) {
        const bool frame = c.t.flags & TILE_FRAME;
        mbar_expect_tx(bar, S::NB * BOX_BYTES + (3 + (frame ? 4 : 0)) * CORE_BYTES);
        float *core = s + S::NB * BOX;
        load_boxes(s, tm, c, AD_TXX, 3, bar);
        load_boxes(s + 3 * BOX, tm, c, C_LAM, 2, bar);
        load_cores(core + 0 * CORE, tm, c, C_IB, 1, bar);
        load_cores(core + 1 * CORE, tm, c, AD_VX, 2, bar);
        if (frame) {
            load_cores(core + 3 * CORE, tm, c, C_DX, 2, bar);
            load_cores(core + 5 * CORE, tm, c, AD_MVX, 2, bar);
        }
    };
    auto body = [&](const TileCtx &c, float *s, StageRelease &release) {
        float *s_P = s, *s_Q = s + BOX, *s_R = s + 2 * BOX;
        const float *core = s + S::NB * BOX;
        lame_weight(s_P, s_Q, s_R, s + 3 * BOX, s + 4 * BOX);
        consumer_sync();
        const CellMap m = cell_map(p, c.t, c.g);
        if (!m.live) return;
        const bool frame = c.t.flags & TILE_FRAME;
        float ib[CPT], ex[CPT], ez[CPT];
        core4(core, 0, m.ci, ib);
        if (frame) {
            core4(core, 3, m.ci, ex);
            core4(core, 4, m.ci, ez);
        }
        VState ad;
        core4(core, 1, m.ci, ad.vx);
        core4(core, 2, m.ci, ad.vz);
        if (frame) {
            core4(core, 5, m.ci, ad.mx);
            core4(core, 6, m.ci, ad.mz);
        }
        const VC aax = dxp(s_P, m.r, m.c);
        const VC abz = dzm(loadw(s_R, m.r, m.c));
        const VC adx = dxm(s_R, m.r, m.c);
        const VC acz = dzp(loadw(s_Q, m.r, m.c));
        release();
        if (frame) {
            const Damp dm = make_damp(p, ex, ez);
            v_apply<true>(p, m, p.ad, ad, ib, dm, adj_dir, aax, abz, adx, acz);
        } else {
            const Damp dm{};
            v_apply<false>(p, m, p.ad, ad, ib, dm, adj_dir, aax, abz, adx, acz);
        }
    };
    run_tiles<S::STAGE, S::NST>(p, p.counters + 4 * it + 3, issue, body, 3);
}

// ---------------------------------------------------------------------------
// wait probe: the tile pipeline with a producer that stages nothing, so every
// consumer's wait on its first stage runs out after p.wait_limit tries and the
// producer's wait for a free stage does too.  Both set the error flag and
// return (nothing is in flight); the host reads the flag as it does after a
// real run.  It exercises the failure path of the bounded waits without a
// fault, a trap or an unbounded spin.
// ---------------------------------------------------------------------------
constexpr int PROBE_STAGE = 32;
__global__ void __launch_bounds__(BLOCK_THREADS, CTAS_PER_SM) k_wait_probe(const Params p) {
    auto issue = [&](const TileCtx &, float *, uint64_t *) {};
    auto body = [&](const TileCtx &, float *, StageRelease &) {};
    run_tiles<PROBE_STAGE, NSTAGE>(p, p.counters, issue, body, 0);
}

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------
template <class S>
constexpr size_t stage_smem() {
    return stage_bytes(S::STAGE, S::NST);
}
static_assert(fits_stages(FwdV<true>::STAGE, FwdV<true>::NST, 1024) && fits_stages(FwdS<true>::STAGE, FwdS<true>::NST, 1024) &&
                  fits_stages(BwdS::STAGE, BwdS::NST, 1024) && fits_stages(BwdV::STAGE, BwdV::NST, 1024) &&
                  fits_stages(BwdSSnap<SNAP_F32, true>::STAGE, BwdSSnap<SNAP_F32, true>::NST, 8192) &&
                  fits_stages(BwdSSnap<SNAP_F16, true>::STAGE, BwdSSnap<SNAP_F16, true>::NST, 8192) &&
                  fits_stages(BwdVSnap::STAGE, BwdVSnap::NST, 1024),
              "tile shape too large for CTAS_PER_SM resident CTAs");

int g_nsm = 0;

cudaError_t configure_step_kernels() {
    cudaError_t e;
#define SET_SMEM(K, BYTES) \
    if ((e = cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(BYTES))) != cudaSuccess) return e;
    SET_SMEM((k_fwd_v<true, true>), stage_smem<FwdV<true>>());
    SET_SMEM((k_fwd_v<false, true>), stage_smem<FwdV<false>>());
    SET_SMEM((k_fwd_s<true, true>), stage_smem<FwdS<true>>());
    SET_SMEM((k_fwd_s<false, true>), stage_smem<FwdS<false>>());
    SET_SMEM((k_fwd_v<true, false>), stage_smem<FwdV<true>>());
    SET_SMEM((k_fwd_v<false, false>), stage_smem<FwdV<false>>());
    SET_SMEM((k_fwd_s<true, false>), stage_smem<FwdS<true>>());
    SET_SMEM((k_fwd_s<false, false>), stage_smem<FwdS<false>>());
    SET_SMEM(k_bwd_s, stage_smem<BwdS>());
    SET_SMEM(k_bwd_v<true>, stage_smem<BwdV>());
    SET_SMEM(k_bwd_v<false>, stage_smem<BwdV>());
    SET_SMEM((k_bwd_s_snap<SNAP_F32, true>), (stage_smem<BwdSSnap<SNAP_F32, true>>()));
    SET_SMEM((k_bwd_s_snap<SNAP_F16, true>), (stage_smem<BwdSSnap<SNAP_F16, true>>()));
    SET_SMEM((k_bwd_s_snap<SNAP_BF16, true>), (stage_smem<BwdSSnap<SNAP_BF16, true>>()));
    SET_SMEM((k_bwd_s_snap<SNAP_F32, false>), (stage_smem<BwdSSnap<SNAP_F32, false>>()));
    SET_SMEM((k_bwd_s_snap<SNAP_F16, false>), (stage_smem<BwdSSnap<SNAP_F16, false>>()));
    SET_SMEM((k_bwd_s_snap<SNAP_BF16, false>), (stage_smem<BwdSSnap<SNAP_BF16, false>>()));
    SET_SMEM(k_bwd_v_snap, stage_smem<BwdVSnap>());
#undef SET_SMEM
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&g_nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    return cudaSuccess;
}

static int persistent_grid(int ntiles) { return ntiles < CTAS_PER_SM * g_nsm ? ntiles : CTAS_PER_SM * g_nsm; }

// one persistent launch with programmatic stream serialisation (when
// p.overlap): the kernel may begin while the previous one in the stream
// drains, and waits for it in griddep_wait
template <class... KArgs, class... Args>
static void launch_step(void (*k)(KArgs...), size_t smem, const Params &p, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(persistent_grid(p.ntiles));
    cfg.blockDim = dim3(BLOCK_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = p.overlap ? 1 : 0;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, p, args...);
}

// one CTA; with p.ntiles >= 4 its producer draws real tiles (it reads their
// records) until it waits for a free stage
void launch_wait_probe(const Params &p, cudaStream_t st) {
    k_wait_probe<<<1, BLOCK_THREADS, stage_bytes(PROBE_STAGE, NSTAGE), st>>>(p);
}

// the snapshot-mode adjoint stress sweep: the imaging form at snapshot steps
template <int FMT>
static void launch_bwd_s_snap(const Params &p, const TmaMaps &tm, int it, float adj_dir, cudaStream_t st) {
    if (snap_step_host(p, it))
        launch_step(k_bwd_s_snap<FMT, true>, stage_smem<BwdSSnap<FMT, true>>(), p, st, tm, it, adj_dir);
    else
        launch_step(k_bwd_s_snap<FMT, false>, stage_smem<BwdSSnap<FMT, false>>(), p, st, tm, it, adj_dir);
}

void launch_step_kernel(int which, const Params &p, const TmaMaps &tm, int it, bool born, float adj_dir,
                        cudaStream_t st) {
    switch (which) {
        case 0:
            if (born)
                launch_step(p.snap ? k_fwd_v<true, true> : k_fwd_v<true, false>, stage_smem<FwdV<true>>(), p, st, tm,
                            it);
            else
                launch_step(p.snap ? k_fwd_v<false, true> : k_fwd_v<false, false>, stage_smem<FwdV<false>>(), p, st,
                            tm, it);
            break;
        case 1:
            if (born)
                launch_step(p.snap ? k_fwd_s<true, true> : k_fwd_s<true, false>, stage_smem<FwdS<true>>(), p, st, tm,
                            it);
            else
                launch_step(p.snap ? k_fwd_s<false, true> : k_fwd_s<false, false>, stage_smem<FwdS<false>>(), p, st,
                            tm, it);
            break;
        case 2:
            if (!p.snap)
                launch_step(k_bwd_s, stage_smem<BwdS>(), p, st, tm, it, adj_dir);
            else if (p.snap_fmt == SNAP_F32)
                launch_bwd_s_snap<SNAP_F32>(p, tm, it, adj_dir, st);
            else if (p.snap_fmt == SNAP_F16)
                launch_bwd_s_snap<SNAP_F16>(p, tm, it, adj_dir, st);
            else
                launch_bwd_s_snap<SNAP_BF16>(p, tm, it, adj_dir, st);
            break;
        default:
            if (!p.snap)
                launch_step(p.grho ? k_bwd_v<true> : k_bwd_v<false>, stage_smem<BwdV>(), p, st, tm, it, adj_dir);
            else
                launch_step(k_bwd_v_snap, stage_smem<BwdVSnap>(), p, st, tm, it, adj_dir);
            break;
    }
}

}  // namespace SFWI_VARIANT_NS

#define SFWI_STR2(x) #x
#define SFWI_STR(x) SFWI_STR2(x)
const TileVariant *SFWI_VARIANT_FN() {
    static const TileVariant v{TX, TZ, HALO, CTAS_PER_SM, SFWI_VARIANT_NS::NSTAGE, SFWI_STR(SFWI_VARIANT_NS),
                               &SFWI_VARIANT_NS::configure_step_kernels, &SFWI_VARIANT_NS::launch_step_kernel,
                               &SFWI_VARIANT_NS::launch_wait_probe};
    return &v;
}

}  // namespace sfwi
