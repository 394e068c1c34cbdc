// sfwi_common.cuh — data layout and device helpers shared by the kernels.
//
// Layout in HBM.  A batch of shots is packed along x: every wavefield,
// memory-variable and coefficient array is ONE 2-D array [X][P] (z fastest),
// X = sum over shots of the shot's padded width nxpml_s, P = nzpml rounded up
// to a multiple of 4 floats (16-byte rows, float4 access).  Shot s owns rows
// [row0_s, row0_s + nxpml_s).  A cell updated by a stencil is at least nop=4
// rows from its shot's first and last row, and the outer 4 rows/columns of a
// shot are never written (they stay zero, as in the reference, where the
// update kernels skip them: sfwi-stage1/born.cu:362), so no guard rows are
// needed between shots.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sfwi {

constexpr int NOP = 4;          // stencil half-width (8th order)
// Tile shape of the step kernels.  The kernel file is compiled once per
// shape (SFWI_TILE_X x SFWI_TILE_Z cells, SFWI_CTAS persistent CTAs per SM);
// the engine picks one per batch at run time (sfwi_autotune).
#ifndef SFWI_TILE_X
#define SFWI_TILE_X 16
#endif
#ifndef SFWI_TILE_Z
#define SFWI_TILE_Z 32
#endif
#ifndef SFWI_CTAS
#define SFWI_CTAS 2
#endif
constexpr int TX = SFWI_TILE_X;  // tile rows (x)
constexpr int TZ = SFWI_TILE_Z;  // tile columns (z)
constexpr int HALO = 4;
constexpr int BX = TX + 2 * HALO;  // staged box rows
constexpr int BZ = TZ + 2 * HALO;  // staged box columns (multiple of 4)
constexpr int BOX = BX * BZ;       // floats per staged box
#ifndef SFWI_CPT
#define SFWI_CPT 4
#endif
// cells per compute thread, consecutive in z (4: one float4, 2: one float2)
constexpr int CPT = SFWI_CPT;
static_assert(CPT == 2 || CPT == 4, "2 or 4 cells per thread");
constexpr int NP = CPT / 2;            // FP32x2 pairs per thread
constexpr int NTHREADS = TX * TZ / CPT;  // compute threads of a tile
constexpr int CTAS_PER_SM = SFWI_CTAS;  // persistent CTAs per SM (independent tile pipelines)

// Arrays of the packed batch grid, in allocation order: one [X][P] array each,
// consecutive in one allocation (array k starts at k*X*P floats), so a single
// 3-D TMA tensor map [array][row][column] reaches all of them.
enum GridArr {
    BG_VX, BG_VZ, BG_TXX, BG_TZZ, BG_TXZ, BG_MVX, BG_MVZ, BG_MTXX, BG_MTZZ, BG_MTXZ,
    SC_VX, SC_VZ, SC_TXX, SC_TZZ, SC_TXZ, SC_MVX, SC_MVZ, SC_MTXX, SC_MTZZ, SC_MTXZ,
    AD_VX, AD_VZ, AD_TXX, AD_TZZ, AD_TXZ, AD_MVX, AD_MVZ, AD_MTXZ,
    G_LAM, G_MU, G_ILL, G_RHO,
    NSTATE,  // arrays above are zeroed per run
    C_IB = NSTATE, C_LAM, C_MU, C_DX, C_DZ, C_BP, C_BS, C_VP, C_VS, C_RHO,
    NGRID
};

// snapshot storage formats
enum SnapFmt : int { SNAP_OFF = 0, SNAP_F32 = 1, SNAP_F16 = 2, SNAP_BF16 = 3 };
constexpr int SNAP_MAX_SHOTS = 512;  // shots of one batch in snapshot mode (per-shot scales in shared memory)

// per-shot geometry (device-resident table)
struct ShotGeo {
    int row0;      // first packed row
    int nxpml;     // padded width (rows)
    int nx;        // interior width = nxpml - 2*pml
    int isx, isz;  // source cell (local row, column)
    int igz;       // receiver column (depth index)
    int ntr;       // traces of this shot
    int tr0;       // first trace in the packed trace arrays
    int win0;      // global-model column of interior column 0 (delta_left + record_left_in_v)
    int model;     // model slot the shot's window is cut from (line searches run several models)
    int nzpml;     // padded depth of the shot's own grid (<= P; equal for every shot of a one-model batch)
};

// tile table entry: shot, first local row, first column, flags
struct Tile {
    int shot;
    int x0;
    int z0;
    int flags;
};
// tile table entry as the step kernels read it: the tile and its shot's
// geometry in one 64-byte record, fetched in one round trip per tile
struct alignas(16) TileRec {
    Tile t;
    ShotGeo g;
    int pad[1];
};
// per-shot data of the set-up, record and reduction kernels only (not read by
// the step kernels): where the shot's model lives and how long it runs
struct ShotAux {
    long long moff;  // offset (floats) of the shot's model in the model arrays
    int allnx, allnz;  // the model's grid
    int nt;          // time steps of the shot (<= the batch's nt; the shot is idle after)
    int pad;
};
static_assert(sizeof(TileRec) == 64, "TileRec is four 16-byte words");
// source kinds: sou[it] into txx and tzz ahead of the velocity sweep (the
// reference's), or a vertical force, sou[it] into vz after it
enum SourceKind : int { SRC_TXX_TZZ = 0, SRC_VZ_FORCE = 1 };
enum TileFlags : int {
    TILE_FRAME = 1,      // intersects the PML frame (damping != 0 somewhere)
    TILE_STRIP = 2,      // core or halo touches an edge strip
    TILE_RECV = 4,       // core or halo touches the receiver row
    TILE_IMAGE = 8,      // core touches the imaging interior
    TILE_SOURCE = 16,    // box contains the source cell
};

// arrays of one propagating field set (background, scattered or adjoint)
struct FieldSet {
    float *vx, *vz, *txx, *tzz, *txz;   // totals
    float *mvx, *mvz;                   // x-parts of vx, vz (frame cells only)
    float *mtxx, *mtzz, *mtxz;          // x-parts of txx, tzz, txz (frame cells only)
};

struct Coef {
    const float *ib;      // 1/rho
    const float *lam, *mu;
    const float *dampx, *dampz;
    const float *bp, *bs; // Born: 2 rho vp dvp, 2 rho vs dvs
};

struct Params {
    int X, P;            // packed rows, pitch
    int nzpml, pml, nt;
    int born_lo;         // Born source region [born_lo, n-born_lo)
    float dt, dtdx, dtdz, idx, idz;
    FieldSet bg, sc, ad;
    Coef c;
    float *glam, *gmu, *illum;  // per-cell imaging accumulators
    float *grho;                // density kernel accumulator, null unless requested
    const ShotGeo *geo;
    const TileRec *tiles;
    const float *sou;           // [nt]
    float *tb, *lr;             // edge strips (layout below); null in modelling-only runs
    int strip_steps;            // steps the strip arrays hold: nt, or the device ring of a run whose
                                // strips are kept in host memory (step it is at it % strip_steps)
    float *rrow;                // receiver-row records [nt][nrc][X]
    int nrc;                    // record components: vz, vx (+ background vz, vx in stage 2)
    // forward snapshots (snap_every = k > 0, no reconstruction): the
    // background vx, vz after every k-th step, [snapshot][vx|vz][X][PS], FP32
    // or 16-bit values in units of sscale[(shot * nsnap + snapshot) * 2 + comp]
    // (the snapshot's max |v| over the shot)
    void *snap;
    float *sscale;
    int snap_every, snap_fmt, nsnap, PS;
    int nshots;
    int ntiles;
    int *err;                   // set to a nonzero code when a bounded device wait gives up
    int *counters;              // tile counters, one per (time step, kernel): counters[4*it + kernel]
    int overlap;                // host side: launch step kernels with programmatic dependent launch
    int src_kind;               // SRC_TXX_TZZ (the reference's) or SRC_VZ_FORCE
    unsigned wait_limit;        // tries of a pipeline mbarrier wait before it is declared lost
    unsigned reverse_tiles;     // bit k: step kernel k draws its tiles in reverse table order
};
// tries of mbarrier.try_wait before a pipeline wait is declared lost (each try
// may suspend the thread for a while; the bound is several seconds)
constexpr unsigned PIPE_WAIT_LIMIT = 1u << 24;

// Edge strips of vx and vz saved each forward step and restored in the
// backward step (the reference's record_edge_wavefield/load_edge_wavefield,
// sfwi-stage1/FD2DGPU.cu:3842-3899): 2*NOP-wide bands around the interior,
//   top/bottom (band 0/1): rows [pml, nxpml-pml), columns [z0, z0+8),
//       z0 = pml-NOP or nzpml-pml-NOP;
//   left/right (band 0/1): rows [x0, x0+8), x0 = pml-NOP or nxpml-pml-NOP,
//       columns [pml, nzpml-pml).
// They are stored batch-wide and time-major, shaped so that the part of a
// band inside one tile's staged box is a single 2-D TMA box:
//   TB[tb_row(it, comp, band, X, packed row)][column - z0]   (8 floats a row)
//   LR[lr_row(it, comp, band, nshots, shot, row - x0)][column] (P floats a row)
// with comp 0 = vx, 1 = vz.  A cell in two bands is stored in both.
__host__ __device__ __forceinline__ long long tb_row(int it, int comp, int band, int X, int prow) {
    return ((long long)(it * 2 + comp) * 2 + band) * X + prow;
}
__host__ __device__ __forceinline__ long long lr_row(int it, int comp, int band, int nshots, int shot, int r) {
    return (((long long)(it * 2 + comp) * 2 + band) * nshots + shot) * 8 + r;
}
struct Band {
    int x0, x1, z0, z1;  // cell rectangle [x0, x1) x [z0, z1)
};
// b = 0 top, 1 bottom, 2 left, 3 right
__host__ __device__ __forceinline__ Band band_rect(int b, int pml, int nxpml, int nzpml) {
    Band r;
    if (b < 2) {
        r.x0 = pml;
        r.x1 = nxpml - pml;
        r.z0 = b == 0 ? pml - NOP : nzpml - pml - NOP;
        r.z1 = r.z0 + 2 * NOP;
    } else {
        r.z0 = pml;
        r.z1 = nzpml - pml;
        r.x0 = b == 2 ? pml - NOP : nxpml - pml - NOP;
        r.x1 = r.x0 + 2 * NOP;
    }
    return r;
}

__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float4 ldg4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }

}  // namespace sfwi
