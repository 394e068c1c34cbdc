// sfwi_engine.cu — host runtime behind include/sfwi_gb300.h.
//
// A handle is the counterpart of one FD2DGPU_ELASTIC object
// (sfwi-stage1/FD2DGPU.cuh:146-459).  A run packs the queued shots into one
// batch (see sfwi_common.cuh for the layout), computes their coefficients,
// then advances all of them together: nt forward steps (2 launches each),
// the residual or OT adjoint source, nt backward steps (2 launches each), and
// the FP64 reduction into the global gradients.  The forward and backward
// loops are captured once per batch shape as CUDA graphs and replayed.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <cmath>
#include <mutex>

#include "../../include/sfwi_gb300.h"
#include <cudaTypedefs.h>

#include <nvtx3/nvToolsExt.h>
#include "sfwi_launch.h"


using namespace sfwi;

namespace {

constexpr int kTimeKernelsMaxReps = 64;
// step kernels that draw their tiles in reverse order (k_fwd_s, k_bwd_v):
// each sweep starts on the tiles the sweep before finished with
constexpr unsigned kReverseTiles = (1u << 1) | (1u << 3);
constexpr double kOtSigmaFloor = OT_SIGMA_FLOOR;
thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(e_ == cudaErrorMemoryAllocation ? SFWI_E_NOMEM : SFWI_E_CUDA, "%s: %s (%s:%d)", \
                        #call, cudaGetErrorString(e_), __FILE__, __LINE__);                             \
    } while (0)

// Device buffer that grows on demand.  With a stream attached, allocation
// and release are stream-ordered (cudaMallocAsync / cudaFreeAsync on the
// owning handle's stream), so a handle that grows or frees its buffers never
// waits for work other handles have in flight on the same device.
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t st = nullptr;
    cudaError_t ensure(size_t m) {
        if (m <= n && p) return cudaSuccess;
        release();
        const size_t bytes = std::max<size_t>(m, 1) * sizeof(T);
        cudaError_t e = st ? cudaMallocAsync(reinterpret_cast<void **>(&p), bytes, st)
                           : cudaMalloc(reinterpret_cast<void **>(&p), bytes);
        if (e == cudaSuccess) {
            n = m;
        } else {
            p = nullptr;
            cudaGetLastError();  // the failure is returned here; later launch checks must not see it again
        }
        return e;
    }
    void release() {
        if (p) {
            if (st)
                cudaFreeAsync(p, st);
            else
                cudaFree(p);
        }
        p = nullptr;
        n = 0;
    }
};

// Pinned host memory for edge strips kept in host memory.  Page-locking
// takes about a second per 10 GB, so released blocks can be kept in a
// process-wide cache (up to sfwi_set_pinned_cache bytes, none by default)
// and handed to the next buffer that fits: a server that builds one engine
// per request then pins each size once.
struct PinnedCache {
    std::mutex mu;
    std::vector<std::pair<void *, size_t>> blocks;  // cached, not in use
    size_t cached = 0, limit = 0;
    // a cached block of at least `bytes` (the smallest such), or nullptr
    void *take(size_t bytes, size_t *got) {
        std::lock_guard<std::mutex> g(mu);
        size_t best = blocks.size();
        for (size_t i = 0; i < blocks.size(); i++)
            if (blocks[i].second >= bytes && (best == blocks.size() || blocks[i].second < blocks[best].second))
                best = i;
        if (best == blocks.size()) return nullptr;
        void *p = blocks[best].first;
        *got = blocks[best].second;
        cached -= *got;
        blocks.erase(blocks.begin() + best);
        return p;
    }
    // keep the block if the cache has room for it, else free it
    void give(void *p, size_t bytes) {
        {
            std::lock_guard<std::mutex> g(mu);
            if (cached + bytes <= limit) {
                blocks.emplace_back(p, bytes);
                cached += bytes;
                return;
            }
        }
        cudaFreeHost(p);
    }
    // free cached blocks until at most `keep` bytes remain
    void trim(size_t keep) {
        std::vector<void *> drop;
        {
            std::lock_guard<std::mutex> g(mu);
            std::sort(blocks.begin(), blocks.end(),
                      [](const std::pair<void *, size_t> &a, const std::pair<void *, size_t> &b) { return a.second < b.second; });
            while (cached > keep && !blocks.empty()) {
                drop.push_back(blocks.back().first);
                cached -= blocks.back().second;
                blocks.pop_back();
            }
        }
        for (void *p : drop) cudaFreeHost(p);
    }
};
PinnedCache &pinned_cache() {
    static PinnedCache c;
    return c;
}

// Pinned host buffer that grows on demand.  Growing it returns the old block
// to the cache (or frees it with cudaFreeHost, which waits for the device);
// it only grows while no run is in flight.
template <class T>
struct HostBuf {
    T *p = nullptr;
    size_t n = 0;       // elements asked for
    size_t bytes = 0;   // bytes of the block held
    cudaError_t ensure(size_t m) {
        if (m <= n && p) return cudaSuccess;
        release();
        const size_t want = std::max<size_t>(m, 1) * sizeof(T);
        size_t got = 0;
        if (void *c = pinned_cache().take(want, &got)) {
            p = static_cast<T *>(c);
            n = got / sizeof(T);
            bytes = got;
            return cudaSuccess;
        }
        cudaError_t e = cudaHostAlloc(reinterpret_cast<void **>(&p), want, cudaHostAllocDefault);
        if (e == cudaSuccess) {
            n = m;
            bytes = want;
        } else {
            p = nullptr;
            cudaGetLastError();
        }
        return e;
    }
    void release() {
        if (p) pinned_cache().give(p, bytes);
        p = nullptr;
        n = 0;
        bytes = 0;
    }
};

struct ShotIn {
    int nx, win0, isx, isz, igz, ngx_left, ntr;
    int model = 0;  // model slot (line searches)
    int req = -1;   // model of a several-model batch (sfwi_run_models), -1: the uploaded model
    int nt = 0;     // time steps of the shot (0: the handle's nt)
    std::vector<int> gc;
    const float *obs_z = nullptr, *obs_x = nullptr;  // host [ntr][nt]
};

// trace-major [ntr_tot][nt] record arrays; the first four are in the
// component order of the receiver-row records (Params::rrow)
enum RecArr { R_SYN_Z, R_SYN_X, R_SYN2_Z, R_SYN2_X, R_OBS_Z, R_OBS_X, R_RES_Z, R_RES_X, NREC };

struct Batch {
    int nshots = 0, ntiles = 0, X = 0, P = 0, ntr_tot = 0, max_nxpml = 0;
    bool ready = false;  // the batch described here is the one on the device (its upload completed)
    std::vector<ShotGeo> geo;
    std::vector<Tile> tiles;
    std::vector<std::vector<int>> rcols;  // per shot: recording and injection columns (tile flags)
    std::vector<int> trow;      // packed receiver row of each trace, -1 outside the update region
    std::vector<int> rtr;       // per packed row: the trace whose residual is injected there, or -1
    std::vector<ShotAux> aux;   // per shot: model offset and grid, time steps (several-model batches)
    std::vector<int> tlen;      // per trace: samples of its shot, empty when every shot runs nt steps
    std::vector<int> active;    // per time step: tiles of the shots still running (empty: all tiles)
    int rsp = 0;                // row length of the residual source (2 nt rounded up to 4)
    // device
    DevBuf<float> grid;      // NGRID * X * P
    DevBuf<float> tb, lr;    // edge strips (sfwi_common.cuh layout)
    // steps the strip arrays hold (nt, or a ring of two chunks when the
    // strips live in host memory), the chunk length and count of that ring
    // (0 when the strips stay on the device), and the strip bytes of the run
    int strip_steps = 0, strip_chunk = 0, strip_chunks = 0;
    size_t strip_dev_bytes = 0, strip_host_bytes = 0;
    DevBuf<float> rrow;      // receiver-row records [nt][nrc][X]
    DevBuf<float> rsrc;      // residual source [X][rsp]
    DevBuf<float> snap;      // forward snapshots (FP32 or 16-bit elements)
    DevBuf<float> sscale;    // snapshot scales [shot][snapshot][vx|vz]
    int nsnap = 0, PS = 0;   // snapshots of a run, their row pitch in elements
    DevBuf<float> recs;      // NREC * ntr_tot * nt
    DevBuf<double> tmis;     // 2 * ntr_tot
    DevBuf<double> dsigma;
    DevBuf<double> otscr;    // OT work arrays of traces longer than shared memory holds
    DevBuf<ShotGeo> dgeo;
    std::vector<TileRec> trecs;  // tiles with their shot geometry, as uploaded
    DevBuf<TileRec> dtiles;
    DevBuf<int> dtrow, drtr;
    DevBuf<ShotAux> daux;
    DevBuf<int> dtlen;
    size_t cells = 0;        // X * P
    DevBuf<int> derr;        // device-side error flag (bounded waits)
    DevBuf<int> dctr;        // dynamic tile counters of the step kernels (zeroed per run)
    TmaMaps tm;              // tensor maps of `grid` for the current X, P
    // graphs of the time loops for the current shape
    cudaGraphExec_t gfwd = nullptr, gbwd = nullptr;
    std::vector<long long> gsig;  // shape signature of the captured graphs
    float *g(int k) { return grid.p + (size_t)k * cells; }
    float *r(int k, int nt) { return recs.p + (size_t)k * ntr_tot * nt; }
    void drop_graphs() {
        if (gfwd) cudaGraphExecDestroy(gfwd);
        if (gbwd) cudaGraphExecDestroy(gbwd);
        gfwd = gbwd = nullptr;
        gsig.clear();
    }
};

}  // namespace

struct sfwi_handle {
    int stage = 1;
    int allnx = 0, allnz = 0, nxpml = 0, nzpml = 0, pml = 0, nt = 0, nop = 4, ntr = 0, scale = 1;
    float dx = 0, dz = 0, dt = 0;
    int misfit_kind = SFWI_MISFIT_L2;
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    DevBuf<float> sou, vp_all, vs_all, rho_all, dvp_all, dvs_all;
    bool have_model = false, have_rho = false, have_m = false;
    DevBuf<double> gpp, gps, gil, grh;
    bool want_rho = false;       // accumulate the density kernel as well
    int snap_every = 0;          // > 0: image from forward snapshots every k steps (no reconstruction)
    int snap_fmt = SNAP_OFF;     // storage format of the snapshots
    // one-shot state written by the reference-shaped calls
    int ngx_min = 0;
    std::vector<float> rec_z, rec_x;
    std::vector<int> gc;
    int isx = 0, isz = 0, igz = 0, ngx_left = 0, delta_left = 0, record_left_in_v = 0;
    bool have_geom = false, have_rec = false;
    std::vector<ShotIn> queue;
    Batch b;
    std::vector<int> last_ntr;   // traces of each shot of the last run
    std::vector<int> last_tr0;
    long long launches = 0;
    float fwd_ms = 0, bwd_ms = 0, other_ms = 0, total_ms = 0;
    bool use_graphs = true;
    bool launch_overlap = true;  // programmatic dependent launch of the step kernels
    unsigned tile_order = kReverseTiles;  // bit k: step kernel k draws its tiles in reverse order
    int src_kind = SRC_TXX_TZZ;  // source: the reference's txx+tzz, or a vertical force
    bool last_forward_only = false;
    const TileVariant *tv = nullptr;  // tile shape of the step kernels
    bool tile_auto = true;            // shape picked per batch by its size (until one is set)
    int nsm = 0;                      // multiprocessors of the device
    // trial models of a line search: while set, shots cut their windows from
    // these slot arrays instead of the uploaded model
    const float *slot_vp = nullptr, *slot_vs = nullptr, *slot_dvp = nullptr, *slot_dvs = nullptr;
    bool force_l2 = false;  // the exact step length is defined on the L2 residual
    // edge strips kept in host memory (the reference's cpu_mem and ntt,
    // sfwi-stage1/FD2DGPU.cu:4382-4421, :4548-4561, :4600-4622): the device
    // holds a ring of two chunks of ntt steps; every full chunk but the last
    // two moves to pinned host memory during the forward sweeps and comes
    // back during the backward sweeps, copied on a second stream while the
    // step kernels run
    int cpu_mem = 0, ntt = 0;
    // observed records go to the device on their own stream while the
    // forward sweeps run (they are first read by the misfit); obs_pending:
    // copies issued that the run's stream has not waited for yet
    cudaStream_t os = nullptr;
    cudaEvent_t ev_obs_fork = nullptr, ev_obs = nullptr;
    bool obs_pending = false;
    cudaStream_t cs = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_copy[2] = {nullptr, nullptr};
    HostBuf<float> htb, hlr;
    DevBuf<float> ls_buf;   // trial models and search directions
    // a batch over several models (sfwi_run_models): each model's grid, time
    // steps and offset in the concatenated model and gradient arrays; empty
    // while shots use the uploaded model
    struct ModelIn {
        int allnx, allnz, nt;
        size_t off;
    };
    std::vector<ModelIn> models;
    DevBuf<float> mvp, mvs, mrho, mdvp, mdvs;
    DevBuf<double> mgrad;   // [grad_pp | grad_ps | illum | grad_rho] over the models' cells
    size_t mcells = 0;
    bool m_rho = false, m_dm = false;
    std::vector<int> last_perm;  // queue index -> batch index of the last several-model run
    // exact Born adjoint (sfwi_born_adjoint): adjoint state and gathered
    // fields, accumulators, per-row shot and receiver tables, the image
    DevBuf<float> adj_f;
    DevBuf<double> adj_d, adj_img;
    DevBuf<int> adj_i;
};

namespace {

int receiver_ix(int stage, int pml, int gc, int ngx_left, float dx) {
    // GPUrecord_scatterwavefield, sfwi-stage1/FD2DGPU.cu:3161; stage 2 passes dx as int
    if (stage == 2) return pml + (int)((float)(gc - ngx_left) / (int)dx);
    return pml + (int)((float)(gc - ngx_left) / dx);
}

// column where a trace's residual is injected, GPUapplysource_backward_from_record
// (sfwi-stage1/FD2DGPU.cu:3425-3441, sfwi-stage2/FD2DGPU.cu:3357-3370): dx is a
// float in both stages, so in stage 2 it can differ from the recording column
int injection_ix(int pml, int gc, int ngx_left, float dx) { return pml + (int)((float)(gc - ngx_left) / dx); }

bool box_hits(int bx0, int bx1, int bz0, int bz1, int x0, int x1, int z0, int z1) {
    return bx0 < x1 && x0 < bx1 && bz0 < z1 && z0 < bz1;
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }
    return fn;
}

// 3-D tiled map over the packed grid: dims (P, X, NGRID) floats, boxes of
// bz x bx x depth (depth consecutive arrays); out-of-range elements of a box
// load arrive as zeros
int encode_grid_map(CUtensorMap *m, float *base, int P, int X, int bz, int bx, int depth) {
    auto enc = tensor_map_encoder();
    if (!enc) return fail(SFWI_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t dims[3] = {(cuuint64_t)P, (cuuint64_t)X, (cuuint64_t)NGRID};
    const cuuint64_t strides[2] = {(cuuint64_t)P * 4, (cuuint64_t)P * X * 4};
    const cuuint32_t box[3] = {(cuuint32_t)bz, (cuuint32_t)bx, (cuuint32_t)depth};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SFWI_E_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return SFWI_OK;
}

// 2-D tiled map over a row-major float array of `outer` rows of `inner`
// floats (row pitch a multiple of 16 bytes), boxes of box_inner x box_outer
int encode_2d_map(CUtensorMap *m, float *base, unsigned long long inner, unsigned long long outer, int box_inner,
                  int box_outer) {
    auto enc = tensor_map_encoder();
    if (!enc) return fail(SFWI_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
    const cuuint64_t strides[1] = {(cuuint64_t)inner * 4};
    const cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_outer};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SFWI_E_CUDA, "cuTensorMapEncodeTiled (2-D) failed (%d)", (int)r);
    return SFWI_OK;
}

// 3-D map over the snapshots [depth][X][PS] (FP32 or raw 16-bit elements),
// boxes of bz x bx x 2 (vx and vz of one snapshot)
int encode_snap_map(CUtensorMap *m, void *base, int fmt, int PS, int X, int depth, int bx, int bz) {
    auto enc = tensor_map_encoder();
    if (!enc) return fail(SFWI_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const size_t es = fmt == SNAP_F32 ? 4 : 2;
    const cuuint64_t dims[3] = {(cuuint64_t)PS, (cuuint64_t)X, (cuuint64_t)depth};
    const cuuint64_t strides[2] = {(cuuint64_t)PS * es, (cuuint64_t)PS * X * es};
    const cuuint32_t box[3] = {(cuuint32_t)bz, (cuuint32_t)bx, 2};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(m, fmt == SNAP_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, base,
                     dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SFWI_E_CUDA, "cuTensorMapEncodeTiled (snapshots) failed (%d)", (int)r);
    return SFWI_OK;
}

// The step kernels compiled for each tile shape, in the order of the
// SFWI_TILE_* shape indices.
const TileVariant *tile_variant(int shape) {
    switch (shape) {
    case SFWI_TILE_32x32: return tile_variant_32x32();
    case SFWI_TILE_16x64: return tile_variant_16x64();
    case SFWI_TILE_8x32_3CTA: return tile_variant_8x32x3();
    case SFWI_TILE_16x32_2CELL: return tile_variant_16x32c2();
    case SFWI_TILE_8x32_2CELL_3STAGE: return tile_variant_8x32c2s3();
    default: return tile_variant_16x32();
    }
}

// Default tile shape for a batch: the 16x32 tiles when they give every CTA
// slot (2 per SM) at least four tiles, else 8x32 tiles with two cells per
// thread and three pipeline stages, which double the tiles of a small batch
// and keep more of them in flight (one 376x201 shot: 196 16x32 tiles for 304
// slots; a step is 20 % faster on those tiles; a 38-shot batch is 14 %
// faster on 16x32).  sfwi_set_tile_shape or sfwi_autotune replace the rule.
// padded depth of a shot: its own model's in a several-model batch
int shot_nzpml(const sfwi_handle *h, const ShotIn &in) {
    return in.req >= 0 ? h->models[in.req].allnz + 2 * h->pml : h->nzpml;
}

void pick_tile_shape(sfwi_handle *h, const std::vector<ShotIn> &shots) {
    long long tiles = 0;
    for (const ShotIn &in : shots) {
        const int zt = (shot_nzpml(h, in) - 2 * NOP + 31) / 32;
        tiles += (long long)((in.nx + 2 * h->pml - 2 * NOP + 15) / 16) * zt;
    }
    h->tv = tile_variant(tiles < 4LL * 2 * std::max(h->nsm, 1) ? SFWI_TILE_8x32_2CELL_3STAGE : SFWI_TILE_16x32);
}

// Tiles of one axis of length n (with PML width pml) that start at `start`
// and cover the updated cells [NOP, n-NOP): how many, and how many of them
// hold a damped cell (index < pml or > n-pml).
struct AxisTiling {
    int start, count, frame;
};
AxisTiling axis_tiling(int n, int pml, int t, int start) {
    AxisTiling a{start, (n - NOP - start + t - 1) / t, 0};
    for (int k = 0; k < a.count; k++) {
        const int lo = std::max(start + k * t, NOP), hi = std::min(start + (k + 1) * t, n - NOP) - 1;
        if (lo < pml || hi > n - pml) a.frame++;
    }
    return a;
}
// Relative step cost of a shot's tiles: a tile holding PML cells also stages
// damping and x-parts and runs the split update, about twice an interior
// tile.
double tiling_cost(const AxisTiling &x, const AxisTiling &z) {
    const double all = (double)x.count * z.count;
    return all + (all - (double)(x.count - x.frame) * (z.count - z.frame));
}
// The best start of the x tiles of a shot for a given z tiling: any row at or
// before NOP whose first tile still holds an updated row.
AxisTiling best_x_tiling(int nxpml, int pml, int tx, const AxisTiling &z) {
    AxisTiling best = axis_tiling(nxpml, pml, tx, NOP);
    for (int st = NOP - 1; st > NOP - tx; st--) {
        const AxisTiling a = axis_tiling(nxpml, pml, tx, st);
        if (tiling_cost(a, z) < tiling_cost(best, z)) best = a;
    }
    return best;
}

// The tile table of the batch for the handle's tile shape: tiles over each
// shot's update region [NOP, n-NOP), flagged by what their core or halo box
// touches (PML frame, edge-strip bands, receiver cells, imaging interior,
// source cell).
//
// The tile grid may start before NOP so that fewer tiles hold PML cells: the
// z start is one for the batch, the x start one per shot, a function of the
// shot's width alone.  A TMA copy's first column times the element size must
// be a multiple of 16 bytes: the boxes start HALO = 4 columns before a tile,
// so z starts are NOP - 8k, which keeps box columns multiples of 8 (16-bit
// snapshot boxes) and core columns multiples of 4 (FP32).
// Cells before the grid are loaded as zeros by TMA and never updated, rows
// before a shot's first row belong to the shot before it and are only read,
// and every cell takes the same arithmetic in any tile, so the choice changes
// no result.
// The batch's z tiling: the start (NOP - 8k, k >= 0, with an updated column
// in the first tile) of least summed cost over the shots, each with its best
// x start; NOP on ties.
// Shots of different depths (several-model batches) share the start; each
// shot's tiles run to its own depth.
int plan_z_start(int pml, const int *nzpml, int tx, int tz, const int *nxpml, int nshots) {
    int start = NOP;
    double best = 0;
    static_assert(NOP % 8 == HALO % 8, "box columns NOP - HALO - 8k stay multiples of 8");
    for (int st = NOP; st > NOP - tz; st -= 8) {
        double cost = 0;
        for (int s = 0; s < nshots; s++) {
            const AxisTiling z = axis_tiling(nzpml[s], pml, tz, st);
            cost += tiling_cost(best_x_tiling(nxpml[s], pml, tx, z), z);
        }
        if (st == NOP || cost < best) {
            best = cost;
            start = st;
        }
    }
    return start;
}
AxisTiling plan_z_tiling(int pml, int nzpml, int tx, int tz, const int *nxpml, int nshots) {
    const std::vector<int> depth(std::max(nshots, 1), nzpml);
    return axis_tiling(nzpml, pml, tz, plan_z_start(pml, depth.data(), tx, tz, nxpml, nshots));
}

void build_tiles(sfwi_handle *h) {
    Batch &b = h->b;
    const int pml = h->pml, tx = h->tv->tx, tz = h->tv->tz, halo = h->tv->halo;
    std::vector<int> widths, depths;
    for (const ShotGeo &g : b.geo) {
        widths.push_back(g.nxpml);
        depths.push_back(g.nzpml);
    }
    const int zstart = plan_z_start(pml, depths.data(), tx, tz, widths.data(), b.nshots);
    b.tiles.clear();
    std::vector<int> shot_tiles(b.nshots, 0);
    for (int s = 0; s < b.nshots; s++) {
        const ShotGeo &g = b.geo[s];
        const int nxpml = g.nxpml, nzpml = g.nzpml;
        const AxisTiling zt = axis_tiling(nzpml, pml, tz, zstart);
        const std::vector<int> &cols = b.rcols[s];
        const AxisTiling xt = best_x_tiling(nxpml, pml, tx, zt);
        for (int x0 = xt.start; x0 < nxpml - NOP; x0 += tx)
            for (int z0 = zt.start; z0 < nzpml - NOP; z0 += tz) {
                const int cx1 = std::min(x0 + tx, nxpml - NOP), cz1 = std::min(z0 + tz, nzpml - NOP);
                const int cx0 = std::max(x0, NOP), cz0 = std::max(z0, NOP);
                const int bx0 = x0 - halo, bx1 = x0 + tx + halo, bz0 = z0 - halo, bz1 = z0 + tz + halo;
                int f = 0;
                // frame: updated cells with lx < pml, lx > nxpml-pml, lz < pml or lz > nzpml-pml
                if (cx0 < pml || cx1 - 1 > nxpml - pml || cz0 < pml || cz1 - 1 > nzpml - pml) f |= TILE_FRAME;
                if (box_hits(cx0, cx1, cz0, cz1, pml, nxpml - pml, pml, nzpml - pml)) f |= TILE_IMAGE;
                if (box_hits(bx0, bx1, bz0, bz1, pml, nxpml - pml, pml - NOP, pml + NOP) ||
                    box_hits(bx0, bx1, bz0, bz1, pml, nxpml - pml, nzpml - pml - NOP, nzpml - pml + NOP) ||
                    box_hits(bx0, bx1, bz0, bz1, pml - NOP, pml + NOP, pml, nzpml - pml) ||
                    box_hits(bx0, bx1, bz0, bz1, nxpml - pml - NOP, nxpml - pml + NOP, pml, nzpml - pml))
                    f |= TILE_STRIP;
                if (g.igz >= bz0 && g.igz < bz1)
                    for (int c : cols)
                        if (c >= bx0 && c < bx1) {
                            f |= TILE_RECV;
                            break;
                        }
                if (g.isx >= bx0 && g.isx < bx1 && g.isz >= bz0 && g.isz < bz1) f |= TILE_SOURCE;
                b.tiles.push_back(Tile{s, x0, z0, f});
                shot_tiles[s]++;
            }
    }
    b.ntiles = (int)b.tiles.size();
    // Every sweep ends at one end of the table (forward-order sweeps at the
    // last shots, reversed ones at the first), and its last wave of tiles is
    // its tail.  A shot's block starts and ends with PML rows, whose tiles
    // cost about twice an interior tile, so in the shots that make up the
    // last two waves at either end the interior tiles are moved to that end
    // (stable, each class in table order).  Not when shots run different
    // numbers of steps: their tiles must stay grouped by shot (below).
    bool uneven = false;
    for (const ShotAux &a : b.aux) uneven |= a.nt != h->nt;
    if (!uneven) {
        const long long wave = (long long)h->tv->ctas * std::max(h->nsm, 1);
        int head = 0, tail = 0;  // shots at the start / end covering two waves
        for (long long n = 0; head < b.nshots && n < 2 * wave; head++) n += shot_tiles[head];
        for (long long n = 0; tail < b.nshots && n < 2 * wave; tail++) n += shot_tiles[b.nshots - 1 - tail];
        // (a batch of a wave or two keeps its order: interior tiles at both
        // ends and the PML tiles in the middle made one 376x201 shot 4 %
        // slower)
        auto interior = [](const Tile &t) { return !(t.flags & TILE_FRAME); };
        if (head + tail <= b.nshots) {
            auto first = b.tiles.begin();
            for (int s = 0; s < head; s++) first += shot_tiles[s];
            std::stable_partition(b.tiles.begin(), first, interior);
            auto last = b.tiles.end();
            for (int s = 0; s < tail; s++) last -= shot_tiles[b.nshots - 1 - s];
            std::stable_partition(last, b.tiles.end(), [&](const Tile &t) { return !interior(t); });
        }
    }
    // shots that run fewer steps than the batch come last (non-increasing
    // nt): at step it the tiles of the shots still running are a prefix of
    // the table
    b.active.clear();
    if (uneven) {
        b.active.assign(h->nt, 0);
        for (int s = 0; s < b.nshots; s++)
            for (int it = 0; it < b.aux[s].nt; it++) b.active[it] += shot_tiles[s];
    }
}

// The tile table as the step kernels read it: each tile with its shot's
// geometry (b.trecs stays alive until the copy has run)
int upload_tiles(sfwi_handle *h) {
    Batch &b = h->b;
    b.trecs.resize(b.tiles.size());
    for (size_t i = 0; i < b.tiles.size(); i++) {
        b.trecs[i] = TileRec{};
        b.trecs[i].t = b.tiles[i];
        b.trecs[i].g = b.geo[b.tiles[i].shot];
    }
    CK(b.dtiles.ensure(b.trecs.size()));
    CK(cudaMemcpyAsync(b.dtiles.p, b.trecs.data(), b.trecs.size() * sizeof(TileRec), cudaMemcpyHostToDevice, h->st));
    return SFWI_OK;
}

// Tensor maps of the batch's arrays with the boxes of the handle's tile shape
// (halo boxes BX x BZ, core tiles TX x TZ); the strip, residual-source and
// snapshot maps only exist for gradient runs.
int encode_tile_maps(sfwi_handle *h, bool forward_only) {
    Batch &b = h->b;
    const int tx = h->tv->tx, tz = h->tv->tz, bx = tx + 2 * h->tv->halo, bz = tz + 2 * h->tv->halo;
    for (int d = 0; d < 3; d++) {
        if (int rc = encode_grid_map(&b.tm.box[d], b.grid.p, b.P, b.X, bz, bx, d + 1)) return rc;
        if (int rc = encode_grid_map(&b.tm.core[d], b.grid.p, b.P, b.X, tz, tx, d + 1)) return rc;
    }
    if (forward_only) return SFWI_OK;
    if (h->snap_every > 0) {
        // snapshots: [snapshot * 2 + comp][X][PS], vx and vz in one box
        if (int rc = encode_snap_map(&b.tm.snap, b.snap.p, h->snap_fmt, b.PS, b.X, 2 * b.nsnap, bx, bz)) return rc;
    } else {
        // strips: boxes of (BX rows x 8) and (8 rows x BZ)
        const unsigned long long ns = b.strip_steps;
        if (int rc = encode_2d_map(&b.tm.tb, b.tb.p, 8, ns * 4 * b.X, 8, bx)) return rc;
        if (int rc = encode_2d_map(&b.tm.lr, b.lr.p, b.P, ns * 4 * b.nshots * 8, bz, 8)) return rc;
    }
    // residual source: BX rows x 4
    return encode_2d_map(&b.tm.rs, b.rsrc.p, b.rsp, b.X, 4, bx);
}

int build_batch(sfwi_handle *h, const std::vector<ShotIn> &shots) {
    Batch &b = h->b;
    const int pml = h->pml, nt = h->nt;
    b.nshots = (int)shots.size();
    int maxz = 0;
    for (const ShotIn &in : shots) maxz = std::max(maxz, shot_nzpml(h, in));
    b.P = (maxz + 3) & ~3;
    b.geo.assign(b.nshots, ShotGeo{});
    b.aux.assign(b.nshots, ShotAux{});
    b.tiles.clear();
    b.rcols.clear();
    b.trow.clear();
    b.rtr.clear();
    b.tlen.clear();
    int row = 0, tr0 = 0;
    b.max_nxpml = 0;
    bool uneven = false;
    for (int s = 0; s < b.nshots; s++) {
        const ShotIn &in = shots[s];
        ShotGeo &g = b.geo[s];
        ShotAux &a = b.aux[s];
        const int nxpml = in.nx + 2 * pml, nzpml = shot_nzpml(h, in);
        const int allnx = in.req >= 0 ? h->models[in.req].allnx : h->allnx;
        a.moff = in.req >= 0 ? (long long)h->models[in.req].off : 0;
        a.allnx = allnx;
        a.allnz = nzpml - 2 * pml;
        a.nt = in.nt > 0 ? in.nt : nt;
        if (a.nt > nt || (s > 0 && a.nt > b.aux[s - 1].nt))
            return fail(SFWI_E_ARG, "shot %d: %d steps (at most %d, and no more than the shot before)", s, a.nt, nt);
        uneven |= a.nt != nt;
        if (in.nx < 1 || in.win0 < 0 || in.win0 + in.nx > allnx)
            return fail(SFWI_E_ARG, "shot %d: window [%d, %d) outside the model width %d", s, in.win0,
                        in.win0 + in.nx, allnx);
        if (in.isx < 0 || in.isx >= nxpml || in.isz < 0 || in.isz >= nzpml)
            return fail(SFWI_E_ARG, "shot %d: source cell (%d, %d) outside the %d x %d grid", s, in.isx, in.isz, nxpml,
                        nzpml);
        if (in.igz < 0 || in.igz >= nzpml) return fail(SFWI_E_ARG, "shot %d: receiver depth %d outside the grid", s, in.igz);
        if (in.ntr < 0 || (int)in.gc.size() != in.ntr) return fail(SFWI_E_ARG, "shot %d: bad trace count", s);
        g.row0 = row;
        g.nxpml = nxpml;
        g.nx = in.nx;
        g.isx = in.isx;
        g.isz = in.isz;
        g.igz = in.igz;
        g.ntr = in.ntr;
        g.tr0 = tr0;
        g.win0 = in.win0;
        g.model = in.model;
        g.nzpml = nzpml;
        // receiver rows: the record of a trace is its cell (rix, igz), which
        // stays zero outside the update region [NOP, n-NOP); the residual
        // injected at a cell (iix, igz) is the highest-index trace injected there
        std::vector<int> rix(in.ntr), iix(in.ntr);
        b.rtr.resize((size_t)row + nxpml, -1);
        const bool igz_live = in.igz >= NOP && in.igz < nzpml - NOP;
        for (int t = 0; t < in.ntr; t++) {
            rix[t] = receiver_ix(h->stage, pml, in.gc[t], in.ngx_left, h->dx);
            iix[t] = injection_ix(pml, in.gc[t], in.ngx_left, h->dx);
            if (rix[t] < 0 || rix[t] >= nxpml || iix[t] < 0 || iix[t] >= nxpml)
                return fail(SFWI_E_ARG, "shot %d trace %d: receiver column %d (%d) outside the %d-wide grid", s, t,
                            rix[t], iix[t], nxpml);
            const bool live = igz_live && rix[t] >= NOP && rix[t] < nxpml - NOP;
            b.trow.push_back(live ? row + rix[t] : -1);
            b.rtr[(size_t)row + iix[t]] = std::max(b.rtr[(size_t)row + iix[t]], tr0 + t);
        }
        {
            std::vector<int> cols(rix);
            cols.insert(cols.end(), iix.begin(), iix.end());
            b.rcols.push_back(std::move(cols));
        }
        row += nxpml;
        tr0 += in.ntr;
        b.max_nxpml = std::max(b.max_nxpml, nxpml);
    }
    b.X = row;
    b.ntr_tot = tr0;
    if (uneven)
        for (int s = 0; s < b.nshots; s++) b.tlen.insert(b.tlen.end(), b.geo[s].ntr, b.aux[s].nt);
    build_tiles(h);
    b.rsp = (2 * nt + 3) & ~3;
    b.cells = (size_t)b.X * b.P;
    h->last_ntr.clear();
    h->last_tr0.clear();
    for (auto &g : b.geo) {
        h->last_ntr.push_back(g.ntr);
        h->last_tr0.push_back(g.tr0);
    }
    return SFWI_OK;
}

Params make_params(sfwi_handle *h, bool forward_only) {
    Batch &b = h->b;
    Params p{};
    p.overlap = h->launch_overlap ? 1 : 0;
    p.wait_limit = PIPE_WAIT_LIMIT;
    p.reverse_tiles = h->tile_order;
    p.src_kind = h->src_kind;
    p.X = b.X;
    p.P = b.P;
    p.nzpml = h->nzpml;
    p.pml = h->pml;
    p.nt = h->nt;
    p.born_lo = h->stage == 2 ? NOP : h->pml;
    p.dt = h->dt;
    p.dtdx = h->dt / h->dx;
    p.dtdz = h->dt / h->dz;
    p.idx = 1.0f / h->dx;
    p.idz = 1.0f / h->dz;
    p.bg = FieldSet{b.g(BG_VX), b.g(BG_VZ), b.g(BG_TXX), b.g(BG_TZZ), b.g(BG_TXZ),
                    b.g(BG_MVX), b.g(BG_MVZ), b.g(BG_MTXX), b.g(BG_MTZZ), b.g(BG_MTXZ)};
    p.sc = FieldSet{b.g(SC_VX), b.g(SC_VZ), b.g(SC_TXX), b.g(SC_TZZ), b.g(SC_TXZ),
                    b.g(SC_MVX), b.g(SC_MVZ), b.g(SC_MTXX), b.g(SC_MTZZ), b.g(SC_MTXZ)};
    p.ad = FieldSet{b.g(AD_VX), b.g(AD_VZ), b.g(AD_TXX), b.g(AD_TZZ), b.g(AD_TXZ),
                    b.g(AD_MVX), b.g(AD_MVZ), nullptr, nullptr, b.g(AD_MTXZ)};
    p.c = Coef{b.g(C_IB), b.g(C_LAM), b.g(C_MU), b.g(C_DX), b.g(C_DZ), b.g(C_BP), b.g(C_BS)};
    p.glam = b.g(G_LAM);
    p.gmu = b.g(G_MU);
    p.illum = b.g(G_ILL);
    p.grho = h->want_rho && !forward_only ? b.g(G_RHO) : nullptr;
    p.geo = b.dgeo.p;
    p.tiles = b.dtiles.p;
    p.sou = h->sou.p;
    const bool snap = !forward_only && h->snap_every > 0;
    p.tb = forward_only || snap ? nullptr : b.tb.p;  // modelling only / snapshots: no strips
    p.strip_steps = b.strip_steps > 0 ? b.strip_steps : std::max(h->nt, 1);
    p.lr = forward_only || snap ? nullptr : b.lr.p;
    p.snap = snap ? b.snap.p : nullptr;
    p.sscale = snap ? b.sscale.p : nullptr;
    p.snap_every = snap ? h->snap_every : 0;
    p.snap_fmt = snap ? h->snap_fmt : SNAP_OFF;
    p.nsnap = snap ? b.nsnap : 0;
    p.PS = b.PS;
    p.rrow = b.rrow.p;
    p.nrc = h->stage == 2 ? 4 : 2;
    p.nshots = b.nshots;
    p.ntiles = b.ntiles;
    p.err = b.derr.p;
    p.counters = b.dctr.p;
    return p;
}

int upload_batch(sfwi_handle *h, const std::vector<ShotIn> &shots, bool forward_only, bool with_obs) {
    Batch &b = h->b;
    const int nt = h->nt;
    const size_t recs = (size_t)NREC * std::max(b.ntr_tot, 1) * nt;
    const int nrc = h->stage == 2 ? 4 : 2;
    const bool snap = !forward_only && h->snap_every > 0;
    b.PS = (b.P + 7) & ~7;
    b.nsnap = snap ? (nt + h->snap_every - 1) / h->snap_every : 0;
    const bool strips = !forward_only && !snap;
    const bool offload = strips && h->cpu_mem && 2 * h->ntt < nt;
    b.strip_chunk = offload ? h->ntt : 0;
    b.strip_chunks = offload ? (nt + h->ntt - 1) / h->ntt : 0;
    b.strip_steps = offload ? 2 * h->ntt : nt;
    // floats of one step of each strip array
    const size_t tb_step = (size_t)4 * b.X * 8, lr_step = (size_t)4 * b.nshots * 8 * b.P;
    b.strip_dev_bytes = strips ? (size_t)b.strip_steps * (tb_step + lr_step) * sizeof(float) : 0;
    b.strip_host_bytes = offload ? (size_t)(b.strip_chunks - 2) * h->ntt * (tb_step + lr_step) * sizeof(float) : 0;
    // TMA row coordinates of the strip arrays are 32-bit
    if (strips && ((long long)b.strip_steps * 4 * b.X >= (1LL << 31) ||
                   (long long)b.strip_steps * 4 * b.nshots * 8 >= (1LL << 31)))
        return fail(SFWI_E_ARG, "batch too large for one run (strip steps x packed rows = %lld); split the shots "
                    "or keep the strips in host memory", (long long)b.strip_steps * b.X);
    if (snap && b.nshots > SNAP_MAX_SHOTS)
        return fail(SFWI_E_ARG, "snapshot runs take at most %d shots at a time", SNAP_MAX_SHOTS);
    CK(b.grid.ensure((size_t)NGRID * b.cells));
    if (!forward_only) {
        if (snap) {
            const size_t elems = (size_t)b.nsnap * 2 * b.X * b.PS;
            CK(b.snap.ensure(h->snap_fmt == SNAP_F32 ? elems : (elems + 1) / 2));
            CK(b.sscale.ensure((size_t)b.nshots * b.nsnap * 2));
            CK(cudaMemsetAsync(b.sscale.p, 0, (size_t)b.nshots * b.nsnap * 2 * sizeof(float), h->st));
        } else {
            const size_t ntb = (size_t)b.strip_steps * tb_step, nlr = (size_t)b.strip_steps * lr_step;
            if (offload) {
                // the ring replaces strips of a larger earlier run
                if (b.tb.n > ntb) b.tb.release();
                if (b.lr.n > nlr) b.lr.release();
            }
            CK(b.tb.ensure(ntb));
            CK(b.lr.ensure(nlr));
            if (offload) {
                if (!h->cs) {
                    CK(cudaStreamCreateWithFlags(&h->cs, cudaStreamNonBlocking));
                    CK(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
                    for (auto &ev : h->ev_copy) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
                }
                const size_t held = (size_t)(b.strip_chunks - 2) * h->ntt;
                if (h->htb.n < held * tb_step || h->hlr.n < held * lr_step) {
                    CK(cudaStreamSynchronize(h->st));  // no copy of an earlier run still reads them
                    CK(h->htb.ensure(held * tb_step));
                    CK(h->hlr.ensure(held * lr_step));
                }
            }
        }
        CK(b.rsrc.ensure((size_t)b.X * b.rsp));
    }
    CK(b.rrow.ensure((size_t)nt * nrc * b.X));
    CK(b.recs.ensure(recs));
    CK(b.tmis.ensure(2 * (size_t)std::max(b.ntr_tot, 1)));
    CK(b.dsigma.ensure(2 * (size_t)std::max(b.ntr_tot, 1)));
    CK(b.dgeo.ensure(b.geo.size()));
    CK(b.dtrow.ensure(std::max<size_t>(b.trow.size(), 1)));
    CK(b.drtr.ensure(b.rtr.size()));
    CK(b.daux.ensure(b.aux.size()));
    if (!b.tlen.empty()) CK(b.dtlen.ensure(b.tlen.size()));
    CK(b.derr.ensure(1));
    CK(cudaMemsetAsync(b.derr.p, 0, sizeof(int), h->st));
    const size_t nctr = 4 * (size_t)std::max(h->nt, kTimeKernelsMaxReps + 1);
    CK(b.dctr.ensure(nctr));
    CK(cudaMemsetAsync(b.dctr.p, 0, nctr * sizeof(int), h->st));
    if (int rc = encode_tile_maps(h, forward_only)) return rc;

    cudaStream_t st = h->st;
    CK(cudaMemcpyAsync(b.dgeo.p, b.geo.data(), b.geo.size() * sizeof(ShotGeo), cudaMemcpyHostToDevice, st));
    if (int rc = upload_tiles(h)) return rc;
    if (!b.trow.empty())
        CK(cudaMemcpyAsync(b.dtrow.p, b.trow.data(), b.trow.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(b.drtr.p, b.rtr.data(), b.rtr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(b.daux.p, b.aux.data(), b.aux.size() * sizeof(ShotAux), cudaMemcpyHostToDevice, st));
    if (!b.tlen.empty())
        CK(cudaMemcpyAsync(b.dtlen.p, b.tlen.data(), b.tlen.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    // zero the state (fields, memory variables, accumulators) and the records
    CK(cudaMemsetAsync(b.grid.p, 0, (size_t)NSTATE * b.cells * sizeof(float), st));
    CK(cudaMemsetAsync(b.recs.p, 0, recs * sizeof(float), st));
    // observed records, trace-major ([ntr][its nt] on the host; a shot with
    // fewer steps than the batch keeps zeros after its last sample), copied
    // on the records stream after the zeroing above; the run's stream waits
    // for them before the misfit (wait_observed)
    if (with_obs) {
        CK(cudaEventRecord(h->ev_obs_fork, st));
        CK(cudaStreamWaitEvent(h->os, h->ev_obs_fork, 0));
        h->obs_pending = true;
        for (size_t s = 0; s < shots.size(); s++) {
            const ShotIn &in = shots[s];
            const int ns = b.aux[s].nt;
            const size_t off = (size_t)b.geo[s].tr0 * nt, n = (size_t)in.ntr * nt;
            if (!n) continue;
            const float *src[2] = {in.obs_z, in.obs_x};
            float *dst[2] = {b.r(R_OBS_Z, nt) + off, b.r(R_OBS_X, nt) + off};
            for (int c = 0; c < 2; c++) {
                if (!src[c]) continue;
                if (ns == nt)
                    CK(cudaMemcpyAsync(dst[c], src[c], n * sizeof(float), cudaMemcpyHostToDevice, h->os));
                else
                    CK(cudaMemcpy2DAsync(dst[c], (size_t)nt * sizeof(float), src[c], (size_t)ns * sizeof(float),
                                         (size_t)ns * sizeof(float), in.ntr, cudaMemcpyHostToDevice, h->os));
            }
        }
        CK(cudaEventRecord(h->ev_obs, h->os));
    }
    SetupArgs a{};
    a.X = b.X;
    a.P = b.P;
    a.nzpml = h->nzpml;
    a.pml = h->pml;
    a.allnz = h->allnz;
    a.stage = h->stage;
    a.born_lo = h->stage == 2 ? NOP : h->pml;
    a.dt = h->dt;
    const size_t nmodel = (size_t)h->allnx * h->allnz;
    a.vp_all = h->slot_vp ? h->slot_vp : h->vp_all.p;
    a.vs_all = h->slot_vs ? h->slot_vs : h->vs_all.p;
    a.vslot = h->slot_vp ? nmodel : 0;
    a.rho_all = h->have_rho ? h->rho_all.p : h->vp_all.p;
    a.dvp_all = h->slot_dvp ? h->slot_dvp : (h->stage == 2 && h->have_m ? h->dvp_all.p : nullptr);
    a.dvs_all = h->slot_dvs ? h->slot_dvs : (h->stage == 2 && h->have_m ? h->dvs_all.p : nullptr);
    a.mslot = h->slot_dvp ? nmodel : 0;
    if (!h->models.empty()) {
        // several models: each shot's own, at its offset in the concatenated arrays
        a.vp_all = h->mvp.p;
        a.vs_all = h->mvs.p;
        a.rho_all = h->m_rho ? h->mrho.p : h->mvp.p;
        a.dvp_all = h->stage == 2 && h->m_dm ? h->mdvp.p : nullptr;
        a.dvs_all = h->stage == 2 && h->m_dm ? h->mdvs.p : nullptr;
        a.vslot = a.mslot = 0;
        a.aux = b.daux.p;
    }
    a.ib = b.g(C_IB);
    a.lam = b.g(C_LAM);
    a.mu = b.g(C_MU);
    a.dampx = b.g(C_DX);
    a.dampz = b.g(C_DZ);
    a.bp = b.g(C_BP);
    a.bs = b.g(C_BS);
    a.vp = b.g(C_VP);
    a.vs = b.g(C_VS);
    a.rho = b.g(C_RHO);
    a.geo = b.dgeo.p;
    CK(cudaEventRecord(h->ev[4], st));
    launch_setup(a, b.nshots, b.max_nxpml, st);
    h->launches++;
    CK(cudaGetLastError());
    return SFWI_OK;
}

// The run's stream waits for the observed records issued by upload_batch.
int wait_observed(sfwi_handle *h) {
    if (h->obs_pending) {
        CK(cudaStreamWaitEvent(h->st, h->ev_obs, 0));
        h->obs_pending = false;
    }
    return SFWI_OK;
}

// A run that ends early (an error) must not leave a copy reading the
// caller's host records behind it.
struct ObservedGuard {
    sfwi_handle *h;
    ~ObservedGuard() {
        if (h->obs_pending) {
            cudaStreamSynchronize(h->os);
            h->obs_pending = false;
        }
    }
};

std::vector<long long> shape_signature(sfwi_handle *h, bool forward_only) {
    Batch &b = h->b;
    std::vector<long long> s = {h->nt, h->stage, forward_only, h->want_rho, h->snap_every, h->snap_fmt,
                                (long long)(uintptr_t)h->tv, h->launch_overlap, h->tile_order, h->src_kind,
                                (long long)(uintptr_t)b.snap.p, (long long)(uintptr_t)b.sscale.p, b.nshots, b.ntiles,
                                b.X, b.P,
                                b.ntr_tot, b.rsp, (long long)(uintptr_t)b.grid.p, (long long)(uintptr_t)b.tb.p,
                                (long long)(uintptr_t)b.lr.p, (long long)(uintptr_t)b.rrow.p,
                                (long long)(uintptr_t)b.rsrc.p, (long long)(uintptr_t)b.dtiles.p,
                                (long long)(uintptr_t)b.dgeo.p, (long long)(uintptr_t)h->sou.p, b.strip_steps,
                                b.strip_chunk, (long long)(uintptr_t)h->htb.p, (long long)(uintptr_t)h->hlr.p};
    for (auto &t : b.tiles) s.push_back(((long long)t.shot << 40) ^ ((long long)t.x0 << 24) ^ (t.z0 << 8) ^ t.flags);
    for (auto &g : b.geo) {
        s.push_back(g.isx * 100003LL + g.isz);
        s.push_back(g.igz * 1000003LL + g.nx);
        s.push_back(g.row0 * 100003LL + g.nzpml);
    }
    s.insert(s.end(), b.active.begin(), b.active.end());
    return s;
}

// the launch parameters of step `it`: with shots of different lengths, only
// the tiles of the shots still running (a prefix of the table)
Params step_params(const sfwi_handle *h, const Params &p, int it) {
    Params q = p;
    if (!h->b.active.empty()) q.ntiles = h->b.active[it];
    return q;
}

// Copy chunk `chunk` of the edge strips between its ring slot (chunk % 2) on
// the device and its place in host memory, on the copy stream, after the
// work queued so far on the run's stream; ev_copy[slot] marks its end.
int strip_copy(sfwi_handle *h, int chunk, bool to_host) {
    Batch &b = h->b;
    const size_t tb_step = (size_t)4 * b.X * 8, lr_step = (size_t)4 * b.nshots * 8 * b.P;
    const size_t n = b.strip_chunk, slot = chunk % 2;
    float *dtb = b.tb.p + slot * n * tb_step, *htb = h->htb.p + (size_t)chunk * n * tb_step;
    float *dlr = b.lr.p + slot * n * lr_step, *hlr = h->hlr.p + (size_t)chunk * n * lr_step;
    CK(cudaEventRecord(h->ev_fork, h->st));
    CK(cudaStreamWaitEvent(h->cs, h->ev_fork, 0));
    if (to_host) {
        CK(cudaMemcpyAsync(htb, dtb, n * tb_step * sizeof(float), cudaMemcpyDeviceToHost, h->cs));
        CK(cudaMemcpyAsync(hlr, dlr, n * lr_step * sizeof(float), cudaMemcpyDeviceToHost, h->cs));
    } else {
        CK(cudaMemcpyAsync(dtb, htb, n * tb_step * sizeof(float), cudaMemcpyHostToDevice, h->cs));
        CK(cudaMemcpyAsync(dlr, hlr, n * lr_step * sizeof(float), cudaMemcpyHostToDevice, h->cs));
    }
    CK(cudaEventRecord(h->ev_copy[slot], h->cs));
    return SFWI_OK;
}

// The forward time loop.  With the strips in host memory, chunk c (steps
// [c ntt, (c+1) ntt)) is written into ring slot c % 2 once the copy of chunk
// c - 2 out of that slot has ended, and goes to host memory itself when it
// is full, unless it is one of the last two chunks (those stay in the ring
// for the first backward steps).
int enqueue_forward(sfwi_handle *h, const Params &p, bool forward_only) {
    const bool born = h->stage == 2;
    (void)forward_only;
    const int n = h->b.strip_chunk, nc = h->b.strip_chunks;
    for (int it = 0; it < h->nt; it++) {
        if (n && it % n == 0 && it / n >= 2) CK(cudaStreamWaitEvent(h->st, h->ev_copy[(it / n) % 2], 0));
        const Params q = step_params(h, p, it);
        h->tv->launch(0, q, h->b.tm, it, born, 1.f, h->st);
        h->tv->launch(1, q, h->b.tm, it, born, 1.f, h->st);
        if (n && (it + 1) % n == 0 && (it + 1) / n <= nc - 2)
            if (int rc = strip_copy(h, it / n, true)) return rc;
    }
    return SFWI_OK;
}

// The backward time loop.  With the strips in host memory, the first
// backward step of chunk c <= nc - 3 waits for its copy back into slot c % 2,
// which starts once chunk c + 2, the slot's last user, is done.
int enqueue_backward(sfwi_handle *h, const Params &p) {
    const float adj = h->stage == 1 ? 1.f : -1.f;
    const int n = h->b.strip_chunk, nc = h->b.strip_chunks;
    for (int it = h->nt - 1; it >= 0; it--) {
        const int c = n ? it / n : 0;
        if (n && (it + 1) % n == 0 && c <= nc - 3) CK(cudaStreamWaitEvent(h->st, h->ev_copy[c % 2], 0));
        const Params q = step_params(h, p, it);
        h->tv->launch(2, q, h->b.tm, it, false, adj, h->st);
        h->tv->launch(3, q, h->b.tm, it, false, adj, h->st);
        if (n && it % n == 0 && c >= 2)
            if (int rc = strip_copy(h, c - 2, false)) return rc;
    }
    return SFWI_OK;
}

int capture(sfwi_handle *h, cudaGraphExec_t *out, bool fwd, const Params &p, bool forward_only) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    const int rc = fwd ? enqueue_forward(h, p, forward_only) : enqueue_backward(h, p);
    cudaError_t e = cudaStreamEndCapture(h->st, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc;
    }
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(SFWI_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
    }
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(SFWI_E_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    return SFWI_OK;
}

// Wait for the run, check the device error flag, read the per-trace misfits
// back and sum them per shot (in shot and trace order) into per_shot[] and
// *misfit (added).
int collect_misfit(sfwi_handle *h, int misfit_kind, double *misfit, double *per_shot, bool backward) {
    Batch &b = h->b;
    cudaStream_t st = h->st;
    std::vector<double> tm(2 * (size_t)b.ntr_tot);
    const size_t nm = misfit_kind == SFWI_MISFIT_L2 ? b.ntr_tot : 2 * (size_t)b.ntr_tot;
    if (nm) CK(cudaMemcpyAsync(tm.data(), b.tmis.p, nm * sizeof(double), cudaMemcpyDeviceToHost, st));
    int derr = 0;
    CK(cudaMemcpyAsync(&derr, b.derr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (derr) return fail(SFWI_E_CUDA, "a device-side pipeline wait timed out (code %d)", derr);
    cudaEventElapsedTime(&h->fwd_ms, h->ev[0], h->ev[1]);
    if (backward) {
        cudaEventElapsedTime(&h->other_ms, h->ev[1], h->ev[2]);
        cudaEventElapsedTime(&h->bwd_ms, h->ev[2], h->ev[3]);
    } else {
        h->other_ms = h->bwd_ms = 0.f;
    }
    cudaEventElapsedTime(&h->total_ms, h->ev[4], h->ev[5]);
    double total = 0.0;
    for (int s = 0; s < b.nshots; s++) {
        double ms = 0.0;
        const ShotGeo &g = b.geo[s];
        for (int t = 0; t < g.ntr; t++) {
            if (misfit_kind == SFWI_MISFIT_L2)
                ms += tm[g.tr0 + t];
            else
                ms += tm[2 * (size_t)(g.tr0 + t)] + tm[2 * (size_t)(g.tr0 + t) + 1];
        }
        if (per_shot) per_shot[s] = ms;
        total += ms;
    }
    if (misfit) *misfit += total;
    return SFWI_OK;
}

int finish_misfit(sfwi_handle *h, int misfit_kind, double *misfit, double *per_shot) {
    h->launches++;
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev[5], h->st));
    return collect_misfit(h, misfit_kind, misfit, per_shot, false);
}

// what a run computes: a shot-gradient pass, the forward records only, or
// the forward records with the residual and misfit (line searches)
enum RunMode { RUN_GRADIENT, RUN_FORWARD, RUN_MISFIT };

int run_batch(sfwi_handle *h, const std::vector<ShotIn> &shots, int mode, double *misfit, double *per_shot) {
    if (!h->have_model && h->models.empty()) return fail(SFWI_E_STATE, "no model: call sfwi_gpu_buffer_vpvs first");
    if (shots.empty()) return fail(SFWI_E_ARG, "no shots queued");
    const bool forward_only = mode != RUN_GRADIENT;
    const int misfit_kind = h->force_l2 ? SFWI_MISFIT_L2 : h->misfit_kind;
    h->last_forward_only = forward_only;
    CK(cudaSetDevice(h->device));
    // NVTX ranges mark the host side of each phase for timeline profilers
    struct NvtxRange {
        explicit NvtxRange(const char *n) { nvtxRangePushA(n); }
        ~NvtxRange() { nvtxRangePop(); }
    } nvtx_run("sfwi run_batch");
    if (h->tile_auto) pick_tile_shape(h, shots);
    h->b.ready = false;  // until this batch is on the device
    int rc = build_batch(h, shots);
    if (rc) return rc;
    if (!h->b.tlen.empty() && ((mode != RUN_FORWARD && misfit_kind != SFWI_MISFIT_L2) || h->snap_every > 0))
        return fail(SFWI_E_ARG, "shots of different lengths in one run take the L2 misfit and no snapshots");
    ObservedGuard obs_guard{h};
    rc = upload_batch(h, shots, forward_only, mode != RUN_FORWARD);
    if (rc) return rc;
    Batch &b = h->b;
    b.ready = true;
    const Params p = make_params(h, forward_only);
    const int nt = h->nt;
    cudaStream_t st = h->st;
    std::vector<long long> sig = shape_signature(h, forward_only);
    if (h->use_graphs && sig != b.gsig) {
        b.drop_graphs();
        rc = capture(h, &b.gfwd, true, p, forward_only);
        if (rc) return rc;
        if (!forward_only) {
            rc = capture(h, &b.gbwd, false, p, false);
            if (rc) return rc;
        }
        b.gsig = sig;
    }
    nvtxMarkA("sfwi forward sweeps");
    CK(cudaEventRecord(h->ev[0], st));
    if (h->use_graphs)
        CK(cudaGraphLaunch(b.gfwd, st));
    else if ((rc = enqueue_forward(h, p, forward_only)))
        return rc;
    h->launches += 2LL * nt;
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev[1], st));
    // receiver-row records to trace-major records
    if (b.ntr_tot) {
        launch_record_gather(b.rrow.p, b.dtrow.p, b.tlen.empty() ? nullptr : b.dtlen.p, nt, h->stage == 2 ? 4 : 2,
                             b.X, b.ntr_tot, b.r(R_SYN_Z, nt), (size_t)b.ntr_tot * nt, st);
        h->launches++;
    }
    CK(cudaGetLastError());
    if (mode == RUN_FORWARD) {
        CK(cudaEventRecord(h->ev[5], st));
        int derr = 0;
        CK(cudaMemcpyAsync(&derr, b.derr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (derr) return fail(SFWI_E_CUDA, "a device-side pipeline wait timed out (code %d)", derr);
        cudaEventElapsedTime(&h->fwd_ms, h->ev[0], h->ev[1]);
        cudaEventElapsedTime(&h->total_ms, h->ev[4], h->ev[5]);
        h->bwd_ms = 0.f;
        h->other_ms = 0.f;
        return SFWI_OK;
    }
    // adjoint source and misfit, once the observed records are in
    nvtxMarkA("sfwi misfit");
    if ((rc = wait_observed(h))) return rc;
    // OT scales: max|obs| per trace and component, floored at a fraction of
    // the shot's largest (a trace without signal must not blow the transform
    // up), or the shot's largest for every trace
    if (misfit_kind != SFWI_MISFIT_L2 && b.ntr_tot) {
        launch_ot_scales(b.r(R_OBS_Z, nt), b.r(R_OBS_X, nt), nt, b.ntr_tot, b.dgeo.p, b.nshots,
                         h->misfit_kind == SFWI_MISFIT_OT_ALLTRACE, b.dsigma.p, st);
        h->launches += 2;
    }
    if (misfit_kind == SFWI_MISFIT_L2) {
        launch_residual_l2(h->stage, nt, b.ntr_tot, b.r(R_SYN_Z, nt), b.r(R_SYN_X, nt), b.r(R_SYN2_Z, nt),
                           b.r(R_SYN2_X, nt), b.r(R_OBS_Z, nt), b.r(R_OBS_X, nt), b.r(R_RES_Z, nt), b.r(R_RES_X, nt),
                           b.tmis.p, st);
    } else {
        OtArgs o{};
        o.kind = misfit_kind;
        o.nt = nt;
        o.ntr = b.ntr_tot;
        o.stage = h->stage;
        o.dt = h->dt;
        o.cal_z = b.r(R_SYN_Z, nt);
        o.cal_x = b.r(R_SYN_X, nt);
        o.cal2_z = h->stage == 2 ? b.r(R_SYN2_Z, nt) : nullptr;
        o.cal2_x = h->stage == 2 ? b.r(R_SYN2_X, nt) : nullptr;
        o.obs_z = b.r(R_OBS_Z, nt);
        o.obs_x = b.r(R_OBS_X, nt);
        o.res_z = b.r(R_RES_Z, nt);
        o.res_x = b.r(R_RES_X, nt);
        o.sigma = b.dsigma.p;
        o.trace_misfit = b.tmis.p;
        if (const size_t nscr = ot_scratch_doubles(nt, b.ntr_tot)) {
            CK(b.otscr.ensure(nscr));
            o.scratch = b.otscr.p;
        }
        CK(launch_ot(o, st));
    }
    if (mode == RUN_MISFIT) return finish_misfit(h, misfit_kind, misfit, per_shot);
    // the adjoint sources per packed row, time-major, for the backward sweeps
    launch_recv_source(b.r(R_RES_Z, nt), b.r(R_RES_X, nt), b.drtr.p, nt, b.X, b.rsp, b.rsrc.p, st);
    h->launches++;
    h->launches++;
    CK(cudaGetLastError());
    nvtxMarkA("sfwi backward sweeps");
    CK(cudaEventRecord(h->ev[2], st));
    if (h->use_graphs)
        CK(cudaGraphLaunch(b.gbwd, st));
    else if ((rc = enqueue_backward(h, p)))
        return rc;
    h->launches += 2LL * nt;
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev[3], st));
    FinalArgs fa{};
    fa.allnx = h->allnx;
    fa.allnz = h->allnz;
    fa.P = b.P;
    fa.pml = h->pml;
    fa.nshots = b.nshots;
    fa.geo = b.dgeo.p;
    fa.glam = b.g(G_LAM);
    fa.gmu = b.g(G_MU);
    fa.illum = b.g(G_ILL);
    fa.vp = b.g(C_VP);
    fa.vs = b.g(C_VS);
    fa.rho = b.g(C_RHO);
    fa.gpp = h->gpp.p;
    fa.gps = h->gps.p;
    fa.gil = h->gil.p;
    fa.grho = h->want_rho ? b.g(G_RHO) : nullptr;
    fa.grh = h->grh.p;
    if (h->models.empty()) {
        launch_finalize(fa, st);
        h->launches++;
    } else {
        // several models: each model's shots (consecutive in the batch) into
        // that model's own gradients, zeroed before the run
        const size_t mc = h->mcells;
        for (int s0 = 0; s0 < b.nshots;) {
            const int m = shots[s0].req;
            int s1 = s0 + 1;
            while (s1 < b.nshots && shots[s1].req == m) s1++;
            const sfwi_handle::ModelIn &mi = h->models[m];
            FinalArgs f = fa;
            f.allnx = mi.allnx;
            f.allnz = mi.allnz;
            f.nshots = s1 - s0;
            f.geo = b.dgeo.p + s0;
            f.gpp = h->mgrad.p + mi.off;
            f.gps = h->mgrad.p + mc + mi.off;
            f.gil = h->mgrad.p + 2 * mc + mi.off;
            f.grh = h->mgrad.p + 3 * mc + mi.off;
            launch_finalize(f, st);
            h->launches++;
            s0 = s1;
        }
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev[5], st));
    return collect_misfit(h, misfit_kind, misfit, per_shot, true);
}

// every device buffer of a handle
template <class F>
void for_each_buf(sfwi_handle *h, F f) {
    Batch &b = h->b;
    f(b.grid), f(b.tb), f(b.lr), f(b.rrow), f(b.rsrc), f(b.recs), f(b.tmis), f(b.dsigma), f(b.dgeo), f(b.dtiles);
    f(b.dtrow), f(b.drtr), f(b.derr), f(b.dctr), f(b.snap), f(b.sscale), f(b.otscr);
    f(h->sou), f(h->vp_all), f(h->vs_all), f(h->rho_all), f(h->dvp_all), f(h->dvs_all);
    f(h->gpp), f(h->gps), f(h->gil), f(h->grh), f(h->ls_buf);
    f(h->mvp), f(h->mvs), f(h->mrho), f(h->mdvp), f(h->mdvs), f(h->mgrad);
    f(h->adj_f), f(h->adj_d), f(h->adj_img), f(h->adj_i), f(b.daux), f(b.dtlen);
}

int check(sfwi_handle *h) {
    if (!h) return fail(SFWI_E_ARG, "null handle");
    return SFWI_OK;
}

// the shot described by the reference-shaped per-shot calls
int current_shot(sfwi_handle *h, ShotIn &s) {
    if (!h->have_geom || !h->have_rec) return fail(SFWI_E_STATE, "shot geometry and records must be set first");
    s.nx = h->nxpml - 2 * h->pml;
    // the window is the one bufferVpVsHtoD cut; the gradient lands at delta_left + record_left_in_v
    s.win0 = h->delta_left + h->record_left_in_v;
    if (s.win0 != h->ngx_min)
        return fail(SFWI_E_ARG, "bufferVpVsHtoD(%d) and delta_left+record_left_in_v=%d differ", h->ngx_min, s.win0);
    s.isx = h->isx;
    s.isz = h->isz;
    s.igz = h->igz;
    s.ngx_left = h->ngx_left;
    s.ntr = h->ntr;
    s.gc = h->gc;
    s.obs_z = h->rec_z.data();
    s.obs_x = h->rec_x.data();
    return SFWI_OK;
}

// Stage-1 parabola line search over shots q: the misfit of every shot at the
// trial models m - step_k g, k = 0, 1, 2 (steps 0, step1, step2), all shots and
// all three models advancing in the same forward launches.
int line_search_parabola(sfwi_handle *h, const std::vector<ShotIn> &q, const float *grad_pp, const float *grad_ps,
                         float step1, float step2, double m[3], double *per_shot) {
    if (h->stage != 1) return fail(SFWI_E_STATE, "the parabola line search belongs to stage 1");
    if (!grad_pp || !grad_ps) return fail(SFWI_E_ARG, "null search direction");
    if (q.empty()) return fail(SFWI_E_ARG, "no shots queued");
    if (!h->have_model) return fail(SFWI_E_STATE, "no model: call sfwi_gpu_buffer_vpvs first");
    const size_t n = (size_t)h->allnx * h->allnz;
    const int ns = (int)q.size();
    CK(cudaSetDevice(h->device));
    CK(h->ls_buf.ensure(8 * n + 4));
    float *gpp = h->ls_buf.p, *gps = gpp + n, *vps = gps + n, *vss = vps + 3 * n, *steps = vss + 3 * n;
    const float st3[3] = {0.f, step1, step2};
    CK(cudaMemcpyAsync(gpp, grad_pp, n * sizeof(float), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(gps, grad_ps, n * sizeof(float), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(steps, st3, sizeof st3, cudaMemcpyHostToDevice, h->st));
    launch_trial_models(h->vp_all.p, gpp, steps, 3, n, vps, h->st);
    launch_trial_models(h->vs_all.p, gps, steps, 3, n, vss, h->st);
    h->launches += 2;
    CK(cudaGetLastError());
    std::vector<ShotIn> all;
    for (int k = 0; k < 3; k++)
        for (const ShotIn &s : q) {
            all.push_back(s);
            all.back().model = k;
        }
    std::vector<double> per(3 * (size_t)ns);
    h->slot_vp = vps;
    h->slot_vs = vss;
    const int rc = run_batch(h, all, RUN_MISFIT, nullptr, per.data());
    h->slot_vp = h->slot_vs = nullptr;
    if (rc) return rc;
    for (int k = 0; k < 3; k++)
        for (int s = 0; s < ns; s++) {
            m[k] += per[(size_t)k * ns + s];
            if (per_shot) per_shot[(size_t)s * 3 + k] = per[(size_t)k * ns + s];
        }
    return SFWI_OK;
}

// Stage-2 exact step length over shots q: a Born run with the model
// perturbation `image` gives the residual r = (du - d) + u0, a Born run with
// the search direction `cg` gives its scattered records q; fenzi += sum q.r,
// fenmu += sum q.q (alpha = fenzi / fenmu).  Both runs of every shot advance
// in the same forward launches.
int line_search_exact(sfwi_handle *h, const std::vector<ShotIn> &q, const float *image_pp, const float *image_ps,
                      const float *cg_pp, const float *cg_ps, double *fenzi, double *fenmu, double *per_shot) {
    if (h->stage != 2) return fail(SFWI_E_STATE, "the exact line search belongs to stage 2");
    if (!image_pp || !image_ps || !cg_pp || !cg_ps) return fail(SFWI_E_ARG, "null model perturbation");
    if (q.empty()) return fail(SFWI_E_ARG, "no shots queued");
    if (!h->have_model) return fail(SFWI_E_STATE, "no model: call sfwi_gpu_buffer_vpvs first");
    const size_t n = (size_t)h->allnx * h->allnz;
    const int ns = (int)q.size();
    CK(cudaSetDevice(h->device));
    CK(h->ls_buf.ensure(4 * n));
    float *dvp = h->ls_buf.p, *dvs = dvp + 2 * n;
    CK(cudaMemcpyAsync(dvp, image_pp, n * sizeof(float), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(dvp + n, cg_pp, n * sizeof(float), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(dvs, image_ps, n * sizeof(float), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(dvs + n, cg_ps, n * sizeof(float), cudaMemcpyHostToDevice, h->st));
    std::vector<ShotIn> all;
    for (int k = 0; k < 2; k++)
        for (const ShotIn &s : q) {
            all.push_back(s);
            all.back().model = k;
        }
    h->slot_dvp = dvp;
    h->slot_dvs = dvs;
    h->force_l2 = true;
    int rc = run_batch(h, all, RUN_MISFIT, nullptr, nullptr);
    h->slot_dvp = h->slot_dvs = nullptr;
    h->force_l2 = false;
    if (rc) return rc;
    Batch &b = h->b;
    const int nt = h->nt, T = b.ntr_tot / 2;
    const size_t off = (size_t)T * nt;
    launch_trace_dots(b.r(R_SYN_Z, nt) + off, b.r(R_SYN_X, nt) + off, b.r(R_RES_Z, nt), b.r(R_RES_X, nt), nt, T,
                      b.tmis.p, b.tmis.p + T, h->st);
    h->launches++;
    CK(cudaGetLastError());
    std::vector<double> d(2 * (size_t)T);
    if (T) CK(cudaMemcpyAsync(d.data(), b.tmis.p, 2 * (size_t)T * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (int s = 0; s < ns; s++) {
        const ShotGeo &g = b.geo[s];
        double zi = 0.0, mu = 0.0;
        for (int t = 0; t < g.ntr; t++) {
            zi += d[g.tr0 + t];
            mu += d[T + g.tr0 + t];
        }
        *fenzi += zi;
        *fenmu += mu;
        if (per_shot) {
            per_shot[2 * (size_t)s] = zi;
            per_shot[2 * (size_t)s + 1] = mu;
        }
    }
    return SFWI_OK;
}

// The exact adjoint of the stage-2 Born modelling operator over shots q, the
// queued shots' records being the data d: img_vp, img_vs += L^T d.  The
// background forward runs first and keeps its velocity after every step's
// velocity sweep (FP32 snapshots, the fields the Born source differentiates);
// then the transposed sweeps run from the last step to the first
// (sfwi_adjoint.cu) and the window accumulators are folded into the model.
int born_adjoint(sfwi_handle *h, const std::vector<ShotIn> &q, double *img_vp, double *img_vs) {
    if (h->stage != 2) return fail(SFWI_E_STATE, "the Born operator belongs to stage 2");
    if (!h->have_model) return fail(SFWI_E_STATE, "no model: call sfwi_gpu_buffer_vpvs first");
    if (q.empty()) return fail(SFWI_E_ARG, "no shots queued");
    if (!img_vp || !img_vs) return fail(SFWI_E_ARG, "null output");
    CK(cudaSetDevice(h->device));
    const int snap_every = h->snap_every, snap_fmt = h->snap_fmt, misfit_kind = h->misfit_kind;
    const bool want_rho = h->want_rho;
    h->snap_every = 1;
    h->snap_fmt = SNAP_F32;
    h->want_rho = false;
    h->misfit_kind = SFWI_MISFIT_L2;
    struct Restore {
        sfwi_handle *h;
        int se, sf, mk;
        bool wr;
        ~Restore() {
            h->snap_every = se;
            h->snap_fmt = sf;
            h->misfit_kind = mk;
            h->want_rho = wr;
        }
    } restore{h, snap_every, snap_fmt, misfit_kind, want_rho};
    if (h->tile_auto) pick_tile_shape(h, q);
    h->b.ready = false;
    h->last_perm.clear();
    if (int rc = build_batch(h, q)) return rc;
    ObservedGuard obs_guard{h};
    if (int rc = upload_batch(h, q, false, true)) return rc;
    Batch &b = h->b;
    b.ready = true;
    const Params p = make_params(h, false);
    const int nt = h->nt;
    cudaStream_t st = h->st;
    // the strains of the Born source reach the outer rows and columns of a
    // shot, which no tile stores: they must read as the zeros they are
    CK(cudaMemsetAsync(b.snap.p, 0, (size_t)b.nsnap * 2 * b.X * b.PS * sizeof(float), st));
    // the background forward with its snapshots (no scattered field)
    CK(cudaEventRecord(h->ev[0], st));
    for (int it = 0; it < nt; it++) {
        h->tv->launch(0, p, b.tm, it, false, 1.f, st);
        h->tv->launch(1, p, b.tm, it, false, 1.f, st);
    }
    h->launches += 2LL * nt;
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev[1], st));
    // adjoint workspace: 18 float fields, 2 double accumulators, tables
    const size_t cells = b.cells, gcells = (size_t)h->allnx * h->allnz;
    CK(h->adj_f.ensure(18 * cells));
    CK(h->adj_d.ensure(2 * cells));
    CK(h->adj_img.ensure(2 * gcells));
    CK(cudaMemsetAsync(h->adj_f.p, 0, 18 * cells * sizeof(float), st));
    CK(cudaMemsetAsync(h->adj_d.p, 0, 2 * cells * sizeof(double), st));
    CK(cudaMemsetAsync(h->adj_img.p, 0, 2 * gcells * sizeof(double), st));
    // per packed row: its shot, and the traces recorded at its receiver cell
    std::vector<int> tab(b.X + (b.X + 1) + std::max(b.ntr_tot, 1), 0);
    int *rowshot = tab.data(), *rstart = rowshot + b.X, *rtr = rstart + b.X + 1;
    for (int s2 = 0; s2 < b.nshots; s2++)
        for (int r = 0; r < b.geo[s2].nxpml; r++) rowshot[b.geo[s2].row0 + r] = s2;
    std::vector<int> cnt(b.X, 0);
    for (int t = 0; t < b.ntr_tot; t++)
        if (b.trow[t] >= 0) cnt[b.trow[t]]++;
    for (int r = 0; r < b.X; r++) rstart[r + 1] = rstart[r] + cnt[r];
    std::vector<int> fill(rstart, rstart + b.X);
    for (int t = 0; t < b.ntr_tot; t++)
        if (b.trow[t] >= 0) rtr[fill[b.trow[t]]++] = t;
    CK(h->adj_i.ensure(tab.size()));
    CK(cudaMemcpyAsync(h->adj_i.p, tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    AdjArgs a{};
    a.X = b.X;
    a.P = b.P;
    a.PS = b.PS;
    a.pml = h->pml;
    a.nt = nt;
    a.born_lo = NOP;
    a.dt = h->dt;
    a.dtdx = h->dt / h->dx;
    a.dtdz = h->dt / h->dz;
    a.idx = 1.0f / h->dx;
    a.idz = 1.0f / h->dz;
    a.geo = b.dgeo.p;
    a.rowshot = h->adj_i.p;
    a.rstart = h->adj_i.p + b.X;
    a.rtr = h->adj_i.p + 2 * b.X + 1;
    a.ib = b.g(C_IB);
    a.lam = b.g(C_LAM);
    a.mu = b.g(C_MU);
    a.dampx = b.g(C_DX);
    a.dampz = b.g(C_DZ);
    float *w = h->adj_f.p;
    float **fields[18] = {&a.avx, &a.avz, &a.amx, &a.amz, &a.atxx, &a.atzz, &a.atxz, &a.amxx, &a.amzz,
                          &a.amxz, &a.gax, &a.gbz, &a.gcz, &a.gdx, &a.hax, &a.hbz, &a.hdx, &a.hcz};
    for (int k = 0; k < 18; k++) *fields[k] = w + (size_t)k * cells;
    a.dbp = h->adj_d.p;
    a.dbs = h->adj_d.p + cells;
    a.snap = reinterpret_cast<const float *>(b.snap.p);
    a.dz = b.r(R_OBS_Z, nt);
    a.dx = b.r(R_OBS_X, nt);
    if (int rc = wait_observed(h)) return rc;  // the records to back-propagate
    CK(cudaEventRecord(h->ev[2], st));
    for (int it = nt - 1; it >= 0; it--) launch_adjoint_step(a, it, st);
    h->launches += 3LL * nt;
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev[3], st));
    ImageArgs im{};
    im.allnx = h->allnx;
    im.allnz = h->allnz;
    im.P = b.P;
    im.pml = h->pml;
    im.nshots = b.nshots;
    im.geo = b.dgeo.p;
    im.dbp = a.dbp;
    im.dbs = a.dbs;
    im.vp = b.g(C_VP);
    im.vs = b.g(C_VS);
    im.rho = b.g(C_RHO);
    im.img_vp = h->adj_img.p;
    im.img_vs = h->adj_img.p + gcells;
    launch_born_image(im, st);
    h->launches++;
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev[5], st));
    std::vector<double> out(2 * gcells);
    CK(cudaMemcpyAsync(out.data(), h->adj_img.p, 2 * gcells * sizeof(double), cudaMemcpyDeviceToHost, st));
    int derr = 0;
    CK(cudaMemcpyAsync(&derr, b.derr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (derr) return fail(SFWI_E_CUDA, "a device-side pipeline wait timed out (code %d)", derr);
    cudaEventElapsedTime(&h->fwd_ms, h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&h->bwd_ms, h->ev[2], h->ev[3]);
    cudaEventElapsedTime(&h->total_ms, h->ev[4], h->ev[5]);
    h->other_ms = 0.f;
    for (size_t i = 0; i < gcells; i++) {
        img_vp[i] += out[i];
        img_vs[i] += out[gcells + i];
    }
    return SFWI_OK;
}

int ensure_grads(sfwi_handle *h) {
    const size_t n = (size_t)h->allnx * h->allnz;
    if (h->gpp.p) return SFWI_OK;
    CK(h->gpp.ensure(n));
    CK(h->gps.ensure(n));
    CK(h->gil.ensure(n));
    CK(h->grh.ensure(n));
    CK(cudaMemsetAsync(h->gpp.p, 0, n * sizeof(double), h->st));
    CK(cudaMemsetAsync(h->gps.p, 0, n * sizeof(double), h->st));
    CK(cudaMemsetAsync(h->gil.p, 0, n * sizeof(double), h->st));
    CK(cudaMemsetAsync(h->grh.p, 0, n * sizeof(double), h->st));
    return SFWI_OK;
}

int upload_model(DevBuf<float> &d, const float *src, size_t n) {
    CK(d.ensure(n));
    CK(cudaMemcpyAsync(d.p, src, n * sizeof(float), cudaMemcpyHostToDevice, d.st));
    CK(cudaStreamSynchronize(d.st));
    return SFWI_OK;
}

int ot_host(int kind, const float *obs_x, const float *obs_z, const float *cal_x, const float *cal_z, float *res_x,
            float *res_z, int length, int tracenum, float dt, double *misfit) {
    if (!obs_x || !obs_z || !cal_x || !cal_z || !res_x || !res_z || !misfit || length < 1 || tracenum < 0)
        return fail(SFWI_E_ARG, "sfwi_ot: bad argument");
    if (tracenum == 0) return SFWI_OK;
    const size_t n = (size_t)length * tracenum;
    float *d = nullptr;
    double *dd = nullptr;
    CK(cudaMalloc(&d, 6 * n * sizeof(float)));
    // traces too long for shared memory work in global scratch after the sums
    const size_t nscr = ot_scratch_doubles(length, tracenum);
    cudaError_t e = cudaMalloc(&dd, (4 * (size_t)tracenum + nscr) * sizeof(double));
    if (e != cudaSuccess) {
        cudaFree(d);
        return fail(SFWI_E_NOMEM, "sfwi_ot: %s", cudaGetErrorString(e));
    }
    std::vector<double> sig(2 * (size_t)tracenum);
    double gz = 0, gx = 0;
    for (int t = 0; t < tracenum; t++) {
        double mz = 0, mx = 0;
        for (int k = 0; k < length; k++) {
            mz = std::max(mz, (double)std::fabs(obs_z[(size_t)t * length + k]));
            mx = std::max(mx, (double)std::fabs(obs_x[(size_t)t * length + k]));
        }
        sig[2 * t] = mz;
        sig[2 * t + 1] = mx;
        gz = std::max(gz, mz);
        gx = std::max(gx, mx);
    }
    for (int t = 0; t < tracenum; t++) {
        const bool all = kind == SFWI_MISFIT_OT_ALLTRACE;
        sig[2 * t] = all ? gz : std::max(sig[2 * t], kOtSigmaFloor * gz);
        sig[2 * t + 1] = all ? gx : std::max(sig[2 * t + 1], kOtSigmaFloor * gx);
    }
    int rc = SFWI_OK;
    std::vector<double> tm(2 * (size_t)tracenum);
    do {
        if ((e = cudaMemcpy(d, obs_z, n * 4, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((e = cudaMemcpy(d + n, obs_x, n * 4, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((e = cudaMemcpy(d + 2 * n, cal_z, n * 4, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((e = cudaMemcpy(d + 3 * n, cal_x, n * 4, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((e = cudaMemcpy(dd, sig.data(), sig.size() * 8, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        OtArgs o{};
        o.kind = kind;
        o.nt = length;
        o.ntr = tracenum;
        o.stage = 1;
        o.dt = dt;
        o.obs_z = d;
        o.obs_x = d + n;
        o.cal_z = d + 2 * n;
        o.cal_x = d + 3 * n;
        o.res_z = d + 4 * n;
        o.res_x = d + 5 * n;
        o.sigma = dd;
        o.trace_misfit = dd + 2 * tracenum;
        o.scratch = nscr ? dd + 4 * (size_t)tracenum : nullptr;
        if ((e = launch_ot(o, 0)) != cudaSuccess) break;
        if ((e = cudaMemcpy(res_z, d + 4 * n, n * 4, cudaMemcpyDeviceToHost)) != cudaSuccess) break;
        if ((e = cudaMemcpy(res_x, d + 5 * n, n * 4, cudaMemcpyDeviceToHost)) != cudaSuccess) break;
        if ((e = cudaMemcpy(tm.data(), dd + 2 * tracenum, tm.size() * 8, cudaMemcpyDeviceToHost)) != cudaSuccess) break;
    } while (0);
    cudaFree(d);
    cudaFree(dd);
    if (e != cudaSuccess) return fail(SFWI_E_CUDA, "sfwi_ot: %s", cudaGetErrorString(e));
    double w = 0;
    for (double v : tm) w += v;
    *misfit += w;
    return rc;
}

}  // namespace

namespace sfwi {
int record_error(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}
}  // namespace sfwi

extern "C" {

const char *sfwi_last_error(void) { return g_err.c_str(); }
const char *sfwi_version(void) { return "sfwi_gb300 0.1 (sm_103a)"; }

int sfwi_create(sfwi_handle **out, int stage, const float *sou, float dx, float dz, float dt, int nxpml, int nzpml,
                int allnx, int allnz, int scale, int pml, int nt, int nop, int ntr) {
    if (!out) return fail(SFWI_E_ARG, "out is null");
    *out = nullptr;
    if (stage != 1 && stage != 2) return fail(SFWI_E_ARG, "stage must be 1 or 2");
    if (nop != NOP) return fail(SFWI_E_ARG, "nop must be %d (8th-order stencil)", NOP);
    if (!sou || nt < 1 || dx <= 0 || dz <= 0 || dt <= 0 || pml < 2 * NOP || allnx < 1 || allnz < 1 || ntr < 0)
        return fail(SFWI_E_ARG, "bad size or spacing");
    if (nzpml != allnz + 2 * pml) return fail(SFWI_E_ARG, "nzpml must be allnz + 2*pml");
    if (nxpml < 2 * pml + 1) return fail(SFWI_E_ARG, "nxpml must exceed 2*pml");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(SFWI_E_NODEVICE, "no CUDA device");
    sfwi_handle *h = new sfwi_handle();
    h->stage = stage;
    h->dx = dx;
    h->dz = dz;
    h->dt = dt;
    h->nxpml = nxpml;
    h->nzpml = nzpml;
    h->allnx = allnx;
    h->allnz = allnz;
    h->scale = scale;
    h->pml = pml;
    h->nt = nt;
    h->nop = nop;
    h->ntr = ntr;
    cudaGetDevice(&h->device);
    cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device);
    int rc = SFWI_OK;
    do {
        cudaError_t e = cudaSuccess;
        h->tv = tile_variant(SFWI_TILE_16x32);
        for (int v = 0; v < SFWI_NUM_TILE_SHAPES && e == cudaSuccess; v++) e = tile_variant(v)->configure();
        if (e != cudaSuccess) {
            rc = fail(SFWI_E_CUDA, "kernel attributes: %s", cudaGetErrorString(e));
            break;
        }
        if ((e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking)) != cudaSuccess) {
            rc = fail(SFWI_E_CUDA, "stream: %s", cudaGetErrorString(e));
            break;
        }
        for_each_buf(h, [h](auto &d) { d.st = h->st; });
        for (auto &ev : h->ev)
            if ((e = cudaEventCreate(&ev)) != cudaSuccess) {
                rc = fail(SFWI_E_CUDA, "event: %s", cudaGetErrorString(e));
                break;
            }
        if (rc) break;
        if ((e = cudaStreamCreateWithFlags(&h->os, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&h->ev_obs_fork, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&h->ev_obs, cudaEventDisableTiming)) != cudaSuccess) {
            rc = fail(SFWI_E_CUDA, "records stream: %s", cudaGetErrorString(e));
            break;
        }
        if ((rc = upload_model(h->sou, sou, nt))) break;
        rc = ensure_grads(h);
    } while (0);
    if (rc) {
        sfwi_destroy(h);
        return rc;
    }
    *out = h;
    return SFWI_OK;
}

int sfwi_destroy(sfwi_handle *h) {
    if (!h) return SFWI_OK;
    cudaSetDevice(h->device);
    if (h->st) cudaStreamSynchronize(h->st);
    h->b.drop_graphs();
    for_each_buf(h, [](auto &d) { d.release(); });
    if (h->st) cudaStreamSynchronize(h->st);  // the stream-ordered frees
    if (h->cs) cudaStreamSynchronize(h->cs);
    if (h->os) cudaStreamSynchronize(h->os);
    h->htb.release();
    h->hlr.release();
    for (auto &ev : h->ev)
        if (ev) cudaEventDestroy(ev);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    for (auto &ev : h->ev_copy)
        if (ev) cudaEventDestroy(ev);
    if (h->cs) cudaStreamDestroy(h->cs);
    if (h->ev_obs_fork) cudaEventDestroy(h->ev_obs_fork);
    if (h->ev_obs) cudaEventDestroy(h->ev_obs);
    if (h->os) cudaStreamDestroy(h->os);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
    return SFWI_OK;
}

int sfwi_gpu_buffer_vpvs(sfwi_handle *h, const float *vp_all, const float *vs_all, const float *rho_all) {
    if (int rc = check(h)) return rc;
    if (!vp_all || !vs_all) return fail(SFWI_E_ARG, "vp/vs null");
    if (h->stage == 1 && !rho_all) return fail(SFWI_E_ARG, "stage 1 needs rho_all");
    const size_t n = (size_t)h->allnx * h->allnz;
    int rc;
    if ((rc = upload_model(h->vp_all, vp_all, n))) return rc;
    if ((rc = upload_model(h->vs_all, vs_all, n))) return rc;
    h->have_rho = false;
    if (rho_all) {
        if ((rc = upload_model(h->rho_all, rho_all, n))) return rc;
        h->have_rho = true;
    }
    h->have_model = true;
    return SFWI_OK;
}

int sfwi_gpu_buffer_m(sfwi_handle *h, const float *dvp_all, const float *dvs_all) {
    if (int rc = check(h)) return rc;
    if (!dvp_all || !dvs_all) return fail(SFWI_E_ARG, "dvp/dvs null");
    const size_t n = (size_t)h->allnx * h->allnz;
    int rc;
    if ((rc = upload_model(h->dvp_all, dvp_all, n))) return rc;
    if ((rc = upload_model(h->dvs_all, dvs_all, n))) return rc;
    h->have_m = true;
    return SFWI_OK;
}

int sfwi_buffer_vpvs_htod(sfwi_handle *h, int ngx_min) {
    if (int rc = check(h)) return rc;
    const int nx = h->nxpml - 2 * h->pml;
    if (ngx_min < 0 || ngx_min + nx > h->allnx)
        return fail(SFWI_E_ARG, "window [%d, %d) outside the model width %d", ngx_min, ngx_min + nx, h->allnx);
    h->ngx_min = ngx_min;
    return SFWI_OK;
}

int sfwi_record_copy_to_gpu(sfwi_handle *h, const float *rec_z, const float *rec_x, const int *gc) {
    if (int rc = check(h)) return rc;
    if ((!rec_z || !rec_x || !gc) && h->ntr > 0) return fail(SFWI_E_ARG, "null record or coordinates");
    const size_t n = (size_t)h->ntr * h->nt;
    h->rec_z.assign(rec_z, rec_z + n);
    h->rec_x.assign(rec_x, rec_x + n);
    h->gc.assign(gc, gc + h->ntr);
    h->have_rec = true;
    return SFWI_OK;
}

int sfwi_set_shot_geometry(sfwi_handle *h, int isx, int isz, int igz, int ngx_left, int delta_left,
                           int record_left_in_v, int ntr) {
    if (int rc = check(h)) return rc;
    if (ntr < 0) return fail(SFWI_E_ARG, "ntr < 0");
    if (ntr != h->ntr) h->have_rec = false;  // the records must be copied again for a new trace count
    h->isx = isx;
    h->isz = isz;
    h->igz = igz;
    h->ngx_left = ngx_left;
    h->delta_left = delta_left;
    h->record_left_in_v = record_left_in_v;
    h->ntr = ntr;
    h->have_geom = true;
    return SFWI_OK;
}

int sfwi_set_misfit(sfwi_handle *h, int kind) {
    if (int rc = check(h)) return rc;
    if (kind < SFWI_MISFIT_L2 || kind > SFWI_MISFIT_OT_ALLTRACE) return fail(SFWI_E_ARG, "unknown misfit %d", kind);
    h->misfit_kind = kind;
    return SFWI_OK;
}

int sfwi_set_density_gradient(sfwi_handle *h, int on) {
    if (int rc = check(h)) return rc;
    if (on && h->snap_every > 0) return fail(SFWI_E_STATE, "the density kernel needs the reconstruction (snapshots on)");
    h->want_rho = on != 0;
    return SFWI_OK;
}

int sfwi_set_snapshots(sfwi_handle *h, int every, int format) {
    if (int rc = check(h)) return rc;
    if (every < 0 || (every > 0 && (format < SFWI_SNAP_F32 || format > SFWI_SNAP_BF16)))
        return fail(SFWI_E_ARG, "snapshots: interval %d, format %d", every, format);
    if (every > 0 && h->want_rho) return fail(SFWI_E_STATE, "the density kernel needs the reconstruction");
    h->snap_every = every;
    h->snap_fmt = every > 0 ? format : SNAP_OFF;
    return SFWI_OK;
}

int sfwi_set_cpu_mem(sfwi_handle *h, int cpu_mem, int ntt) {
    if (int rc = check(h)) return rc;
    if (cpu_mem && ntt < 1) return fail(SFWI_E_ARG, "ntt must be at least 1 step when cpu_mem is set (got %d)", ntt);
    h->cpu_mem = cpu_mem ? 1 : 0;
    h->ntt = cpu_mem ? ntt : 0;
    return SFWI_OK;
}

int sfwi_set_pinned_cache(size_t bytes) {
    PinnedCache &c = pinned_cache();
    {
        std::lock_guard<std::mutex> g(c.mu);
        c.limit = bytes;
    }
    c.trim(bytes);
    return SFWI_OK;
}

int sfwi_strip_bytes(sfwi_handle *h, size_t *device_bytes, size_t *host_bytes) {
    if (int rc = check(h)) return rc;
    if (device_bytes) *device_bytes = h->b.strip_dev_bytes;
    if (host_bytes) *host_bytes = h->b.strip_host_bytes;
    return SFWI_OK;
}

int sfwi_read_density_gradient_f64(sfwi_handle *h, double *grad_rho) {
    if (int rc = check(h)) return rc;
    if (!grad_rho) return fail(SFWI_E_ARG, "null output");
    const size_t n = (size_t)h->allnx * h->allnz;
    CK(cudaSetDevice(h->device));
    CK(cudaStreamSynchronize(h->st));
    if (int rc = ensure_grads(h)) return rc;
    CK(cudaMemcpyAsync(grad_rho, h->grh.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return SFWI_OK;
}

int sfwi_image_singleshot(sfwi_handle *h, double *misfit) {
    if (int rc = check(h)) return rc;
    std::vector<ShotIn> v(1);
    if (int rc = current_shot(h, v[0])) return rc;
    double m = 0.0;
    int rc = run_batch(h, v, RUN_GRADIENT, &m, nullptr);
    if (rc) return rc;
    if (misfit) *misfit += m;
    return SFWI_OK;
}

int sfwi_imagebuffer_resettozero(sfwi_handle *h, float *grad_pp, float *grad_ps, float *illum, float *b1, float *b2,
                                 float *b3, float *b4) {
    if (int rc = check(h)) return rc;
    const size_t n = (size_t)h->allnx * h->allnz;
    std::vector<double> tmp(n);
    CK(cudaSetDevice(h->device));
    CK(cudaStreamSynchronize(h->st));
    float *outs[3] = {grad_pp, grad_ps, illum};
    DevBuf<double> *src[3] = {&h->gpp, &h->gps, &h->gil};
    for (int k = 0; k < 3; k++) {
        if (outs[k]) {
            CK(cudaMemcpyAsync(tmp.data(), src[k]->p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
            CK(cudaStreamSynchronize(h->st));
            for (size_t i = 0; i < n; i++) outs[k][i] = (float)tmp[i];
        }
        CK(cudaMemsetAsync(src[k]->p, 0, n * sizeof(double), h->st));
    }
    if (h->grh.p) CK(cudaMemsetAsync(h->grh.p, 0, n * sizeof(double), h->st));
    CK(cudaStreamSynchronize(h->st));
    for (float *bb : {b1, b2, b3, b4})
        if (bb) std::memset(bb, 0, n * sizeof(float));
    return SFWI_OK;
}

int sfwi_read_gradients_f64(sfwi_handle *h, double *grad_pp, double *grad_ps, double *illum) {
    if (int rc = check(h)) return rc;
    const size_t n = (size_t)h->allnx * h->allnz;
    CK(cudaSetDevice(h->device));
    CK(cudaStreamSynchronize(h->st));
    if (grad_pp) CK(cudaMemcpyAsync(grad_pp, h->gpp.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    if (grad_ps) CK(cudaMemcpyAsync(grad_ps, h->gps.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    if (illum) CK(cudaMemcpyAsync(illum, h->gil.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return SFWI_OK;
}

int sfwi_read_records(sfwi_handle *h, int i, float *syn_z, float *syn_x, float *syn2_z, float *syn2_x, float *res_z,
                      float *res_x) {
    if (int rc = check(h)) return rc;
    if (!h->b.ready) return fail(SFWI_E_STATE, "no records: the last run did not complete");
    if (i < 0 || i >= (int)h->last_ntr.size()) return fail(SFWI_E_ARG, "shot %d not in the last run", i);
    if (!h->last_perm.empty()) i = h->last_perm[i];  // several-model runs reorder the shots
    const int nt = h->nt;
    const size_t off = (size_t)h->last_tr0[i] * nt, n = (size_t)h->last_ntr[i] * nt;
    Batch &b = h->b;
    CK(cudaSetDevice(h->device));
    CK(cudaStreamSynchronize(h->st));
    struct {
        float *dst;
        int k;
    } items[6] = {{syn_z, R_SYN_Z}, {syn_x, R_SYN_X}, {syn2_z, R_SYN2_Z}, {syn2_x, R_SYN2_X}, {res_z, R_RES_Z},
                  {res_x, R_RES_X}};
    for (auto &it : items)
        if (it.dst && n)
            CK(cudaMemcpyAsync(it.dst, b.r(it.k, nt) + off, n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return SFWI_OK;
}

int sfwi_enqueue_shot(sfwi_handle *h, const sfwi_shot_desc *d) {
    if (int rc = check(h)) return rc;
    if (!d) return fail(SFWI_E_ARG, "null shot");
    if (d->ntr < 0 || (d->ntr > 0 && (!d->gc || !d->rec_z || !d->rec_x)))
        return fail(SFWI_E_ARG, "shot needs gc and records");
    ShotIn s;
    s.nx = d->nx;
    s.win0 = d->delta_left + d->record_left_in_v;
    s.isx = d->isx;
    s.isz = d->isz;
    s.igz = d->igz;
    s.ngx_left = d->ngx_left;
    s.ntr = d->ntr;
    s.gc.assign(d->gc, d->gc + d->ntr);
    s.obs_z = d->rec_z;
    s.obs_x = d->rec_x;
    h->queue.push_back(std::move(s));
    return SFWI_OK;
}

int sfwi_clear_queue(sfwi_handle *h) {
    if (int rc = check(h)) return rc;
    h->queue.clear();
    return SFWI_OK;
}

int sfwi_run(sfwi_handle *h, double *misfit, double *per_shot_misfit) {
    if (int rc = check(h)) return rc;
    std::vector<ShotIn> q;
    q.swap(h->queue);
    h->last_perm.clear();
    double m = 0.0;
    int rc = run_batch(h, q, RUN_GRADIENT, &m, per_shot_misfit);
    if (rc) return rc;
    if (misfit) *misfit += m;
    return SFWI_OK;
}

int sfwi_run_models(sfwi_handle *h, int nmodels, const sfwi_model_desc *models, const int *shot_model,
                    double *per_shot_misfit, double *grad_pp, double *grad_ps, double *illum, double *grad_rho) {
    if (int rc = check(h)) return rc;
    std::vector<ShotIn> q;
    q.swap(h->queue);
    h->last_perm.clear();
    if (nmodels < 1 || !models || !shot_model) return fail(SFWI_E_ARG, "no models");
    if (q.empty()) return fail(SFWI_E_ARG, "no shots queued");
    // the models: grids within the handle's depth, lengths within its nt
    std::vector<sfwi_handle::ModelIn> mi(nmodels);
    size_t cells = 0;
    bool any_rho = false, any_dm = false;
    for (int k = 0; k < nmodels; k++) {
        const sfwi_model_desc &m = models[k];
        if (m.allnx < 1 || m.allnz < 1 || m.allnz + 2 * h->pml > h->nzpml || m.nt < 1 || m.nt > h->nt || !m.vp ||
            !m.vs)
            return fail(SFWI_E_ARG, "model %d: %d x %d, nt %d (depth at most %d, nt at most %d)", k, m.allnx, m.allnz,
                        m.nt, h->nzpml - 2 * h->pml, h->nt);
        if (h->stage == 1 && !m.rho) return fail(SFWI_E_ARG, "model %d: stage 1 needs rho", k);
        if ((m.dvp == nullptr) != (m.dvs == nullptr)) return fail(SFWI_E_ARG, "model %d: dvp and dvs go together", k);
        mi[k] = sfwi_handle::ModelIn{m.allnx, m.allnz, m.nt, cells};
        cells += (size_t)m.allnx * m.allnz;
        any_rho |= m.rho != nullptr;
        any_dm |= m.dvp != nullptr;
    }
    for (size_t i = 0; i < q.size(); i++)
        if (shot_model[i] < 0 || shot_model[i] >= nmodels)
            return fail(SFWI_E_ARG, "shot %zu: model %d of %d", i, shot_model[i], nmodels);
    // batch order: longer runs first (the shots still running at a step are
    // a prefix of the tile table), each model's shots together, queue order
    std::vector<int> order(q.size());
    for (size_t i = 0; i < q.size(); i++) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const int na = mi[shot_model[a]].nt, nb = mi[shot_model[b]].nt;
        return na != nb ? na > nb : shot_model[a] < shot_model[b];
    });
    std::vector<ShotIn> batch;
    for (int i : order) {
        batch.push_back(q[i]);
        batch.back().req = shot_model[i];
        batch.back().nt = mi[shot_model[i]].nt;
    }
    CK(cudaSetDevice(h->device));
    const size_t bytes = std::max<size_t>(cells, 1);
    DevBuf<float> *arr[5] = {&h->mvp, &h->mvs, &h->mrho, &h->mdvp, &h->mdvs};
    for (int a = 0; a < 5; a++)
        if (a < 2 || (a == 2 && any_rho) || (a > 2 && any_dm)) CK(arr[a]->ensure(bytes));
    for (int k = 0; k < nmodels; k++) {
        const sfwi_model_desc &m = models[k];
        const size_t n = (size_t)m.allnx * m.allnz, o = mi[k].off;
        const float *src[5] = {m.vp, m.vs, m.rho, m.dvp, m.dvs};
        for (int a = 0; a < 5; a++) {
            if (!arr[a]->p) continue;
            if (src[a])
                CK(cudaMemcpyAsync(arr[a]->p + o, src[a], n * sizeof(float), cudaMemcpyHostToDevice, h->st));
            else
                CK(cudaMemsetAsync(arr[a]->p + o, 0, n * sizeof(float), h->st));
        }
    }
    CK(h->mgrad.ensure(4 * bytes));
    CK(cudaMemsetAsync(h->mgrad.p, 0, 4 * bytes * sizeof(double), h->st));
    h->models = mi;
    h->mcells = cells;
    h->m_rho = any_rho;
    h->m_dm = any_dm;
    std::vector<double> per(batch.size());
    int rc = run_batch(h, batch, RUN_GRADIENT, nullptr, per.data());
    h->models.clear();
    if (rc) return rc;
    h->last_perm.assign(q.size(), 0);
    for (size_t k = 0; k < order.size(); k++) {
        h->last_perm[order[k]] = (int)k;
        if (per_shot_misfit) per_shot_misfit[order[k]] = per[k];
    }
    double *outs[4] = {grad_pp, grad_ps, illum, grad_rho};
    for (int a = 0; a < 4; a++)
        if (outs[a] && cells)
            CK(cudaMemcpyAsync(outs[a], h->mgrad.p + a * bytes, cells * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return SFWI_OK;
}

int sfwi_calculate_alpha_parabola_mb(sfwi_handle *h, const float *grad_pp, const float *grad_ps, float step1,
                                     float step2, double *misfit_step0, double *misfit_step1, double *misfit_step2) {
    if (int rc = check(h)) return rc;
    if (!misfit_step0 || !misfit_step1 || !misfit_step2) return fail(SFWI_E_ARG, "null output");
    std::vector<ShotIn> v(1);
    if (int rc = current_shot(h, v[0])) return rc;
    double m[3] = {0.0, 0.0, 0.0};
    if (int rc = line_search_parabola(h, v, grad_pp, grad_ps, step1, step2, m, nullptr)) return rc;
    *misfit_step0 += m[0];
    *misfit_step1 += m[1];
    *misfit_step2 += m[2];
    return SFWI_OK;
}

int sfwi_calculate_alpha(sfwi_handle *h, const float *image_pp, const float *image_ps, const float *cg_pp,
                         const float *cg_ps, double *fenzi, double *fenmu) {
    if (int rc = check(h)) return rc;
    if (!fenzi || !fenmu) return fail(SFWI_E_ARG, "null output");
    std::vector<ShotIn> v(1);
    if (int rc = current_shot(h, v[0])) return rc;
    return line_search_exact(h, v, image_pp, image_ps, cg_pp, cg_ps, fenzi, fenmu, nullptr);
}

int sfwi_line_search_parabola(sfwi_handle *h, const float *grad_pp, const float *grad_ps, float step1, float step2,
                              double *misfit3, double *per_shot3) {
    if (int rc = check(h)) return rc;
    if (!misfit3) return fail(SFWI_E_ARG, "null output");
    std::vector<ShotIn> q;
    q.swap(h->queue);
    return line_search_parabola(h, q, grad_pp, grad_ps, step1, step2, misfit3, per_shot3);
}

int sfwi_line_search_exact(sfwi_handle *h, const float *image_pp, const float *image_ps, const float *cg_pp,
                           const float *cg_ps, double *fenzi, double *fenmu, double *per_shot2) {
    if (int rc = check(h)) return rc;
    if (!fenzi || !fenmu) return fail(SFWI_E_ARG, "null output");
    std::vector<ShotIn> q;
    q.swap(h->queue);
    return line_search_exact(h, q, image_pp, image_ps, cg_pp, cg_ps, fenzi, fenmu, per_shot2);
}

int sfwi_born_adjoint(sfwi_handle *h, double *img_vp, double *img_vs) {
    if (int rc = check(h)) return rc;
    std::vector<ShotIn> q;
    q.swap(h->queue);
    return born_adjoint(h, q, img_vp, img_vs);
}

int sfwi_hessian_vector(sfwi_handle *h, const float *dvp, const float *dvs, double *hv_vp, double *hv_vs) {
    if (int rc = check(h)) return rc;
    if (h->stage != 2) return fail(SFWI_E_STATE, "the Born operator belongs to stage 2");
    if (!dvp || !dvs || !hv_vp || !hv_vs) return fail(SFWI_E_ARG, "null argument");
    std::vector<ShotIn> q;
    q.swap(h->queue);
    if (q.empty()) return fail(SFWI_E_ARG, "no shots queued");
    for (const ShotIn &in : q)
        if (in.nt > 0 && in.nt != h->nt) return fail(SFWI_E_ARG, "Hessian-vector products run the handle's nt");
    // L m: the scattered records of every queued shot
    if (int rc = sfwi_gpu_buffer_m(h, dvp, dvs)) return rc;
    if (int rc = run_batch(h, q, RUN_FORWARD, nullptr, nullptr)) return rc;
    std::vector<std::vector<float>> rec(2 * q.size());
    for (size_t i = 0; i < q.size(); i++) {
        const size_t n = std::max<size_t>((size_t)q[i].ntr * h->nt, 1);
        rec[2 * i].resize(n);
        rec[2 * i + 1].resize(n);
        if (int rc = sfwi_read_records(h, (int)i, rec[2 * i].data(), rec[2 * i + 1].data(), nullptr, nullptr, nullptr,
                                       nullptr))
            return rc;
        q[i].obs_z = rec[2 * i].data();
        q[i].obs_x = rec[2 * i + 1].data();
    }
    // L^T (L m)
    return born_adjoint(h, q, hv_vp, hv_vs);
}

int sfwi_run_forward(sfwi_handle *h) {
    if (int rc = check(h)) return rc;
    std::vector<ShotIn> q;
    q.swap(h->queue);
    return run_batch(h, q, RUN_FORWARD, nullptr, nullptr);
}

int sfwi_ot(const float *obs_x, const float *obs_z, const float *cal_x, const float *cal_z, float *res_x, float *res_z,
            int length, int tracenum, float dt, double *misfit) {
    return ot_host(SFWI_MISFIT_OT, obs_x, obs_z, cal_x, cal_z, res_x, res_z, length, tracenum, dt, misfit);
}
int sfwi_ot_power(const float *obs_x, const float *obs_z, const float *cal_x, const float *cal_z, float *res_x,
                  float *res_z, int length, int tracenum, float dt, double *misfit) {
    return ot_host(SFWI_MISFIT_OT_POWER, obs_x, obs_z, cal_x, cal_z, res_x, res_z, length, tracenum, dt, misfit);
}
int sfwi_ot_alltrace(const float *obs_x, const float *obs_z, const float *cal_x, const float *cal_z, float *res_x,
                     float *res_z, int length, int tracenum, float dt, double *misfit) {
    return ot_host(SFWI_MISFIT_OT_ALLTRACE, obs_x, obs_z, cal_x, cal_z, res_x, res_z, length, tracenum, dt, misfit);
}

int sfwi_normalize(float *matrix, int length, int tracenum) {
    // sfwi-stage1/main.cpp:24-32
    if (!matrix || length < 0 || tracenum < 0) return fail(SFWI_E_ARG, "bad argument");
    const size_t n = (size_t)length * tracenum;
    float mx = 0;
    for (size_t i = 0; i < n; i++) mx = (std::fabs(matrix[i]) > mx) ? std::fabs(matrix[i]) : mx;
    for (size_t i = 0; i < n; i++) matrix[i] = matrix[i] / mx;
    return SFWI_OK;
}

long long sfwi_kernel_launches(sfwi_handle *h) { return h ? h->launches : 0; }

int sfwi_last_timing(sfwi_handle *h, float *fwd_ms, float *bwd_ms, float *other_ms, float *total_ms) {
    if (int rc = check(h)) return rc;
    if (fwd_ms) *fwd_ms = h->fwd_ms;
    if (bwd_ms) *bwd_ms = h->bwd_ms;
    if (other_ms) *other_ms = h->other_ms;
    if (total_ms) *total_ms = h->total_ms;
    return SFWI_OK;
}

int sfwi_time_kernels(sfwi_handle *h, int reps, float *out_ms) {
    if (int rc = check(h)) return rc;
    if (!out_ms || reps < 1) return fail(SFWI_E_ARG, "bad argument");
    if (!h->b.ready || h->b.ntiles == 0) return fail(SFWI_E_STATE, "no batch on the device (none run, or the last run failed)");
    CK(cudaSetDevice(h->device));
    const Params p = make_params(h, false);
    const bool born = h->stage == 2;
    const float adj = h->stage == 1 ? 1.f : -1.f;
    if (h->last_forward_only) return fail(SFWI_E_STATE, "the last run was forward-only (no edge strips)");
    if (reps > kTimeKernelsMaxReps) reps = kTimeKernelsMaxReps;
    if (reps > h->nt - 1) reps = h->nt - 1;  // step indices 0..reps must exist
    if (reps < 1) return fail(SFWI_E_ARG, "nt too small to time the kernels");
    for (int k = 0; k < 4; k++) {
        // step indices 0..reps select fresh tile counters; the kernels read
        // records and strips at those steps, which exist for every run
        CK(cudaMemsetAsync(h->b.dctr.p, 0, 4 * (size_t)(reps + 1) * sizeof(int), h->st));
        // consecutive launches alternate the tile order, as consecutive
        // sweeps of a time loop do: each starts where the one before ended
        Params q = p;
        h->tv->launch(k, q, h->b.tm, reps, born, adj, h->st);  // warm
        CK(cudaEventRecord(h->ev[0], h->st));
        for (int r = 0; r < reps; r++) {
            q.reverse_tiles = p.reverse_tiles ^ ((unsigned)((r + 1) & 1) << k);
            h->tv->launch(k, q, h->b.tm, r, born, adj, h->st);
        }
        CK(cudaEventRecord(h->ev[1], h->st));
        CK(cudaEventSynchronize(h->ev[1]));
        CK(cudaGetLastError());
        float ms = 0.f;
        cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
        out_ms[k] = ms / reps;
        h->launches += reps + 1;
    }
    return SFWI_OK;
}

int sfwi_autotune(sfwi_handle *h, int reps, int *choice, float *out_ms) {
    if (int rc = check(h)) return rc;
    if (reps < 1) return fail(SFWI_E_ARG, "bad argument");
    if (!h->b.ready || h->b.ntiles == 0) return fail(SFWI_E_STATE, "no batch on the device (none run, or the last run failed)");
    if (h->last_forward_only) return fail(SFWI_E_STATE, "the last run was forward-only (no edge strips)");
    CK(cudaSetDevice(h->device));
    // one gradient step of the batch (the four step kernels) per tile shape;
    // the kernels only read the state and the strips and write the
    // accumulators, which the next run clears
    float best = 0.f;
    int pick = 0;
    for (int v = 0; v < SFWI_NUM_TILE_SHAPES; v++) {
        if (int rc = sfwi_set_tile_shape(h, v)) return rc;
        float ms[4];
        if (int rc = sfwi_time_kernels(h, reps, ms)) return rc;
        const float t = ms[0] + ms[1] + ms[2] + ms[3];
        if (out_ms) out_ms[v] = t;
        if (v == 0 || t < best) best = t, pick = v;
    }
    if (choice) *choice = pick;
    return sfwi_set_tile_shape(h, pick);
}

int sfwi_debug_tile_grid(int pml, int nzpml, int tx, int tz, const int *nxpml, int nshots, int *z_start,
                         int *x_start, int *tiles, int *frame_tiles) {
    if (!nxpml || !z_start || !x_start || nshots < 1 || pml < NOP || nzpml < 2 * pml + 1 || tx < 1 || tz < 8 ||
        tz % 8)
        return fail(SFWI_E_ARG, "bad tile-grid arguments");
    for (int s = 0; s < nshots; s++)
        if (nxpml[s] < 2 * pml + 1) return fail(SFWI_E_ARG, "shot %d: padded width %d too small", s, nxpml[s]);
    const AxisTiling zt = plan_z_tiling(pml, nzpml, tx, tz, nxpml, nshots);
    *z_start = zt.start;
    for (int s = 0; s < nshots; s++) {
        const AxisTiling xt = best_x_tiling(nxpml[s], pml, tx, zt);
        x_start[s] = xt.start;
        if (tiles) tiles[s] = xt.count * zt.count;
        if (frame_tiles) frame_tiles[s] = xt.count * zt.count - (xt.count - xt.frame) * (zt.count - zt.frame);
    }
    return SFWI_OK;
}

int sfwi_debug_grid_shape(sfwi_handle *h, int *X, int *P, int *narrays, int *nstate) {
    if (int rc = check(h)) return rc;
    if (!h->b.ready) return fail(SFWI_E_STATE, "no batch on the device");
    if (X) *X = h->b.X;
    if (P) *P = h->b.P;
    if (narrays) *narrays = NGRID;
    if (nstate) *nstate = NSTATE;
    return SFWI_OK;
}

int sfwi_debug_read_grid(sfwi_handle *h, int array, float *dst) {
    if (int rc = check(h)) return rc;
    if (!dst || array < 0 || array >= NGRID) return fail(SFWI_E_ARG, "bad array %d", array);
    Batch &b = h->b;
    if (!b.ready) return fail(SFWI_E_STATE, "no batch on the device");
    CK(cudaSetDevice(h->device));
    CK(cudaMemcpyAsync(dst, b.g(array), b.cells * sizeof(float), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return SFWI_OK;
}

int sfwi_wait_selftest(sfwi_handle *h, unsigned tries) {
    if (int rc = check(h)) return rc;
    if (tries < 1 || tries > PIPE_WAIT_LIMIT) return fail(SFWI_E_ARG, "tries must be in 1..%u", PIPE_WAIT_LIMIT);
    Batch &b = h->b;
    if (!b.ready || b.ntiles < 4) return fail(SFWI_E_STATE, "run a batch of at least 4 tiles first");
    CK(cudaSetDevice(h->device));
    Params p = make_params(h, h->last_forward_only);
    p.wait_limit = tries;
    CK(cudaMemsetAsync(b.dctr.p, 0, sizeof(int), h->st));
    CK(cudaMemsetAsync(b.derr.p, 0, sizeof(int), h->st));
    h->tv->wait_probe(p, h->st);
    h->launches++;
    CK(cudaGetLastError());
    int derr = 0;
    CK(cudaMemcpyAsync(&derr, b.derr.p, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    CK(cudaMemsetAsync(b.derr.p, 0, sizeof(int), h->st));
    CK(cudaStreamSynchronize(h->st));
    if (derr) return fail(SFWI_E_CUDA, "a device-side pipeline wait timed out (code %d)", derr);
    return fail(SFWI_E_STATE, "the wait probe completed without a timeout");
}

int sfwi_set_source(sfwi_handle *h, int kind) {
    if (int rc = check(h)) return rc;
    if (kind != SFWI_SOURCE_TXX_TZZ && kind != SFWI_SOURCE_VZ_FORCE) return fail(SFWI_E_ARG, "unknown source kind %d", kind);
    h->src_kind = kind == SFWI_SOURCE_VZ_FORCE ? SRC_VZ_FORCE : SRC_TXX_TZZ;
    return SFWI_OK;
}

int sfwi_set_launch_overlap(sfwi_handle *h, int on) {
    if (int rc = check(h)) return rc;
    h->launch_overlap = on != 0;
    return SFWI_OK;
}

int sfwi_set_tile_order(sfwi_handle *h, unsigned reverse_bits) {
    if (int rc = check(h)) return rc;
    if (reverse_bits > 15u) return fail(SFWI_E_ARG, "tile order bits must be in 0..15");
    h->tile_order = reverse_bits;
    return SFWI_OK;
}

int sfwi_set_tile_shape(sfwi_handle *h, int shape) {
    if (int rc = check(h)) return rc;
    if (shape < 0 || shape >= SFWI_NUM_TILE_SHAPES) return fail(SFWI_E_ARG, "tile shape %d out of range", shape);
    h->tile_auto = false;
    if (h->tv == tile_variant(shape)) return SFWI_OK;
    h->tv = tile_variant(shape);
    Batch &b = h->b;
    if (!b.ready || b.nshots == 0) return SFWI_OK;  // applies to the next batch
    // re-tile the resident batch and re-encode its maps for the new boxes
    CK(cudaSetDevice(h->device));
    build_tiles(h);
    if (int rc = upload_tiles(h)) return rc;
    CK(cudaStreamSynchronize(h->st));  // b.trecs may change again before the copy ran
    return encode_tile_maps(h, h->last_forward_only);
}

int sfwi_get_tile_shape(sfwi_handle *h, int *shape, int *tx, int *tz) {
    if (int rc = check(h)) return rc;
    for (int v = 0; v < SFWI_NUM_TILE_SHAPES; v++)
        if (h->tv == tile_variant(v)) {
            if (shape) *shape = v;
            if (tx) *tx = h->tv->tx;
            if (tz) *tz = h->tv->tz;
        }
    return SFWI_OK;
}

int sfwi_host_alloc(size_t bytes, void **ptr) {
    if (!ptr) return fail(SFWI_E_ARG, "null pointer");
    *ptr = nullptr;
    cudaError_t e = cudaMallocHost(ptr, bytes ? bytes : 1);
    if (e != cudaSuccess) return fail(SFWI_E_NOMEM, "cudaMallocHost(%zu): %s", bytes, cudaGetErrorString(e));
    return SFWI_OK;
}

int sfwi_host_free(void *ptr) {
    if (ptr) cudaFreeHost(ptr);
    return SFWI_OK;
}

}  // extern "C"
