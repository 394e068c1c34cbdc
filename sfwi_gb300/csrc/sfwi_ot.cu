// sfwi_ot.cu — per-trace 1D quadratic-Wasserstein misfit and adjoint source.
//
// The reference declares OT, OT_power and OT_alltrace (sfwi-stage1/FD2DGPU.cuh:
// 21-25, argument order obs_x, obs_z, cal_x, cal_z, res_x, res_z, length,
// tracenum, misfit) and defines none of them.  This is the 1D W2 misfit
// between positive-normalised traces, written from its definition:
//   weights   p(u) = exp((u - max u)/sigma)          (OT, OT_alltrace)
//             p(u) = u^2 + 1e-3 sigma^2              (OT_power)
//             sigma = max|obs| of the trace, floored at 1e-3 max|obs| of the
//             gather (OT, OT_power), or max|obs| of the gather (OT_alltrace)
//   densities f = p(cal)/sum p(cal), g = p(obs)/sum p(obs)
//   CDFs      F_k = sum_{j<=k} f_j,  G_k likewise
//   transport T_k = G^-1(F_k) = dt (m + (F_k - G_{m-1})/g_m), G_{m-1} <= F_k < G_m
//   misfit    W = sum_k ((k+1) dt - T_k)^2 f_k
//   adjoint   A_j = ((j+1)dt - T_j)^2 - 2 sum_{k>=j} ((k+1)dt - T_k) f_k dt / g_m(k)
//             res_i = (1/2) (A_i - sum_j f_j A_j) / sum p(cal) * p'(cal_i)
// res is (1/2) dW/dcal, the scaling of the L2 residual (misfit sum r^2,
// adjoint source r).  The CDFs, the quantile search and every sum are FP64.
// The exponential weights are FP32 (expf of the argument rounded to FP32,
// then widened): their argument is at most 0, so a weight is 1 at the
// trace's maximum and its relative rounding of about 1e-7 stays far below
// the 1e-4 parity bar, while a double exp would be most of the kernel's
// FP64 work.
// One CTA handles one (trace, component); prefix and suffix sums are block
// scans built on warp shuffles.
#include <cfloat>
#include <cudaTypedefs.h>
#include <mutex>

#include "sfwi_launch.h"

namespace sfwi {

constexpr int OT_THREADS = 256;

__device__ __forceinline__ double warp_incl_scan(double v) {
    const int l = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, v, o);
        if (l >= o) v += u;
    }
    return v;
}

// exclusive block scan of one value per thread (thread order)
__device__ double block_excl_scan(double v, double *wsum) {
    const double inc = warp_incl_scan(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        double t = l < nw ? wsum[l] : 0.0;
        const double ti = warp_incl_scan(t);
        if (l < nw) wsum[l] = ti - t;
    }
    __syncthreads();
    const double r = wsum[w] + inc - v;
    __syncthreads();
    return r;
}

__device__ double block_reduce(double v, double *wsum) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) wsum[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += wsum[i];
    __syncthreads();
    return t;
}

__device__ double block_max(double v, double *wsum) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) wsum[w] = v;
    __syncthreads();
    double t = -DBL_MAX;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t = fmax(t, wsum[i]);
    __syncthreads();
    return t;
}

// in-place inclusive prefix (reverse=false) or suffix (reverse=true) sums of a[0..n)
__device__ void block_scan_array(double *a, int n, bool reverse, double *wsum) {
    const int chunk = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * chunk, e = min(n, b + chunk);
    double s = 0.0;
    for (int i = b; i < e; i++) s += a[reverse ? n - 1 - i : i];
    const double off = block_excl_scan(s, wsum);
    double run = off;
    for (int i = b; i < e; i++) {
        const int k = reverse ? n - 1 - i : i;
        run += a[k];
        a[k] = run;
    }
    __syncthreads();
}

// exclusive suffix sums over the threads of the block: thread t gets the sum
// of v over threads t+1 .. blockDim.x-1 (cs: blockDim.x doubles of shared
// memory; wsum as block_excl_scan)
__device__ double block_excl_suffix(double v, double *cs, double *wsum) {
    const int t = threadIdx.x, T = blockDim.x;
    cs[t] = v;
    __syncthreads();
    const double e = block_excl_scan(cs[T - 1 - t], wsum);  // sum over threads after T-1-t
    cs[T - 1 - t] = e;
    __syncthreads();
    const double r = cs[t];
    __syncthreads();
    return r;
}

// smallest m >= lo with G[m] > y, capped at n-1 (G non-decreasing and every
// index below lo known to hold G <= y): a galloping search from lo, so
// consecutive quantiles of one thread cost a few probes instead of a full
// binary search; the answer is that of a binary search over [0, n-1)
__device__ __forceinline__ int first_above(const double *G, int n, double y, int lo) {
    if (lo >= n - 1) return n - 1;
    if (G[lo] > y) return lo;
    int prev = lo, step = 1, hi;
    for (;;) {
        const int nx = prev + step;
        if (nx >= n - 1) {
            hi = n - 1;
            break;
        }
        if (G[nx] > y) {
            hi = nx;
            break;
        }
        prev = nx;
        step <<= 1;
    }
    int l = prev + 1;
    while (l < hi) {
        const int mid = (l + hi) >> 1;
        if (G[mid] > y)
            hi = mid;
        else
            l = mid + 1;
    }
    return l;
}

// The GB300's FP64 rate is a small fraction of its FP32 rate, so the kernel
// spends FP64 operations sparingly: each thread owns one contiguous chunk of
// samples, the positivity transform (one exp per sample and trace) is
// evaluated once and kept, the CDF of the synthetic trace is formed on the
// fly from the chunk's running sum, the quantile search continues from the
// previous sample's quantile, and divisions by per-trace constants are
// multiplications by their reciprocals.
constexpr int OT_MAX_CHUNK = 32;  // samples per thread of the shared-memory form: nt <= 32 * OT_THREADS

// LONG = false: the per-trace arrays in shared memory (traces up to
// ot_max_nt() samples); LONG = true: in the caller's global scratch, five
// arrays of nt doubles per (trace, component), for longer traces (the
// transport residuals r then go to the fifth array instead of registers).
template <bool LONG>
__global__ void __launch_bounds__(OT_THREADS) k_ot(OtArgs a) {
    extern __shared__ double ot_sm[];
    __shared__ double wsum[32];
    __shared__ double cs[OT_THREADS];
    const int n = a.nt;
    // G: CDF of the observed trace; g: its density; P: p(cal); Q: the terms
    // r f dt / g, then the adjoint weights A; R (long form): r
    double *G = LONG ? a.scratch + (size_t)blockIdx.x * 5 * n : ot_sm;
    double *g = G + n, *P = g + n, *Q = P + n;
    double *R = LONG ? Q + n : nullptr;
    const int tr = blockIdx.x >> 1, comp = blockIdx.x & 1;
    const size_t o = (size_t)tr * n;
    const float *cal = (comp ? a.cal_x : a.cal_z) + o;
    const float *cal2 = a.cal2_z ? (comp ? a.cal2_x : a.cal2_z) + o : nullptr;
    const float *obs = (comp ? a.obs_x : a.obs_z) + o;
    float *res = (comp ? a.res_x : a.res_z) + o;
    double sigma = a.sigma[2 * tr + comp];
    if (!(sigma > 0.0)) sigma = 1.0;
    const double inv_sigma = 1.0 / sigma;
    const bool pw = a.kind == 2;
    auto pred = [&](int k) -> double { return cal2 ? (double)(cal[k] + cal2[k]) : (double)cal[k]; };
    const int chunk = (n + blockDim.x - 1) / blockDim.x;
    const int k0 = min(n, (int)threadIdx.x * chunk), k1 = min(n, k0 + chunk);

    double mc = -DBL_MAX, mo = -DBL_MAX;
    for (int k = k0; k < k1; k++) {
        mc = fmax(mc, pred(k));
        mo = fmax(mo, (double)obs[k]);
    }
    const double cmax = block_max(mc, wsum), omax = block_max(mo, wsum);
    const double eps = 1e-3 * sigma * sigma;
    auto pf = [&](double u) { return pw ? u * u + eps : (double)expf((float)((u - cmax) * inv_sigma)); };
    auto pg = [&](double u) { return pw ? u * u + eps : (double)expf((float)((u - omax) * inv_sigma)); };

    double sf = 0.0, sg = 0.0;
    for (int k = k0; k < k1; k++) {
        const double x = pf(pred(k)), y = pg((double)obs[k]);
        P[k] = x;
        g[k] = y;
        sf += x;
        sg += y;
    }
    const double Sf = block_reduce(sf, wsum), Sg = block_reduce(sg, wsum);
    const double inv_Sf = 1.0 / Sf, inv_Sg = 1.0 / Sg;
    // densities, the chunk sums of both, and the CDF G of the observed trace
    double cf = 0.0, cg = 0.0;
    for (int k = k0; k < k1; k++) {
        g[k] *= inv_Sg;
        cg += g[k];
        cf += P[k] * inv_Sf;
    }
    const double offF = block_excl_scan(cf, wsum), offG = block_excl_scan(cg, wsum);
    {
        double run = offG;
        for (int k = k0; k < k1; k++) {
            run += g[k];
            G[k] = run;
        }
    }
    __syncthreads();

    // transport T_k = G^-1(F_k) and the misfit terms
    double w = 0.0, sq = 0.0, Fk = offF;
    double r_loc[LONG ? 1 : OT_MAX_CHUNK];
    int m = 0;
    for (int i = 0; i < k1 - k0; i++) {
        const int k = k0 + i;
        const double fk = P[k] * inv_Sf;
        Fk += fk;
        m = first_above(G, n, Fk, m);
        const double gm = g[m];
        const double inv_gm = 1.0 / gm;
        const double Gm1 = m > 0 ? G[m - 1] : 0.0;
        const double T = a.dt * (m + (Fk - Gm1) * inv_gm);
        const double r = (k + 1) * a.dt - T;
        w += r * r * fk;
        if (LONG)
            R[k] = r;
        else
            r_loc[i] = r;
        const double q = r * fk * a.dt * inv_gm;
        Q[k] = q;
        sq += q;
    }
    // suffix sums of q, the adjoint weights A_k = r_k^2 - 2 sum_{j>=k} q_j and
    // their f-weighted sum
    const double offQ = block_excl_suffix(sq, cs, wsum);
    double fa = 0.0, run = offQ;
    for (int i = k1 - k0 - 1; i >= 0; i--) {
        const int k = k0 + i;
        run += Q[k];
        const double rk = LONG ? R[k] : r_loc[i];
        const double A = rk * rk - 2.0 * run;
        Q[k] = A;
        fa += P[k] * inv_Sf * A;
    }
    const double FA = block_reduce(fa, wsum);
    const double W = block_reduce(w, wsum);
    for (int k = k0; k < k1; k++) {
        const double dp = pw ? 2.0 * pred(k) : P[k] * inv_sigma;
        res[k] = (float)(0.5 * (Q[k] - FA) * inv_Sf * dp);
    }
    if (threadIdx.x == 0) a.trace_misfit[2 * tr + comp] = W;
}

size_t ot_smem_bytes(int nt) { return (size_t)4 * nt * sizeof(double); }

// longest trace k_ot takes: four FP64 arrays of nt samples next to the static
// block-scan buffers within 227 KB, and at most OT_MAX_CHUNK samples a thread
int ot_max_nt() {
    const int by_smem = (int)((227 * 1024 - (OT_THREADS + 32) * sizeof(double) - 1024) / (4 * sizeof(double)));
    return by_smem < OT_MAX_CHUNK * OT_THREADS ? by_smem : OT_MAX_CHUNK * OT_THREADS;
}

size_t ot_scratch_doubles(int nt, int ntr) { return nt > ot_max_nt() ? (size_t)5 * nt * 2 * ntr : 0; }

cudaError_t launch_ot(const OtArgs &a, cudaStream_t st) {
    if (a.nt > ot_max_nt()) {
        if (!a.scratch) return cudaErrorInvalidValue;
        k_ot<true><<<2 * a.ntr, OT_THREADS, 0, st>>>(a);
        return cudaGetLastError();
    }
    const size_t sm = ot_smem_bytes(a.nt);
    cudaError_t e = cudaFuncSetAttribute(k_ot<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_ot<false><<<2 * a.ntr, OT_THREADS, sm, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free OT entry point (sfwi_ot_noalloc in include/sfwi_gb300.h).
//
// Its working memory -- the per-trace scale of the positivity transform, the
// per-trace misfits and their sum -- lives in the fixed array below instead
// of buffers from cudaMalloc.  It serves callers that cannot allocate device
// memory: a host program whose own allocator has reserved every device byte
// up front, and inner loops where a cudaMalloc/cudaFree may synchronise the
// device and stall other work in flight.
// Every device that loads this library holds the array (256 KB) until the
// process exits.  All calls on a device share it, so calls that overlap on the
// GPU (different streams or threads at the same time) race on it.
// ---------------------------------------------------------------------------
constexpr int OT_NOALLOC_MAX_TRACES = 8192;
// [0, 2*max): scale per (trace, component); [2*max, 4*max): misfit per
// (trace, component); [4*max]: the summed misfit
static __device__ __align__(256) double g_ot_noalloc_scratch[4 * OT_NOALLOC_MAX_TRACES + 32];

// scale of trace `blockIdx.x>>1`, component `blockIdx.x&1`: max |obs|
__global__ void k_ot_trace_scale(const float *obs_z, const float *obs_x, int nt, double *sigma) {
    __shared__ double wsum[32];
    const int tr = blockIdx.x >> 1, comp = blockIdx.x & 1;
    const float *o = (comp ? obs_x : obs_z) + (size_t)tr * nt;
    double m = 0.0;
    for (int k = threadIdx.x; k < nt; k += blockDim.x) m = fmax(m, fabs((double)o[k]));
    const double t = block_max(m, wsum);
    if (threadIdx.x == 0) sigma[blockIdx.x] = t;
}

// gather-wide scale: every trace of a component takes the largest (kind 3),
// or its own floored at OT_SIGMA_FLOOR times the largest (kinds 1, 2)
__global__ void k_ot_gather_scale(double *sigma, int ntr, int all) {
    __shared__ double wsum[32];
    const int comp = blockIdx.x;
    double m = 0.0;
    for (int t = threadIdx.x; t < ntr; t += blockDim.x) m = fmax(m, sigma[2 * t + comp]);
    const double g = block_max(m, wsum);
    __syncthreads();
    for (int t = threadIdx.x; t < ntr; t += blockDim.x)
        sigma[2 * t + comp] = all ? g : fmax(sigma[2 * t + comp], OT_SIGMA_FLOOR * g);
}

// per-shot floor of the trace scales (kinds 1, 2) or the shot's largest
// scale for every trace (kind 3); block = (shot, component)
__global__ void k_ot_shot_scale(double *sigma, const ShotGeo *geo, int all) {
    __shared__ double wsum[32];
    const int s = blockIdx.x >> 1, comp = blockIdx.x & 1;
    const int t0 = geo[s].tr0, n = geo[s].ntr;
    double m = 0.0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) m = fmax(m, sigma[2 * (t0 + t) + comp]);
    const double g = block_max(m, wsum);
    __syncthreads();
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        double &v = sigma[2 * (t0 + t) + comp];
        v = all ? g : fmax(v, OT_SIGMA_FLOOR * g);
    }
}

void launch_ot_scales(const float *obs_z, const float *obs_x, int nt, int ntr, const ShotGeo *geo, int nshots,
                      int all, double *sigma, cudaStream_t st) {
    if (ntr < 1) return;
    k_ot_trace_scale<<<2 * ntr, 256, 0, st>>>(obs_z, obs_x, nt, sigma);
    k_ot_shot_scale<<<2 * nshots, 256, 0, st>>>(sigma, geo, all);
}

// misfit = sum over traces of the two components, in trace order
__global__ void k_ot_sum(const double *trace_misfit, int ntr, double *out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double w = 0.0;
        for (int i = 0; i < 2 * ntr; i++) w += trace_misfit[i];
        *out = w;
    }
}

}  // namespace sfwi

namespace {
// Device address of g_ot_noalloc_scratch, looked up once per CUDA context with
// the device current: host code cannot take the address of a __device__
// array (its name there is a host-side stand-in), and a new context on the
// same device (after cudaDeviceReset) loads the module, and the array, anew.
// The context is identified by cuCtxGetId, which never repeats in a process;
// where the driver does not offer it, the address is kept per device.
struct ScratchAddr {
    unsigned long long ctx;
    double *addr;
};
std::mutex g_noalloc_mu;
ScratchAddr g_noalloc_addr[128] = {};

unsigned long long current_context_id() {
    static PFN_cuCtxGetCurrent_v4000 get_cur = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    static bool looked = false;
    if (!looked) {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f);
        looked = true;
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (get_cur && get_id && get_cur(&c) == CUDA_SUCCESS && c && get_id(c, &id) == CUDA_SUCCESS) return id + 1;
    return 0;  // unknown: one address per device
}
}  // namespace

extern "C" int sfwi_ot_noalloc(int kind, const float *obs_x, const float *obs_z, const float *cal_x,
                               const float *cal_z, float *res_x, float *res_z, int length, int tracenum, float dt,
                               double *misfit, void *stream) {
    using namespace sfwi;
    if (kind < 1 || kind > 3) return record_error(-1, "sfwi_ot_noalloc: kind must be 1, 2 or 3");
    if (!misfit || length < 1 || tracenum < 0) return record_error(-1, "sfwi_ot_noalloc: bad argument");
    // an empty gather (a shot without receivers) adds nothing, as sfwi_ot
    if (tracenum == 0) return 0;
    if (!obs_x || !obs_z || !cal_x || !cal_z || !res_x || !res_z)
        return record_error(-1, "sfwi_ot_noalloc: bad argument");
    if (tracenum > OT_NOALLOC_MAX_TRACES)
        return record_error(-1, "sfwi_ot_noalloc: %d traces exceed the fixed scratch of %d traces", tracenum,
                            OT_NOALLOC_MAX_TRACES);
    if (length > ot_max_nt())
        return record_error(-1, "sfwi_ot_noalloc: length %d exceeds %d samples", length, ot_max_nt());
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return record_error(-2, "sfwi_ot_noalloc: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= 128) return record_error(-1, "sfwi_ot_noalloc: device %d out of range", dev);
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        unsigned long long ctx = current_context_id();
        if (ctx == 0) {
            // no context current yet: make the device's primary context
            // current (it allocates nothing) so that its id can be read
            if ((e = cudaSetDevice(dev)) != cudaSuccess)
                return record_error(-2, "sfwi_ot_noalloc: %s", cudaGetErrorString(e));
            ctx = current_context_id();
        }
        ScratchAddr &a = g_noalloc_addr[dev];
        if (!a.addr || a.ctx != ctx) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_ot_noalloc_scratch);
            if (e != cudaSuccess) return record_error(-2, "sfwi_ot_noalloc: scratch address: %s", cudaGetErrorString(e));
            a.addr = static_cast<double *>(p);
            a.ctx = ctx;
        }
        scratch = a.addr;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *sigma = scratch, *tmis = scratch + 2 * OT_NOALLOC_MAX_TRACES, *sum = scratch + 4 * OT_NOALLOC_MAX_TRACES;
    k_ot_trace_scale<<<2 * tracenum, 256, 0, st>>>(obs_z, obs_x, length, sigma);
    k_ot_gather_scale<<<2, 256, 0, st>>>(sigma, tracenum, kind == 3);
    OtArgs o{};
    o.kind = kind;
    o.nt = length;
    o.ntr = tracenum;
    o.stage = 1;
    o.dt = dt;
    o.obs_z = obs_z;
    o.obs_x = obs_x;
    o.cal_z = cal_z;
    o.cal_x = cal_x;
    o.res_z = res_z;
    o.res_x = res_x;
    o.sigma = sigma;
    o.trace_misfit = tmis;
    if ((e = launch_ot(o, st)) != cudaSuccess) return record_error(-2, "sfwi_ot_noalloc: %s", cudaGetErrorString(e));
    k_ot_sum<<<1, 32, 0, st>>>(tmis, tracenum, sum);
    double w = 0.0;
    if ((e = cudaMemcpyAsync(&w, sum, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return record_error(-2, "sfwi_ot_noalloc: %s", cudaGetErrorString(e));
    *misfit += w;
    return 0;
}
