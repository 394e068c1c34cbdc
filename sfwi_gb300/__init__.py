"""sfwi_gb300 — GB300 (sm_103a) engine for the SFWI per-shot gradient path.

Python face of the C ABI (include/sfwi_gb300.h), shaped like the reference's
per-shot engine so a driver written against it reads the same:

    fd = FD2DGPU_ELASTIC(sou, dx, dz, dt, nxpml, nzpml, allnx, allnz,
                         scale, pml, nt, nop, ntr, stage=1)   # FD2DGPU.cuh:152
    fd.GPUbufferVPVS(vp_all, vs_all, rho_all)                 # :296
    fd.ntr = ntr; fd.record_copytoGPU(rec_z, rec_x, gc)      # FD2DGPU.cu:3507
    fd.bufferVpVsHtoD(delta_left + record_left_in_v)          # :1348
    fd.isx, fd.isz, fd.igz = ...; fd.ngx_left = ...; fd.delta_left = ...
    misfit = IMAGE_SINGLESHOT(fd, misfit)                     # FD2DGPU.cuh:466
    grads = fd.imagebuffer_resettozero()                      # FD2DGPU.cu:3646

plus batched entry points (enqueue_shot / run) that advance many shots in the
same kernel launches.  Arrays are numpy float32 in the reference's layouts:
models [allnx, allnz], records [ntr, nt].
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import SfwiError, ShotDesc

__all__ = ["FD2DGPU_ELASTIC", "IMAGE_SINGLESHOT", "OT", "OT_power", "OT_alltrace", "normalize", "SfwiError",
           "set_pinned_cache",
           "MISFIT_L2", "MISFIT_OT", "MISFIT_OT_POWER", "MISFIT_OT_ALLTRACE", "library_path"]

MISFIT_L2, MISFIT_OT, MISFIT_OT_POWER, MISFIT_OT_ALLTRACE = 0, 1, 2, 3


def library_path():
    return _lib.LIB_PATH


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None and a.shape != tuple(shape):
        a = a.reshape(shape)
    return a


def _fp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _ip(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


class FD2DGPU_ELASTIC:
    """One per-shot engine (the reference's FD2DGPU_ELASTIC object).

    stage=1 reproduces sfwi-stage1's IMAGE_SINGLESHOT, stage=2 sfwi-stage2's
    (Born forward, residual (du-obs)+u0, adjoint direction -1, rho = 2000)."""

    def __init__(self, sou, dx, dz, dt, nxpml, nzpml, allnx, allnz, scale, pml, nt, nop, ntr, stage=1):
        lib = _lib.load()
        self._sou = _f32(sou)
        h = C.c_void_p()
        _lib.check(lib.sfwi_create(C.byref(h), stage, _fp(self._sou), dx, dz, dt, nxpml, nzpml, allnx, allnz, scale,
                                   pml, nt, nop, ntr))
        self._h = h
        self.stage, self.dx, self.dz, self.dt = stage, dx, dz, dt
        self.nxpml, self.nzpml, self.allnx, self.allnz = nxpml, nzpml, allnx, allnz
        self.pml, self.nt, self.nop, self.scale = pml, nt, nop, scale
        self.nx, self.nz = nxpml - 2 * pml, nzpml - 2 * pml
        # public fields written by the driver before IMAGE_SINGLESHOT (main.cpp:619-625)
        self.ntr = ntr
        self.isx = self.isz = self.igz = 0
        self.ngx_left = self.delta_left = self.record_left_in_v = 0
        self._keep = []
        self._lens = []  # record length of each queued shot

    # -- lifetime --
    def close(self):
        if getattr(self, "_h", None):
            _lib.load().sfwi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _sync(self):
        _lib.check(_lib.load().sfwi_set_shot_geometry(self._h, self.isx, self.isz, self.igz, self.ngx_left,
                                                      self.delta_left, self.record_left_in_v, self.ntr))

    # -- the reference's methods --
    def GPUbufferVPVS(self, vp_all, vs_all, rho_all=None):
        shp = (self.allnx, self.allnz)
        vp, vs = _f32(vp_all, shp), _f32(vs_all, shp)
        rho = None if rho_all is None else _f32(rho_all, shp)
        _lib.check(_lib.load().sfwi_gpu_buffer_vpvs(self._h, _fp(vp), _fp(vs), _fp(rho)))

    def GPUbufferM(self, pp, ps):
        shp = (self.allnx, self.allnz)
        a, b = _f32(pp, shp), _f32(ps, shp)
        _lib.check(_lib.load().sfwi_gpu_buffer_m(self._h, _fp(a), _fp(b)))

    def bufferVpVsHtoD(self, ngx_min):
        _lib.check(_lib.load().sfwi_buffer_vpvs_htod(self._h, int(ngx_min)))

    def record_copytoGPU(self, record, record_x, gc):
        self._sync()
        rz, rx = _f32(record, (self.ntr, self.nt)), _f32(record_x, (self.ntr, self.nt))
        g = np.ascontiguousarray(gc, dtype=np.int32)
        _lib.check(_lib.load().sfwi_record_copy_to_gpu(self._h, _fp(rz), _fp(rx), _ip(g)))

    def set_misfit(self, kind):
        _lib.check(_lib.load().sfwi_set_misfit(self._h, int(kind)))

    def image_singleshot(self):
        """One shot-gradient; returns this shot's misfit."""
        self._sync()
        m = C.c_double(0.0)
        _lib.check(_lib.load().sfwi_image_singleshot(self._h, C.byref(m)))
        return m.value

    def imagebuffer_resettozero(self):
        """(grad_pp, grad_ps, illumination) as float32 [allnx, allnz]; the
        device accumulators are zeroed."""
        shp = (self.allnx, self.allnz)
        out = [np.zeros(shp, np.float32) for _ in range(3)]
        _lib.check(_lib.load().sfwi_imagebuffer_resettozero(self._h, _fp(out[0]), _fp(out[1]), _fp(out[2]), None,
                                                            None, None, None))
        return tuple(out)

    def read_gradients_f64(self):
        shp = (self.allnx, self.allnz)
        out = [np.zeros(shp, np.float64) for _ in range(3)]
        dp = C.POINTER(C.c_double)
        _lib.check(_lib.load().sfwi_read_gradients_f64(self._h, *[o.ctypes.data_as(dp) for o in out]))
        return tuple(out)

    def set_density_gradient(self, on=True):
        """Also accumulate the density kernel -sum_t v_adj . dv/dt (no
        reference counterpart) in later gradient runs."""
        _lib.check(_lib.load().sfwi_set_density_gradient(self._h, 1 if on else 0))

    def set_snapshots(self, every, fmt="f16"):
        """Image from forward snapshots every `every` steps ("f32", "f16",
        "bf16"; every=0: reconstruction, as the reference)."""
        code = {"f32": SNAP_F32, "f16": SNAP_F16, "bf16": SNAP_BF16}[fmt] if every else 0
        _lib.check(_lib.load().sfwi_set_snapshots(self._h, int(every), code))
        self._snap = (int(every), fmt) if every else None

    def set_cpu_mem(self, cpu_mem, ntt=0):
        """Keep the edge strips of later gradient runs in pinned host memory,
        with a device ring of two chunks of `ntt` steps (IMAGE_SINGLESHOT's
        cpu_mem and ntt); the results are the same bits."""
        _lib.check(_lib.load().sfwi_set_cpu_mem(self._h, 1 if cpu_mem else 0, int(ntt)))

    def strip_bytes(self):
        """(device bytes, pinned host bytes) of the last run's edge strips"""
        dev, host = C.c_size_t(0), C.c_size_t(0)
        _lib.check(_lib.load().sfwi_strip_bytes(self._h, C.byref(dev), C.byref(host)))
        return dev.value, host.value

    def read_density_gradient_f64(self):
        out = np.zeros((self.allnx, self.allnz), np.float64)
        _lib.check(_lib.load().sfwi_read_density_gradient_f64(self._h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def read_records(self, i=0, ntr=None):
        """dict of syn_z, syn_x, syn2_z, syn2_x, res_z, res_x ([ntr, nt]) of
        shot i of the last run."""
        ntr = self.ntr if ntr is None else ntr
        names = ("syn_z", "syn_x", "syn2_z", "syn2_x", "res_z", "res_x")
        out = {k: np.zeros((ntr, self.nt), np.float32) for k in names}
        _lib.check(_lib.load().sfwi_read_records(self._h, i, *[_fp(out[k]) for k in names]))
        return out

    # -- batched shots --
    def _plain_lengths(self):
        """the runs of the handle's own model read [ntr, nt] records of every
        queued shot: a shot queued with another length (for run_models) is
        refused, and the queue dropped"""
        if any(n != self.nt for n in self._lens):
            _lib.load().sfwi_clear_queue(self._h)
            self._keep, self._lens = [], []
            raise SfwiError("a queued shot's records are not [ntr, %d]: shots of other lengths run through "
                            "run_models" % self.nt)

    def enqueue_shot(self, nx, isx, isz, igz, ngx_left, delta_left, record_left_in_v, gc, rec_z=None, rec_x=None,
                     nt=None):
        """Queue a shot; records are [ntr, nt] (nt: the handle's, or the
        shot's model's for run_models)."""
        g = np.ascontiguousarray(gc, dtype=np.int32)
        ntr = int(g.size)
        n = self.nt if nt is None else int(nt)
        rz = _f32(rec_z if rec_z is not None else np.zeros((ntr, n), np.float32), (ntr, n))
        rx = _f32(rec_x if rec_x is not None else np.zeros((ntr, n), np.float32), (ntr, n))
        self._keep += [g, rz, rx]  # must outlive run()
        self._lens.append(n)
        d = ShotDesc(nx=nx, isx=isx, isz=isz, igz=igz, ngx_left=ngx_left, delta_left=delta_left,
                     record_left_in_v=record_left_in_v, ntr=ntr, gc=_ip(g), rec_z=_fp(rz), rec_x=_fp(rx))
        _lib.check(_lib.load().sfwi_enqueue_shot(self._h, C.byref(d)))

    def run(self, nshots=None):
        """Advance all queued shots together; returns (misfit, per-shot misfits)."""
        n = nshots if nshots is not None else len(self._keep) // 3
        per = np.zeros(max(n, 1), np.float64)
        m = C.c_double(0.0)
        self._plain_lengths()
        try:
            _lib.check(_lib.load().sfwi_run(self._h, C.byref(m), per.ctypes.data_as(C.POINTER(C.c_double))))
        finally:
            self._keep, self._lens = [], []
        return m.value, per[:n]

    def born_adjoint(self):
        """L^T d of the Born operator (stage 2) for the queued shots, their
        records being d: (img_vp, img_vs) float64 [allnx, allnz]."""
        shp = (self.allnx, self.allnz)
        ip, isv = np.zeros(shp, np.float64), np.zeros(shp, np.float64)
        dp = C.POINTER(C.c_double)
        self._plain_lengths()
        try:
            _lib.check(_lib.load().sfwi_born_adjoint(self._h, ip.ctypes.data_as(dp), isv.ctypes.data_as(dp)))
        finally:
            self._keep, self._lens = [], []
        return ip, isv

    def hessian_vector(self, dvp, dvs):
        """Gauss-Newton Hessian-vector product L^T L m of the queued shots for
        m = (dvp, dvs) (stage 2; replaces the uploaded perturbation):
        (hv_vp, hv_vs) float64 [allnx, allnz]."""
        shp = (self.allnx, self.allnz)
        dvp, dvs = _f32(dvp, shp), _f32(dvs, shp)
        hp, hs = np.zeros(shp, np.float64), np.zeros(shp, np.float64)
        dp = C.POINTER(C.c_double)
        self._plain_lengths()
        try:
            _lib.check(_lib.load().sfwi_hessian_vector(self._h, _fp(dvp), _fp(dvs), hp.ctypes.data_as(dp),
                                                       hs.ctypes.data_as(dp)))
        finally:
            self._keep, self._lens = [], []
        return hp, hs

    def run_models(self, models, shot_model):
        """One gradient run of the queued shots, shot i on models[shot_model[i]]
        (sfwi_run_models).  `models` are dicts with vp, vs, rho (stage 1),
        optional dvp, dvs ([allnx, allnz] each) and nt.  Returns
        (per_shot_misfit, [(grad_pp, grad_ps, illum, grad_rho) per model]) in
        FP64."""
        descs = (_lib.ModelDesc * len(models))()
        keep = []
        sizes = []
        for d, m in zip(descs, models):
            vp = _f32(m["vp"])
            allnx, allnz = vp.shape
            arrs = {k: (None if m.get(k) is None else _f32(m[k], (allnx, allnz))) for k in ("vs", "rho", "dvp", "dvs")}
            keep.append((vp, arrs))
            d.allnx, d.allnz, d.nt = allnx, allnz, int(m["nt"])
            d.vp = _fp(vp)
            for k, a in arrs.items():
                setattr(d, k, _fp(a))
            sizes.append((allnx, allnz))
        n = sum(a * b for a, b in sizes)
        sm = np.ascontiguousarray(shot_model, dtype=np.int32)
        nq = len(sm)
        per = np.zeros(max(nq, 1), np.float64)
        g = [np.zeros(max(n, 1), np.float64) for _ in range(4)]
        dp = C.POINTER(C.c_double)
        try:
            _lib.check(_lib.load().sfwi_run_models(self._h, len(models), descs, _ip(sm), per.ctypes.data_as(dp),
                                                   *[a.ctypes.data_as(dp) for a in g]))
        finally:
            self._keep, self._lens = [], []
        out, o = [], 0
        for allnx, allnz in sizes:
            k = allnx * allnz
            out.append(tuple(a[o:o + k].reshape(allnx, allnz).copy() for a in g))
            o += k
        return per[:nq], out

    # -- line searches --
    def CALCULATE_ALPHA_parabola_mb(self, grad_pp, grad_ps, step1, step2):
        """Misfits (m0, m1, m2) of the current shot at the trial models
        m - s*grad, s = 0, step1, step2 (stage 1)."""
        g1, g2 = _f32(grad_pp), _f32(grad_ps)
        m = [C.c_double(0.0) for _ in range(3)]
        _lib.check(_lib.load().sfwi_calculate_alpha_parabola_mb(self._h, _fp(g1), _fp(g2), float(step1), float(step2),
                                                               *[C.byref(x) for x in m]))
        return tuple(x.value for x in m)

    def CALCULATE_ALPHA(self, image_pp, image_ps, cg_pp, cg_ps):
        """(fenzi, fenmu) of the current shot (stage 2)."""
        arrs = [_f32(a) for a in (image_pp, image_ps, cg_pp, cg_ps)]
        zi, mu = C.c_double(0.0), C.c_double(0.0)
        _lib.check(_lib.load().sfwi_calculate_alpha(self._h, *[_fp(a) for a in arrs], C.byref(zi), C.byref(mu)))
        return zi.value, mu.value

    def line_search_parabola(self, grad_pp, grad_ps, step1, step2, nshots=None):
        """Queued shots at three trial models: (misfit[3], per_shot[nshots, 3])."""
        n = nshots if nshots is not None else len(self._keep) // 3
        g1, g2 = _f32(grad_pp), _f32(grad_ps)
        m = np.zeros(3, np.float64)
        per = np.zeros((max(n, 1), 3), np.float64)
        dp = C.POINTER(C.c_double)
        self._plain_lengths()
        try:
            _lib.check(_lib.load().sfwi_line_search_parabola(self._h, _fp(g1), _fp(g2), float(step1), float(step2),
                                                             m.ctypes.data_as(dp), per.ctypes.data_as(dp)))
        finally:
            self._keep, self._lens = [], []
        return m, per[:n]

    def line_search_exact(self, image_pp, image_ps, cg_pp, cg_ps, nshots=None):
        """Queued shots: (fenzi, fenmu, per_shot[nshots, 2])."""
        n = nshots if nshots is not None else len(self._keep) // 3
        arrs = [_f32(a) for a in (image_pp, image_ps, cg_pp, cg_ps)]
        zi, mu = C.c_double(0.0), C.c_double(0.0)
        per = np.zeros((max(n, 1), 2), np.float64)
        self._plain_lengths()
        try:
            _lib.check(_lib.load().sfwi_line_search_exact(self._h, *[_fp(a) for a in arrs], C.byref(zi), C.byref(mu),
                                                          per.ctypes.data_as(C.POINTER(C.c_double))))
        finally:
            self._keep, self._lens = [], []
        return zi.value, mu.value, per[:n]

    def run_forward(self):
        self._plain_lengths()
        try:
            _lib.check(_lib.load().sfwi_run_forward(self._h))
        finally:
            self._keep, self._lens = [], []

    def time_kernels(self, reps=20):
        """Average launch duration (ms) of each time-step kernel on the last
        run's batch (overwrites that run's wavefields)."""
        out = np.zeros(4, np.float32)
        _lib.check(_lib.load().sfwi_time_kernels(self._h, int(reps), _fp(out)))
        born = self.stage == 2
        snap = getattr(self, "_snap", None)
        names = ["k_fwd_v<born>" if born else "k_fwd_v", "k_fwd_s<born>" if born else "k_fwd_s",
                 "k_bwd_s_snap<%s>" % snap[1] if snap else "k_bwd_s", "k_bwd_v_snap" if snap else "k_bwd_v"]
        return {n: float(v) for n, v in zip(names, out)}

    def set_tile_shape(self, shape):
        """Tile shape of the step kernels: a name in TILE_SHAPES or its
        index; a batch already on the device is re-tiled."""
        if isinstance(shape, str):
            shape = TILE_SHAPES.index(shape)
        _lib.check(_lib.load().sfwi_set_tile_shape(self._h, int(shape)))

    def debug_grid(self):
        """(arrays [narrays, X, P] float32 of the batch on the device, number
        of state arrays): wavefields, PML memory variables and accumulators
        first, coefficients after."""
        X, P, na, ns = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _lib.check(_lib.load().sfwi_debug_grid_shape(self._h, C.byref(X), C.byref(P), C.byref(na), C.byref(ns)))
        out = np.zeros((na.value, X.value, P.value), np.float32)
        for a in range(na.value):
            _lib.check(_lib.load().sfwi_debug_read_grid(self._h, a, _fp(out[a])))
        return out, ns.value

    def wait_selftest(self, tries=4096):
        """Make the device-side pipeline waits of the last batch's tile
        pipeline run out (bounded, no fault); raises SfwiError carrying the
        timeout report a real run would give."""
        _lib.check(_lib.load().sfwi_wait_selftest(self._h, int(tries)))

    def set_source(self, kind):
        """Source of the forward sweeps: SOURCE_TXX_TZZ (the reference's
        stress source, default) or SOURCE_VZ_FORCE (vertical force)."""
        _lib.check(_lib.load().sfwi_set_source(self._h, int(kind)))

    def set_launch_overlap(self, on=True):
        """Programmatic dependent launch of the time-step kernels (default on)."""
        _lib.check(_lib.load().sfwi_set_launch_overlap(self._h, int(bool(on))))

    def set_tile_order(self, reverse_bits):
        """Bit k: time-step sweep k (forward velocity, forward stress,
        backward stress, backward velocity) draws its tiles in reverse table
        order (default 0b1010).  Results do not depend on it."""
        _lib.check(_lib.load().sfwi_set_tile_order(self._h, int(reverse_bits)))

    def tile_shape(self):
        """Name of the current tile shape (TILE_SHAPES)."""
        s, tx, tz = C.c_int(), C.c_int(), C.c_int()
        _lib.check(_lib.load().sfwi_get_tile_shape(self._h, C.byref(s), C.byref(tx), C.byref(tz)))
        return TILE_SHAPES[s.value]

    def autotune(self, reps=10):
        """Time one step of the four step kernels for every tile shape on the
        last run's batch and keep the fastest; returns (chosen name,
        {name: ms per step}).  Overwrites the last run's wavefields."""
        choice = C.c_int()
        ms = np.zeros(len(TILE_SHAPES), np.float32)
        _lib.check(_lib.load().sfwi_autotune(self._h, int(reps), C.byref(choice), _fp(ms)))
        return TILE_SHAPES[choice.value], {t: float(v) for t, v in zip(TILE_SHAPES, ms)}

    def kernel_launches(self):
        return int(_lib.load().sfwi_kernel_launches(self._h))

    def last_timing(self):
        f, b, o, t = C.c_float(), C.c_float(), C.c_float(), C.c_float()
        _lib.check(_lib.load().sfwi_last_timing(self._h, C.byref(f), C.byref(b), C.byref(o), C.byref(t)))
        return {"forward_ms": f.value, "backward_ms": b.value, "misfit_ms": o.value, "total_ms": t.value}


def set_pinned_cache(nbytes):
    """Keep up to `nbytes` of the pinned host memory that engines release
    (their host-held edge strips) for reuse by later engines; 0 frees it."""
    _lib.check(_lib.load().sfwi_set_pinned_cache(int(nbytes)))


def IMAGE_SINGLESHOT(fdtdgpu, misfit=0.0, *reference_args):
    """IMAGE_SINGLESHOT(fd, misfit) -> misfit + this shot's misfit
    (sfwi-stage1/FD2DGPU.cuh:466-467).  Of the reference's remaining
    arguments (sxnum, nDim, myid, record, record_x, gc, rbc, cpu_mem, ntt,
    iter, ...), cpu_mem and ntt keep the edge strips in host memory
    (set_cpu_mem) and rbc = True (random boundary) is refused; the others
    are MPI bookkeeping or disabled options and are not read."""
    if len(reference_args) >= 7 and reference_args[6]:
        raise SfwiError("IMAGE_SINGLESHOT: the random boundary (rbc) is not provided")
    if len(reference_args) >= 9:
        fdtdgpu.set_cpu_mem(reference_args[7], reference_args[8])
    return misfit + fdtdgpu.image_singleshot()


def _ot(fn, obs_x, obs_z, cal_x, cal_z, dt):
    obs_x, obs_z, cal_x, cal_z = (_f32(a) for a in (obs_x, obs_z, cal_x, cal_z))
    tracenum, length = obs_x.shape
    rx, rz = np.zeros_like(obs_x), np.zeros_like(obs_z)
    m = C.c_double(0.0)
    _lib.check(getattr(_lib.load(), fn)(_fp(obs_x), _fp(obs_z), _fp(cal_x), _fp(cal_z), _fp(rx), _fp(rz), length,
                                        tracenum, dt, C.byref(m)))
    return rx, rz, m.value


def OT(obs_x, obs_z, cal_x, cal_z, dt):
    """1D W2 misfit (exponential weights, per-trace scale) of [tracenum, length]
    gathers; returns (res_x, res_z, misfit)."""
    return _ot("sfwi_ot", obs_x, obs_z, cal_x, cal_z, dt)


def OT_power(obs_x, obs_z, cal_x, cal_z, dt):
    return _ot("sfwi_ot_power", obs_x, obs_z, cal_x, cal_z, dt)


def OT_alltrace(obs_x, obs_z, cal_x, cal_z, dt):
    return _ot("sfwi_ot_alltrace", obs_x, obs_z, cal_x, cal_z, dt)


SNAP_F32, SNAP_F16, SNAP_BF16 = 1, 2, 3
SOURCE_TXX_TZZ, SOURCE_VZ_FORCE = 0, 1
# tile shapes of the step kernels in SFWI_TILE_* order: core cells x by z,
# "x3" for three CTAs per SM, "c2" for two cells per compute thread, "s3"
# for three pipeline stages
TILE_SHAPES = ["16x32", "32x32", "16x64", "8x32x3", "16x32c2", "8x32c2s3"]


class PinnedArray:
    """numpy float32 array in page-locked host memory (sfwi_host_alloc)."""

    def __init__(self, shape):
        n = int(np.prod(shape))
        p = C.c_void_p()
        _lib.check(_lib.load().sfwi_host_alloc(max(n, 1) * 4, C.byref(p)))
        self._p = p
        buf = (C.c_float * max(n, 1)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=np.float32, count=n).reshape(shape)

    def free(self):
        if self._p:
            self.array = None
            _lib.load().sfwi_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def normalize(matrix):
    """In-place division by the largest absolute value (main.cpp:24-32)."""
    a = np.ascontiguousarray(matrix, dtype=np.float32)
    tracenum, length = a.shape
    _lib.check(_lib.load().sfwi_normalize(_fp(a), length, tracenum))
    return a
