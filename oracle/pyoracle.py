"""ctypes front end of the oracle libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the sfwi_gb300 package.

Libraries (built by build() into oracle/lib, and by oracle/ref_build.py into
oracle/_ref where the reference sources are mounted):
  "f64"  oracle/lib/liboracle64.so  FP64 restatement (sfwi_oracle.c)
  "f32"  oracle/lib/liboracle32.so  FP32 transliteration (same source)
  "ref1" oracle/_ref/libsfwi_ref_s1.so  the reference's stage-1 kernels on the CPU
  "ref2" oracle/_ref/libsfwi_ref_s2.so  the reference's stage-2 kernels on the CPU
  "gpu1" oracle/_ref/libsfwi_refgpu_s1.so  the reference's stage-1 kernels on the GPU
  "gpu2" oracle/_ref/libsfwi_refgpu_s2.so  the reference's stage-2 kernels on the GPU
The "gpu" libraries are built on the GPU machine by build_refgpu() from
oracle/ref_gpu_harness.cpp and the device-code modules that oracle/ref_build.py
left in oracle/_ref.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")
REFDIR = os.path.join(HERE, "_ref")

_PATHS = {
    "f64": os.path.join(LIBDIR, "liboracle64.so"),
    "f32": os.path.join(LIBDIR, "liboracle32.so"),
    "ref1": os.path.join(REFDIR, "libsfwi_ref_s1.so"),
    "ref2": os.path.join(REFDIR, "libsfwi_ref_s2.so"),
    "gpu1": os.path.join(REFDIR, "libsfwi_refgpu_s1.so"),
    "gpu2": os.path.join(REFDIR, "libsfwi_refgpu_s2.so"),
}
_PREFIX = {"f64": "orc64_", "f32": "orc32_", "ref1": "sfwi_ref_", "ref2": "sfwi_ref_", "gpu1": "sfwi_refgpu_",
           "gpu2": "sfwi_refgpu_"}
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def refgpu_modules_present():
    return all(os.path.exists(os.path.join(REFDIR, f % st)) for st in (1, 2)
               for f in ("ref_born_s%d.cubin", "ref_fdk_s%d.cubin", "ref_kernels_s%d.txt"))


def build_refgpu(force=False):
    """Compile oracle/ref_gpu_harness.cpp into oracle/_ref/libsfwi_refgpu_s{1,2}.so
    where the reference's device-code modules are present; returns whether
    both libraries exist afterwards."""
    if not refgpu_modules_present():
        return False
    src = os.path.join(HERE, "ref_gpu_harness.cpp")
    deps = [src, os.path.join(HERE, "ref_sequence.inc"), os.path.join(HERE, "sfwi_oracle.h")]
    for st in (1, 2):
        out = _PATHS["gpu%d" % st]
        if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
            continue
        subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-DSFWI_STAGE=%d" % st, "-I", HERE,
                        "-I", os.path.join(CUDA_HOME, "include"), src, "-o", out,
                        "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart_static", "-ldl", "-lpthread", "-lrt",
                        "-L", os.path.join(CUDA_HOME, "lib64", "stubs"), "-lcuda"], check=True)
    return all(os.path.exists(_PATHS["gpu%d" % st]) for st in (1, 2))


class Shot(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("stage", "allnx", "allnz", "nx", "pml", "nop", "nt", "ntr")] + \
               [(n, C.c_float) for n in ("dx", "dz", "dt")] + \
               [(n, C.c_int) for n in ("isx", "isz", "igz", "ngx_left", "delta_left", "record_left_in_v",
                                       "forward_only", "misfit_kind", "nthreads", "snap_every", "src_kind")]


_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)


class IO(C.Structure):
    _fields_ = [("vp_all", _fp), ("vs_all", _fp), ("rho_all", _fp), ("dvp_all", _fp), ("dvs_all", _fp),
                ("sou", _fp), ("obs_z", _fp), ("obs_x", _fp), ("gc", C.POINTER(C.c_int)),
                ("syn_z", _dp), ("syn_x", _dp), ("syn2_z", _dp), ("syn2_x", _dp),
                ("res_z", _dp), ("res_x", _dp), ("grad_pp", _dp), ("grad_ps", _dp), ("illum", _dp),
                ("grad_rho", _dp), ("misfit", _dp)]


def build(force=False):
    """Compile sfwi_oracle.c twice (FP64 and FP32) into oracle/lib."""
    os.makedirs(LIBDIR, exist_ok=True)
    src = os.path.join(HERE, "sfwi_oracle.c")
    for real, prefix, key in (("double", "orc64_", "f64"), ("float", "orc32_", "f32")):
        out = _PATHS[key]
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            continue
        subprocess.run(["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                        "-DORC_REAL=%s" % real, "-DORC_PREFIX=%s" % prefix, "-I", HERE,
                        "-o", out, src, "-lm"], check=True)


def available(kind):
    return os.path.exists(_PATHS[kind])


_LIBS = {}


def load(kind):
    if kind not in _LIBS:
        lib = C.CDLL(_PATHS[kind])
        f = getattr(lib, _PREFIX[kind] + "image_singleshot")
        f.argtypes = [C.POINTER(Shot), C.POINTER(IO)]
        f.restype = C.c_int
        if kind.startswith("gpu"):
            lib.sfwi_refgpu_error.restype = C.c_char_p
            lib.sfwi_refgpu_init.argtypes = [C.c_char_p]
            if lib.sfwi_refgpu_init(REFDIR.encode()) != 0:
                raise RuntimeError("reference GPU kernels: %s" % lib.sfwi_refgpu_error().decode())
        _LIBS[kind] = lib
    return _LIBS[kind]


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def ricker(nt, dt, f0):
    lib = C.CDLL(_PATHS["f64"])
    w = np.zeros(nt, np.float32)
    lib.orc64_ricker(_p(w, C.c_float), C.c_int(nt), C.c_float(dt), C.c_float(f0))
    return w


def run_shot(kind, shot, model, want_rho=False):
    """Run one shot-gradient.  `shot` is a dict of Shot fields; `model` holds
    vp, vs, rho, dvp, dvs ([allnx, allnz]), sou [nt], obs_z, obs_x [ntr, nt],
    gc [ntr].  Returns a dict of float64 numpy arrays."""
    lib = load(kind)
    s = Shot(**{k: shot[k] for k, _ in Shot._fields_ if k in shot})
    nt, ntr = shot["nt"], shot["ntr"]
    allnx, allnz = shot["allnx"], shot["allnz"]
    keep = {}

    def inp(name, shape=None):
        a = model.get(name)
        if a is None:
            return None
        a = _f32(a)
        keep[name] = a
        return a

    vp, vs, rho = inp("vp"), inp("vs"), inp("rho")
    if rho is None:
        rho = keep["rho"] = np.full_like(vp, 2000.0)
    dvp, dvs = inp("dvp"), inp("dvs")
    sou = inp("sou")
    obs_z = inp("obs_z") if model.get("obs_z") is not None else np.zeros((ntr, nt), np.float32)
    obs_x = inp("obs_x") if model.get("obs_x") is not None else np.zeros((ntr, nt), np.float32)
    keep["obs_z"], keep["obs_x"] = obs_z, obs_x
    gc = np.ascontiguousarray(model["gc"], dtype=np.int32)
    out = {k: np.zeros((ntr, nt)) for k in ("syn_z", "syn_x", "syn2_z", "syn2_x", "res_z", "res_x")}
    for k in ("grad_pp", "grad_ps", "illum"):
        out[k] = np.zeros((allnx, allnz))
    if want_rho:
        out["grad_rho"] = np.zeros((allnx, allnz))
    misfit = np.zeros(1)
    io = IO(vp_all=_p(vp, C.c_float), vs_all=_p(vs, C.c_float), rho_all=_p(rho, C.c_float),
            dvp_all=_p(dvp, C.c_float), dvs_all=_p(dvs, C.c_float), sou=_p(sou, C.c_float),
            obs_z=_p(obs_z, C.c_float), obs_x=_p(obs_x, C.c_float), gc=_p(gc, C.c_int),
            misfit=_p(misfit, C.c_double))
    for k, v in out.items():
        setattr(io, k, _p(v, C.c_double))
    rc = getattr(lib, _PREFIX[kind] + "image_singleshot")(C.byref(s), C.byref(io))
    if rc != 0:
        why = lib.sfwi_refgpu_error().decode() if kind.startswith("gpu") else ""
        raise RuntimeError("%s image_singleshot returned %d %s" % (kind, rc, why))
    out["misfit"] = float(misfit[0])
    return out


def ot_gather(kind, dt, obs_x, obs_z, cal_x, cal_z):
    """Oracle OT misfit (kind 1..3) of a gather [ntr, nt]; returns
    (misfit, res_x, res_z) in float64."""
    lib = C.CDLL(_PATHS["f64"])
    obs_x, obs_z, cal_x, cal_z = map(_f32, (obs_x, obs_z, cal_x, cal_z))
    ntr, nt = obs_x.shape
    rx, rz = np.zeros((ntr, nt)), np.zeros((ntr, nt))
    m = np.zeros(1)
    lib.orc64_ot_gather(C.c_int(kind), C.c_float(dt), _p(obs_x, C.c_float), _p(obs_z, C.c_float),
                        _p(cal_x, C.c_float), _p(cal_z, C.c_float), _p(rx, C.c_double), _p(rz, C.c_double),
                        C.c_int(nt), C.c_int(ntr), _p(m, C.c_double))
    return float(m[0]), rx, rz
