"""Build the CUDA library in-tree: sfwi_gb300/lib/libsfwi_gb300.so, plus the
host library libsfwi_host.so and the sfwi_fwi driver next to it.

    python -m sfwi_gb300.build

Each .cu under sfwi_gb300/csrc is compiled for sm_103a in parallel and linked
into one shared library with the C ABI of include/sfwi_gb300.h.  The step
kernels (sfwi_kernels.cu) are compiled once per tile shape into their own
namespace; the engine picks one of them at run time (sfwi_autotune).
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libsfwi_gb300.so")
OBJDIR = os.path.join(ROOT, "_build", "obj")
# (source, object, defines): the step kernels once per tile shape (core
# TX x TZ cells, CTAs per SM, pipeline stages per CTA, cells per compute
# thread, name), then the rest
TILE_SHAPES = [(16, 32, 2, 2, 4, "16x32"), (32, 32, 1, 2, 4, "32x32"), (16, 64, 1, 2, 4, "16x64"),
               (8, 32, 3, 2, 4, "8x32x3"), (16, 32, 2, 2, 2, "16x32c2"), (8, 32, 2, 3, 2, "8x32c2s3")]
# The step kernels build with -fmad=false: the compiler would otherwise fuse a
# multiply into a following add where the product has no other use, so one
# cell's update could round differently in a tile with PML cells (where the
# products also feed the split update) than in an interior tile.  Every fused
# multiply-add in them is written out (fma intrinsics), so results do not
# depend on the tile shape.
UNITS = [("sfwi_kernels.cu", "sfwi_kernels_%s.o" % n,
          ["-fmad=false",
           "-DSFWI_TILE_X=%d" % tx, "-DSFWI_TILE_Z=%d" % tz, "-DSFWI_CTAS=%d" % c, "-DSFWI_STAGES=%d" % ns,
           "-DSFWI_CPT=%d" % cpt, "-DSFWI_VARIANT_NS=v%s" % n, "-DSFWI_VARIANT_FN=tile_variant_%s" % n])
         for tx, tz, c, ns, cpt, n in TILE_SHAPES]
UNITS += [(f, f.replace(".cu", ".o"), []) for f in ("sfwi_aux.cu", "sfwi_ot.cu", "sfwi_adjoint.cu", "sfwi_engine.cu")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "sfwi_gb300.h"))
    headers.append(os.path.abspath(__file__))  # the flags and the unit list
    nv = nvcc()

    def compile_one(unit):
        src, obj, defs = unit
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, obj)
        if force or _stale(o, [s] + headers):
            cmd = [nv] + ARCH + FLAGS + defs + ["-c", s, "-o", o]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
            if verbose:
                sys.stdout.write(r.stdout + r.stderr)
        return o

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    if force or _stale(LIB, objs):
        cmd = [nv] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    build_host(force)
    return LIB


HOST = os.path.join(HERE, "host")
HOST_LIB = os.path.join(LIBDIR, "libsfwi_host.so")
DRIVER = os.path.join(LIBDIR, "sfwi_fwi")
# host code: the same results on x86 and Arm (no contraction into FMA)
CXXFLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-Wall"]


def build_host(force=False):
    """The host library (SU I/O, shot index, parameter files) and the
    sfwi_fwi inversion driver, with the system C++ compiler."""
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    src = os.path.join(HOST, "sfwi_host.cpp")
    hdr = [os.path.join(HOST, "sfwi_host.h"), os.path.join(ROOT, "include", "sfwi_gb300.h")]
    if force or _stale(HOST_LIB, [src] + hdr):
        r = subprocess.run([cxx] + CXXFLAGS + ["-fPIC", "-shared", "-o", HOST_LIB, src], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("host library failed:\n%s%s" % (r.stdout, r.stderr))
    drv = os.path.join(HOST, "sfwi_fwi.cpp")
    if force or _stale(DRIVER, [drv, HOST_LIB, LIB] + hdr):
        cmd = [cxx] + CXXFLAGS + ["-o", DRIVER, drv, "-L", LIBDIR, "-lsfwi_host", "-lsfwi_gb300",
                                  "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver failed:\n%s%s" % (r.stdout, r.stderr))
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
