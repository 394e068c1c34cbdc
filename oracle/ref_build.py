"""Build recipe for oracle/_ref: the reference's own kernels, compiled for the CPU.

TEST INFRASTRUCTURE ONLY.  Run here, where the reference sources are mounted:

    python oracle/ref_build.py [--src /root/reference]

For each stage it compiles, straight from the reference tree,
  * sfwi-stage{N}/born.cu (the stencil and Born kernels), and
  * the kernels listed in FD2DGPU_KERNELS, cut out of sfwi-stage{N}/FD2DGPU.cu
    in memory and piped to g++ on stdin (that file's host code needs MPI-free
    CUDA, cuBLAS and cuFFT, so it cannot be compiled whole),
as host C++ through oracle/cuda_shim, together with oracle/ref_harness.cpp, and
links oracle/_ref/libsfwi_ref_s{N}.so.

With nvcc present it also compiles the same two sources for sm_103a, with the
reference's own nvcc flags (-O3 -w, sfwi-stage1/Makefile; plus a 64-register
cap so that its 1024-thread launches fit, see NVCC_FLAGS), into device-code
modules oracle/_ref/ref_born_s{N}.cubin and ref_fdk_s{N}.cubin, and writes
oracle/_ref/ref_kernels_s{N}.txt: for every kernel its symbol and the kinds of
its parameters, read from the symbol names of the CPU objects (the kernels'
C++ names are the same in both builds).  oracle/ref_gpu_harness.cpp, compiled
on the GPU machine, loads those modules and runs the reference's kernels there
in the same launch sequence as the CPU harness.

No reference source is written into this repository: only object files,
device-code modules, the symbol lists and the shared libraries land in
oracle/_ref/ (git-ignored).  The recipe needs g++ with OpenMP (and nvcc for the
device modules) and nothing else; it never runs the reference's own Makefile.
"""
import argparse
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

# kernels of FD2DGPU.cu on the shot-gradient path (all overloads of each name)
FD2DGPU_KERNELS = [
    "copyvelocityHtoD", "copypmlVz", "copypmlVx", "dampX", "dampZ",
    "GPUcalculate_elastic_rho_C", "GPUapplysource", "GPUrecord_scatterwavefield",
    "GPU_subtract", "GPU_add", "GPUapplysource_backward_from_record",
    "doimage_gradient", "doimage_illum", "record_edge_wavefield", "load_edge_wavefield",
]

CXXFLAGS = ["-std=c++17", "-O2", "-w", "-fPIC", "-ffp-contract=off", "-fopenmp"]


def strip_comments(src):
    """Blank out // and /* */ comments, keeping newlines and string literals."""
    out = []
    i, n = 0, len(src)
    while i < n:
        c = src[i]
        if c == '"' or c == "'":
            q = c
            j = i + 1
            while j < n and src[j] != q:
                j += 2 if src[j] == "\\" else 1
            out.append(src[i:j + 1])
            i = j + 1
        elif src.startswith("//", i):
            j = src.find("\n", i)
            j = n if j < 0 else j
            out.append(" " * (j - i))
            i = j
        elif src.startswith("/*", i):
            j = src.find("*/", i + 2)
            j = n if j < 0 else j + 2
            out.append(re.sub(r"[^\n]", " ", src[i:j]))
            i = j
        else:
            out.append(c)
            i += 1
    return "".join(out)


def extract_kernels(src, names):
    code = strip_comments(src)
    pieces = []
    for m in re.finditer(r"__global__\s+void\s+(\w+)\s*\(", code):
        if m.group(1) not in names:
            continue
        brace = code.find("{", m.end())
        semi = code.find(";", m.end())
        if brace < 0 or (0 <= semi < brace):
            continue  # a declaration
        depth, j = 0, brace
        while True:
            if code[j] == "{":
                depth += 1
            elif code[j] == "}":
                depth -= 1
                if depth == 0:
                    break
            j += 1
        line = code.count("\n", 0, m.start()) + 1
        pieces.append('#line %d "FD2DGPU.cu"\n' % line + code[m.start():j + 1] + "\n")
    found = {re.match(r'#line \d+ "FD2DGPU.cu"\n__global__\s+void\s+(\w+)', p).group(1) for p in pieces}
    missing = set(names) - found
    if missing:
        raise RuntimeError("kernels not found in FD2DGPU.cu: %s" % sorted(missing))
    return "".join(pieces)


def run(cmd, stdin=None):
    r = subprocess.run(cmd, input=stdin, text=True, capture_output=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("compile failed")


def build_stage(src_root, stage, cxx="g++"):
    sdir = os.path.join(src_root, "sfwi-stage%d" % stage)
    inc = ["-I", sdir, "-I", os.path.join(HERE, "cuda_shim"), "-I", HERE]
    born_o = os.path.join(OUT, "born_s%d.o" % stage)
    run([cxx] + CXXFLAGS + inc + ["-x", "c++", "-c", os.path.join(sdir, "born.cu"), "-o", born_o])
    with open(os.path.join(sdir, "FD2DGPU.cu"), encoding="latin-1") as f:
        kernels = extract_kernels(f.read(), FD2DGPU_KERNELS)
    tu = '#include "FD2DGPU.cuh"\n' + kernels + '#include "ref_harness.cpp"\n'
    harness_o = os.path.join(OUT, "harness_s%d.o" % stage)
    run([cxx] + CXXFLAGS + inc + ["-DSFWI_STAGE=%d" % stage, "-x", "c++", "-c", "-", "-o", harness_o], stdin=tu)
    lib = os.path.join(OUT, "libsfwi_ref_s%d.so" % stage)
    run([cxx, "-shared", "-fopenmp", "-o", lib, harness_o, born_o])
    return lib


# The reference's nvcc flags (-O3 -w, sfwi-stage1/Makefile) plus a 64-register
# cap: the reference launches every grid kernel as 32x32 = 1024 threads, and
# for sm_103a nvcc gives GPUcalculate_elastic_vx_vz_back 86 registers, which
# a 1024-thread block cannot get ("too many resources requested for launch";
# the reference checks no launch, so its adjoint velocity update would not
# run).  The cap changes register allocation only, not the arithmetic.
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w", "-DELASTIC", "-maxrregcount=64"]
# kernels the launch sequence (oracle/ref_sequence.inc) runs
SEQUENCE_KERNELS = [
    "copyvelocityHtoD", "copypmlVz", "copypmlVx", "dampX", "dampZ", "GPUcalculate_elastic_rho_C",
    "GPUapplysource", "update_vx_vz", "update_txx_tzz_txz", "add_born_source_components",
    "GPUrecord_scatterwavefield", "record_edge_wavefield", "GPU_subtract", "GPU_add", "load_edge_wavefield",
    "update_txx_tzz_txz_grad", "GPUapplysource_backward_from_record", "GPUcalculate_elastic_txx_tzz_txz_back",
    "GPUcalculate_elastic_vx_vz_back", "doimage_gradient", "doimage_illum",
]
_BUILTIN = {"i": "i", "j": "i", "f": "f", "d": "d", "b": "b", "c": "c", "h": "c", "l": "l", "m": "l", "x": "l",
            "y": "l", "s": "s", "t": "s"}


def param_kinds(mangled):
    """(name, [kind...]) of a function symbol in the Itanium C++ ABI, for the
    parameter types kernels take: builtins, pointers, const and
    substitutions.  Kinds: p pointer, i 32-bit integer, f float, d double,
    b bool, c char, s short, l 64-bit integer."""
    m = re.match(r"_Z(\d+)", mangled)
    if not m:
        raise ValueError(mangled)
    n = int(m.group(1))
    pos = m.end()
    name = mangled[pos:pos + n]
    pos += n
    subs, kinds = [], []

    def parse(i):
        c = mangled[i]
        if c in _BUILTIN:
            return _BUILTIN[c], i + 1
        if c in "PK":
            k, j = parse(i + 1)
            subs.append("p" if c == "P" else k)
            return ("p" if c == "P" else k), j
        if c == "S":
            j = mangled.index("_", i)
            seq = mangled[i + 1:j]
            idx = 0 if seq == "" else int(seq, 36) + 1
            return subs[idx], j + 1
        raise ValueError("unsupported type code %r in %s" % (c, mangled))

    while pos < len(mangled):
        k, pos = parse(pos)
        kinds.append(k)
    return name, kinds


def kernel_symbols(objs, names):
    """Symbols of the named kernels (every overload) defined in `objs`."""
    out = {}
    for o in objs:
        r = subprocess.run(["nm", "-g", "--defined-only", o], capture_output=True, text=True, check=True)
        for line in r.stdout.splitlines():
            parts = line.split()
            if len(parts) != 3 or parts[1] != "T" or not parts[2].startswith("_Z"):
                continue
            try:
                name, kinds = param_kinds(parts[2])
            except (ValueError, IndexError):
                continue
            if name in names:
                out[parts[2]] = (name, kinds)
    missing = set(names) - {v[0] for v in out.values()}
    if missing:
        raise RuntimeError("kernels not found in the CPU objects: %s" % sorted(missing))
    return out


def build_stage_gpu(src_root, stage, nvcc):
    """Device-code modules of the stage's kernels and their symbol list."""
    sdir = os.path.join(src_root, "sfwi-stage%d" % stage)
    born_cubin = os.path.join(OUT, "ref_born_s%d.cubin" % stage)
    run([nvcc, "-cubin"] + NVCC_FLAGS + ["-I", sdir, os.path.join(sdir, "born.cu"), "-o", born_cubin])
    with open(os.path.join(sdir, "FD2DGPU.cu"), encoding="latin-1") as f:
        kernels = extract_kernels(f.read(), FD2DGPU_KERNELS)
    # the cut-out kernels go through a scratch file outside the repository
    tmp = tempfile.mkdtemp(prefix="sfwi_ref_")
    try:
        tu = os.path.join(tmp, "fdk.cu")
        with open(tu, "w") as f:
            f.write('#include "FD2DGPU.cuh"\n' + kernels)
        run([nvcc, "-cubin"] + NVCC_FLAGS + ["-I", sdir, tu, "-o", os.path.join(OUT, "ref_fdk_s%d.cubin" % stage)])
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    syms = kernel_symbols([os.path.join(OUT, "born_s%d.o" % stage), os.path.join(OUT, "harness_s%d.o" % stage)],
                          set(SEQUENCE_KERNELS))
    lst = os.path.join(OUT, "ref_kernels_s%d.txt" % stage)
    with open(lst, "w") as f:
        for sym in sorted(syms):
            name, kinds = syms[sym]
            module = "born" if sym in born_symbols(stage) else "fdk"
            f.write("%s %s %s %s\n" % (name, module, sym, "".join(kinds)))
    return lst


def born_symbols(stage):
    r = subprocess.run(["nm", "-g", "--defined-only", os.path.join(OUT, "born_s%d.o" % stage)], capture_output=True,
                       text=True, check=True)
    return {l.split()[2] for l in r.stdout.splitlines() if len(l.split()) == 3}


# where the reference tree is mounted (override with SFWI_REFERENCE_SRC)
DEFAULT_SRC = os.environ.get("SFWI_REFERENCE_SRC", "/root/reference")


def sources_present(src=DEFAULT_SRC):
    return os.path.isdir(os.path.join(src, "sfwi-stage1"))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=DEFAULT_SRC)
    a = ap.parse_args(argv)
    if not os.path.isdir(os.path.join(a.src, "sfwi-stage1")):
        print("reference sources not found at %s; oracle/_ref not built" % a.src)
        return 1
    os.makedirs(OUT, exist_ok=True)
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    for stage in (1, 2):
        print(build_stage(a.src, stage))
        if nvcc:
            print(build_stage_gpu(a.src, stage, nvcc))
    return 0


if __name__ == "__main__":
    sys.exit(main())
