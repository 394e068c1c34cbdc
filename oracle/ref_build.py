"""Build recipe for oracle/_ref: the reference's own kernels, compiled for the CPU.

TEST INFRASTRUCTURE ONLY.  Run here, where the reference sources are mounted:

    python oracle/ref_build.py [--src /root/reference]

For each stage it compiles, straight from the reference tree,
  * sfwi-stage{N}/born.cu (the stencil and Born kernels), and
  * the kernels listed in FD2DGPU_KERNELS, cut out of sfwi-stage{N}/FD2DGPU.cu
    in memory and piped to g++ on stdin (that file's host code needs MPI-free
    CUDA, cuBLAS and cuFFT, so it cannot be compiled whole),
as host C++ through oracle/cuda_shim, together with oracle/ref_harness.cpp, and
links oracle/_ref/libsfwi_ref_s{N}.so.  No reference source is written into
this repository: only object files and the two shared libraries land in
oracle/_ref/ (git-ignored).  The recipe needs g++ with OpenMP and nothing else;
it never runs the reference's own Makefile.
"""
import argparse
import os
import re
import subprocess
import sys

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


DEFAULT_SRC = "/root/reference"


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
    for stage in (1, 2):
        print(build_stage(a.src, stage))
    return 0


if __name__ == "__main__":
    sys.exit(main())
