"""The class-shaped interface (include/FD2DGPU_compat.hpp) through a C++
caller written in the reference drivers' call order.

tests/compat/compat_driver.cpp follows sfwi-stage1/main.cpp:534-635 and
:1100-1186 (sfwi-stage2/main.cpp:497-594 and :770-850): the FD2DGPU_ELASTIC
constructor, GPUbufferVPVS, GPUbufferM, then per shot record_copytoGPU,
bufferVpVsHtoD, the public fields and IMAGE_SINGLESHOT, then
imagebuffer_resettozero and a line search per shot.  It is compiled here
against the header and libsfwi_gb300.so.  Without a GPU the first call that
needs the device throws, and the caller reports the library's error code;
on the GPU its gradients, misfits and line-search sums equal, bit for bit,
the same sequence run through the C ABI from Python.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests.golden.make_golden import load_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "compat", "compat_driver.cpp")


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime_api.h")):
            return os.path.join(d, "include")
    pytest.skip("CUDA headers not found")


def _build(tmp_path):
    from sfwi_gb300 import build as b
    lib = b.build()
    cxx = shutil.which("g++") or pytest.skip("no C++ compiler")
    exe = str(tmp_path / "compat_driver")
    libdir = os.path.dirname(lib)
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", _cuda_include(),
                        SRC, "-o", exe, "-L", libdir, "-lsfwi_gb300", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _shots(case):
    """two shots of a golden case: its own and one with the source 5 nodes over"""
    shot, inputs, _ = load_case(case)
    other = dict(shot, isx=shot["isx"] + 5)
    return shot, inputs, [shot, other]


def _direction(inputs, seed):
    rng = np.random.default_rng(seed)
    n = inputs["vp"].shape
    g_pp = (0.01 * inputs["vp"] * rng.uniform(0.5, 1.0, n)).astype(np.float32)
    g_ps = (0.5 * g_pp).astype(np.float32)
    return g_pp, g_ps


def _write_case(d, case, rbc=0, steps=(0.5, 1.0)):
    shot, inputs, shots = _shots(case)
    stage = shot["stage"]
    pml = shot["pml"]
    g_pp, g_ps = _direction(inputs, 1)
    lines = ["%d %d %d %d %d %d %d %d %r %r %r %d %d" % (
        stage, shot["allnx"], shot["allnz"], shot["nx"] + 2 * pml, shot["allnz"] + 2 * pml, pml, shot["nt"],
        shot["ntr"], shot["dx"], shot["dz"], shot["dt"], rbc, len(shots))]
    for k, s in enumerate(shots):
        lines.append("%d %d %d %d %d %d %d" % (s["ntr"], s["ngx_left"], s["delta_left"], s["record_left_in_v"],
                                               s["isx"], s["isz"], s["igz"]))
        inputs["obs_z"].astype(np.float32).tofile(os.path.join(d, "shot%d_z.bin" % k))
        inputs["obs_x"].astype(np.float32).tofile(os.path.join(d, "shot%d_x.bin" % k))
        np.asarray(inputs["gc"], np.int32).tofile(os.path.join(d, "shot%d_gc.bin" % k))
    lines.append("%r %r" % steps)
    with open(os.path.join(d, "params.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    for name in ("sou", "vp", "vs", "rho", "dvp", "dvs"):
        if name in inputs:
            np.asarray(inputs[name], np.float32).tofile(os.path.join(d, name + ".bin"))
    g_pp.tofile(os.path.join(d, "dir_pp.bin"))
    g_ps.tofile(os.path.join(d, "dir_ps.bin"))
    return shot, inputs, shots, (g_pp, g_ps)


def _has_gpu():
    return os.path.exists("/dev/nvidia0") or os.path.exists("/dev/nvidiactl")


def test_compat_header_compiles_and_reports_errors_without_a_device(tmp_path):
    if _has_gpu():
        pytest.skip("a GPU is present: the no-device path is not reachable")
    exe = _build(tmp_path)
    _write_case(str(tmp_path), "s1_window")
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 3, (r.returncode, r.stdout, r.stderr)
    assert "error -5" in r.stderr  # SFWI_E_NODEVICE from the first call that needs the device


def _python_sequence(case, shots, inputs, direction, steps):
    import sfwi_gb300 as sg
    from tests.helpers import make_engine
    shot = shots[0]
    fd = make_engine(shot, inputs)
    misfit = 0.0
    for s in shots:
        fd.ntr = s["ntr"]
        fd.isx, fd.isz, fd.igz = s["isx"], s["isz"], s["igz"]
        fd.ngx_left, fd.delta_left, fd.record_left_in_v = s["ngx_left"], s["delta_left"], s["record_left_in_v"]
        fd.record_copytoGPU(inputs["obs_z"], inputs["obs_x"], inputs["gc"])
        fd.bufferVpVsHtoD(s["delta_left"] + s["record_left_in_v"])
        misfit = sg.IMAGE_SINGLESHOT(fd, misfit)
    gpp, gps, ill = fd.imagebuffer_resettozero()
    ls = [0.0] * 5
    for s in shots:
        fd.isx = s["isx"]
        fd.record_copytoGPU(inputs["obs_z"], inputs["obs_x"], inputs["gc"])
        fd.bufferVpVsHtoD(s["delta_left"] + s["record_left_in_v"])
        if shot["stage"] == 1:
            m = fd.CALCULATE_ALPHA_parabola_mb(direction[0], direction[1], steps[0], steps[1])
            for i in range(3):
                ls[i] += m[i]
        else:
            zi, mu = fd.CALCULATE_ALPHA(inputs["dvp"], inputs["dvs"], direction[0], direction[1])
            ls[3] += zi
            ls[4] += mu
    fd.close()
    return gpp, gps, ill, [misfit] + ls


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["s1_window", "s2_window"])
def test_compat_caller_equals_the_c_abi(tmp_path, case):
    exe = _build(tmp_path)
    steps = (0.5, 1.0)
    shot, inputs, shots, direction = _write_case(str(tmp_path), case, steps=steps)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    n = shot["allnx"] * shot["allnz"]
    out = [np.fromfile(str(tmp_path / f), np.float32, n).reshape(shot["allnx"], shot["allnz"])
           for f in ("out_grad_pp.bin", "out_grad_ps.bin", "out_illum.bin")]
    with open(tmp_path / "out.txt") as f:
        nums = [float(x) for x in f.read().split()]
    gpp, gps, ill, ref = _python_sequence(case, shots, inputs, direction, steps)
    assert np.array_equal(out[0], gpp) and np.array_equal(out[1], gps) and np.array_equal(out[2], ill)
    assert np.abs(gpp).max() > 0
    assert nums == ref, (nums, ref)
    if shot["stage"] == 1:
        assert nums[2] != nums[1]  # the trial models give different misfits
    else:
        assert nums[5] > 0


@pytest.mark.gpu
def test_compat_random_boundary_is_refused(tmp_path):
    exe = _build(tmp_path)
    _write_case(str(tmp_path), "s1_window", rbc=1)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 3
    assert "error -1" in r.stderr and "random boundary" in r.stderr
