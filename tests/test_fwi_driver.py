"""The sfwi_fwi inversion driver end to end on a small synthetic survey: SU
records modelled on a true model, a z-smoothed start model, two stage-1
iterations and two stage-2 iterations through the C ABI.  The first
iteration's gradient is the one the Python API gives for the same shots, and
the stage-1 misfit decreases."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _survey(tmp_path):
    import sfwi_gb300 as sg
    from sfwi_gb300 import su, synth
    allnx, allnz, pml, nt, dx, dt = 90, 56, 10, 360, 10.0, 1e-3
    # the drivers keep the top 26 layers at vp[0][0] (the reference's cut
    # layer): a homogeneous near-surface over a layered target
    vp, vs, _ = synth.layered_model(allnx, allnz, dx, vmin=1800.0, vmax=3200.0)
    vp[:, :26] = 1800.0
    vs = (vp / 1.73).astype(np.float32)
    vp0 = synth.smooth_z(vp, 4)
    vp0[:, :26] = 1800.0
    vs0 = (vp0 / 1.73).astype(np.float32)
    rho = np.full_like(vp, 2000.0)
    sou = synth.ricker(nt, dt, 20.0)
    shots = synth.config_shots(allnx, dx, pml, 3, spacing=30, first=15)
    fd = sg.FD2DGPU_ELASTIC(sou, dx, dx, dt, allnx + 2 * pml, allnz + 2 * pml, allnx, allnz, 1, pml, nt, 4,
                            shots[0]["ntr"], stage=1)
    fd.GPUbufferVPVS(vp, vs, rho)
    for d in shots:
        fd.enqueue_shot(d["nx"], d["isx"], pml + 30, pml + 26, d["ngx_left"], d["delta_left"], 0, d["gc"])
    fd.run_forward()
    rz, rx = str(tmp_path / "record-z.su"), str(tmp_path / "record-x.su")
    for i, d in enumerate(shots):
        r = fd.read_records(i, d["ntr"])
        su.write(rz, d["sx"], d["gc"], r["syn_z"], dt, append=i > 0)
        su.write(rx, d["sx"], d["gc"], r["syn_x"], dt, append=i > 0)
    fd.close()
    vp0.tofile(str(tmp_path / "vp0.bin"))
    vs0.tofile(str(tmp_path / "vs0.bin"))
    out = tmp_path / "out"
    (tmp_path / "para").write_text("%g %g %d %d %d 1 3\n%s\n%s\n%s\n%s\n%s\n%s\n20 2 0\n30 26\n1 0 0 1000\n" % (
        dx, dx, pml, allnx, allnz, tmp_path / "vp0.bin", tmp_path / "vs0.bin", tmp_path / "vs0.bin", rz, rx, out))
    return dict(allnx=allnx, allnz=allnz, pml=pml, nt=nt, dx=dx, dt=dt, sou=sou, vp0=vp0, vs0=vs0, shots=shots,
                rz=rz, rx=rx, out=str(out), para=str(tmp_path / "para"))


def test_stage1_and_stage2_drivers(tmp_path):
    import sfwi_gb300 as sg
    from sfwi_gb300 import su
    s = _survey(tmp_path)
    r = subprocess.run([su.DRIVER, s["para"], "--stage", "1", "--iters", "2"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    log = open(os.path.join(s["out"], "misfit.txt")).read()
    m = [float(l.split("misfit = ")[1].split(",")[0]) for l in log.splitlines() if "misfit =" in l]
    assert len(m) == 2 and m[1] < m[0], log
    shape = (s["allnx"], s["allnz"])
    g0 = np.fromfile(os.path.join(s["out"], "sum_grad_pp_0_%d_%d.dat" % shape), np.float32).reshape(shape)
    v1 = np.fromfile(os.path.join(s["out"], "vel_p_1_%d_%d.dat" % shape), np.float32).reshape(shape)
    assert np.all(np.isfinite(v1)) and not np.array_equal(v1, s["vp0"])
    # the same gradient through the Python API, shots read back from the SU files
    nt, dt, table = su.index(s["rz"])
    pml = s["pml"]
    fd = sg.FD2DGPU_ELASTIC(s["sou"], s["dx"], s["dx"], dt, s["allnx"] + 2 * pml, s["allnz"] + 2 * pml, s["allnx"],
                            s["allnz"], 1, pml, nt, 4, table[0]["ntr"], stage=1)
    fd.GPUbufferVPVS(s["vp0"], s["vs0"], np.full_like(s["vp0"], 2000.0))
    for t, d in zip(table, s["shots"]):
        z, gc = su.read(s["rz"], t["pos"], t["ntr"], nt)
        x, _ = su.read(s["rx"], t["pos"], t["ntr"], nt)
        fd.enqueue_shot(d["nx"], d["isx"], pml + 30, pml + 26, d["ngx_left"], d["delta_left"], 0, gc, z, x)
    fd.run()
    gpp, _, _ = fd.imagebuffer_resettozero()
    fd.close()
    # the driver forms its wavelet with the C library's exp and the Python
    # side with numpy's: a few samples differ in the last place
    assert np.linalg.norm(gpp - g0) <= 1e-5 * np.linalg.norm(g0)
    # stage 2 from the stage-1 model
    v1.tofile(s["para"] + ".vp")
    txt = open(s["para"]).read().replace(str(tmp_path / "vp0.bin"), s["para"] + ".vp")
    open(s["para"], "w").write(txt.replace(s["out"], s["out"] + "2"))
    r = subprocess.run([su.DRIVER, s["para"], "--stage", "2", "--iters", "2"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    img = np.fromfile(os.path.join(s["out"] + "2", "sum_image_pp_1_%d_%d.dat" % shape), np.float32)
    assert np.all(np.isfinite(img)) and np.abs(img).max() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [["--misfit", "ot"], ["--snapshots", "4", "f16"], ["--source", "vz"],
                                  ["--misfit", "ot_alltrace", "--snapshots", "2", "bf16"]])
def test_driver_options(tmp_path, opts):
    """The driver's misfit, snapshot and source options: two stage-1
    iterations run and write finite, updated models; with the L2 misfit and
    the source the observed data were modelled with, the misfit decreases."""
    from sfwi_gb300 import su
    s = _survey(tmp_path)
    r = subprocess.run([su.DRIVER, s["para"], "--stage", "1", "--iters", "2"] + opts, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    log = open(os.path.join(s["out"], "misfit.txt")).read()
    m = [float(l.split("misfit = ")[1].split(",")[0]) for l in log.splitlines() if "misfit =" in l]
    assert len(m) == 2 and all(np.isfinite(m)), log
    if "--misfit" not in opts and "--source" not in opts:
        assert m[1] < m[0], log
    shape = (s["allnx"], s["allnz"])
    v1 = np.fromfile(os.path.join(s["out"], "vel_p_1_%d_%d.dat" % shape), np.float32).reshape(shape)
    assert np.all(np.isfinite(v1)) and not np.array_equal(v1, s["vp0"])


def test_gradient_only_writes_one_gradient_and_no_model(tmp_path):
    """--gradient-only: one gradient pass, its misfit logged and its raw
    gradients written, no model update."""
    from sfwi_gb300 import su
    s = _survey(tmp_path)
    r = subprocess.run([su.DRIVER, s["para"], "--stage", "1", "--gradient-only"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    log = open(os.path.join(s["out"], "misfit.txt")).read()
    assert log.count("misfit =") == 1, log
    shape = (s["allnx"], s["allnz"])
    for name in ("sum_grad_pp", "sum_grad_ps", "sum_illum"):
        g = np.fromfile(os.path.join(s["out"], "%s_0_%d_%d.dat" % ((name,) + shape)), np.float32)
        assert g.size == shape[0] * shape[1] and np.all(np.isfinite(g)) and np.abs(g).max() > 0, name
    assert not os.path.exists(os.path.join(s["out"], "vel_p_1_%d_%d.dat" % shape))


def test_driver_with_host_strips_gives_the_same_files(tmp_path):
    """cpu_mem = 1 with iointerval = 50 steps (the reference driver's ntt):
    the edge strips live in host memory and every file the driver writes is
    the same bit for bit; rbc = 1 is refused"""
    from sfwi_gb300 import su
    s = _survey(tmp_path)
    txt = open(s["para"]).read()
    outs = []
    for k, flags in enumerate(("1 0 0 1000", "1 0 1 50")):
        out = s["out"] + str(k)
        open(s["para"], "w").write(txt.replace("1 0 0 1000", flags).replace(s["out"], out))
        r = subprocess.run([su.DRIVER, s["para"], "--stage", "1", "--iters", "1"], capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        outs.append(out)
    names = sorted(f for f in os.listdir(outs[0]) if f.endswith(".dat"))
    assert names
    for f in names:
        a = np.fromfile(os.path.join(outs[0], f), np.float32)
        b = np.fromfile(os.path.join(outs[1], f), np.float32)
        assert np.array_equal(a, b), f
    open(s["para"], "w").write(txt.replace("1 0 0 1000", "1 1 0 1000"))
    r = subprocess.run([su.DRIVER, s["para"], "--stage", "1", "--iters", "1"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode != 0 and "random boundary" in r.stderr


@pytest.mark.parametrize("stage", [1, 2])
def test_resume_from_the_checkpoint_equals_an_uninterrupted_run(tmp_path, stage):
    """Two iterations straight, against one iteration, then --resume to two:
    the second iteration's files are the same bit for bit (the checkpoint
    carries the model or perturbation, the CG direction and denominator)"""
    from sfwi_gb300 import su
    s = _survey(tmp_path)
    txt = open(s["para"]).read()

    def run(out, iters, resume=False):
        open(s["para"], "w").write(txt.replace(s["out"], out))
        cmd = [su.DRIVER, s["para"], "--stage", str(stage), "--iters", str(iters)] + (["--resume"] if resume else [])
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        return r.stdout

    a, b = s["out"] + "a", s["out"] + "b"
    run(a, 2)
    run(b, 1)
    assert "resuming at iteration 1" in run(b, 2, resume=True)
    names = sorted(f for f in os.listdir(a) if f.endswith(".dat") and "_1_" in f)
    assert len(names) >= 4
    for f in names:
        assert np.array_equal(np.fromfile(os.path.join(a, f), np.float32), np.fromfile(os.path.join(b, f), np.float32)), f
    # a checkpoint of the other stage is refused
    other = s["out"] + "c"
    os.makedirs(other)
    os.replace(os.path.join(b, "state.bin"), os.path.join(other, "state.bin"))
    open(s["para"], "w").write(txt.replace(s["out"], other))
    r = subprocess.run([su.DRIVER, s["para"], "--stage", str(3 - stage), "--iters", "3", "--resume"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode != 0 and "another stage" in r.stderr
