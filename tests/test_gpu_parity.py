"""CUDA path vs the reference (golden files) and the FP64 oracle.

Every case goes through the C ABI (include/sfwi_gb300.h) in the call order of
the reference's driver.  Tolerance: 1e-4 relative L2 for records, residuals,
gradients and illumination (the bar for plain FP32), 1e-4 relative for the
misfit.  Batched runs must give the same per-shot results as one-at-a-time
runs, bit for bit.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.golden.make_golden import CASES, load_case
from tests.helpers import rel, run_ref_api

pytestmark = pytest.mark.gpu
TOL = 1e-4
KEYS = ("syn_z", "syn_x", "res_z", "res_x", "grad_pp", "grad_ps", "illum")


@pytest.mark.parametrize("case", sorted(CASES))
def test_matches_reference_golden(case):
    shot, inputs, golden = load_case(case)
    out = run_ref_api(shot, inputs)
    keys = KEYS + (("syn2_z", "syn2_x") if shot["stage"] == 2 else ())
    for k in keys:
        assert rel(out[k], golden[k]) < TOL, (case, k, rel(out[k], golden[k]))
    assert abs(out["misfit"] - golden["misfit"]) <= TOL * abs(golden["misfit"])
    assert out["launches"] > 4 * shot["nt"]


@pytest.mark.parametrize("case", sorted(CASES))
def test_matches_fp64_oracle(case):
    shot, inputs, _ = load_case(case)
    ref = po.run_shot("f64", shot, inputs)
    out = run_ref_api(shot, inputs)
    for k in KEYS:
        assert rel(out[k], ref[k]) < TOL, (case, k, rel(out[k], ref[k]))


def test_receiver_and_source_positions_exact():
    """A forward run with one receiver at the source cell and one far away:
    the first nonzero sample of each trace appears at the step the oracle
    predicts (an off-by-one in either index would move or zero it)."""
    shot, inputs, _ = load_case("s1_window")
    ref = po.run_shot("f64", dict(shot, forward_only=1), inputs)
    out = run_ref_api(shot, inputs)
    for k in ("syn_z", "syn_x"):
        for tr in range(shot["ntr"]):
            a = np.flatnonzero(np.abs(ref[k][tr]) > 1e-30)
            b = np.flatnonzero(np.abs(out[k][tr]) > 1e-30)
            assert (a.size == 0 and b.size == 0) or (a[0] == b[0]), (k, tr)


def _batch_inputs(stage, nshots=4, allnx=64, allnz=30, pml=8, nt=220, uneven=False):
    from sfwi_gb300 import synth
    dx, dt = 10.0, 1e-3
    vp, vs, rho = synth.layered_model(allnx, allnz, dx, vmin=1800, vmax=3000)
    sou = po.ricker(nt, dt, 25.0)
    shots = synth.config_shots(allnx, dx, pml, nshots, spacing=10, first=8,
                               aperture=(20, 50) if uneven else None)
    rng = np.random.default_rng(5)
    for d in shots:
        d["obs_z"] = (1e-8 * rng.standard_normal((d["ntr"], nt))).astype(np.float32)
        d["obs_x"] = (1e-8 * rng.standard_normal((d["ntr"], nt))).astype(np.float32)
    model = dict(vp=vp, vs=vs, rho=rho, dvp=(0.03 * vp).astype(np.float32), dvs=(0.03 * vs).astype(np.float32),
                 sou=sou)
    return dict(allnx=allnx, allnz=allnz, pml=pml, nt=nt, dx=dx, dt=dt, stage=stage), model, shots


@pytest.mark.parametrize("stage", [1, 2])
@pytest.mark.parametrize("uneven", [False, True])
def test_batched_equals_one_at_a_time(stage, uneven):
    import sfwi_gb300 as sg
    cfg, model, shots = _batch_inputs(stage, uneven=uneven)
    pml, allnx, allnz, nt = cfg["pml"], cfg["allnx"], cfg["allnz"], cfg["nt"]
    maxnx = max(d["nx"] for d in shots)
    fd = sg.FD2DGPU_ELASTIC(model["sou"], cfg["dx"], cfg["dx"], cfg["dt"], maxnx + 2 * pml, allnz + 2 * pml, allnx,
                            allnz, 1, pml, nt, 4, shots[0]["ntr"], stage=stage)
    fd.GPUbufferVPVS(model["vp"], model["vs"], model["rho"] if stage == 1 else None)
    fd.GPUbufferM(model["dvp"], model["dvs"])
    for d in shots:
        fd.enqueue_shot(d["nx"], d["isx"], pml + 2, pml, d["ngx_left"], d["delta_left"], 0, d["gc"], d["obs_z"],
                        d["obs_x"])
    m_all, per = fd.run()
    recs_b = [fd.read_records(i, d["ntr"]) for i, d in enumerate(shots)]
    g_b = fd.read_gradients_f64()
    fd.imagebuffer_resettozero()
    per_single, recs_s = [], []
    for i, d in enumerate(shots):
        fd.enqueue_shot(d["nx"], d["isx"], pml + 2, pml, d["ngx_left"], d["delta_left"], 0, d["gc"], d["obs_z"],
                        d["obs_x"])
        m, _ = fd.run()
        per_single.append(m)
        recs_s.append(fd.read_records(0, d["ntr"]))
    g_s = fd.read_gradients_f64()
    fd.close()
    assert np.array_equal(per, np.array(per_single))
    for a, b in zip(recs_b, recs_s):
        for k in a:
            assert np.array_equal(a[k], b[k]), k
    for a, b in zip(g_b, g_s):
        assert np.array_equal(a, b)
    assert m_all == pytest.approx(sum(per_single), rel=1e-15)


def test_uneven_windows_match_oracle():
    """Shots with different window widths in one launch, each checked
    against the FP64 oracle run of that shot alone."""
    import sfwi_gb300 as sg
    cfg, model, shots = _batch_inputs(1, nshots=3, uneven=True)
    pml, allnx, allnz, nt = cfg["pml"], cfg["allnx"], cfg["allnz"], cfg["nt"]
    maxnx = max(d["nx"] for d in shots)
    fd = sg.FD2DGPU_ELASTIC(model["sou"], cfg["dx"], cfg["dx"], cfg["dt"], maxnx + 2 * pml, allnz + 2 * pml, allnx,
                            allnz, 1, pml, nt, 4, shots[0]["ntr"], stage=1)
    fd.GPUbufferVPVS(model["vp"], model["vs"], model["rho"])
    for d in shots:
        fd.enqueue_shot(d["nx"], d["isx"], pml + 2, pml, d["ngx_left"], d["delta_left"], 0, d["gc"], d["obs_z"],
                        d["obs_x"])
    _, per = fd.run()
    gpp, gps, ill = fd.read_gradients_f64()
    recs = [fd.read_records(i, d["ntr"]) for i, d in enumerate(shots)]
    fd.close()
    gref = [np.zeros((allnx, allnz)) for _ in range(3)]
    for i, d in enumerate(shots):
        shot = dict(stage=1, allnx=allnx, allnz=allnz, nx=d["nx"], pml=pml, nop=4, nt=nt, ntr=d["ntr"], dx=cfg["dx"],
                    dz=cfg["dx"], dt=cfg["dt"], isx=d["isx"], isz=pml + 2, igz=pml, ngx_left=d["ngx_left"],
                    delta_left=d["delta_left"], record_left_in_v=0, forward_only=0, misfit_kind=0, nthreads=0)
        ref = po.run_shot("f64", shot, dict(model, gc=d["gc"], obs_z=d["obs_z"], obs_x=d["obs_x"]))
        assert rel(recs[i]["syn_z"], ref["syn_z"]) < TOL
        assert per[i] == pytest.approx(ref["misfit"], rel=TOL)
        for k, g in zip(("grad_pp", "grad_ps", "illum"), gref):
            g += ref[k]
    for a, b in zip((gpp, gps, ill), gref):
        assert rel(a, b) < TOL


def test_born_linearity():
    """Stage 2: the scattered records are linear in the perturbation.  Every
    Born term scales by exactly 2 when the perturbation doubles, so the
    records double up to the rounding of subnormal values in the wavefront
    tails (1e-6 relative); the background records do not change at all."""
    import sfwi_gb300 as sg
    cfg, model, shots = _batch_inputs(2, nshots=2)
    pml, allnx, allnz, nt = cfg["pml"], cfg["allnx"], cfg["allnz"], cfg["nt"]
    out = []
    for scale in (1.0, 2.0):
        fd = sg.FD2DGPU_ELASTIC(model["sou"], cfg["dx"], cfg["dx"], cfg["dt"], shots[0]["nx"] + 2 * pml,
                                allnz + 2 * pml, allnx, allnz, 1, pml, nt, 4, shots[0]["ntr"], stage=2)
        fd.GPUbufferVPVS(model["vp"], model["vs"])
        fd.GPUbufferM(scale * model["dvp"], scale * model["dvs"])
        for d in shots:
            fd.enqueue_shot(d["nx"], d["isx"], pml + 2, pml, d["ngx_left"], d["delta_left"], 0, d["gc"])
        fd.run_forward()
        out.append([fd.read_records(i, d["ntr"]) for i, d in enumerate(shots)])
        fd.close()
    for a, b in zip(out[0], out[1]):
        assert rel(2.0 * a["syn_z"], b["syn_z"]) < 1e-6
        assert rel(2.0 * a["syn_x"], b["syn_x"]) < 1e-6
        assert np.array_equal(a["syn2_z"], b["syn2_z"])


def test_deterministic_repeat():
    shot, inputs, _ = load_case("s2_window")
    a = run_ref_api(shot, inputs)
    b = run_ref_api(shot, inputs)
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), k
    assert a["misfit"] == b["misfit"]


@pytest.mark.parametrize("case", sorted(CASES))
def test_density_gradient_matches_fp64_oracle(case):
    """The density kernel (no reference counterpart, parity with the oracle
    only) next to the Vp/Vs gradients of the same run."""
    from tests.helpers import make_engine
    shot, inputs, _ = load_case(case)
    ref = po.run_shot("f64", shot, inputs, want_rho=True)
    fd = make_engine(shot, inputs)
    fd.set_density_gradient(True)
    out = run_ref_api(shot, inputs, fd=fd)
    grho = fd.read_density_gradient_f64()
    fd.close()
    assert np.linalg.norm(ref["grad_rho"]) > 0
    assert rel(grho, ref["grad_rho"]) < TOL, rel(grho, ref["grad_rho"])
    for k in ("grad_pp", "grad_ps", "illum"):
        assert rel(out[k], ref[k]) < TOL, (k, rel(out[k], ref[k]))


def test_salt_stage2_uneven_apertures_12p5m_match_oracle():
    """The 401x301 stage-2 configuration at test size: a salt body in a
    velocity gradient at 12.5 m spacing (stage 2 records with (int)dx and
    injects with dx), shots with seeded uneven apertures advanced in one run;
    records, residuals, misfits and the summed gradients against the FP64
    oracle run of each shot alone."""
    import sfwi_gb300 as sg
    from sfwi_gb300 import synth
    allnx, allnz, pml, nt, dx, dt = 72, 36, 8, 240, 12.5, 1e-3
    vp, vs, _ = synth.salt_model(allnx, allnz, dx, vmin=1500.0, vmax=3000.0, vsalt=3800.0)
    vp0 = synth.smooth_z(vp, 3)
    vs0 = (vp0 / 1.73).astype(np.float32)
    sou = po.ricker(nt, dt, 20.0)
    shots = synth.config_shots(allnx, dx, pml, 4, spacing=14, first=10, aperture=(24, 60))
    assert len({d["nx"] for d in shots}) > 1
    model0 = dict(vp=vp0, vs=vs0, dvp=(vp - vp0).astype(np.float32), dvs=(vs - vs0).astype(np.float32), sou=sou)
    model_true = dict(vp=vp, vs=vs, dvp=np.zeros_like(vp), dvs=np.zeros_like(vs), sou=sou)
    cfgs, refs = [], []
    for d in shots:
        shot = dict(stage=2, allnx=allnx, allnz=allnz, nx=d["nx"], pml=pml, nop=4, nt=nt, ntr=d["ntr"], dx=dx, dz=dx,
                    dt=dt, isx=d["isx"], isz=pml + 2, igz=pml, ngx_left=d["ngx_left"], delta_left=d["delta_left"],
                    record_left_in_v=0, forward_only=1, misfit_kind=0, nthreads=0)
        obs = po.run_shot("f64", shot, dict(model_true, gc=d["gc"]))
        d["obs_z"] = (obs["syn_z"] + obs["syn2_z"]).astype(np.float32)
        d["obs_x"] = (obs["syn_x"] + obs["syn2_x"]).astype(np.float32)
        shot["forward_only"] = 0
        refs.append(po.run_shot("f64", shot, dict(model0, gc=d["gc"], obs_z=d["obs_z"], obs_x=d["obs_x"])))
    maxnx = max(d["nx"] for d in shots)
    fd = sg.FD2DGPU_ELASTIC(sou, dx, dx, dt, maxnx + 2 * pml, allnz + 2 * pml, allnx, allnz, 1, pml, nt, 4,
                            shots[0]["ntr"], stage=2)
    fd.GPUbufferVPVS(vp0, vs0, None)
    fd.GPUbufferM(model0["dvp"], model0["dvs"])
    for d in shots:
        fd.enqueue_shot(d["nx"], d["isx"], pml + 2, pml, d["ngx_left"], d["delta_left"], 0, d["gc"], d["obs_z"],
                        d["obs_x"])
    _, per = fd.run()
    recs = [fd.read_records(i, d["ntr"]) for i, d in enumerate(shots)]
    g = fd.read_gradients_f64()
    fd.close()
    for i, ref in enumerate(refs):
        for k in ("syn_z", "syn_x", "syn2_z", "res_z", "res_x"):
            assert rel(recs[i][k], ref[k]) < TOL, (i, k, rel(recs[i][k], ref[k]))
        assert per[i] == pytest.approx(ref["misfit"], rel=TOL)
    for k, a in zip(("grad_pp", "grad_ps", "illum"), g):
        b = sum(r[k] for r in refs)
        assert rel(a, b) < TOL, (k, rel(a, b))
