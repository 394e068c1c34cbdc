"""Line searches through the C ABI against the FP64 oracle.

Stage 1 (CALCULATE_ALPHA_parabola_mb, sfwi-stage1/FD2DGPU.cu:4819-5036): the
L2 misfit of a shot at the trial models m - s*g, s in {0, step1, step2}, from
background forward runs.  Stage 2 (CALCULATE_ALPHA, sfwi-stage2/FD2DGPU.cu:
4576-4722): fenzi = sum q.r and fenmu = sum q.q with r the residual of a Born
run with the model perturbation `image` and q the scattered records of a Born
run with the search direction `cg`.  The oracle side forms the trial models
the way the reference does (float32 products and differences) and sums the
same quantities from its FP64 records.  Tolerance: 1e-4 relative.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.golden.make_golden import load_case

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _fwd(shot, model):
    return po.run_shot("f64", dict(shot, forward_only=1), model)


def _trial(base, g, step):
    return (np.float32(base) - np.float32(step) * np.float32(g)).astype(np.float32)


def _direction(shot, inputs, golden):
    """a search direction scaled so the largest step moves vp by ~1 %"""
    g_pp, g_ps = golden["grad_pp"].astype(np.float64), golden["grad_ps"].astype(np.float64)
    scale = 0.01 * float(np.abs(inputs["vp"]).max()) / max(float(np.abs(g_pp).max()), 1e-30)
    return (g_pp * scale).astype(np.float32), (g_ps * scale * 0.5).astype(np.float32)


def _oracle_parabola(shot, inputs, g_pp, g_ps, steps):
    out = []
    for s in steps:
        model = dict(inputs, vp=_trial(inputs["vp"], g_pp, s), vs=_trial(inputs["vs"], g_ps, s))
        r = _fwd(shot, model)
        out.append(float(np.sum((r["syn_z"] - inputs["obs_z"]) ** 2) + np.sum((r["syn_x"] - inputs["obs_x"]) ** 2)))
    return out


@pytest.mark.parametrize("case", ["s1_full", "s1_window"])
def test_parabola_line_search_matches_oracle(case):
    from tests.helpers import make_engine
    shot, inputs, golden = load_case(case)
    g_pp, g_ps = _direction(shot, inputs, golden)
    steps = (0.0, 0.5, 1.0)
    ref = _oracle_parabola(shot, inputs, g_pp, g_ps, steps)
    fd = make_engine(shot, inputs)
    fd.ntr = shot["ntr"]
    fd.isx, fd.isz, fd.igz = shot["isx"], shot["isz"], shot["igz"]
    fd.ngx_left, fd.delta_left, fd.record_left_in_v = shot["ngx_left"], shot["delta_left"], shot["record_left_in_v"]
    fd.record_copytoGPU(inputs["obs_z"], inputs["obs_x"], inputs["gc"])
    fd.bufferVpVsHtoD(shot["delta_left"] + shot["record_left_in_v"])
    m = fd.CALCULATE_ALPHA_parabola_mb(g_pp, g_ps, steps[1], steps[2])
    # the uploaded model is left as it was: a second search gives the same numbers
    m2 = fd.CALCULATE_ALPHA_parabola_mb(g_pp, g_ps, steps[1], steps[2])
    fd.close()
    assert m == m2
    assert max(ref) - min(ref) > 1e-3 * max(ref)  # the trial models give different misfits
    for a, b in zip(m, ref):
        assert abs(a - b) <= TOL * abs(b), (case, m, ref)


def test_batched_parabola_equals_one_at_a_time():
    import sfwi_gb300 as sg
    shot, inputs, golden = load_case("s1_full")
    g_pp, g_ps = _direction(shot, inputs, golden)
    pml = shot["pml"]
    fd = sg.FD2DGPU_ELASTIC(inputs["sou"], shot["dx"], shot["dz"], shot["dt"], shot["nx"] + 2 * pml,
                            shot["allnz"] + 2 * pml, shot["allnx"], shot["allnz"], 1, pml, shot["nt"], 4, shot["ntr"],
                            stage=1)
    fd.GPUbufferVPVS(inputs["vp"], inputs["vs"], inputs["rho"])
    isxs = (shot["isx"], shot["isx"] + 7)

    def enqueue(isx):
        fd.enqueue_shot(shot["nx"], isx, shot["isz"], shot["igz"], shot["ngx_left"], shot["delta_left"], 0,
                        inputs["gc"], inputs["obs_z"], inputs["obs_x"])

    for isx in isxs:
        enqueue(isx)
    m_all, per = fd.line_search_parabola(g_pp, g_ps, 0.5, 1.0)
    singles = []
    for isx in isxs:
        enqueue(isx)
        singles.append(fd.line_search_parabola(g_pp, g_ps, 0.5, 1.0)[0])
    fd.close()
    assert np.array_equal(per[0], singles[0]) and np.array_equal(per[1], singles[1])
    assert np.allclose(m_all, per.sum(axis=0), rtol=0, atol=0)


@pytest.mark.parametrize("case", ["s2_full", "s2_window"])
def test_exact_line_search_matches_oracle(case):
    from tests.helpers import make_engine
    shot, inputs, golden = load_case(case)
    img_pp, img_ps = inputs["dvp"], inputs["dvs"]
    cg_pp, cg_ps = _direction(shot, inputs, golden)
    a = _fwd(shot, dict(inputs, dvp=img_pp, dvs=img_ps))
    r_z = (a["syn_z"] - inputs["obs_z"]) + a["syn2_z"]
    r_x = (a["syn_x"] - inputs["obs_x"]) + a["syn2_x"]
    q = _fwd(shot, dict(inputs, dvp=cg_pp, dvs=cg_ps))
    fenzi = float(np.sum(q["syn_z"] * r_z) + np.sum(q["syn_x"] * r_x))
    fenmu = float(np.sum(q["syn_z"] ** 2) + np.sum(q["syn_x"] ** 2))
    fd = make_engine(shot, inputs)
    fd.ntr = shot["ntr"]
    fd.isx, fd.isz, fd.igz = shot["isx"], shot["isz"], shot["igz"]
    fd.ngx_left, fd.delta_left, fd.record_left_in_v = shot["ngx_left"], shot["delta_left"], shot["record_left_in_v"]
    fd.record_copytoGPU(inputs["obs_z"], inputs["obs_x"], inputs["gc"])
    fd.bufferVpVsHtoD(shot["delta_left"] + shot["record_left_in_v"])
    zi, mu = fd.CALCULATE_ALPHA(img_pp, img_ps, cg_pp, cg_ps)
    fd.close()
    assert fenmu > 0
    assert abs(mu - fenmu) <= TOL * fenmu, (case, mu, fenmu)
    assert abs(zi - fenzi) <= TOL * np.sqrt(fenmu * float(np.sum(r_z ** 2) + np.sum(r_x ** 2))), (case, zi, fenzi)
