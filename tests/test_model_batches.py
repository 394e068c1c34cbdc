"""Shots on several models in one run (sfwi_run_models), the engine under the
batched serving loop.

Models with their own grid (width and depth) and their own number of time
steps advance in the same kernel launches: the shots of a shorter model drop
out of the tile table after their last step.  The bar is identity:

  * one model through sfwi_run_models equals the plain sfwi_run of the same
    shots on a handle of that model's size, bit for bit (records, per-shot
    misfits, FP64 gradients and illumination);
  * in a mix of three models of different sizes and lengths, queued in an
    interleaved order, every model's gradients and every shot's misfit and
    records equal that model run alone, bit for bit, in stages 1 and 2;
  * one shot of the mix against the FP64 oracle, within the 1e-4 bar;
  * mixed lengths with the OT misfit, and a model deeper than the handle,
    are refused.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.helpers import rel

pytestmark = pytest.mark.gpu
PML, DX, DT, F0 = 10, 10.0, 1e-3, 25.0
# (allnx, allnz, nt, shots)
MODELS = [(60, 30, 300, 2), (48, 44, 260, 1), (72, 24, 200, 3)]


def _model(k, allnx, allnz, nt, nshots, stage):
    from sfwi_gb300 import synth
    vp, vs, rho = synth.layered_model(allnx, allnz, DX, vmin=1800.0, vmax=3000.0, seed=11 + k)
    vp0 = synth.smooth_z(vp, 3)
    vs0 = (vp0 / 1.73).astype(np.float32)
    rho0 = (310.0 * vp0.astype(np.float64) ** 0.25).astype(np.float32)
    shots = synth.config_shots(allnx, DX, PML, nshots, max(1, (allnx - 1) // (nshots + 1)), first=8)
    m = dict(allnx=allnx, allnz=allnz, nt=nt, vp=vp0, vs=vs0, rho=rho0 if stage == 1 else None, shots=shots,
             true=(vp, vs, rho))
    if stage == 2:
        m["dvp"] = (vp - vp0).astype(np.float32)
        m["dvs"] = (vs - vs0).astype(np.float32)
    return m


def _handle(nxpml, allnx, allnz, nt, stage):
    import sfwi_gb300 as sg
    from sfwi_gb300 import synth
    return sg.FD2DGPU_ELASTIC(synth.ricker(nt, DT, F0), DX, DX, DT, nxpml, allnz + 2 * PML, allnx, allnz, 1, PML, nt,
                              4, 0, stage=stage)


def _observe(m):
    """background records of the model's true version (stage 1)"""
    fd = _handle(m["allnx"] + 2 * PML, m["allnx"], m["allnz"], m["nt"], 1)
    fd.GPUbufferVPVS(*m["true"])
    for d in m["shots"]:
        fd.enqueue_shot(d["nx"], d["isx"], PML + 2, PML, d["ngx_left"], d["delta_left"], 0, d["gc"])
    fd.run_forward()
    for i, d in enumerate(m["shots"]):
        r = fd.read_records(i, d["ntr"])
        d["obs_z"], d["obs_x"] = r["syn_z"].astype(np.float32), r["syn_x"].astype(np.float32)
    fd.close()


def _enqueue(fd, d, nt):
    fd.enqueue_shot(d["nx"], d["isx"], PML + 2, PML, d["ngx_left"], d["delta_left"], 0, d["gc"], d["obs_z"],
                    d["obs_x"], nt=nt)


def _alone(m, stage):
    """the model's shots through the plain sfwi_run on a handle of its size"""
    fd = _handle(m["allnx"] + 2 * PML, m["allnx"], m["allnz"], m["nt"], stage)
    fd.GPUbufferVPVS(m["vp"], m["vs"], m["rho"])
    if stage == 2:
        fd.GPUbufferM(m["dvp"], m["dvs"])
    for d in m["shots"]:
        _enqueue(fd, d, m["nt"])
    _, per = fd.run(len(m["shots"]))
    g = fd.read_gradients_f64()
    recs = [fd.read_records(i, d["ntr"]) for i, d in enumerate(m["shots"])]
    fd.close()
    return per, g, recs


def _mix(models, order, stage):
    allnx = max(m["allnx"] for m in models)
    allnz = max(m["allnz"] for m in models)
    nt = max(m["nt"] for m in models)
    fd = _handle(allnx + 2 * PML, allnx, allnz, nt, stage)
    shot_model = []
    for k, j in order:
        _enqueue(fd, models[k]["shots"][j], models[k]["nt"])
        shot_model.append(k)
    per, grads = fd.run_models(models, shot_model)
    recs = [fd.read_records(i, models[k]["shots"][j]["ntr"]) for i, (k, j) in enumerate(order)]
    fd.close()
    return per, grads, recs, nt


def _same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b))


@pytest.fixture(scope="module", params=[1, 2])
def setup(request):
    stage = request.param
    models = [_model(k, *spec, stage=stage) for k, spec in enumerate(MODELS)]
    for m in models:
        _observe(m)
    return stage, models


def test_one_model_equals_the_plain_run(setup):
    stage, models = setup
    m = models[0]
    per0, g0, recs0 = _alone(m, stage)
    per, grads, recs, _ = _mix([m], [(0, j) for j in range(len(m["shots"]))], stage)
    assert _same(per, per0)
    for a, b in zip(grads[0][:3], g0):
        assert _same(a, b)
    assert np.abs(g0[0]).max() > 0
    for r, r0 in zip(recs, recs0):
        for k in ("syn_z", "syn_x", "res_z", "res_x"):
            assert _same(r[k], r0[k]), k


def test_mixed_models_equal_each_model_alone(setup):
    stage, models = setup
    # interleaved queue order: the engine groups and sorts the shots itself
    order = [(0, 0), (2, 0), (1, 0), (2, 1), (0, 1), (2, 2)]
    per, grads, recs, nt = _mix(models, order, stage)
    alone = [_alone(m, stage) for m in models]
    for k, (per0, g0, recs0) in enumerate(alone):
        for a, b in zip(grads[k][:3], g0):
            assert _same(a, b), k
    for i, (k, j) in enumerate(order):
        m = models[k]
        assert per[i] == alone[k][0][j], (k, j)
        for key in ("syn_z", "syn_x", "res_z", "res_x"):
            r, r0 = recs[i][key], alone[k][2][j][key]
            assert _same(r[:, :m["nt"]], r0), (k, j, key)
            assert not np.any(r[:, m["nt"]:]), (k, j, key)  # zeros after the model's last step


def test_a_shot_of_the_mix_against_the_oracle(setup):
    stage, models = setup
    m = models[2]  # the shortest model, idle for the last 100 steps of the run
    order = [(0, 0), (2, 1), (1, 0)]
    per, grads, recs, nt = _mix(models, order, stage)
    d = m["shots"][1]
    shot = dict(stage=stage, allnx=m["allnx"], allnz=m["allnz"], nx=d["nx"], pml=PML, nop=4, nt=m["nt"],
                ntr=d["ntr"], dx=DX, dz=DX, dt=DT, isx=d["isx"], isz=PML + 2, igz=PML, ngx_left=d["ngx_left"],
                delta_left=d["delta_left"], record_left_in_v=0, forward_only=0, misfit_kind=0, nthreads=0)
    from sfwi_gb300 import synth
    inp = dict(vp=m["vp"], vs=m["vs"], rho=m["rho"], dvp=m.get("dvp"), dvs=m.get("dvs"),
               sou=synth.ricker(m["nt"], DT, F0), gc=d["gc"], obs_z=d["obs_z"], obs_x=d["obs_x"])
    ref = po.run_shot("f64", shot, inp)
    for key in ("syn_z", "res_z", "res_x"):
        assert rel(recs[1][key][:, :m["nt"]], ref[key]) < 1e-4, key
    for j, key in enumerate(("grad_pp", "grad_ps", "illum")):
        assert rel(grads[2][j], ref[key]) < 1e-4, key
    assert abs(per[1] - ref["misfit"]) <= 1e-4 * abs(ref["misfit"])


def test_refusals(setup):
    import sfwi_gb300 as sg
    stage, models = setup
    fd = _handle(100, 80, 40, 300, stage)
    for k, j in ((0, 0), (2, 0)):
        _enqueue(fd, models[k]["shots"][j], models[k]["nt"])
    fd.set_misfit(sg.MISFIT_OT)
    with pytest.raises(RuntimeError, match="L2 misfit"):
        fd.run_models([models[0], models[2]], [0, 1])
    fd.set_misfit(0)
    _enqueue(fd, models[1]["shots"][0], models[1]["nt"])  # 44 deep: more than the handle's 40
    with pytest.raises(RuntimeError, match="depth at most"):
        fd.run_models([models[1]], [0])
    fd.close()
