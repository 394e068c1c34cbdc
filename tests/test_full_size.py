"""Checks at the full size of the 38-shot 376x201 workload (nt = 3000).

  * one shot at the full nt against the FP64 oracle and the reference's CUDA
    path, with observed data modelled on the true model: within the 1e-4
    relative L2 bar (measured 4e-7 to 2.5e-6).  With white noise as observed
    data the gradient is a correlation of the forward field with a noise-
    driven adjoint field, whose terms cancel to a small sum: there the
    reference's own FP32 path is 1.7e-4 from the FP64 oracle and this
    library 1.7e-4, so that input is not a parity case at this length;
  * a batch of shots equals the same shots run one at a time, bit for bit,
    with the OT misfit;
  * the Born records are linear in the model perturbation;
  * one full 38-shot pass gives finite, non-zero gradients with the misfit the
    per-shot misfits add up to;
  * on the full 376x201 grid (two shots, 400 steps) every tile shape gives
    the same records and gradients bit for bit: there cells sit in PML tiles
    under one shape and in interior tiles under another.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.helpers import make_engine, rel, run_ref_api

pytestmark = pytest.mark.gpu
KEYS = ("syn_z", "syn_x", "res_z", "res_x", "grad_pp", "grad_ps", "illum")


@pytest.fixture(scope="module")
def survey():
    import bench
    w = dict(bench.WORKLOADS["fwi376"])
    data = bench.build_workload(w)
    return w, data


def _shot(w, d, stage):
    return dict(stage=stage, allnx=w["allnx"], allnz=w["allnz"], nx=d["nx"], pml=w["pml"], nop=4, nt=w["nt"],
                ntr=d["ntr"], dx=w["dx"], dz=w["dx"], dt=w["dt"], isx=d["isx"], isz=w["pml"] + w["sy"],
                igz=w["pml"] + w["gy"], ngx_left=d["ngx_left"], delta_left=d["delta_left"], record_left_in_v=0,
                forward_only=0, misfit_kind=0, nthreads=0)


def _inputs(w, data, d, seed=3):
    rng = np.random.default_rng(seed)
    return dict(vp=data["vp0"], vs=data["vs0"], rho=data["rho0"], dvp=data["dvp"], dvs=data["dvs"], sou=data["sou"],
                gc=d["gc"], obs_z=(1e-4 * rng.standard_normal((d["ntr"], w["nt"]))).astype(np.float32),
                obs_x=(1e-4 * rng.standard_normal((d["ntr"], w["nt"]))).astype(np.float32))


@pytest.mark.parametrize("stage", [1, 2])
def test_matches_oracle_and_reference_cuda_path_at_full_nt(survey, stage):
    w, data = survey
    d = data["shots"][7]
    shot = dict(_shot(w, d, stage), nthreads=0)
    # observed records: the same shot on the true model (FP64 oracle)
    true_in = dict(vp=data["vp"], vs=data["vs"], rho=data["rho"], dvp=data["dvp"], dvs=data["dvs"],
                   sou=data["sou"], gc=d["gc"])
    obs = po.run_shot("f64", dict(shot, forward_only=1), true_in)
    inputs = dict(_inputs(w, data, d), obs_z=obs["syn_z"].astype(np.float32), obs_x=obs["syn_x"].astype(np.float32))
    ref64 = po.run_shot("f64", shot, inputs)
    out = run_ref_api(shot, inputs, fd=make_engine(shot, inputs))
    refs = {"oracle": ref64}
    if po.build_refgpu() and po.available("gpu%d" % stage):
        refs["reference GPU"] = po.run_shot("gpu%d" % stage, shot, inputs)
    for name, ref in refs.items():
        errs = {k: rel(out[k], ref[k]) for k in KEYS}
        print("stage", stage, "nt", w["nt"], "vs", name, {k: "%.1e" % v for k, v in errs.items()})
        for k, e in errs.items():
            assert e < 1e-4, (name, k, e)


def _engine(w, data, stage=2, ot=True):
    import sfwi_gb300 as sg
    pml = w["pml"]
    fd = sg.FD2DGPU_ELASTIC(data["sou"], w["dx"], w["dx"], w["dt"], w["allnx"] + 2 * pml, w["allnz"] + 2 * pml,
                            w["allnx"], w["allnz"], 1, pml, w["nt"], 4, data["shots"][0]["ntr"], stage=stage)
    fd.GPUbufferVPVS(data["vp0"], data["vs0"])
    fd.GPUbufferM(data["dvp"], data["dvs"])
    if ot:
        fd.set_misfit(sg.MISFIT_OT)
    return fd


def _enqueue(fd, w, data, d, obs):
    pml = w["pml"]
    fd.enqueue_shot(d["nx"], d["isx"], pml + w["sy"], pml + w["gy"], d["ngx_left"], d["delta_left"], 0, d["gc"],
                    obs[0], obs[1])


def test_batch_equals_one_at_a_time_with_ot(survey):
    w, data = survey
    pick = [data["shots"][i] for i in (0, 19, 37)]
    obs = [(_inputs(w, data, d, seed=i)["obs_z"], _inputs(w, data, d, seed=i)["obs_x"]) for i, d in enumerate(pick)]
    fd = _engine(w, data)
    for d, o in zip(pick, obs):
        _enqueue(fd, w, data, d, o)
    m_b, per_b = fd.run()
    rec_b = [fd.read_records(i, d["ntr"]) for i, d in enumerate(pick)]
    g_b = fd.read_gradients_f64()
    fd.imagebuffer_resettozero()
    per_s = []
    for i, (d, o) in enumerate(zip(pick, obs)):
        _enqueue(fd, w, data, d, o)
        m, _ = fd.run()
        per_s.append(m)
        for k, v in fd.read_records(0, d["ntr"]).items():
            assert np.array_equal(v, rec_b[i][k]), (i, k)
    g_s = fd.read_gradients_f64()
    fd.close()
    assert np.array_equal(per_b, np.array(per_s))
    for a, b in zip(g_b, g_s):
        assert np.array_equal(a, b)
    assert m_b == pytest.approx(sum(per_s), rel=1e-15)


def test_born_records_are_linear_in_the_perturbation(survey):
    import sfwi_gb300 as sg
    w, data = survey
    d = data["shots"][11]
    pml = w["pml"]
    out = []
    for scale in (1.0, 2.0):
        fd = sg.FD2DGPU_ELASTIC(data["sou"], w["dx"], w["dx"], w["dt"], w["allnx"] + 2 * pml, w["allnz"] + 2 * pml,
                                w["allnx"], w["allnz"], 1, pml, w["nt"], 4, d["ntr"], stage=2)
        fd.GPUbufferVPVS(data["vp0"], data["vs0"])
        fd.GPUbufferM(scale * data["dvp"], scale * data["dvs"])
        fd.enqueue_shot(d["nx"], d["isx"], pml + w["sy"], pml + w["gy"], d["ngx_left"], d["delta_left"], 0, d["gc"])
        fd.run_forward()
        out.append(fd.read_records(0, d["ntr"]))
        fd.close()
    # every Born term doubles exactly except where values in the wavefront
    # tails are subnormal; over 3000 steps that reaches 1.6e-6 relative
    assert rel(2.0 * out[0]["syn_z"], out[1]["syn_z"]) < 1e-5
    assert rel(2.0 * out[0]["syn_x"], out[1]["syn_x"]) < 1e-5
    assert np.array_equal(out[0]["syn2_z"], out[1]["syn2_z"])


def test_full_pass_gives_finite_gradients(survey):
    w, data = survey
    fd = _engine(w, data)
    fd.set_density_gradient(True)
    for i, d in enumerate(data["shots"]):
        inp = _inputs(w, data, d, seed=100 + i)
        _enqueue(fd, w, data, d, (inp["obs_z"], inp["obs_x"]))
    m, per = fd.run()
    g = fd.read_gradients_f64()
    grho = fd.read_density_gradient_f64()
    fd.close()
    assert np.isfinite(m) and m > 0 and m == pytest.approx(per.sum(), rel=1e-12)
    for a in g + (grho,):
        assert np.all(np.isfinite(a)) and np.abs(a).max() > 0


def test_every_tile_shape_gives_the_same_bits_on_the_full_grid(survey):
    import sfwi_gb300 as sg
    w, data = survey
    nt = 400
    pml = w["pml"]
    pick = [data["shots"][i] for i in (3, 20)]
    obs = [(_inputs(w, data, d, seed=i)["obs_z"][:, :nt].copy(), _inputs(w, data, d, seed=i)["obs_x"][:, :nt].copy())
           for i, d in enumerate(pick)]

    def run(shape):
        fd = sg.FD2DGPU_ELASTIC(data["sou"][:nt], w["dx"], w["dx"], w["dt"], w["allnx"] + 2 * pml,
                                w["allnz"] + 2 * pml, w["allnx"], w["allnz"], 1, pml, nt, 4, pick[0]["ntr"], stage=2)
        fd.GPUbufferVPVS(data["vp0"], data["vs0"])
        fd.GPUbufferM(data["dvp"], data["dvs"])
        fd.set_tile_shape(shape)
        for d, o in zip(pick, obs):
            _enqueue(fd, w, data, d, o)
        m, per = fd.run()
        out = ([fd.read_records(i, d["ntr"]) for i, d in enumerate(pick)], fd.read_gradients_f64(), per)
        fd.close()
        return out

    base = run("16x32")
    for shape in sg.TILE_SHAPES[1:]:
        recs, grads, per = run(shape)
        assert np.array_equal(per, base[2]), shape
        for a, b in zip(recs, base[0]):
            for k in a:
                assert np.array_equal(a[k], b[k]), (shape, k)
        for a, b in zip(grads, base[1]):
            assert np.array_equal(a, b), shape
