"""Seeded random configurations against the FP64 oracle.

Each case draws a stage, a grid (40-140 x 24-100 nodes), a PML width (8-24),
a grid spacing, a receiver window and a source inside it, nt and a tile
shape, so the tile grid starts at many different offsets before the update
region and cells fall in PML and interior tiles in many ways.  Observed
records are the oracle's forward on the true model; the gradient is taken on
a z-smoothed start model 3 % slower.  Records, residuals, gradients and
illumination must be within the 1e-4 relative L2 bar of the oracle, and
equal to the default tile shape's bit for bit.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.helpers import make_engine, rel, run_ref_api

pytestmark = pytest.mark.gpu
TOL = 1e-4
SEEDS = range(8)


def _case(seed):
    from sfwi_gb300 import synth
    rng = np.random.default_rng(1000 + seed)
    stage = int(rng.integers(1, 3))
    allnx, allnz = int(rng.integers(40, 141)), int(rng.integers(24, 101))
    pml = int(rng.integers(8, 25))
    dx = 10.0 if stage == 2 else float(rng.choice([10.0, 12.5]))
    nt, dt = int(rng.integers(120, 241)), 1e-3
    g0 = int(rng.integers(0, allnx // 3))
    g1 = int(rng.integers(2 * allnx // 3, allnx))
    sxn = int(rng.integers(g0 + 2, g1 - 1))
    vp, vs, rho = synth.layered_model(allnx, allnz, dx, vmin=1800, vmax=3000, seed=seed + 7)
    # start model: z-smoothed and 3 % slow, so the residual is a real misfit
    # within the few hundred steps (a start model that the waves do not tell
    # from the true one leaves a residual of FP32 rounding noise, on which
    # any two FP32 implementations differ)
    vp0 = (0.97 * synth.smooth_z(vp, 4)).astype(np.float32)
    vs0 = (vp0 / 1.73).astype(np.float32)
    gx = (np.arange(g0, g1 + 1) * dx).astype(np.int64)
    d = synth.shot_descriptor(int(sxn * dx), gx, dx, pml, all_left=0, sy=2, gy=0)
    sou = po.ricker(nt, dt, 25.0)
    dvp, dvs = (0.05 * vp).astype(np.float32), (0.05 * vs).astype(np.float32)
    shot = dict(stage=stage, allnx=allnx, allnz=allnz, nx=d["nx"], pml=pml, nop=4, nt=nt, ntr=d["ntr"], dx=dx,
                dz=dx, dt=dt, isx=d["isx"], isz=d["isz"], igz=d["igz"], ngx_left=d["ngx_left"],
                delta_left=d["delta_left"], record_left_in_v=0, forward_only=1, misfit_kind=0, nthreads=0)
    obs = po.run_shot("f64", shot, dict(vp=vp, vs=vs, rho=rho, dvp=dvp, dvs=dvs, sou=sou, gc=d["gc"]))
    obs_z = (obs["syn_z"] + (obs["syn2_z"] if stage == 2 else 0)).astype(np.float32)
    obs_x = (obs["syn_x"] + (obs["syn2_x"] if stage == 2 else 0)).astype(np.float32)
    inputs = dict(vp=vp0, vs=vs0, rho=rho, dvp=(0.02 * vp).astype(np.float32), dvs=(0.02 * vs).astype(np.float32),
                  sou=sou, gc=d["gc"], obs_z=obs_z, obs_x=obs_x)
    shot["forward_only"] = 0
    return shot, inputs, rng


@pytest.mark.parametrize("seed", SEEDS)
def test_random_configuration_matches_oracle_on_any_tile_shape(seed):
    import sfwi_gb300 as sg
    shot, inputs, rng = _case(seed)
    shape = str(rng.choice(sg.TILE_SHAPES))
    keys = ["syn_z", "syn_x", "res_z", "res_x", "grad_pp", "grad_ps", "illum"]
    if shot["stage"] == 2:
        keys += ["syn2_z", "syn2_x"]
    ref = po.run_shot("f64", shot, inputs)
    assert np.linalg.norm(ref["res_z"]) > 0.05 * np.linalg.norm(ref["syn_z"])  # a real misfit
    outs = {}
    for s in ("16x32", shape):
        fd = make_engine(shot, inputs)
        fd.set_tile_shape(s)
        outs[s] = run_ref_api(shot, inputs, fd=fd)
        fd.close()
    desc = {k: shot[k] for k in ("stage", "allnx", "allnz", "pml", "nx", "nt", "dx")}
    errs = {k: rel(outs[shape][k], ref[k]) for k in keys}
    print(seed, shape, desc, {k: "%.1e" % v for k, v in errs.items()})
    for k in keys:
        assert errs[k] < TOL, (seed, shape, desc, k, errs[k])
        assert np.array_equal(outs[shape][k], outs["16x32"][k]), (seed, shape, k)


def _batch_case(seed):
    """Three shots with their own random windows and sources on one grid."""
    from sfwi_gb300 import synth
    rng = np.random.default_rng(2000 + seed)
    stage = int(rng.integers(1, 3))
    allnx, allnz = int(rng.integers(60, 141)), int(rng.integers(24, 81))
    pml = int(rng.integers(8, 25))
    dx, nt, dt = 10.0, int(rng.integers(120, 201)), 1e-3
    vp, vs, rho = synth.layered_model(allnx, allnz, dx, vmin=1800, vmax=3000, seed=seed + 11)
    vp0 = (0.97 * synth.smooth_z(vp, 4)).astype(np.float32)
    vs0 = (vp0 / 1.73).astype(np.float32)
    dvp0, dvs0 = (0.02 * vp).astype(np.float32), (0.02 * vs).astype(np.float32)
    sou = po.ricker(nt, dt, 25.0)
    shots = []
    for _ in range(3):
        w = int(rng.integers(allnx // 3, allnx + 1))
        g0 = int(rng.integers(0, allnx - w + 1))
        sxn = int(rng.integers(g0 + 1, g0 + w - 1))
        gx = (np.arange(g0, g0 + w) * dx).astype(np.int64)
        d = synth.shot_descriptor(int(sxn * dx), gx, dx, pml, all_left=0, sy=2, gy=0)
        shot = dict(stage=stage, allnx=allnx, allnz=allnz, nx=d["nx"], pml=pml, nop=4, nt=nt, ntr=d["ntr"], dx=dx,
                    dz=dx, dt=dt, isx=d["isx"], isz=d["isz"], igz=d["igz"], ngx_left=d["ngx_left"],
                    delta_left=d["delta_left"], record_left_in_v=0, forward_only=1, misfit_kind=0, nthreads=0)
        obs = po.run_shot("f64", shot, dict(vp=vp, vs=vs, rho=rho, dvp=(0.05 * vp).astype(np.float32),
                                            dvs=(0.05 * vs).astype(np.float32), sou=sou, gc=d["gc"]))
        inputs = dict(vp=vp0, vs=vs0, rho=rho, dvp=dvp0, dvs=dvs0, sou=sou, gc=d["gc"],
                      obs_z=(obs["syn_z"] + (obs["syn2_z"] if stage == 2 else 0)).astype(np.float32),
                      obs_x=(obs["syn_x"] + (obs["syn2_x"] if stage == 2 else 0)).astype(np.float32))
        shot["forward_only"] = 0
        shots.append((shot, inputs))
    return shots, rng


@pytest.mark.parametrize("seed", range(4))
def test_random_uneven_batch_matches_oracle_shot_by_shot(seed):
    """The batched entry points: each shot's records within 1e-4 of its own
    oracle run, the batch's gradients within 1e-4 of the sum of the oracle's
    per-shot gradients."""
    import sfwi_gb300 as sg
    shots, rng = _batch_case(seed)
    s0 = shots[0][0]
    pml, maxnx = s0["pml"], max(s["nx"] for s, _ in shots)
    fd = sg.FD2DGPU_ELASTIC(shots[0][1]["sou"], s0["dx"], s0["dz"], s0["dt"], maxnx + 2 * pml, s0["allnz"] + 2 * pml,
                            s0["allnx"], s0["allnz"], 1, pml, s0["nt"], 4, s0["ntr"], stage=s0["stage"])
    inp = shots[0][1]
    fd.GPUbufferVPVS(inp["vp"], inp["vs"], inp["rho"] if s0["stage"] == 1 else None)
    if s0["stage"] == 2:
        fd.GPUbufferM(inp["dvp"], inp["dvs"])
    fd.set_tile_shape(str(rng.choice(sg.TILE_SHAPES)))
    for s, i in shots:
        fd.enqueue_shot(s["nx"], s["isx"], s["isz"], s["igz"], s["ngx_left"], s["delta_left"], 0, i["gc"], i["obs_z"],
                        i["obs_x"])
    m, per = fd.run()
    recs = [fd.read_records(k, s["ntr"]) for k, (s, _) in enumerate(shots)]
    grads = fd.read_gradients_f64()
    fd.close()
    refs = [po.run_shot("f64", s, i) for s, i in shots]
    for k, (rec, ref) in enumerate(zip(recs, refs)):
        for key in ("syn_z", "syn_x", "res_z", "res_x") + (("syn2_z", "syn2_x") if s0["stage"] == 2 else ()):
            assert rel(rec[key], ref[key]) < TOL, (seed, k, key, rel(rec[key], ref[key]))
        assert per[k] == pytest.approx(ref["misfit"], rel=1e-4), (seed, k)
    for g, key in zip(grads, ("grad_pp", "grad_ps", "illum")):
        e = rel(g, sum(r[key] for r in refs))
        print(seed, key, "%.1e" % e)
        assert e < TOL, (seed, key, e)
