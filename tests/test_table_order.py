"""The tile table of a batch of many waves is reordered so that each end
holds interior tiles (build_tiles): the shots covering the last two waves of
tiles at either end keep their interior tiles at that end, so every sweep
ends on cheap tiles.  A small batch keeps the plain order.  Each cell's
update does not depend on the order, so a 96-shot batch (thousands of 16x32
tiles, reordered) gives every shot the same records and misfit, bit for
bit, as the same shots run in batches of 8 (a few hundred tiles, not
reordered); the FP64 gradients differ only by the order of the sum over
shots.  Uneven apertures, stages 1 and 2.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ALLNX, ALLNZ, PML, NT, DX, DT, F0, NSHOTS = 400, 20, 10, 100, 10.0, 1e-3, 25.0, 96


def _handle(stage):
    import sfwi_gb300 as sg
    from sfwi_gb300 import synth
    return sg.FD2DGPU_ELASTIC(synth.ricker(NT, DT, F0), DX, DX, DT, ALLNX + 2 * PML, ALLNZ + 2 * PML, ALLNX, ALLNZ,
                              1, PML, NT, 4, 0, stage=stage)


@pytest.fixture(scope="module")
def survey():
    from sfwi_gb300 import synth
    vp, vs, rho = synth.layered_model(ALLNX, ALLNZ, DX, vmin=1800.0, vmax=3000.0, seed=17)
    vp0 = synth.smooth_z(vp, 3)
    vs0 = (vp0 / 1.73).astype(np.float32)
    rho0 = (310.0 * vp0.astype(np.float64) ** 0.25).astype(np.float32)
    shots = synth.config_shots(ALLNX, DX, PML, NSHOTS, 4, first=8, aperture=(120, 400))
    fd = _handle(1)
    fd.GPUbufferVPVS(vp, vs, rho)
    for d in shots:
        fd.enqueue_shot(d["nx"], d["isx"], PML + 2, PML, d["ngx_left"], d["delta_left"], 0, d["gc"])
    fd.run_forward()
    for i, d in enumerate(shots):
        r = fd.read_records(i, d["ntr"])
        d["obs_z"], d["obs_x"] = r["syn_z"].astype(np.float32), r["syn_x"].astype(np.float32)
    fd.close()
    return dict(vp0=vp0, vs0=vs0, rho0=rho0, dvp=(vp - vp0).astype(np.float32), dvs=(vs - vs0).astype(np.float32),
                shots=shots)


def _runs(s, stage, group):
    fd = _handle(stage)
    fd.GPUbufferVPVS(s["vp0"], s["vs0"], s["rho0"] if stage == 1 else None)
    if stage == 2:
        fd.GPUbufferM(s["dvp"], s["dvs"])
    fd.set_tile_shape("16x32")
    per, recs, grads = [], [], None
    for k in range(0, NSHOTS, group):
        sel = s["shots"][k:k + group]
        for d in sel:
            fd.enqueue_shot(d["nx"], d["isx"], PML + 2, PML, d["ngx_left"], d["delta_left"], 0, d["gc"],
                            d["obs_z"], d["obs_x"])
        _, p = fd.run(len(sel))
        per.extend(p)
        recs.extend(fd.read_records(i, d["ntr"]) for i, d in enumerate(sel))
        g = fd.read_gradients_f64()
        fd.imagebuffer_resettozero()
        grads = g if grads is None else tuple(a + b for a, b in zip(grads, g))
    fd.close()
    return np.array(per), recs, grads


@pytest.mark.parametrize("stage", [1, 2])
def test_reordered_batch_equals_small_batches(survey, stage):
    per_a, recs_a, g_a = _runs(survey, stage, NSHOTS)
    per_b, recs_b, g_b = _runs(survey, stage, 8)
    assert np.array_equal(per_a, per_b)
    for r, q in zip(recs_a, recs_b):
        for k in ("syn_z", "syn_x", "res_z", "res_x"):
            assert np.array_equal(r[k], q[k]), k
    for a, b in zip(g_a, g_b):
        assert np.abs(a).max() > 0
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12 * np.abs(b).max())
