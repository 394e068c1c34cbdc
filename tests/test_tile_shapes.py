"""Launch configurations of the step kernels: tile shapes
(sfwi_set_tile_shape), the autotuner (sfwi_autotune), programmatic
dependent launch (sfwi_set_launch_overlap) and the tile draw order of each
sweep (sfwi_set_tile_order).  Every configuration runs the same
per-cell arithmetic in the same order, so its records, residuals and gradients
equal the default's bit for bit, and each is within the 1e-4 relative L2 of
the FP64 oracle."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.golden.make_golden import load_case
from tests.helpers import make_engine, rel, run_ref_api

pytestmark = pytest.mark.gpu
TOL = 1e-4
KEYS = ("syn_z", "syn_x", "res_z", "res_x", "grad_pp", "grad_ps", "illum")


def _shapes():
    import sfwi_gb300 as sg
    return sg.TILE_SHAPES


def _run(case, shape, snap=None):
    shot, inputs, _ = load_case(case)
    fd = make_engine(shot, inputs)
    fd.set_tile_shape(shape)
    assert fd.tile_shape() == shape
    if snap:
        fd.set_snapshots(*snap)
    out = run_ref_api(shot, inputs, fd=fd)
    fd.close()
    return shot, inputs, out


@pytest.mark.parametrize("case", ["s1_full", "s2_window", "s2_dx12p5"])
def test_every_shape_matches_default_and_oracle(case):
    shot, inputs, base = _run(case, "16x32")
    ref = po.run_shot("f64", shot, inputs)
    for shape in _shapes()[1:]:
        _, _, out = _run(case, shape)
        for k in KEYS:
            assert np.array_equal(out[k], base[k]), (case, shape, k, rel(out[k], base[k]))
            assert rel(out[k], ref[k]) < TOL, (case, shape, k, rel(out[k], ref[k]))
        assert out["misfit"] == base["misfit"]


def _batch(stage, shape, snap=None):
    import sfwi_gb300 as sg
    from tests.test_gpu_parity import _batch_inputs
    cfg, model, shots = _batch_inputs(stage, nshots=3, allnx=150, allnz=83, pml=11, nt=160, uneven=True)
    pml = cfg["pml"]
    maxnx = max(d["nx"] for d in shots)
    fd = sg.FD2DGPU_ELASTIC(model["sou"], cfg["dx"], cfg["dx"], cfg["dt"], maxnx + 2 * pml, cfg["allnz"] + 2 * pml,
                            cfg["allnx"], cfg["allnz"], 1, pml, cfg["nt"], 4, shots[0]["ntr"], stage=stage)
    fd.GPUbufferVPVS(model["vp"], model["vs"], model["rho"] if stage == 1 else None)
    fd.GPUbufferM(model["dvp"], model["dvs"])
    fd.set_tile_shape(shape)
    if snap:
        fd.set_snapshots(*snap)
    elif stage == 1:
        fd.set_density_gradient(True)
    for d in shots:
        fd.enqueue_shot(d["nx"], d["isx"], pml + 2, pml, d["ngx_left"], d["delta_left"], 0, d["gc"], d["obs_z"],
                        d["obs_x"])
    m, per = fd.run()
    out = {"per": per, "recs": [fd.read_records(i, d["ntr"]) for i, d in enumerate(shots)],
           "grads": fd.read_gradients_f64()}
    if stage == 1 and not snap:
        out["grho"] = fd.read_density_gradient_f64()
    fd.close()
    return out


@pytest.mark.parametrize("stage,snap", [(1, None), (2, None), (2, (4, "f16"))])
def test_every_shape_gives_the_same_bits_with_interior_tiles(stage, snap):
    """A 150x83 grid (PML 11) with uneven apertures has tiles without PML
    cells, and each shape tiles it differently: a cell can sit in a PML tile
    under one shape and an interior tile under another, and the tile grids
    start before the first updated row or column.  Every cell takes the same
    arithmetic in any tile, so the records, misfits and FP64 gradients agree
    bit for bit."""
    base = _batch(stage, "16x32", snap)
    for shape in _shapes()[1:]:
        out = _batch(stage, shape, snap)
        assert np.array_equal(out["per"], base["per"]), shape
        for i, (a, b) in enumerate(zip(out["recs"], base["recs"])):
            for k in a:
                assert np.array_equal(a[k], b[k]), (shape, i, k)
        for a, b in zip(out["grads"], base["grads"]):
            assert np.array_equal(a, b), shape
        if "grho" in base:
            assert np.array_equal(out["grho"], base["grho"]), shape


def test_every_shape_with_compressed_snapshots():
    _, _, base = _run("s1_full", "16x32", snap=(4, "f16"))
    for shape in _shapes()[1:]:
        _, _, out = _run("s1_full", shape, snap=(4, "f16"))
        for k in KEYS:
            assert np.array_equal(out[k], base[k]), (shape, k, rel(out[k], base[k]))


def test_autotune_picks_a_shape_and_keeps_results():
    shot, inputs, _ = load_case("s1_full")
    fd = make_engine(shot, inputs)
    first = run_ref_api(shot, inputs, fd=fd)
    choice, ms = fd.autotune(reps=3)
    print("autotune:", choice, ms)
    assert choice in _shapes()
    assert fd.tile_shape() == choice
    assert all(v > 0 for v in ms.values()) and ms[choice] == min(ms.values())
    # the gradients of the run before were accumulated already
    g = fd.read_gradients_f64()
    for k, a in zip(("grad_pp", "grad_ps", "illum"), g):
        assert np.array_equal(a, first[k]), k
    fd.imagebuffer_resettozero()
    again = run_ref_api(shot, inputs, fd=fd)
    fd.close()
    for k in KEYS:
        assert np.array_equal(again[k], first[k]), k


def test_shape_switch_on_resident_batch_then_time_kernels():
    shot, inputs, _ = load_case("s2_window")
    fd = make_engine(shot, inputs)
    run_ref_api(shot, inputs, fd=fd)
    for shape in _shapes():
        fd.set_tile_shape(shape)
        ms = fd.time_kernels(reps=2)
        assert all(v > 0 for v in ms.values()), (shape, ms)
    fd.close()


def test_bad_shape_is_refused():
    import sfwi_gb300 as sg
    shot, inputs, _ = load_case("s1_window")
    fd = make_engine(shot, inputs)
    with pytest.raises(sg.SfwiError):
        fd.set_tile_shape(7)
    fd.close()


@pytest.mark.parametrize("case", ["s1_full", "s2_window"])
def test_launch_overlap_keeps_results(case):
    shot, inputs, _ = load_case(case)
    outs = []
    for on in (True, False):
        fd = make_engine(shot, inputs)
        fd.set_launch_overlap(on)
        outs.append(run_ref_api(shot, inputs, fd=fd))
        ms = fd.time_kernels(reps=5)
        print(case, "overlap" if on else "serial", {k: round(v * 1e3, 2) for k, v in ms.items()})
        fd.close()
    for k in KEYS:
        assert np.array_equal(outs[0][k], outs[1][k]), k


@pytest.mark.parametrize("order", [0, 0b0101, 0b1111])
def test_tile_orders_keep_results(order):
    import sfwi_gb300 as sg
    shot, inputs, _ = load_case("s2_window")
    base = run_ref_api(shot, inputs)
    fd = make_engine(shot, inputs)
    fd.set_tile_order(order)
    out = run_ref_api(shot, inputs, fd=fd)
    with pytest.raises(sg.SfwiError, match="0..15"):
        fd.set_tile_order(16)
    fd.close()
    for k in KEYS:
        assert np.array_equal(out[k], base[k]), k


def test_default_shape_follows_the_batch_size():
    """Without an explicit choice a one-shot batch gets the 8x32 tiles and a
    batch with at least four 16x32 tiles per CTA slot gets 16x32."""
    import bench
    import sfwi_gb300 as sg
    w = dict(bench.WORKLOADS["fwi376"], nt=20)
    data = bench.build_workload(w)
    pml, nxpml, nzpml = w["pml"], w["allnx"] + 2 * w["pml"], w["allnz"] + 2 * w["pml"]
    isz, igz = pml + w["sy"], pml + w["gy"]
    for nshots, want in ((1, "8x32c2s3"), (len(data["shots"]), "16x32")):
        fd = sg.FD2DGPU_ELASTIC(data["sou"][:20], w["dx"], w["dx"], w["dt"], nxpml, nzpml, w["allnx"], w["allnz"], 1,
                                pml, 20, 4, data["shots"][0]["ntr"], stage=1)
        fd.GPUbufferVPVS(data["vp0"], data["vs0"], data["rho0"])
        for d in data["shots"][:nshots]:
            fd.enqueue_shot(d["nx"], d["isx"], isz, igz, d["ngx_left"], d["delta_left"], 0, d["gc"])
        fd.run_forward()
        assert fd.tile_shape() == want, (nshots, fd.tile_shape())
        fd.close()
