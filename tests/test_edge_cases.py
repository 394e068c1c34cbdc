"""Edge cases of the batched entry points: an empty queue, a shot without
receivers inside a batch, shot geometry outside the grid or the model, and the
size limits of one run, which are refused on the host before anything is
allocated or launched."""
import numpy as np
import pytest

from tests.test_gpu_parity import _batch_inputs

pytestmark = pytest.mark.gpu


def _engine(cfg, model, shots, stage=1):
    import sfwi_gb300 as sg
    pml, allnx, allnz = cfg["pml"], cfg["allnx"], cfg["allnz"]
    maxnx = max(d["nx"] for d in shots)
    fd = sg.FD2DGPU_ELASTIC(model["sou"], cfg["dx"], cfg["dx"], cfg["dt"], maxnx + 2 * pml, allnz + 2 * pml, allnx,
                            allnz, 1, pml, cfg["nt"], 4, shots[0]["ntr"], stage=stage)
    fd.GPUbufferVPVS(model["vp"], model["vs"], model["rho"] if stage == 1 else None)
    if stage == 2:
        fd.GPUbufferM(model["dvp"], model["dvs"])
    return fd


def _enqueue(fd, cfg, d, gc=None, obs=True):
    pml = cfg["pml"]
    g = d["gc"] if gc is None else gc
    oz = d["obs_z"][: len(g)] if obs else None
    ox = d["obs_x"][: len(g)] if obs else None
    fd.enqueue_shot(d["nx"], d["isx"], pml + 2, pml, d["ngx_left"], d["delta_left"], 0, g, oz, ox)


def test_run_with_nothing_queued_is_refused():
    import sfwi_gb300 as sg
    cfg, model, shots = _batch_inputs(1, nshots=1)
    fd = _engine(cfg, model, shots)
    with pytest.raises(sg.SfwiError, match="no shots"):
        fd.run()
    fd.close()


@pytest.mark.parametrize("stage", [1, 2])
def test_a_shot_without_receivers_adds_no_gradient(stage):
    """A shot with zero traces has no residual, so no adjoint field: the
    batch's misfit and Vp/Vs gradients equal those of the batch without it
    bit for bit (its exact zeros add nothing to the FP64 sums), and only its
    illumination (the forward field's energy) is added."""
    cfg, model, shots = _batch_inputs(stage, nshots=3)
    a, b, c = shots
    fd = _engine(cfg, model, shots, stage)
    for d, gc in ((a, None), (b, np.zeros(0, np.int32)), (c, None)):
        _enqueue(fd, cfg, d, gc)
    m3, per3 = fd.run()
    g3 = fd.read_gradients_f64()
    fd.imagebuffer_resettozero()
    for d in (a, c):
        _enqueue(fd, cfg, d)
    m2, per2 = fd.run()
    g2 = fd.read_gradients_f64()
    fd.close()
    assert m3 == m2 and per3[1] == 0.0 and per3[0] == per2[0] and per3[2] == per2[1]
    assert np.array_equal(g3[0], g2[0]) and np.array_equal(g3[1], g2[1])
    assert np.all(g3[2] >= g2[2]) and np.any(g3[2] > g2[2])


def test_shot_geometry_outside_the_grid_or_model_is_refused():
    import sfwi_gb300 as sg
    cfg, model, shots = _batch_inputs(1, nshots=2)
    fd = _engine(cfg, model, shots)
    d = dict(shots[0])
    bad_source = dict(d, isx=d["nx"] + 2 * cfg["pml"] + 3)
    bad_window = dict(d, delta_left=cfg["allnx"] - d["nx"] + 5)
    _enqueue(fd, cfg, shots[1])
    fd.run()
    for bad, msg in ((bad_source, "source cell"), (bad_window, "window")):
        _enqueue(fd, cfg, bad)
        with pytest.raises(sg.SfwiError, match=msg):
            fd.run()
        # nothing of the failed batch is on the device: calls that would use
        # it are refused instead of reading past the last batch's buffers
        with pytest.raises(sg.SfwiError, match="no batch on the device"):
            fd.time_kernels(reps=2)
        with pytest.raises(sg.SfwiError, match="did not complete"):
            fd.read_records(0)
        fd.set_tile_shape("16x32")  # applies to the next batch
    # the handle still works afterwards
    _enqueue(fd, cfg, shots[1])
    m, _ = fd.run()
    assert np.isfinite(m) and m > 0
    fd.close()


def test_a_run_too_large_for_32_bit_strip_rows_is_refused_before_allocation():
    """The edge strips are addressed by 32-bit TMA row coordinates
    (nt x 4 x packed rows); a batch past that is refused with advice to split
    it, before any device memory is taken for it."""
    import sfwi_gb300 as sg
    from sfwi_gb300 import synth
    nt, pml, allnx, allnz, dx = 3000, 20, 376, 60, 10.0
    vp, vs, rho = synth.layered_model(allnx, allnz, dx)
    sou = np.zeros(nt, np.float32)
    fd = sg.FD2DGPU_ELASTIC(sou, dx, dx, 1e-3, allnx + 2 * pml, allnz + 2 * pml, allnx, allnz, 1, pml, nt, 4, 1,
                            stage=1)
    fd.GPUbufferVPVS(vp, vs, rho)
    # 440 shots x 416 packed rows x 3000 steps x 4 > 2^31
    for k in range(440):
        fd.enqueue_shot(allnx, pml + 10, pml + 2, pml, 0, 0, 0, np.array([100], np.int32))
    with pytest.raises(sg.SfwiError, match="split the shots"):
        fd.run()
    fd.close()


def test_snapshot_runs_take_a_bounded_number_of_shots():
    import sfwi_gb300 as sg
    cfg, model, shots = _batch_inputs(1, nshots=1, nt=40)
    fd = _engine(cfg, model, shots)
    fd.set_snapshots(4, "f16")
    d = shots[0]
    for _ in range(513):
        _enqueue(fd, cfg, d, gc=d["gc"][:1])
    with pytest.raises(sg.SfwiError, match="snapshot runs take at most"):
        fd.run()
    fd.close()
