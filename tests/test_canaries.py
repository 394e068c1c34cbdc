"""Stray-write and allocation-failure checks on the GPU.

Ghost-cell canaries: shots are packed side by side with no guard rows, and
the outer four rows and columns of every shot (plus the pitch padding below
each column) are outside the update region, as in the reference
(sfwi-stage1/born.cu:362).  They start at zero and no kernel may write
anything else there.  After a run, every wavefield, PML memory variable and
imaging accumulator is read back and those cells are checked to be exactly
zero; a store past a tile, a shot or a column would show there.  Runs cover
uneven windows, both stages, the reconstruction and snapshot modes, both
source kinds and every tile shape.

Allocation failure: a snapshot batch larger than the GPU's memory is refused
with SFWI_E_NOMEM (a plain allocation error, nothing is launched), and the
handle keeps working.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import _batch_inputs

pytestmark = pytest.mark.gpu
NOP = 4


def _run(stage, tile, snap=None, source=0, uneven=True, grid=None):
    import sfwi_gb300 as sg
    cfg, model, shots = _batch_inputs(stage, nshots=3, uneven=uneven, **(grid or {}))
    pml, allnx, allnz, nt = cfg["pml"], cfg["allnx"], cfg["allnz"], cfg["nt"]
    maxnx = max(d["nx"] for d in shots)
    fd = sg.FD2DGPU_ELASTIC(model["sou"], cfg["dx"], cfg["dx"], cfg["dt"], maxnx + 2 * pml, allnz + 2 * pml, allnx,
                            allnz, 1, pml, nt, 4, shots[0]["ntr"], stage=stage)
    fd.GPUbufferVPVS(model["vp"], model["vs"], model["rho"] if stage == 1 else None)
    fd.GPUbufferM(model["dvp"], model["dvs"])
    fd.set_tile_shape(tile)
    fd.set_source(source)
    if snap:
        fd.set_snapshots(*snap)  # (the density kernel needs the reconstruction)
    else:
        fd.set_density_gradient(True)
    for d in shots:
        fd.enqueue_shot(d["nx"], d["isx"], pml + 2, pml, d["ngx_left"], d["delta_left"], 0, d["gc"], d["obs_z"],
                        d["obs_x"])
    fd.run()
    grid, nstate = fd.debug_grid()
    fd.close()
    return cfg, shots, grid, nstate


def _check(cfg, shots, grid, nstate):
    pml, nzpml = cfg["pml"], cfg["allnz"] + 2 * cfg["pml"]
    row0 = 0
    for d in shots:
        nxpml = d["nx"] + 2 * pml
        for a in range(nstate):
            g = grid[a, row0:row0 + nxpml]
            for name, cells in (("top rows", g[:NOP]), ("bottom rows", g[nxpml - NOP:]),
                                ("left columns", g[:, :NOP]), ("right columns and padding", g[:, nzpml - NOP:])):
                assert not np.any(cells), (a, row0, name, np.flatnonzero(cells)[:5])
        row0 += nxpml
    assert row0 == grid.shape[1]
    # the checked arrays did hold results: background vx and the lambda
    # accumulator (the first of the four accumulators that end the state)
    assert np.any(grid[0]) and np.any(grid[nstate - 4])


@pytest.mark.parametrize("tile", ["16x32", "32x32", "16x64", "8x32x3", "16x32c2", "8x32c2s3"])
def test_no_writes_outside_the_update_region_for_every_tile_shape(tile):
    _check(*_run(2, tile))


@pytest.mark.parametrize("stage,snap,source", [(1, None, 1), (1, (4, "f16"), 0), (2, (2, "bf16"), 1),
                                               (2, (1, "f32"), 0)])
def test_no_writes_outside_the_update_region_in_every_mode(stage, snap, source):
    _check(*_run(stage, "16x32", snap=snap, source=source))


@pytest.mark.parametrize("tile", ["16x32", "32x32", "8x32c2s3"])
def test_no_writes_outside_the_update_region_with_tile_grids_starting_early(tile):
    """On this grid the tile grids start before the first updated row and
    column (fewer tiles hold PML cells): the cells there are loaded as zeros
    or from the shot before and must not be written."""
    _check(*_run(2, tile, grid=dict(allnx=150, allnz=83, pml=11, nt=120)))


def test_batch_larger_than_the_gpu_is_refused_and_the_handle_keeps_working():
    import sfwi_gb300 as sg
    from sfwi_gb300 import synth
    allnx, allnz, pml, dx, nt = 2001, 801, 20, 5.0, 6000
    vp, vs, rho = synth.layered_model(allnx, allnz, dx)
    sou = synth.ricker(nt, 5e-4, 25.0)
    fd = sg.FD2DGPU_ELASTIC(sou, dx, dx, 5e-4, allnx + 2 * pml, allnz + 2 * pml, allnx, allnz, 1, pml, nt, 4, 1,
                            stage=1)
    fd.GPUbufferVPVS(vp, vs, rho)
    # FP32 snapshots of every step: 6000 x 2 x 2041 x 848 floats (83 GB) a
    # shot; five shots ask for 415 GB at once
    fd.set_snapshots(1, "f32")
    for k in range(5):
        fd.enqueue_shot(allnx, pml + 100 + 300 * k, pml + 2, pml, 0, 0, 0, np.array([500], np.int32))
    with pytest.raises(sg.SfwiError, match="sfwi error -3"):
        fd.run()
    # the same handle then runs one shot with the reconstruction
    fd.set_snapshots(0)
    fd.enqueue_shot(allnx, pml + 1000, pml + 2, pml, 0, 0, 0, np.array([1000], np.int32))
    m, _ = fd.run()
    assert np.isfinite(m)
    fd.close()
