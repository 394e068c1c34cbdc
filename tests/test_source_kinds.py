"""Vertical-force source (sfwi_set_source(h, SFWI_SOURCE_VZ_FORCE)).

The reference injects sou[it] into txx and tzz ahead of the velocity sweep
(sfwi-stage1/FD2DGPU.cu:2104-2114).  The vertical force has no reference
counterpart: sou[it] goes into vz at the source cell after the velocity sweep,
into the total field only, like the reference's stress source.  The oracle
states it (oracle/sfwi_oracle.c, src_kind); the CPU tests check the oracle's
physics, the GPU tests hold the CUDA path to the FP64 oracle within the 1e-4
relative L2 of the plain FP32 path.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.golden.make_golden import load_case
from tests.helpers import make_engine, rel, run_ref_api

TOL = 1e-4
KEYS = ("syn_z", "syn_x", "res_z", "res_x", "grad_pp", "grad_ps", "illum")


def _homogeneous(nt=260):
    """A homogeneous model, the source in the middle column two nodes below
    the receiver row, receivers on every column."""
    allnx, allnz, pml, dx, dt = 61, 40, 10, 10.0, 1e-3
    vp = np.full((allnx, allnz), 2500.0, np.float32)
    vs = (vp / 1.73).astype(np.float32)
    rho = np.full_like(vp, 2000.0)
    shot = dict(stage=1, allnx=allnx, allnz=allnz, nx=allnx, pml=pml, nop=4, nt=nt, ntr=allnx, dx=dx, dz=dx,
                dt=dt, isx=pml + allnx // 2, isz=pml + 8, igz=pml + 2, ngx_left=0, delta_left=0,
                record_left_in_v=0, forward_only=1, misfit_kind=0, nthreads=0)
    inputs = dict(vp=vp, vs=vs, rho=rho, sou=po.ricker(nt, dt, 25.0), gc=np.arange(allnx, dtype=np.int32) * 10,
                  obs_z=np.zeros((allnx, nt), np.float32), obs_x=np.zeros((allnx, nt), np.float32))
    return shot, inputs


def test_oracle_vertical_force_radiates_symmetrically():
    po.build()
    shot, inputs = _homogeneous()
    f = po.run_shot("f64", dict(shot, src_kind=1), inputs)
    e = po.run_shot("f64", dict(shot, src_kind=0), inputs)
    mid = shot["allnx"] // 2
    vz, vx = f["syn_z"], f["syn_x"]
    assert np.abs(vz[mid]).max() > 0
    # a vertical force is even in x for vz and odd for vx.  vz sits on the
    # source's columns and vx half a cell to the right (its x derivative is
    # D+x), so vz[mid-d] mirrors vz[mid+d] and vx[mid-d-1] mirrors vx[mid+d];
    # the PML profiles, indexed by cell, break the mirror by ~1e-4
    for d in (3, 5, 12):
        assert np.abs(vz[mid - d] - vz[mid + d]).max() < 1e-3 * np.abs(vz).max(), d
        assert np.abs(vx[mid - d - 1] + vx[mid + d]).max() < 2e-3 * np.abs(vx).max(), d
        assert np.abs(vx[mid + d]).max() > 1e-2 * np.abs(vx).max(), d
    # it is a different source from the reference's stress source, and both
    # first reach the receivers above them at the same step
    assert rel(f["syn_z"], e["syn_z"]) > 0.1
    a = np.flatnonzero(np.abs(vz[mid]) > 1e-30)[0]
    b = np.flatnonzero(np.abs(e["syn_z"][mid]) > 1e-30)[0]
    assert abs(int(a) - int(b)) <= 1


def test_oracle_fp32_transliteration_agrees_for_vertical_force():
    po.build()
    shot, inputs, _ = load_case("s1_window")
    a = po.run_shot("f64", dict(shot, src_kind=1), inputs)
    b = po.run_shot("f32", dict(shot, src_kind=1), inputs)
    for k in KEYS:
        assert rel(b[k], a[k]) < TOL, (k, rel(b[k], a[k]))


def _gpu(case, kind, snap=None):
    import sfwi_gb300 as sg
    shot, inputs, _ = load_case(case)
    fd = make_engine(shot, inputs)
    fd.set_source(kind)
    if snap:
        fd.set_snapshots(*snap)
    out = run_ref_api(shot, inputs, fd=fd)
    fd.close()
    del sg
    return shot, inputs, out


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["s1_full", "s1_window", "s2_window", "s2_dx12p5"])
def test_gpu_vertical_force_matches_oracle(case):
    import sfwi_gb300 as sg
    shot, inputs, out = _gpu(case, sg.SOURCE_VZ_FORCE)
    ref = po.run_shot("f64", dict(shot, src_kind=1), inputs)
    for k in KEYS:
        assert rel(out[k], ref[k]) < TOL, (case, k, rel(out[k], ref[k]))
    # and it differs from the reference's source
    _, _, exp = _gpu(case, sg.SOURCE_TXX_TZZ)
    assert rel(out["syn_z"], exp["syn_z"]) > 1e-2


@pytest.mark.gpu
def test_gpu_vertical_force_with_snapshots():
    import sfwi_gb300 as sg
    shot, inputs, out = _gpu("s1_full", sg.SOURCE_VZ_FORCE, snap=(1, "f32"))
    ref = po.run_shot("f64", dict(shot, src_kind=1, snap_every=1), inputs)
    for k in KEYS:
        assert rel(out[k], ref[k]) < TOL, (k, rel(out[k], ref[k]))
    # 16-bit snapshots: the source cell's value is inside the snapshot scale
    shot, inputs, out = _gpu("s1_full", sg.SOURCE_VZ_FORCE, snap=(4, "f16"))
    ref = po.run_shot("f64", dict(shot, src_kind=1, snap_every=4), inputs)
    for k in ("grad_pp", "grad_ps", "illum"):
        assert np.all(np.isfinite(out[k]))
        assert rel(out[k], ref[k]) < 1e-3, (k, rel(out[k], ref[k]))


@pytest.mark.gpu
def test_unknown_source_kind_is_refused():
    import sfwi_gb300 as sg
    shot, inputs, _ = load_case("s1_window")
    fd = make_engine(shot, inputs)
    with pytest.raises(sg.SfwiError):
        fd.set_source(5)
    fd.close()
