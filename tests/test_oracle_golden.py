"""The oracle pinned to the reference.

tests/golden/*.npz hold the outputs of the reference's own kernels, built for
the CPU from the reference sources by oracle/ref_build.py and driven through
IMAGE_SINGLESHOT's launch sequence (tests/golden/make_golden.py).  The FP32
restatement keeps the reference's arithmetic (same operation order and
literal types) and agrees to rounding; the FP64 oracle agrees to the FP32
rounding of the reference.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.golden.make_golden import CASES, load_case

KEYS = ("syn_z", "syn_x", "res_z", "res_x", "grad_pp", "grad_ps", "illum")


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(np.asarray(b, np.float64)), 1e-300)


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("kind,tol", [("f32", 1e-6), ("f64", 2e-5)])
def test_oracle_matches_reference_golden(case, kind, tol):
    shot, inputs, golden = load_case(case)
    out = po.run_shot(kind, shot, inputs)
    for k in KEYS + (("syn2_z", "syn2_x") if shot["stage"] == 2 else ()):
        assert rel(out[k], golden[k]) < tol, (case, kind, k, rel(out[k], golden[k]))
    assert abs(out["misfit"] - golden["misfit"]) <= tol * abs(golden["misfit"])


@pytest.mark.parametrize("case", sorted(CASES))
def test_reference_build_reproduces_golden(case):
    """Where oracle/_ref exists (it needs the reference sources) the golden
    files are reproduced exactly."""
    shot, inputs, golden = load_case(case)
    kind = "ref%d" % shot["stage"]
    if not po.available(kind):
        pytest.skip("oracle/_ref not built")
    out = po.run_shot(kind, shot, inputs)
    for k in KEYS:
        assert np.array_equal(out[k].astype(np.float32), golden[k]), k


def test_receiver_and_source_indices():
    """Receiver columns and source position follow the reference's integer
    arithmetic (sfwi-stage1/FD2DGPU.cu:3161, main.cpp:621-623)."""
    from sfwi_gb300 import synth
    d = synth.shot_descriptor(1000, [600, 610, 1200], 10.0, pml=20, all_left=0, sy=2, gy=0)
    assert d["ngx_left"] == 600 and d["nx"] == 61 and d["isx"] == 20 + 40 and d["isz"] == 22 and d["igz"] == 20
    assert d["delta_left"] == 60


def test_ricker_restatements_agree():
    """The package's wavelet (used by the benchmarks and the serving loop) and
    the oracle's both restate ricker_wave (sfwi-stage1/main.cpp:251-260)."""
    from sfwi_gb300 import synth
    for nt, dt, f in ((3000, 1e-3, 15.0), (6000, 5e-4, 25.0), (257, 1e-3, 20.0)):
        assert np.array_equal(synth.ricker(nt, dt, f), po.ricker(nt, dt, f))
