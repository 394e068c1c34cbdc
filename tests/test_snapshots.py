"""Snapshot imaging (sfwi_set_snapshots) against the FP64 oracle's snapshot
mode (oracle/sfwi_oracle.c, snap_every): the forward vx, vz are kept every
k-th step and the backward pass images at those steps with weight k, without
the reconstruction.

Bars: FP32 snapshots within the 1e-4 relative L2 of the plain FP32 path;
compressed snapshots (16-bit, scaled by each snapshot's max |v|) within a
stated bound -- 1e-3 for FP16 and 6e-3 for BF16 -- of the FP64 oracle with
exact snapshots (measured at these sizes: about 1.5e-4 and 1.3e-3).  The
measured errors are printed.  Records and residuals do
not depend on the snapshot mode at all.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.golden.make_golden import load_case
from tests.helpers import make_engine, rel, run_ref_api

pytestmark = pytest.mark.gpu
TOL = 1e-4
BOUND = {"f16": 1e-3, "bf16": 6e-3}
KEYS = ("grad_pp", "grad_ps", "illum")


def _gpu(case, every, fmt):
    shot, inputs, _ = load_case(case)
    fd = make_engine(shot, inputs)
    fd.set_snapshots(every, fmt)
    out = run_ref_api(shot, inputs, fd=fd)
    fd.close()
    return shot, inputs, out


@pytest.mark.parametrize("case", ["s1_full", "s2_window", "s2_dx12p5"])
@pytest.mark.parametrize("every", [1, 4])
def test_fp32_snapshots_match_oracle(case, every):
    shot, inputs, out = _gpu(case, every, "f32")
    ref = po.run_shot("f64", dict(shot, snap_every=every), inputs)
    for k in KEYS + ("syn_z", "res_z"):
        assert rel(out[k], ref[k]) < TOL, (case, every, k, rel(out[k], ref[k]))


@pytest.mark.parametrize("case", ["s1_full", "s2_window"])
@pytest.mark.parametrize("fmt", ["f16", "bf16"])
def test_compressed_snapshots_within_bound(case, fmt):
    shot, inputs, out = _gpu(case, 4, fmt)
    ref = po.run_shot("f64", dict(shot, snap_every=4), inputs)
    errs = {k: rel(out[k], ref[k]) for k in KEYS}
    print("%s %s every 4: %s" % (case, fmt, {k: "%.2e" % v for k, v in errs.items()}))
    for k, e in errs.items():
        assert e < BOUND[fmt], (case, fmt, k, e)
    # the records are those of the reconstruction path, bit for bit
    plain = run_ref_api(shot, inputs)
    for k in ("syn_z", "syn_x", "res_z", "res_x"):
        assert np.array_equal(out[k], plain[k]), k


def test_snapshot_mode_switches_back():
    shot, inputs, _ = load_case("s1_window")
    fd = make_engine(shot, inputs)
    fd.set_snapshots(2, "f16")
    a = run_ref_api(shot, inputs, fd=fd)
    fd.imagebuffer_resettozero()
    fd.set_snapshots(0)
    b = run_ref_api(shot, inputs, fd=fd)
    fd.close()
    c = run_ref_api(shot, inputs)
    for k in KEYS:
        assert np.array_equal(b[k], c[k]), k
        assert not np.array_equal(a[k], c[k]), k
