"""Edge strips in host memory (sfwi_set_cpu_mem: IMAGE_SINGLESHOT's cpu_mem
and ntt, sfwi-stage1/FD2DGPU.cu:4382-4421, :4548-4561, :4600-4622).

With cpu_mem set the device holds a ring of two chunks of ntt steps of edge
strips; every full chunk but the last two goes to pinned host memory during
the forward sweeps and comes back during the backward sweeps.  The strips are
the same numbers wherever they are kept, so the bar is identity with the
device-held run: records, per-shot misfits and FP64 gradients (and the
density kernel) bit for bit, for chunk lengths that divide nt unevenly
(7, 64), one that sends a single chunk to the host (149), one whose ring
would hold every step (150: the strips stay on the device), with the L2 and
OT misfits, in stages 1 and 2, and over repeated runs on one handle.  The
device strip bytes shrink to the ring's share: 2 ntt / nt.  Pinned blocks
that engines release can be cached and handed to later engines
(sfwi_set_pinned_cache): a reused block holds another run's strips, which
the new run overwrites before it reads them.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ALLNX, ALLNZ, PML, NT, DX, DT, F0 = 70, 34, 10, 300, 10.0, 1e-3, 25.0


def _handle(stage):
    import sfwi_gb300 as sg
    from sfwi_gb300 import synth
    return sg.FD2DGPU_ELASTIC(synth.ricker(NT, DT, F0), DX, DX, DT, ALLNX + 2 * PML, ALLNZ + 2 * PML, ALLNX, ALLNZ,
                              1, PML, NT, 4, 0, stage=stage)


@pytest.fixture(scope="module")
def survey():
    from sfwi_gb300 import synth
    vp, vs, rho = synth.layered_model(ALLNX, ALLNZ, DX, vmin=1800.0, vmax=3000.0, seed=5)
    vp0 = synth.smooth_z(vp, 3)
    vs0 = (vp0 / 1.73).astype(np.float32)
    rho0 = (310.0 * vp0.astype(np.float64) ** 0.25).astype(np.float32)
    # three shots, seeded windows of uneven width
    shots = synth.config_shots(ALLNX, DX, PML, 3, 20, first=12, aperture=(30, 60))
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


def _run(s, stage, cpu_mem, ntt, misfit=0, rho=False, repeat=1):
    fd = _handle(stage)
    fd.GPUbufferVPVS(s["vp0"], s["vs0"], s["rho0"] if stage == 1 else None)
    if stage == 2:
        fd.GPUbufferM(s["dvp"], s["dvs"])
    if rho:
        fd.set_density_gradient(True)
    fd.set_misfit(misfit)
    fd.set_cpu_mem(cpu_mem, ntt)
    out = []
    for _ in range(repeat):
        for d in s["shots"]:
            fd.enqueue_shot(d["nx"], d["isx"], PML + 2, PML, d["ngx_left"], d["delta_left"], 0, d["gc"], d["obs_z"],
                            d["obs_x"])
        _, per = fd.run(len(s["shots"]))
        g = fd.read_gradients_f64()
        if rho:
            g = g + (fd.read_density_gradient_f64(),)
        recs = [fd.read_records(i, d["ntr"]) for i, d in enumerate(s["shots"])]
        fd.imagebuffer_resettozero()
        out.append(dict(per=per, grads=g, recs=recs, bytes=fd.strip_bytes()))
    fd.close()
    return out


def _same_run(a, b):
    assert np.array_equal(a["per"], b["per"])
    for x, y in zip(a["grads"], b["grads"]):
        assert np.array_equal(x, y)
    assert np.abs(a["grads"][0]).max() > 0
    for r, q in zip(a["recs"], b["recs"]):
        for k in ("syn_z", "syn_x", "res_z", "res_x"):
            assert np.array_equal(r[k], q[k]), k


@pytest.mark.parametrize("stage", [1, 2])
@pytest.mark.parametrize("ntt", [7, 64, 149, 150])
def test_host_strips_equal_device_strips(survey, stage, ntt):
    base = _run(survey, stage, 0, 0)[0]
    off = _run(survey, stage, 1, ntt)[0]
    _same_run(off, base)
    dev0, host0 = base["bytes"]
    dev, host = off["bytes"]
    assert dev0 > 0 and host0 == 0
    chunks = -(-NT // ntt)
    if 2 * ntt < NT:
        assert dev * NT == dev0 * 2 * ntt
        assert host * NT == dev0 * (chunks - 2) * ntt
    else:
        assert (dev, host) == (dev0, 0)


def test_host_strips_with_ot_and_density_over_repeated_runs(survey):
    """OT misfit and the density kernel; three runs on one handle reuse the
    captured time loops and the pinned buffers"""
    import sfwi_gb300 as sg
    base = _run(survey, 1, 0, 0, misfit=sg.MISFIT_OT, rho=True)[0]
    runs = _run(survey, 1, 1, 13, misfit=sg.MISFIT_OT, rho=True, repeat=3)
    for r in runs:
        _same_run(r, base)
        assert np.abs(r["grads"][3]).max() > 0


def test_switching_back_to_device_strips(survey):
    import sfwi_gb300 as sg
    base = _run(survey, 2, 0, 0)[0]
    fd = _handle(2)
    fd.GPUbufferVPVS(survey["vp0"], survey["vs0"])
    fd.GPUbufferM(survey["dvp"], survey["dvs"])
    got = []
    for cpu_mem, ntt in ((1, 11), (0, 0), (1, 40)):
        fd.set_cpu_mem(cpu_mem, ntt)
        for d in survey["shots"]:
            fd.enqueue_shot(d["nx"], d["isx"], PML + 2, PML, d["ngx_left"], d["delta_left"], 0, d["gc"],
                            d["obs_z"], d["obs_x"])
        _, per = fd.run(len(survey["shots"]))
        got.append((per, fd.imagebuffer_resettozero()))
    for per, g in got:
        assert np.array_equal(per, base["per"])
        for x, y in zip(g, got[0][1]):
            assert np.array_equal(x, y)
    assert np.array_equal(got[0][1][0], base["grads"][0].astype(np.float32))
    with pytest.raises(sg.SfwiError, match="ntt"):
        fd.set_cpu_mem(1, 0)
    fd.close()


def test_reused_pinned_blocks_give_the_same_results(survey):
    import sfwi_gb300 as sg
    base1 = _run(survey, 1, 0, 0)[0]
    base2 = _run(survey, 2, 0, 0)[0]
    sg.set_pinned_cache(1 << 30)
    try:
        # each engine takes the block the one before released, holding that
        # engine's strips (another stage, another model)
        runs = [(1, _run(survey, 1, 1, 7)[0]), (2, _run(survey, 2, 1, 7)[0]), (1, _run(survey, 1, 1, 9)[0]),
                (2, _run(survey, 2, 1, 5)[0])]
    finally:
        sg.set_pinned_cache(0)
    for stage, r in runs:
        _same_run(r, base1 if stage == 1 else base2)


@pytest.mark.parametrize("tile", ["8x32c2s3", "32x32"])
def test_host_strips_on_other_tile_shapes(survey, tile):
    """the ring is addressed by step, not by tile: other tile shapes give the
    same bits with the strips in host memory"""
    def run(cpu_mem):
        fd = _handle(2)
        fd.GPUbufferVPVS(survey["vp0"], survey["vs0"])
        fd.GPUbufferM(survey["dvp"], survey["dvs"])
        fd.set_tile_shape(tile)
        fd.set_cpu_mem(cpu_mem, 17)
        for d in survey["shots"]:
            fd.enqueue_shot(d["nx"], d["isx"], PML + 2, PML, d["ngx_left"], d["delta_left"], 0, d["gc"],
                            d["obs_z"], d["obs_x"])
        _, per = fd.run(len(survey["shots"]))
        g = fd.read_gradients_f64()
        fd.close()
        return per, g
    a, b = run(0), run(1)
    assert np.array_equal(a[0], b[0])
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y)


def test_host_strips_leave_snapshot_runs_alone(survey):
    """snapshot runs keep no strips: cpu_mem changes nothing and reports no
    strip bytes"""
    def run(cpu_mem):
        fd = _handle(2)
        fd.GPUbufferVPVS(survey["vp0"], survey["vs0"])
        fd.GPUbufferM(survey["dvp"], survey["dvs"])
        fd.set_snapshots(4, "f16")
        fd.set_cpu_mem(cpu_mem, 17)
        for d in survey["shots"]:
            fd.enqueue_shot(d["nx"], d["isx"], PML + 2, PML, d["ngx_left"], d["delta_left"], 0, d["gc"],
                            d["obs_z"], d["obs_x"])
        _, per = fd.run(len(survey["shots"]))
        g = fd.read_gradients_f64()
        sb = fd.strip_bytes()
        fd.close()
        return per, g, sb
    a, b = run(0), run(1)
    assert np.array_equal(a[0], b[0])
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y)
    assert a[2] == (0, 0) and b[2] == (0, 0)
