"""The drivers' model-update arithmetic (host library, sfwi_gb300/update.py)
against the numpy restatement of the reference (oracle/fwi_update.py), bit
for bit: three stage-1 iterations (preconditioning, cut layer, CG
recurrence, normalised direction, parabola step with its clamp, update and
cut-layer flattening) and three stage-2 iterations (cut, preconditioning,
CG, exact step), with the CG state carried between iterations.  The GPU
test replays the same arithmetic on the outputs of the sfwi_fwi driver."""
import os
import subprocess

import numpy as np
import pytest

from oracle import fwi_update as ref


@pytest.fixture(scope="module", autouse=True)
def _built():
    from sfwi_gb300 import build
    build.build_host()


def _fields(rng, shape):
    g_pp = (rng.standard_normal(shape) * 1e-3).astype(np.float32)
    g_ps = (rng.standard_normal(shape) * 4e-4).astype(np.float32)
    illum = (rng.uniform(0.5, 2.0, shape) * 1e-2).astype(np.float32)
    return g_pp, g_ps, illum


def _same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def test_stage1_update_matches_restatement():
    from sfwi_gb300 import update
    rng = np.random.default_rng(7)
    shape = (37, 45)
    cg, st = update.CG(*shape), ref.State(shape)
    vp = rng.uniform(1500, 4500, shape).astype(np.float32)
    vs = (vp / 1.73).astype(np.float32)
    vp_r, vs_r = vp.copy(), vs.copy()
    # misfit triples: a parabola with an interior vertex, one whose vertex is
    # beyond +300 and one beyond -100 (the clamp)
    triples = [(10.0, 7.5, 9.0), (3.5, 3.209, 2.225), (5.0, 6.29, 13.25)]
    for it in range(3):
        g_pp, g_ps, il = _fields(rng, shape)
        beta, cp, cs, d_pp, d_ps = cg.stage1(it, g_pp, g_ps, il)
        beta_r, cp_r, cs_r, dp_r, ds_r = ref.stage1_direction(st, it, g_pp, g_ps, il)
        assert beta == beta_r and (it == 0) == (beta == 0.0)
        for a, b in ((cp, cp_r), (cs, cs_r), (d_pp, dp_r), (d_ps, ds_r), (cg.old_pp, st.old_pp)):
            assert _same(a, b)
        assert cg.beta_fenmu.value == st.beta_fenmu
        assert np.all(cp[:, :ref.CUT_LAYER] == 0) and np.abs(d_pp).max() <= 1.0
        alpha = update.stage1_alpha(*triples[it])
        assert alpha == ref.stage1_alpha(*triples[it])
        update.stage1_update(alpha, d_pp, d_ps, vp, vs)
        vp_r, vs_r = ref.stage1_update(alpha, dp_r, ds_r, vp_r, vs_r)
        assert _same(vp, vp_r) and _same(vs, vs_r)
    assert update.stage1_alpha(*triples[1]) == 300.0
    assert update.stage1_alpha(*triples[2]) == -100.0
    assert -100.0 < update.stage1_alpha(*triples[0]) < 300.0


def test_stage2_update_matches_restatement():
    from sfwi_gb300 import update
    rng = np.random.default_rng(11)
    shape = (41, 33)
    cg, st = update.CG(*shape), ref.State(shape)
    img = np.zeros(shape, np.float32)
    img2 = np.zeros(shape, np.float32)
    img_r, img2_r = img.copy(), img2.copy()
    for it in range(3):
        g_pp, g_ps, il = _fields(rng, shape)
        beta, gp, gs, cp, cs = cg.stage2(it, g_pp, g_ps, il)
        beta_r, gp_r, gs_r, cp_r, cs_r = ref.stage2_direction(st, it, g_pp, g_ps, il)
        assert beta == beta_r
        for a, b in ((gp, gp_r), (gs, gs_r), (cp, cp_r), (cs, cs_r)):
            assert _same(a, b)
        fenzi, fenmu = float(rng.uniform(1, 2)), float(rng.uniform(3, 4))
        alpha = update.stage2_update(fenzi, fenmu, cp, cs, img, img2)
        alpha_r, img_r, img2_r = ref.stage2_update(fenzi, fenmu, cp_r, cs_r, img_r, img2_r)
        assert alpha == alpha_r
        assert _same(img, img_r) and _same(img2, img2_r)


@pytest.mark.gpu
def test_driver_updates_replayed_by_the_restatement(tmp_path):
    """Two stage-1 and two stage-2 iterations of sfwi_fwi: from the gradients,
    illumination and line-search sums the driver wrote, the restatement gives
    the driver's models bit for bit."""
    from sfwi_gb300 import su
    from tests.test_fwi_driver import _survey
    s = _survey(tmp_path)
    shape = (s["allnx"], s["allnz"])

    def load(out, name, it):
        return np.fromfile(os.path.join(out, "%s_%d_%d_%d.dat" % ((name, it) + shape)), np.float32).reshape(shape)

    r = subprocess.run([su.DRIVER, s["para"], "--stage", "1", "--iters", "2"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    sums = [[float(x) for x in l.split("misfits ")[1].split(" alpha")[0].split()]
            for l in r.stdout.splitlines() if "line search misfits" in l]
    assert len(sums) == 2
    st = ref.State(shape)
    vp, vs = s["vp0"].copy(), s["vs0"].copy()
    for it in range(2):
        _, cp, _, d_pp, d_ps = ref.stage1_direction(st, it, load(s["out"], "sum_grad_pp", it),
                                                    load(s["out"], "sum_grad_ps", it), load(s["out"], "sum_illum", it))
        assert _same(cp, load(s["out"], "sum_cg_pp", it))
        vp, vs = ref.stage1_update(ref.stage1_alpha(*sums[it]), d_pp, d_ps, vp, vs)
        assert _same(vp, load(s["out"], "vel_p", it)) and _same(vs, load(s["out"], "vel_s", it))
    # stage 2 from the stage-1 model
    vp.tofile(s["para"] + ".vp")
    txt = open(s["para"]).read().replace(str(tmp_path / "vp0.bin"), s["para"] + ".vp")
    out2 = s["out"] + "2"
    open(s["para"], "w").write(txt.replace(s["out"], out2))
    r = subprocess.run([su.DRIVER, s["para"], "--stage", "2", "--iters", "2"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    steps = [(float(l.split("fenzi ")[1].split()[0]), float(l.split("fenmu ")[1].split()[0]))
             for l in r.stdout.splitlines() if " fenzi " in l]
    assert len(steps) == 2
    st = ref.State(shape)
    ip, ips = np.zeros(shape, np.float32), np.zeros(shape, np.float32)
    for it in range(2):
        _, _, _, cp, cs = ref.stage2_direction(st, it, load(out2, "sum_grad_pp", it), load(out2, "sum_grad_ps", it),
                                               load(out2, "sum_illum", it))
        assert _same(cp, load(out2, "sum_cggrad_pp", it))
        _, ip, ips = ref.stage2_update(steps[it][0], steps[it][1], cp, cs, ip, ips)
        assert _same(ip, load(out2, "sum_image_pp", it)) and _same(ips, load(out2, "sum_image_ps", it))
