"""Finite-difference check of the Vp, Vs and density gradients.

The reference forms its gradients by zero-lag correlation of the forward field
(reconstructed backwards from saved edge strips) with the adjoint field, and
scales them for its line search, not as the exact derivative of the misfit.
So the check is one of direction: for smooth Gaussian perturbations dm at
several places, the central difference of the L2 misfit,
(J(m + dm) - J(m - dm)) / 2, divided by <g, dm>, must be positive and the same
for every place, within the tolerance written below (the adjoint of the
continuous equations, discretised, is not the exact adjoint of the
discretisation).

  * Vp, the Lame parameters lambda and mu, and the density: each ratio within
    SPREAD of the others.  The lambda and mu gradients are formed from the Vp
    and Vs ones (g_lam = g_vp / (2 rho vp), g_mu = (g_vs + 4 rho vs g_lam) /
    (2 rho vs)), and their perturbations hold the other two of lambda, mu, rho
    fixed.  The density gradient, which has no reference counterpart, is the
    derivative at fixed Lame parameters.
  * Vs: g_vs = 2 rho vs (g_mu - 2 g_lam) is a difference of two terms of
    nearly equal size, so the few per cent by which each of them misses the
    exact derivative become a large part of their difference, and the ratios
    scatter from place to place (measured 0.3 to 4.5 times the Vp ratio, and
    the opposite sign at one of nine places).  The check there is that the
    finite differences and <g_vs, dm> correlate over the places.
  * All four of Vp, lambda, mu and rho share one scale: their median ratios
    agree within SCALES (measured 2.76e-6 to 2.81e-6), so the gradients are
    one multiple of the derivative and can be combined.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALLNX, ALLNZ, PML, NT, DX, DT = 100, 70, 10, 700, 10.0, 1e-3
# interior (x, z) nodes of the bumps
PLACES = [(45, 35), (30, 48), (68, 28), (50, 40), (40, 25), (60, 50), (55, 32), (35, 40), (65, 45)]
# largest / smallest ratio FD / <g, dm> over the places (all positive)
SPREAD = 0.25
# Pearson correlation of FD and <g_vs, dm> over the places
VS_CORRELATION = 0.8
# largest / smallest median ratio over Vp, lambda, mu and rho
SCALES = 0.1


def _models():
    from sfwi_gb300 import synth
    vp, vs, rho = synth.layered_model(ALLNX, ALLNZ, DX, vmin=1800.0, vmax=3000.0, n_anom=0)
    x, z = np.meshgrid(np.arange(ALLNX), np.arange(ALLNZ), indexing="ij")
    blob = np.exp(-((x - 50) ** 2 + (z - 40) ** 2) / (2 * 8.0 ** 2))
    true = dict(vp=(vp * (1 + 0.05 * blob)).astype(np.float32), vs=(vs * (1 + 0.05 * blob)).astype(np.float32),
                rho=(rho * (1 + 0.05 * blob)).astype(np.float32))
    start = dict(vp=vp.astype(np.float32), vs=vs.astype(np.float32), rho=rho.astype(np.float32))
    return true, start


def _engine(sou, ntr):
    import sfwi_gb300 as sg
    return sg.FD2DGPU_ELASTIC(sou, DX, DX, DT, ALLNX + 2 * PML, ALLNZ + 2 * PML, ALLNX, ALLNZ, 1, PML, NT, 4, ntr,
                              stage=1)


def _enqueue(fd, shots, obs=None):
    for i, d in enumerate(shots):
        o = obs[i] if obs else (None, None)
        fd.enqueue_shot(d["nx"], d["isx"], PML + 2, PML + 2, d["ngx_left"], d["delta_left"], 0, d["gc"], o[0], o[1])


@pytest.fixture(scope="module")
def problem():
    from sfwi_gb300 import synth
    sou = synth.ricker(NT, DT, 15.0)
    shots = synth.config_shots(ALLNX, DX, PML, 2, spacing=40, first=30)
    true, start = _models()
    fd = _engine(sou, shots[0]["ntr"])
    fd.GPUbufferVPVS(true["vp"], true["vs"], true["rho"])
    _enqueue(fd, shots)
    fd.run_forward()
    obs = [(r["syn_z"], r["syn_x"]) for r in (fd.read_records(i, d["ntr"]) for i, d in enumerate(shots))]
    # gradients at the start model
    fd.GPUbufferVPVS(start["vp"], start["vs"], start["rho"])
    fd.set_density_gradient(True)
    _enqueue(fd, shots, obs)
    fd.run()
    gpp, gps, _ = fd.read_gradients_f64()
    grho = fd.read_density_gradient_f64()
    fd.imagebuffer_resettozero()
    vp, vs, rho = (start[k].astype(np.float64) for k in ("vp", "vs", "rho"))
    glam = gpp / (2 * rho * vp)
    gmu = (gps + 4 * rho * vs * glam) / (2 * rho * vs)
    return dict(fd=fd, shots=shots, obs=obs, start=start, g=dict(vp=gpp, vs=gps, rho=grho, lam=glam, mu=gmu))


def _misfit(pb, model):
    fd = pb["fd"]
    fd.GPUbufferVPVS(model["vp"], model["vs"], model["rho"])
    _enqueue(fd, pb["shots"], pb["obs"])
    m, _ = fd.run()
    fd.imagebuffer_resettozero()
    return m


def _bump(place, sigma=4.0):
    x, z = np.meshgrid(np.arange(ALLNX), np.arange(ALLNZ), indexing="ij")
    return np.exp(-((x - place[0]) ** 2 + (z - place[1]) ** 2) / (2 * sigma ** 2))


def _lame(m):
    rho, vp, vs = (m[k].astype(np.float64) for k in ("rho", "vp", "vs"))
    return dict(lam=rho * (vp ** 2 - 2 * vs ** 2), mu=rho * vs ** 2, rho=rho)


def _from_lame(lam, mu, rho):
    return dict(vp=np.sqrt((lam + 2 * mu) / rho), vs=np.sqrt(mu / rho), rho=rho)


def _perturbed(start, param, bump, sign):
    """The start model with `param` scaled by (1 + sign bump); for rho, lam
    and mu the other two of lambda, mu and rho stay fixed, for vp and vs the
    other two of vp, vs and rho."""
    if param in ("vp", "vs"):
        m = {k: v.astype(np.float64) for k, v in start.items()}
        m[param] = m[param] * (1 + sign * bump)
    else:
        l = _lame(start)
        l[param] = l[param] * (1 + sign * bump)
        m = _from_lame(l["lam"], l["mu"], l["rho"])
    return {k: v.astype(np.float32) for k, v in m.items()}


def _value(model, param):
    return _lame(model)[param] if param in ("lam", "mu") else model[param].astype(np.float64)


def _ratios(problem, param):
    fds, projs = [], []
    for place in PLACES:
        bump = 0.003 * _bump(place)
        up = _perturbed(problem["start"], param, bump, +1)
        dn = _perturbed(problem["start"], param, bump, -1)
        dm = (_value(up, param) - _value(dn, param)) / 2
        fds.append((_misfit(problem, up) - _misfit(problem, dn)) / 2)
        projs.append(float(np.sum(problem["g"][param] * dm)))
    return np.array(fds), np.array(projs)


@pytest.mark.parametrize("param", ["vp", "lam", "mu", "rho"])
def test_gradient_matches_finite_differences_in_direction(problem, param):
    fds, projs = _ratios(problem, param)
    r = fds / projs
    print(param, "FD / <g, dm> at", PLACES, ["%.4g" % x for x in r])
    assert np.all(r > 0), r
    assert r.max() / r.min() < 1 + SPREAD, r


def test_vs_gradient_correlates_with_finite_differences(problem):
    fds, projs = _ratios(problem, "vs")
    c = np.corrcoef(fds, projs)[0, 1]
    print("vs FD / <g, dm> at", PLACES, ["%.4g" % x for x in fds / projs], "correlation %.3f" % c)
    assert c > VS_CORRELATION, (c, fds, projs)


def test_one_scale_for_every_parameter(problem):
    med = {}
    for param in ("vp", "lam", "mu", "rho"):
        fds, projs = _ratios(problem, param)
        med[param] = float(np.median(fds / projs))
    print("median FD / <g, dm>", {k: "%.4g" % v for k, v in med.items()})
    v = np.array(list(med.values()))
    assert np.all(v > 0) and v.max() / v.min() < 1 + SCALES, med
