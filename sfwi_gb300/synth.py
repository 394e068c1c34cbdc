"""Seeded synthetic models and shot geometry.

The reference is run on observed SU records that are not distributed with it;
these builders make models of the same shapes and value ranges, and the shot
descriptors the reference's driver derives from an SU index
(sfwi-stage1/main.cpp:76-180 index_shot, :585-625 per-shot set-up).

Seeds: model 1, anomalies 2, shots/apertures 3, request stream 4.
Layouts: models are float32 [allnx, allnz] (z fastest), as the reference
reads them (sfwi-stage1/main.cpp:1462-1470).
"""
import math

import numpy as np

SEED_MODEL, SEED_ANOMALY, SEED_SHOTS, SEED_REQUESTS = 1, 2, 3, 4


def layered_model(allnx, allnz, dx, vmin=1500.0, vmax=4500.0, nlayers=8, n_anom=3, anom=0.10,
                  seed=SEED_MODEL, anom_seed=SEED_ANOMALY):
    """Layered Vp increasing with depth plus `n_anom` Gaussian anomalies of
    +-`anom`; Vs = Vp/1.73; rho = 310 Vp^0.25 (Gardner)."""
    rng = np.random.default_rng(seed)
    depth = np.arange(allnz) / max(allnz - 1, 1)
    bounds = np.sort(rng.uniform(0.05, 0.95, nlayers - 1))
    layer = np.searchsorted(bounds, depth)
    v_layer = np.linspace(vmin, vmax, nlayers)
    # gentle lateral dip on the layer boundaries
    vp = np.empty((allnx, allnz), np.float64)
    dip = rng.uniform(-0.05, 0.05)
    for ix in range(allnx):
        shift = dip * (ix / max(allnx - 1, 1) - 0.5)
        vp[ix] = v_layer[np.searchsorted(bounds, np.clip(depth - shift, 0, 1))]
    arng = np.random.default_rng(anom_seed)
    xx, zz = np.meshgrid(np.arange(allnx), np.arange(allnz), indexing="ij")
    for k in range(n_anom):
        cx = arng.uniform(0.15, 0.85) * allnx
        cz = arng.uniform(0.3, 0.85) * allnz
        r = arng.uniform(0.05, 0.12) * min(allnx, allnz) + 1.0
        sign = 1.0 if k % 2 == 0 else -1.0
        vp *= 1.0 + sign * anom * np.exp(-((xx - cx) ** 2 + (zz - cz) ** 2) / (2 * r * r))
    vp = vp.astype(np.float32)
    vs = (vp / 1.73).astype(np.float32)
    rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(np.float32)
    return vp, vs, rho


def salt_model(allnx, allnz, dx, vmin=1500.0, vmax=3500.0, vsalt=4500.0, seed=SEED_MODEL, anom_seed=SEED_ANOMALY):
    """Vertical-gradient background 1500-3500 m/s with a seeded salt polygon
    of 4500 m/s."""
    rng = np.random.default_rng(anom_seed)
    depth = np.arange(allnz) / max(allnz - 1, 1)
    vp = np.repeat((vmin + (vmax - vmin) * depth)[None, :], allnx, axis=0)
    # star-shaped polygon around a centre in the upper-middle part
    cx, cz = rng.uniform(0.35, 0.65) * allnx, rng.uniform(0.35, 0.55) * allnz
    nv = 9
    ang = np.sort(rng.uniform(0, 2 * math.pi, nv))
    rad = rng.uniform(0.10, 0.22, nv) * min(allnx, allnz * 1.5)
    xx, zz = np.meshgrid(np.arange(allnx), np.arange(allnz), indexing="ij")
    th = np.arctan2(zz - cz, xx - cx) % (2 * math.pi)
    rr = np.hypot(xx - cx, zz - cz)
    ang_ext = np.concatenate([ang - 2 * math.pi, ang, ang + 2 * math.pi])
    rad_ext = np.concatenate([rad, rad, rad])
    boundary = np.interp(th, ang_ext, rad_ext)
    vp = np.where(rr <= boundary, vsalt, vp).astype(np.float32)
    vs = (vp / 1.73).astype(np.float32)
    rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(np.float32)
    return vp, vs, rho


def ricker(nt, dt, fm):
    """Ricker wavelet as the reference computes it (sfwi-stage1/main.cpp:251-260):
    Nk = pi^2 f^2 dt^2 formed in double and stored as float, t0 = ceil(1/(f dt)),
    w = (1 - 2 Nk t^2) exp(-Nk t^2) with the exponent a float product."""
    PI = 3.14159265358979
    fm, dt = np.float32(fm), np.float32(dt)
    Nk = np.float32(PI * PI * float(fm) * float(fm) * float(dt) * float(dt))
    t0 = int(math.ceil(1.0 / float(np.float32(fm * dt))))
    t = np.arange(nt, dtype=np.int64) - t0
    a = 1.0 - 2.0 * float(Nk) * t * t
    tf = t.astype(np.float32)
    e = (-Nk * tf) * tf
    return (a * np.exp(e.astype(np.float64))).astype(np.float32)


def smooth_z(a, half_width):
    """Box-smooth a model along z (the starting model of an inversion)."""
    if half_width <= 0:
        return a.copy()
    k = np.ones(2 * half_width + 1) / (2 * half_width + 1)
    pad = np.pad(a.astype(np.float64), ((0, 0), (half_width, half_width)), mode="edge")
    out = np.stack([np.convolve(row, k, mode="valid") for row in pad])
    return out.astype(np.float32)


def shot_descriptor(sx, gx_list, dx, pml, all_left, sy=0, gy=0):
    """Per-shot geometry exactly as the reference derives it.

    sx, gx_list are integer coordinates (the SU header's sx/gx, metres);
    cx_min/cx_max = min/max over sx and gx (index_shot, main.cpp:123-161);
    nx = (int)(cx_max/dx+0.5) - (int)(cx_min/dx+0.5) + 1 (main.cpp:1383);
    delta_left = int((ngx_left-all_left)/dx), isx = pml+(int)((sx-ngx_left)/dx),
    isz = pml+sy, igz = pml+gy (main.cpp:587-625)."""
    gx = np.asarray(gx_list, dtype=np.int64)
    cmin = int(min(int(sx), int(gx.min())))
    cmax = int(max(int(sx), int(gx.max())))
    nx = int(cmax / dx + 0.5) - int(cmin / dx + 0.5) + 1
    return {
        "sx": int(sx), "gc": gx.astype(np.int32), "ntr": int(len(gx)),
        "ngx_left": cmin, "cx_max": cmax, "nx": nx,
        "delta_left": int((cmin - all_left) / dx),
        "isx": pml + int((sx - cmin) / dx), "isz": pml + int(sy), "igz": pml + int(gy),
    }


def config_shots(allnx, dx, pml, nshots, spacing, first=None, aperture=None, seed=SEED_SHOTS):
    """`nshots` shots `spacing` nodes apart.  Without `aperture` every shot
    records on all allnx surface nodes (one window = the whole model).  With
    aperture=(wmin, wmax) each shot gets a seeded window width in nodes,
    placed around its source and clipped to the model."""
    rng = np.random.default_rng(seed)
    if first is None:
        first = max(0, (allnx - 1 - spacing * (nshots - 1)) // 2)
    out = []
    for k in range(nshots):
        sxn = first + k * spacing
        if aperture is None:
            g0, g1 = 0, allnx - 1
        else:
            w = int(rng.integers(aperture[0], aperture[1] + 1))
            w = min(w, allnx)
            g0 = int(np.clip(sxn - w // 2, 0, allnx - w))
            g1 = g0 + w - 1
        gx = (np.arange(g0, g1 + 1) * dx).astype(np.int64)
        out.append(shot_descriptor(int(sxn * dx), gx, dx, pml, all_left=0))
    return out
