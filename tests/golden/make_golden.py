"""Generate the golden vectors in tests/golden/*.npz from the reference itself.

Run here, where the reference sources are mounted, after
`python oracle/ref_build.py` has built oracle/_ref (the reference's own
kernels compiled for the CPU):

    python tests/golden/make_golden.py [case ...]

Each case stores its float32 inputs and the reference's outputs (records,
residuals, misfit, Vp/Vs gradients, illumination).  Observed data are the
reference's own forward records on a "true" model; the gradient is taken on a
z-smoothed start model.  The reference ships no records, tests or golden
vectors for this path, so these files are the parity pin for the oracle.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402
from sfwi_gb300 import synth  # noqa: E402

CASES = {
    # name: (stage, allnx, allnz, pml, nt, f0, window (g0, g1) in nodes or None, source node[, dx])
    "s1_full": (1, 48, 32, 10, 300, 25.0, None, 21),
    "s1_window": (1, 56, 28, 8, 260, 25.0, (10, 45), 30),
    "s2_full": (2, 48, 32, 10, 300, 25.0, None, 21),
    "s2_window": (2, 56, 28, 8, 260, 25.0, (6, 41), 20),
    # 12.5 m spacing: receiver coordinates in whole metres, and stage 2 divides
    # them by (int)dx = 12 (sfwi-stage2/FD2DGPU.cu:3109), stage 1 by 12.5
    "s1_dx12p5": (1, 60, 30, 8, 240, 20.0, (4, 52), 27, 12.5),
    "s2_dx12p5": (2, 60, 30, 8, 240, 20.0, (4, 52), 27, 12.5),
}


def make_case(name):
    stage, allnx, allnz, pml, nt, f0, win, sxn = CASES[name][:8]
    dx = CASES[name][8] if len(CASES[name]) > 8 else 10.0
    dt = 1e-3
    vp, vs, rho = synth.layered_model(allnx, allnz, dx, vmin=1800, vmax=3000)
    vp0 = synth.smooth_z(vp, 4)
    vs0 = (vp0 / 1.73).astype(np.float32)
    g0, g1 = win if win else (0, allnx - 1)
    gx = (np.arange(g0, g1 + 1) * dx).astype(np.int64)
    d = synth.shot_descriptor(int(sxn * dx), gx, dx, pml, all_left=0, sy=2, gy=0)
    sou = po.ricker(nt, dt, f0)
    dvp = (0.05 * vp).astype(np.float32)
    dvs = (0.05 * vs).astype(np.float32)
    shot = dict(stage=stage, allnx=allnx, allnz=allnz, nx=d["nx"], pml=pml, nop=4, nt=nt, ntr=d["ntr"],
                dx=dx, dz=dx, dt=dt, isx=d["isx"], isz=d["isz"], igz=d["igz"], ngx_left=d["ngx_left"],
                delta_left=d["delta_left"], record_left_in_v=0, forward_only=1, misfit_kind=0, nthreads=0)
    ref = "ref%d" % stage
    obs = po.run_shot(ref, shot, dict(vp=vp, vs=vs, rho=rho, dvp=dvp, dvs=dvs, sou=sou, gc=d["gc"]))
    obs_z = (obs["syn_z"] + (obs["syn2_z"] if stage == 2 else 0)).astype(np.float32)
    obs_x = (obs["syn_x"] + (obs["syn2_x"] if stage == 2 else 0)).astype(np.float32)
    dvp0 = (0.02 * vp).astype(np.float32)
    dvs0 = (0.02 * vs).astype(np.float32)
    inputs = dict(vp=vp0, vs=vs0, rho=rho, dvp=dvp0, dvs=dvs0, sou=sou, gc=d["gc"], obs_z=obs_z, obs_x=obs_x)
    shot["forward_only"] = 0
    out = po.run_shot(ref, shot, inputs)
    arrays = {"in_" + k: np.asarray(v) for k, v in inputs.items()}
    for k in ("syn_z", "syn_x", "res_z", "res_x", "grad_pp", "grad_ps", "illum"):
        arrays["out_" + k] = out[k].astype(np.float32)
    if stage == 2:
        arrays["out_syn2_z"] = out["syn2_z"].astype(np.float32)
        arrays["out_syn2_x"] = out["syn2_x"].astype(np.float32)
    arrays["out_misfit"] = np.array(out["misfit"])
    arrays["shot"] = np.array([shot[k] for k, _ in po.Shot._fields_], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    return arrays


def load_case(name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    vals = z["shot"]
    shot = {}
    for (k, t), v in zip(po.Shot._fields_, vals):
        shot[k] = float(v) if k in ("dx", "dz", "dt") else int(v)
    inputs = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    outputs = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    outputs["misfit"] = float(z["out_misfit"])
    return shot, inputs, outputs


if __name__ == "__main__":
    if not po.available("ref1"):
        sys.exit("oracle/_ref not built: run python oracle/ref_build.py first")
    for n in sys.argv[1:] or CASES:
        make_case(n)
        print("wrote", n)
