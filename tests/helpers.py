"""Shared test helpers: run a shot through the C ABI the way the reference's
driver calls its engine (sfwi-stage1/main.cpp:585-631)."""
import numpy as np


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_engine(shot, inputs, misfit_kind=0):
    import sfwi_gb300 as sg
    pml, nx = shot["pml"], shot["nx"]
    nxpml, nzpml = nx + 2 * pml, shot["allnz"] + 2 * pml
    fd = sg.FD2DGPU_ELASTIC(inputs["sou"], shot["dx"], shot["dz"], shot["dt"], nxpml, nzpml, shot["allnx"],
                            shot["allnz"], 1, pml, shot["nt"], 4, shot["ntr"], stage=shot["stage"])
    fd.GPUbufferVPVS(inputs["vp"], inputs["vs"], inputs.get("rho") if shot["stage"] == 1 else None)
    if shot["stage"] == 2:
        fd.GPUbufferM(inputs["dvp"], inputs["dvs"])
    if misfit_kind:
        fd.set_misfit(misfit_kind)
    return fd


def run_ref_api(shot, inputs, misfit_kind=0, fd=None):
    """One IMAGE_SINGLESHOT through the reference-shaped API; returns a dict
    like oracle.pyoracle.run_shot (records, residuals, FP64 gradients, misfit)."""
    import sfwi_gb300 as sg
    own = fd is None
    if own:
        fd = make_engine(shot, inputs, misfit_kind)
    fd.ntr = shot["ntr"]
    fd.isx, fd.isz, fd.igz = shot["isx"], shot["isz"], shot["igz"]
    fd.ngx_left, fd.delta_left, fd.record_left_in_v = shot["ngx_left"], shot["delta_left"], shot["record_left_in_v"]
    fd.record_copytoGPU(inputs["obs_z"], inputs["obs_x"], inputs["gc"])
    fd.bufferVpVsHtoD(shot["delta_left"] + shot["record_left_in_v"])
    misfit = sg.IMAGE_SINGLESHOT(fd, 0.0)
    out = {k: v.astype(np.float64) for k, v in fd.read_records(0).items()}
    gpp, gps, ill = fd.read_gradients_f64()
    out.update(grad_pp=gpp, grad_ps=gps, illum=ill, misfit=misfit, launches=fd.kernel_launches())
    if own:
        fd.close()
    return out
