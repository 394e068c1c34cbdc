"""The allocation-free OT entry point (sfwi_ot_noalloc) against the
allocating one (sfwi_ot and its siblings).

sfwi_ot_noalloc serves callers that may not allocate device memory (stream
capture, external allocators, latency-bound loops): it works on device
buffers the caller owns and keeps its own working memory in a fixed array
inside the library.  This file is collected last so that a failure here
stops a run only after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-4  # the parity tolerance of the GPU tests


def _case(seed, ntr, nt):
    rng = np.random.default_rng(seed)
    t = np.arange(nt)
    obs_x = np.exp(-((t[None, :] - rng.uniform(0.2, 0.6, (ntr, 1)) * nt) / 25.0) ** 2).astype(np.float32)
    obs_z = (0.7 * obs_x + 0.05 * rng.standard_normal((ntr, nt))).astype(np.float32)
    cal_x = np.roll(obs_x, 7, axis=1) + 0.01 * rng.standard_normal((ntr, nt)).astype(np.float32)
    cal_z = np.roll(obs_z, -5, axis=1).astype(np.float32)
    return obs_x, obs_z, cal_x.astype(np.float32), cal_z


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    import sfwi_gb300 as sg
    from sfwi_gb300 import _lib
    lib = _lib.load()
    dt = 1e-3
    fns = {1: sg.OT, 2: sg.OT_power, 3: sg.OT_alltrace}
    for call, (seed, ntr, nt) in enumerate(((1, 37, 700), (2, 53, 512))):
        obs_x, obs_z, cal_x, cal_z = _case(seed, ntr, nt)
        dev = [torch.from_numpy(a).cuda() for a in (obs_x, obs_z, cal_x, cal_z)]
        for kind, fn in fns.items():
            rx_ref, rz_ref, m_ref = fn(obs_x, obs_z, cal_x, cal_z, dt)
            rx = torch.zeros((ntr, nt), dtype=torch.float32, device="cuda")
            rz = torch.zeros((ntr, nt), dtype=torch.float32, device="cuda")
            m = C.c_double(0.0)
            torch.cuda.synchronize()
            rc = lib.sfwi_ot_noalloc(kind, *[C.c_void_p(t.data_ptr()) for t in dev], C.c_void_p(rx.data_ptr()),
                                     C.c_void_p(rz.data_ptr()), nt, ntr, dt, C.byref(m), None)
            assert rc == 0, lib.sfwi_last_error()
            rx, rz = rx.cpu().numpy(), rz.cpu().numpy()
            for a, b in ((rx, rx_ref), (rz, rz_ref)):
                err = np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b)
                assert err < TOL, (call, kind, err)
            assert m.value == pytest.approx(m_ref, rel=TOL), (call, kind)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from sfwi_gb300 import _lib
    lib = _lib.load()
    m = C.c_double(0.0)
    p = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.sfwi_ot_noalloc(1, p, p, p, p, p, p, 100, 8193, 1e-3, C.byref(m), None)
    assert rc == -1
    assert b"8192" in lib.sfwi_last_error()
