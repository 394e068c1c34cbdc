"""The allocation-free OT entry point (sfwi_ot_noalloc) against the
allocating one (sfwi_ot and its siblings) and the FP64 oracle.

sfwi_ot_noalloc serves callers that cannot allocate device memory (a host
program whose own allocator reserves every device byte, or a loop where a
cudaMalloc would synchronise the device): it works on device buffers the
caller owns and keeps its own working memory in a fixed array inside the
library.  This file is collected last so that a failure here stops a run only
after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po

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


def _rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


def _call(lib, kind, dev, rx, rz, nt, ntr, dt, stream=None):
    m = C.c_double(0.0)
    rc = lib.sfwi_ot_noalloc(kind, *[C.c_void_p(t.data_ptr()) for t in dev], C.c_void_p(rx.data_ptr()),
                             C.c_void_p(rz.data_ptr()), nt, ntr, dt, C.byref(m), stream)
    assert rc == 0, lib.sfwi_last_error()
    return m.value


def test_noalloc_matches_allocating_entry_point_and_oracle_twice():
    torch = pytest.importorskip("torch")
    import sfwi_gb300 as sg
    from sfwi_gb300 import _lib
    lib = _lib.load()
    po.build()
    dt = 1e-3
    fns = {1: sg.OT, 2: sg.OT_power, 3: sg.OT_alltrace}
    for call, (seed, ntr, nt) in enumerate(((1, 37, 700), (2, 53, 512))):
        obs_x, obs_z, cal_x, cal_z = _case(seed, ntr, nt)
        dev = [torch.from_numpy(a).cuda() for a in (obs_x, obs_z, cal_x, cal_z)]
        for kind, fn in fns.items():
            rx_ref, rz_ref, m_ref = fn(obs_x, obs_z, cal_x, cal_z, dt)
            m64, rx64, rz64 = po.ot_gather(kind, dt, obs_x, obs_z, cal_x, cal_z)
            rx = torch.zeros((ntr, nt), dtype=torch.float32, device="cuda")
            rz = torch.zeros((ntr, nt), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            m = _call(lib, kind, dev, rx, rz, nt, ntr, dt)
            rx, rz = rx.cpu().numpy(), rz.cpu().numpy()
            for a, b, c in ((rx, rx_ref, rx64), (rz, rz_ref, rz64)):
                assert _rel(a, b) < TOL, (call, kind, _rel(a, b))
                assert _rel(a, c) < TOL, (call, kind, _rel(a, c))
            assert m == pytest.approx(m_ref, rel=TOL), (call, kind)
            assert m == pytest.approx(m64, rel=TOL), (call, kind)


def test_noalloc_on_a_caller_stream():
    """Inputs written on the caller's stream and no device-wide synchronize
    before the call: the call must order its work on that stream."""
    torch = pytest.importorskip("torch")
    import sfwi_gb300 as sg
    from sfwi_gb300 import _lib
    lib = _lib.load()
    dt = 1e-3
    ntr, nt = 41, 900
    obs_x, obs_z, cal_x, cal_z = _case(3, ntr, nt)
    rx_ref, rz_ref, m_ref = sg.OT(obs_x, obs_z, cal_x, cal_z, dt)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        host = [torch.from_numpy(a).pin_memory() for a in (obs_x, obs_z, cal_x, cal_z)]
        dev = [h.to("cuda", non_blocking=True) for h in host]
        # a second pass over the inputs on the same stream, so that they are
        # not complete when the call's kernels are enqueued unless ordered
        dev = [d * 1.0 for d in dev]
        rx = torch.full((ntr, nt), 7.0, dtype=torch.float32, device="cuda")
        rz = torch.full((ntr, nt), 7.0, dtype=torch.float32, device="cuda")
        m = _call(lib, 1, dev, rx, rz, nt, ntr, dt, C.c_void_p(s.cuda_stream))
        out_x, out_z = rx.cpu().numpy(), rz.cpu().numpy()
    assert _rel(out_x, rx_ref) < TOL
    assert _rel(out_z, rz_ref) < TOL
    assert m == pytest.approx(m_ref, rel=TOL)


def test_noalloc_empty_gather_adds_nothing():
    from sfwi_gb300 import _lib
    lib = _lib.load()
    m = C.c_double(1.5)
    rc = lib.sfwi_ot_noalloc(1, None, None, None, None, None, None, 100, 0, 1e-3, C.byref(m), None)
    assert rc == 0, lib.sfwi_last_error()
    assert m.value == 1.5


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from sfwi_gb300 import _lib
    lib = _lib.load()
    m = C.c_double(0.0)
    p = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.sfwi_ot_noalloc(1, p, p, p, p, p, p, 100, 8193, 1e-3, C.byref(m), None)
    assert rc == -1
    assert b"8192" in lib.sfwi_last_error()


def test_noalloc_rejects_traces_longer_than_its_shared_memory():
    """The fixed scratch holds per-trace sums only: a trace is worked in
    shared memory, so the allocation-free form keeps the 7160-sample limit
    (the allocating entry points take longer traces in global scratch)."""
    from sfwi_gb300 import _lib
    lib = _lib.load()
    m = C.c_double(0.0)
    p = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.sfwi_ot_noalloc(1, p, p, p, p, p, p, 7161, 4, 1e-3, C.byref(m), None)
    assert rc == -1
    assert b"7160" in lib.sfwi_last_error()
