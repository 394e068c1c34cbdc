"""Shots over several ranks (sfwi_gb300/shard.py), on the host: the cost
partition, and a world-size-2 gloo run of the sharded gradient pass with a
stand-in engine whose per-shot gradients are known, against the sum of all
shots in one process."""
import os
import socket

import numpy as np
import pytest

from sfwi_gb300 import shard


def test_partition_covers_every_shot_once_and_balances_cost():
    rng = np.random.default_rng(3)
    costs = [int(c) for c in rng.integers(150, 401, 80)]
    for world in (1, 2, 3, 8):
        parts = shard.partition(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(80))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
    assert shard.partition(costs, 4) == shard.partition(list(costs), 4)  # deterministic


class FakeEngine:
    """Stands in for FD2DGPU_ELASTIC: shot i contributes gradients i+1 at its
    source column and misfit (i+1)^2."""
    pml, nzpml, nt, allnx, allnz = 4, 20, 10, 12, 6

    def __init__(self):
        self.q = []
        self.g = [np.zeros((self.allnx, self.allnz)) for _ in range(3)]

    def enqueue_shot(self, nx, isx, isz, igz, ngx_left, delta_left, rl, gc, rz, rx):
        self.q.append(isx)

    def run(self):
        m = 0.0
        for isx in self.q:
            for k, g in enumerate(self.g):
                g[isx % self.allnx, k] += isx + 1
            m += (isx + 1) ** 2
        self.q = []
        return m, None

    def read_gradients_f64(self):
        return tuple(g.copy() for g in self.g)

    def imagebuffer_resettozero(self):
        for g in self.g:
            g[...] = 0.0


def _shots(n):
    return [dict(nx=8 + (i % 5), isx=i, isz=0, igz=0, ngx_left=0, delta_left=0, gc=None, obs_z=None, obs_x=None)
            for i in range(n)]


def _worker(rank, world, port, n, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        m, grads = shard.run_sharded(FakeEngine(), _shots(n), rank, world)
        np.savez(os.path.join(out_dir, "r%d.npz" % rank), m=m, *grads)
    finally:
        dist.destroy_process_group()


def test_sharded_pass_equals_one_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    n = 11
    mp.spawn(_worker, args=(2, port, n, str(tmp_path)), nprocs=2, join=True)
    ref = FakeEngine()
    for d in _shots(n):
        ref.enqueue_shot(d["nx"], d["isx"], 0, 0, 0, 0, 0, None, None, None)
    m_ref, _ = ref.run()
    for r in range(2):
        z = np.load(os.path.join(tmp_path, "r%d.npz" % r))
        assert float(z["m"]) == m_ref
        for k, g in enumerate(ref.g):
            assert np.array_equal(z["arr_%d" % k], g)
    del torch


def _engine_survey():
    from sfwi_gb300 import synth
    allnx, allnz, pml, nt, dx, dt = 90, 40, 10, 220, 10.0, 1e-3
    vp, vs, rho = synth.layered_model(allnx, allnz, dx, vmin=1800.0, vmax=3000.0)
    vp0 = synth.smooth_z(vp, 3)
    shots = synth.config_shots(allnx, dx, pml, 5, 14, first=10)
    rng = np.random.default_rng(5)
    for d in shots:
        d["isz"], d["igz"] = pml + 2, pml
        d["obs_z"] = (1e-6 * rng.standard_normal((d["ntr"], nt))).astype(np.float32)
        d["obs_x"] = (1e-6 * rng.standard_normal((d["ntr"], nt))).astype(np.float32)
    return dict(allnx=allnx, allnz=allnz, pml=pml, nt=nt, dx=dx, dt=dt, sou=synth.ricker(nt, dt, 20.0), vp=vp0,
                vs=(vp0 / 1.73).astype(np.float32), rho=rho, shots=shots)


def _engine(s):
    import sfwi_gb300 as sg
    pml = s["pml"]
    fd = sg.FD2DGPU_ELASTIC(s["sou"], s["dx"], s["dx"], s["dt"], s["allnx"] + 2 * pml, s["allnz"] + 2 * pml,
                            s["allnx"], s["allnz"], 1, pml, s["nt"], 4, s["shots"][0]["ntr"], stage=1)
    fd.GPUbufferVPVS(s["vp"], s["vs"], s["rho"])
    return fd


def _engine_worker(rank, world, port, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        s = _engine_survey()
        fd = _engine(s)
        m, grads = shard.run_sharded(fd, s["shots"], rank, world)
        fd.close()
        np.savez(os.path.join(out_dir, "e%d.npz" % rank), m=m, *grads)
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_sharded_pass_with_the_engine_equals_one_process(tmp_path):
    """Two gloo ranks, each with its own engine on the one GPU and its share
    of the shots (their kernels never wait on each other), then the FP64
    all-reduce: every rank ends with the one-process gradients and misfit
    (to the rounding of the different summation order)."""
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    s = _engine_survey()
    fd = _engine(s)
    for d in s["shots"]:
        fd.enqueue_shot(d["nx"], d["isx"], d["isz"], d["igz"], d["ngx_left"], d["delta_left"], 0, d["gc"], d["obs_z"],
                        d["obs_x"])
    m_ref, _ = fd.run()
    ref = fd.read_gradients_f64()
    fd.close()
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    mp.spawn(_engine_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        z = np.load(os.path.join(tmp_path, "e%d.npz" % r))
        assert float(z["m"]) == pytest.approx(m_ref, rel=1e-12)
        for k, g in enumerate(ref):
            assert np.abs(g).max() > 0
            assert np.allclose(z["arr_%d" % k], g, rtol=1e-12, atol=1e-12 * np.abs(g).max())
    del torch
