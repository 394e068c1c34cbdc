"""Serving loop: forward-plus-gradient requests of different grid sizes on one
GPU, admitted against a fixed HBM budget while others are running.

A request is one model (vp, vs, rho on its own allnx x allnz grid) with 1..8
shots and their observed records; its result is the misfit and the FP64
Vp/Vs gradients and illumination.  Requests arrive over time.  The server
admits an arrived request as soon as a slot is free and its device memory
fits in what the running requests leave of the budget (oldest first; a
younger request that fits may pass an older one that does not yet fit).
Each admitted request runs on its own engine, whose kernels, graphs and
stream-ordered allocations live on its own CUDA stream, so the work of
concurrent requests overlaps on the device.  `Server(max_active=1)` is the
plain one-job-at-a-time FIFO loop.

Results do not depend on what else is running: every request's engine is
independent and its kernels are deterministic, so a request gives the same
numbers alone and in the mix (tests/test_serve.py).
"""
import dataclasses
import threading
import time

import numpy as np

NGRID = 42     # packed grid arrays per shot cell (sfwi_common.cuh GridArr)
NREC = 8       # trace-major record arrays


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float  # seconds after the start of the request stream
    allnx: int
    allnz: int
    dx: float
    dt: float
    nt: int
    pml: int
    sou: np.ndarray
    vp: np.ndarray
    vs: np.ndarray
    rho: np.ndarray
    shots: list  # dicts: nx, isx, isz, igz, ngx_left, delta_left, gc, obs_z, obs_x
    misfit_kind: int = 0

    @property
    def shot_gradients(self):
        return len(self.shots)


@dataclasses.dataclass
class Result:
    rid: int
    misfit: float
    grad_pp: np.ndarray
    grad_ps: np.ndarray
    illum: np.ndarray
    arrival: float
    admitted: float
    done: float

    @property
    def latency(self):
        return self.done - self.arrival


def request_bytes(req):
    """Device memory of one request's engine (the engine's allocations,
    sfwi_engine.cu:upload_batch, plus the model and the FP64 gradients)."""
    P = (req.allnz + 2 * req.pml + 3) // 4 * 4
    X = sum(int(d["nx"]) + 2 * req.pml for d in req.shots)
    ntr = sum(len(d["gc"]) for d in req.shots)
    nt, ns = req.nt, len(req.shots)
    floats = (NGRID * X * P                       # wavefields, memory variables, coefficients
              + nt * 4 * X * 8 + nt * 4 * ns * 8 * P  # edge strips
              + nt * 2 * X                        # receiver-row records
              + X * ((2 * nt + 3) // 4 * 4)       # residual source
              + NREC * ntr * nt                   # records
              + 5 * req.allnx * req.allnz + nt)   # model, wavelet
    return 4 * floats + 8 * 4 * req.allnx * req.allnz + (1 << 20)


def request_work(req):
    """Cell-steps of one request (its shots' padded cells times nt): the
    order of the shortest-first policy."""
    P = req.allnz + 2 * req.pml
    return sum((int(d["nx"]) + 2 * req.pml) * P for d in req.shots) * req.nt


def run_request(req):
    """One request on a fresh engine: (misfit, grad_pp, grad_ps, illum)."""
    import sfwi_gb300 as sg
    maxnx = max(int(d["nx"]) for d in req.shots)
    fd = sg.FD2DGPU_ELASTIC(req.sou, req.dx, req.dx, req.dt, maxnx + 2 * req.pml, req.allnz + 2 * req.pml, req.allnx,
                            req.allnz, 1, req.pml, req.nt, 4, len(req.shots[0]["gc"]), stage=1)
    try:
        fd.GPUbufferVPVS(req.vp, req.vs, req.rho)
        if req.misfit_kind:
            fd.set_misfit(req.misfit_kind)
        for d in req.shots:
            fd.enqueue_shot(d["nx"], d["isx"], d["isz"], d["igz"], d["ngx_left"], d["delta_left"], 0, d["gc"],
                            d["obs_z"], d["obs_x"])
        m, _ = fd.run()
        g = fd.read_gradients_f64()
    finally:
        fd.close()
    return (m,) + tuple(g)


class Server:
    """Admission loop: arrived requests start as slots (max_active) and the
    HBM budget free up.  policy "oldest" admits in arrival order, letting a
    later request that fits overtake one that does not; "shortest" admits the
    request with the least work first (request_work); with max_active=1 the
    loop is the plain FIFO."""

    def __init__(self, budget_bytes, max_active=4, runner=run_request, sizer=request_bytes, clock=time.perf_counter,
                 policy="oldest", work=request_work):
        if policy not in ("oldest", "shortest"):
            raise ValueError("policy must be 'oldest' or 'shortest'")
        self.budget = int(budget_bytes)
        self.max_active = int(max_active)
        self.runner, self.sizer, self.clock = runner, sizer, clock
        self.policy, self.work = policy, work

    def run(self, requests):
        """Replay `requests` (arrival offsets in seconds) against the wall
        clock and serve them; returns the results in request-id order."""
        reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
        for r in reqs:
            if self.sizer(r) > self.budget:
                raise ValueError("request %d needs %d bytes, more than the whole budget" % (r.rid, self.sizer(r)))
        cv = threading.Condition()
        waiting, results, errors = [], {}, []
        state = {"used": 0, "active": 0}
        t0 = self.clock()

        def now():
            return self.clock() - t0

        def worker(r, size, admitted):
            try:
                out = self.runner(r)
                done = now()
                with cv:
                    results[r.rid] = Result(r.rid, out[0], out[1], out[2], out[3], r.arrival, admitted, done)
            except BaseException as e:  # surfaced to the caller after the loop
                with cv:
                    errors.append(e)
            finally:
                with cv:
                    state["used"] -= size
                    state["active"] -= 1
                    cv.notify_all()

        threads, nxt = [], 0
        with cv:
            while len(results) + len(errors) < len(reqs):
                t = now()
                while nxt < len(reqs) and reqs[nxt].arrival <= t:
                    waiting.append(reqs[nxt])
                    nxt += 1
                # admit every arrived request that fits, oldest or least work first
                order = list(waiting) if self.policy == "oldest" else sorted(waiting, key=lambda q: (self.work(q), q.rid))
                for r in order:
                    if state["active"] >= self.max_active:
                        break
                    size = self.sizer(r)
                    if state["used"] + size <= self.budget:
                        waiting.remove(r)
                        state["used"] += size
                        state["active"] += 1
                        th = threading.Thread(target=worker, args=(r, size, now()), daemon=True)
                        th.start()
                        threads.append(th)
                    elif self.max_active == 1:
                        break  # plain FIFO: no overtaking
                if errors:
                    break
                timeout = None if nxt >= len(reqs) else max(0.0, reqs[nxt].arrival - now())
                cv.wait(timeout=timeout if timeout is None else min(timeout, 0.5))
        for th in threads:
            th.join()
        if errors:
            raise errors[0]
        return [results[r.rid] for r in sorted(reqs, key=lambda r: r.rid)]


def latency_stats(results):
    lat = np.array([r.latency for r in results])
    span = max(r.done for r in results) - min(r.arrival for r in results)
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "requests": len(results), "span_s": float(span)}


def poisson_requests(n, rate, seed=4, grid=((200, 100), (2001, 1001)), nt=(2000, 6000), shots=(1, 8), dx=10.0,
                     dt=1e-3, pml=20, f0=15.0, grid_scale=1.0, nt_scale=1.0):
    """A seeded Poisson stream of `n` requests at `rate` per second: grids
    uniform in [grid[0], grid[1]] nodes, nt uniform in `nt`, 1..8 shots each;
    layered-plus-anomaly models; observed records are low-level noise (the
    work of a gradient does not depend on them).  grid_scale/nt_scale shrink
    the drawn sizes for bounded runs."""
    from sfwi_gb300 import synth
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    for rid in range(n):
        t += rng.exponential(1.0 / rate)
        allnx = max(48, int(rng.integers(grid[0][0], grid[1][0] + 1) * grid_scale))
        allnz = max(24, int(rng.integers(grid[0][1], grid[1][1] + 1) * grid_scale))
        nsteps = max(60, int(rng.integers(nt[0], nt[1] + 1) * nt_scale))
        ns = int(rng.integers(shots[0], shots[1] + 1))
        vp, vs, rho = synth.layered_model(allnx, allnz, dx, vmin=1500.0, vmax=3500.0, seed=seed + rid)
        sou = synth.ricker(nsteps, dt, f0)
        spacing = max(1, (allnx - 1) // max(ns, 1))
        sh = synth.config_shots(allnx, dx, pml, ns, spacing)
        for d in sh:
            d["isz"], d["igz"] = pml + 2, pml
            d["obs_z"] = (1e-9 * rng.standard_normal((d["ntr"], nsteps))).astype(np.float32)
            d["obs_x"] = (1e-9 * rng.standard_normal((d["ntr"], nsteps))).astype(np.float32)
        out.append(Request(rid, t, allnx, allnz, dx, dt, nsteps, pml, sou, vp, vs, rho, sh))
    return out
