"""Serving loop: forward-plus-gradient requests of different grid sizes on one
GPU, admitted against a fixed HBM budget while others are running.

A request is one model (vp, vs, rho on its own allnx x allnz grid) with 1..8
shots and their observed records; its result is the misfit and the FP64
Vp/Vs gradients and illumination.  Requests arrive over time.  The server
admits arrived requests as soon as a slot is free and their device memory
fits in what the running work leaves of the budget (oldest first; a younger
request that fits may pass an older one that does not yet fit).

Two ways to run what is admitted:
  - batched (Server(batch=True)): every request admitted at once joins ONE
    run of the engine, sfwi_run_models: all their shots, on their own models,
    grids and numbers of time steps, advance in the same kernel launches, so
    small requests fill the tile queue of large ones instead of running
    launch-bound on their own.  Up to max_active such runs overlap on the
    device, each on its own engine and stream, and requests that arrive
    while runs are in flight form the next run as soon as a slot frees up;
  - one engine per request (the default), each on its own stream.
`Server(max_active=1)` without batching is the plain one-job-at-a-time FIFO.

Results do not depend on what else is running: every shot's arithmetic is
independent of the other shots of its run and the kernels are
deterministic, so a request gives the same numbers, bit for bit, alone and
in the mix, batched or not (tests/test_serve.py, tests/test_model_batches.py).
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


def strip_steps(nt, strip_chunk=0):
    """Steps of edge strips the device holds: nt, or the two-chunk ring when
    the strips live in host memory (sfwi_set_cpu_mem)"""
    return 2 * strip_chunk if 0 < strip_chunk and 2 * strip_chunk < nt else nt


def request_bytes(req, strip_chunk=0):
    """Device memory of one request's engine (the engine's allocations,
    sfwi_engine.cu:upload_batch, plus the model and the FP64 gradients);
    strip_chunk > 0: edge strips in host memory in chunks of that many steps."""
    P = (req.allnz + 2 * req.pml + 3) // 4 * 4
    X = sum(int(d["nx"]) + 2 * req.pml for d in req.shots)
    ntr = sum(len(d["gc"]) for d in req.shots)
    nt, ns = req.nt, len(req.shots)
    ss = strip_steps(nt, strip_chunk)
    floats = (NGRID * X * P                       # wavefields, memory variables, coefficients
              + ss * 4 * X * 8 + ss * 4 * ns * 8 * P  # edge strips
              + nt * 2 * X                        # receiver-row records
              + X * ((2 * nt + 3) // 4 * 4)       # residual source
              + NREC * ntr * nt                   # records
              + 5 * req.allnx * req.allnz + nt)   # model, wavelet
    return 4 * floats + 8 * 4 * req.allnx * req.allnz + (1 << 20)


def batch_bytes(reqs, strip_chunk=0):
    """Device memory of one shared run of several requests: the packed grid
    at the deepest request's depth, strips and records for the longest
    request's nt, the models and their FP64 gradients."""
    pml = reqs[0].pml
    P = (max(r.allnz for r in reqs) + 2 * pml + 3) // 4 * 4
    X = sum(int(d["nx"]) + 2 * pml for r in reqs for d in r.shots)
    ntr = sum(len(d["gc"]) for r in reqs for d in r.shots)
    nt = max(r.nt for r in reqs)
    ns = sum(len(r.shots) for r in reqs)
    cells = sum(r.allnx * r.allnz for r in reqs)
    ss = strip_steps(nt, strip_chunk)
    floats = (NGRID * X * P + ss * 4 * X * 8 + ss * 4 * ns * 8 * P + nt * 2 * X + X * ((2 * nt + 3) // 4 * 4)
              + NREC * ntr * nt + 5 * cells + nt)
    return 4 * floats + 8 * 4 * cells + (1 << 20)


def run_requests(reqs, strip_chunk=0):
    """Several requests in one run of one engine (sfwi_run_models): a list of
    (misfit, grad_pp, grad_ps, illum), one per request."""
    import sfwi_gb300 as sg
    pml, dx, dt = reqs[0].pml, reqs[0].dx, reqs[0].dt
    for r in reqs:
        if (r.pml, r.dx, r.dt) != (pml, dx, dt) or r.misfit_kind != reqs[0].misfit_kind:
            raise ValueError("requests of one run share spacing, dt, PML width and misfit")
    nt = max(r.nt for r in reqs)
    longest = max(reqs, key=lambda r: r.nt)
    for r in reqs:  # every request's wavelet is the start of the run's
        if not np.array_equal(np.asarray(r.sou, np.float32), np.asarray(longest.sou, np.float32)[:r.nt]):
            raise ValueError("request %d: its wavelet is not the start of the run's" % r.rid)
    allnx = max(r.allnx for r in reqs)
    allnz = max(r.allnz for r in reqs)
    maxnx = max(int(d["nx"]) for r in reqs for d in r.shots)
    fd = sg.FD2DGPU_ELASTIC(longest.sou, dx, dx, dt, maxnx + 2 * pml, allnz + 2 * pml, allnx, allnz, 1, pml, nt, 4,
                            0, stage=1)
    try:
        if reqs[0].misfit_kind:
            fd.set_misfit(reqs[0].misfit_kind)
        if strip_chunk:
            fd.set_cpu_mem(1, strip_chunk)
        shot_model = []
        for k, r in enumerate(reqs):
            for d in r.shots:
                fd.enqueue_shot(d["nx"], d["isx"], d["isz"], d["igz"], d["ngx_left"], d["delta_left"], 0, d["gc"],
                                d["obs_z"], d["obs_x"], nt=r.nt)
                shot_model.append(k)
        models = [dict(vp=r.vp, vs=r.vs, rho=r.rho, nt=r.nt) for r in reqs]
        per, grads = fd.run_models(models, shot_model)
    finally:
        fd.close()
    out, i = [], 0
    for r, g in zip(reqs, grads):
        m = 0.0
        for _ in r.shots:  # the request's shots in its own order, as a run of it alone sums them
            m += float(per[i])
            i += 1
        out.append((m,) + tuple(g[:3]))
    return out


def request_work(req):
    """Cell-steps of one request (its shots' padded cells times nt): the
    order of the shortest-first policy."""
    P = req.allnz + 2 * req.pml
    return sum((int(d["nx"]) + 2 * req.pml) * P for d in req.shots) * req.nt


def run_request(req, strip_chunk=0):
    """One request on a fresh engine: (misfit, grad_pp, grad_ps, illum)."""
    import sfwi_gb300 as sg
    maxnx = max(int(d["nx"]) for d in req.shots)
    fd = sg.FD2DGPU_ELASTIC(req.sou, req.dx, req.dx, req.dt, maxnx + 2 * req.pml, req.allnz + 2 * req.pml, req.allnx,
                            req.allnz, 1, req.pml, req.nt, 4, len(req.shots[0]["gc"]), stage=1)
    try:
        fd.GPUbufferVPVS(req.vp, req.vs, req.rho)
        if req.misfit_kind:
            fd.set_misfit(req.misfit_kind)
        if strip_chunk:
            fd.set_cpu_mem(1, strip_chunk)
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
    loop is the plain FIFO.  Requests are admitted once the oldest waiting
    request has waited `window` seconds (or no request is still due), so
    that requests arriving close together are ordered (and, batched, run)
    together.

    Batched (batch=True): the requests admitted together share one run, at
    most max_batch of them.  strip_chunk > 0 keeps every run's edge strips in host memory
    in chunks of that many steps (sfwi_set_cpu_mem): the budget then counts
    the device ring only, and more requests fit at once.  During run() the
    pinned blocks that finished engines release are kept (up to
    pinned_cache_bytes) for the next engines, and freed when it returns."""

    def __init__(self, budget_bytes, max_active=4, runner=None, sizer=None, clock=time.perf_counter,
                 policy="oldest", work=request_work, batch=False, batch_runner=None, batch_sizer=None,
                 max_batch=64, window=0.0, strip_chunk=0, pinned_cache_bytes=64 << 30):
        if policy not in ("oldest", "shortest"):
            raise ValueError("policy must be 'oldest' or 'shortest'")
        self.budget = int(budget_bytes)
        self.max_active = int(max_active)
        sc = int(strip_chunk)
        self.runner = runner or (lambda r: run_request(r, sc))
        self.sizer = sizer or (lambda r: request_bytes(r, sc))
        self.clock = clock
        self.policy, self.work = policy, work
        # batched: the requests admitted together share one run (batch_runner)
        self.batch = batch
        self.batch_runner = batch_runner or (lambda g: run_requests(g, sc))
        self.batch_sizer = batch_sizer or (lambda g: batch_bytes(g, sc))
        self.max_batch = int(max_batch)
        self.window = float(window)
        self.strip_chunk = sc
        self.pinned_cache_bytes = int(pinned_cache_bytes)

    def run(self, requests):
        """Replay `requests` (arrival offsets in seconds) against the wall
        clock and serve them; returns the results in request-id order."""
        if self.strip_chunk <= 0:
            return self._run(requests)
        import sfwi_gb300 as sg
        sg.set_pinned_cache(self.pinned_cache_bytes)
        try:
            return self._run(requests)
        finally:
            sg.set_pinned_cache(0)

    def _run(self, requests):
        reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
        for r in reqs:
            need = self.batch_sizer([r]) if self.batch else self.sizer(r)
            if need > self.budget:
                raise ValueError("request %d needs %d bytes, more than the whole budget" % (r.rid, need))
        cv = threading.Condition()
        waiting, results, errors = [], {}, []
        state = {"used": 0, "active": 0}
        t0 = self.clock()

        def now():
            return self.clock() - t0

        def worker(group, size, admitted):
            try:
                outs = self.batch_runner(group) if self.batch else [self.runner(group[0])]
                done = now()
                with cv:
                    for r, out in zip(group, outs):
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
                # admit every arrived request that fits, oldest or least work first,
                # once the oldest waiting one has waited `window` seconds (or
                # no request is still due)
                order = list(waiting) if self.policy == "oldest" else sorted(waiting, key=lambda q: (self.work(q), q.rid))
                due = bool(waiting) and (nxt >= len(reqs) or t - min(q.arrival for q in waiting) >= self.window)
                if not due:
                    order = []
                if self.batch:
                    # one shared run of every waiting request that fits the budget
                    if state["active"] < self.max_active and order:
                        group, size = [], 0
                        for r in order:
                            if len(group) >= self.max_batch:
                                break
                            trial = self.batch_sizer(group + [r])
                            if state["used"] + trial <= self.budget:
                                group.append(r)
                                size = trial
                        if group:
                            for r in group:
                                waiting.remove(r)
                            state["used"] += size
                            state["active"] += 1
                            th = threading.Thread(target=worker, args=(group, size, now()), daemon=True)
                            th.start()
                            threads.append(th)
                    order = []
                for r in order:
                    if state["active"] >= self.max_active:
                        break
                    size = self.sizer(r)
                    if state["used"] + size <= self.budget:
                        waiting.remove(r)
                        state["used"] += size
                        state["active"] += 1
                        th = threading.Thread(target=worker, args=([r], size, now()), daemon=True)
                        th.start()
                        threads.append(th)
                    elif self.max_active == 1:
                        break  # plain FIFO: no overtaking
                if errors:
                    break
                timeout = None if nxt >= len(reqs) else max(0.0, reqs[nxt].arrival - now())
                if self.window > 0 and waiting and state["active"] < self.max_active and nxt < len(reqs):
                    # wake when the oldest waiting request's window closes
                    dl = max(0.0, min(q.arrival for q in waiting) + self.window - now())
                    timeout = dl if timeout is None else min(timeout, dl)
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
