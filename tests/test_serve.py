"""The serving loop (sfwi_gb300/serve.py): admission against the HBM budget,
FIFO order for the one-job loop, latency statistics (host logic, stand-in
runner), and on the GPU the same result for a request alone and in the mix."""
import threading
import time

import numpy as np
import pytest

from sfwi_gb300 import serve


def _fake_requests(sizes, arrivals):
    out = []
    for rid, (size, t) in enumerate(zip(sizes, arrivals)):
        r = serve.Request(rid, t, 0, 0, 10.0, 1e-3, 0, 0, None, None, None, None, [dict(gc=[0])])
        r.size = size
        out.append(r)
    return out


class Recorder:
    """Runner that sleeps and records what ran concurrently."""

    def __init__(self, dur=0.05):
        self.lock = threading.Lock()
        self.active, self.bytes, self.max_active, self.max_bytes = 0, 0, 0, 0
        self.order = []
        self.dur = dur

    def __call__(self, r):
        with self.lock:
            self.active += 1
            self.bytes += r.size
            self.max_active = max(self.max_active, self.active)
            self.max_bytes = max(self.max_bytes, self.bytes)
            self.order.append(r.rid)
        time.sleep(self.dur)
        with self.lock:
            self.active -= 1
            self.bytes -= r.size
        z = np.zeros((1, 1))
        return (float(r.rid), z, z, z)


def test_admission_respects_budget_and_slots():
    reqs = _fake_requests([40, 30, 50, 20, 60, 10], [0.0, 0.0, 0.01, 0.01, 0.02, 0.02])
    rec = Recorder()
    res = serve.Server(100, max_active=3, runner=rec, sizer=lambda r: r.size).run(reqs)
    assert [r.rid for r in res] == list(range(6))
    assert rec.max_bytes <= 100 and rec.max_active <= 3
    assert rec.max_active >= 2  # work overlapped
    assert all(r.done >= r.admitted >= r.arrival - 1e-9 for r in res)


def test_fifo_runs_one_job_at_a_time_in_arrival_order():
    reqs = _fake_requests([40, 30, 50, 20], [0.03, 0.0, 0.02, 0.01])
    rec = Recorder(0.02)
    serve.Server(100, max_active=1, runner=rec, sizer=lambda r: r.size).run(reqs)
    assert rec.max_active == 1
    assert rec.order == [1, 3, 2, 0]


def test_shortest_first_admits_the_least_work_among_the_waiting():
    # one slot; the others arrive while the first runs and start by work
    reqs = _fake_requests([10, 10, 10, 10], [0.0, 0.001, 0.002, 0.003])
    work = {0: 5, 1: 30, 2: 10, 3: 20}
    rec = Recorder(0.05)
    serve.Server(100, max_active=1, runner=rec, sizer=lambda r: r.size, policy="shortest",
                 work=lambda r: work[r.rid]).run(reqs)
    assert rec.order == [0, 2, 3, 1]
    with pytest.raises(ValueError):
        serve.Server(100, policy="random")


def test_oversized_request_is_refused():
    reqs = _fake_requests([200], [0.0])
    with pytest.raises(ValueError):
        serve.Server(100, runner=Recorder(), sizer=lambda r: r.size).run(reqs)


def test_latency_stats():
    z = np.zeros(1)
    res = [serve.Result(i, 0.0, z, z, z, 0.0, 0.0, 0.1 * (i + 1)) for i in range(100)]
    st = serve.latency_stats(res)
    assert st["p50_ms"] == pytest.approx(5050.0) and st["p99_ms"] == pytest.approx(9901.0)


def test_request_bytes_grows_with_the_request():
    a, b = serve.poisson_requests(2, 10.0, grid=((60, 30), (60, 30)), nt=(100, 100), shots=(1, 1))
    b.shots = b.shots + b.shots
    assert serve.request_bytes(b) > serve.request_bytes(a) > 0


class BatchRecorder:
    """Batch runner that sleeps and records the groups it was given."""

    def __init__(self, dur=0.05):
        self.lock = threading.Lock()
        self.groups, self.active, self.max_active = [], 0, 0
        self.dur = dur

    def __call__(self, group):
        with self.lock:
            self.active += 1
            self.max_active = max(self.max_active, self.active)
            self.groups.append([r.rid for r in group])
        time.sleep(self.dur)
        with self.lock:
            self.active -= 1
        z = np.zeros((1, 1))
        return [(float(r.rid), z, z, z) for r in group]


def test_batched_admission_groups_the_waiting_requests():
    # two arrive at once and share the first run; the next three arrive while
    # it runs (one slot) and share the second, within the budget of 60
    reqs = _fake_requests([20, 20, 20, 20, 20, 30], [0.0, 0.0, 0.01, 0.01, 0.02, 0.02])
    rec = BatchRecorder(0.05)
    srv = serve.Server(60, max_active=1, batch=True, batch_runner=rec,
                       batch_sizer=lambda g: sum(r.size for r in g))
    res = srv.run(reqs)
    assert [r.rid for r in res] == list(range(6))
    assert rec.groups[0] == [0, 1]
    assert rec.groups[1] == [2, 3, 4]  # 20+20+20 fit; request 5 (30) waits for the next run
    assert rec.groups[2] == [5]
    assert rec.max_active == 1
    # results of a run complete together
    assert res[2].done == res[3].done == res[4].done
    # at most max_batch requests per run
    rec2 = BatchRecorder(0.02)
    serve.Server(1000, max_active=1, batch=True, batch_runner=rec2, batch_sizer=lambda g: len(g),
                 max_batch=2).run(_fake_requests([1] * 5, [0.0] * 5))
    assert [len(g) for g in rec2.groups] == [2, 2, 1]


def test_batching_window_collects_requests_arriving_close_together():
    # without a window the first request runs alone; with a window the three
    # arrivals within 0.06 s share one run
    arrivals = [0.0, 0.03, 0.06]
    rec = BatchRecorder(0.05)
    serve.Server(100, max_active=1, batch=True, batch_runner=rec, batch_sizer=lambda g: len(g)).run(
        _fake_requests([1] * 3, arrivals))
    assert rec.groups[0] == [0]
    rec = BatchRecorder(0.05)
    res = serve.Server(100, max_active=1, batch=True, batch_runner=rec, batch_sizer=lambda g: len(g),
                       window=2.0).run(_fake_requests([1] * 3, arrivals))
    assert rec.groups == [[0, 1, 2]]
    # the run forms at the last arrival, not when the window closes: no
    # request is still due
    assert 0.06 <= res[0].admitted < 1.0


def test_window_lets_shortest_first_see_requests_arriving_together():
    # one engine at a time: without a window the first arrival (the largest)
    # starts alone; with a window covering the arrivals the least work goes first
    reqs = _fake_requests([50, 10, 40, 20, 30], [0.0, 0.005, 0.01, 0.015, 0.02])
    rec = Recorder(0.02)
    serve.Server(1000, max_active=1, runner=rec, sizer=lambda r: r.size, policy="shortest",
                 work=lambda r: r.size).run(reqs)
    assert rec.order[0] == 0
    rec = Recorder(0.02)
    serve.Server(1000, max_active=1, runner=rec, sizer=lambda r: r.size, policy="shortest", work=lambda r: r.size,
                 window=0.05).run(reqs)
    assert rec.order == [1, 3, 4, 2, 0]


def test_batched_shortest_first_takes_the_least_work_into_the_first_runs():
    # sizes double as work: with a window covering every arrival the runs
    # are the two smallest, then the next two, then the largest
    reqs = _fake_requests([50, 10, 40, 20, 30], [0.0, 0.005, 0.01, 0.015, 0.02])
    rec = BatchRecorder(0.03)
    serve.Server(1000, max_active=1, batch=True, batch_runner=rec, batch_sizer=lambda g: len(g), policy="shortest",
                 work=lambda r: r.size, max_batch=2, window=0.05).run(reqs)
    assert rec.groups == [[1, 3], [4, 2], [0]]


def test_host_strips_shrink_the_device_bytes_of_a_request():
    r = serve.poisson_requests(1, 10.0, grid=((300, 150), (300, 150)), nt=(2000, 2000), shots=(4, 4))[0]
    full, ring = serve.request_bytes(r), serve.request_bytes(r, strip_chunk=100)
    assert ring < full / 2  # records and the grid stay
    assert serve.request_bytes(r, strip_chunk=1000) == full  # a ring of 2 x 1000 steps holds them all
    assert serve.batch_bytes([r], strip_chunk=100) < serve.batch_bytes([r]) / 2
    assert serve.strip_steps(2000, 100) == 200 and serve.strip_steps(2000, 0) == 2000


def test_batch_bytes_covers_its_requests():
    a, b = serve.poisson_requests(2, 10.0, grid=((60, 30), (90, 50)), nt=(100, 140), shots=(1, 2))
    both = serve.batch_bytes([a, b])
    assert both >= max(serve.batch_bytes([a]), serve.batch_bytes([b]))
    assert serve.batch_bytes([a]) >= serve.request_bytes(a) * 0.9


@pytest.mark.gpu
def test_batched_serving_gives_each_request_its_result_alone():
    """The shared-run path: requests of different grids and lengths served in
    shared runs equal each request run alone on its own engine, bit for bit."""
    reqs = serve.poisson_requests(5, 1000.0, seed=9, grid=((64, 32), (110, 48)), nt=(180, 260), shots=(1, 3))
    assert len({r.nt for r in reqs}) > 1 and len({(r.allnx, r.allnz) for r in reqs}) > 1
    alone = [serve.run_request(r) for r in reqs]
    mixed = serve.run_requests(reqs)
    host = serve.run_requests(reqs, strip_chunk=37)  # edge strips in host memory
    res = serve.Server(8 << 30, max_active=2, batch=True).run(reqs)
    sjf = serve.Server(8 << 30, max_active=2, batch=True, policy="shortest", max_batch=2, window=0.05).run(reqs)
    # host-held strips with the pinned cache on: engines reuse each other's blocks
    hsrv = serve.Server(8 << 30, max_active=2, batch=True, max_batch=2, strip_chunk=23).run(reqs)
    for a, m, h, r, q, k in zip(alone, mixed, host, res, sjf, hsrv):
        assert a[0] == m[0] == h[0] == r.misfit == q.misfit == k.misfit
        for x, y, u, z, w, v in zip(a[1:], m[1:], h[1:], (r.grad_pp, r.grad_ps, r.illum),
                                    (q.grad_pp, q.grad_ps, q.illum), (k.grad_pp, k.grad_ps, k.illum)):
            assert np.array_equal(x, y) and np.array_equal(x, u) and np.array_equal(x, z) and np.array_equal(x, w)
            assert np.array_equal(x, v)


@pytest.mark.gpu
def test_request_gives_the_same_result_alone_and_in_the_mix():
    reqs = serve.poisson_requests(4, 1000.0, seed=7, grid=((64, 32), (110, 48)), nt=(180, 260), shots=(1, 3))
    alone = [serve.run_request(r) for r in reqs]
    res = serve.Server(8 << 30, max_active=4).run(reqs)
    for a, r in zip(alone, res):
        assert a[0] == r.misfit
        for x, y in zip(a[1:], (r.grad_pp, r.grad_ps, r.illum)):
            assert np.array_equal(x, y)


def test_a_budget_of_zero_refuses_every_request():
    reqs = _fake_requests([1, 2], [0.0, 0.0])
    srv = serve.Server(0, max_active=4, runner=Recorder(), sizer=lambda r: r.size)
    with pytest.raises(ValueError, match="more than the whole budget"):
        srv.run(reqs)


def test_a_failing_request_is_reported_and_frees_its_slot():
    """A runner that dies in one request (its worker thread ends with an
    exception): the others still run to completion or are not started, the
    failure reaches the caller, and no slot or budget stays taken."""
    rec = Recorder(dur=0.02)

    def runner(r):
        if r.rid == 1:
            raise RuntimeError("request 1 failed")
        return rec(r)

    reqs = _fake_requests([10, 10, 10, 10], [0.0, 0.0, 0.01, 0.02])
    srv = serve.Server(20, max_active=2, runner=runner, sizer=lambda r: r.size)
    t = time.perf_counter()
    with pytest.raises(RuntimeError, match="request 1 failed"):
        srv.run(reqs)
    assert time.perf_counter() - t < 5.0
    assert rec.active == 0 and rec.bytes == 0
