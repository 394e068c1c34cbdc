"""Benchmark: shot-gradients per second of one FWI gradient pass.

Workload (default): one stage-1 FWI iteration at 376x201, dx=dz=10 m, PML 20,
nt=3000, dt=1 ms, 15 Hz Ricker; 38 shots 10 nodes apart, 376 surface
receivers each (full-aperture windows); each shot runs the background +
Born-scattered forward, the 1D optimal-transport adjoint source and the
adjoint gradient.  Models are seeded synthetics (layered Vp 1500-4500 m/s with
three +-10% Gaussian anomalies, Vs = Vp/1.73, Gardner rho); observed data are
modelled on the true model, the gradient is taken on a z-smoothed start model
with the Born perturbation = true - start.

A step = one gradient pass over all 38 shots (one sfwi_run call).  `value`
counts device time only (CUDA events on the engine's stream, inputs resident);
`e2e` times the public API call from host buffers: per step the observed
records are copied host->device from page-locked memory and the gradients and
misfit are read back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# one process per GPU under torchrun: pin this process's device before any CUDA use
# (SFWI_SHARE_GPU=1 keeps every rank on the first device: a check of the
# multi-rank path on a one-GPU machine, whose ranks never wait on each other)
if ("LOCAL_RANK" in os.environ and int(os.environ.get("WORLD_SIZE", "1")) > 1
        and os.environ.get("SFWI_SHARE_GPU") != "1"):
    os.environ["CUDA_VISIBLE_DEVICES"] = os.environ["LOCAL_RANK"]

import numpy as np  # noqa: E402

WORKLOADS = {
    # one plain stage-1 shot-gradient at 376x201: vertical-force source at
    # node (188, 2), OT misfit, no Born term
    "shot376": dict(name="plain-shot-376x201-stage1-vzforce-ot", allnx=376, allnz=201, dx=10.0, pml=20, nt=3000,
                    dt=1e-3, f0=15.0, nshots=1, spacing=10, first=188, sy=2, gy=0, model="layered", aperture=None,
                    misfit="OT", stage=1, source="vz",
                    # forward 72 + adjoint 72 + reconstruction 72 + imaging 32
                    pass_bytes=248),
    # one FWI iteration at 376x201 (the headline line)
    "fwi376": dict(name="fwi-iteration-376x201-38shots-born-ot", allnx=376, allnz=201, dx=10.0, pml=20, nt=3000,
                   dt=1e-3, f0=15.0, nshots=38, spacing=10, sy=2, gy=0, model="layered", aperture=None, misfit="OT",
                   rho_grad=True),
    # stage-2 batch at 401x301, 12.5 m: salt body, 80 shots with seeded
    # window widths of 150-401 nodes
    "salt401": dict(name="stage2-salt-401x301-80shots-uneven-apertures", allnx=401, allnz=301, dx=12.5, pml=20,
                    nt=4000, dt=1e-3, f0=15.0, nshots=80, spacing=5, sy=2, gy=0, model="salt", aperture=(150, 401),
                    misfit="L2"),
    # compressed-snapshot gradient at 2001x801, 5 m, dt 0.5 ms, 25 Hz: FP16
    # snapshots of vx, vz every 4th step instead of the reconstruction
    "snap2001": dict(name="snapshot-gradient-2001x801-16shots-fp16-every4", allnx=2001, allnz=801, dx=5.0, pml=20,
                     nt=6000, dt=5e-4, f0=25.0, nshots=16, spacing=125, sy=2, gy=0, model="layered", aperture=None,
                     misfit="OT", snap=(4, "f16"),
                     # forward 152 + adjoint 72 + imaging 32/4 + snapshot write and read 2 comps x 2 B x 2 / 4
                     pass_bytes=234),
}
WORKLOAD = WORKLOADS["fwi376"]
METRIC = "shot-gradients/s"

# algorithmic bytes per padded cell per time step of each kernel (FP32; each
# array read once and written once per sweep, stencil neighbours reused on
# chip, PML memory variables not counted)
KERNEL_BYTES = {
    "k_fwd_v": 32,         # read sigma(3) + 1/rho; RMW v(2)
    "k_fwd_s": 40,         # read v(2) + lam, mu; RMW sigma(3)
    "k_fwd_v<born>": 60,   # read sigma(3) + sigma_s(3) + 1/rho; RMW v(2) + v_s(2)
    "k_fwd_s<born>": 80,   # read v(2) + v_s(2) + lam, mu, bp, bs; RMW sigma(3) + sigma_s(3)
    "k_bwd_s": 88,         # read v(2) + v_adj(2) + lam, mu; RMW sigma(3) + sigma_adj(3) + G_lam, G_mu
    "k_bwd_v": 76,         # read sigma(3) + sigma_adj(3) + lam, mu, 1/rho; RMW v(2) + v_adj(2) + illum
    # snapshot mode, every 4th step imaging (per-launch average): read v_adj(2), RMW sigma_adj(3);
    # at 1 launch in 4: snapshot vx, vz (2 x 2 B) + RMW G_lam, G_mu, illum
    "k_bwd_s_snap<f16>": 32 + (4 + 24) / 4,
    "k_bwd_s_snap<bf16>": 32 + (4 + 24) / 4,
    "k_bwd_s_snap<f32>": 32 + (8 + 24) / 4,
    "k_bwd_v_snap": 40,    # read sigma_adj(3) + lam, mu, 1/rho; RMW v_adj(2)
}
# algorithmic bytes per padded cell per time step of a Born shot-gradient:
# forward 72 + reconstruction 72 + adjoint 72 + imaging 32 + Born add-on 80
PASS_BYTES_PER_CELL_STEP = 328


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def build_workload(w):
    from sfwi_gb300 import synth
    if w.get("model") == "salt":
        vp, vs, rho = synth.salt_model(w["allnx"], w["allnz"], w["dx"])
    else:
        vp, vs, rho = synth.layered_model(w["allnx"], w["allnz"], w["dx"])
    vp0 = synth.smooth_z(vp, 10)
    vs0 = (vp0 / 1.73).astype(np.float32)
    rho0 = (310.0 * vp0.astype(np.float64) ** 0.25).astype(np.float32)
    shots = synth.config_shots(w["allnx"], w["dx"], w["pml"], w["nshots"], w["spacing"], first=w.get("first"),
                               aperture=w.get("aperture"))
    sou = ricker(w["nt"], w["dt"], w["f0"])
    return dict(vp=vp, vs=vs, rho=rho, vp0=vp0, vs0=vs0, rho0=rho0, dvp=(vp - vp0).astype(np.float32),
                dvs=(vs - vs0).astype(np.float32), shots=shots, sou=sou)


L2_BYTES = 129e6  # GB300 L2


def l2_note(cells, nt, nshots, w):
    """How the timed steps relate to L2: a step is a whole pass of nt time
    steps, each of which reads and writes the whole wavefield state once per
    sweep; the state either exceeds L2 or stays in it across the sweeps."""
    state = cells * 4 * 41
    strips = 0 if w.get("snap") else 4 * nt * 2 * 8 * 4 * (cells / max(1, nshots)) ** 0.5 * nshots
    if state > L2_BYTES:
        return "inputs larger than L2: wavefield state %.2f GB per sweep" % (state / 1e9)
    return ("wavefield state %.0f MB fits in L2 and stays there across the sweeps of a pass (a step is a whole "
            "pass of %d time steps, no flush between steps); records and edge strips (~%.0f MB per pass) "
            "stream through HBM" % (state / 1e6, nt, strips / 1e6))


def ricker(nt, dt, fm):
    """Ricker wavelet as the reference computes it (sfwi-stage1/main.cpp:251-260)."""
    from sfwi_gb300 import synth
    return synth.ricker(nt, dt, fm)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.samples, self.proc = [], None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx = max(mx, float(s[2]))
                for n, v in zip(names, s[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def traffic_per_cell(kernel):
    """DRAM bytes per padded cell per launch of `kernel` from the committed
    ncu capture summary (profiles/traffic_per_cell.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic_per_cell.json")) as f:
            v = json.load(f).get(kernel)
        return float(v) if v is not None else None
    except (OSError, ValueError):
        return None


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_baseline_sample(w, data, nthreads, nt_sample, kind="port"):
    """Time one shot-gradient of the workload with nt_sample time steps on the
    host (the oracle: 'port' = FP32 transliteration, 'reference' = the
    reference's kernels built for the CPU), scaled to the full nt."""
    from oracle import pyoracle as po
    po.build()
    d = data["shots"][len(data["shots"]) // 2]
    nt = nt_sample
    stage = w.get("stage", 2)
    shot = dict(stage=stage, allnx=w["allnx"], allnz=w["allnz"], nx=d["nx"], pml=w["pml"], nop=4, nt=nt, ntr=d["ntr"],
                dx=w["dx"], dz=w["dx"], dt=w["dt"], isx=d["isx"], isz=w["pml"] + w["sy"], igz=w["pml"] + w["gy"],
                ngx_left=d["ngx_left"], delta_left=d["delta_left"], record_left_in_v=0, forward_only=0,
                misfit_kind=0 if kind == "reference" else 1, nthreads=nthreads,
                src_kind=1 if w.get("source") == "vz" and kind != "reference" else 0)
    rng = np.random.default_rng(0)
    model = dict(vp=data["vp0"], vs=data["vs0"], rho=data["rho0"], dvp=data["dvp"], dvs=data["dvs"],
                 sou=data["sou"][:nt], gc=d["gc"],
                 obs_z=(1e-9 * rng.standard_normal((d["ntr"], nt))).astype(np.float32),
                 obs_x=(1e-9 * rng.standard_normal((d["ntr"], nt))).astype(np.float32))
    lib = {"port": "f32", "reference": "ref%d" % stage}[kind]
    t = time.perf_counter()
    po.run_shot(lib, shot, model)
    el = time.perf_counter() - t
    per_shot = el * w["nt"] / nt
    return 1.0 / per_shot, el


def reference_gpu_sample(w, data, nshots, warm=True):
    """The reference's own CUDA kernels (oracle/ref_gpu_harness.cpp) on this
    GPU, one shot at a time as the reference runs them: `nshots` shots of the
    workload at the full nt, wall-clock per shot including the per-shot
    allocations and copies the reference makes.  Its misfit is L2 (the
    reference has no OT)."""
    from oracle import pyoracle as po
    stage = w.get("stage", 2)
    try:
        if not po.build_refgpu() or not po.available("gpu%d" % stage):
            return {"unavailable": "the reference's device-code modules are not in oracle/_ref"}
        po.load("gpu%d" % stage)
    except Exception as e:  # noqa: BLE001 - reported, not fatal
        return {"unavailable": "reference GPU harness: %s" % e}
    shots = data["shots"]
    pick = shots[:: max(1, len(shots) // nshots)][:nshots]
    rng = np.random.default_rng(0)
    els = []
    for j, d in enumerate((pick[:1] if warm else []) + pick):  # the first run is a warm-up
        shot = dict(stage=stage, allnx=w["allnx"], allnz=w["allnz"], nx=d["nx"], pml=w["pml"], nop=4, nt=w["nt"],
                    ntr=d["ntr"], dx=w["dx"], dz=w["dx"], dt=w["dt"], isx=d["isx"], isz=w["pml"] + w["sy"],
                    igz=w["pml"] + w["gy"], ngx_left=d["ngx_left"], delta_left=d["delta_left"], record_left_in_v=0,
                    forward_only=0, misfit_kind=0, nthreads=0)
        model = dict(vp=data["vp0"], vs=data["vs0"], rho=data["rho0"], dvp=data["dvp"], dvs=data["dvs"],
                     sou=data["sou"], gc=d["gc"],
                     obs_z=(1e-9 * rng.standard_normal((d["ntr"], w["nt"]))).astype(np.float32),
                     obs_x=(1e-9 * rng.standard_normal((d["ntr"], w["nt"]))).astype(np.float32))
        t = time.perf_counter()
        po.run_shot("gpu%d" % stage, shot, model)
        if j > 0 or not warm:
            els.append(time.perf_counter() - t)
    per = float(np.mean(els))
    return {"value": round(1.0 / per, 3), "unit": "shot-gradients/s", "ms_per_shot": round(per * 1e3, 1),
            "shots_sampled": len(els),
            "sample": "the reference's CUDA kernels (its born.cu and FD2DGPU.cu kernels, nvcc -O3 for sm_103a, "
                      "64-register cap) in IMAGE_SINGLESHOT's launch sequence, one shot at a time, L2 misfit, "
                      "wall clock per shot"}


def run_serving(n, budget_gb=64.0, full=True):
    """Serving loop on a seeded Poisson stream (50 requests/s; grids 200x100
    to 2001x1001, nt 2000-6000 and 1-8 shots drawn per request; with
    full=False scaled by 0.3 in each grid dimension and 0.1 in nt).  Four
    servers on the same stream, each replayed once after one warm request:
      fifo                   one request at a time in arrival order;
      served_shortest_first  two requests at once, each on its own engine and
                             stream, least work first, admitted once the
                             oldest waiting request has waited 0.3 s;
      batched                the requests admitted together share one engine
                             run (sfwi_run_models), two runs in flight;
      batched_shortest_first as batched, but a run forms once the oldest
                             waiting request has waited 0.3 s, from the
                             least-work requests, at most 4 per run;
      served_shortest_first_host_strips_8gb
                             served_shortest_first in an 8 GB budget, the
                             edge strips in pinned host memory (100-step
                             chunks; pinned blocks reused across engines).
    FIFO is replayed first and last (the line reports the first; `fifo_last`
    shows the drift between replays on the same box).
    At the drawn sizes a request takes up to several seconds of GPU time, so
    a stream at 50/s queues: the latencies measure the backlog."""
    from sfwi_gb300 import serve
    gs, ns = (1.0, 1.0) if full else (0.3, 0.1)
    reqs = serve.poisson_requests(n, 50.0, seed=4, grid_scale=gs, nt_scale=ns)
    serve.run_request(reqs[0])  # warm the kernels and the allocator
    out = {"requests": n, "rate_per_s": 50.0, "budget_gb": budget_gb,
           "shot_gradients": sum(r.shot_gradients for r in reqs),
           "scale": "the drawn sizes" if full else "grids x0.3 per dimension, nt x0.1 of the drawn sizes"}
    B = budget_gb * 2 ** 30
    for name, srv in (("fifo", serve.Server(B, max_active=1)),
                      ("served_shortest_first", serve.Server(B, max_active=2, policy="shortest", window=0.3)),
                      ("batched", serve.Server(B, max_active=2, batch=True)),
                      ("batched_shortest_first", serve.Server(B, max_active=2, batch=True, policy="shortest",
                                                              max_batch=4, window=0.3)),
                      ("served_shortest_first_host_strips_8gb",
                       serve.Server(min(B, 8 << 30), max_active=2, policy="shortest", window=0.3, strip_chunk=100)),
                      ("fifo_last", serve.Server(B, max_active=1))):
        if not full:
            srv.run(reqs)  # short requests: a first replay settles the allocator pools and host threads
        res = srv.run(reqs)
        st = serve.latency_stats(res)
        st["shot_gradients_per_s"] = sum(r.shot_gradients for r in reqs) / st["span_s"]
        out[name] = {k: round(v, 3) if isinstance(v, float) else v for k, v in st.items()}
    f = out["fifo"]
    for name in ("served_shortest_first", "batched", "batched_shortest_first", "served_shortest_first_host_strips_8gb"):
        o = out[name]
        o["vs_fifo"] = {"p50": round(o["p50_ms"] / f["p50_ms"], 3), "p99": round(o["p99_ms"] / f["p99_ms"], 3),
                        "throughput": round(o["shot_gradients_per_s"] / f["shot_gradients_per_s"], 3)}
    return out


def run_reference_arm(args, w):
    ws, rank = dist_info()
    if rank != 0:
        return 0
    from oracle import pyoracle as po
    ref = "ref%d" % w.get("stage", 2)
    kind = "reference" if po.available(ref) else "port"
    try:
        if kind == "reference":
            po.load(ref)
    except OSError:
        kind = "port"
    data = build_workload(w)
    threads = os.cpu_count() or 1
    nt_sample = 200
    for _ in range(args.warmup):
        cpu_baseline_sample(w, data, threads, 20, kind)
    vals, els = [], []
    for _ in range(args.steps):
        v, el = cpu_baseline_sample(w, data, threads, nt_sample, kind)
        vals.append(v)
        els.append(el)
    value = float(np.mean(vals))
    sample = "one %dx%d shot (stage-2 Born forward + %s adjoint), %d of %d time steps, scaled by nt" % (
        w["allnx"], w["allnz"], "L2" if kind == "reference" else "OT", nt_sample, w["nt"])
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "shot-gradients/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.mean(els)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["name"], "cpu": True, "sample": sample},
            "cpu_baseline": {"value": value, "unit": "shot-gradients/s", "cores": threads, "cpu_model": cpu_model(),
                             "kind": kind,
                             "sample": sample},
            "e2e": {"value": value, "unit": "shot-gradients/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def cpu_model():
    """the host CPU's model name (lscpu), for the baseline lines"""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


def observed_records(sg, w, data):
    """background records of the true model (untimed), in page-locked host
    buffers: the observed data of every shot"""
    pml, nt = w["pml"], w["nt"]
    shots = data["shots"]
    isz, igz = pml + w["sy"], pml + w["gy"]
    fwd = sg.FD2DGPU_ELASTIC(data["sou"], w["dx"], w["dx"], w["dt"], w["allnx"] + 2 * pml, w["allnz"] + 2 * pml,
                             w["allnx"], w["allnz"], 1, pml, nt, 4, shots[0]["ntr"], stage=1)
    fwd.GPUbufferVPVS(data["vp"], data["vs"], data["rho"])
    if w.get("source") == "vz":
        fwd.set_source(sg.SOURCE_VZ_FORCE)
    for d in shots:
        fwd.enqueue_shot(d["nx"], d["isx"], isz, igz, d["ngx_left"], d["delta_left"], 0, d["gc"])
    fwd.run_forward()
    obs = []
    for i, d in enumerate(shots):
        r = fwd.read_records(i, d["ntr"])
        pz, px = sg.PinnedArray((d["ntr"], nt)), sg.PinnedArray((d["ntr"], nt))
        pz.array[...] = r["syn_z"]
        px.array[...] = r["syn_x"]
        obs.append((pz, px))
    fwd.close()
    return obs


def measure(w, args, steps, warmup, plain_shots, pg=None, ws=1, rank=0, clocks=None, snap_check=0):
    """One workload: `warmup` untimed passes (the autotuner after the first),
    then `steps` timed passes through sfwi_run (device time from CUDA events
    inside the engine; wall clock around the whole public call for e2e), the
    per-kernel launch times, and the plain one-shot-at-a-time form on an
    evenly spread sample of `plain_shots` shots.  With N ranks the survey's
    shots are taken N times over and split by cost (sfwi_gb300.shard), each
    rank runs its share and the FP64 gradients and misfit are summed over
    the ranks inside every timed step (weak scaling).  Returns a dict."""
    import sfwi_gb300 as sg
    from sfwi_gb300 import shard
    data = build_workload(w)
    stage = w.get("stage", 2)
    nt, pml = w["nt"], w["pml"]
    nxpml, nzpml = w["allnx"] + 2 * pml, w["allnz"] + 2 * pml
    base = data["shots"]
    isz, igz = pml + w["sy"], pml + w["gy"]
    obs = observed_records(sg, w, data)
    # this rank's shots, as indices into the survey's (all of them on one rank)
    mine = list(range(len(base)))
    if pg is not None and ws > 1:
        every = [i for _ in range(ws) for i in range(len(base))]
        part = shard.partition([shard.shot_cost(base[i], pml, nzpml, nt) for i in every], ws)[rank]
        mine = [every[k] for k in part]
    shots = [base[i] for i in mine]
    kbytes = dict(KERNEL_BYTES)
    fd = sg.FD2DGPU_ELASTIC(data["sou"], w["dx"], w["dx"], w["dt"], nxpml, nzpml, w["allnx"], w["allnz"], 1, pml, nt,
                            4, shots[0]["ntr"], stage=stage)
    if stage == 2:
        fd.GPUbufferVPVS(data["vp0"], data["vs0"])
        fd.GPUbufferM(data["dvp"], data["dvs"])
    else:
        fd.GPUbufferVPVS(data["vp0"], data["vs0"], data["rho0"])
    if w.get("source") == "vz":
        fd.set_source(sg.SOURCE_VZ_FORCE)
    if getattr(args, "tile_order", None) is not None:
        fd.set_tile_order(args.tile_order)
    if w["misfit"] == "OT":
        fd.set_misfit(sg.MISFIT_OT)
    if w.get("snap"):
        fd.set_snapshots(*w["snap"])
    if w.get("rho_grad"):
        fd.set_density_gradient(True)
        kbytes["k_bwd_v"] += 8  # the density kernel's accumulator, read and written

    def enqueue(d, i):
        b = mine[i]  # the survey shot whose observed records these are
        fd.enqueue_shot(d["nx"], d["isx"], isz, igz, d["ngx_left"], d["delta_left"], 0, d["gc"], obs[b][0].array,
                        obs[b][1].array)

    allreduce_s = []

    def step():
        for i, d in enumerate(shots):
            enqueue(d, i)
        m, _ = fd.run()
        if pg is not None:
            # the reference's gradient reduction (sfwi-stage1/main.cpp:637-666)
            g64 = list(fd.read_gradients_f64())
            if w.get("rho_grad"):
                g64.append(fd.read_density_gradient_f64())
            t = time.perf_counter()
            m = shard.allreduce_gradients(g64, m)
            allreduce_s.append(time.perf_counter() - t)
            fd.imagebuffer_resettozero()
            return m, g64
        grho = fd.read_density_gradient_f64() if w.get("rho_grad") else None
        g = fd.imagebuffer_resettozero()
        return m, (g, grho)

    tune = None
    if args.tile != "auto":
        fd.set_tile_shape(args.tile)
    t0 = time.perf_counter()
    m = None
    for i in range(warmup):
        m, g = step()
        if i == 0 and args.tile == "auto":
            # tile shape: time every shape on the resident batch, keep the
            # fastest; the remaining warm-up steps capture its graphs
            choice, tms = fd.autotune(reps=5)
            tune = {"choice": choice, "ms_per_step": {k: round(v, 4) for k, v in tms.items()}}
            log("%s autotune: %s" % (w["name"], tune))
    if tune and warmup < 2:
        m, g = step()  # the chosen shape's graphs are captured outside the timed steps
    log("%s warm-up: %d steps in %.2f s, misfit %.6e" % (w["name"], warmup, time.perf_counter() - t0, m or 0.0))
    out = {"fd": fd, "shots": shots, "obs": obs, "tune": tune, "data": data}
    if args.profile_kernels:
        return out

    if pg:
        pg.barrier()
    if clocks:
        clocks.start()
    launches0 = fd.kernel_launches()
    dev_ms, fwd_ms, bwd_ms, mis_ms = [], [], [], []
    del allreduce_s[:]
    wall0 = time.perf_counter()
    step_walls = []
    for _ in range(steps):
        ts = time.perf_counter()
        m, g = step()
        step_walls.append(time.perf_counter() - ts)
        t = fd.last_timing()
        dev_ms.append(t["total_ms"])
        fwd_ms.append(t["forward_ms"])
        bwd_ms.append(t["backward_ms"])
        mis_ms.append(t["misfit_ms"])
    wall = time.perf_counter() - wall0
    launches = fd.kernel_launches() - launches0
    clk = clocks.stop() if clocks else None
    total_dev_s = sum(dev_ms) / 1000.0
    if pg:
        import torch
        tt = torch.tensor([total_dev_s, wall], dtype=torch.float64)
        pg.all_reduce(tt, op=pg.ReduceOp.MAX)
        total_dev_s, wall = float(tt[0]), float(tt[1])
    nsh = len(shots) * ws
    value = nsh * steps / total_dev_s
    e2e = nsh * steps / wall
    h2d = sum(2 * d["ntr"] * nt * 4 for d in shots)
    d2h = 3 * w["allnx"] * w["allnz"] * 4 + 8 * len(shots) + (8 * w["allnx"] * w["allnz"] if w.get("rho_grad") else 0)

    # per-kernel average launch durations (CUDA events on the engine stream)
    kt = fd.time_kernels(reps=20)
    peak, peak_kind = measured_peak_hbm()
    cells = sum((d["nx"] + 2 * pml) * nzpml for d in shots)
    roof, fracs = None, None
    if kt:
        fracs = {k: round(kbytes[k] * cells / (v / 1000.0) / 1e9 / peak, 4) for k, v in kt.items()}
        dom = max(kt, key=kt.get)
        achieved = kbytes[dom] * cells / (kt[dom] / 1000.0) / 1e9
        tpc = traffic_per_cell(dom)
        roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": round(tpc * cells) if tpc else None,
                "traffic_note": "DRAM bytes per launch: ncu capture of a 16-shot launch scaled by cells",
                # the DRAM side of the same launch: measured bytes over the event time
                "dram_achieved": round(tpc * cells / (kt[dom] / 1000.0) / 1e9, 1) if tpc else None,
                "alg_bytes_per_launch": kbytes[dom] * cells, "peak_source": peak_kind,
                "launch_ms": round(kt[dom], 5), "all_kernels_ms": {k: round(v, 5) for k, v in kt.items()},
                "all_kernels_frac": fracs}
    pass_bytes = w.get("pass_bytes", PASS_BYTES_PER_CELL_STEP)
    kernel_bytes = sum(kbytes[k] for k in kt) if kt else None
    alg_bytes_step = pass_bytes * cells * nt

    # plain form: the same engine, one shot per run (the reference's per-shot
    # call pattern), device-timed on an evenly spread sample of the shots,
    # with the tile shape the autotuner picks for a one-shot batch
    plain = None
    if plain_shots > 0 and len(shots) > 1:
        pick = shots[:: max(1, len(shots) // plain_shots)][:plain_shots]
        plain_ms = []
        batch_tile = fd.tile_shape()
        plain_tile = None
        for j, d in enumerate(pick[:1] + pick):  # the first run warms the one-shot graph shape
            i = shots.index(d)
            enqueue(d, i)
            fd.run()
            if j == 0:
                plain_tile = fd.autotune(reps=5)[0] if args.tile == "auto" else batch_tile
                enqueue(d, i)
                fd.run()  # captures the graphs of the chosen shape
            else:
                plain_ms.append(fd.last_timing()["total_ms"])
        fd.imagebuffer_resettozero()
        fd.set_tile_shape(batch_tile)
        pv = len(pick) / (sum(plain_ms) / 1000.0)
        plain = {"value": round(pv, 3), "unit": "shot-gradients/s", "shots_sampled": len(pick), "tile": plain_tile,
                 "ms_per_shot": round(float(np.mean(plain_ms)), 2), "batched_over_plain": round(value / pv, 2)}
    # compressed snapshots against FP32 snapshots at full size, on a few shots
    snap_err = None
    if w.get("snap") and snap_check > 0:
        pick = shots[:: max(1, len(shots) // snap_check)][:snap_check]
        grads = {}
        for fmt in ("f32", "f16", "bf16"):
            fd.set_snapshots(w["snap"][0], fmt)
            for d in pick:
                enqueue(d, shots.index(d))
            fd.run()
            grads[fmt] = fd.read_gradients_f64()
            fd.imagebuffer_resettozero()
        fd.set_snapshots(*w["snap"])

        def rel(a, b):
            return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

        snap_err = {"shots": len(pick), "reference": "FP32 snapshots, same interval (the FP64-oracle errors are "
                                                      "measured by the parity tests)"}
        for fmt in ("f16", "bf16"):
            snap_err[fmt] = {k: float("%.3g" % rel(grads[fmt][j], grads["f32"][j]))
                             for j, k in enumerate(("grad_vp", "grad_vs", "illum"))}
    out.update(value=value, e2e=e2e, wall=wall, step_walls_ms=[round(1000.0 * x, 2) for x in step_walls], total_dev_s=total_dev_s, steps=steps, launches=launches, clk=clk,
               allreduce_ms=round(1000.0 * float(np.mean(allreduce_s)), 3) if allreduce_s else None,
               h2d=h2d, d2h=d2h, kt=kt, roof=roof, fracs=fracs, cells=cells, alg_bytes_step=alg_bytes_step,
               kernel_bytes=kernel_bytes, plain=plain, snap_err=snap_err, tile=fd.tile_shape(),
               phase_ms={"forward": round(float(np.mean(fwd_ms)), 2), "backward": round(float(np.mean(bwd_ms)), 2),
                         "misfit": round(float(np.mean(mis_ms)), 2)})
    return out


def close_workload(r):
    r["fd"].close()
    for pz, px in r["obs"]:
        pz.free()
        px.free()


def sub_record(w, r):
    """the short form of a workload's measurement, nested in the main line"""
    ms = 1000.0 * r["total_dev_s"] / r["steps"]
    rec = {"workload": w["name"], "shots": len(r["shots"]), "nt": w["nt"],
           "grid": "%dx%d+pml%d" % (w["allnx"], w["allnz"], w["pml"]), "dx_m": w["dx"], "stage": w.get("stage", 2),
           "misfit": w["misfit"], "value": round(r["value"], 3), "unit": "shot-gradients/s", "steps": r["steps"],
           "ms_per_step": round(ms, 3), "e2e": round(r["e2e"], 3), "tile": r["tile"],
           "alg_GBps_whole_step": round(r["alg_bytes_step"] / (ms / 1000.0) / 1e9, 1),
           "roofline": r["roof"] and {k: r["roof"][k] for k in ("kernel", "achieved", "peak", "frac", "launch_ms",
                                                                 "all_kernels_ms", "all_kernels_frac")},
           "plain": r["plain"]}
    if r.get("snap_err"):
        rec["snapshot_error"] = r["snap_err"]
    return rec


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fwi376", choices=sorted(WORKLOADS))
    ap.add_argument("--nt", type=int, default=None, help="override the number of time steps (testing)")
    ap.add_argument("--shots", type=int, default=None, help="override the number of shots (testing)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-shots", type=int, default=8, help="shots timed one at a time for the plain form")
    ap.add_argument("--serving-requests", type=int, default=12, help="requests of the serving-loop measurement")
    ap.add_argument("--serving-scaled", action="store_true",
                    help="serve the requests scaled to 0.3x grid and 0.1x nt (default: the drawn sizes, 200x100 to "
                         "2001x1001, nt 2000-6000)")
    ap.add_argument("--snap-check", type=int, default=4, help="shots of the compressed-vs-FP32 snapshot check")
    ap.add_argument("--profile-kernels", action="store_true", help="only run warm-up steps (for ncu captures)")
    ap.add_argument("--reference-gpu-shots", type=int, default=1,
                    help="shots of the reference's own CUDA path timed on this GPU (0: skip)")
    ap.add_argument("--profile-reference-gpu", action="store_true",
                    help="only run the reference's CUDA path on one shot of the workload (for ncu captures)")
    ap.add_argument("--tile", default="auto", help="tile shape of the step kernels: auto (autotuner) or a name in sfwi_gb300.TILE_SHAPES")
    ap.add_argument("--extra-workloads", default="salt401,shot376,snap2001",
                    help="workloads measured after the main one and reported as sub-records (comma list; '' for none)")
    ap.add_argument("--extra-steps", type=int, default=3, help="timed steps of each extra workload")
    ap.add_argument("--tile-order", type=int, default=None,
                    help="reverse-order bits of the four step kernels' tile draws (default: the engine's)")
    args = ap.parse_args()
    w = dict(WORKLOADS[args.workload])
    if args.nt:
        w["nt"] = args.nt
    if args.shots:
        w["nshots"] = args.shots
        w["spacing"] = max(1, min(w["spacing"], (w["allnx"] - 1) // max(1, args.shots)))
    if args.impl == "reference":
        return run_reference_arm(args, w)
    if args.profile_reference_gpu:
        r = reference_gpu_sample(w, build_workload(w), 1, warm=False)
        log("reference GPU: %s" % r)
        return 0 if "value" in r else 1

    ws, rank = dist_info()
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="gloo", init_method="env://")
        pg = dist

    r = measure(w, args, args.steps, args.warmup, args.plain_shots if ws == 1 else 0, pg=pg, ws=ws, rank=rank,
                clocks=Clocks(), snap_check=args.snap_check)
    if args.profile_kernels:
        close_workload(r)
        return 0
    data, shots = r["data"], r["shots"]
    nt, pml = w["nt"], w["pml"]
    ref_gpu = None
    if rank == 0 and args.reference_gpu_shots > 0 and not w.get("snap"):
        ref_gpu = reference_gpu_sample(w, data, args.reference_gpu_shots)
        if "value" in ref_gpu:
            ref_gpu["batched_over_reference_gpu"] = round(r["value"] / ref_gpu["value"], 1)
    close_workload(r)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, el = cpu_baseline_sample(w, data, 1, min(nt, 1000), "port")
        cpu = {"value": v, "unit": "shot-gradients/s", "cores": 1, "cpu_model": cpu_model(), "kind": "port",
               "sample": "one shot, %d of %d time steps (%.1f s), FP32 single-thread transliteration, scaled by nt"
                         % (min(nt, 1000), nt, el)}
    # the other benchmark workloads, short: batched, plain and per-kernel frac
    extras = {}
    if rank == 0 and not args.nt and not args.shots:
        for name in [x for x in args.extra_workloads.split(",") if x and x != args.workload]:
            we = dict(WORKLOADS[name])
            # the 2001x801 survey takes seconds a pass: two timed passes, and
            # its compressed snapshots checked against FP32 ones on two shots
            big = bool(we.get("snap"))
            re = measure(we, args, min(args.extra_steps, 2) if big else args.extra_steps, 2,
                         min(args.plain_shots, 4) if big else args.plain_shots, snap_check=2 if big else 0)
            extras[name] = sub_record(we, re)
            close_workload(re)
    serving = (run_serving(args.serving_requests, full=not args.serving_scaled)
               if args.serving_requests > 0 and rank == 0 else None)
    if rank != 0:
        return 0
    steps = args.steps
    total_dev_s = r["total_dev_s"]
    line = {"metric": METRIC, "value": round(r["value"], 3), "unit": "shot-gradients/s", "n_gpus": ws, "steps": steps,
            "warmup": args.warmup, "ms_per_step": round(1000.0 * total_dev_s / steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["name"], "shots": len(shots), "grid": "%dx%d+pml%d" % (w["allnx"], w["allnz"], pml),
                       "nt": nt, "misfit": w["misfit"], "born": w.get("stage", 2) == 2, "dx_m": w["dx"],
                       "source": "vertical force" if w.get("source") == "vz" else "txx+tzz",
                       "gradients": "vp, vs, rho" if w.get("rho_grad") else "vp, vs",
                       "tile": r["tile"], "autotune": r["tune"],
                       "imaging": ("%s snapshots every %d steps" % (w["snap"][1], w["snap"][0]) if w.get("snap")
                                   else "reconstruction with saved edge strips"),
                       "parallelism": ("shots split by cost over %d ranks, FP64 gradient all-reduce in every step"
                                       % ws if ws > 1 else "shots-per-gpu"),
                       "l2": l2_note(r["cells"], nt, len(shots), w),
                       "alg_bytes_per_step_GB": round(r["alg_bytes_step"] / 1e9, 2),
                       "alg_GBps_whole_step": round(r["alg_bytes_step"] / (total_dev_s / steps) / 1e9, 1),
                       "alg_GBps_whole_step_kernel_accounting": (
                           round(r["kernel_bytes"] * r["cells"] * nt / (total_dev_s / steps) / 1e9, 1)
                           if r["kernel_bytes"] else None)},
            "e2e": {"value": round(r["e2e"], 3), "unit": "shot-gradients/s", "wall_ms_per_step": r["step_walls_ms"],
                    "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"]},
            "gpu_launches": r["launches"], "roofline": r["roof"], "cpu_baseline": cpu, "clocks": r["clk"],
            "plain": r["plain"], "serving": serving, "snapshot_error": r["snap_err"], "reference_gpu": ref_gpu,
            "workloads": extras or None, "phase_ms": r["phase_ms"],
            "allreduce_ms": r["allreduce_ms"]}
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
