"""Benchmark of the GB300 split-operator step on the plain 2D workload.

Workload (the plain-method configuration the headline metric is quoted on): two
electrons in 1D each, a 2048 x 2048 grid with dx = 0.3, soft-core e-n charge 2 and
e-e softening 1 (Eberly model), absorber of 205 nodes per side, velocity gauge,
3-cycle sin^2 pulse at 800 nm and 5e14 W/cm^2, dt = 0.05, with the norm, the
potential energy and the seven ZOA_FLUX_2D border fluxes computed every step.
Data are synthetic: a normalised Gaussian start state on the host (seeded), no
datasets.

One "step" is one Strang step X(dt/2) P(dt) X(dt/2) of the whole grid plus its
observables.  `value` is grid-point-steps/s over K consecutive steps run as one call
with psi resident in HBM (CUDA events on the grid's stream around the call and around
every kernel of it; a step's working set -- psi and its static tables, 160 MiB --
exceeds L2, which is also flushed before the call); `e2e` is the same metric measured
through the C ABI with
host buffers: pinned host psi uploaded, K fused steps whose per-step coupling rows
come from host memory and whose observables rows come back to host memory, psi
downloaded -- all inside the host-timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank runs an independent replica of the workload on
its own GPU (a single solve does not shard without an all-to-all); `value` is the
sum over ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-pt-steps/s batched+served vs plain @1e-10 L2; HBM GB/s; p50/p99 solve"
UNIT = "grid-pt-steps/s"
N_EDGE, DX, NCAP = 2048, 0.3, 205
NCHARGE, ECHARGE, NSOFT, ESOFT = 2.0, -1.0, 1.0, 1.0
DT = 0.05
INTENSITY, WAVELENGTH, NCYCLES = 5e14, 800.0, 3.0
BYTES_PER_PT_STEP = 64  # algorithmic psi traffic of a 2D step: 2 passes x (16 B read + 16 B write)
BYTES_PER_PT_PASS = 32


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def _initial_psi(seed=0):
    """Seeded synthetic start state: a normalised Gaussian with small seeded noise."""
    rng = np.random.default_rng(seed)
    x = (np.arange(N_EDGE) - (N_EDGE - 1) / 2.0) * DX
    g = np.exp(-0.5 * x * x)
    psi = np.outer(g, g).astype(np.complex128)
    psi += 1e-6 * (rng.standard_normal(psi.shape) + 1j * rng.standard_normal(psi.shape))
    psi /= math.sqrt(float(np.sum(np.abs(psi) ** 2)) * DX * DX)
    return psi


def _pulse_args():
    import qsf_gb300 as Q
    return dict(field=Q.field_from_intensity(INTENSITY), omega=Q.omega_from_wavelength(WAVELENGTH), ncycles=NCYCLES)


class _Clocks:
    """nvidia-smi clock/throttle sampling during the timed region."""

    def __init__(self, index):
        self.path = tempfile.mktemp(suffix=".csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [t.strip() for t in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _ncu_traffic(kernel_kind):
    """dram bytes per launch of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"{kernel_kind}_2d2048.md")
    try:
        txt = open(path).read()
        m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", txt)
        return float(m.group(1)) if m else None
    except OSError:
        return None


# ------------------------------------------------------------------ CPU legs
def _oracle_sample(nsteps, barrier=None):
    """Time `nsteps` steps of the CPU oracle (C restatement) on the full workload; the
    grid, its tables and the start state are built before the timed region.  Returns
    (seconds, monotonic start, monotonic end)."""
    from oracle import oracle as O
    O.set_border_nodes(25, 14, 10, 40)
    pa = _pulse_args()
    c = O.Coupling(O.GAUGE_VELOCITY, [O.Field(3, [O.Pulse(**pa)])])
    g = O.Grid(2, N_EDGE, DX, nCAP=NCAP, Ncharge=NCHARGE, Echarge=ECHARGE, Nsoft=NSOFT, Esoft=ESOFT, coupling=c)
    g.psi[...] = _initial_psi()
    prop = O.Propagator(O.MODE_RE, DT, 0, g, ["norm", "epot", ("flux", O.ZOA_FLUX_2D, 0)])
    prop.make_step()  # untimed: first-touch of every table
    prop.compute_each()
    if barrier is not None:
        barrier.wait()
    t0 = time.monotonic()
    for _ in range(nsteps):
        prop.make_step()
        prop.compute_each()
    t1 = time.monotonic()
    return t1 - t0, t0, t1


_BARRIER = None


def _cpu_init(barrier):
    global _BARRIER
    _BARRIER = barrier


def _cpu_worker(nsteps):
    return _oracle_sample(nsteps, _BARRIER)


def cpu_baseline(all_cores: bool, budget_s: float = 20.0):
    """The oracle port timed on host cores over a bounded sample of the workload."""
    from oracle import oracle as O
    O.build()
    t1 = _oracle_sample(1)[0]
    nsteps = max(1, min(8, int(budget_s / max(t1, 1e-3))))
    m = N_EDGE * N_EDGE
    what = ("the reference's split step as the oracle restates it (oracle/qsf_oracle.c, gcc -O2, its own FP64 "
            "mixed-radix FFT in place of FFTW, which neither machine has)")
    if not all_cores:
        t = _oracle_sample(nsteps)[0]
        return {"value": m * nsteps / t, "unit": UNIT, "cores": 1, "kind": "port",
                "sample": f"{nsteps} Strang steps of the 2048^2 workload (norm, E_pot, 7 ZOA_FLUX_2D fluxes) "
                          f"on one core, after one untimed step; {what}"}
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(cores)
    with ctx.Pool(cores, initializer=_cpu_init, initargs=(barrier,)) as pool:
        res = pool.map(_cpu_worker, [nsteps] * cores)
    wall = max(r[2] for r in res) - min(r[1] for r in res)
    return {"value": m * nsteps * cores / wall, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{cores} independent single-core replicas x {nsteps} Strang steps of the 2048^2 workload, "
                      f"started together after their set-up; wall clock from the first replica's first timed "
                      f"step to the last one's end (process start, grid and table set-up excluded); {what}"}


# ------------------------------------------------------------------ batched / served
BATCH_EDGES = [256, 384, 512, 768, 1024]
SERVE_1D = (1024, 16384)  # 1D N uniform over the integers of this range (Bluestein lengths included)
SERVE_2D = [256, 320, 384, 512, 640, 768, 1024]  # 2D edges with fused kernels in 256..1024


def _gauss_state(dim, n, dx):
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    line = np.exp(-0.5 * x * x)
    psi = line
    for _ in range(dim - 1):
        psi = np.multiply.outer(psi, line)
    psi = psi.astype(np.complex128)
    return psi / math.sqrt(float(np.sum(np.abs(psi) ** 2)) * dx ** dim)


def _schedule(Q, dim, inten, lam, ncycles, nsteps):
    c = Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field({1: 1, 2: 3}[dim], [Q.Pulse(field=Q.field_from_intensity(inten),
                                                                          omega=Q.omega_from_wavelength(lam),
                                                                          ncycles=ncycles)])])
    from qsf_gb300.propagator import coupling_schedule
    return coupling_schedule(c, DT, nsteps)[0]


def batch_specs(nsolves=256, seed=0):
    """The batched workload's solve list: (edge, intensity W/cm^2, wavelength nm) per
    solve, edges uniform over {256..1024}, intensity log-uniform 1e14-1e15, wavelength
    uniform 400-1600 nm (numpy PCG64, seed 0)."""
    rng = np.random.default_rng(seed)
    edges = rng.choice(BATCH_EDGES, nsolves)
    inten = 10.0 ** rng.uniform(14.0, 15.0, nsolves)
    lam = rng.uniform(400.0, 1600.0, nsolves)
    return [(int(e), float(i), float(l)) for e, i, l in zip(edges, inten, lam)]


def batch_share(specs, steps, world_size, rank):
    """Indices of the solves this rank runs: shard.partition on grid points x steps
    (every rank computes the same split; no communication)."""
    from qsf_gb300 import shard
    return shard.my_share([shard.cost(e * e, steps) for e, _, _ in specs], world_size, rank)


def run_batched(steps, warmup, nsolves=256, seed=0, plain_arm=True, ws=1, rank=0):
    """256 independent 2-electron solves, edges uniform over {256..1024}, intensity
    log-uniform 1e14-1e15 W/cm^2, wavelength uniform 400-1600 nm, 3-cycle sin^2, VG,
    advanced together through qsf_batch; grid-point-steps/s over `steps` steps.  With
    several ranks each rank runs its share of the solve list (weak in the solves per
    GPU only through the split: the list is fixed) and `value` is the sum over ranks
    divided by the slowest rank's time."""
    import torch
    import qsf_gb300 as Q
    specs = batch_specs(nsolves, seed)
    mine = batch_share(specs, warmup + steps, ws, rank)
    edges = [specs[i][0] for i in mine]
    inten = [specs[i][1] for i in mine]
    lam = [specs[i][2] for i in mine]
    stream = torch.cuda.Stream()
    batch = Q.Batch(stream=stream.cuda_stream)
    grids, states = [], {}
    total = warmup + steps
    m_sum = 0
    for e, I, L in zip(edges, inten, lam):
        e = int(e)
        g = Q.Grid(2, e, DX, nCAP=e // 10, potential=Q.POT_EBERLY, Ncharge=NCHARGE, Echarge=ECHARGE, Nsoft=NSOFT,
                   Esoft=ESOFT, gauge=Q.GAUGE_VELOCITY, n_fields=1, stream=stream.cuda_stream)
        if e not in states:
            states[e] = _gauss_state(2, e, DX)
        g.upload(states[e])
        batch.add(g, Q.MODE_RE, DT, total, _schedule(Q, 2, I, L, NCYCLES, total), obs=Q.OBS_NORM | Q.OBS_EPOT,
                  borders=Q.ZOA_FLUX_2D)
        grids.append(g)
        m_sum += e * e
    batch.run(warmup)
    torch.cuda.synchronize()
    _barrier(ws)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    batch.run(steps)
    b.record(stream)
    torch.cuda.synchronize()
    ms = _max_over_ranks(ws, a.elapsed_time(b))
    batch.close()
    m_all = _sum_over_ranks(ws, float(m_sum))
    out = {"value": m_all * steps / (ms / 1e3), "unit": UNIT, "solves": nsolves, "steps": steps,
           "ms_per_step": ms / steps, "grid_points": int(m_all), "solves_this_rank": len(mine),
           "workload": "batched: 256 2D solves, edges U{256,384,512,768,1024}, I log-U[1e14,1e15], "
                       "lambda U[400,1600] nm, 3-cycle sin^2 VG, norm+E_pot+ZOA_FLUX_2D every step, seed 0"}
    if plain_arm:
        # the same solves one after another through the plain single-solve path (qsf_step,
        # one call of `steps` steps per solve, graph-replayed), after one untimed call of
        # `warmup` steps per solve; all grids share one stream, timed with CUDA events
        for g, e, I, L in zip(grids, edges, inten, lam):
            g.upload(states[int(e)])
        scheds = [_schedule(Q, 2, I, L, NCYCLES, total) for I, L in zip(inten, lam)]
        for g, sc in zip(grids, scheds):
            g.step(Q.MODE_RE, DT, warmup, sc[:warmup], obs=Q.OBS_NORM | Q.OBS_EPOT, borders=Q.ZOA_FLUX_2D)
        torch.cuda.synchronize()
        _barrier(ws)
        a.record(stream)
        for g, sc in zip(grids, scheds):
            g.step(Q.MODE_RE, DT, steps, sc[warmup:], obs=Q.OBS_NORM | Q.OBS_EPOT, borders=Q.ZOA_FLUX_2D)
        b.record(stream)
        torch.cuda.synchronize()
        pms = _max_over_ranks(ws, a.elapsed_time(b))
        out["plain_same_solves"] = {
            "value": m_all * steps / (pms / 1e3), "unit": UNIT, "ms_per_step_all_solves": pms / steps,
            "method": "each of the 256 solves alone through qsf_step (one call of the timed steps per solve), "
                      "one after another on one stream"}
        out["batched_vs_plain_same_solves"] = out["value"] / out["plain_same_solves"]["value"]
    for g in grids:
        g.close()
    return out


def _plain_sample_rate(Q, reqs):
    """The plain path on a sample of the served requests: each solve alone through
    qsf_step (grids made beforehand, one step call per solve, one after another on one
    stream), grid-point-steps over the summed device time."""
    import torch
    stream = torch.cuda.Stream()
    grids = []
    for dim, n, dx, coupling, psi0, borders, box, nsteps in reqs:
        g = Q.Grid(dim, n, dx, nCAP=n // 10, Ncharge=float(dim), gauge=Q.GAUGE_VELOCITY, n_fields=1,
                   stream=stream.cuda_stream)
        g.upload(psi0)
        grids.append(g)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pts = 0.0
    a.record(stream)
    for g, (dim, n, dx, coupling, psi0, borders, box, nsteps) in zip(grids, reqs):
        g.step(Q.MODE_RE, DT, nsteps, coupling, obs=Q.OBS_NORM | Q.OBS_EPOT, borders=borders, box_size=box)
        pts += float(n ** dim) * nsteps
    b.record(stream)
    torch.cuda.synchronize()
    for g in grids:
        g.close()
    return pts / (a.elapsed_time(b) / 1e3)


def run_served(rate, duration_s, steps_per_solve=256, seed=0, max_slots=128, steps_per_round=16, ws=1, rank=0,
               plain_sample=0):
    """Poisson arrivals at `rate`/s for `duration_s`: 50/50 1D (N uniform over 1024..16384)
    and 2D (edge in 256..1024 with fused kernels) solves with seeded pulses; each solve runs its first
    `steps_per_solve` steps.  Returns throughput and p50/p99 submit->completion.  With
    several ranks every rank follows the same seeded stream and serves the requests
    shard.StreamAssigner gives it (serve.ShardedServer).  With plain_sample = k the first k
    requests also run one by one through qsf_step after the served run, and the line
    reports that plain rate and the served value over it."""
    import qsf_gb300 as Q
    from qsf_gb300 import serve as S
    rng = np.random.default_rng(seed)
    sample = []
    srv = S.ShardedServer(rank, ws, max_slots=max_slots, hbm_reserve_gb=16.0, steps_per_round=steps_per_round)
    tickets, pts = [], 0.0
    t0 = time.perf_counter()
    t_next = t0
    states = {}
    while True:
        now = time.perf_counter()
        if now - t0 >= duration_s:
            break
        if now < t_next:
            time.sleep(min(t_next - now, 0.01))
            continue
        t_next += rng.exponential(1.0 / rate)
        dim = 1 if rng.random() < 0.5 else 2
        n = int(rng.integers(SERVE_1D[0], SERVE_1D[1] + 1)) if dim == 1 else int(rng.choice(SERVE_2D))
        dx = 0.2 if dim == 1 else DX
        inten = 10.0 ** rng.uniform(14.0, 15.0)
        lam = rng.uniform(400.0, 1600.0)
        gd = S.grid_desc(dim, n, dx, nCAP=n // 10, Ncharge=float(dim), gauge=Q.GAUGE_VELOCITY, n_fields=1)
        key = (dim, n)
        if key not in states:
            states[key] = _gauss_state(dim, n, dx)
        borders = ["BOX"] if dim == 1 else Q.ZOA_FLUX_2D
        box = int(0.4 * n) if dim == 1 else 0
        sched = _schedule(Q, dim, inten, lam, NCYCLES, steps_per_solve)
        t = srv.submit(gd, Q.MODE_RE, DT, steps_per_solve, coupling=sched, psi0=states[key],
                       obs=Q.OBS_NORM | Q.OBS_EPOT, borders=borders, box_size=box)
        if len(sample) < plain_sample:
            sample.append((dim, n, dx, sched, states[key], borders, box, steps_per_solve))
        if t is not None:
            tickets.append((t, float(n ** dim) * steps_per_solve))
    lat, statuses = [], {}
    for t, tp in tickets:  # grid-point-steps of the solves that completed
        r = srv.wait(t, 3600)
        statuses[r["status"]] = statuses.get(r["status"], 0) + 1
        if r["status"] == 0:
            lat.append(r["latency_s"])
            pts += tp
    wall = _max_over_ranks(ws, time.perf_counter() - t0)
    srv.stop()
    pts = _sum_over_ranks(ws, pts)
    if ws > 1:  # latencies of every rank's solves
        import torch.distributed as dist
        allv = [None] * ws
        dist.all_gather_object(allv, lat)
        lat = [v for part in allv for v in part]
    lat.sort()
    pct = lambda q: lat[min(len(lat) - 1, int(q * len(lat)))] if lat else None
    extra = {}
    if sample and rank == 0:
        plain = _plain_sample_rate(Q, sample)
        extra = {"plain_same_solves_sample": {"value": plain, "unit": UNIT, "solves": len(sample),
                                              "method": "the first requests of the stream, each alone through "
                                                        "qsf_step, one after another on one stream"},
                 "served_vs_plain_same_solves": pts / wall / plain}
    return {"rate_per_s": rate, "submitted": _sum_over_ranks(ws, len(tickets)), "completed": len(lat), **extra,
            "statuses": {str(k): v for k, v in sorted(statuses.items())},
            "value": pts / wall, "unit": UNIT,
            "p50_s": pct(0.50), "p99_s": pct(0.99), "wall_s": wall,
            "workload": f"served: Poisson {rate}/s for {duration_s}s, 50/50 1D N uniform over the integers "
                        f"1024..16384 (lengths outside the fused-kernel list through Bluestein transforms and "
                        f"member operations) / 2D edge in {SERVE_2D}, I log-U[1e14,1e15], lambda U[400,1600] nm, "
                        f"{steps_per_solve} steps per solve, seed {seed}"}


# ------------------------------------------------------------------ GPU arm
MG_EDGE, MG_NCAP = 1024, 102


def _mg_oracle_rate(n: int, nsteps: int) -> float:
    """Grid-pt-steps/s of the oracle's multi-region propagator (one core), n^2 regions."""
    from oracle import oracle as O
    pa = _pulse_args()
    regs = O.region_axes(2)
    cs = [O.Coupling(O.GAUGE_VELOCITY, [O.Field(3, [O.Pulse(**pa)])]) for _ in regs]
    gs = [O.Grid(2, n, DX, nCAP=max(1, n // 10), Ncharge=NCHARGE, Echarge=ECHARGE, Nsoft=NSOFT, Esoft=ESOFT,
                 coupling=c) for c in cs]
    gs[0].psi[...] = _gauss_state(2, n, DX)
    mp = O.MultiRegionPropagator(DT, gs, cs, ["norm", "epot"])
    t0 = time.perf_counter()
    for _ in range(nsteps):
        mp._step_all()
        mp.props[0].compute_each()
        mp.post_compute()
    return len(regs) * n * n * nsteps / (time.perf_counter() - t0)


def run_multigrid(steps, warmup, cpu=True, dim=2):
    """Multi-region grid: 2D regions NO, X, Y, XY of 1024^2 each (the C2 pulse), or 3D
    regions NO ... XYZ of 256^3 each (three electrons, e-n charge 3, 2-cycle 800 nm 1e15
    W/cm^2; velocity gauge, the gauge the reference's multi-region grids support): one
    step = the Strang step of every region, norm and E_pot of the main region, the region
    transfers and the region masks.  Timed on the host around `steps` steps with every
    region's stream synchronised at both ends (each region runs on its own stream)."""
    import qsf_gb300 as Q
    from qsf_gb300.multigrid import MultiGrid, MultiRegionPropagator
    if dim == 2:
        edge, ncap, dx, charge, axis, pa = MG_EDGE, MG_NCAP, DX, NCHARGE, 3, _pulse_args()
    else:
        edge, ncap, dx, charge, axis = 256, 26, 0.4, 3.0, 7
        pa = dict(field=Q.field_from_intensity(1e15), omega=Q.omega_from_wavelength(800.0), ncycles=2.0)
    mg = MultiGrid(dim, edge, dx, ncap, potential=Q.POT_EBERLY, Ncharge=charge, Echarge=ECHARGE, Nsoft=NSOFT,
                   Esoft=ESOFT, gauge=Q.GAUGE_VELOCITY, n_fields=1)
    mg.main.upload(_gauss_state(dim, edge, dx))
    prop = MultiRegionPropagator(DT, mg, Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field(axis, [Q.Pulse(**pa)])]),
                                 ["norm", "epot"])

    def one():
        prop._make_step()
        prop._compute_each()
        mg.post_compute()

    for _ in range(warmup):
        one()
    mg.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    mg.synchronize()
    wall = time.perf_counter() - t0
    nreg = 2 ** dim
    pts = float(nreg) * edge ** dim * steps
    out = {"value": pts / wall, "unit": UNIT, "ms_per_step": wall * 1e3 / steps, "steps": steps,
           "config": f"{dim}D multi-region grid, {nreg} regions x {edge}^{dim}, nCAP {ncap}, VG sin^2 pulse, "
                     f"norm + E_pot of the main region every step, transfers + masks every step"}
    if cpu and dim == 2:
        n_cpu = 256
        out["cpu_baseline"] = {"value": _mg_oracle_rate(n_cpu, 4), "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"4 steps of the same multi-region propagator on 4 x {n_cpu}^2 regions "
                                         f"(oracle, one core)"}
    mg.close()
    return out


def _timed_steps(Q, grid, stream, mode, dt, steps, warmup, sched, obs, borders, box, flush):
    """One warm-up call, then one call of `steps` graph-replayed steps timed with CUDA
    events on the grid's stream (L2 flushed before it); then a profiled call of the
    same steps for the per-kernel split.  Returns (ms per step, {kind: (ms, launches)})."""
    import torch
    grid.step(mode, dt, warmup, sched[:warmup], obs=obs, borders=borders, box_size=box)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        flush.zero_()
        e0.record(stream)
        grid.step(mode, dt, steps, sched[warmup:warmup + steps], obs=obs, borders=borders, box_size=box)
        e1.record(stream)
    torch.cuda.synchronize()
    prof = {}
    with torch.cuda.stream(stream):
        flush.zero_()
        grid.step(mode, dt, steps, sched[warmup:warmup + steps], obs=obs, borders=borders, box_size=box,
                  profile=prof)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, {k: v for k, v in prof.items() if v[1] > 0}


def _roofline(bytes_per_pt_step, m, steps, prof, note):
    peak, peak_kind = _peaks()
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms = prof[dom][0] / prof[dom][1]
    # bytes per launch of the dominant kernel: one pass over psi (32 B per point), or the
    # whole step's psi traffic for a one-kernel 1D step
    per_launch = (32 if bytes_per_pt_step > 32 else bytes_per_pt_step) * m
    ach = per_launch / (dom_ms / 1e3) / 1e9
    return {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
            "traffic": None, "peak_source": f"{peak_kind} hbm_gbs", "algorithmic_bytes_per_launch": per_launch,
            "avg_launch_ms": dom_ms, "note": note}


def run_c1(steps, warmup, flush):
    """The 1D plain configuration: 4096 points, dx 0.2, soft-core H, length gauge,
    2-cycle 800 nm 1e14 W/cm^2 pulse, cos^(1/8) mask on the outer 10%, norm + E_pot +
    BOX flux every step.  Step timing of the real-time propagation, plus the wall time
    of the whole job as a user runs it (2000 imaginary-time steps with Normalize, then
    the full real-time run) through SplitPropagator."""
    import torch
    import qsf_gb300 as Q
    n, dx, ncap, box = 4096, 0.2, 410, 1638
    stream = torch.cuda.Stream()
    common = dict(nCAP=ncap, potential=Q.POT_EBERLY, Ncharge=1.0, Echarge=-1.0, Nsoft=1.0, absorber=Q.ABS_COS8,
                  mask_dt=DT, stream=stream.cuda_stream)
    pulse = dict(field=Q.field_from_intensity(1e14), omega=Q.omega_from_wavelength(800.0), ncycles=2.0)
    t0 = time.perf_counter()
    gi = Q.Grid(1, n, dx, gauge=Q.GAUGE_VELOCITY, n_fields=0, **common)
    gi.add_gaussian(0.0, 1.0)
    Q.SplitPropagator(Q.MODE_IM, 0.01, 2000, gi, Q.Coupling(Q.GAUGE_VELOCITY),
                      ["step", "norm", "normalize", "epot", "ekin", "etot", "ediff"]).run()
    psi0 = gi.download()
    gr = Q.Grid(1, n, dx, gauge=Q.GAUGE_LENGTH, n_fields=1, **common)
    gr.upload(psi0)
    c = Q.Coupling(Q.GAUGE_LENGTH, [Q.Field(1, [Q.Pulse(**pulse)])])
    prop = Q.SplitPropagator(Q.MODE_RE, DT, 0, gr, c, ["step", "time", "norm", "epot", ("flux", ["BOX"], box)])
    rows = prop.run()
    torch.cuda.synchronize()
    job_s = time.perf_counter() - t0
    gr.upload(psi0)
    from qsf_gb300.propagator import coupling_schedule
    sched, _ = coupling_schedule(Q.Coupling(Q.GAUGE_LENGTH, [Q.Field(1, [Q.Pulse(**pulse)])]), DT, warmup + steps)
    ms, prof = _timed_steps(Q, gr, stream, Q.MODE_RE, DT, steps, warmup, sched, Q.OBS_NORM | Q.OBS_EPOT, ["BOX"],
                            box, flush)
    value = n * 1000.0 / ms
    return {"value": value, "unit": UNIT, "ms_per_step": ms, "steps": steps,
            "roofline": _roofline(32, n, steps, prof, "1D: the line is held on chip for the whole step (one "
                                  "pass, 32 B per point-step); latency-bound on one SM, not HBM-bound"),
            "kernels_ms_per_step": {k: v[0] / steps for k, v in prof.items()},
            "job_s": job_s, "job_steps": 2000 + len(rows) - 1,
            "yield_1_minus_norm": 1.0 - rows[-1]["norm"],
            "workload": "1D plain: 4096 points, dx 0.2, soft-core H (e-n charge 1, eps 1), IM ground state "
                        "(dt 0.01, 2000 steps) then RE dt 0.05, LG 2-cycle sin^2 800 nm 1e14 W/cm^2, cos^(1/8) "
                        "mask on the outer 10%, norm + E_pot + BOX flux every step"}


def run_c4(steps, warmup, flush):
    """The 3D plain configuration: 256^3, dx 0.4, three electrons (e-n charge 3, all
    e-e pairs), length gauge, 2-cycle 800 nm 1e15 W/cm^2, CAP over 26 nodes, norm +
    E_pot + the eight ZOA_FLUX_3D fluxes every step."""
    import torch
    import qsf_gb300 as Q
    n, dx, ncap = 256, 0.4, 26
    stream = torch.cuda.Stream()
    g = Q.Grid(3, n, dx, nCAP=ncap, potential=Q.POT_EBERLY, Ncharge=3.0, gauge=Q.GAUGE_LENGTH, n_fields=1,
               stream=stream.cuda_stream)
    g.upload(_gauss_state(3, n, dx))
    c = Q.Coupling(Q.GAUGE_LENGTH, [Q.Field(7, [Q.Pulse(field=Q.field_from_intensity(1e15),
                                                        omega=Q.omega_from_wavelength(800.0), ncycles=2.0)])])
    prop = Q.SplitPropagator(Q.MODE_RE, DT, 0, g, c, ["norm", "epot", ("flux", Q.ZOA_FLUX_3D, 0)])
    sched = prop._schedule(warmup + steps)
    ms, prof = _timed_steps(Q, g, stream, Q.MODE_RE, DT, steps, warmup, sched, Q.OBS_NORM | Q.OBS_EPOT,
                            Q.ZOA_FLUX_3D, 0, flush)
    m = n ** 3
    g.close()
    return {"value": m * 1000.0 / ms, "unit": UNIT, "ms_per_step": ms, "steps": steps,
            "roofline": _roofline(128, m, steps, prof, "3D: 4 passes over psi per step (128 B per point-step)"),
            "hbm_gbs_step": 128 * m * 1000.0 / ms / 1e9,
            "kernels_ms_per_step": {k: v[0] / steps for k, v in prof.items()},
            "workload": "3D plain: 256^3, dx 0.4, 3 electrons (e-n charge 3, all e-e pairs), LG 2-cycle sin^2 "
                        "800 nm 1e15 W/cm^2, CAP 26 nodes, norm + E_pot + ZOA_FLUX_3D every step"}


def run_ekin(steps, flush):
    """Imaginary-time steps with the kinetic energy as an output: every step (the
    reference's computeEach), every 10th step (ekin_interval = 10, the steps between
    fused) and never, on the 2D 2048^2 grid and the 1D 4096-point line (where the
    line kernel computes it in place at no extra launch)."""
    import torch
    import qsf_gb300 as Q
    out = {}
    for name, dim, n, dx, ncap in (("2d2048", 2, N_EDGE, DX, NCAP), ("1d4096", 1, 4096, 0.2, 410)):
        stream = torch.cuda.Stream()
        g = Q.Grid(dim, n, dx, nCAP=ncap, potential=Q.POT_EBERLY, Ncharge=float(dim), gauge=Q.GAUGE_VELOCITY,
                   n_fields=0, stream=stream.cuda_stream)
        psi = _gauss_state(dim, n, dx)
        row = {}
        for label, obs, k in (("ekin_every_step", Q.OBS_NORM | Q.OBS_EPOT | Q.OBS_EKIN, 1),
                              ("ekin_every_10", Q.OBS_NORM | Q.OBS_EPOT | Q.OBS_EKIN, 10),
                              ("no_ekin", Q.OBS_NORM | Q.OBS_EPOT, 1)):
            g.upload(psi)
            g.step(Q.MODE_IM, 0.01, 10, None, obs=obs, normalize=True, ekin_interval=k)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                flush.zero_()
                e0.record(stream)
                g.step(Q.MODE_IM, 0.01, steps, None, obs=obs, normalize=True, ekin_interval=k)
                e1.record(stream)
            torch.cuda.synchronize()
            row[label + "_ms_per_step"] = e0.elapsed_time(e1) / steps
        g.close()
        out[name] = row
    out["workload"] = ("imaginary time dt 0.01 with Normalize every step, norm + E_pot (+ E_kin) rows; "
                       f"{steps} steps per timed call")
    return out


def run_gpu(args):
    ws, rank, local = _dist()
    import torch
    torch.cuda.set_device(local)
    import qsf_gb300 as Q

    stream = torch.cuda.Stream()
    pa = _pulse_args()
    coupling = Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field(3, [Q.Pulse(**pa)])])
    grid = Q.Grid(2, N_EDGE, DX, nCAP=NCAP, potential=Q.POT_EBERLY, Ncharge=NCHARGE, Echarge=ECHARGE, Nsoft=NSOFT,
                  Esoft=ESOFT, gauge=Q.GAUGE_VELOCITY, n_fields=1, stream=stream.cuda_stream)
    psi0 = _initial_psi(seed=rank)
    grid.upload(psi0)
    outputs = ["norm", "epot", ("flux", Q.ZOA_FLUX_2D, 0)]
    prop = Q.SplitPropagator(Q.MODE_RE, DT, 0, grid, coupling, outputs)
    m = grid.m
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def run_steps(nsteps, profile=None):
        sched = prop._schedule(nsteps)
        rows, _ = grid.step(Q.MODE_RE, DT, nsteps, sched, obs=Q.OBS_NORM | Q.OBS_EPOT, borders=Q.ZOA_FLUX_2D,
                            profile=profile)
        return rows

    # warm-up: W steps as in the timed call (one call, the fused multi-step path)
    run_steps(args.warmup)
    _barrier(ws)
    torch.cuda.synchronize()
    clocks = _Clocks(local)
    # timed: K consecutive steps in one call (the graph-replayed path a user gets), CUDA
    # events on the grid's stream around the call.  A step's working set (psi 64 MiB,
    # static X table 64 MiB, potential 32 MiB) exceeds the 129 MB L2; L2 is also flushed
    # before the timed call.
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        flush.zero_()
        ev0.record(stream)
        run_steps(args.steps)
        ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = _max_over_ranks(ws, float(ev0.elapsed_time(ev1)))
    # the per-kernel split (and the dominant kernel's launch time for the roofline): a
    # second call of K steps with every launch bracketed by CUDA events
    profile = {}
    with torch.cuda.stream(stream):
        flush.zero_()
        run_steps(args.steps, profile)
    torch.cuda.synchronize()
    _barrier(ws)
    pts = _sum_over_ranks(ws, float(m) * args.steps)
    value = pts / (total_ms / 1e3)

    # e2e through the C ABI with host buffers (pinned psi, coupling rows from host)
    pinned = torch.empty((m * 2,), dtype=torch.float64, pin_memory=True)
    host_psi = pinned.numpy().view(np.complex128).reshape(grid.shape)
    host_psi[...] = psi0
    e2e_prop = Q.SplitPropagator(Q.MODE_RE, DT, 0, grid, Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field(3, [Q.Pulse(**pa)])]),
                                 outputs)
    sched = e2e_prop._schedule(args.steps)
    _barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    grid.upload(host_psi)
    rows, done = grid.step(Q.MODE_RE, DT, args.steps, sched, obs=Q.OBS_NORM | Q.OBS_EPOT, borders=Q.ZOA_FLUX_2D)
    grid.download(out=host_psi)
    e2e_s = _max_over_ranks(ws, time.perf_counter() - t0)
    e2e_value = _sum_over_ranks(ws, float(m) * args.steps) / e2e_s
    ncol = rows.shape[1]

    # roofline of the dominant kernel
    kinds = {k: v for k, v in profile.items() if v[1] > 0}
    dom = max(kinds, key=lambda k: kinds[k][0])
    dom_ms = kinds[dom][0] / kinds[dom][1]
    peak, peak_kind = _peaks()
    achieved = BYTES_PER_PT_PASS * m / (dom_ms / 1e3) / 1e9
    traffic = _ncu_traffic(dom)
    # launches of the timed call: the profiled call launches every kernel every step; the
    # graph-replayed call runs the opening row pass (work only in a fused call's first
    # step) once
    launches = sum(v[1] for v in kinds.values()) - max(0, kinds.get("row_open", (0.0, 1))[1] - 1)

    batched = run_batched(steps=20, warmup=3, ws=ws, rank=rank)
    served = [run_served(rate=r, duration_s=2.0, ws=ws, rank=rank, plain_sample=100 if r >= 1000.0 else 0)
              for r in (10.0, 100.0, 1000.0)]
    multigrid = run_multigrid(steps=20, warmup=3, cpu=rank == 0)
    multigrid_3d = run_multigrid(steps=5, warmup=2, cpu=False, dim=3)
    c1 = run_c1(steps=max(args.steps, 200), warmup=args.warmup, flush=flush)
    c4 = run_c4(steps=max(args.steps, 10), warmup=args.warmup, flush=flush)
    ekin = run_ekin(steps=max(args.steps, 40), flush=flush)

    if rank == 0:
        cpu = cpu_baseline(all_cores=False)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128/f64", "data": "synthetic (seeded Gaussian start state, sin^2 pulse)",
            "config": plain_config(ws),
            "l2_flush": "a buffer larger than L2 is written before the timed call",
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": (16 * m + 24 * args.steps) / args.steps,
                    "d2h_bytes_per_step": (16 * m + 8 * ncol * args.steps) / args.steps},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": f"{peak_kind} hbm_gbs",
                         "algorithmic_bytes_per_launch": BYTES_PER_PT_PASS * m,
                         "avg_launch_ms": dom_ms},
            "kernels_ms_per_step": {k: v[0] / args.steps for k, v in kinds.items()},
            "hbm_gbs_step": BYTES_PER_PT_STEP * value / ws / 1e9,
            "cpu_baseline": cpu,
            "clocks": clk,
            "batched": batched,
            "served": served,
            "multigrid": multigrid,
            "c4_multi_region": multigrid_3d,
            "c1": c1,
            "c4": c4,
            "ekin": ekin,
            "batched_vs_plain": batched["value"] / value,
            "batched_vs_plain_same_solves": batched.get("batched_vs_plain_same_solves"),
        }
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def plain_config(ws: int) -> dict:
    """The plain workload's config, the same in both arms: one 2048^2 solve per GPU (the
    reference arm times the same grid and step on the host cores)."""
    return {"workload": "plain 2D split step, 2 electrons (1D each), 2048x2048, dx=0.3, dt=0.05, "
                        "VG 800 nm 5e14 W/cm^2 3-cycle sin^2, absorber 205 nodes, norm+E_pot+ZOA_FLUX_2D every step",
            "grid": [N_EDGE, N_EDGE], "parallelism": f"replicas x{ws}",
            "l2": "working set per step > L2 (psi + static tables 160 MiB)"}


def run_reference(args):
    """The reference arm: the reference algorithm's CPU implementation (oracle port,
    the reference's own build needs MPI/FFTW and the reference checkout) on all host
    cores, same workload, metric and unit."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    t0 = time.perf_counter()
    samples = []
    for _ in range(max(1, args.steps // 10)):
        samples.append(cpu_baseline(all_cores=True, budget_s=10.0))
    v = statistics.median(s["value"] for s in samples)
    cb = dict(samples[0])
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128/f64", "data": "synthetic (seeded Gaussian start state, sin^2 pulse)",
            "config": plain_config(ws),
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="plain", choices=["plain", "batched", "served", "multigrid"])
    ap.add_argument("--rates", default="10,30,100,300,1000")
    ap.add_argument("--duration", type=float, default=5.0)
    ap.add_argument("--mg-dim", type=int, default=2, choices=[2, 3], help="multigrid workload: 2D 1024^2 or 3D 256^3")
    ap.add_argument("--plain-sample", type=int, default=0,
                    help="served workload: also run the first K requests one by one through qsf_step")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"metric": METRIC, **run_batched(args.steps, args.warmup)}))
    elif args.workload == "served":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        for r in [float(v) for v in args.rates.split(",")]:
            print(json.dumps({"metric": METRIC, **run_served(r, args.duration, plain_sample=args.plain_sample)}),
                  flush=True)
    elif args.workload == "multigrid":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"metric": METRIC, **run_multigrid(args.steps, args.warmup, dim=args.mg_dim)}), flush=True)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
