"""A stream of solve requests served with continuous batching (lbm_gpu_server).

The stream: Poisson arrivals; each request a channel, a cylinder or a liner
duct (uniform); grid Nx x Ny with aspect 4:1 and Nx * Ny log-uniform between
128 x 32 and 2048 x 512; steps log-uniform in [5000, 50000]; FP32-shifted or
FP64 storage with probability 0.8 / 0.2; all drawn from one seed. `scale`
shrinks every request's step count (same shape of the stream, shorter run).

Requests are submitted at their arrival times while the server's own thread
admits, batches and retires them. Reported: per-request latency (arrival to
result in host memory) p50/p99, and aggregate MLUPS over the makespan, next to
the time the same stream takes run one request at a time in plain FP64.
"""
from __future__ import annotations

import dataclasses
import math
import time
from typing import List

import numpy as np

from . import cases, impedance as imp
from .cases import BC, Case, equilibrium_state
from .runtime import F32_SHIFTED, F64, GpuServer, GpuSolver

TAU = 0.6  # all serving cases


@dataclasses.dataclass
class Req:
    kind: str
    nx: int
    ny: int
    steps: int
    storage: int
    arrival: float
    seed: int


def channel(nx: int, ny: int, u_max: float = 0.05):
    """Plane channel: solid top/bottom rows, regularized parabolic velocity
    inlet, regularized constant-pressure outlet."""
    mask = np.zeros((ny, nx), np.int32)
    mask[0, :] = 1
    mask[ny - 1, :] = 1
    H = ny - 2
    y = np.arange(ny, dtype=np.float64) - 0.5
    prof = 4.0 * u_max * y * (H - y) / (H * H)
    prof[0] = prof[-1] = 0.0
    bcs = [BC("velocity_inlet_regularized", 0, prof.copy(), np.zeros(ny)),
           BC("pressure_outlet_regularized", nx - 1, np.ones(ny), np.zeros(ny))]
    case = Case("channel", nx, ny, mask, np.full((ny, nx), 1.0 / TAU), np.zeros((ny, nx)), bcs)
    ux = np.repeat(prof[:, None], nx, axis=1)
    return case, equilibrium_state(np.ones((ny, nx)), ux, np.zeros((ny, nx)))


def build_request(r: Req):
    """(case, state, impedance spec or None) of one request."""
    if r.kind == "channel":
        case, st = channel(r.nx, r.ny)
        return case, st, None
    if r.kind == "cylinder":
        D = max(4.0, r.ny / 8.0)
        u_max = 0.05
        Re = u_max * D / ((TAU - 0.5) / 3.0)
        case, st = cases.cylinder_wake(r.nx, r.ny, D=D, xc=r.nx / 4.0, yc=r.ny / 2.0, u_max=u_max, Re=Re,
                                       seed=r.seed)
        return case, st, None
    rng = np.random.default_rng(r.seed)
    p = imp.LinerParams(r.nx, r.ny, float(rng.uniform(0.0, 0.3)), float(rng.uniform(0.5, 3.0)) * imp.CS,
                        float(rng.uniform(1e-3, 1e-2)), float(rng.uniform(0.02, 0.1)))
    case, st = imp.liner_duct(p)
    R, m, K = imp.liner_arrays(p)
    spec = (imp.LINER_ENTRY, R, m, K, imp.TRACKED_OMEGAS, 1.0, imp.MEAN_RATE, r.steps)
    return case, st, spec


def make_stream(n: int = 2000, seed: int = 2026, rate: float = 50.0, scale: float = 1.0,
                max_nodes: int = 2048 * 512, f64_storage: int = F64) -> List[Req]:
    """A seeded Poisson stream of channel / cylinder / liner requests. The 20 %
    of requests that ask for FP64 storage get f64_storage: F64 (lbc's
    arithmetic, bit for bit) or F64_FMA (the fused multiply-add step, lbc's
    results to rounding at 1.6-1.9x the speed)."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    lo, hi = math.log(128 * 32), math.log(min(2048 * 512, max_nodes))
    for q in range(n):
        t += float(rng.exponential(1.0 / rate))
        kind = ("channel", "cylinder", "liner")[int(rng.integers(0, 3))]
        nodes = math.exp(rng.uniform(lo, hi))
        ny = max(32, int(round(math.sqrt(nodes / 4.0))))
        nx = 4 * ny
        steps = int(round(math.exp(rng.uniform(math.log(5000), math.log(50000))) * scale))
        steps = max(steps, 2)
        storage = F32_SHIFTED if rng.uniform() < 0.8 else f64_storage
        out.append(Req(kind, nx, ny, steps, storage, t, seed * 100003 + q))
    return out


def serve(stream: List[Req], max_active: int = 64, chunk: int = 1000, budget_bytes: int = 0,
          prebuild: bool = True):
    """Submit each request at its arrival time to a running server; wait for
    all; return per-request latencies and totals. Every request starts from
    the equilibrium of its initial rho, u, v (formed by the server at
    admission). prebuild=False builds each request's case at its arrival
    instead of all of them up front (long streams: bounded host memory)."""
    built = [build_request(r) for r in stream] if prebuild else None
    srv = GpuServer(budget_bytes, max_active, chunk)
    srv.start()
    t0 = time.perf_counter()
    ids = []
    for q, r in enumerate(stream):
        if built is not None:
            case, st, spec = built[q]
        now = time.perf_counter() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        if built is None:
            case, st, spec = build_request(r)
        ids.append(srv.submit(case, st, r.steps, r.storage, impedance=spec, from_equilibrium=True))
        del case, st
    lat, done = {}, set()
    failed = []
    while len(done) < len(ids):
        for rid in ids:
            if rid in done:
                continue
            state, ts, ta, td = srv.status(rid)
            if state >= 3:
                done.add(rid)
                if state == 4:
                    failed.append(rid)
                lat[rid] = td - ts
                srv.release(rid)
        time.sleep(0.002)
    makespan = time.perf_counter() - t0
    srv.stop()
    stats = srv.stats()
    prof = srv.profile()
    srv.close()
    lups = sum(r.nx * r.ny * r.steps for r in stream)
    lats = np.array([lat[i] for i in ids])
    return {"requests": len(stream), "failed": len(failed), "lups": lups, "makespan_s": makespan,
            "mlups": lups / makespan / 1e6, "p50_s": float(np.percentile(lats, 50)),
            "p99_s": float(np.percentile(lats, 99)), "busy_s": stats["busy_s"],
            "phases": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in prof.items()},
            "latencies_s": lats.tolist()}


def serial_fp64_estimate(stream: List[Req], sample: int = 8, seed: int = 1):
    """Time to run the stream one request at a time in plain FP64, from timing
    a seeded sample of its requests (device time per LUP by request size)."""
    rng = np.random.default_rng(seed)
    idx = rng.choice(len(stream), size=min(sample, len(stream)), replace=False)
    t_sum, l_sum = 0.0, 0
    for q in idx:
        r = dataclasses.replace(stream[q], storage=F64, steps=min(stream[q].steps, 400))
        case, st, spec = build_request(r)
        s = GpuSolver(case, F64)
        if spec is not None:
            s.set_impedance_wall(spec[0], *spec[1:4], spec[4], spec[5], spec[6], spec[7])
        s.set_state(st)
        s.run(2)
        ms = s.run_timed(r.steps)
        t_sum += ms / 1e3
        l_sum += r.nx * r.ny * r.steps
        del s
    lups = sum(r.nx * r.ny * r.steps for r in stream)
    sec = t_sum / l_sum * lups  # ratio estimator: seconds per LUP of the sample
    return {"seconds": sec, "mlups": lups / sec / 1e6, "sampled": int(len(idx))}
