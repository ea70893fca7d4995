"""Acoustic liner ducts with a time-domain impedance wall, and impedance eduction.

A duct is a 2D channel with a uniform grazing flow: regularized velocity inlet,
regularized constant-pressure outlet, solid top wall, and a bottom wall whose
middle section (the liner) is a row of impedance-wall nodes (a
velocity_bottom_regularized Boundary entry with a per-node mass-spring-damper
attached, include/lbm_gpu.h). A Gaussian acoustic pulse starts near the inlet.

lbc drives one impedance model from the outlet-averaged pressure on the host
every step (cases/nit/nit.c:276-303) and educes the impedance offline with an
external toolkit (cases/nit/process.py:22-27). Here every liner node carries its
own model on the device and keeps running, Hann-windowed DFTs of its pressure
and velocity (the window suppresses the end-of-run state of the slow spring
mode, which an unweighted finite sum would fold into every bin), so the
impedance is educed per node as Z(w) = P(w) / V(w), with P the DFT of the
pressure p'_n the wall sees at step n and V the DFT of the velocity v_{n+1} it
imposes in response (the pair the lattice sees at the same step), and compared
with the imposed model Z = R + i (w m - K / w). The difference is the time
discretisation of the model, O(w^2) for the step-held update.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List

import numpy as np

from .cases import BC, Case, equilibrium_state

CS = 1.0 / math.sqrt(3.0)


@dataclasses.dataclass
class LinerParams:
    nx: int
    ny: int
    mach: float
    R: float          # resistance (lattice units, rho c = 1/sqrt(3) at rho = 1)
    m: float          # mass reactance coefficient
    f_res: float      # resonance frequency (cycles / step)
    liner_frac: float = 0.4
    tau: float = 0.6
    pulse_amp: float = 1e-3
    pulse_width: float = 8.0

    @property
    def K(self) -> float:
        return self.m * (2.0 * math.pi * self.f_res) ** 2

    @property
    def liner_span(self):
        i0 = int(round(self.nx * (0.5 - self.liner_frac / 2)))
        i1 = int(round(self.nx * (0.5 + self.liner_frac / 2)))
        return i0, i1


LINER_ENTRY = 2   # position of the liner in the Boundary list below
# Rate of the running mean density the wall's pressure fluctuation is taken
# about: the mean-flow static pressure (tens of times the acoustic pulse at
# Mach 0.3) would otherwise load the springs.
MEAN_RATE = 1e-3
EDUCTION_OMEGAS = np.array([0.05, 0.1, 0.15, 0.2])
# Frequencies tracked on the device: a zero bin first (the running sums used to
# remove the mean of p' and v before eduction), then the eduction frequencies.
TRACKED_OMEGAS = np.concatenate([[0.0], EDUCTION_OMEGAS])


def liner_duct(p: LinerParams):
    """(case, state) for one duct. Row 0 is the bottom wall (liner nodes fluid,
    the rest solid), row ny-1 the solid top wall."""
    nx, ny = p.nx, p.ny
    u0 = p.mach * CS
    mask = np.zeros((ny, nx), dtype=np.int32)
    mask[ny - 1, :] = 1
    mask[0, :] = 1
    i0, i1 = p.liner_span
    mask[0, i0:i1] = 0
    bcs = [BC("velocity_inlet_regularized", 0, np.full(ny, u0), np.zeros(ny)),
           BC("pressure_outlet_regularized", nx - 1, np.ones(ny), np.zeros(ny)),
           BC("velocity_bottom_regularized", 0, np.zeros(nx), np.zeros(nx))]
    case = Case("liner_duct", nx, ny, mask, np.full((ny, nx), 1.0 / p.tau), np.zeros((ny, nx)), bcs)
    x = np.arange(nx, dtype=np.float64)[None, :]
    x0 = 3.0 * p.pulse_width + 2.0
    drho = p.pulse_amp * np.exp(-((x - x0) ** 2) / (2.0 * p.pulse_width ** 2)) * np.ones((ny, 1))
    rho = 1.0 + drho
    ux = u0 + CS * drho           # right-running acoustic pulse on the mean flow
    uy = np.zeros((ny, nx))
    ux[mask == 1] = 0.0
    return case, equilibrium_state(rho, ux, uy)


def liner_arrays(p: LinerParams):
    """Per-node R, m, K along the bottom row (m = 0 outside the liner)."""
    i0, i1 = p.liner_span
    R = np.zeros(p.nx)
    m = np.zeros(p.nx)
    K = np.zeros(p.nx)
    R[i0:i1], m[i0:i1], K[i0:i1] = p.R, p.m, p.K
    return R, m, K


def sample_liners(n: int = 64, seed: int = 2026) -> List[LinerParams]:
    """The seeded batch of the liner configuration: nx ~ U[512, 2048],
    ny ~ U[64, 256], Ma ~ U[0, 0.3], R ~ U[0.5, 3] rho c, m ~ U[1e-3, 1e-2],
    f_res ~ U[0.02, 0.1]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx = int(rng.integers(512, 2049))
        ny = int(rng.integers(64, 257))
        mach = float(rng.uniform(0.0, 0.3))
        R = float(rng.uniform(0.5, 3.0)) * CS
        m = float(rng.uniform(1e-3, 1e-2))
        f_res = float(rng.uniform(0.02, 0.1))
        out.append(LinerParams(nx, ny, mach, R, m, f_res))
    return out


def model_impedance(R, m, K, omegas):
    w = np.asarray(omegas, dtype=np.float64)
    return R + 1j * (w * m - K / w)


def educe(spectra: np.ndarray, omegas, demean_steps: int = 0) -> np.ndarray:
    """spectra[node, f, 4] (P re, P im, V re, V im) -> Z[node, f] = P / V.

    When omegas[0] == 0 the first bin holds the plain (window-weighted) sums of
    p' and v and is dropped from the result. For an unwindowed run of
    demean_steps steps, those sums first give the means of p' and v, which are
    removed from the other bins."""
    w = np.asarray(omegas, dtype=np.float64)
    P = spectra[..., 0] + 1j * spectra[..., 1]
    V = spectra[..., 2] + 1j * spectra[..., 3]
    if w.size and w[0] == 0.0:
        if demean_steps > 0:
            n = demean_steps
            ww = w[1:]
            D = (1.0 - np.exp(-1j * ww * n)) / (1.0 - np.exp(-1j * ww))
            P = P[..., 1:] - P[..., :1] / n * D
            V = V[..., 1:] - V[..., :1] / n * D
        else:
            P, V = P[..., 1:], V[..., 1:]
    with np.errstate(divide="ignore", invalid="ignore"):
        return P / V


def eduction_error(p: LinerParams, spectra: np.ndarray, omegas=TRACKED_OMEGAS):
    """Relative error |Z_educed - Z_model| / |Z_model| over the liner nodes at
    each eduction frequency (windowed run): (median, max) per frequency."""
    i0, i1 = p.liner_span
    Z = educe(spectra[i0:i1], omegas)
    w = np.asarray(omegas)[1:] if np.asarray(omegas)[0] == 0.0 else np.asarray(omegas)
    Zm = model_impedance(p.R, p.m, p.K, w)[None, :]
    err = np.abs(Z - Zm) / np.abs(Zm)
    return np.median(err, axis=0), np.max(err, axis=0)


def run_liner_batch(n: int = 64, steps: int = 20000, storage: int = 1, seed: int = 2026,
                    params: List[LinerParams] = None):
    """Build the seeded ducts, attach each liner's impedance wall, advance all
    of them in one batch (timed with CUDA events) and educe every liner.
    Returns a dict with the aggregate MLUPS and the eduction errors."""
    from .runtime import GpuBatch, GpuSolver
    params = params if params is not None else sample_liners(n, seed)
    solvers = []
    fluid = 0
    for p in params:
        case, st = liner_duct(p)
        fluid += int(np.count_nonzero(case.solid_mask == 0))
        s = GpuSolver(case, storage)
        R, m, K = liner_arrays(p)
        s.set_impedance_wall(LINER_ENTRY, R, m, K, TRACKED_OMEGAS, 1.0, MEAN_RATE, steps)
        s.set_state(st)
        solvers.append(s)
    batch = GpuBatch(solvers)
    nodes, lps = batch.info()
    ms = batch.run_timed(steps)
    tuned, tile, _ = batch.autotune_status()
    med, mx, finite = [], [], True
    for p, s in zip(params, solvers):
        spec, _ = s.impedance_readback(LINER_ENTRY)
        a, b = eduction_error(p, spec)
        med.append(a)
        mx.append(b)
        rho, _, _ = s.get_fields()
        finite = finite and bool(np.all(np.isfinite(rho[1:-1, 1:-1])))
    med, mx = np.array(med), np.array(mx)
    return {"ducts": len(params), "nodes": int(nodes), "fluid_nodes": fluid, "steps": steps, "ms": ms,
            "mlups": nodes * steps / (ms / 1e3) / 1e6, "launches_per_step": lps,
            "tile": list(tile), "tile_tuned": tuned,
            "omegas": EDUCTION_OMEGAS.tolist(),
            "eduction_err_median": np.median(med, axis=0).tolist(),
            "eduction_err_max": np.max(mx, axis=0).tolist(), "finite": finite}
