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


# ---------------------------------------------------------------------------
# Eduction from the acoustic field (probes in the lattice), independent of the
# wall's own state: it tests that the lattice feels the wall with the imposed
# impedance, which the wall's self-ratio P / V cannot (that ratio recovers the
# model whether or not the coupling to the lattice is right).


def wavenumber(omegas, c: float = CS, nu: float = 0.0):
    """Complex wavenumber of plane sound waves on the lattice, e^{i(w t +- k y)}
    convention: k = w / c - i alpha, with the spatial attenuation alpha = nu w^2
    / c^3 of BGK D2Q9, whose sound amplitude decays at nu K^2 in time (its bulk
    viscosity equals nu in 2D)."""
    w = np.asarray(omegas, dtype=np.float64)
    return w / c - 1j * nu * w ** 2 / c ** 3


def two_microphone(P1, P2, y1: float, y2: float, omegas, c: float = CS, nu: float = 0.0, rho: float = 1.0):
    """The transfer-function (two-microphone) method of Chung & Blaser (J.
    Acoust. Soc. Am. 68, 1980; standardised as ASTM E1050) for a plane-wave
    field normal to a surface at y = 0: P1, P2 the spectra of the pressure at
    distances y1 < y2 from it. With p(y) = A (e^{i k y} + G e^{-i k y}) and
    H = P2 / P1, the reflection coefficient is
    G = (e^{i k y2} - H e^{i k y1}) / (H e^{-i k y1} - e^{-i k y2}) and the
    surface impedance Z = rho c (1 + G) / (1 - G). Returns (G, Z)."""
    k = wavenumber(omegas, c, nu)
    H = np.asarray(P2) / np.asarray(P1)
    G = (np.exp(1j * k * y2) - H * np.exp(1j * k * y1)) / (H * np.exp(-1j * k * y1) - np.exp(-1j * k * y2))
    return G, rho * c * (1.0 + G) / (1.0 - G)


def insitu(P, U):
    """In-situ impedance at a wall from field spectra at the first three rows
    above it: P[r], U[r] the spectra of the pressure and of the wall-normal
    velocity u_y at rows r = 1, 2, 3 (arrays [3, ...]); both are extrapolated to
    the wall row by the quadratic through the three rows (3 f1 - 3 f2 + f3),
    and Z = p / v_n with v_n = -u_y the velocity into the wall."""
    P, U = np.asarray(P), np.asarray(U)
    P0 = 3.0 * P[0] - 3.0 * P[1] + P[2]
    U0 = 3.0 * U[0] - 3.0 * U[1] + U[2]
    with np.errstate(divide="ignore", invalid="ignore"):
        return P0 / (-U0)


def spectra(x: np.ndarray, omegas, window: np.ndarray = None) -> np.ndarray:
    """DFT sum_n w_n x_n e^{-i w n} of time series x[n, ...] at each omega
    (leading axis of the result), with window weights w (default 1)."""
    x = np.asarray(x, dtype=np.float64)
    n = np.arange(x.shape[0], dtype=np.float64)
    wts = np.ones_like(n) if window is None else np.asarray(window, dtype=np.float64)
    return np.stack([np.tensordot(wts * np.exp(-1j * w * n), x, axes=(0, 0)) for w in omegas])


@dataclasses.dataclass
class TubeParams:
    """A normal-incidence impedance tube: plane waves in y on a grid periodic in
    x, the impedance wall on the whole bottom row, a solid top row. A Gaussian
    pulse starts at y0, travelling down."""
    R: float
    m: float
    f_res: float
    ny: int = 512
    nx: int = 4
    tau: float = 0.6
    y0: float = 120.0
    width: float = 4.0
    amp: float = 1e-3
    mics: tuple = (3, 7)

    @property
    def K(self) -> float:
        return self.m * (2.0 * math.pi * self.f_res) ** 2

    @property
    def nu(self) -> float:
        return (self.tau - 0.5) / 3.0

    def gate(self) -> int:
        """Steps before the wave reflected by the top wall returns to the
        microphones (the window of the two-microphone spectra: incident pulse
        and its reflection from the wall only, no tube modes)."""
        return int((self.y0 + 2.0 * (self.ny - 1.5 - self.y0) - 6.0 * self.width - self.mics[1]) / CS)


TUBE_ENTRY = 1  # the impedance wall's position in the tube's Boundary list


def impedance_tube(p: TubeParams):
    """(case, state) of the tube."""
    nx, ny = p.nx, p.ny
    mask = np.zeros((ny, nx), dtype=np.int32)
    mask[ny - 1, :] = 1
    bcs = [BC("periodic_x"), BC("velocity_bottom_regularized", 0, np.zeros(nx), np.zeros(nx))]
    case = Case("impedance_tube", nx, ny, mask, np.full((ny, nx), 1.0 / p.tau), np.zeros((ny, nx)), bcs)
    y = np.arange(ny, dtype=np.float64)[:, None] * np.ones((1, nx))
    drho = p.amp * np.exp(-((y - p.y0) ** 2) / (2.0 * p.width ** 2))
    uy = -CS * drho                 # downward-running pulse
    uy[mask == 1] = 0.0
    return case, equilibrium_state(1.0 + drho, np.zeros((ny, nx)), uy)


def run_impedance_tube(p: TubeParams, storage: int = 0, omegas=EDUCTION_OMEGAS):
    """Run the tube on the device with probes at the two microphones and at
    rows 1..3 above the wall; educe the wall's impedance from the field by the
    two-microphone method and in situ, next to the model and the wall's own
    self-ratio. Returns a dict of complex arrays (per omega)."""
    from .runtime import GpuSolver
    case, st = impedance_tube(p)
    s = GpuSolver(case, storage)
    n = p.nx
    s.set_impedance_wall(TUBE_ENTRY, np.full(n, p.R), np.full(n, p.m), np.full(n, p.K), omegas, 1.0, 0.0, 0)
    y1, y2 = p.mics
    nodes = [(0, y1), (0, y2), (0, 1), (0, 2), (0, 3)]
    steps = p.gate()
    s.set_probes(nodes, steps)
    s.set_state(st)
    s.run(steps)
    h = s.probe_history(steps)                      # [steps, probes, (rho, ux, uy)]
    spec, _ = s.impedance_readback(TUBE_ENTRY)
    s.close()
    pr = (h[:, :, 0] - 1.0) * CS * CS               # p' = c^2 (rho - 1)
    Pm = spectra(pr, omegas)                        # [omega, probe]
    Um = spectra(h[:, :, 2], omegas)
    _, Z2 = two_microphone(Pm[:, 0], Pm[:, 1], y1, y2, omegas, CS, p.nu)
    Zi = insitu(Pm[:, 2:5].T, Um[:, 2:5].T)
    Zw = educe(spec[:1], omegas)[0]                 # the wall's own ratio (unwindowed, run of `steps`)
    return {"omegas": np.asarray(omegas), "model": model_impedance(p.R, p.m, p.K, omegas), "two_mic": Z2,
            "insitu": Zi, "wall": Zw, "steps": steps,
            "excitation": np.abs(Pm[:, 0]) / np.max(np.abs(Pm[:, 0]))}


def running_mean(x: np.ndarray, rate: float) -> np.ndarray:
    """Exponential running mean along axis 0 (m_n = m_{n-1} + rate (x_n -
    m_{n-1}), m_0 = x_0): the same slow reference the wall takes its p' about."""
    x = np.asarray(x, dtype=np.float64)
    out = np.empty_like(x)
    m = x[0].copy()
    for n in range(x.shape[0]):
        m += rate * (x[n] - m)
        out[n] = m
    return out


def field_probe_nodes(p: LinerParams, positions: int = 4):
    """Probe nodes for the in-situ eduction of a duct: rows 1, 2, 3 above the
    liner at `positions` points spread over the middle half of its span."""
    i0, i1 = p.liner_span
    xs = np.linspace(i0 + (i1 - i0) // 4, i1 - (i1 - i0) // 4, positions).round().astype(int)
    return [(int(x), r) for x in xs for r in (1, 2, 3)], len(xs)


def insitu_from_history(h: np.ndarray, npos: int, omegas=EDUCTION_OMEGAS, rate: float = MEAN_RATE):
    """In-situ impedance per probe position from a duct's probe history
    [steps, 3 npos, (rho, ux, uy)] (rows 1, 2, 3 per position): p' = c^2 (rho
    - running mean), Hann-windowed spectra, quadratic extrapolation to the
    wall. Returns Z[omega, position]."""
    rho = h[:, :, 0]
    pr = (rho - running_mean(rho, rate)) * CS * CS
    uy = h[:, :, 2] - running_mean(h[:, :, 2], rate)
    win = np.hanning(h.shape[0])
    P = spectra(pr, omegas, win).reshape(len(omegas), npos, 3)
    U = spectra(uy, omegas, win).reshape(len(omegas), npos, 3)
    return insitu(np.moveaxis(P, 2, 0), np.moveaxis(U, 2, 0))


def run_liner_batch(n: int = 64, steps: int = 20000, storage: int = 1, seed: int = 2026,
                    params: List[LinerParams] = None, field: bool = False, excited: float = 1e-2):
    """Build the seeded ducts, attach each liner's impedance wall, advance all
    of them in one batch (timed with CUDA events) and educe every liner.
    Returns a dict with the aggregate MLUPS and the eduction errors.

    The wall's self-ratio is reported over all bins and over the excited bins
    only: a bin is excited when the wall's mean |P| there is at least
    `excited` times its largest bin (the 8-cell Gaussian pulse has little
    content near w = 0.2), and over the excited bins' strong nodes (|P| at
    least a tenth of the liner's median: off the interference nulls along the
    liner). field=True also records probes at rows 1..3 above each liner and
    educes the impedance in situ from the lattice's field (insitu_from_history)."""
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
        if field:
            s.set_probes(field_probe_nodes(p)[0], steps)
        s.set_state(st)
        solvers.append(s)
    batch = GpuBatch(solvers)
    nodes, lps = batch.info()
    ms = batch.run_timed(steps)
    tuned, tile, _ = batch.autotune_status()
    med, mx, finite = [], [], True
    exc_all, err_all, fld_err, err_strong = [], [], [], []
    w = EDUCTION_OMEGAS
    for p, s in zip(params, solvers):
        spec, _ = s.impedance_readback(LINER_ENTRY)
        a, b = eduction_error(p, spec)
        med.append(a)
        mx.append(b)
        i0, i1 = p.liner_span
        Pn = np.abs(spec[i0:i1, 1:, 0] + 1j * spec[i0:i1, 1:, 1])      # [node, omega]
        Pm = Pn.mean(axis=0)
        exc_all.append(Pm / Pm.max())
        Zw = educe(spec[i0:i1], TRACKED_OMEGAS)
        Zm = model_impedance(p.R, p.m, p.K, w)[None, :]
        en = np.abs(Zw - Zm) / np.abs(Zm)
        err_all.append(np.max(en, axis=0))
        strong = Pn >= 0.1 * np.median(Pn, axis=0)[None, :]
        err_strong.append([float(np.max(en[strong[:, f], f])) for f in range(len(w))])
        if field:
            h = s.probe_history(steps)
            Zi = insitu_from_history(h, field_probe_nodes(p)[1])
            fld_err.append(np.median(np.abs(Zi - Zm.T) / np.abs(Zm.T), axis=1))
        rho, _, _ = s.get_fields()
        finite = finite and bool(np.all(np.isfinite(rho[1:-1, 1:-1])))
    med, mx = np.array(med), np.array(mx)
    exc, errs, es = np.array(exc_all), np.array(err_all), np.array(err_strong)
    ok = exc >= excited
    out = {"ducts": len(params), "nodes": int(nodes), "fluid_nodes": fluid, "steps": steps, "ms": ms,
           "mlups": nodes * steps / (ms / 1e3) / 1e6, "launches_per_step": lps,
           "tile": list(tile), "tile_tuned": tuned,
           "omegas": EDUCTION_OMEGAS.tolist(),
           "eduction_err_median": np.median(med, axis=0).tolist(),
           "eduction_err_max": np.max(mx, axis=0).tolist(),
           "excited_threshold": excited,
           "excited_ducts": ok.sum(axis=0).tolist(),
           "eduction_err_max_excited": [float(errs[ok[:, f], f].max()) if ok[:, f].any() else None
                                        for f in range(len(w))],
           "max_err_bin_excitation": [float(exc[int(np.argmax(errs[:, f])), f]) for f in range(len(w))],
           "eduction_err_max_excited_strong_nodes": [float(es[ok[:, f], f].max()) if ok[:, f].any() else None
                                                     for f in range(len(w))],
           "finite": finite}
    if field:
        fe = np.array(fld_err)
        out["field_insitu_err_median"] = [float(np.median(fe[ok[:, f], f])) if ok[:, f].any() else None
                                          for f in range(len(w))]
        out["field_insitu_err_max"] = [float(np.max(fe[ok[:, f], f])) if ok[:, f].any() else None
                                       for f in range(len(w))]
        out["per_duct"] = [{"nx": p.nx, "ny": p.ny, "mach": round(p.mach, 4), "R": p.R, "m": p.m, "f_res": p.f_res,
                            "excitation": [round(float(x), 5) for x in e],
                            "self_ratio_err_max": [round(float(x), 5) for x in er],
                            "self_ratio_err_max_strong_nodes": [round(float(x), 5) for x in ss],
                            "field_insitu_err": [round(float(x), 5) for x in fe_]}
                           for p, e, er, ss, fe_ in zip(params, exc, errs, es, fe)]
    return out
