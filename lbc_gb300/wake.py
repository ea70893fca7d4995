"""Cylinder wake statistics: drag and lift coefficients and the Strouhal number.

The configuration is lbc's cylinder case in a channel (cases/cylinder/cylinder.c):
2048 x 512 nodes, D = 64 at (512, 256), interpolated bounce-back on the
cylinder, regularized parabolic velocity inlet (u_max = 0.05), regularized
pressure outlet, solid top and bottom rows, Re = u_max D / nu = 100. The
momentum-exchange force (D, L) of every step is recorded on the device;
Cd = 2 D / (rho u_max^2 D_cyl), Cl likewise (lbc normalises by its own
reference force, cases/cylinder/cylinder.c:48-49); St = f D_cyl / u_max with f
the dominant frequency of Cl over the second half of the run
(cases/cylinder/process.py:134-151 takes the FFT peak of Cl the same way).
"""
from __future__ import annotations

import numpy as np

from . import cases
from .runtime import GpuSolver


def strouhal(cl: np.ndarray, D: float, u: float) -> float:
    """Dominant frequency of a lift history (per step), as f D / u: the peak of
    a Hann-windowed FFT zero-padded eightfold, refined by parabolic
    interpolation of the log spectrum. 0 for a constant history."""
    x = np.asarray(cl, dtype=np.float64)
    mean = float(x.mean()) if len(x) else 0.0
    x = x - mean
    n = len(x)
    if n < 16 or np.max(np.abs(x)) <= 1e-12 * max(1.0, abs(mean)):
        return 0.0
    m = 8 * n
    spec = np.abs(np.fft.rfft(x * np.hanning(n), m))
    k = int(np.argmax(spec[1:])) + 1
    kf = float(k)
    if k < len(spec) - 1 and spec[k - 1] > 0 and spec[k + 1] > 0:
        a, b, c = np.log(spec[k - 1]), np.log(spec[k]), np.log(spec[k + 1])
        kf = k + 0.5 * (a - c) / (a - 2 * b + c)
    return float(kf / m * D / u)


def cylinder_forces(storage: int, steps: int, Nx: int = 2048, Ny: int = 512, D: float = 64.0,
                    u_max: float = 0.05, Re: float = 100.0, seed: int = 0):
    """Run the cylinder case for `steps` steps in one storage type; return the
    per-step (Cd, Cl) history and the device time."""
    case, st = cases.cylinder_wake(Nx, Ny, D=D, xc=Nx / 4.0, yc=Ny / 2.0, u_max=u_max, Re=Re, seed=seed)
    s = GpuSolver(case, storage)
    s.enable_force_history(steps)
    s.set_state(st)
    ms = s.run_timed(steps)
    hist = s.force_history(steps)  # columns (x, y): drag, lift
    scale = 2.0 / (1.0 * u_max * u_max * D)
    cd = hist[:, 0] * scale
    cl = hist[:, 1] * scale
    return {"cd": cd, "cl": cl, "ms": ms, "nodes": case.nodes}


def summary(h, D: float = 64.0, u_max: float = 0.05) -> dict:
    """Mean Cd, rms Cl and St over the second half of a history."""
    n = len(h["cd"])
    cd, cl = h["cd"][n // 2:], h["cl"][n // 2:]
    return {"cd_mean": float(np.mean(cd)), "cl_rms": float(np.sqrt(np.mean((cl - cl.mean()) ** 2))),
            "st": strouhal(cl, D, u_max), "mlups": h["nodes"] * n / (h["ms"] / 1e3) / 1e6}
