"""Case setup recipes: geometry, boundary list and initial state of lbc-style cases.

Each builder returns a :class:`Case` whose arrays follow lbc's layout
(``f[Ny][Nx][Q]`` AoS with k fastest, scalar fields ``[Ny][Nx]``, ``int`` solid
mask) and whose boundary list names lbc's BC functions, exactly as a C case main
fills its ``Boundary[]`` array (e.g. cases/nit/nit.c:153-174). The same
``Case`` drives the GPU drop-in through the C ABI, and tests hand it to CPU
checkers with the same signatures.

Initial populations follow the equilibrium start of cases/cylinder/cylinder.c:133-145
(``w_k rho (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u.u)``, evaluated in that order) and
``f_new`` is a copy of ``f`` (cases/cylinder/cylinder.c:145).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

Q = 9
# lbc's D2Q9 ordering (cases/nit/nit.c:195-202).
CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], dtype=np.int32)
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1], dtype=np.int32)
OPP = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6], dtype=np.int32)
W = np.array([4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
              1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0], dtype=np.float64)

# lbc BC function names (include/lbm_bc.h). "line" tells which edge line a BC acts on.
BC_COLUMN = (
    "velocity_inlet", "velocity_outlet", "pressure_inlet", "pressure_outlet",
    "velocity_inlet_regularized", "velocity_outlet_regularized",
    "pressure_inlet_regularized", "pressure_outlet_regularized",
    "convective_inlet", "convective_outlet",
)
BC_ROW = (
    "velocity_top", "velocity_bottom", "velocity_bottom_corrected",
    "velocity_top_regularized", "velocity_bottom_regularized",
    "pressure_top_regularized", "pressure_bottom_regularized",
)
BC_PERIODIC = ("periodic_x", "periodic_y")
BC_NAMES = BC_COLUMN + BC_ROW + BC_PERIODIC


@dataclasses.dataclass
class BC:
    """One entry of lbc's ``Boundary`` list (include/lbm_types.h:21-26)."""
    name: str
    index: int = 0
    val1: Optional[np.ndarray] = None
    val2: Optional[np.ndarray] = None


@dataclasses.dataclass
class Case:
    name: str
    Nx: int
    Ny: int
    solid_mask: np.ndarray          # int32 [Ny, Nx]
    omega_eff: np.ndarray           # float64 [Ny, Nx]
    phi: np.ndarray                 # float64 [Ny, Nx] level set (IBB)
    bcs: List[BC]
    Fx: float = 0.0
    Fy: float = 0.0
    use_IBB: int = 0
    # Moving-wall extension: wall velocity of solid nodes (zero means fixed wall).
    wall_u: Optional[np.ndarray] = None
    wall_v: Optional[np.ndarray] = None
    cx: np.ndarray = dataclasses.field(default_factory=lambda: CX.copy())
    cy: np.ndarray = dataclasses.field(default_factory=lambda: CY.copy())
    w: np.ndarray = dataclasses.field(default_factory=lambda: W.copy())
    opp: np.ndarray = dataclasses.field(default_factory=lambda: OPP.copy())

    @property
    def isperiodic_x(self) -> int:
        # Derived by function identity, as cases/nit/nit.c:187-192 does.
        return int(any(b.name == "periodic_x" for b in self.bcs))

    @property
    def isperiodic_y(self) -> int:
        return int(any(b.name == "periodic_y" for b in self.bcs))

    @property
    def nodes(self) -> int:
        return self.Nx * self.Ny


@dataclasses.dataclass
class State:
    f: np.ndarray       # float64 [Ny, Nx, Q]
    f_new: np.ndarray   # float64 [Ny, Nx, Q]
    rho: np.ndarray     # float64 [Ny, Nx]
    u: np.ndarray
    v: np.ndarray

    def copy(self) -> "State":
        return State(self.f.copy(), self.f_new.copy(), self.rho.copy(), self.u.copy(), self.v.copy())


def equilibrium(rho: np.ndarray, ux: np.ndarray, uy: np.ndarray, w: np.ndarray = W,
                cx: np.ndarray = CX, cy: np.ndarray = CY) -> np.ndarray:
    """f_eq in lbc's operation order (cases/cylinder/cylinder.c:135-141)."""
    Ny, Nx = rho.shape
    f = np.empty((Ny, Nx, Q), dtype=np.float64)
    v_sq = ux * ux + uy * uy
    for k in range(Q):
        cu = float(cx[k]) * ux + float(cy[k]) * uy
        f[:, :, k] = w[k] * rho * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * v_sq)
    return f


def equilibrium_state(rho: np.ndarray, ux: np.ndarray, uy: np.ndarray) -> State:
    f = equilibrium(rho, ux, uy)
    return State(f, f.copy(), rho.copy(), ux.copy(), uy.copy())


def _uniform(Ny, Nx, value):
    return np.full((Ny, Nx), value, dtype=np.float64)


def poiseuille(Nx: int = 256, Ny: int = 64, tau: float = 0.8, Fx: float = 1e-6):
    """Body-force driven channel: solid rows j=0 and j=Ny-1 (halfway BB),
    periodic in x, rho=1, u=0, f=w (cases/poiseuille/poiseuille.c:47-107)."""
    mask = np.zeros((Ny, Nx), dtype=np.int32)
    mask[0, :] = 1
    mask[Ny - 1, :] = 1
    case = Case("poiseuille", Nx, Ny, mask, _uniform(Ny, Nx, 1.0 / tau), _uniform(Ny, Nx, 0.0),
                [BC("periodic_x")], Fx=Fx)
    rho = _uniform(Ny, Nx, 1.0)
    zero = _uniform(Ny, Nx, 0.0)
    f = np.empty((Ny, Nx, Q))
    f[:] = W  # f = w rho0 (cases/poiseuille/poiseuille.c:100-105)
    return case, State(f, f.copy(), rho, zero, zero.copy())


def couette_zh(Nx: int = 16, Ny: int = 12, tau: float = 0.8, U: float = 0.05,
               bottom: str = "velocity_bottom_corrected"):
    """Plane Couette flow between Zou-He walls, periodic in x: the bottom row
    moves at U (`bottom`: velocity_bottom_corrected or lbc's velocity_bottom),
    the top row is at rest (velocity_top). The steady profile is linear between
    the wall nodes, u(j) = U (1 - j / (Ny - 1))."""
    mask = np.zeros((Ny, Nx), dtype=np.int32)
    bcs = [BC("periodic_x"), BC(bottom, 0, np.full(Nx, U), np.zeros(Nx)),
           BC("velocity_top", Ny - 1, np.zeros(Nx), np.zeros(Nx))]
    case = Case("couette_zh", Nx, Ny, mask, _uniform(Ny, Nx, 1.0 / tau), _uniform(Ny, Nx, 0.0), bcs)
    return case, equilibrium_state(_uniform(Ny, Nx, 1.0), _uniform(Ny, Nx, 0.0), _uniform(Ny, Nx, 0.0))


def poiseuille_analytic(Ny: int, tau: float, Fx: float) -> np.ndarray:
    """u(y) = F/(2 nu) (y - 1/2)(H - (y - 1/2)), H = Ny - 2 (walls at y = 1/2,
    cases/poiseuille/process.py:59-70)."""
    nu = (tau - 0.5) / 3.0
    H = Ny - 2
    y = np.arange(Ny, dtype=np.float64) - 0.5
    u = Fx / (2.0 * nu) * y * (H - y)
    u[0] = u[-1] = np.nan
    return u


def taylor_green(Nx: int = 4096, Ny: Optional[int] = None, u0: float = 0.04, tau: float = 0.56):
    """Fully periodic Taylor-Green vortex, wavenumber 2 pi / L in x and y,
    initialised at equilibrium (cases/taylorgreen/taylorgreen.c:46-57)."""
    Ny = Nx if Ny is None else Ny
    kx = 2.0 * math.pi / Nx
    ky = 2.0 * math.pi / Ny
    i = np.arange(Nx, dtype=np.float64)[None, :]
    j = np.arange(Ny, dtype=np.float64)[:, None]
    ux = -u0 * math.sqrt(ky / kx) * np.cos(kx * i) * np.sin(ky * j)
    uy = u0 * math.sqrt(kx / ky) * np.sin(kx * i) * np.cos(ky * j)
    rho = _uniform(Ny, Nx, 1.0)
    mask = np.zeros((Ny, Nx), dtype=np.int32)
    case = Case("taylor_green", Nx, Ny, mask, _uniform(Ny, Nx, 1.0 / tau), _uniform(Ny, Nx, 0.0),
                [BC("periodic_x"), BC("periodic_y")])
    return case, equilibrium_state(rho, ux, uy)


def taylor_green_decay_rate(Nx: int, Ny: int, tau: float) -> float:
    """Velocity amplitude decays as exp(-nu (kx^2 + ky^2) t)
    (cases/taylorgreen/process.py:56-58)."""
    nu = (tau - 0.5) / 3.0
    return nu * ((2 * math.pi / Nx) ** 2 + (2 * math.pi / Ny) ** 2)


def cavity_zouhe(N: int = 128, u_lid: float = 0.1, Re: float = 100.0):
    """Lid-driven cavity as cases/ldcf/ldcf.c:63-105: solid rows/columns j=0,
    i=0, i=N-1 and a Zou-He velocity_top lid on j=N-1."""
    Nx = Ny = N
    L = N - 2
    tau = 0.5 + 3.0 * u_lid * L / Re
    mask = np.zeros((Ny, Nx), dtype=np.int32)
    mask[0, :] = 1
    mask[:, 0] = 1
    mask[:, Nx - 1] = 1
    val1 = np.full(Nx, u_lid)
    val2 = np.zeros(Nx)
    case = Case("cavity_zouhe", Nx, Ny, mask, _uniform(Ny, Nx, 1.0 / tau), _uniform(Ny, Nx, 0.0),
                [BC("velocity_top", Ny - 1, val1, val2)])
    zero = _uniform(Ny, Nx, 0.0)
    return case, equilibrium_state(_uniform(Ny, Nx, 1.0), zero, zero.copy())


def cavity_moving_wall(N: int = 2048, u_lid: float = 0.1, Re: float = 1000.0):
    """Lid-driven cavity with solid walls on all four sides and a moving-wall
    bounce-back lid (row j=N-1 moves with u_lid). lattice L = N - 2."""
    Nx = Ny = N
    L = N - 2
    tau = 0.5 + 3.0 * u_lid * L / Re
    mask = np.zeros((Ny, Nx), dtype=np.int32)
    mask[0, :] = 1
    mask[Ny - 1, :] = 1
    mask[:, 0] = 1
    mask[:, Nx - 1] = 1
    wu = _uniform(Ny, Nx, 0.0)
    wu[Ny - 1, 1:Nx - 1] = u_lid
    wv = _uniform(Ny, Nx, 0.0)
    case = Case("cavity_moving_wall", Nx, Ny, mask, _uniform(Ny, Nx, 1.0 / tau),
                _uniform(Ny, Nx, 0.0), [], wall_u=wu, wall_v=wv)
    zero = _uniform(Ny, Nx, 0.0)
    return case, equilibrium_state(_uniform(Ny, Nx, 1.0), zero, zero.copy())


def cylinder_golden(res: int = 20, Re: float = 20.0, tau: float = 0.9):
    """The cylinder run behind cases/cylinder/sol/forces_IBB_res_20_Re_20.00_tau_0.90.bin
    (cases/cylinder/cylinder.c:28-145): 50R x 20R box, cylinder at (Lx/4, Ly/2),
    Zou-He velocity inlet, convective outlet, periodic in y, IBB.
    Returns (case, state, cf) with cf the lattice-to-physical force factor."""
    R = 1.0
    Lx, Ly = 50 * R, 20 * R
    xc, yc = Lx / 4, Ly / 2
    U_inf = 1.0
    nu = U_inf * (2 * R) / Re
    dx = R / res
    Nx = int(Lx / dx)
    Ny = int(Ly / dx)
    cu = 3.0 * nu / (dx * (tau - 0.5))
    cf = 1.0 * cu * cu * dx
    U_in = U_inf / cu
    x = np.arange(Nx, dtype=np.float64)[None, :] * dx
    y = np.arange(Ny, dtype=np.float64)[:, None] * dx
    d2 = (x - xc) * (x - xc) + (y - yc) * (y - yc)
    mask = (d2 <= R * R).astype(np.int32)
    phi = np.sqrt(d2) - R
    bcs = [BC("periodic_y"),
           BC("velocity_inlet", 0, np.full(Ny, U_in), np.zeros(Ny)),
           BC("convective_outlet", Nx - 1, np.full(Ny, 1.0), np.zeros(Ny))]
    case = Case("cylinder_golden", Nx, Ny, mask, _uniform(Ny, Nx, 1.0 / tau), phi, bcs, use_IBB=1)
    rho = _uniform(Ny, Nx, 1.0)
    ux = _uniform(Ny, Nx, U_in)
    uy = _uniform(Ny, Nx, 0.0)
    return case, equilibrium_state(rho, ux, uy), cf


def cylinder_wake(Nx: int = 2048, Ny: int = 512, D: float = 64.0, xc: float = 512.0,
                  yc: float = 256.0, u_max: float = 0.05, Re: float = 100.0, seed: int = 0):
    """Cylinder in a channel: regularized parabolic velocity inlet, regularized
    constant-pressure outlet (rho = 1), solid top/bottom rows, IBB on the
    cylinder (phi = r - R as cases/cylinder/cylinder.c:99-108). nu from u_max,
    D and Re. A seeded 64x64 patch of transverse velocity 1e-3 u_max behind the
    cylinder triggers shedding."""
    R = D / 2.0
    nu = u_max * D / Re
    tau = 0.5 + 3.0 * nu
    x = np.arange(Nx, dtype=np.float64)[None, :]
    y = np.arange(Ny, dtype=np.float64)[:, None]
    d2 = (x - xc) ** 2 + (y - yc) ** 2
    mask = (d2 <= R * R).astype(np.int32)
    mask[0, :] = 1
    mask[Ny - 1, :] = 1
    phi = np.sqrt(d2) - R
    H = Ny - 2
    yy = np.arange(Ny, dtype=np.float64) - 0.5
    prof = 4.0 * u_max * yy * (H - yy) / (H * H)
    prof[0] = prof[-1] = 0.0
    bcs = [BC("velocity_inlet_regularized", 0, prof.copy(), np.zeros(Ny)),
           BC("pressure_outlet_regularized", Nx - 1, np.ones(Ny), np.zeros(Ny))]
    case = Case("cylinder_wake", Nx, Ny, mask, _uniform(Ny, Nx, 1.0 / tau), phi, bcs, use_IBB=1)
    rng = np.random.default_rng(seed)
    ux = np.repeat(prof[:, None], Nx, axis=1)
    uy = _uniform(Ny, Nx, 0.0)
    ps = min(64, Ny // 2, Nx // 4)
    i0, j0 = int(xc + D), int(yc - ps // 2)
    patch = rng.uniform(-1.0, 1.0, size=(ps, ps))
    uy[j0:j0 + ps, i0:i0 + ps] = 1e-3 * u_max * patch
    ux[mask == 1] = 0.0
    uy[mask == 1] = 0.0
    return case, equilibrium_state(_uniform(Ny, Nx, 1.0), ux, uy)


def all_regularized_box(Nx: int = 40, Ny: int = 30, tau: float = 0.7, seed: int = 1):
    """Box with a regularized BC on every edge, in the order of
    cases/testbc/testbc.c:58-76 (inlet, outlet, bottom, top), per-node omega
    with a second value on i <= Nx/4 (testbc.c:107-116) and a random smooth
    start."""
    rng = np.random.default_rng(seed)
    om = _uniform(Ny, Nx, 1.0 / tau)
    om[:, : Nx // 4 + 1] = 1.0 / 0.9
    mask = np.zeros((Ny, Nx), dtype=np.int32)
    bcs = [BC("velocity_inlet_regularized", 0, 0.01 * rng.standard_normal(Ny), 0.01 * rng.standard_normal(Ny)),
           BC("velocity_outlet_regularized", Nx - 1, 0.01 * rng.standard_normal(Ny), 0.01 * rng.standard_normal(Ny)),
           BC("velocity_bottom_regularized", 0, 0.01 * rng.standard_normal(Nx), 0.01 * rng.standard_normal(Nx)),
           BC("velocity_top_regularized", Ny - 1, 0.01 * rng.standard_normal(Nx), 0.01 * rng.standard_normal(Nx))]
    case = Case("all_regularized_box", Nx, Ny, mask, om, _uniform(Ny, Nx, 0.0), bcs)
    rho = 1.0 + 1e-3 * rng.standard_normal((Ny, Nx))
    ux = 0.02 * rng.standard_normal((Ny, Nx))
    uy = 0.02 * rng.standard_normal((Ny, Nx))
    return case, equilibrium_state(rho, ux, uy)


def random_state(case: Case, seed: int = 0, amp: float = 0.02) -> State:
    """A seeded non-equilibrium state: equilibrium of a random smooth field
    plus independent noise on every population of both buffers, and stored
    rho/u/v that differ from the moments of f (lbc collides the first step
    with the stored fields, not with the moments)."""
    rng = np.random.default_rng(seed)
    Ny, Nx = case.Ny, case.Nx
    rho = 1.0 + 0.01 * rng.standard_normal((Ny, Nx))
    ux = amp * rng.standard_normal((Ny, Nx))
    uy = amp * rng.standard_normal((Ny, Nx))
    f = equilibrium(rho, ux, uy) * (1.0 + 1e-3 * rng.standard_normal((Ny, Nx, Q)))
    f_new = equilibrium(rho, ux, uy) * (1.0 + 1e-3 * rng.standard_normal((Ny, Nx, Q)))
    rho2 = rho + 1e-4 * rng.standard_normal((Ny, Nx))
    return State(f, f_new, rho2, ux + 1e-4 * rng.standard_normal((Ny, Nx)),
                 uy + 1e-4 * rng.standard_normal((Ny, Nx)))
