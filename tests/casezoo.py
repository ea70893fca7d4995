"""Small seeded cases that together exercise every path of lbc's step.

Each builder returns (case, state). The zoo covers: halfway bounce-back on
walls and on an interior obstacle (MEM force), interpolated bounce-back (both
q branches, behind node solid or off-grid), all 18 of lbc's edge BCs including
non-redundant periodic entries, per-node omega, a body force, stale slots on
non-periodic edges, and step 0 colliding with stored fields that differ from
the moments of f.
"""
import numpy as np

from lbc_gb300 import cases
from lbc_gb300.cases import BC, Case


def _rng_vals(rng, n, scale=0.01):
    return scale * rng.standard_normal(n)


def _obstacle(mask, i0, j0, w, h):
    mask[j0:j0 + h, i0:i0 + w] = 1


def zoo_zh_mixed(seed=11):
    """Zou-He pressure inlet / velocity outlet / velocity bottom (lbc's bug at
    src/bc/velocity_bottom.c:39 included) + regularized top, obstacle, body force."""
    rng = np.random.default_rng(seed)
    Nx, Ny = 48, 24
    mask = np.zeros((Ny, Nx), np.int32)
    _obstacle(mask, 20, 9, 5, 4)
    om = np.full((Ny, Nx), 1.0 / 0.75)
    bcs = [BC("pressure_inlet", 0, 1.0 + _rng_vals(rng, Ny, 1e-3), None),
           BC("velocity_outlet", Nx - 1, 0.02 + _rng_vals(rng, Ny, 1e-3), _rng_vals(rng, Ny, 1e-3)),
           BC("velocity_bottom", 0, _rng_vals(rng, Nx, 1e-3), _rng_vals(rng, Nx, 1e-3)),
           BC("velocity_top_regularized", Ny - 1, 0.01 + _rng_vals(rng, Nx, 1e-3), _rng_vals(rng, Nx, 1e-3))]
    case = Case("zoo_zh_mixed", Nx, Ny, mask, om, np.zeros((Ny, Nx)), bcs, Fx=2e-6, Fy=-1e-6)
    return case, cases.random_state(case, seed)


def zoo_pressure_reg(seed=12):
    """Convective inlet, Zou-He pressure outlet, regularized pressure top and
    bottom, per-node omega."""
    rng = np.random.default_rng(seed)
    Nx, Ny = 40, 20
    mask = np.zeros((Ny, Nx), np.int32)
    _obstacle(mask, 15, 7, 4, 6)
    om = 1.0 / (0.7 + 0.2 * rng.random((Ny, Nx)))
    bcs = [BC("convective_inlet", 0, None, None),
           BC("pressure_outlet", Nx - 1, 1.0 + _rng_vals(rng, Ny, 1e-3), None),
           BC("pressure_bottom_regularized", 0, 1.0 + _rng_vals(rng, Nx, 1e-3), None),
           BC("pressure_top_regularized", Ny - 1, 1.0 + _rng_vals(rng, Nx, 1e-3), None)]
    case = Case("zoo_pressure_reg", Nx, Ny, mask, om, np.zeros((Ny, Nx)), bcs)
    return case, cases.random_state(case, seed)


def zoo_reg_periodic(seed=13):
    """Regularized pressure inlet / velocity outlet, periodic in y, solid
    obstacle touching the top/bottom wrap."""
    rng = np.random.default_rng(seed)
    Nx, Ny = 36, 22
    mask = np.zeros((Ny, Nx), np.int32)
    _obstacle(mask, 12, 0, 3, 3)
    _obstacle(mask, 12, Ny - 2, 3, 2)
    bcs = [BC("periodic_y"),
           BC("pressure_inlet_regularized", 0, 1.0 + _rng_vals(rng, Ny, 1e-3), None),
           BC("velocity_outlet_regularized", Nx - 1, 0.02 + _rng_vals(rng, Ny, 1e-3), _rng_vals(rng, Ny, 1e-3))]
    case = Case("zoo_reg_periodic", Nx, Ny, mask, np.full((Ny, Nx), 1.0 / 0.8), np.zeros((Ny, Nx)), bcs)
    return case, cases.random_state(case, seed)


def zoo_periodic_late(seed=14):
    """A periodic_x entry after a Zou-He lid: it runs as a real stage and
    overwrites the lid's corner nodes, as lbc does."""
    rng = np.random.default_rng(seed)
    Nx, Ny = 32, 18
    mask = np.zeros((Ny, Nx), np.int32)
    mask[0, :] = 1
    bcs = [BC("velocity_top", Ny - 1, 0.05 + _rng_vals(rng, Nx, 1e-3), _rng_vals(rng, Nx, 1e-4)),
           BC("periodic_x")]
    case = Case("zoo_periodic_late", Nx, Ny, mask, np.full((Ny, Nx), 1.0 / 0.9), np.zeros((Ny, Nx)), bcs)
    return case, cases.random_state(case, seed)


def zoo_ibb(seed=15):
    """Interpolated bounce-back on a cylinder near an open inlet: both q
    branches, solid behind nodes and behind nodes off the grid; Zou-He
    velocity inlet, convective outlet, periodic y (the golden run's BCs)."""
    Nx, Ny = 60, 30
    x = np.arange(Nx, dtype=np.float64)[None, :]
    y = np.arange(Ny, dtype=np.float64)[:, None]
    R = 5.3
    d2 = (x - 2.4) ** 2 + (y - 15.2) ** 2          # cut by the inlet column
    d2b = (x - 30.3) ** 2 + (y - 14.7) ** 2
    mask = ((d2 <= R * R) | (d2b <= R * R)).astype(np.int32)
    phi = np.minimum(np.sqrt(d2), np.sqrt(d2b)) - R
    rng = np.random.default_rng(seed)
    bcs = [BC("periodic_y"),
           BC("velocity_inlet", 0, 0.03 + _rng_vals(rng, Ny, 1e-3), _rng_vals(rng, Ny, 1e-4)),
           BC("convective_outlet", Nx - 1, None, None)]
    case = Case("zoo_ibb", Nx, Ny, mask, np.full((Ny, Nx), 1.0 / 0.85), phi, bcs, use_IBB=1)
    return case, cases.random_state(case, seed)


def zoo_open_edges(seed=16):
    """No BC on the left/right edges and no periodicity: populations pulled
    from off the grid keep their old buffer content (src/core/streaming.c:36-37)."""
    Nx, Ny = 30, 16
    mask = np.zeros((Ny, Nx), np.int32)
    mask[0, :] = 1
    mask[Ny - 1, :] = 1
    case = Case("zoo_open_edges", Nx, Ny, mask, np.full((Ny, Nx), 1.0 / 0.9), np.zeros((Ny, Nx)), [],
                Fx=1e-5)
    return case, cases.random_state(case, seed)


def zoo_convective_chain(seed=17):
    """Convective outlet reading a column another BC wrote earlier in the list
    (the later BC sees the earlier one's values)."""
    rng = np.random.default_rng(seed)
    Nx, Ny = 28, 14
    mask = np.zeros((Ny, Nx), np.int32)
    bcs = [BC("velocity_inlet_regularized", 0, 0.02 + _rng_vals(rng, Ny, 1e-3), _rng_vals(rng, Ny, 1e-3)),
           BC("velocity_outlet_regularized", Nx - 2, 0.02 + _rng_vals(rng, Ny, 1e-3), _rng_vals(rng, Ny, 1e-3)),
           BC("convective_outlet", Nx - 1, None, None),
           BC("velocity_bottom_regularized", 0, _rng_vals(rng, Nx, 1e-3), _rng_vals(rng, Nx, 1e-3)),
           BC("velocity_top_regularized", Ny - 1, _rng_vals(rng, Nx, 1e-3), _rng_vals(rng, Nx, 1e-3))]
    case = Case("zoo_convective_chain", Nx, Ny, mask, np.full((Ny, Nx), 1.0 / 0.8), np.zeros((Ny, Nx)), bcs)
    return case, cases.random_state(case, seed)


def zoo_moving_lid(seed=18):
    """Cavity with a moving-wall bounce-back lid (extension; not in lbc)."""
    case, st = cases.cavity_moving_wall(N=24, u_lid=0.1, Re=50.0)
    return case, cases.random_state(case, seed, amp=0.01)


def zoo_zh_corrected(seed=19):
    """The corrected Zou-He bottom closure (extension; not in lbc) beside
    lbc's Zou-He top, a convective outlet, a velocity inlet and an obstacle."""
    rng = np.random.default_rng(seed)
    Nx, Ny = 44, 20
    mask = np.zeros((Ny, Nx), np.int32)
    _obstacle(mask, 18, 8, 4, 4)
    bcs = [BC("velocity_inlet", 0, 0.02 + _rng_vals(rng, Ny, 1e-3), _rng_vals(rng, Ny, 1e-3)),
           BC("convective_outlet", Nx - 1, None, None),
           BC("velocity_bottom_corrected", 0, 0.03 + _rng_vals(rng, Nx, 1e-3), _rng_vals(rng, Nx, 1e-3)),
           BC("velocity_top", Ny - 1, _rng_vals(rng, Nx, 1e-3), _rng_vals(rng, Nx, 1e-3))]
    case = Case("zoo_zh_corrected", Nx, Ny, mask, np.full((Ny, Nx), 1.0 / 0.7), np.zeros((Ny, Nx)), bcs)
    return case, cases.random_state(case, seed)


def standard_cases():
    """(name, builder, steps) for lbc-semantics parity tests."""
    return [
        ("poiseuille", lambda: cases.poiseuille(64, 16, 0.8, 1e-5), 200),
        ("taylor_green", lambda: cases.taylor_green(48, 32, 0.04, 0.56), 100),
        ("cavity_zouhe", lambda: cases.cavity_zouhe(32, 0.1, 100.0), 150),
        ("all_regularized_box", lambda: cases.all_regularized_box(), 80),
        ("cylinder_golden_res2", lambda: cases.cylinder_golden(res=2, tau=0.53)[:2], 60),
        ("cylinder_wake_small", lambda: cases.cylinder_wake(96, 32, D=8, xc=24, yc=16), 60),
        ("zoo_zh_mixed", zoo_zh_mixed, 60),
        ("zoo_pressure_reg", zoo_pressure_reg, 60),
        ("zoo_reg_periodic", zoo_reg_periodic, 60),
        ("zoo_periodic_late", zoo_periodic_late, 60),
        ("zoo_ibb", zoo_ibb, 60),
        ("zoo_open_edges", zoo_open_edges, 60),
        ("zoo_convective_chain", zoo_convective_chain, 60),
        # odd widths: the last column has no pair partner (per-node path in
        # the plain kernel, special-node list in geometry kernels and batches)
        ("taylor_green_odd", lambda: cases.taylor_green(47, 33, 0.04, 0.56), 100),
        ("cylinder_odd", lambda: cases.cylinder_wake(95, 33, D=8, xc=24, yc=16), 60),
    ]


def extension_cases():
    """(name, builder, steps) for extensions with no counterpart in lbc
    (checked against the oracle's restatement, not against lbc's build)."""
    return [("zoo_moving_lid", zoo_moving_lid, 60), ("zoo_zh_corrected", zoo_zh_corrected, 60)]


def build(name):
    for n, b, s in standard_cases() + extension_cases():
        if n == name:
            return b(), s
    raise KeyError(name)
