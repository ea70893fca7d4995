"""FP64 storage with the fused multiply-add step (LBM_GPU_F64_FMA): lbc's FP64
step with fewer FP64 instructions, rounded differently, so it agrees with lbc
to rounding, not bit for bit. Error measure: max |a - b| / max |b| over the
fluid nodes (solid nodes are NaN in lbc) for rho and the populations, and for
the velocity as a vector (the largest component difference over the largest
speed); forces to 1e-12 of the gross link sum. Checked against the oracle
(lbc's FP64 step restated, itself pinned bit for bit to lbc's build) at 1e-12
relative, and on the 20,000-step channel, where 1e-12 is the size of FP64
rounding itself, against the same step in extended precision
(tests/golden/poiseuille_extended.c): there both lbc's arithmetic (3e-13 in
u) and this one stay within 1e-12 of the exact-arithmetic solution, and so
within 2e-12 of each other."""
import os

import numpy as np
import pytest

import casezoo
from conftest import GOLDEN, force_close, gross_force, same
from lbc_gb300 import cases

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def _relerr(a, b, m):
    """max |a - b| / max |b| over the nodes m."""
    b = b[m]
    return float(np.max(np.abs(a[m] - b)) / max(np.max(np.abs(b)), 1e-300))


def _velerr(got, want, m):
    """max |(u, v) - (u, v)_ref| / max |(u, v)_ref|: the velocity as a vector,
    so a component that is only round-off around zero (v in a channel) is
    measured against the flow's speed, not against its own noise."""
    du = np.maximum(np.abs(got.u[m] - want.u[m]), np.abs(got.v[m] - want.v[m]))
    return float(np.max(du) / np.max(np.hypot(want.u[m], want.v[m])))


def _check(case, got, want, what):
    m = case.solid_mask == 0
    e = _relerr(got.rho, want.rho, m)
    assert e <= RTOL, (what, "rho", e)
    e = _velerr(got, want, m)
    assert e <= RTOL, (what, "u", e)
    for fld in ("f", "f_new"):
        e = _relerr(getattr(got, fld), getattr(want, fld), m)
        assert e <= RTOL, (what, fld, e)


def _run_fma(case, st, steps, hist=False):
    from lbc_gb300 import F64_FMA, GpuSolver
    s = GpuSolver(case, F64_FMA)
    if hist:
        s.enable_force_history(steps)
    s.set_state(st)
    s.run(steps)
    out = s.get_state()
    h = s.force_history(steps) if hist else None
    s.close()
    return out, h


def test_poiseuille_256x64_20000_steps(oracle):
    """The small plain-method configuration at its full length."""
    case, st = cases.poiseuille(256, 64, 0.8, 1e-6)
    got, _ = _run_fma(case, st, 20000)
    oracle.run(case, st, 20000)
    ext = np.load(os.path.join(GOLDEN, "ext_poiseuille_256x64_20000.npz"))
    rows = slice(1, 63)
    umax = float(np.max(np.abs(ext["u"][rows])))
    for name, run in (("fma", got), ("lbc", st)):
        e_u = float(np.max(np.abs(run.u[rows] - ext["u"][rows, None]))) / umax
        e_r = float(np.max(np.abs(run.rho[rows] - ext["rho"][rows, None])))
        assert e_u <= 1e-12 and e_r <= 1e-12, (name, e_u, e_r)
    m = case.solid_mask == 0
    assert _relerr(got.rho, st.rho, m) <= 1e-13
    assert _relerr(got.u, st.u, m) <= 2e-12
    # v is zero in exact arithmetic: both runs hold only round-off there
    # (lbc's own reaches about 1e-14 over this run)
    assert np.max(np.abs(got.v[m])) <= 2e-14 and np.max(np.abs(st.v[m])) <= 2e-14


@pytest.mark.parametrize("n,steps", [(1024, 500), (4096, 20)])
def test_taylor_green(oracle, n, steps):
    case, st = cases.taylor_green(n, n, 0.04, 0.56)
    got, _ = _run_fma(case, st, steps)
    oracle.run(case, st, steps)
    _check(case, got, st, f"taylor_green {n}")


@pytest.mark.parametrize("name", [n for n, _, _ in casezoo.standard_cases()])
def test_every_edge_case_within_tolerance(oracle, name):
    """Walls, IBB, every Boundary kind, body forces, open edges, odd widths."""
    (case, st), steps = casezoo.build(name)
    hist = bool(case.solid_mask.any())
    got, h = _run_fma(case, st, steps, hist)
    fo = oracle.run(case, st, steps, record_forces=True)
    _check(case, got, st, name)
    if hist:
        mag = gross_force(case)
        assert force_close(h[:, 0], fo[:, 1], rtol=RTOL, scale=mag), name
        assert force_close(h[:, 1], fo[:, 0], rtol=RTOL, scale=mag), name


def test_cylinder_wake_2048x512(oracle):
    """The cylinder configuration at full size, 200 steps: IBB, regularized
    inlet and outlet, wall force."""
    case, st = cases.cylinder_wake(2048, 512, 64.0, 512.0, 256.0, 0.05, 100.0)
    got, h = _run_fma(case, st, 200, hist=True)
    fo = oracle.run(case, st, 200, record_forces=True)
    _check(case, got, st, "cylinder")
    mag = gross_force(case)
    assert force_close(h[:, 0], fo[:, 1], rtol=RTOL, scale=mag)
    assert force_close(h[:, 1], fo[:, 0], rtol=RTOL, scale=mag)


def test_batch_equals_alone():
    """A batch of FMA cases (one persistent kernel per step) leaves each case
    exactly as when it runs alone, bit for bit, across run boundaries."""
    from lbc_gb300 import F64_FMA, GpuBatch, GpuSolver
    names = ["zoo_ibb", "taylor_green", "poiseuille", "cylinder_wake_small", "zoo_convective_chain"]
    built = [casezoo.build(n)[0] for n in names]
    alone = []
    for case, st in built:
        s = GpuSolver(case, F64_FMA)
        s.set_state(st)
        s.run(45)
        alone.append(s.get_state())
        s.close()
    solvers = []
    for case, st in built:
        s = GpuSolver(case, F64_FMA)
        s.set_state(st)
        solvers.append(s)
    b = GpuBatch(solvers)
    b.run(20)
    b.run(25)
    for s, a, n in zip(solvers, alone, names):
        got = s.get_state()
        for fld in ("f", "f_new", "rho", "u", "v"):
            assert same(getattr(got, fld), getattr(a, fld)), (n, fld)
    b.close()


def test_rejects_weights_without_pair_symmetry():
    from lbc_gb300 import F64_FMA, GpuSolver
    case, st = cases.taylor_green(32, 32, 0.04, 0.56)
    case.w = case.w.copy()
    case.w[1], case.w[2] = case.w[1] * 1.5, case.w[2] * 0.5
    with pytest.raises(RuntimeError, match="weight symmetry"):
        GpuSolver(case, F64_FMA)
