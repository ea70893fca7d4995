"""The oracle (oracle/lbm_oracle.c) pinned against lbc itself.

Three anchors: (1) golden fixtures produced by lbc's own src/ (tests/golden,
made by tests/golden/make_golden.py), (2) lbc's src/ compiled here
(oracle/_ref) when its sources are present, (3) lbc's shipped cylinder force
history (cases/cylinder/sol/forces_IBB_res_20_Re_20.00_tau_0.90.bin).
"""
import os

import numpy as np
import pytest

import casezoo
from conftest import GOLDEN, maxrel, same
from lbc_gb300 import cases

NAMES = [n for n, _, _ in casezoo.standard_cases()]


def force_close(a, b, case, rtol=1e-12):
    """Per-step forces agree to rtol of the gross link sum (0.5 per wall link):
    lbc sums the links with OpenMP atomics in no fixed order, and the net lift
    of a symmetric flow is pure cancellation."""
    a, b = np.asarray(a), np.asarray(b)
    m = case.solid_mask.astype(bool)
    n = sum(int(np.sum(~m & np.roll(np.roll(m, -int(case.cy[k]), 0), -int(case.cx[k]), 1))) for k in range(1, 9))
    return np.max(np.abs(a - b)) <= rtol * 0.5 * max(n, 1) if b.size else True


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_lbc_fixture(oracle, name):
    (case, st), steps = casezoo.build(name)
    fr = oracle.run(case, st, steps, record_forces=True)
    g = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    for fld in ("f", "f_new", "rho", "u", "v"):
        assert same(getattr(st, fld), g[fld]), (name, fld, maxrel(getattr(st, fld), g[fld]))
    assert force_close(fr, g["forces"], case), name


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_lbc_build(oracle, ref, name):
    (case, st), steps = casezoo.build(name)
    st2 = st.copy()
    fa = oracle.run(case, st, 20, record_forces=True)
    fb = ref.run(case, st2, 20, record_forces=True)
    for fld in ("f", "f_new", "rho", "u", "v"):
        assert same(getattr(st, fld), getattr(st2, fld)), (name, fld)
    assert force_close(fa, fb, case)


def test_oracle_cylinder_golden_forces(oracle):
    """lbc's shipped drag record (res 20, Re 20, tau 0.9, IBB): D matches to
    round-off; L (near zero, summed with atomics in lbc) to 1e-9 of D."""
    g = np.load(os.path.join(GOLDEN, "lbc_cylinder_forces_res20_first300.npy"))
    case, st, cf = cases.cylinder_golden()
    n = 40
    fr = oracle.run(case, st, n, record_forces=True)
    D = fr[:, 1] * cf
    L = fr[:, 0] * cf
    assert np.max(np.abs(D - g[:n, 2]) / np.abs(g[:n, 2])) < 1e-13
    assert np.max(np.abs(L - g[:n, 1])) < 1e-9 * np.max(np.abs(g[:n, 2]))
