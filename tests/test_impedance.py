"""Time-domain impedance wall: the zero-order-hold update, the oracle
restatement, the eduction formula, and the GPU wall against the oracle."""
import ctypes as C
import math

import numpy as np
import pytest

from conftest import same
from lbc_gb300 import impedance as imp
from lbc_gb300.abi import dptr, iptr

OI_N = 12  # fields before the per-frequency block (shared layout)


def _zoh_oracle(oracle, R, m, K):
    A, b = np.zeros(4), np.zeros(2)
    fn = oracle.lib.orc_ext_msd_zoh
    fn.restype = C.c_int
    assert fn(C.c_double(R), C.c_double(m), C.c_double(K), dptr(A), dptr(b)) == 1
    return A, b


@pytest.mark.parametrize("R,m,K", [(0.3, 1e-3, 1e-3 * (2 * math.pi * 0.05) ** 2),
                                   (1.7, 1e-2, 1e-2 * (2 * math.pi * 0.1) ** 2),
                                   (1e-4, 1e-2, 1e-2 * (2 * math.pi * 0.1) ** 2),   # underdamped
                                   (1.0, 5e-3, 5e-3 * (2 * math.pi * 0.02) ** 2)])
def test_zoh_matches_matrix_exponential(oracle, R, m, K):
    scipy_linalg = pytest.importorskip("scipy.linalg")
    A, b = _zoh_oracle(oracle, R, m, K)
    M = np.array([[0.0, 1.0], [-K / m, -R / m]])
    Ae = scipy_linalg.expm(M)
    be = np.linalg.solve(M, (Ae - np.eye(2)) @ np.array([0.0, 1.0 / m]))
    assert np.allclose(A.reshape(2, 2), Ae, rtol=1e-10, atol=1e-13)
    assert np.allclose(b, be, rtol=1e-9, atol=1e-13)


def test_library_zoh_matches_oracle(oracle):
    import lbc_gb300
    lib = lbc_gb300.load_library()
    for R, m, K in [(0.3, 1e-3, 2e-4), (1.7, 1e-2, 3e-3), (1e-4, 1e-2, 1e-2)]:
        A, b = np.zeros(4), np.zeros(2)
        assert lib.lbm_gpu_msd_zoh(R, m, K, dptr(A), dptr(b)) == 0
        A2, b2 = _zoh_oracle(oracle, R, m, K)
        assert same(A, A2) and same(b, b2)


def _imp_array(p, omegas, Nx):
    """Impedance-wall state in the shared layout for a liner."""
    R, m, K = imp.liner_arrays(p)
    nf = len(omegas)
    a = np.zeros((OI_N + 6 * nf, Nx))
    for t in range(Nx):
        if m[t] <= 0:
            continue
        A, b = np.zeros(4), np.zeros(2)
        import lbc_gb300
        assert lbc_gb300.load_library().lbm_gpu_msd_zoh(R[t], m[t], K[t], dptr(A), dptr(b)) == 0
        a[0, t] = 1.0
        a[1:5, t] = A
        a[5:7, t] = b
        a[9, t] = 1.0   # mean density starts at rho_ref
        a[10, t] = 1.0  # window phasor cos
        for f in range(nf):
            a[OI_N + 6 * f, t] = 1.0
    return a


def oracle_liner_run(oracle, p, case, st, steps, omegas, alpha=0.0, window=0):
    """The host coupling of cases/nit/nit.c:276-306, per node: impedance step
    from the stored density, then main_lbm with val2 = -v."""
    impa = _imp_array(p, omegas, case.Nx)
    cw, sw = np.cos(omegas), np.sin(omegas)
    v2 = np.zeros(case.Nx)
    bcs = list(case.bcs)
    step_fn = oracle.lib.orc_ext_impedance_step
    step_fn.restype = None
    for _ in range(steps):
        step_fn(C.c_int(case.Nx), C.c_int(0), dptr(st.rho), C.c_double(alpha), dptr(impa), C.c_int(len(omegas)),
                dptr(cw), dptr(sw), C.c_double(math.cos(2 * math.pi / window) if window else 1.0),
                C.c_double(math.sin(2 * math.pi / window) if window else 0.0), C.c_int(1 if window else 0),
                iptr(case.solid_mask), None, dptr(v2))
        bcs[imp.LINER_ENTRY] = imp.BC("velocity_bottom_regularized", 0, bcs[imp.LINER_ENTRY].val1, v2.copy())
        case2 = imp.Case(case.name, case.Nx, case.Ny, case.solid_mask, case.omega_eff, case.phi, bcs)
        oracle.step(case2, st)
    return impa


def test_eduction_recovers_the_model(oracle):
    """Drive one node with a smooth pressure pulse: the educed impedance
    matches R + i (w m - K / w) at the eduction frequencies."""
    p = imp.LinerParams(nx=4, ny=3, mach=0.0, R=0.9 * imp.CS, m=4e-3, f_res=0.05, liner_frac=1.0)
    om = imp.EDUCTION_OMEGAS
    impa = _imp_array(p, om, p.nx)
    cw, sw = np.cos(om), np.sin(om)
    rho = np.ones((3, p.nx))
    mask = np.zeros((3, p.nx), np.int32)
    v2 = np.zeros(p.nx)
    fn = oracle.lib.orc_ext_impedance_step
    fn.restype = None
    n_steps = 20000
    for n in range(n_steps):
        rho[1, :] = 1.0 + 3.0e-4 * math.exp(-((n - 200.0) ** 2) / (2 * 12.0 ** 2))
        fn(C.c_int(p.nx), C.c_int(0), dptr(rho), C.c_double(0.0), dptr(impa), C.c_int(len(om)), dptr(cw),
           dptr(sw), C.c_double(1.0), C.c_double(0.0), C.c_int(0), iptr(mask), None, dptr(v2))
    spec = np.stack([impa[OI_N + 6 * f + 2: OI_N + 6 * f + 6].T for f in range(len(om))], axis=1)
    Z = imp.educe(spec, om)[0]
    Zm = imp.model_impedance(p.R, p.m, p.K, om)
    err = np.abs(Z - Zm) / np.abs(Zm)
    print("eduction error per frequency", err)
    assert np.all(err < 2e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_liner_duct_matches_oracle(oracle, storage):
    """A small duct with an impedance-wall liner on the device against the
    oracle's host coupling: FP64 bit for bit (populations and wall state),
    FP32 close."""
    from lbc_gb300 import STORAGE, GpuSolver
    p = imp.LinerParams(nx=160, ny=24, mach=0.15, R=1.2 * imp.CS, m=5e-3, f_res=0.05)
    case, st = imp.liner_duct(p)
    om = imp.EDUCTION_OMEGAS
    s = GpuSolver(case, STORAGE[storage])
    R, m, K = imp.liner_arrays(p)
    s.set_impedance_wall(imp.LINER_ENTRY, R, m, K, om, 1.0, 2e-3, 400)
    s.set_state(st)
    steps = 150
    s.run(steps)
    out = s.get_state()
    spec, state = s.impedance_readback(imp.LINER_ENTRY)
    impa = oracle_liner_run(oracle, p, case, st, steps, om, alpha=2e-3, window=400)
    ospec = np.stack([impa[OI_N + 6 * f + 2: OI_N + 6 * f + 6].T for f in range(len(om))], axis=1)
    ostate = impa[7:9].T
    if storage == "f64":
        for fld in ("f", "f_new", "rho", "u", "v"):
            assert same(getattr(out, fld), getattr(st, fld)), fld
        assert same(state, ostate) and same(spec, ospec)
    else:
        fl = case.solid_mask == 0
        assert np.max(np.abs(out.rho[fl] - st.rho[fl])) < 1e-6
        assert np.max(np.abs(state[:, 1] - ostate[:, 1])) < 1e-3 * np.max(np.abs(ostate[:, 1])) + 1e-12


@pytest.mark.gpu
def test_liner_batch_eduction():
    """Six small random ducts in one batch (FP32-shifted populations, FP64
    walls): every duct stays finite and the educed impedance of every liner
    node matches the imposed model."""
    from lbc_gb300 import F32_SHIFTED
    rng = np.random.default_rng(7)
    params = [imp.LinerParams(int(rng.integers(160, 320)), int(rng.integers(24, 48)), float(rng.uniform(0, 0.3)),
                              float(rng.uniform(0.5, 3.0)) * imp.CS, float(rng.uniform(1e-3, 1e-2)),
                              float(rng.uniform(0.02, 0.1))) for _ in range(6)]
    r = imp.run_liner_batch(steps=3000, storage=F32_SHIFTED, params=params)
    print(r)
    assert r["finite"]
    assert max(r["eduction_err_median"]) < 5e-2


# ---------------------------------------------------------------------------
# Eduction from the lattice's acoustic field (probes), which tests the wall's
# coupling to the lattice rather than the wall's own ODE.

def test_two_microphone_recovers_a_known_reflection():
    """Synthetic plane-wave spectra p(y) = A (e^{iky} + G e^{-iky}) with
    attenuation: the transfer-function method returns G and Z to round-off."""
    om = np.array([0.03, 0.07, 0.11, 0.2])
    nu = 0.04
    k = imp.wavenumber(om, imp.CS, nu)
    G = np.array([0.3 - 0.2j, -0.5 + 0.1j, 0.0 + 0.6j, 0.9 + 0.0j])
    A = np.array([1.0, 0.3 + 0.2j, 2.0j, 0.1])
    y1, y2 = 3.0, 7.0
    P = lambda y: A * (np.exp(1j * k * y) + G * np.exp(-1j * k * y))  # noqa: E731
    G2, Z = imp.two_microphone(P(y1), P(y2), y1, y2, om, imp.CS, nu)
    assert np.allclose(G2, G, rtol=0, atol=1e-12)
    assert np.allclose(Z, imp.CS * (1 + G) / (1 - G), rtol=1e-12)


def test_insitu_extrapolates_quadratic_fields_exactly():
    y = np.array([1.0, 2.0, 3.0])
    p = 0.3 - 0.2 * y + 0.05 * y ** 2
    u = -0.1 + 0.04 * y - 0.01 * y ** 2
    assert abs(imp.insitu(p, u) - 0.3 / 0.1) < 1e-12


def test_two_microphone_sees_a_rigid_wall_in_the_oracle(oracle):
    """The method itself on lbc's step: a tube closed by a solid row (halfway
    bounce-back, wall at y = 1/2) reflects everything, G = 1 at the wall
    plane, to 1 % (the window holds the incident pulse and its reflection
    only)."""
    from lbc_gb300.cases import BC, Case, equilibrium_state
    Nx, Ny, tau = 4, 512, 0.6
    mask = np.zeros((Ny, Nx), np.int32)
    mask[0, :] = 1
    mask[Ny - 1, :] = 1
    case = Case("rigid_tube", Nx, Ny, mask, np.full((Ny, Nx), 1 / tau), np.zeros((Ny, Nx)), [BC("periodic_x")])
    tp = imp.TubeParams(1.0, 1e-3, 0.05, ny=Ny, tau=tau)
    y = np.arange(Ny, dtype=float)[:, None] * np.ones((1, Nx))
    drho = 1e-3 * np.exp(-(y - tp.y0) ** 2 / (2 * tp.width ** 2))
    st = equilibrium_state(1 + drho, np.zeros((Ny, Nx)), -imp.CS * drho)
    y1, y2 = tp.mics
    steps = tp.gate()
    bnd = oracle.boundaries(case.bcs)
    rec = np.zeros((steps, 2))
    for n in range(steps):
        oracle.step(case, st, bnd)
        rec[n] = (st.rho[y1, 0] - 1) / 3, (st.rho[y2, 0] - 1) / 3
    P = imp.spectra(rec, imp.EDUCTION_OMEGAS)
    G, _ = imp.two_microphone(P[:, 0], P[:, 1], y1 - 0.5, y2 - 0.5, imp.EDUCTION_OMEGAS, imp.CS, tp.nu)
    assert np.all(np.abs(G - 1.0) < 1e-2), G


TUBES = [(2.0, 4e-3, 0.03), (0.5, 4e-3, 0.03), (1.0, 1e-2, 0.016), (3.0, 1e-3, 0.1), (1.0, 2e-1, 0.02)]


@pytest.mark.gpu
@pytest.mark.parametrize("R,m,f_res", TUBES)
@pytest.mark.parametrize("storage", [0, 1])
def test_impedance_tube_field_eduction(R, m, f_res, storage):
    """A normal-incidence impedance tube on the device: the impedance educed
    from the lattice's field by the two-microphone method and in situ (probes
    at rows 1..3) matches the imposed R + i (w m - K / w). The resistance to 3 %
    up to w = 0.1; the whole Z to 1.5 w rho c + 0.01 rho c (two-microphone) and
    2.5 w rho c + 0.01 rho c (in situ), the first-order error of the coupling
    (the wall is driven by the pressure one cell into the fluid, one step
    before the velocity it imposes). A coupling with the wrong sign, a wrong
    population or no velocity at all gives a resistance off by far more
    (|G| > 1, or G = 1)."""
    tp = imp.TubeParams(R * imp.CS, m, f_res)
    r = imp.run_impedance_tube(tp, storage)
    w = r["omegas"]
    Zm, Z2, Zi = r["model"], r["two_mic"], r["insitu"]
    print("model", Zm, "two-mic", Z2, "in situ", Zi)
    low = w <= 0.1
    assert np.all(np.abs(Z2.real[low] - Zm.real[low]) <= 0.03 * Zm.real[low])
    assert np.all(np.abs(Z2 - Zm) <= (1.5 * w + 0.01) * imp.CS)
    assert np.all(np.abs(Zi - Zm) <= (2.5 * w + 0.01) * imp.CS)
