"""Per-step records on the device: probes (rho and velocity at chosen nodes
after every step) and the impedance wall's trace written in lbc's text format
(cases/nit/nit.c:262-273). Probes are checked against the oracle's fields after
each step, alone and in a batch; the trace against the oracle's host coupling
of the same wall."""
import ctypes as C
import math
import os

import numpy as np
import pytest

import casezoo
from conftest import same
from lbc_gb300 import impedance as imp
from lbc_gb300.abi import dptr, iptr

pytestmark = pytest.mark.gpu


def _nodes(case, k=7, seed=3):
    rng = np.random.default_rng(seed)
    fl = np.argwhere(case.solid_mask == 0)
    pick = fl[rng.choice(len(fl), size=min(k, len(fl)), replace=False)]
    return [(int(ji[1]), int(ji[0])) for ji in pick]


@pytest.mark.parametrize("name,storage", [("zoo_open_edges", 0), ("cylinder_wake_small", 0), ("zoo_ibb", 0),
                                          ("cylinder_wake_small", 1)])
def test_probes_follow_the_oracle_step_by_step(oracle, name, storage):
    """Probe q at step t equals the oracle's rho, u, v at that node after t + 1
    main_lbm calls (FP64: to the rounding of summing the populations in
    another order; FP32-shifted: to its storage precision)."""
    from lbc_gb300 import GpuSolver
    (case, st), _ = casezoo.build(name)
    nodes = _nodes(case)
    steps = 40
    s = GpuSolver(case, storage)
    s.set_probes(nodes, steps)
    s.set_state(st)
    s.run(steps // 2)      # two runs: the first step of a run collides with the stored fields
    s.run(steps - steps // 2)
    h = s.probe_history(steps)
    assert h.shape == (steps, len(nodes), 3)
    bnd = oracle.boundaries(case.bcs)
    tol = 1e-13 if storage == 0 else 2e-5
    for t in range(steps):
        oracle.step(case, st, bnd)
        for q, (i, j) in enumerate(nodes):
            want = np.array([st.rho[j, i], st.u[j, i], st.v[j, i]])
            assert np.all(np.abs(h[t, q] - want) <= tol * np.maximum(1.0, np.abs(want))), (t, q, h[t, q], want)


def test_probes_in_a_batch_equal_alone():
    from lbc_gb300 import GpuBatch, GpuSolver
    names = ["zoo_ibb", "taylor_green", "cylinder_wake_small"]
    built = [casezoo.build(n)[0] for n in names]
    alone = []
    for case, st in built:
        s = GpuSolver(case, 1)
        s.set_probes(_nodes(case), 64)
        s.set_state(st)
        s.run(30)
        alone.append(s.probe_history(64))
        s.close()
    solvers = []
    for case, st in built:
        s = GpuSolver(case, 1)
        s.set_probes(_nodes(case), 64)
        s.set_state(st)
        solvers.append(s)
    b = GpuBatch(solvers)
    b.run(30)
    for s, a, n in zip(solvers, alone, names):
        assert same(s.probe_history(64), a), n
    b.close()


def test_probe_ring_keeps_the_last_capacity_steps():
    from lbc_gb300 import GpuSolver
    (case, st), _ = casezoo.build("taylor_green")
    nodes = _nodes(case, 3)
    a = GpuSolver(case, 0)
    a.set_probes(nodes, 100)
    a.set_state(st)
    a.run(50)
    b = GpuSolver(case, 0)
    b.set_probes(nodes, 16)
    b.set_state(st)
    b.run(50)
    assert same(b.probe_history(100), a.probe_history(100)[-16:])
    with pytest.raises(RuntimeError):
        b.set_probes([(case.Nx, 0)], 8)


def _imp_array(p, omegas, Nx, oi_n=12):
    """Impedance-wall state in the oracle's layout for a liner."""
    import lbc_gb300
    R, m, K = imp.liner_arrays(p)
    nf = len(omegas)
    a = np.zeros((oi_n + 6 * nf, Nx))
    for t in range(Nx):
        if m[t] <= 0:
            continue
        A, b = np.zeros(4), np.zeros(2)
        assert lbc_gb300.load_library().lbm_gpu_msd_zoh(R[t], m[t], K[t], dptr(A), dptr(b)) == 0
        a[0, t] = 1.0
        a[1:5, t] = A
        a[5:7, t] = b
        a[9, t] = 1.0   # mean density starts at rho_ref
        a[10, t] = 1.0  # window phasor cos
        for f in range(nf):
            a[oi_n + 6 * f, t] = 1.0
    return a


def test_impedance_trace_in_lbc_format(oracle, tmp_path):
    """The liner's per-step mean p' and v against the oracle's host coupling
    of the same wall (FP64), streamed in two parts to lbc's text format."""
    from lbc_gb300 import GpuSolver
    p = imp.LinerParams(nx=160, ny=24, mach=0.15, R=1.2 * imp.CS, m=5e-3, f_res=0.05)
    case, st = imp.liner_duct(p)
    om = imp.EDUCTION_OMEGAS
    R, m, K = imp.liner_arrays(p)
    s = GpuSolver(case, 0)
    s.set_impedance_wall(imp.LINER_ENTRY, R, m, K, om, 1.0, 2e-3, 400)
    s.enable_impedance_trace(imp.LINER_ENTRY, 64)
    s.set_state(st)
    path = str(tmp_path / "tdibc.txt")
    dt, cp, cu = 1e-5, 1e3, 1e3
    s.run(60)
    assert s.write_impedance_trace(imp.LINER_ENTRY, path, dt, cp, cu) == 61   # the zero line, then 60 steps
    s.run(50)
    assert s.write_impedance_trace(imp.LINER_ENTRY, path, dt, cp, cu, append=True) == 50
    lines = open(path).read().splitlines()
    assert len(lines) == 111 and lines[0] == "0.000000 0.000000 0.000000"
    got = np.array([[float(x) for x in ln.split()] for ln in lines])
    # the oracle's coupling, step by step: mean over active nodes of the p'
    # each node was driven with and of the velocity it imposed
    impa = _imp_array(p, om, case.Nx)
    cw, sw = np.cos(om), np.sin(om)
    step_fn = oracle.lib.orc_ext_impedance_step
    step_fn.restype = None
    act = impa[0] != 0.0
    v2 = np.zeros(case.Nx)
    want = [(0.0, 0.0, 0.0)]
    for n in range(110):
        pbar = float(np.mean((st.rho[1, act] - impa[9, act]) / 3.0))
        step_fn(C.c_int(case.Nx), C.c_int(0), dptr(st.rho), C.c_double(2e-3), dptr(impa), C.c_int(len(om)),
                dptr(cw), dptr(sw), C.c_double(math.cos(2 * math.pi / 400)), C.c_double(math.sin(2 * math.pi / 400)),
                C.c_int(1), iptr(case.solid_mask), None, dptr(v2))
        vbar = float(np.mean(impa[8, act]))
        want.append(((n + 1) * dt, pbar * cp, vbar * cu))
        bcs = list(case.bcs)
        bcs[imp.LINER_ENTRY] = imp.BC("velocity_bottom_regularized", 0, bcs[imp.LINER_ENTRY].val1, v2.copy())
        oracle.step(imp.Case(case.name, case.Nx, case.Ny, case.solid_mask, case.omega_eff, case.phi, bcs), st)
    want = np.array(want)
    assert np.all(np.abs(got - want) <= 1e-6 + 1e-9 * np.abs(want)), np.max(np.abs(got - want))
    assert np.max(np.abs(want[:, 1])) > 1e-3   # the pulse reaches the liner: a trace with content
    os.remove(path)
