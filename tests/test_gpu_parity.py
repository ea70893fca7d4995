"""GPU parity: the CUDA engine (through its C ABI) against the oracle and
against fixtures made by lbc itself. FP64 storage must match bit for bit
(NaN at solids and signed zeros aside); forces, which lbc sums with OpenMP
atomics in no fixed order, to 1e-12 relative."""
import ctypes as C
import os

import numpy as np
import pytest

import casezoo
from conftest import GOLDEN, maxrel, same
from lbc_gb300 import cases
from lbc_gb300.abi import dptr, iptr
from lbc_gb300.cases import Q

pytestmark = pytest.mark.gpu
NAMES = [n for n, _, _ in casezoo.standard_cases()]
FIELDS = ("f", "f_new", "rho", "u", "v")


def force_close(a, b, rtol=1e-12, scale=None):
    """|a - b| <= rtol * scale; scale defaults to the largest |b| (pass the
    force magnitude for a component that is only round-off, like the lift of
    a symmetric flow)."""
    a, b = np.asarray(a), np.asarray(b)
    if not b.size:
        return True
    if scale is None:
        scale = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) <= rtol * max(scale, 1e-300)


def gross_force(case):
    """Sum of |c_k| (f_k + f_opp) over all wall links, bounded by 0.5 per link:
    the scale of the round-off in a force summed over the links in another
    order (the net lift of a symmetric flow is pure cancellation)."""
    m = case.solid_mask.astype(bool)
    n = 0
    for k in range(1, 9):
        nb = np.roll(np.roll(m, -int(case.cy[k]), axis=0), -int(case.cx[k]), axis=1)
        n += int(np.sum(~m & nb))
    return 0.5 * max(n, 1)


def fixture(name):
    return np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))


@pytest.mark.parametrize("staged", [False, True])
@pytest.mark.parametrize("name", NAMES)
def test_dropin_main_lbm_matches_lbc(gpu, oracle, name, staged):
    """lbc's main_lbm, called step by step with host arrays, as a case main does;
    both the direct path (kernels read and write the host arrays) and the
    staged path (copies)."""
    import lbc_gb300
    lib = lbc_gb300.load_library()
    lib.lbm_gpu_dropin_set_staged(1 if staged else 0)
    lib.lbm_gpu_dropin_release()
    (case, st), steps = casezoo.build(name)
    st_o = st.copy()
    fg = gpu.run(case, st, steps, record_forces=True)
    lib.lbm_gpu_dropin_set_staged(0)
    fo = oracle.run(case, st_o, steps, record_forces=True)
    g = fixture(name)
    for fld in FIELDS:
        assert same(getattr(st, fld), getattr(st_o, fld)), (name, fld, maxrel(getattr(st, fld), getattr(st_o, fld)))
        assert same(getattr(st, fld), g[fld]), (name, fld)
    mag = gross_force(case)
    assert force_close(fg, fo, scale=mag) and force_close(fg, g["forces"], scale=mag), name


@pytest.mark.parametrize("name", NAMES)
def test_resident_run_matches_lbc(oracle, name):
    """lbm_gpu_run(n): n steps on the device (graph-captured loop) leave what n
    main_lbm calls leave."""
    from lbc_gb300 import F64, GpuSolver
    (case, st), steps = casezoo.build(name)
    s = GpuSolver(case, F64)
    hist = s.info().has_geometry
    try:
        s.enable_force_history(steps)
    except RuntimeError:
        hist = False
    s.set_state(st)
    s.run(steps)
    out = s.get_state()
    fo = oracle.run(case, st, steps, record_forces=True)
    for fld in FIELDS:
        assert same(getattr(out, fld), getattr(st, fld)), (name, fld, maxrel(getattr(out, fld), getattr(st, fld)))
    if hist:
        h = s.force_history(steps)
        assert h.shape[0] == steps
        mag = gross_force(case)
        assert force_close(h[:, 0], fo[:, 1], scale=mag) and force_close(h[:, 1], fo[:, 0], scale=mag)


@pytest.mark.parametrize("storage", ["f64", "f32"])
@pytest.mark.parametrize("name", ["zoo_ibb", "cylinder_wake_small", "zoo_zh_mixed", "poiseuille"])
def test_last_force_without_a_history(oracle, name, storage):
    """Without a force history only a run's last step reduces the wall force:
    lbm_gpu_forces after run(n) is the force of the n-th main_lbm call (FP64
    to the link-sum tolerance, FP32-shifted within 1e-4 of the gross link sum)."""
    from lbc_gb300 import STORAGE, GpuSolver
    (case, st), steps = casezoo.build(name)
    s = GpuSolver(case, STORAGE[storage])
    s.set_state(st)
    s.run(steps // 2)
    s.run(steps - steps // 2)
    L, D = s.forces()
    fo = oracle.run(case, st, steps, record_forces=True)
    mag = gross_force(case)
    if storage == "f64":
        assert force_close(np.array([D]), fo[-1:, 1], scale=mag) and force_close(np.array([L]), fo[-1:, 0], scale=mag)
    else:
        assert abs(D - fo[-1, 1]) <= 1e-4 * mag and abs(L - fo[-1, 0]) <= 1e-4 * mag, (D, L, fo[-1], mag)


@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
@pytest.mark.parametrize("name", ["zoo_ibb", "zoo_convective_chain", "taylor_green", "zoo_open_edges",
                                  "taylor_green_odd", "cylinder_odd", "zoo_moving_lid"])
def test_chunked_runs_and_block_shapes_agree(name, storage):
    """run(a); run(b) == run(a + b) bit for bit, and the result does not
    depend on the thread-block shape (no races between nodes)."""
    from lbc_gb300 import STORAGE, GpuSolver
    (case, st), steps = casezoo.build(name)
    ref = None
    for bx, by, chunks in [(64, 4, [steps]), (32, 8, [7, steps - 7]), (128, 2, [1, 2, steps - 3]),
                           (256, 1, [steps - 1, 1])]:
        s = GpuSolver(case, STORAGE[storage])
        s.set_block(bx, by)
        s.set_state(st)
        for c in chunks:
            s.run(c)
        out = s.get_state()
        if ref is None:
            ref = out
        else:
            for fld in FIELDS:
                assert same(getattr(out, fld), getattr(ref, fld)), (name, storage, bx, by, chunks, fld)


def test_moving_wall_matches_oracle(oracle):
    """Moving-wall bounce-back (an extension, the lid of the cavity
    configuration): a resident FP64 run is bit-identical to the oracle's
    restatement (ext_main_lbm_moving), forces to the link-sum tolerance."""
    from lbc_gb300 import F64, GpuSolver
    (case, st), steps = casezoo.build("zoo_moving_lid")
    s = GpuSolver(case, F64)
    s.enable_force_history(steps)
    s.set_state(st)
    s.run(steps)
    out = s.get_state()
    fo = oracle.run(case, st, steps, record_forces=True)
    for fld in FIELDS:
        assert same(getattr(out, fld), getattr(st, fld)), (fld, maxrel(getattr(out, fld), getattr(st, fld)))
    h = s.force_history(steps)
    mag = gross_force(case)
    assert force_close(h[:, 0], fo[:, 1], scale=mag) and force_close(h[:, 1], fo[:, 0], scale=mag)


@pytest.mark.parametrize("storage", ["f64", "f32", "f64fma"])
def test_corrected_bottom_zou_he_matches_oracle(oracle, storage):
    """velocity_bottom_corrected (an extension: the Zou-He bottom closure
    written to population 6) beside lbc's BCs and an obstacle: FP64 resident
    runs bit-identical to the oracle's restatement, forces to the link-sum
    tolerance; the FMA form within 1e-12; FP32-shifted within 1e-5."""
    from lbc_gb300 import STORAGE, GpuSolver
    (case, st), steps = casezoo.build("zoo_zh_corrected")
    s = GpuSolver(case, STORAGE[storage])
    s.enable_force_history(steps)
    s.set_state(st)
    s.run(steps)
    out = s.get_state()
    h = s.force_history(steps)
    fo = oracle.run(case, st, steps, record_forces=True)
    fl = case.solid_mask == 0
    mag = gross_force(case)
    if storage == "f64":
        for fld in FIELDS:
            assert same(getattr(out, fld), getattr(st, fld)), (fld, maxrel(getattr(out, fld), getattr(st, fld)))
        assert force_close(h[:, 0], fo[:, 1], scale=mag) and force_close(h[:, 1], fo[:, 0], scale=mag)
    elif storage == "f64fma":
        for fld in ("rho", "u", "v"):
            a, b = getattr(out, fld)[fl], getattr(st, fld)[fl]
            assert np.max(np.abs(a - b)) <= 1e-12 * max(np.max(np.abs(b)), 1e-3), fld
        assert force_close(h[:, 0], fo[:, 1], rtol=1e-12, scale=mag)
    else:
        assert np.max(np.abs(out.u[fl] - st.u[fl])) < 1e-5
        assert np.max(np.abs(out.rho[fl] - st.rho[fl])) < 1e-5


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_corrected_bottom_zou_he_couette_on_the_device(storage):
    """The corrected closure on the device settles plane Couette flow on the
    linear profile (FP64 to round-off, FP32-shifted to its storage
    precision) and keeps the density at 1."""
    from lbc_gb300 import STORAGE, GpuSolver
    from lbc_gb300 import cases as lc
    U, Ny = 0.05, 12
    case, st = lc.couette_zh(16, Ny, 0.8, U)
    s = GpuSolver(case, STORAGE[storage])
    s.set_state(st)
    s.run(4000)
    rho, u, v = s.get_fields()
    lin = U * (1.0 - np.arange(Ny) / (Ny - 1))
    tol = 1e-10 if storage == "f64" else 1e-5
    assert np.max(np.abs(u - lin[:, None])) <= tol * U * (1 if storage == "f64" else 20)
    assert np.max(np.abs(rho - 1.0)) <= (1e-9 if storage == "f64" else 1e-5)


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_set_bc_values_between_runs(oracle, storage):
    """lbm_gpu_set_bc_values between two resident runs acts from the next step,
    as a case main that rewrites a Boundary entry's val1 between main_lbm calls
    (cases/nit/nit.c:276-303 rewrites its wall values every step). FP64:
    bit-identical to the oracle given the same values; FP32: within 1e-5 of
    it, while the new inlet moves the flow far more than that."""
    import dataclasses

    from lbc_gb300 import STORAGE, GpuSolver
    (case, st), _ = casezoo.build("cylinder_wake_small")
    inlet = case.bcs[0]
    case2 = dataclasses.replace(case, bcs=[dataclasses.replace(inlet, val1=inlet.val1 * 1.25)] + case.bcs[1:])
    s = GpuSolver(case, STORAGE[storage])
    s.set_state(st)
    s.run(20)
    s.set_bc_values(0, case2.bcs[0].val1)
    s.run(30)
    out = s.get_state()
    with pytest.raises(RuntimeError):
        s.set_bc_values(len(case.bcs), case2.bcs[0].val1)
    s.close()
    st_same = st.copy()
    oracle.run(case, st, 20)
    oracle.run(case2, st, 30)
    oracle.run(case, st_same, 50)
    if storage == "f64":
        for fld in FIELDS:
            assert same(getattr(out, fld), getattr(st, fld)), (fld, maxrel(getattr(out, fld), getattr(st, fld)))
    else:
        fluid = case.solid_mask == 0
        err = max(float(np.max(np.abs(getattr(out, c)[fluid] - getattr(st, c)[fluid]))) for c in ("u", "v"))
        moved = float(np.max(np.abs(st.u[fluid] - st_same.u[fluid])))
        assert err < 1e-5 and moved > 100 * err, (err, moved)


def test_cylinder_golden_forces_on_gpu():
    """lbc's shipped drag history (1000 x 400, IBB, Zou-He inlet, convective
    outlet, periodic y): the first 300 steps."""
    from lbc_gb300 import F64, GpuSolver
    g = np.load(os.path.join(GOLDEN, "lbc_cylinder_forces_res20_first300.npy"))
    case, st, cf = cases.cylinder_golden()
    s = GpuSolver(case, F64)
    s.enable_force_history(300)
    s.set_state(st)
    s.run(300)
    h = s.force_history(300)
    D, L = h[:, 0] * cf, h[:, 1] * cf
    assert np.max(np.abs(D - g[:, 2]) / np.abs(g[:, 2])) < 1e-13
    assert np.max(np.abs(L - g[:, 1])) < 1e-9 * np.max(np.abs(g[:, 2]))


def test_force_records_stream_lbc_format(tmp_path):
    """lbm_gpu_write_force_records writes lbc's {t, L, D} record file
    (cases/cylinder/cylinder.c:162-185) from the device's force ring, drained
    twice during the run: times bit for bit and forces as lbc's shipped record
    of the first 300 steps. A ring drained too late loses its oldest steps and
    says so, after writing the ones it still holds."""
    from lbc_gb300 import F64, GpuSolver
    g = np.load(os.path.join(GOLDEN, "lbc_cylinder_forces_res20_first300.npy"))
    case, st, cf = cases.cylinder_golden()
    dt = float(g[1, 0])
    path = str(tmp_path / "forces.bin")
    s = GpuSolver(case, F64)
    s.enable_force_history(200)
    s.set_state(st)
    s.run(120)
    assert s.write_force_records(path, dt, cf) == 120
    s.run(180)
    assert s.write_force_records(path, dt, cf, append=True) == 180
    rec = np.fromfile(path, dtype=np.float64).reshape(-1, 3)
    assert rec.shape == (300, 3) and same(rec[:, 0], g[:, 0])
    assert np.max(np.abs(rec[:, 2] - g[:, 2]) / np.abs(g[:, 2])) < 1e-13
    assert np.max(np.abs(rec[:, 1] - g[:, 1])) < 1e-9 * np.max(np.abs(g[:, 2]))
    s.run(250)
    with pytest.raises(RuntimeError):
        s.write_force_records(path, dt, cf, append=True)
    rec = np.fromfile(path, dtype=np.float64).reshape(-1, 3)
    assert rec.shape == (500, 3) and rec[300, 0] == 350 * dt


def _bc_call(lib, case, st, b):
    arr, keep = lib.boundaries([b])
    getattr(lib, b.name)(case.Nx, case.Ny, Q, b.index, arr[0].val1, arr[0].val2, dptr(st.f),
                         dptr(st.f_new), dptr(st.rho), dptr(st.u), dptr(st.v),
                         iptr(case.solid_mask), iptr(case.cx), iptr(case.cy), dptr(case.w))


@pytest.mark.parametrize("name", ["zoo_zh_mixed", "zoo_pressure_reg", "zoo_reg_periodic",
                                  "zoo_periodic_late", "zoo_ibb", "zoo_convective_chain",
                                  "all_regularized_box", "cavity_zouhe"])
def test_standalone_functions_match_lbc(gpu, oracle, name):
    """Each of lbc's functions called on its own (lbm_core.h, lbm_bc.h)."""
    (case, st0), _ = casezoo.build(name)
    for b in case.bcs:
        a, r = st0.copy(), st0.copy()
        _bc_call(gpu, case, a, b)
        _bc_call(oracle, case, r, b)
        assert same(a.f_new, r.f_new), (name, b.name)
    outs = []
    for lib in (gpu, oracle):
        st = st0.copy()
        args = (case.Nx, case.Ny, Q)
        lib.collision(*args, dptr(st.f), dptr(st.rho), dptr(st.u), dptr(st.v), dptr(case.omega_eff),
                      iptr(case.solid_mask), iptr(case.cx), iptr(case.cy), dptr(case.w), 1e-5, -2e-6)
        st2 = st.copy()
        lib.bounce_back(*args, dptr(st.f), dptr(st.f_new), iptr(case.solid_mask), iptr(case.cx),
                        iptr(case.cy), iptr(case.opp), case.isperiodic_x, case.isperiodic_y)
        phi = case.phi if case.use_IBB else np.sqrt(np.abs(case.phi) + 0.3) - 0.1 * case.solid_mask
        phi = np.ascontiguousarray(phi)
        lib.interpolated_bounce_back(*args, dptr(st2.f), dptr(st2.f_new), iptr(case.solid_mask), dptr(phi),
                                     iptr(case.opp), iptr(case.cx), iptr(case.cy), case.isperiodic_x,
                                     case.isperiodic_y)
        Fx, Fy = C.c_double(), C.c_double()
        lib.compute_force_mem(*args, dptr(st.f), dptr(st.f_new), iptr(case.solid_mask), case.isperiodic_x,
                              case.isperiodic_y, iptr(case.cx), iptr(case.cy), iptr(case.opp),
                              C.byref(Fx), C.byref(Fy))
        lib.streaming(*args, dptr(st.f), dptr(st.f_new), iptr(case.solid_mask), iptr(case.cx),
                      iptr(case.cy), case.isperiodic_x, case.isperiodic_y)
        lib.compute_macroscopic_fields(*args, dptr(st.f_new), iptr(case.solid_mask), iptr(case.cx),
                                       iptr(case.cy), dptr(st.rho), dptr(st.u), dptr(st.v), 1e-5, 0.0)
        outs.append((st, st2, Fx.value, Fy.value))
    (a, a2, ax, ay), (b, b2, bx, by) = outs
    for fld in FIELDS:
        assert same(getattr(a, fld), getattr(b, fld)), (name, fld)
    assert same(a2.f_new, b2.f_new), name
    assert force_close([ax, ay], [bx, by], scale=gross_force(case))


def test_mei_initialization_matches_lbc(gpu, oracle):
    case, _ = cases.taylor_green(40, 24, 0.04, 0.6)
    rng = np.random.default_rng(3)
    rho_in = 1.0 + 1e-3 * rng.standard_normal((case.Ny, case.Nx))
    U = 0.02 * rng.standard_normal((case.Ny, case.Nx))
    V = 0.02 * rng.standard_normal((case.Ny, case.Nx))
    mask = case.solid_mask.copy()
    mask[5:9, 10:14] = 1
    res = []
    for lib in (gpu, oracle):
        fn = getattr(lib.lib, lib.prefix + "mei_initialization")
        fn.restype = None
        f = np.zeros((case.Ny, case.Nx, Q))
        fnew = np.full((case.Ny, case.Nx, Q), 0.1)
        rho, u, v = (np.zeros((case.Ny, case.Nx)) for _ in range(3))
        fn(C.c_int(case.Nx), C.c_int(case.Ny), C.c_int(Q), dptr(f), dptr(fnew), dptr(rho_in), dptr(U),
           dptr(V), dptr(rho), dptr(u), dptr(v), iptr(case.cx), iptr(case.cy), dptr(case.w),
           dptr(case.omega_eff), C.c_int(1), C.c_int(1), C.c_int(7), C.c_double(1e-16), iptr(mask))
        res.append((f, fnew, rho, u, v))
    for x, y in zip(*res):
        assert same(x, y)


@pytest.mark.parametrize("storage,tol", [("f32", 2e-6), ("f16", 2e-3)])
def test_shifted_storage_error_vs_fp64(oracle, storage, tol):
    """Taylor-Green 128 x 128, u0 = 0.04, tau = 0.56, 200 steps: relative L2
    error of u against the FP64 oracle (the FP32 accuracy target is 1e-5)."""
    from lbc_gb300 import STORAGE, GpuSolver
    case, st = cases.taylor_green(128, 128, 0.04, 0.56)
    s = GpuSolver(case, STORAGE[storage])
    s.set_state(st)
    s.run(200)
    rho, u, v = s.get_fields()
    oracle.run(case, st, 200)
    err = np.sqrt(np.sum((u - st.u) ** 2 + (v - st.v) ** 2) / np.sum(st.u ** 2 + st.v ** 2))
    print(f"{storage}: u L2 rel error {err:.3e}")
    assert err < tol


@pytest.mark.parametrize("name", ["zoo_ibb", "zoo_convective_chain", "zoo_zh_mixed", "cylinder_wake_small"])
def test_shifted_storage_on_edge_bcs(oracle, name):
    """FP32-shifted storage through every edge BC path stays close to FP64."""
    from lbc_gb300 import F32_SHIFTED, GpuSolver
    (case, st), steps = casezoo.build(name)
    s = GpuSolver(case, F32_SHIFTED)
    s.set_state(st)
    s.run(steps)
    rho, u, v = s.get_fields()
    oracle.run(case, st, steps)
    fl = case.solid_mask == 0
    assert np.max(np.abs(u[fl] - st.u[fl])) < 1e-5
    assert np.max(np.abs(rho[fl] - st.rho[fl])) < 1e-5


def test_dropin_main_lbm_with_a_user_bc_matches_lbc(gpu, oracle):
    """A Boundary list that holds a function of the caller's own: main_lbm runs
    lbc's sequence from the standalone device functions and calls the
    caller's function on the host arrays in its place in the list. Fields
    bit-identical to the oracle's main_lbm with the same callback, forces to
    the link-sum tolerance."""
    from test_capi import _host_outflow_bc
    (case, st), _ = casezoo.build("cylinder_wake_small")
    calls = []
    cb = _host_outflow_bc(calls)
    outs = []
    for lib in (gpu, oracle):
        s = st.copy()
        arr, keep = lib.boundaries(case.bcs)
        arr[1].apply = C.cast(cb, C.c_void_p).value
        forces = [lib.step(case, s, bnd=(arr, keep)) for _ in range(12)]
        outs.append((s, np.array(forces)))
    (a, fa), (b, fb) = outs
    assert calls == [case.Nx - 1] * 24
    for fld in FIELDS:
        assert same(getattr(a, fld), getattr(b, fld)), (fld, maxrel(getattr(a, fld), getattr(b, fld)))
    assert force_close(fa, fb, scale=gross_force(case))


@pytest.mark.parametrize("name", ["cylinder_wake_small", "zoo_convective_chain", "taylor_green_odd"])
def test_lazy_dropin_matches_lbc(gpu, oracle, name):
    """lbm_gpu_dropin_set_lazy(1): main_lbm calls that follow the caller's swap
    continue on the device and leave the caller's arrays untouched; *L and *D
    arrive every call. lbm_gpu_dropin_sync (and switching lazy off) writes what
    lbc leaves, bit for bit, whereupon the calls go on as usual."""
    import lbc_gb300
    lib = lbc_gb300.load_library()
    (case, st), steps = casezoo.build(name)
    st_o = st.copy()
    half = steps // 2
    lib.lbm_gpu_dropin_release()
    lib.lbm_gpu_dropin_set_lazy(1)
    try:
        rho0 = st.rho.copy()
        fg1 = gpu.run(case, st, half, record_forces=True)
        assert same(st.rho, rho0)                    # still on the device
        assert lib.lbm_gpu_dropin_sync() == 0
        fo1 = oracle.run(case, st_o, half, record_forces=True)
        for fld in FIELDS:
            assert same(getattr(st, fld), getattr(st_o, fld)), (name, fld)
        fg2 = gpu.run(case, st, steps - half, record_forces=True)
    finally:
        lib.lbm_gpu_dropin_set_lazy(0)                # writes the pending result back
    fo2 = oracle.run(case, st_o, steps - half, record_forces=True)
    for fld in FIELDS:
        assert same(getattr(st, fld), getattr(st_o, fld)), (name, fld)
    mag = gross_force(case)
    assert force_close(np.concatenate([fg1, fg2]), np.concatenate([fo1, fo2]), scale=mag)


@pytest.mark.parametrize("args", [(60, 40, 0.5, 15.0, 10.0, 5.0, 12.0, 0.6, 3.0, 0.4),
                                  (2048, 512, 1.0, 512.0, 256.0, 300.0, 700.0, 0.55, 5.0, 0.01)])
def test_sponge_layer_on_the_device(gpu, oracle, args):
    """lbc's sponge_layer (src/core/sponge_layer.c:3-45) filled by a device
    kernel: nodes inside r_inner and outside r_outer are lbc's bits; the ramp
    between uses CUDA's exp, so it agrees to 1e-14 relative, well inside the
    1e-12 the FP64 path is held to."""
    Nx, Ny = args[0], args[1]
    dx, xc, yc, ri, ro = args[2:7]
    got = np.full((Ny, Nx), np.nan)
    want = np.zeros((Ny, Nx))
    gpu.sponge_layer(*args, dptr(got))
    oracle.sponge_layer(*args, dptr(want))
    j, i = np.mgrid[0:Ny, 0:Nx]
    r = np.sqrt((i * dx - xc) ** 2 + (j * dx - yc) ** 2)
    flat = (r <= ri) | (r > ro)
    assert same(got[flat], want[flat])
    assert np.max(np.abs(got - want) / np.abs(want)) <= 1e-14
    assert (~flat).sum() > 100
