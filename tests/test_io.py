"""Checkpoint/restart and device-packed VTK output (GPU).

A run saved after a steps, loaded into a fresh solver of the same case and
continued for b steps ends exactly as one run of a + b steps: populations,
fields, force, force history and impedance-wall state, in every storage type.
The device-packed VTK file has the bytes of the host writer (itself lbc's
writer byte for byte, tests/test_vtk.py)."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import same
from lbc_gb300 import cases

pytestmark = pytest.mark.gpu
FIELDS = ("f", "f_new", "rho", "u", "v")


def _liner():
    from lbc_gb300 import impedance as imp
    p = imp.LinerParams(nx=200, ny=28, mach=0.2, R=1.1 * imp.CS, m=4e-3, f_res=0.06)
    return imp.liner_duct(p), p


def _make(storage, name):
    from lbc_gb300 import GpuSolver
    from lbc_gb300 import impedance as imp
    lp = None
    if name == "liner":
        (case, st), lp = _liner()
    else:
        case, st = cases.cylinder_wake(160, 48, D=10.0, xc=40.0, yc=24.0, u_max=0.05, Re=60.0, seed=5)
    s = GpuSolver(case, storage)
    if lp is not None:
        s.set_impedance_wall(imp.LINER_ENTRY, *imp.liner_arrays(lp), imp.TRACKED_OMEGAS, 1.0, imp.MEAN_RATE, 60)
    s.enable_force_history(128)
    s.set_state(st)
    return s, lp


@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
@pytest.mark.parametrize("name", ["liner", "cylinder"])
def test_checkpoint_continues_bit_for_bit(storage, name, tmp_path):
    from lbc_gb300 import STORAGE
    from lbc_gb300 import impedance as imp
    a, lp = _make(STORAGE[storage], name)
    a.run(37)
    path = str(tmp_path / "ck.bin")
    a.checkpoint_save(path)
    b, _ = _make(STORAGE[storage], name)
    b.checkpoint_load(path)
    a.run(23)
    b.run(23)
    sa, sb = a.get_state(), b.get_state()
    for fld in FIELDS:
        assert same(getattr(sa, fld), getattr(sb, fld)), (storage, name, fld)
    assert same(np.array(a.forces()), np.array(b.forces()))
    assert same(a.force_history(60), b.force_history(60))
    assert a.force_history(60).shape == (60, 2)
    if lp is not None:
        pa, xa = a.impedance_readback(imp.LINER_ENTRY)
        pb, xb = b.impedance_readback(imp.LINER_ENTRY)
        assert same(pa, pb) and same(xa, xb)


def test_checkpoint_rejects_other_cases_and_garbage(tmp_path):
    from lbc_gb300 import F32_SHIFTED, GpuSolver
    a, _ = _make(F32_SHIFTED, "cylinder")
    a.run(5)
    path = str(tmp_path / "ck.bin")
    a.checkpoint_save(path)
    case, st = cases.poiseuille(64, 16, 0.8, 1e-6)
    other = GpuSolver(case, F32_SHIFTED)
    other.set_state(st)
    with pytest.raises(RuntimeError):
        other.checkpoint_load(path)
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"not a checkpoint at all")
    with pytest.raises(RuntimeError):
        a.checkpoint_load(str(bad))
    with pytest.raises(RuntimeError):
        a.checkpoint_load(str(tmp_path / "missing.bin"))
    # A failed load leaves the solver usable.
    a.run(3)


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_device_vtk_equals_host_writer(storage, tmp_path):
    import lbc_gb300
    from lbc_gb300 import STORAGE
    s, _ = _make(STORAGE[storage], "cylinder")
    s.run(11)
    rho, u, v = s.get_fields()
    dev = tmp_path / "dev.vtk"
    s.write_vtk(str(dev), 0.5, 2.0, 3.0)
    s.run(4)          # stepping continues while the file is written
    s.sync()
    host = tmp_path / "host.vtk"
    lib = lbc_gb300.load_library()
    fn = lib.write_vtk_binary_2D
    DP = C.POINTER(C.c_double)
    fn.restype = None
    fn.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_double, DP, DP, DP, C.c_double, C.c_double]
    Ny, Nx = rho.shape
    u, v, rho = (np.ascontiguousarray(x) for x in (u, v, rho))
    fn(os.fsencode(str(host)), Nx, Ny, 0.5, u.ctypes.data_as(DP), v.ctypes.data_as(DP), rho.ctypes.data_as(DP),
       2.0, 3.0)
    assert dev.read_bytes() == host.read_bytes()
