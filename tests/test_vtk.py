"""write_vtk_binary_2D of this library (host code, no GPU) writes the bytes of
lbc's own writer (src/utils/write_vtk_binary_2D.c), checked against a file
made by lbc's build (tests/golden/lbc_small.vtk, tests/golden/make_golden.py)."""
import ctypes as C
import os
import sys

import numpy as np

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402

DP = C.POINTER(C.c_double)


def _write(lib, path, prefix=""):
    Nx, Ny, dx, cu, crho = make_golden.VTK_ARGS
    u, v, rho = make_golden.vtk_inputs()
    fn = getattr(lib, prefix + "write_vtk_binary_2D")
    fn.restype = None
    fn.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_double, DP, DP, DP, C.c_double, C.c_double]
    fn(os.fsencode(path), Nx, Ny, dx, u.ctypes.data_as(DP), v.ctypes.data_as(DP), rho.ctypes.data_as(DP), cu,
       crho)


def test_host_vtk_writer_matches_lbc_golden(tmp_path):
    import lbc_gb300
    lib = lbc_gb300.load_library()
    out = tmp_path / "ours.vtk"
    _write(lib, out)
    golden = open(os.path.join(GOLDEN, "lbc_small.vtk"), "rb").read()
    assert out.read_bytes() == golden


def test_golden_vtk_is_lbcs_writer(ref, tmp_path):
    out = tmp_path / "lbc.vtk"
    _write(ref.lib, out, "ref_")
    assert out.read_bytes() == open(os.path.join(GOLDEN, "lbc_small.vtk"), "rb").read()
