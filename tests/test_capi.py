"""The C ABI without a GPU: the library builds, loads and exports every
function include/*.h declares; the headers compile as C and C++; lbc's own
case mains compile against them; without a device, calls fail loudly and
leave the caller's arrays untouched (no CPU fallback)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT

INCLUDE = os.path.join(ROOT, "include")
def _ref_source():
    """lbc's source tree: $LBC_REF, else the one oracle/build_ref.sh built from."""
    if os.environ.get("LBC_REF"):
        return os.environ["LBC_REF"]
    try:
        with open(os.path.join(ROOT, "oracle", "_ref", "SOURCE")) as fh:
            return fh.read().strip()
    except OSError:
        return ""


REF = _ref_source()


def declared_functions():
    names = set()
    for h in os.listdir(INCLUDE):
        if not h.endswith(".h"):
            continue
        txt = open(os.path.join(INCLUDE, h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"#define[^\n]*(\\\n[^\n]*)*", "", txt)
        for m in re.finditer(r"^\s*(?:const\s+)?(?:void|int|char|double)\s*\*?\s*(\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    from lbc_gb300 import build
    path = build.build()
    return C.CDLL(path)


def test_exports_every_declared_function(lib):
    names = declared_functions()
    # lbc's 7 core + 20 BC + 2 util functions are all in the set
    for n in ("main_lbm", "collision", "streaming", "compute_macroscopic_fields", "compute_force_mem",
              "mei_initialization", "sponge_layer", "bounce_back", "interpolated_bounce_back",
              "velocity_bottom_regularized", "pressure_top_regularized", "write_vtk_binary_2D",
              "ensure_directory_exists", "lbm_gpu_create", "lbm_gpu_run"):
        assert n in names, n
    assert len(names) >= 29 + 15
    for n in sorted(names):
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"


def test_headers_compile_as_c_and_cpp():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        open(src, "w").write('#include "lbm.h"\n#include "lbm_gpu.h"\n'
                             'int main(void){Boundary b[1]; b[0].apply = periodic_x; (void)b; return 0;}\n')
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I", INCLUDE, src], check=True)
        cpp = os.path.join(d, "t.cpp")
        open(cpp, "w").write('#include "lbm.h"\n#include "lbm_gpu.h"\n'
                             'int main(){Boundary b[1]; b[0].apply = periodic_x; (void)b; return 0;}\n')
        subprocess.run(["g++", "-Wall", "-Werror", "-fsyntax-only", "-I", INCLUDE, cpp], check=True)


@pytest.mark.parametrize("case", ["nit", "testbc"])
def test_lbc_case_mains_compile_against_headers(case):
    """lbc's case mains that build against lbc's current API also build,
    warning-free, against these headers (drop-in at the source level)."""
    path = os.path.join(REF, "cases", case, f"{case}.c")
    if not os.path.exists(path):
        pytest.skip("lbc sources not present")
    subprocess.run(["gcc", "-std=gnu99", "-Wall", "-Werror", "-fsyntax-only", "-I", INCLUDE, path], check=True)


def test_no_device_fails_loudly(lib):
    import lbc_gb300
    lbc_gb300.load_library()
    if lib.lbm_gpu_device_count() > 0:
        pytest.skip("a GPU is visible; covered by the gpu tests")
    from lbc_gb300 import cases
    api = lbc_gb300.dropin()
    case, st = cases.poiseuille(16, 8)
    before = st.copy()
    api.step(case, st, swap=False)
    assert np.array_equal(st.f, before.f) and np.array_equal(st.rho, before.rho)
    assert lbc_gb300.last_error() != ""


def _host_outflow_bc(calls):
    """A Boundary function of the caller's own (not one of lbc's): copies the
    populations of column index - 1 into column index."""
    BCFN = C.CFUNCTYPE(None, *([C.c_int] * 4 + [C.c_void_p] * 11))

    def outflow(Nx, Ny, Q, index, val1, val2, f, f_new, rho, u, v, mask, cx, cy, w):
        calls.append(index)
        fn = np.ctypeslib.as_array(C.cast(f_new, C.POINTER(C.c_double)), shape=(Ny, Nx, Q))
        fn[:, index, :] = fn[:, index - 1, :]

    return BCFN(outflow)


def test_user_bc_without_device_fails_loudly(lib):
    """A main_lbm call whose Boundary list holds a function of the caller's own
    fails before anything runs when there is no device: the caller's arrays
    are untouched and the callback is never reached."""
    import lbc_gb300
    if lib.lbm_gpu_device_count() > 0:
        pytest.skip("a GPU is visible; covered by the gpu tests")
    from lbc_gb300 import cases
    api = lbc_gb300.dropin()
    case, st = cases.cylinder_wake(48, 16, D=4, xc=12, yc=8)
    calls = []
    cb = _host_outflow_bc(calls)
    arr, keep = api.boundaries(case.bcs)
    arr[1].apply = C.cast(cb, C.c_void_p).value
    before = st.copy()
    api.step(case, st, bnd=(arr, keep), swap=False)
    assert np.array_equal(st.f, before.f) and np.array_equal(st.f_new, before.f_new)
    assert calls == [] and lbc_gb300.last_error() != ""


def test_entry_points_reject_bad_arguments_on_the_host(lib):
    """Argument checks that need no device: a null solver or batch, a pending
    lazy result that does not exist, an unknown Boundary entry."""
    import lbc_gb300
    api = lbc_gb300.load_library()       # the bound signatures
    ERR_ARG = -1
    assert api.lbm_gpu_write_force_records(None, b"forces.bin", 1.0, 1.0, 0) == ERR_ARG
    assert "null solver" in lbc_gb300.last_error()
    assert api.lbm_gpu_set_bc_values(None, 0, None, None) == ERR_ARG
    assert api.lbm_gpu_run(None, 1) == ERR_ARG
    assert api.lbm_gpu_batch_run(None, 1) == ERR_ARG
    assert api.lbm_gpu_dropin_sync() == 0          # nothing pending: nothing to write
    api.lbm_gpu_dropin_set_lazy(1)
    api.lbm_gpu_dropin_set_lazy(0)
    assert api.lbm_gpu_dropin_sync() == 0
