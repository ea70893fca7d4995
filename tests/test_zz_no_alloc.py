"""lbm_gpu_compute_force_mem_noalloc: the momentum-exchange force on device
arrays the caller owns, for callers that cannot let a library allocate device
memory (their memory is held by their own pool, or they must not stall the
device with cudaMalloc / cudaFree). It must give what lbc's
compute_force_mem entry point gives, on every call of a sequence, since all
calls share one fixed scratch array inside the library.

Collected last on purpose (file name), so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import casezoo
from lbc_gb300.abi import dptr, iptr
from lbc_gb300.cases import Q

pytestmark = pytest.mark.gpu


def _gross(case):
    m = case.solid_mask.astype(bool)
    n = sum(int(np.sum(~m & np.roll(np.roll(m, -int(case.cy[k]), 0), -int(case.cx[k]), 1))) for k in range(1, 9))
    return 0.5 * max(n, 1)


def _expected(api, case, f, f_new):
    Fx, Fy = C.c_double(), C.c_double()
    api.compute_force_mem(case.Nx, case.Ny, Q, dptr(f), dptr(f_new), iptr(case.solid_mask), case.isperiodic_x,
                          case.isperiodic_y, iptr(case.cx), iptr(case.cy), iptr(case.opp), C.byref(Fx), C.byref(Fy))
    return np.array([Fx.value, Fy.value])


def test_force_mem_noalloc_matches_compute_force_mem():
    torch = pytest.importorskip("torch")
    import lbc_gb300
    lib = lbc_gb300.load_library()
    api = lbc_gb300.dropin()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for name in ("zoo_ibb", "cylinder_wake_small", "zoo_zh_mixed"):
        (case, st), _ = casezoo.build(name)
        tol = 1e-12 * _gross(case)
        # Two calls in a row on different inputs: the shared scratch must not
        # carry anything from one call to the next.
        for f, f_new in ((st.f, st.f_new), (st.f_new, st.f)):
            want = _expected(api, case, f, f_new)
            d_f = torch.from_numpy(np.ascontiguousarray(f)).cuda()
            d_fn = torch.from_numpy(np.ascontiguousarray(f_new)).cuda()
            d_m = torch.from_numpy(case.solid_mask).cuda()
            torch.cuda.synchronize()
            rc = lib.lbm_gpu_compute_force_mem_noalloc(case.Nx, case.Ny, Q, d_f.data_ptr(), d_fn.data_ptr(),
                                                       d_m.data_ptr(), case.isperiodic_x, case.isperiodic_y,
                                                       iptr(case.cx), iptr(case.cy), iptr(case.opp),
                                                       out.data_ptr(), stream)
            assert rc == 0, lbc_gb300.last_error()
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.max(np.abs(got - want)) <= tol, (name, got, want)


def test_force_mem_noalloc_rejects_oversized_grid():
    import lbc_gb300
    lib = lbc_gb300.load_library()
    rc = lib.lbm_gpu_compute_force_mem_noalloc(8192, 8192, Q, 1, 1, 1, 0, 0, None, None, None, 1, None)
    assert rc != 0 and "too large" in lbc_gb300.last_error()
