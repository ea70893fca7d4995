"""lbm_gpu_compute_force_mem_noalloc: the momentum-exchange force on device
arrays the caller owns, for callers that cannot let a library allocate device
memory (their memory is held by their own pool, or they must not stall the
device with cudaMalloc / cudaFree). It must give what lbc's compute_force_mem
gives (the oracle, a CPU restatement of lbc's function), on every call of a
sequence, since all calls share one fixed scratch array inside the library.

Checked here: calls issued back to back on one stream with no synchronisation
between them, on different inputs and into different output buffers; a grid at
the documented limit (4096 x 4096: exactly 65536 blocks, the whole scratch);
that calls after the first take no device memory; and that grids beyond the
limit are rejected with a clear error.

Collected last on purpose (file name), so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import casezoo
from lbc_gb300.abi import dptr, iptr
from lbc_gb300.cases import BC, CX, CY, OPP, Q, Case

pytestmark = pytest.mark.gpu


def _gross(case, f, f_new):
    """Sum of |f_k + f_new,opp| over the wall links (periodic neighbours): the
    scale of the rounding in any summation order of the link terms."""
    m = case.solid_mask.astype(bool)
    g = 0.0
    for k in range(1, 9):
        nb_solid = np.roll(np.roll(m, -int(CY[k]), 0), -int(CX[k]), 1)
        sel = ~m & nb_solid
        g += float(np.sum(np.abs(f[:, :, k][sel] + f_new[:, :, OPP[k]][sel])))
    return max(g, 1.0)


def _oracle_force(oracle, case, f, f_new):
    Fx, Fy = C.c_double(), C.c_double()
    oracle.compute_force_mem(case.Nx, case.Ny, Q, dptr(f), dptr(f_new), iptr(case.solid_mask),
                             case.isperiodic_x, case.isperiodic_y, iptr(case.cx), iptr(case.cy),
                             iptr(case.opp), C.byref(Fx), C.byref(Fy))
    return np.array([Fx.value, Fy.value])


def _limit_case(seed=7):
    """4096 x 4096 (64 x 4 node blocks: 64 x 1024 = 65536, the scratch limit),
    solid walls at the bottom and top rows, periodic in x, a field of seeded
    circular obstacles, random populations in both buffers."""
    N = 4096
    rng = np.random.default_rng(seed)
    mask = np.zeros((N, N), dtype=np.int32)
    mask[0, :] = 1
    mask[N - 1, :] = 1
    y, x = np.ogrid[:N, :N]
    for _ in range(24):
        cx, cy, r = rng.integers(200, N - 200), rng.integers(200, N - 200), rng.integers(20, 120)
        mask[(x - cx) ** 2 + (y - cy) ** 2 <= r * r] = 1
    case = Case("noalloc_limit", N, N, mask, np.ones((N, N)), np.zeros((N, N)), [BC("periodic_x")])
    f = rng.uniform(0.0, 0.5, size=(N, N, Q))
    f_new = rng.uniform(0.0, 0.5, size=(N, N, Q))
    return case, f, f_new


def _call(lib, case, d_f, d_fn, d_m, out, stream):
    return lib.lbm_gpu_compute_force_mem_noalloc(case.Nx, case.Ny, Q, d_f.data_ptr(), d_fn.data_ptr(),
                                                 d_m.data_ptr(), case.isperiodic_x, case.isperiodic_y,
                                                 iptr(case.cx), iptr(case.cy), iptr(case.opp),
                                                 out.data_ptr(), stream)


def _inputs():
    for name in ("zoo_ibb", "cylinder_wake_small", "zoo_zh_mixed"):
        (case, st), _ = casezoo.build(name)
        yield name, case, st.f, st.f_new
    case, f, f_new = _limit_case()
    yield "limit_4096x4096", case, f, f_new


def test_force_mem_noalloc_matches_oracle(oracle):
    torch = pytest.importorskip("torch")
    import lbc_gb300
    lib = lbc_gb300.load_library()
    stream = torch.cuda.current_stream().cuda_stream
    for name, case, f, f_new in _inputs():
        d_f = torch.from_numpy(np.ascontiguousarray(f)).cuda()
        d_fn = torch.from_numpy(np.ascontiguousarray(f_new)).cuda()
        d_m = torch.from_numpy(case.solid_mask).cuda()
        outs = [torch.full((2,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(3)]
        # First call (the first in this context loads the scratch array), then
        # the device's memory use is the baseline for the calls after it.
        assert _call(lib, case, d_f, d_fn, d_m, outs[0], stream) == 0, lbc_gb300.last_error()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        reserved0 = torch.cuda.memory_reserved()
        # Two calls back to back on the same stream, no synchronisation between
        # them: different inputs (the buffers swapped), different outputs. The
        # second must see none of the first's partials or counter.
        assert _call(lib, case, d_f, d_fn, d_m, outs[1], stream) == 0, lbc_gb300.last_error()
        assert _call(lib, case, d_fn, d_f, d_m, outs[2], stream) == 0, lbc_gb300.last_error()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0, name
        assert torch.cuda.memory_reserved() == reserved0, name
        for out, (a, b) in zip(outs, ((f, f_new), (f, f_new), (f_new, f))):
            want = _oracle_force(oracle, case, a, b)
            got = out.cpu().numpy()
            tol = 1e-12 * _gross(case, a, b)
            assert np.max(np.abs(got - want)) <= tol, (name, got, want, tol)
        del d_f, d_fn, d_m, outs
        torch.cuda.empty_cache()


def test_force_mem_noalloc_rejects_oversized_grid():
    import lbc_gb300
    lib = lbc_gb300.load_library()
    # More blocks than the scratch holds.
    rc = lib.lbm_gpu_compute_force_mem_noalloc(8192, 8192, Q, 1, 1, 1, 0, 0, None, None, None, 1, None)
    assert rc != 0 and "too large" in lbc_gb300.last_error()
    # Few enough blocks, but more block rows than a launch may have.
    rc = lib.lbm_gpu_compute_force_mem_noalloc(64, 262144, Q, 1, 1, 1, 0, 0, None, None, None, 1, None)
    assert rc != 0 and "too large" in lbc_gb300.last_error()
