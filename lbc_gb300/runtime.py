"""Python bindings of liblbm_gpu.so (lbc's C API plus the extended lbm_gpu_* API).

The library is the product: every call here goes through its C ABI. There is
no CPU path; loading fails loudly when the shared library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from .abi import LbcAbi, dptr, iptr
from .cases import Case, State, Q

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblbm_gpu.so")

F64, F32_SHIFTED, F16_SHIFTED, F64_FMA = 0, 1, 2, 3
STORAGE = {"f64": F64, "f32": F32_SHIFTED, "f16": F16_SHIFTED, "f64fma": F64_FMA}
BYTES_PER_POP = {F64: 8, F32_SHIFTED: 4, F16_SHIFTED: 2, F64_FMA: 8}

_lib: Optional[C.CDLL] = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load liblbm_gpu.so (built by lbc_gb300.build). Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m lbc_gb300.build` "
                           "(or __graft_entry__.build())")
    lib = C.CDLL(path)
    _bind_ext(lib)
    _lib = lib
    return lib


class CaseDesc(C.Structure):
    """lbm_gpu_case (include/lbm_gpu.h)."""
    _fields_ = [
        ("Nx", C.c_int), ("Ny", C.c_int),
        ("cx", C.POINTER(C.c_int)), ("cy", C.POINTER(C.c_int)), ("opp", C.POINTER(C.c_int)),
        ("w", C.POINTER(C.c_double)),
        ("omega_eff", C.POINTER(C.c_double)), ("solid_mask", C.POINTER(C.c_int)),
        ("phi", C.POINTER(C.c_double)), ("use_IBB", C.c_int),
        ("boundaries", C.c_void_p), ("num_boundaries", C.c_int),
        ("isperiodic_x", C.c_int), ("isperiodic_y", C.c_int),
        ("Fx", C.c_double), ("Fy", C.c_double),
        ("wall_u", C.POINTER(C.c_double)), ("wall_v", C.POINTER(C.c_double)),
        ("storage", C.c_int),
    ]


class Info(C.Structure):
    """lbm_gpu_info (include/lbm_gpu.h)."""
    _fields_ = [("Nx", C.c_int), ("Ny", C.c_int), ("pitch", C.c_int), ("storage", C.c_int),
                ("has_geometry", C.c_int), ("edge_stages", C.c_int),
                ("launches_per_step", C.c_int), ("device_bytes", C.c_size_t),
                ("steps_done", C.c_longlong), ("edge_launches", C.c_int)]


def _bind_ext(lib: C.CDLL) -> None:
    vp, dp = C.c_void_p, C.POINTER(C.c_double)
    sig = {
        "lbm_gpu_last_error": (C.c_char_p, []),
        "lbm_gpu_device_count": (C.c_int, []),
        "lbm_gpu_fp64_rate": (C.c_int, [dp]),
        "lbm_gpu_host_access": (C.c_int, [vp]),
        "lbm_gpu_create": (C.c_int, [C.POINTER(CaseDesc), C.POINTER(vp)]),
        "lbm_gpu_destroy": (C.c_int, [vp]),
        "lbm_gpu_set_state": (C.c_int, [vp, dp, dp, dp, dp, dp]),
        "lbm_gpu_get_state": (C.c_int, [vp, dp, dp, dp, dp, dp]),
        "lbm_gpu_get_fields": (C.c_int, [vp, dp, dp, dp]),
        "lbm_gpu_set_bc_values": (C.c_int, [vp, C.c_int, dp, dp]),
        "lbm_gpu_run": (C.c_int, [vp, C.c_int]),
        "lbm_gpu_run_timed": (C.c_int, [vp, C.c_int, dp]),
        "lbm_gpu_sync": (C.c_int, [vp]),
        "lbm_gpu_forces": (C.c_int, [vp, dp, dp]),
        "lbm_gpu_enable_force_history": (C.c_int, [vp, C.c_int]),
        "lbm_gpu_force_history": (C.c_int, [vp, dp, C.c_int]),
        "lbm_gpu_write_force_records": (C.c_longlong, [vp, C.c_char_p, C.c_double, C.c_double, C.c_int]),
        "lbm_gpu_set_probes": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]),
        "lbm_gpu_probe_history": (C.c_int, [vp, dp, C.c_int]),
        "lbm_gpu_enable_impedance_trace": (C.c_int, [vp, C.c_int, C.c_int]),
        "lbm_gpu_write_impedance_trace": (C.c_longlong, [vp, C.c_int, C.c_char_p, C.c_double, C.c_double,
                                                         C.c_double, C.c_int]),
        "lbm_gpu_get_info": (C.c_int, [vp, C.POINTER(Info)]),
        "lbm_gpu_set_block": (C.c_int, [vp, C.c_int, C.c_int]),
        "lbm_gpu_get_block": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "lbm_gpu_checkpoint_save": (C.c_int, [vp, C.c_char_p]),
        "lbm_gpu_checkpoint_load": (C.c_int, [vp, C.c_char_p]),
        "lbm_gpu_write_vtk": (C.c_int, [vp, C.c_char_p, C.c_double, C.c_double, C.c_double]),
        "lbm_gpu_set_autotune": (C.c_int, [vp, C.c_int]),
        "lbm_gpu_autotune_status": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                              C.POINTER(C.c_double)]),
        "lbm_gpu_tune_cache_clear": (None, []),
        "lbm_gpu_batch_set_tile": (C.c_int, [vp, C.c_int, C.c_int]),
        "lbm_gpu_batch_set_autotune": (C.c_int, [vp, C.c_int]),
        "lbm_gpu_batch_autotune_status": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                                    C.POINTER(C.c_int), C.POINTER(C.c_double)]),
        "lbm_gpu_batch_create": (C.c_int, [C.POINTER(vp), C.c_int, C.POINTER(vp)]),
        "lbm_gpu_batch_run": (C.c_int, [vp, C.c_int]),
        "lbm_gpu_batch_run_timed": (C.c_int, [vp, C.c_int, dp]),
        "lbm_gpu_batch_info": (C.c_int, [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_int)]),
        "lbm_gpu_batch_destroy": (C.c_int, [vp]),
        "lbm_gpu_set_impedance_wall": (C.c_int, [vp, C.c_int, dp, dp, dp, C.c_int, dp, C.c_double, C.c_double,
                                                 C.c_int]),
        "lbm_gpu_impedance_readback": (C.c_int, [vp, C.c_int, dp, dp]),
        "lbm_gpu_msd_zoh": (C.c_int, [C.c_double, C.c_double, C.c_double, dp, dp]),
        "lbm_gpu_server_create": (C.c_int, [C.c_size_t, C.c_int, C.c_int, C.POINTER(vp)]),
        "lbm_gpu_server_prepare": (C.c_int, [vp, C.POINTER(CaseDesc), dp, dp, dp, dp, dp, C.c_int, C.c_int]),
        "lbm_gpu_server_set_impedance": (C.c_int, [vp, C.c_int, C.c_int, dp, dp, dp, C.c_int, dp, C.c_double,
                                                   C.c_double, C.c_int]),
        "lbm_gpu_server_enqueue": (C.c_int, [vp, C.c_int]),
        "lbm_gpu_server_poll": (C.c_int, [vp]),
        "lbm_gpu_server_start": (C.c_int, [vp]),
        "lbm_gpu_server_stop": (C.c_int, [vp]),
        "lbm_gpu_server_status": (C.c_int, [vp, C.c_int, dp, dp, dp]),
        "lbm_gpu_server_fetch": (C.c_int, [vp, C.c_int, dp, dp, dp, dp, dp, dp]),
        "lbm_gpu_server_release": (C.c_int, [vp, C.c_int]),
        "lbm_gpu_server_stats": (C.c_int, [vp, C.POINTER(C.c_longlong), dp, C.POINTER(C.c_int),
                                           C.POINTER(C.c_int), C.POINTER(C.c_size_t)]),
        "lbm_gpu_server_profile": (C.c_int, [vp, dp, C.c_int]),
        "lbm_gpu_server_set_reserve": (C.c_int, [vp, C.c_size_t]),
        "lbm_gpu_server_available": (C.c_int, [vp, C.POINTER(C.c_size_t)]),
        "lbm_gpu_server_destroy": (C.c_int, [vp]),
        "lbm_gpu_compute_force_mem_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, vp, vp, vp, C.c_int, C.c_int,
                                                        C.POINTER(C.c_int), C.POINTER(C.c_int),
                                                        C.POINTER(C.c_int), vp, vp]),
        "lbm_gpu_host_alloc": (vp, [C.c_size_t]),
        "lbm_gpu_host_free": (None, [vp]),
        "lbm_gpu_dropin_release": (None, []),
        "lbm_gpu_dropin_set_staged": (None, [C.c_int]),
        "lbm_gpu_dropin_set_lazy": (None, [C.c_int]),
        "lbm_gpu_dropin_sync": (C.c_int, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def last_error() -> str:
    return load_library().lbm_gpu_last_error().decode()


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed ({rc}): {last_error()}")


def dropin() -> LbcAbi:
    """lbc's own API (main_lbm, collision, BCs, ...) as exported by the GPU library."""
    return LbcAbi(load_library())


class PinnedArray:
    """A numpy array over page-locked host memory (lbm_gpu_host_alloc)."""

    def __init__(self, shape, dtype=np.float64):
        lib = load_library()
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self._p = lib.lbm_gpu_host_alloc(max(n, 1))
        if not self._p:
            raise RuntimeError("lbm_gpu_host_alloc failed: " + last_error())
        buf = (C.c_char * n).from_address(self._p)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def __del__(self):
        if getattr(self, "_p", None):
            load_library().lbm_gpu_host_free(self._p)
            self._p = None


def case_desc(lib, case: Case, storage: int):
    """lbm_gpu_case for a Case; returns (desc, keep-alive list)."""
    abi = LbcAbi(lib)
    bnd = abi.boundaries(case.bcs)
    keep = [bnd, case.cx, case.cy, case.opp, case.w, case.omega_eff, case.solid_mask, case.phi]
    d = CaseDesc()
    d.Nx, d.Ny = case.Nx, case.Ny
    d.cx, d.cy, d.opp = iptr(case.cx), iptr(case.cy), iptr(case.opp)
    d.w = dptr(case.w)
    d.omega_eff = dptr(case.omega_eff)
    d.solid_mask = iptr(case.solid_mask)
    d.phi = dptr(case.phi)
    d.use_IBB = case.use_IBB
    d.boundaries = C.cast(bnd[0], C.c_void_p)
    d.num_boundaries = len(case.bcs)
    d.isperiodic_x, d.isperiodic_y = case.isperiodic_x, case.isperiodic_y
    d.Fx, d.Fy = case.Fx, case.Fy
    if case.wall_u is not None:
        wu = np.ascontiguousarray(case.wall_u, dtype=np.float64)
        wv = np.ascontiguousarray(case.wall_v if case.wall_v is not None else np.zeros_like(wu))
        keep += [wu, wv]
        d.wall_u, d.wall_v = dptr(wu), dptr(wv)
    d.storage = storage
    return d, keep


class GpuSolver:
    """A case resident on the GPU (lbm_gpu_create / run / get_state)."""

    def __init__(self, case: Case, storage: int = F64):
        self.lib = load_library()
        self.case = case
        self.storage = storage
        self._abi = LbcAbi(self.lib)
        self._bnd = self._abi.boundaries(case.bcs)
        self._keep = [case.cx, case.cy, case.opp, case.w, case.omega_eff, case.solid_mask, case.phi]
        d = CaseDesc()
        d.Nx, d.Ny = case.Nx, case.Ny
        d.cx, d.cy, d.opp = iptr(case.cx), iptr(case.cy), iptr(case.opp)
        d.w = dptr(case.w)
        d.omega_eff = dptr(case.omega_eff)
        d.solid_mask = iptr(case.solid_mask)
        d.phi = dptr(case.phi)
        d.use_IBB = case.use_IBB
        d.boundaries = C.cast(self._bnd[0], C.c_void_p)
        d.num_boundaries = len(case.bcs)
        d.isperiodic_x, d.isperiodic_y = case.isperiodic_x, case.isperiodic_y
        d.Fx, d.Fy = case.Fx, case.Fy
        if case.wall_u is not None:
            wu = np.ascontiguousarray(case.wall_u, dtype=np.float64)
            wv = np.ascontiguousarray(case.wall_v if case.wall_v is not None else np.zeros_like(wu))
            self._keep += [wu, wv]
            d.wall_u, d.wall_v = dptr(wu), dptr(wv)
        d.storage = storage
        h = C.c_void_p()
        _check(self.lib.lbm_gpu_create(C.byref(d), C.byref(h)), "lbm_gpu_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.lbm_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_state(self, st: State):
        _check(self.lib.lbm_gpu_set_state(self.h, dptr(st.f), dptr(st.f_new), dptr(st.rho),
                                          dptr(st.u), dptr(st.v)), "lbm_gpu_set_state")

    def get_state(self) -> State:
        Ny, Nx = self.case.Ny, self.case.Nx
        st = State(np.empty((Ny, Nx, Q)), np.empty((Ny, Nx, Q)), np.empty((Ny, Nx)),
                   np.empty((Ny, Nx)), np.empty((Ny, Nx)))
        _check(self.lib.lbm_gpu_get_state(self.h, dptr(st.f), dptr(st.f_new), dptr(st.rho),
                                          dptr(st.u), dptr(st.v)), "lbm_gpu_get_state")
        return st

    def get_fields(self):
        Ny, Nx = self.case.Ny, self.case.Nx
        rho, u, v = np.empty((Ny, Nx)), np.empty((Ny, Nx)), np.empty((Ny, Nx))
        _check(self.lib.lbm_gpu_get_fields(self.h, dptr(rho), dptr(u), dptr(v)), "lbm_gpu_get_fields")
        return rho, u, v

    def set_bc_values(self, entry: int, val1=None, val2=None):
        a1 = None if val1 is None else np.ascontiguousarray(val1, dtype=np.float64)
        a2 = None if val2 is None else np.ascontiguousarray(val2, dtype=np.float64)
        _check(self.lib.lbm_gpu_set_bc_values(self.h, entry, dptr(a1) if a1 is not None else None,
                                              dptr(a2) if a2 is not None else None),
               "lbm_gpu_set_bc_values")

    def run(self, nsteps: int):
        _check(self.lib.lbm_gpu_run(self.h, nsteps), "lbm_gpu_run")

    def run_timed(self, nsteps: int) -> float:
        ms = C.c_double(0.0)
        _check(self.lib.lbm_gpu_run_timed(self.h, nsteps, C.byref(ms)), "lbm_gpu_run_timed")
        return ms.value

    def sync(self):
        _check(self.lib.lbm_gpu_sync(self.h), "lbm_gpu_sync")

    def forces(self):
        L, D = C.c_double(), C.c_double()
        _check(self.lib.lbm_gpu_forces(self.h, C.byref(L), C.byref(D)), "lbm_gpu_forces")
        return L.value, D.value

    def enable_force_history(self, capacity: int):
        _check(self.lib.lbm_gpu_enable_force_history(self.h, capacity), "lbm_gpu_enable_force_history")

    def force_history(self, max_steps: int) -> np.ndarray:
        out = np.empty((max_steps, 2))
        n = self.lib.lbm_gpu_force_history(self.h, dptr(out), max_steps)
        if n < 0:
            raise RuntimeError(last_error())
        return out[:n]

    def set_probes(self, nodes, capacity: int):
        """Record (rho, ux, uy) at nodes [(i, j), ...] after every step
        (lbm_gpu_set_probes); an empty list removes the probes."""
        nodes = list(nodes)
        ii = np.ascontiguousarray([int(n[0]) for n in nodes], dtype=np.int32)
        jj = np.ascontiguousarray([int(n[1]) for n in nodes], dtype=np.int32)
        self._nprobes = len(nodes)
        _check(self.lib.lbm_gpu_set_probes(self.h, len(nodes), iptr(ii), iptr(jj), capacity), "lbm_gpu_set_probes")

    def probe_history(self, max_steps: int) -> np.ndarray:
        """[steps, probes, 3] (rho, ux, uy), oldest first (lbm_gpu_probe_history)."""
        n = getattr(self, "_nprobes", 0)
        out = np.empty((max_steps, max(n, 1), 3))
        k = self.lib.lbm_gpu_probe_history(self.h, dptr(out), max_steps)
        if k < 0:
            raise RuntimeError(last_error())
        return out[:k, :n]

    def enable_impedance_trace(self, entry: int, capacity: int):
        _check(self.lib.lbm_gpu_enable_impedance_trace(self.h, entry, capacity), "lbm_gpu_enable_impedance_trace")

    def write_impedance_trace(self, entry: int, path: str, dt: float = 1.0, cp: float = 1.0, cu: float = 1.0,
                              append: bool = False) -> int:
        """lbc's TDIBC text trace for the steps not written yet
        (lbm_gpu_write_impedance_trace); returns the number of lines."""
        n = self.lib.lbm_gpu_write_impedance_trace(self.h, entry, path.encode(), dt, cp, cu, 1 if append else 0)
        if n < 0:
            raise RuntimeError(f"lbm_gpu_write_impedance_trace failed ({n}): {last_error()}")
        return n

    def write_force_records(self, path: str, dt: float, cf: float = 1.0, append: bool = False) -> int:
        """lbc's {t, L, D} force record file for the steps not written yet
        (lbm_gpu_write_force_records); returns the number of records."""
        n = self.lib.lbm_gpu_write_force_records(self.h, path.encode(), dt, cf, 1 if append else 0)
        if n < 0:
            raise RuntimeError(f"lbm_gpu_write_force_records failed ({n}): {last_error()}")
        return n

    def set_impedance_wall(self, entry: int, R, m, K, omegas=(), rho_ref: float = 1.0, alpha: float = 0.0,
                           window: int = 0):
        R, m, K = (np.ascontiguousarray(a, dtype=np.float64) for a in (R, m, K))
        om = np.ascontiguousarray(omegas, dtype=np.float64)
        self._imp = (R, m, K, om)
        _check(self.lib.lbm_gpu_set_impedance_wall(self.h, entry, dptr(R), dptr(m), dptr(K), len(om),
                                                   dptr(om) if len(om) else None, rho_ref, alpha, window),
               "lbm_gpu_set_impedance_wall")

    def impedance_readback(self, entry: int):
        """(spectra[Nx, nf, 4], state[Nx, 2]) of the impedance wall on `entry`."""
        nf = len(self._imp[3])
        n = self.case.Nx
        spec = np.zeros((n, max(nf, 1), 4))
        state = np.zeros((n, 2))
        _check(self.lib.lbm_gpu_impedance_readback(self.h, entry, dptr(spec), dptr(state)),
               "lbm_gpu_impedance_readback")
        return spec[:, :nf], state

    def info(self) -> Info:
        inf = Info()
        _check(self.lib.lbm_gpu_get_info(self.h, C.byref(inf)), "lbm_gpu_get_info")
        return inf

    def set_block(self, bx: int, by: int):
        _check(self.lib.lbm_gpu_set_block(self.h, bx, by), "lbm_gpu_set_block")

    def block(self):
        bx, by = C.c_int(), C.c_int()
        _check(self.lib.lbm_gpu_get_block(self.h, C.byref(bx), C.byref(by)), "lbm_gpu_get_block")
        return bx.value, by.value

    def checkpoint_save(self, path: str):
        _check(self.lib.lbm_gpu_checkpoint_save(self.h, os.fsencode(path)), "lbm_gpu_checkpoint_save")

    def checkpoint_load(self, path: str):
        _check(self.lib.lbm_gpu_checkpoint_load(self.h, os.fsencode(path)), "lbm_gpu_checkpoint_load")

    def write_vtk(self, path: str, dx: float = 1.0, cu: float = 1.0, crho: float = 1.0):
        """lbc's VTK file of the stored fields, packed on the device; complete
        after sync()."""
        _check(self.lib.lbm_gpu_write_vtk(self.h, os.fsencode(path), dx, cu, crho), "lbm_gpu_write_vtk")

    def set_autotune(self, mode: int = 1):
        """Tune the fused step's block shape on the next long enough run."""
        _check(self.lib.lbm_gpu_set_autotune(self.h, mode), "lbm_gpu_set_autotune")

    def autotune_status(self):
        """(tuned, (bx, by), microseconds per step in the trial windows)."""
        t, bx, by, us = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        _check(self.lib.lbm_gpu_autotune_status(self.h, C.byref(t), C.byref(bx), C.byref(by), C.byref(us)),
               "lbm_gpu_autotune_status")
        return bool(t.value), (bx.value, by.value), us.value


class GpuBatch:
    """Independent cases of one storage type advanced together (lbm_gpu_batch_*)."""

    def __init__(self, solvers):
        self.lib = load_library()
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        h = C.c_void_p()
        _check(self.lib.lbm_gpu_batch_create(arr, len(self.solvers), C.byref(h)), "lbm_gpu_batch_create")
        self.h = h

    def run(self, nsteps: int):
        _check(self.lib.lbm_gpu_batch_run(self.h, nsteps), "lbm_gpu_batch_run")

    def run_timed(self, nsteps: int) -> float:
        ms = C.c_double(0.0)
        _check(self.lib.lbm_gpu_batch_run_timed(self.h, nsteps, C.byref(ms)), "lbm_gpu_batch_run_timed")
        return ms.value

    def info(self):
        n, l = C.c_longlong(), C.c_int()
        _check(self.lib.lbm_gpu_batch_info(self.h, C.byref(n), C.byref(l)), "lbm_gpu_batch_info")
        return n.value, l.value

    def set_tile(self, tw: int, th: int):
        _check(self.lib.lbm_gpu_batch_set_tile(self.h, tw, th), "lbm_gpu_batch_set_tile")

    def set_autotune(self, mode: int = 1):
        """Tune the bulk kernel's tile shape on the next long enough run."""
        _check(self.lib.lbm_gpu_batch_set_autotune(self.h, mode), "lbm_gpu_batch_set_autotune")

    def autotune_status(self):
        """(tuned, (tw, th), microseconds per step in the trial windows)."""
        t, tw, th, us = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        _check(self.lib.lbm_gpu_batch_autotune_status(self.h, C.byref(t), C.byref(tw), C.byref(th),
                                                      C.byref(us)), "lbm_gpu_batch_autotune_status")
        return bool(t.value), (tw.value, th.value), us.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.lbm_gpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class GpuServer:
    """Continuous-batching request loop (lbm_gpu_server_*)."""

    def __init__(self, budget_bytes: int = 0, max_active: int = 64, chunk_steps: int = 1000):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib.lbm_gpu_server_create(budget_bytes, max_active, chunk_steps, C.byref(h)),
               "lbm_gpu_server_create")
        self.h = h
        self.meta = {}

    def submit(self, case: Case, st: State, nsteps: int, storage: int, keep_populations=False,
               impedance=None, from_equilibrium=False) -> int:
        """impedance: (entry, R, m, K, omegas, rho_ref, alpha, window) or None.
        from_equilibrium: start from f = f_eq(rho, u, v) formed at admission
        (st.f and st.f_new are not sent)."""
        d, keep = case_desc(self.lib, case, storage)
        f = None if from_equilibrium else dptr(st.f)
        fn = None if from_equilibrium else dptr(st.f_new)
        rid = self.lib.lbm_gpu_server_prepare(self.h, C.byref(d), f, fn, dptr(st.rho),
                                              dptr(st.u), dptr(st.v), nsteps, 1 if keep_populations else 0)
        if rid <= 0:
            raise RuntimeError("lbm_gpu_server_prepare failed: " + last_error())
        if impedance is not None:
            entry, R, m, K, om, rho_ref, alpha, window = impedance
            R, m, K, om = (np.ascontiguousarray(a, dtype=np.float64) for a in (R, m, K, om))
            _check(self.lib.lbm_gpu_server_set_impedance(self.h, rid, entry, dptr(R), dptr(m), dptr(K), len(om),
                                                         dptr(om), rho_ref, alpha, window),
                   "lbm_gpu_server_set_impedance")
        self.meta[rid] = (case.Nx, case.Ny, nsteps, len(impedance[4]) if impedance else 0)
        _check(self.lib.lbm_gpu_server_enqueue(self.h, rid), "lbm_gpu_server_enqueue")
        return rid

    def poll(self) -> int:
        return self.lib.lbm_gpu_server_poll(self.h)

    def start(self):
        _check(self.lib.lbm_gpu_server_start(self.h), "lbm_gpu_server_start")

    def stop(self):
        self.lib.lbm_gpu_server_stop(self.h)

    def status(self, rid: int):
        ts, ta, td = C.c_double(), C.c_double(), C.c_double()
        st = self.lib.lbm_gpu_server_status(self.h, rid, C.byref(ts), C.byref(ta), C.byref(td))
        return st, ts.value, ta.value, td.value

    def fetch(self, rid: int, populations=False):
        Nx, Ny, _, nf = self.meta[rid]
        rho, u, v = np.empty((Ny, Nx)), np.empty((Ny, Nx)), np.empty((Ny, Nx))
        f = np.empty((Ny, Nx, Q)) if populations else None
        fn = np.empty((Ny, Nx, Q)) if populations else None
        spec = np.zeros((Nx, max(nf, 1), 4))
        _check(self.lib.lbm_gpu_server_fetch(self.h, rid, dptr(f) if populations else None,
                                             dptr(fn) if populations else None, dptr(rho), dptr(u), dptr(v),
                                             dptr(spec)), "lbm_gpu_server_fetch")
        return {"rho": rho, "u": u, "v": v, "f": f, "f_new": fn, "spectra": spec[:, :nf]}

    def release(self, rid: int):
        self.lib.lbm_gpu_server_release(self.h, rid)
        self.meta.pop(rid, None)

    def stats(self):
        l, b, q, a, m = C.c_longlong(), C.c_double(), C.c_int(), C.c_int(), C.c_size_t()
        _check(self.lib.lbm_gpu_server_stats(self.h, C.byref(l), C.byref(b), C.byref(q), C.byref(a), C.byref(m)),
               "lbm_gpu_server_stats")
        return {"lups": l.value, "busy_s": b.value, "queued": q.value, "active": a.value, "bytes": m.value}

    def set_reserve(self, reserve_bytes: int):
        """Device memory admissions leave free (lbm_gpu_server_set_reserve)."""
        _check(self.lib.lbm_gpu_server_set_reserve(self.h, int(reserve_bytes)), "lbm_gpu_server_set_reserve")

    def available(self) -> int:
        """Device memory a request could be admitted into now (lbm_gpu_server_available)."""
        b = C.c_size_t()
        _check(self.lib.lbm_gpu_server_available(self.h, C.byref(b)), "lbm_gpu_server_available")
        return b.value

    def profile(self):
        """Host seconds per phase of the scheduling rounds (lbm_gpu_server_profile)."""
        out = np.zeros(9)
        _check(self.lib.lbm_gpu_server_profile(self.h, dptr(out), 9), "lbm_gpu_server_profile")
        return {"rounds": int(out[0]), "admit_s": out[1], "build_s": out[2], "run_s": out[3], "retire_s": out[4],
                "lane_f64_s": out[5], "lane_f32_s": out[6], "lane_f16_s": out[7], "lane_f64fma_s": out[8]}

    def close(self):
        if getattr(self, "h", None):
            self.lib.lbm_gpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
