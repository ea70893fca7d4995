"""ctypes adapter for any library that exposes lbc's C signatures.

lbc's public functions (include/lbm_core.h:6-128, include/lbm_bc.h:4-354,
include/lbm_utils.h:4-15) take VLA-typed arrays that decay to plain pointers at
the ABI level. :class:`LbcAbi` binds those signatures on a ``ctypes.CDLL``
handle, optionally with a symbol prefix, and runs them on numpy arrays in lbc's
layout. The GPU drop-in ``liblbm_gpu.so`` exports the unprefixed names.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence

import numpy as np

from .cases import BC, Case, State, Q

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Boundary(C.Structure):
    """lbc's ``Boundary`` (include/lbm_types.h:21-26)."""
    _fields_ = [("index", C.c_int), ("val1", _dp), ("val2", _dp), ("apply", C.c_void_p)]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


_BC_ARGS = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _ip, _dp]
_BC_NAMES = (
    "velocity_inlet", "velocity_outlet", "velocity_top", "velocity_bottom",
    "pressure_inlet", "pressure_outlet", "convective_inlet", "convective_outlet",
    "periodic_x", "periodic_y",
    "velocity_inlet_regularized", "velocity_outlet_regularized",
    "velocity_top_regularized", "velocity_bottom_regularized",
    "pressure_inlet_regularized", "pressure_outlet_regularized",
    "pressure_top_regularized", "pressure_bottom_regularized",
)
# Extensions with no counterpart in lbc (its own build does not export them).
_BC_EXT_NAMES = ("velocity_bottom_corrected",)


class LbcAbi:
    def __init__(self, cdll: C.CDLL, prefix: str = ""):
        self.lib = cdll
        self.prefix = prefix
        g = self._fn
        g("main_lbm", None, [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _dp, _ip,
                             _dp, _ip, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                             _dp, _dp, _dp, C.c_int])
        g("collision", None, [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _ip, _dp,
                              C.c_double, C.c_double])
        g("streaming", None, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _ip, C.c_int, C.c_int])
        g("compute_macroscopic_fields", None, [C.c_int, C.c_int, C.c_int, _dp, _ip, _ip, _ip, _dp, _dp,
                                               _dp, C.c_double, C.c_double])
        g("compute_force_mem", None, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, C.c_int, C.c_int, _ip,
                                      _ip, _ip, _dp, _dp])
        g("bounce_back", None, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _ip, _ip, C.c_int, C.c_int])
        g("interpolated_bounce_back", None, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _dp, _ip, _ip, _ip,
                                             C.c_int, C.c_int])
        g("sponge_layer", None, [C.c_int, C.c_int] + [C.c_double] * 8 + [_dp])
        for n in _BC_NAMES:
            g(n, None, _BC_ARGS)
        for n in _BC_EXT_NAMES:
            if hasattr(self.lib, self.prefix + n):
                g(n, None, _BC_ARGS)

    def _fn(self, name, restype, argtypes):
        fn = getattr(self.lib, self.prefix + name)
        fn.restype = restype
        fn.argtypes = argtypes
        setattr(self, name, fn)

    def bc_address(self, name: str) -> int:
        return C.cast(getattr(self.lib, self.prefix + name), C.c_void_p).value

    def boundaries(self, bcs: Sequence[BC]):
        """Build a ``Boundary[]`` whose ``apply`` pointers are this library's
        own BC symbols. Returned object keeps the value arrays alive."""
        arr = (Boundary * max(1, len(bcs)))()
        keep: List[np.ndarray] = []
        for t, b in enumerate(bcs):
            arr[t].index = b.index
            for fld in ("val1", "val2"):
                a = getattr(b, fld)
                if a is not None:
                    a = np.ascontiguousarray(a, dtype=np.float64)
                    keep.append(a)
                    setattr(arr[t], fld, dptr(a))
            arr[t].apply = self.bc_address(b.name)
        return arr, keep

    def step(self, case: Case, st: State, bnd=None, swap: bool = True):
        """One ``main_lbm`` call followed by the caller-side swap of
        cases/nit/nit.c:309-311. Returns (L, D). A case with moving walls
        (wall_u / wall_v, an extension with no counterpart in lbc) takes the
        oracle's ext_main_lbm_moving, which only the oracle library has."""
        if bnd is None:
            bnd = self.boundaries(case.bcs)
        arr, _keep = bnd
        L = C.c_double(0.0)
        D = C.c_double(0.0)
        if case.wall_u is not None or case.wall_v is not None:
            fn = getattr(self.lib, self.prefix + "ext_main_lbm_moving")
            zero = np.zeros((case.Ny, case.Nx))
            uw = np.ascontiguousarray(case.wall_u if case.wall_u is not None else zero, dtype=np.float64)
            vw = np.ascontiguousarray(case.wall_v if case.wall_v is not None else zero, dtype=np.float64)
            fn.restype = None
            fn(case.Nx, case.Ny, Q, dptr(st.f), dptr(st.f_new), dptr(st.rho), dptr(st.u), dptr(st.v),
               iptr(case.cx), iptr(case.cy), dptr(case.w), iptr(case.opp), dptr(case.omega_eff),
               iptr(case.solid_mask), C.cast(arr, C.c_void_p), len(case.bcs), case.isperiodic_x,
               case.isperiodic_y, C.c_double(case.Fx), C.c_double(case.Fy), C.byref(L), C.byref(D),
               dptr(uw), dptr(vw))
            if swap:
                st.f, st.f_new = st.f_new, st.f
            return L.value, D.value
        self.main_lbm(case.Nx, case.Ny, Q, dptr(st.f), dptr(st.f_new), dptr(st.rho), dptr(st.u),
                      dptr(st.v), iptr(case.cx), iptr(case.cy), dptr(case.w), iptr(case.opp),
                      dptr(case.omega_eff), iptr(case.solid_mask), C.cast(arr, C.c_void_p),
                      len(case.bcs), case.isperiodic_x, case.isperiodic_y, case.Fx, case.Fy,
                      C.byref(L), C.byref(D), dptr(case.phi), case.use_IBB)
        if swap:
            st.f, st.f_new = st.f_new, st.f
        return L.value, D.value

    def run(self, case: Case, st: State, nsteps: int, record_forces: bool = False):
        bnd = self.boundaries(case.bcs)
        forces = []
        for _ in range(nsteps):
            LD = self.step(case, st, bnd)
            if record_forces:
                forces.append(LD)
        return np.array(forces) if record_forces else None
