"""Test configuration: the `gpu` marker, the oracle libraries and shared helpers.

The oracle (oracle/lbm_oracle.c, a CPU restatement of lbc's FP64 step) and the
reference build (oracle/_ref, lbc's own src/ compiled here when its sources
are present) are checkers only; they are loaded here, never by the product.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from lbc_gb300.abi import LbcAbi  # noqa: E402

ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liblbm_oracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libref_lbc.so")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_oracle():
    src = os.path.join(ROOT, "oracle", "lbm_oracle.c")
    if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_oracle.sh")], check=True,
                       capture_output=True)


def oracle_abi():
    """The oracle's lbc-style API (built on first use)."""
    _ensure_oracle()
    return LbcAbi(C.CDLL(ORACLE_SO), "orc_")


@pytest.fixture(scope="session")
def oracle():
    return oracle_abi()


@pytest.fixture(scope="session")
def ref():
    if not os.path.exists(REF_SO):
        pytest.skip("oracle/_ref (lbc's own src/) is not built here")
    return LbcAbi(C.CDLL(REF_SO), "ref_")


@pytest.fixture(scope="session")
def gpu():
    """The GPU library through lbc's own C API."""
    import lbc_gb300
    lib = lbc_gb300.load_library()
    if lib.lbm_gpu_device_count() < 1:
        pytest.fail("no CUDA device visible to liblbm_gpu.so")
    return lbc_gb300.dropin()


def same(a, b):
    """Bitwise-equal values (NaN == NaN, +0 == -0)."""
    return np.array_equal(a, b, equal_nan=True)


def maxrel(a, b):
    m = np.isfinite(b)
    den = np.max(np.abs(b[m])) if m.any() else 1.0
    return float(np.max(np.abs(a[m] - b[m])) / den) if m.any() else 0.0


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
