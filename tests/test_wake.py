"""Cylinder wake statistics (lbc_gb300.wake): the Strouhal estimator on
synthetic lift histories and the coefficient summary (CPU)."""
import numpy as np
import pytest

from lbc_gb300 import wake


@pytest.mark.parametrize("period", [600.0, 2000.0, 7531.0])
def test_strouhal_recovers_a_known_frequency(period):
    n = 40000
    t = np.arange(n)
    rng = np.random.default_rng(3)
    cl = 0.2 * np.sin(2 * np.pi * t / period + 0.4) + 0.02 * rng.standard_normal(n) + 0.05
    st = wake.strouhal(cl, 64.0, 0.05)
    exact = 64.0 / 0.05 / period
    assert abs(st / exact - 1.0) < 2e-3


def test_strouhal_of_a_constant_is_zero():
    assert wake.strouhal(np.full(1000, 0.3), 64.0, 0.05) == 0.0
    assert wake.strouhal(np.zeros(8), 64.0, 0.05) == 0.0


def test_summary_uses_the_second_half():
    n = 10000
    t = np.arange(n)
    cd = np.where(t < n // 2, 10.0, 2.0)
    cl = np.where(t < n // 2, 0.0, 0.1 * np.sin(2 * np.pi * t / 500.0))
    s = wake.summary({"cd": cd, "cl": cl, "ms": 1000.0, "nodes": 100}, 64.0, 0.05)
    assert s["cd_mean"] == pytest.approx(2.0)
    assert s["cl_rms"] == pytest.approx(0.1 / np.sqrt(2), rel=1e-2)
    assert s["st"] == pytest.approx(64.0 / 0.05 / 500.0, rel=5e-3)
    assert s["mlups"] == pytest.approx(100 * n / 1.0 / 1e6)
