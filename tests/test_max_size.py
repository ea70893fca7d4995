"""The largest grids. When the nine population planes hold 2^31 elements or
more, the shifted-storage step kernels use 64-bit element offsets instead of
32-bit ones. A field that repeats with the period of a small periodic grid
evolves on a large periodic grid exactly as on the small one, because every
node's update sees the same values. So the large grid's fields must equal the
small grid's fields, tiled, bit for bit: a size-independent check of the
64-bit path against the 32-bit path, which the oracle pins on small grids.

The large case is 16384 x 14592 nodes (9 planes x 239,075,328 elements =
2.15e9 >= 2^31). It holds about 35 GB of host memory (lbc's FP64 AoS arrays)
and 32 GB of device memory, and it is skipped on a host with less than
128 GB available."""
import dataclasses

import numpy as np
import pytest

from lbc_gb300 import cases
from lbc_gb300.cases import State

pytestmark = pytest.mark.gpu

TX, TY = 64, 48          # the small grid
RX, RY = 256, 304        # repeats along x and y
STEPS = 20


def _mem_available_gb():
    try:
        with open("/proc/meminfo") as fh:
            for line in fh:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 2**20
    except OSError:
        pass
    return 0.0


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_64bit_offsets_match_the_tiled_small_grid(storage):
    from lbc_gb300 import STORAGE, GpuSolver
    Nx, Ny = TX * RX, TY * RY
    pitch = (Nx + 63) // 64 * 64
    assert 9 * pitch * Ny >= 2**31          # the case takes the 64-bit offset path
    if _mem_available_gb() < 128:
        pytest.skip("fewer than 128 GB of host memory available for the 16384 x 14592 case")

    small, st = cases.taylor_green(TX, TY, 0.04, 0.56)
    s = GpuSolver(small, STORAGE[storage])
    s.set_state(st)
    s.run(STEPS)
    want = s.get_fields()
    s.close()

    big = dataclasses.replace(small, name="taylor_green_tiled", Nx=Nx, Ny=Ny,
                              solid_mask=np.zeros((Ny, Nx), np.int32),
                              omega_eff=np.tile(small.omega_eff, (RY, RX)),
                              phi=np.zeros((Ny, Nx)))
    f = np.tile(st.f, (RY, RX, 1))
    g = GpuSolver(big, STORAGE[storage])
    # a periodic case without solids never reads f_new's old content
    g.set_state(State(f, f, np.tile(st.rho, (RY, RX)), np.tile(st.u, (RY, RX)), np.tile(st.v, (RY, RX))))
    del f, big
    g.run(STEPS)
    got = g.get_fields()
    g.close()
    for name, a, b in zip(("rho", "u", "v"), got, want):
        tiles = a.reshape(RY, TY, RX, TX)
        assert np.array_equal(tiles, np.broadcast_to(b[None, :, None, :], tiles.shape)), name
