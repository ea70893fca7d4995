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


def test_state_round_trip_over_several_staging_chunks():
    """set_state / get_state convert lbc's FP64 AoS arrays through a staging
    buffer of at most 64 MiB, a chunk of rows at a time: a 1024 x 1536 grid
    (113 MB per array, two chunks) comes back bit for bit in FP64 storage."""
    from lbc_gb300 import F64, GpuSolver
    Nx, Ny = 1024, 1536
    small, _ = cases.taylor_green(64, 48, 0.04, 0.56)
    big = dataclasses.replace(small, name="round_trip", Nx=Nx, Ny=Ny, solid_mask=np.zeros((Ny, Nx), np.int32),
                              omega_eff=np.full((Ny, Nx), small.omega_eff[0, 0]), phi=np.zeros((Ny, Nx)))
    rng = np.random.default_rng(7)
    st = State(rng.random((Ny, Nx, 9)), rng.random((Ny, Nx, 9)), rng.random((Ny, Nx)),
               rng.random((Ny, Nx)), rng.random((Ny, Nx)))
    s = GpuSolver(big, F64)
    s.set_state(st)
    out = s.get_state()
    s.close()
    assert np.array_equal(out.f, st.f) and np.array_equal(out.f_new, st.f_new)
