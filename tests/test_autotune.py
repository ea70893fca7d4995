"""Launch-shape autotuner. No result may depend on the launch shape: every
block shape of the single-case kernel and every tile shape of the batched
kernel give bit-identical populations, fields and momentum-exchange forces,
so a run that tunes itself on its own first steps ends exactly as a run that
does not."""
import numpy as np
import pytest

import casezoo
from conftest import same
from lbc_gb300 import cases

pytestmark = pytest.mark.gpu
FIELDS = ("f", "f_new", "rho", "u", "v")
BLOCKS = [(64, 4), (32, 8), (128, 2), (256, 1), (32, 4), (64, 2), (128, 1), (32, 1)]
TILES = [(64, 4), (32, 8), (128, 2), (256, 1)]


def _cylinder():
    # IBB links, MEM force, regularized inlet and outlet, solid rows.
    return cases.cylinder_wake(300, 76, D=12.0, xc=70.0, yc=37.0, u_max=0.05, Re=60.0, seed=3)


def _solver(storage, built, hist=64):
    from lbc_gb300 import GpuSolver
    case, st = built
    s = GpuSolver(case, storage)
    if hist:
        try:
            s.enable_force_history(hist)
        except RuntimeError:  # no wall links: no force to record
            pass
    s.set_state(st)
    return s


def _assert_same(sa, sb, nsteps, tag):
    a, b = sa.get_state(), sb.get_state()
    for fld in FIELDS:
        assert same(getattr(a, fld), getattr(b, fld)), (tag, fld)
    assert same(np.array(sa.forces()), np.array(sb.forces())), (tag, "force")
    assert same(sa.force_history(nsteps), sb.force_history(nsteps)), (tag, "force history")


@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
def test_block_shape_changes_no_result(storage):
    from lbc_gb300 import STORAGE
    built = _cylinder()
    ref = _solver(STORAGE[storage], built)
    ref.run(23)
    for bx, by in BLOCKS[1:]:
        s = _solver(STORAGE[storage], built)
        s.set_block(bx, by)
        assert s.block() == (bx, by)
        s.run(23)
        _assert_same(ref, s, 23, (storage, bx, by))


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_solver_autotune_changes_no_result(storage):
    from lbc_gb300 import STORAGE, load_library
    load_library().lbm_gpu_tune_cache_clear()
    built = _cylinder()
    ref = _solver(STORAGE[storage], built, hist=128)
    tuned = _solver(STORAGE[storage], built, hist=128)
    tuned.set_autotune(1)
    assert tuned.autotune_status()[0] is False
    for n in (5, 60, 41):  # the first run is too short to tune; the second tunes
        ref.run(n)
        tuned.run(n)
    ok, blk, us = tuned.autotune_status()
    assert ok and blk in BLOCKS and us > 0.0
    _assert_same(ref, tuned, 106, storage)
    # A new solver of the same key takes the cached shape at once.
    again = _solver(STORAGE[storage], built)
    again.set_autotune(1)
    ok2, blk2, _ = again.autotune_status()
    assert ok2 and blk2 == blk


def _mix():
    return [_cylinder(), casezoo.build("zoo_ibb")[0], casezoo.build("poiseuille")[0],
            casezoo.build("zoo_convective_chain")[0], casezoo.build("taylor_green")[0]]


@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
def test_batch_tile_shape_changes_no_result(storage):
    from lbc_gb300 import STORAGE, GpuBatch
    built = _mix()
    alone = [_solver(STORAGE[storage], b) for b in built]
    for s in alone:
        s.run(21)
    for tw, th in TILES:
        mixed = [_solver(STORAGE[storage], b) for b in built]
        bt = GpuBatch(mixed)
        bt.set_tile(tw, th)
        assert bt.autotune_status()[1] == (tw, th)
        bt.run(21)
        for k, (sa, sb) in enumerate(zip(alone, mixed)):
            _assert_same(sa, sb, 21, (storage, tw, th, k))
        bt.close()


def test_batch_rejects_bad_tile():
    from lbc_gb300 import F32_SHIFTED, GpuBatch
    bt = GpuBatch([_solver(F32_SHIFTED, _cylinder())])
    with pytest.raises(RuntimeError):
        bt.set_tile(48, 5)
    with pytest.raises(RuntimeError):
        bt.set_tile(16, 16)


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_batch_autotune_changes_no_result(storage):
    from lbc_gb300 import STORAGE, GpuBatch, load_library
    load_library().lbm_gpu_tune_cache_clear()
    built = _mix()
    alone = [_solver(STORAGE[storage], b, hist=128) for b in built]
    mixed = [_solver(STORAGE[storage], b, hist=128) for b in built]
    bt = GpuBatch(mixed)
    bt.set_autotune(1)
    for n in (7, 70, 13):
        for s in alone:
            s.run(n)
        bt.run(n)
    ok, tile, us = bt.autotune_status()
    assert ok and tile in TILES and us > 0.0
    for k, (sa, sb) in enumerate(zip(alone, mixed)):
        _assert_same(sa, sb, 90, (storage, k))
