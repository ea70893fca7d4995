"""Batches: many uneven cases advanced by one persistent kernel per step must
each end exactly as when run alone: populations, fields, impedance-wall state
and the per-step force record bit for bit."""
import numpy as np
import pytest

import casezoo
from conftest import same
from lbc_gb300 import cases

pytestmark = pytest.mark.gpu
FIELDS = ("f", "f_new", "rho", "u", "v")
MIX = ["zoo_ibb", "zoo_convective_chain", "zoo_zh_mixed", "taylor_green", "poiseuille",
       "zoo_periodic_late", "zoo_pressure_reg", "cylinder_wake_small", "zoo_open_edges", "liner",
       "taylor_green_odd", "cylinder_odd", "zoo_moving_lid"]
# Cases without cut-link records (plain bounce-back only): in shifted storage
# the batch's special-node kernel leaves out the link path. Body forces,
# every edge-BC family, an odd width.
MIX_PLAIN = ["zoo_convective_chain", "zoo_zh_mixed", "poiseuille", "zoo_periodic_late", "zoo_pressure_reg",
             "zoo_open_edges", "zoo_reg_periodic", "liner", "liner_odd"]


def _build(n):
    if n in ("liner", "liner_odd"):
        from lbc_gb300 import impedance as imp
        p = imp.LinerParams(nx=200, ny=28, mach=0.2, R=1.1 * imp.CS, m=4e-3, f_res=0.06)
        if n == "liner_odd":
            p = imp.LinerParams(nx=201, ny=27, mach=0.1, R=2.0 * imp.CS, m=6e-3, f_res=0.04)
        return imp.liner_duct(p), p
    return casezoo.build(n)[0], None


def _solvers(storage, names):
    from lbc_gb300 import GpuSolver
    from lbc_gb300 import impedance as imp
    out = []
    for n in names:
        (case, st), lp = _build(n)
        s = GpuSolver(case, storage)
        if lp is not None:
            s.set_impedance_wall(imp.LINER_ENTRY, *imp.liner_arrays(lp), imp.TRACKED_OMEGAS, 1.0, imp.MEAN_RATE, 37)
        try:
            s.enable_force_history(64)
        except RuntimeError:
            pass
        s.set_state(st)
        out.append((n, case, st, s))
    return out


@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
@pytest.mark.parametrize("chunks", [[37], [1, 20, 9]])
@pytest.mark.parametrize("mix", ["links", "plain"])
def test_batch_equals_alone(storage, chunks, mix):
    from lbc_gb300 import STORAGE, GpuBatch
    names = MIX if mix == "links" else MIX_PLAIN
    alone = _solvers(STORAGE[storage], names)
    mixed = _solvers(STORAGE[storage], names)
    for _, _, _, s in alone:
        for c in chunks:
            s.run(c)
    b = GpuBatch([s for _, _, _, s in mixed])
    for c in chunks:
        b.run(c)
    total = sum(chunks)
    for (n, case, _, sa), (_, _, _, sb) in zip(alone, mixed):
        a, m = sa.get_state(), sb.get_state()
        for fld in FIELDS:
            assert same(getattr(a, fld), getattr(m, fld)), (storage, n, fld)
        if n in ("liner", "liner_odd"):
            from lbc_gb300 import impedance as imp
            sa_, ta_ = sa.impedance_readback(imp.LINER_ENTRY)
            sb_, tb_ = sb.impedance_readback(imp.LINER_ENTRY)
            assert same(sa_, sb_) and same(ta_, tb_), (storage, n, "impedance wall")
        ha, hb = sa.force_history(total), sb.force_history(total)
        assert ha.shape == hb.shape
        assert same(ha, hb), (storage, n, "force history")


@pytest.mark.parametrize("storage", ["f64", "f32"])
@pytest.mark.parametrize("mix", ["links", "plain"])
def test_batch_without_force_history(storage, mix):
    """Without a force history the batched steps store and reduce no wall
    force; populations, fields and the force of the run's last step (each
    case's own step, which lbm_gpu_forces reports) are still exactly those of
    the case alone."""
    from lbc_gb300 import STORAGE, GpuBatch, GpuSolver
    names = MIX if mix == "links" else MIX_PLAIN

    def plain(n):
        (case, st), lp = _build(n)
        s = GpuSolver(case, STORAGE[storage])
        if lp is not None:
            from lbc_gb300 import impedance as imp
            s.set_impedance_wall(imp.LINER_ENTRY, *imp.liner_arrays(lp), imp.TRACKED_OMEGAS, 1.0, imp.MEAN_RATE, 37)
        s.set_state(st)
        return s

    alone = [plain(n) for n in names]
    for s in alone:
        s.run(20)
        s.run(17)
    mixed = [plain(n) for n in names]
    b = GpuBatch(mixed)
    b.run(20)
    b.run(17)
    for n, sa, sb in zip(names, alone, mixed):
        a, m = sa.get_state(), sb.get_state()
        for fld in FIELDS:
            assert same(getattr(a, fld), getattr(m, fld)), (storage, n, fld)
        assert same(np.array(sa.forces()), np.array(sb.forces())), (storage, n)
    b.close()


def test_batch_info_counts_launches():
    from lbc_gb300 import GpuBatch, F32_SHIFTED
    mixed = _solvers(F32_SHIFTED, MIX)
    b = GpuBatch([s for _, _, _, s in mixed])
    nodes, lps = b.info()
    assert nodes == sum(c.nodes for _, c, _, _ in mixed)
    levels = max(s.info().edge_launches for _, _, _, s in mixed)
    assert 1 <= levels <= max(s.info().edge_stages for _, _, _, s in mixed)
    # special nodes + clean pairs + one launch per stage level; the levels
    # also advance the impedance walls, finish the BC-written nodes and reduce
    # the wall forces
    assert lps == 2 + levels
    for _, _, _, s in mixed:
        i = s.info()
        bulk = 2 if i.has_geometry else 1  # flag-free grids: one plain kernel
        if i.edge_launches:
            assert i.launches_per_step == bulk + i.edge_launches
        else:  # the bulk step, and the force reduction when there are walls
            assert i.launches_per_step in (bulk, bulk + 1)

