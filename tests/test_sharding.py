"""Cases across ranks (lbc_gb300.sharding): the work-balanced partition, and a
world-size-2 gloo run on CPU in which each rank advances its share of seeded
cases with the oracle and the gathered results equal a one-process run bit
for bit."""
import os
import socket
import tempfile

import numpy as np
import pytest

from lbc_gb300 import sharding


def test_partition_covers_each_case_once_and_balances():
    rng = np.random.default_rng(5)
    for ws in (1, 2, 3, 4, 8):
        for n in (0, 1, 5, 64, 200):
            costs = rng.uniform(1.0, 100.0, n)
            parts = sharding.partition(costs, ws)
            assert len(parts) == ws
            flat = sorted(i for p in parts for i in p)
            assert flat == list(range(n))
            assert all(p == sorted(p) for p in parts)
            if n:
                ld = sharding.loads(costs, parts)
                assert max(ld) - min(ld) <= max(costs) + 1e-9
            assert parts == sharding.partition(list(costs), ws)  # deterministic


def test_partition_rejects_bad_arguments():
    with pytest.raises(ValueError):
        sharding.partition([1.0], 0)
    with pytest.raises(ValueError):
        sharding.share([1.0], 2, 2)


def test_gather_one_rank_and_errors():
    assert sharding.gather_results(None, 3, [0, 1, 2], ["a", "b", "c"]) == ["a", "b", "c"]
    with pytest.raises(RuntimeError):
        sharding.gather_results(None, 3, [0, 1], ["a", "b"])
    with pytest.raises(ValueError):
        sharding.gather_results(None, 2, [0, 1], ["a"])
    assert sharding.all_max(None, 2.5) == 2.5 and sharding.all_sum(None, 2.5) == 2.5


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cases():
    from lbc_gb300 import cases
    out = []
    for k, (nx, ny) in enumerate([(40, 12), (24, 10), (64, 16), (16, 8), (48, 20)]):
        case, st = cases.poiseuille(nx, ny, 0.6 + 0.05 * k, 1e-5 * (k + 1))
        out.append((case, st))
    out.append(cases.taylor_green(32, 24, 0.04, 0.56))
    return out


def _advance(items, steps=25):
    """Run each (case, state) through the oracle's main_lbm; return rho, u, v."""
    from conftest import oracle_abi
    lib = oracle_abi()
    res = []
    for case, st in items:
        st = st.copy()
        bnd = lib.boundaries(case.bcs)
        for _ in range(steps):
            lib.step(case, st, bnd)
        res.append((st.rho.copy(), st.u.copy(), st.v.copy()))
    return res


def _rank_main(rank, ws, port, outdir):
    import torch.distributed as td
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    td.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        items = _cases()
        costs = [c.Nx * c.Ny for c, _ in items]
        got = sharding.run_sharded(items, costs, _advance, td)
        mx = sharding.all_max(td, float(rank + 1))
        sm = sharding.all_sum(td, float(rank + 1))
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), mx=mx, sm=sm,
                 mine=np.array(sharding.share(costs, ws, rank)),
                 **{f"r{i}_{k}": a for i, t in enumerate(got) for k, a in zip("ruv", t)})
    finally:
        td.destroy_process_group()


def test_two_ranks_gloo_equal_one_process():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ws = 2
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(ws, _free_port(), d), nprocs=ws, join=True,
                           start_method="spawn")
        ref = _advance(_cases())
        shares = []
        for rank in range(ws):
            z = np.load(os.path.join(d, f"rank{rank}.npz"))
            assert float(z["mx"]) == 2.0 and float(z["sm"]) == 3.0
            shares.append(set(z["mine"].tolist()))
            for i, t in enumerate(ref):
                for k, a in zip("ruv", t):
                    assert np.array_equal(z[f"r{i}_{k}"], a, equal_nan=True), (rank, i, k)
        assert shares[0].isdisjoint(shares[1]) and len(shares[0] | shares[1]) == len(ref)
        assert shares[0] and shares[1]
