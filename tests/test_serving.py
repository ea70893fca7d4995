"""Serving with continuous batching: requests join and leave between chunks,
FP32 and FP64 batches run side by side, and every result equals the same
request run alone. Failures are injected on the host (a request whose setup
is invalid) and must not disturb the others."""
import numpy as np
import pytest

from conftest import same
from lbc_gb300 import serving
from lbc_gb300.serving import Req

pytestmark = pytest.mark.gpu


def _stream():
    rng = np.random.default_rng(5)
    out = []
    for q in range(10):
        ny = int(rng.choice([32, 40, 48]))
        out.append(Req(("channel", "cylinder", "liner")[q % 3], 4 * ny, ny, int(rng.integers(40, 300)),
                       1 if q % 4 else 0, 0.0, 1000 + q))
    return out


def _alone(r):
    from lbc_gb300 import GpuSolver
    case, st, spec = serving.build_request(r)
    s = GpuSolver(case, r.storage)
    if spec is not None:
        s.set_impedance_wall(spec[0], *spec[1:4], spec[4], spec[5], spec[6], spec[7])
    s.set_state(st)
    s.run(r.steps)
    rho, u, v = s.get_fields()
    spec_out = s.impedance_readback(spec[0])[0] if spec is not None else None
    return rho, u, v, spec_out


@pytest.mark.parametrize("budget,max_active,chunk", [(0, 4, 37), (0, 64, 1000), (1 << 20, 64, 50)])
def test_results_same_alone_and_in_the_mix(budget, max_active, chunk):
    from lbc_gb300 import GpuServer
    stream = _stream()
    srv = GpuServer(budget, max_active, chunk)
    ids = []
    for r in stream:
        case, st, spec = serving.build_request(r)
        ids.append(srv.submit(case, st, r.steps, r.storage, impedance=spec))
    while srv.poll() > 0:
        pass
    for r, rid in zip(stream, ids):
        state, ts, ta, td = srv.status(rid)
        assert state == 3
        res = srv.fetch(rid)
        rho, u, v, spec = _alone(r)
        assert same(res["rho"], rho) and same(res["u"], u) and same(res["v"], v), (r, budget, chunk)
        if spec is not None:
            assert same(res["spectra"], spec)
        srv.release(rid)
    srv.close()


def test_threaded_server_and_failed_request():
    """Background scheduling thread with requests arriving while others run;
    one request is invalid (Boundary index outside the grid) and fails alone."""
    from lbc_gb300 import GpuServer, F32_SHIFTED
    from lbc_gb300.cases import BC
    stream = _stream()[:6]
    srv = GpuServer(0, 3, 40)
    srv.start()
    ids = []
    bad = None
    for q, r in enumerate(stream):
        case, st, spec = serving.build_request(r)
        ids.append(srv.submit(case, st, r.steps, r.storage, impedance=spec))
        if q == 2:
            c2, s2, _ = serving.build_request(stream[0])
            c2.bcs[0] = BC(c2.bcs[0].name, c2.Nx + 5, c2.bcs[0].val1, c2.bcs[0].val2)
            bad = srv.submit(c2, s2, 50, F32_SHIFTED)
    import time
    t0 = time.time()
    while any(srv.status(i)[0] < 3 for i in ids + [bad]):
        assert time.time() - t0 < 120
        time.sleep(0.01)
    srv.stop()
    assert srv.status(bad)[0] == 4
    for r, rid in zip(stream, ids):
        assert srv.status(rid)[0] == 3
        res = srv.fetch(rid)
        rho, u, v, _ = _alone(r)
        assert same(res["rho"], rho)
    srv.close()


def test_requests_started_from_equilibrium():
    """A request sent without populations starts from lbc's f_eq(rho, u, v),
    formed by the server: the result equals the request run alone from the
    same equilibrium computed on the host."""
    from lbc_gb300 import GpuServer
    stream = _stream()[:5]
    srv = GpuServer(0, 64, 60)
    ids = []
    for r in stream:
        case, st, spec = serving.build_request(r)
        ids.append(srv.submit(case, st, r.steps, r.storage, impedance=spec, from_equilibrium=True))
    while srv.poll() > 0:
        pass
    for r, rid in zip(stream, ids):
        assert srv.status(rid)[0] == 3
        res = srv.fetch(rid)
        rho, u, v, spec = _alone(r)
        assert same(res["rho"], rho) and same(res["u"], u) and same(res["v"], v), r
        if spec is not None:
            assert same(res["spectra"], spec)
        srv.release(rid)
    srv.close()


def _max_active_run(srv, stream):
    ids = []
    for r in stream:
        case, st, spec = serving.build_request(r)
        ids.append(srv.submit(case, st, r.steps, r.storage, impedance=spec))
    most = 0
    while srv.poll() > 0:
        most = max(most, srv.stats()["active"])
    return ids, most


def test_admission_follows_live_free_memory():
    """Admission reads the device's free memory every round: a small
    allocation made after the server started holds admissions back (fewer
    requests active at once), no request fails, and every result is the one
    the request gives alone. With the allocation freed, more run at once."""
    torch = pytest.importorskip("torch")
    from lbc_gb300 import GpuServer
    stream = [Req("channel", 1024, 256, 120, 1, 0.0, 3000 + q) for q in range(6)]
    srv = GpuServer(0, 64, 40)
    # One request's estimated footprint (all six are alike).
    case, st, _ = serving.build_request(stream[0])
    rid = srv.submit(case, st, 40, stream[0].storage)
    srv.poll()
    est = srv.stats()["bytes"]
    while srv.poll() > 0:
        pass
    srv.release(rid)
    assert est > 0
    # Leave room for 4.5 requests beyond the reserve, then take 2 of them
    # with an allocation the server knows nothing about.
    total = torch.cuda.mem_get_info()[1]
    reserve0 = total // 20
    avail0 = srv.available()
    assert avail0 > 10 * est
    srv.set_reserve(avail0 + reserve0 - int(4.5 * est))
    extra = torch.empty(2 * est, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    assert srv.available() < 3 * est
    ids, most_held = _max_active_run(srv, stream)
    assert 1 <= most_held <= 2, most_held
    for r, rid in zip(stream, ids):
        assert srv.status(rid)[0] == 3, srv.status(rid)
        res = srv.fetch(rid)
        rho, u, v, _ = _alone(r)
        assert same(res["rho"], rho) and same(res["u"], u) and same(res["v"], v)
        srv.release(rid)
    del extra
    torch.cuda.empty_cache()
    ids, most_free = _max_active_run(srv, stream)
    assert most_free > most_held, (most_free, most_held)
    for rid in ids:
        assert srv.status(rid)[0] == 3
        srv.release(rid)
    srv.close()
