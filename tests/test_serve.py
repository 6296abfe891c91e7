"""Host logic of the request server: admission by HBM budget and slots, request
stream generation, latency statistics.  A fake runner stands in for the device
so these run without a GPU."""

import threading
import time

import pytest

from spinorbec import serve


def _fake_runner(active, lock, peak, service=0.02):
    def run(req):
        with lock:
            active[0] += 1
            peak[0] = max(peak[0], active[0])
        time.sleep(service)
        with lock:
            active[0] -= 1
        return dict(energy=float(req.rid), norm=1.0, converged=True, steps=req.steps)
    return run


def test_poisson_stream_is_seeded_and_in_range():
    a = serve.poisson_requests(200, rate=200.0, seed=3)
    b = serve.poisson_requests(200, rate=200.0, seed=3)
    assert [(r.n_points, r.F, r.c0, r.arrival) for r in a] == [(r.n_points, r.F, r.c0, r.arrival) for r in b]
    arr = [r.arrival for r in a]
    assert arr == sorted(arr)
    mean_gap = arr[-1] / len(arr)
    assert 0.5 / 200 < mean_gap < 2.0 / 200
    for r in a:
        nd = len(r.n_points)
        n = r.n_points[0]
        assert all(m == n for m in r.n_points) and n & (n - 1) == 0
        lo, hi = {1: (256, 4096), 2: (64, 512), 3: (32, 128)}[nd]
        assert lo <= n <= hi
        assert r.F in (1, 2, 6) and r.enable_ddi == (r.F == 6)
        assert 5.0 <= r.c0 <= 20.0 and -1.0 <= r.c1 <= 1.0 and 500 <= r.steps <= 5000
    assert {len(r.n_points) for r in a} == {1, 2, 3}
    assert {r.kind for r in a} == {"ground_state", "dynamics"}


def test_footprint_grows_with_size_precision_and_ddi():
    r = serve.SolveRequest(0, "dynamics", (64, 64, 64), (16.0,) * 3, 6, 10.0, 0.0, 100)
    f32 = serve.footprint_bytes(r)
    r64 = serve.SolveRequest(0, "dynamics", (64, 64, 64), (16.0,) * 3, 6, 10.0, 0.0, 100, precision="fp64")
    assert serve.footprint_bytes(r64) > f32
    rd = serve.SolveRequest(0, "dynamics", (64, 64, 64), (16.0,) * 3, 6, 10.0, 0.0, 100, enable_ddi=True)
    assert serve.footprint_bytes(rd) > f32
    # at least the five psi-sized buffers
    assert f32 >= 5 * 64 ** 3 * 13 * 8


@pytest.mark.parametrize("budget_requests", [1, 3])
def test_admission_respects_budget_and_serves_all(budget_requests):
    reqs = [serve.SolveRequest(i, "dynamics", (256, 256), (20.0, 20.0), 1, 10.0, 0.0, 500, arrival=0.001 * i)
            for i in range(12)]
    fp = serve.footprint_bytes(reqs[0])
    active, peak, lock = [0], [0], threading.Lock()
    srv = serve.Server(hbm_budget_bytes=fp * budget_requests + 1, max_slots=8,
                       runner=_fake_runner(active, lock, peak))
    out = srv.run(reqs, realtime=True)
    assert [r.rid for r in out["results"]] == list(range(12))
    assert peak[0] <= budget_requests and srv.peak_active <= budget_requests
    assert srv.peak_used <= srv.budget
    for r in out["results"]:
        assert r.finished >= r.admitted >= r.arrival - 1e-6
        assert r.energy == float(r.rid)
    assert out["p99_latency_s"] >= out["p50_latency_s"] > 0
    assert out["solves_per_s"] > 0


def test_slots_bound_concurrency():
    reqs = [serve.SolveRequest(i, "ground_state", (64,), (20.0,), 1, 10.0, 0.0, 500) for i in range(10)]
    active, peak, lock = [0], [0], threading.Lock()
    srv = serve.Server(hbm_budget_bytes=1e12, max_slots=2, runner=_fake_runner(active, lock, peak))
    srv.run(reqs, realtime=False)
    assert peak[0] == 2


def test_request_beyond_budget_is_refused():
    req = serve.SolveRequest(0, "dynamics", (128, 128, 128), (16.0,) * 3, 6, 10.0, 0.0, 500)
    srv = serve.Server(hbm_budget_bytes=1e6, runner=lambda r: {})
    with pytest.raises(MemoryError):
        srv.run([req], realtime=False)
