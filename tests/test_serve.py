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


def _gs(rid, arrival, n=(64, 64), F=1, **kw):
    return serve.SolveRequest(rid, "ground_state", n, (20.0,) * len(n), F, 10.0 + rid, 0.1, 500 + 10 * rid,
                              arrival=arrival, **kw)


def test_batch_supported_follows_the_fused_passes(libsbec):
    from spinorbec import api
    from spinorbec.host import GridConfig, make_grid

    assert api.batch_supported(make_grid(GridConfig((256, 256), (20.0, 20.0))), 1)
    assert api.batch_supported(make_grid(GridConfig((512, 512), (20.0, 20.0))), 2)
    assert not api.batch_supported(make_grid(GridConfig((48, 40), (12.0, 10.0))), 1)  # Bluestein axes
    assert not api.batch_supported(make_grid(GridConfig((16, 16, 16), (8.0,) * 3)), 6)  # D = 13
    assert not api.batch_supported(make_grid(GridConfig((4096,), (40.0,))), 1)
    # the nematic c2 rides on the fused passes
    assert api.batch_supported(make_grid(GridConfig((64, 64), (20.0, 20.0))), 2, c2=0.4)


def test_merge_key_admits_only_contact_ground_states(libsbec):
    assert serve.merge_key(_gs(0, 0.0)) is not None
    assert serve.merge_key(_gs(0, 0.0, F=2)) == serve.merge_key(_gs(1, 0.3, F=2))
    assert serve.merge_key(_gs(0, 0.0, F=6)) is None
    assert serve.merge_key(_gs(0, 0.0, enable_ddi=True)) is None
    dyn = serve.SolveRequest(0, "dynamics", (64, 64), (20.0, 20.0), 1, 10.0, 0.0, 500)
    assert serve.merge_key(dyn) is None
    # grid, dt, tol and precision separate keys
    assert serve.merge_key(_gs(0, 0.0)) != serve.merge_key(_gs(0, 0.0, n=(128, 128)))
    assert serve.merge_key(_gs(0, 0.0)) != serve.merge_key(_gs(0, 0.0, dt=0.001))
    assert serve.merge_key(_gs(0, 0.0)) != serve.merge_key(_gs(0, 0.0, tol=1e-6))
    assert serve.merge_key(_gs(0, 0.0)) != serve.merge_key(_gs(0, 0.0, precision="fp64"))
    # grids the batch does not take (a row pass beyond the block limits) are not merged
    assert serve.merge_key(_gs(0, 0.0, n=(4096,))) is None
    assert serve.merge_key(_gs(0, 0.0, n=(2048,), F=2)) is None
    assert serve.merge_key(_gs(0, 0.0, n=(2048,))) is not None


def test_dispatch_units_group_by_key_and_window(libsbec):
    dyn = serve.SolveRequest(9, "dynamics", (64, 64), (20.0, 20.0), 1, 10.0, 0.0, 500, arrival=0.05)
    reqs = [_gs(0, 0.01), _gs(1, 0.02), _gs(2, 0.03, n=(128, 128)), _gs(3, 0.12), _gs(4, 0.09), dyn]
    assert [(t, [r.rid for r in rs]) for t, rs in serve.dispatch_units(reqs)] == \
        [(r.arrival, [r.rid]) for r in sorted(reqs, key=lambda q: q.arrival)]
    units = serve.dispatch_units(reqs, merge_window_s=0.1)
    got = [(round(t, 9), [r.rid for r in rs]) for t, rs in units]
    # window [0, 0.1): 0, 1, 4 share a key, 2 has its own grid; 3 falls in [0.1, 0.2); the
    # dynamics request is dispatched at its arrival
    assert got == [(0.05, [9]), (0.1, [0, 1, 4]), (0.1, [2]), (0.2, [3])]
    # the same arrivals always give the same units
    assert got == [(round(t, 9), [r.rid for r in rs]) for t, rs in serve.dispatch_units(reqs, merge_window_s=0.1)]


def test_dispatch_units_respect_max_merge_and_budget(libsbec):
    reqs = [_gs(i, 0.001 * i) for i in range(7)]
    sizes = [len(rs) for _, rs in serve.dispatch_units(reqs, merge_window_s=1.0, max_merge=3)]
    assert sizes == [3, 3, 1]
    fp = serve.footprint_bytes(reqs[0])
    sizes = [len(rs) for _, rs in serve.dispatch_units(reqs, merge_window_s=1.0, budget_bytes=2.5 * fp)]
    assert sizes == [2, 2, 2, 1]


def test_server_runs_merged_units_through_the_batch_runner(libsbec):
    calls = []

    def batch_runner(rs):
        calls.append([r.rid for r in rs])
        return [dict(energy=100.0 + r.rid, norm=1.0, converged=True, steps=r.steps) for r in rs]

    active, peak, lock = [0], [0], threading.Lock()
    reqs = [_gs(0, 0.001), _gs(1, 0.002), _gs(2, 0.003, F=6), _gs(3, 0.004)]
    srv = serve.Server(hbm_budget_bytes=1e12, max_slots=4, runner=_fake_runner(active, lock, peak),
                       batch_runner=batch_runner, merge_window_s=0.05)
    out = srv.run(reqs, realtime=True)
    assert calls == [[0, 1, 3]]
    assert srv.merged_units == 1 and srv.merged_requests == 3
    res = {r.rid: r for r in out["results"]}
    assert sorted(res) == [0, 1, 2, 3]
    for rid in (0, 1, 3):
        assert res[rid].energy == 100.0 + rid and res[rid].admitted >= 0.05 - 1e-3
        assert res[rid].steps == reqs[rid].steps
    assert res[2].energy == 2.0  # the fake single runner


@pytest.mark.parametrize("policy", ["fifo", "sjf"])
def test_admission_policy_order(policy):
    """One slot: after the first request, the queued ones are admitted in arrival order
    (fifo) or by estimated work (sjf); every request is served either way."""
    order, lock = [], threading.Lock()

    def runner(req):
        with lock:
            order.append(req.rid)
        time.sleep(0.03)
        return dict(energy=0.0, norm=1.0, converged=True, steps=req.steps)

    steps = [3000, 2500, 600, 4000, 500, 1000]
    reqs = [serve.SolveRequest(i, "dynamics", (64, 64), (20.0, 20.0), 1, 10.0, 0.0, st, arrival=0.0)
            for i, st in enumerate(steps)]
    srv = serve.Server(hbm_budget_bytes=1e12, max_slots=1, runner=runner, policy=policy)
    out = srv.run(reqs, realtime=False)
    assert sorted(r.rid for r in out["results"]) == list(range(6))
    rest = order[1:]  # the first admission races with the other threads' arrival in the queue
    if policy == "fifo":
        assert rest == sorted(rest), order
    else:
        assert rest == sorted(rest, key=lambda i: steps[i]), order
    assert srv.peak_active == 1


def test_work_estimate_orders_by_size_steps_and_ddi():
    small = serve.SolveRequest(0, "dynamics", (64, 64), (20.0, 20.0), 1, 10.0, 0.0, 500)
    longer = serve.SolveRequest(1, "dynamics", (64, 64), (20.0, 20.0), 1, 10.0, 0.0, 5000)
    bigger = serve.SolveRequest(2, "dynamics", (256, 256), (20.0, 20.0), 1, 10.0, 0.0, 500)
    f6 = serve.SolveRequest(3, "dynamics", (64, 64), (20.0, 20.0), 6, 10.0, 0.0, 500)
    f6d = serve.SolveRequest(4, "dynamics", (64, 64), (20.0, 20.0), 6, 10.0, 0.0, 500, enable_ddi=True)
    w = serve.work_estimate
    assert w(small) < w(longer) and w(small) < w(bigger) and w(small) < w(f6) < w(f6d)
    with pytest.raises(ValueError):
        serve.Server(policy="lifo")


def test_batch_eligibility_takes_a_nematic_c2():
    """find_ground_state_multistart / find_phase_boundary route spin-1/2 contact couplings,
    the nematic c2 included, through a batch; higher c_extra entries and DDI keep the
    one-at-a-time loop."""
    from spinorbec import api
    from spinorbec.host import AtomSpecies, InteractionParams

    f2 = AtomSpecies("f2", 2)
    assert api._nematic_c2(InteractionParams(10.0, 0.5)) == 0.0
    assert api._nematic_c2(InteractionParams(10.0, 0.5, 0.0, (0.4,))) == 0.4
    assert api._nematic_c2(InteractionParams(10.0, 0.5, 0.0, (0.4, 0.0, 0.2))) is None
    assert api._batch_eligible(f2, InteractionParams(10.0, 0.5, 0.0, (0.4,)), {})
    assert not api._batch_eligible(f2, InteractionParams(10.0, 0.5, 0.0, (0.4, 0.0, 0.2)), {})
    assert not api._batch_eligible(f2, InteractionParams(10.0, 0.5, 0.0, (0.4,)), {"enable_ddi": True})
    assert not api._batch_eligible(AtomSpecies("f3", 3), InteractionParams(10.0, 0.5), {})
