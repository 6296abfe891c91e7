"""Served solves on the device: each request's result is the same alone and in a
mix of concurrently running requests, and a served FP32 ground state is within
1e-6 (energy) of the same solve in the plain FP64 form."""

import pytest

from spinorbec import serve

pytestmark = pytest.mark.gpu

# Small, mixed requests: 1-D / 2-D / 3-D, F = 1, 2, 6 (DDI on), ground states and dynamics.
MIX = [
    serve.SolveRequest(0, "ground_state", (256,), (40.0,), 1, 10.0, -0.5, 600, dt=0.005),
    serve.SolveRequest(1, "dynamics", (64, 64), (20.0, 20.0), 1, 12.0, 0.5, 300, dt=1e-3),
    serve.SolveRequest(2, "ground_state", (64, 64), (20.0, 20.0), 2, 8.0, 0.3, 500, dt=0.005),
    serve.SolveRequest(3, "dynamics", (16, 16, 16), (16.0,) * 3, 6, 6.0, 0.1, 200, dt=1e-3, enable_ddi=True,
                       c_dd=20.0),
    serve.SolveRequest(4, "ground_state", (16, 16, 16), (16.0,) * 3, 6, 6.0, -0.2, 300, dt=0.005,
                       enable_ddi=True, c_dd=20.0),
    serve.SolveRequest(5, "dynamics", (512,), (40.0,), 2, 15.0, -0.8, 400, dt=1e-3),
]


def test_same_result_alone_and_in_mix(gpu):
    alone = {r.rid: serve.run_request(r) for r in MIX}
    srv = serve.Server(hbm_budget_bytes=4e9, max_slots=4)
    mixed = srv.run(MIX, realtime=False)
    assert srv.peak_active >= 2  # the requests really overlapped
    for res in mixed["results"]:
        a = alone[res.rid]
        # the engine is deterministic: the tolerance is exact equality
        assert res.energy == a["energy"], (res.rid, res.energy, a["energy"])
        assert res.norm == a["norm"], (res.rid, res.norm, a["norm"])
        assert res.steps == a["steps"]


def test_served_fp32_ground_state_energy_matches_fp64(gpu):
    reqs = [MIX[0], MIX[2]]
    for r in reqs:
        r64 = serve.SolveRequest(**{**r.__dict__, "precision": "fp64"})
        e32 = serve.run_request(r)["energy"]
        e64 = serve.run_request(r64)["energy"]
        assert abs(e32 - e64) / abs(e64) < 1e-6, (r.rid, e32, e64)


def _same_key(precision):
    return [serve.SolveRequest(10 + i, "ground_state", (64, 64), (20.0, 20.0), 1, c0, c1, st, dt=0.005,
                               precision=precision, arrival=0.001 * i)
            for i, (c0, c1, st) in enumerate([(10.0, -0.5, 600), (14.0, 0.4, 900), (7.0, 0.1, 450)])]


def test_merged_ground_states_match_single_requests_fp64(gpu):
    """Requests of one merge_key run as one batch give each request's own find_ground_state."""
    reqs = _same_key("fp64")
    merged = serve.run_batch(reqs)
    for r, m in zip(reqs, merged):
        a = serve.run_request(r)
        assert m["steps"] == a["steps"] and m["converged"] == a["converged"]
        assert abs(m["energy"] - a["energy"]) <= 1e-12 * abs(a["energy"])
        assert abs(m["norm"] - a["norm"]) <= 1e-12


def test_served_merged_fp32_deterministic_and_within_1e6_of_fp64(gpu):
    reqs = _same_key("fp32")
    direct = serve.run_batch(reqs)
    srv = serve.Server(hbm_budget_bytes=4e9, max_slots=4, merge_window_s=0.05)
    out = srv.run(reqs, realtime=True)
    assert srv.merged_units == 1 and srv.merged_requests == 3
    for res, d, r in zip(out["results"], direct, reqs):
        assert res.energy == d["energy"] and res.steps == d["steps"]  # same batch, same kernels
        e64 = serve.run_request(serve.SolveRequest(**{**r.__dict__, "precision": "fp64"}))["energy"]
        assert abs(res.energy - e64) / abs(e64) < 1e-6, (r.rid, res.energy, e64)
