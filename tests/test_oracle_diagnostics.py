"""Pins of the oracle's ``estimate_splitting_error`` and ``validate_conservation``
(src/diagnostics.jl:214-293) to the reference's own tests (test/test_diagnostics.jl:206-249)."""

import numpy as np

import oracle as O


def _ws(dt):
    g = O.make_grid(O.GridConfig((64,), (10.0,)))
    return O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                            V=O.harmonic_potential(g, (1.0,)), sim_params=O.SimParams(dt, 10, False, None, 10))


def test_splitting_error_shrinks_with_dt():  # test/test_diagnostics.jl:206-223
    err1 = O.estimate_splitting_error(_ws(0.01))
    err2 = O.estimate_splitting_error(_ws(0.005))
    assert err1 > 0 and err2 > 0 and err2 < err1
    # second order: halving dt divides the one-step difference by about four (1 dt vs 2 dt/2)
    assert 2.0 < err1 / err2 < 8.0


def test_splitting_error_restores_state():
    ws = _ws(0.01)
    psi0, t0, s0 = ws.psi.copy(), ws.t, ws.step
    O.estimate_splitting_error(ws)
    assert np.array_equal(ws.psi, psi0) and ws.t == t0 and ws.step == s0
    assert ws.sim_params.dt == 0.01


def test_conservation_passes_for_reasonable_dt():  # test/test_diagnostics.jl:231-238
    r = O.validate_conservation(_ws(0.001), n_steps=50)
    assert r["passed"]
    assert r["norm_drift"] < 1e-12


def test_conservation_restores_state():  # test/test_diagnostics.jl:240-248
    ws = _ws(0.001)
    psi0 = ws.psi.copy()
    O.validate_conservation(ws, n_steps=20)
    assert np.allclose(ws.psi, psi0)
