"""Pins of the oracle's phase diagnostics and ground-state sweeps to the reference's own tests:
``classify_phase`` (test/test_diagnostics.jl:250-280), ``pair_amplitude_spectrum``
(test/test_observables.jl:80-125), ``scan_continuation`` (test/test_continuation.jl),
``find_phase_boundary`` (test/test_phase_boundary.jl) and the adaptive-dt ground state
(test/test_adaptive_dt.jl:6-24), plus the step-1 NaN guard of ``_find_ground_state_adaptive``
(src/ground_state.jl:193)."""

import math

import numpy as np
import pytest

import oracle as O


def test_classify_ferromagnetic_f1():  # test/test_diagnostics.jl:255-260
    g = O.make_grid(O.GridConfig((64,), (10.0,)))
    r = O.classify_phase(O.init_psi(g, 1, "ferromagnetic"), 1, g)
    assert r["phase"] == "ferromagnetic"
    assert r["spin_order"] > 0.9


def test_classify_polar_f1():  # test/test_diagnostics.jl:262-268
    g = O.make_grid(O.GridConfig((64,), (10.0,)))
    r = O.classify_phase(O.init_psi(g, 1, "polar"), 1, g)
    assert r["phase"] == "polar"
    assert r["nematic_order"] == pytest.approx(1.0, rel=1e-10)
    assert abs(r["spin_order"]) < 1e-10


def test_classify_ferromagnetic_f2():  # test/test_diagnostics.jl:270-277
    g = O.make_grid(O.GridConfig((32,), (10.0,)))
    assert O.classify_phase(O.init_psi(g, 2, "ferromagnetic"), 2, g)["phase"] == "ferromagnetic"


def test_classify_vacuum():  # src/diagnostics.jl:177-178
    g = O.make_grid(O.GridConfig((16,), (10.0,)))
    r = O.classify_phase(np.zeros((16, 3), dtype=np.complex128), 1, g)
    assert r["phase"] == "vacuum" and r["spin_order"] == 0.0


def test_pair_spectrum_polar_weights():  # test/test_observables.jl:108-115
    g = O.make_grid(O.GridConfig((32,), (10.0,)))
    w = O.pair_amplitude_spectrum(O.init_psi(g, 1, "polar"), 1, g)["channel_weights"]
    tot = w[0] + w[2]
    assert w[0] / tot == pytest.approx(1 / 3, rel=1e-10)
    assert w[2] / tot == pytest.approx(2 / 3, rel=1e-10)


def test_pair_spectrum_ferromagnetic_dominant_s2():  # test/test_observables.jl:117-122
    g = O.make_grid(O.GridConfig((32,), (10.0,)))
    w = O.pair_amplitude_spectrum(O.init_psi(g, 1, "ferromagnetic"), 1, g)["channel_weights"]
    assert w[2] / (w[0] + w[2]) > 0.99


def test_pair_spectrum_interaction_identity():  # test/test_observables.jl:80-101
    """c0 n^2 + c1 |F|^2 = g0 W_0 + g2 W_2 (integrated) for a random spin-1 state."""
    g = O.make_grid(O.GridConfig((32,), (10.0,)))
    rng = np.random.Generator(np.random.PCG64(42))
    psi = (rng.standard_normal((32, 3)) + 1j * rng.standard_normal((32, 3))) / math.sqrt(2)
    psi /= math.sqrt(float(np.sum(np.abs(psi) ** 2)) * O.cell_volume(g))
    c0, c1 = 10.0, -0.5
    dV = O.cell_volume(g)
    n = O.total_density(psi)
    fx, fy, fz = O.spin_density(psi, 1)
    lhs = c0 * float(np.sum(n ** 2)) * dV + c1 * float(np.sum(fx ** 2 + fy ** 2 + fz ** 2)) * dV
    w = O.pair_amplitude_spectrum(psi, 1, g)["channel_weights"]
    rhs = (c0 - 2 * c1) * w[0] + (c0 + c1) * w[2]
    assert lhs == pytest.approx(rhs, rel=1e-10)


def _continuation(values, n_cont, n_fresh, dt):
    g = O.make_grid(O.GridConfig((16,), (10.0,)))
    return O.scan_continuation(param_values=values, make_interactions=lambda v: O.InteractionParams(10.0, v),
                               grid=g, atom=O.Rb87, n_steps_continuation=n_cont, n_steps_fresh=n_fresh, dt=dt,
                               tol=1e-6)


def test_continuation_basic_sweep():  # test/test_continuation.jl:6-27
    res = _continuation([-2.0, -1.0, 0.0, 1.0, 2.0], 100, 500, 0.01)
    assert len(res) == 5
    assert all({"param", "energy", "phase"} <= set(r) for r in res)
    assert res[0]["param"] == -2.0 and res[-1]["param"] == 2.0


def test_continuation_uses_previous_psi():  # test/test_continuation.jl:29-45
    res = _continuation([1.0, 1.01], 100, 500, 0.01)
    assert abs(res[0]["energy"] - res[1]["energy"]) / abs(res[0]["energy"]) < 0.1


def test_continuation_valid_phases():  # test/test_continuation.jl:47-65
    res = _continuation([-5.0, -2.0, 2.0, 5.0], 200, 1000, 0.005)
    assert len(res) == 4
    assert all(r["phase"] in {"ferromagnetic", "polar", "nematic", "cyclic", "mixed", "vacuum"} for r in res)


def test_adaptive_ground_state_matches_fixed():  # test/test_adaptive_dt.jl:6-24
    """Rb87 couplings from scattering lengths (compute_interaction_params) are not restated;
    the 1-D spin-1 c0=10, c1=-0.5 trap ground state stands in for them."""
    g = O.make_grid(O.GridConfig((64,), (15.0,)))
    kw = dict(grid=g, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5), V=O.harmonic_potential(g, (1.0,)),
              dt=0.001, n_steps=5000, tol=1e-8)
    fixed = O.find_ground_state(**kw)
    adapt = O.find_ground_state(adaptive_dt=True, dt_max=0.01, **kw)
    assert abs(fixed["energy"] - adapt["energy"]) / abs(fixed["energy"]) < 0.01
    assert adapt["final_dt"] != 0.001   # the controller moved dt


def test_adaptive_ground_state_nan_guard_at_step_1():  # src/ground_state.jl:193
    g = O.make_grid(O.GridConfig((32,), (10.0,)))
    psi = O.init_psi(g, 1, "polar")
    psi[3, 1] = np.nan
    with pytest.raises(ValueError, match="NaN detected in ITP at step 1"):
        O.find_ground_state(grid=g, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5), psi_init=psi,
                            dt=0.005, n_steps=200, tol=1e-8, adaptive_dt=True)


# ---- find_phase_boundary (src/phase_boundary.jl:9-60), ported from test/test_phase_boundary.jl

def _pb_kw():
    return dict(grid=O.make_grid(O.GridConfig((16,), (10.0,))), atom=O.Rb87, dt=0.01, n_steps=500,
                make_interactions=lambda v: O.InteractionParams(10.0, v))


def test_phase_boundary_returns_valid_result():
    r = O.find_phase_boundary(param_range=(-10.0, 10.0), tol=1.0, max_bisections=5, **_pb_kw())
    assert set(r) == {"boundary_value", "phase_left", "phase_right", "n_evaluations"}
    assert r["n_evaluations"] >= 2
    assert -10.0 <= r["boundary_value"] <= 10.0


def test_phase_boundary_same_phase_returns_midpoint():
    r = O.find_phase_boundary(param_range=(-10.0, -5.0), tol=0.1, max_bisections=3, **_pb_kw())
    assert r["n_evaluations"] == 2
    assert r["phase_left"] == r["phase_right"]
    assert r["boundary_value"] == -7.5


def test_phase_boundary_bisection_narrows_interval():
    r1 = O.find_phase_boundary(param_range=(-20.0, 20.0), tol=5.0, max_bisections=3, **_pb_kw())
    r2 = O.find_phase_boundary(param_range=(-20.0, 20.0), tol=2.0, max_bisections=10, **_pb_kw())
    assert r2["n_evaluations"] >= r1["n_evaluations"]


def test_phase_boundary_bisects_a_ferromagnetic_edge():
    """From the 'uniform' start the spin-mixing step selects the phase: ferromagnetic for c1 < 0,
    another phase for c1 > 0; the bisection keeps the ferromagnetic left end and closes on 0."""
    g = O.make_grid(O.GridConfig((32,), (16.0,)))
    r = O.find_phase_boundary(param_range=(-0.7, 0.4), make_interactions=lambda v: O.InteractionParams(10.0, v),
                              grid=g, atom=O.Rb87, tol=0.05, max_bisections=10, V=O.harmonic_potential(g, (1.0,)),
                              dt=0.01, n_steps=600, initial_state="uniform")
    assert r["phase_left"] == "ferromagnetic" and r["phase_right"] != "ferromagnetic"
    assert r["n_evaluations"] == 2 + 5  # 1.1 halved five times is below 0.05
    assert -0.2 < r["boundary_value"] < 0.2
