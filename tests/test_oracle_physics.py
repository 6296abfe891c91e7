"""Pins the oracle's dynamics to the reference's invariant and known-answer tests:
conservation laws (test/test_physics_level1.jl, test/test_split_step.jl), splitting
orders, DDI (test/test_ddi.jl, test/test_ddi_padded.jl), tensor interaction
(test/test_tensor_interaction.jl), analytic energies and constrained normalisation
(test/test_analytical_validation.jl), spin mixing (test/test_spin_mixing.jl),
batched kinetic step (test/test_batched_kinetic.jl) and ground states
(test/test_simulation.jl, test/test_analytic_ground_states.jl)."""

import math

import numpy as np
import pytest
import scipy.fft as sfft

import oracle as O


def ws1d(n=128, L=20.0, F=1, c0=1.0, c1=0.1, state="polar", dt=1e-3, itp=False, zeeman=(0.0, 0.0), omega=None,
         **kw):
    g = O.make_grid(O.GridConfig((n,), (L,)))
    psi = O.init_psi(g, F, state)
    V = O.harmonic_potential(g, omega) if omega else None
    return O.make_workspace(grid=g, atom=O.AtomSpecies("x", F), interactions=O.InteractionParams(c0, c1),
                            zeeman=O.ZeemanParams(*zeeman), V=V, sim_params=O.SimParams(dt, 10, itp),
                            psi_init=psi, **kw)


def test_energy_and_norm_conservation_rt():  # test/test_split_step.jl:5-47
    ws = ws1d(c0=1.0, c1=0.1)
    E0 = O.total_energy(ws)
    for _ in range(100):
        O.split_step(ws)
    assert abs(O.total_energy(ws) - E0) / abs(E0) < 1e-4
    ws = ws1d(c0=0.5, c1=0.05, state="uniform")
    N0 = O.total_norm(ws.psi, ws.grid)
    for _ in range(200):
        O.split_step(ws)
    assert abs(O.total_norm(ws.psi, ws.grid) - N0) / N0 < 1e-10


def _energy_error(dt, integrator, T=0.1):
    ws = ws1d(c0=1.0, c1=0.1, dt=dt)
    E0 = O.total_energy(ws)
    for _ in range(round(T / dt)):
        if integrator == "strang":
            O.split_step(ws)
        else:
            O.yoshida_core(ws, dt)
            ws.t += dt
    return abs(O.total_energy(ws) - E0)


def test_strang_order():  # test/test_split_step.jl:49-78
    e = [_energy_error(dt, "strang") for dt in (0.01, 0.005, 0.0025)]
    assert e[0] / e[1] > 3.0 and e[1] / e[2] > 3.0


def test_yoshida_order_and_conservation():  # test/test_split_step.jl:80-188
    ey = [_energy_error(dt, "yoshida") for dt in (0.02, 0.01, 0.005)]
    es = [_energy_error(dt, "strang") for dt in (0.02, 0.01)]
    assert ey[0] / ey[1] > 6 and ey[1] / ey[2] > 6
    assert ey[0] / ey[1] > (es[0] / es[1]) * 1.5
    ws = ws1d(c0=1.0, c1=0.1, dt=0.01)
    E0 = O.total_energy(ws)
    for _ in range(100):
        O.yoshida_core(ws, 0.01)
        ws.t += 0.01
    assert abs(O.total_energy(ws) - E0) / abs(E0) < 1e-4
    ws = ws1d(c0=0.5, c1=0.05, state="uniform", dt=0.01)
    N0 = O.total_norm(ws.psi, ws.grid)
    for _ in range(200):
        O.yoshida_core(ws, 0.01)
    assert abs(O.total_norm(ws.psi, ws.grid) - N0) / N0 < 1e-10


def test_yoshida_adaptive_1d():  # test/test_split_step.jl:159-188
    ws = ws1d(n=64, c0=1.0, c1=0.0, state="ferromagnetic", dt=0.01, zeeman=(0.1, 0.0))
    r = O.run_simulation_yoshida(ws, O.AdaptiveDtParams(dt_init=0.005, dt_min=1e-4, dt_max=0.05, tol=0.01), 0.5, 0.1)
    assert r["n_accepted"] > 0 and len(r["result"].times) >= 2
    N = r["result"].norms
    assert abs(N[-1] - N[0]) / N[0] < 1e-6


def test_level1_conservation_2000_steps():  # test/test_physics_level1.jl:6-82
    kw = dict(c0=10.0, c1=-0.5, dt=0.002, zeeman=(0.0, 0.1), omega=(1.0,))
    ws = ws1d(state="uniform", **kw)
    N0 = O.total_norm(ws.psi, ws.grid)
    for _ in range(2000):
        O.split_step(ws)
    assert abs(O.total_norm(ws.psi, ws.grid) - N0) / N0 < 1e-12
    ws = ws1d(state="polar", **kw)
    E0 = O.total_energy(ws)
    for _ in range(2000):
        O.split_step(ws)
    assert abs(O.total_energy(ws) - E0) / abs(E0) < 0.001
    ws = ws1d(state="ferromagnetic", **kw)
    M0 = O.magnetization(ws.psi, ws.grid, 1)
    for _ in range(2000):
        O.split_step(ws)
    assert abs(O.magnetization(ws.psi, ws.grid, 1) - M0) < 1e-10


def test_q_tensor_symmetric_traceless_and_secular():  # test/test_ddi.jl:2-18, 104-129
    g = O.make_grid(O.GridConfig((16, 16, 16), (10.0, 10.0, 10.0)))
    full = O.make_ddi_params(g, 1.0).Q
    sec = O.make_ddi_params(g, 1.0, secular=True).Q
    kx = O.rfftfreq(16, 16 * g.dk[0])
    K2 = kx[:, None, None] ** 2 + g.k[1][None, :, None] ** 2 + g.k[2][None, None, :] ** 2
    nz = K2 > 0
    assert np.max(np.abs((full["xx"] + full["yy"] + full["zz"])[nz])) < 1e-12
    for k in ("xy", "xz", "yz"):
        assert np.max(np.abs(sec[k])) == 0.0
    assert np.allclose(sec["zz"], full["zz"])
    assert np.allclose(sec["xx"], sec["yy"]) and np.allclose(sec["xx"], -sec["zz"] / 2)
    assert np.max(np.abs((sec["xx"] + sec["yy"] + sec["zz"])[nz])) < 1e-12


def _ddi_ws(n, L, state, c_dd=5.0, secular=False, padded=False):
    g = O.make_grid(O.GridConfig(n, L))
    psi = O.init_psi(g, 1, state)
    return O.make_workspace(grid=g, atom=O.AtomSpecies("x", 1), interactions=O.InteractionParams(0.0, 0.0),
                            sim_params=O.SimParams(1e-3, 1), psi_init=psi, enable_ddi=True, c_dd=c_dd,
                            secular_ddi=secular, ddi_padding=padded)


def test_ddi_conservation():  # test/test_ddi.jl:39-102, 131-145
    ws = _ddi_ws((64,), (20.0,), "uniform")
    N0 = O.total_norm(ws.psi, ws.grid)
    O.apply_ddi_step(ws, 0.001, False)
    assert abs(O.total_norm(ws.psi, ws.grid) - N0) / N0 < 1e-10
    ws = _ddi_ws((64,), (20.0,), "ferromagnetic")
    M0 = O.magnetization(ws.psi, ws.grid, 1)
    O.apply_ddi_step(ws, 0.001, False)
    assert abs(O.magnetization(ws.psi, ws.grid, 1) - M0) < 1e-10
    ws = _ddi_ws((64,), (20.0,), "uniform", c_dd=0.0)
    p0 = ws.psi.copy()
    O.apply_ddi_step(ws, 0.01, False)
    assert np.max(np.abs(ws.psi - p0)) < 1e-12
    for sec in (False, True):
        ws = _ddi_ws((16, 16, 16), (10.0, 10.0, 10.0), "uniform", secular=sec)
        N0 = O.total_norm(ws.psi, ws.grid)
        O.apply_ddi_step(ws, 0.001, False)
        assert abs(O.total_norm(ws.psi, ws.grid) - N0) / N0 < 1e-10


def test_secular_equals_full_for_z_polarised():  # test/test_ddi.jl:147-166
    # the reference runs this with compute_c_dd(Eu151) = mu0 * mu^2 in SI units
    c_dd_si = 4e-7 * math.pi * (7.0 * 9.2740100783e-24) ** 2
    a = _ddi_ws((16, 16, 16), (10.0, 10.0, 10.0), "ferromagnetic", c_dd=c_dd_si)
    b = _ddi_ws((16, 16, 16), (10.0, 10.0, 10.0), "ferromagnetic", c_dd=c_dd_si, secular=True)
    O.apply_ddi_step(a, 0.001, False)
    O.apply_ddi_step(b, 0.001, False)
    assert np.max(np.abs(a.psi - b.psi)) < 1e-12


def test_ddi_padded_shapes_and_localised_agreement():  # test/test_ddi_padded.jl:2-76
    g = O.make_grid(O.GridConfig((64,), (20.0,)))
    ctx = O.make_ddi_padded(g, 1.0)
    assert ctx.padded_shape == (128,) and ctx.Q["xx"].shape == O.rfft_output_shape((128,))
    g2 = O.make_grid(O.GridConfig((32, 32), (10.0, 10.0)))
    assert O.make_ddi_padded(g2, 1.0).padded_shape == (64, 64)
    a = _ddi_ws((64,), (20.0,), "ferromagnetic", c_dd=5.0, padded=True)
    b = _ddi_ws((64,), (20.0,), "ferromagnetic", c_dd=5.0)
    for _ in range(10):
        O.apply_ddi_step(a, 0.001, False)
        O.apply_ddi_step(b, 0.001, False)
    assert abs(O.total_norm(a.psi, a.grid) - 1.0) < 1e-4
    assert np.max(np.abs(a.psi - b.psi)) < 0.1


def test_ddi_energy_zero_uniform_polarised():  # test/test_analytical_validation.jl:50-73
    g = O.make_grid(O.GridConfig((16, 16, 16), (10.0, 10.0, 10.0)))
    n0 = 1.0 / 1000.0
    psi = np.zeros((16, 16, 16, 3), dtype=np.complex128, order="F")
    psi[..., 0] = math.sqrt(n0)
    ws = O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(0.0, 0.0),
                          sim_params=O.SimParams(0.01, 1), psi_init=psi, enable_ddi=True, c_dd=1.0)
    assert abs(O.energy_terms(ws)["ddi"]) < 1e-12


def test_uniform_interaction_energies_f1():  # test/test_analytical_validation.jl:9-48
    g = O.make_grid(O.GridConfig((64,), (10.0,)))
    n0 = 1.0 / 10.0
    for comps, c1_expected in (({0: 1.0}, 1.0), ({1: 1.0}, 0.0), ({0: 0.5, 2: 0.5}, 0.0)):
        psi = np.zeros((64, 3), dtype=np.complex128, order="F")
        for c, frac in comps.items():
            psi[:, c] = math.sqrt(n0 * frac) * (-1 if c == 2 else 1)
        ws = O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(100.0, 10.0),
                              sim_params=O.SimParams(0.01, 1), psi_init=psi)
        e = O.energy_terms(ws)
        assert e["c0"] == pytest.approx(0.5 * 100.0 * n0 ** 2 * 10.0, rel=1e-10)
        if c1_expected:
            assert e["c1"] == pytest.approx(0.5 * 10.0 * n0 ** 2 * 10.0, rel=1e-10)
        else:
            assert abs(e["c1"]) < 1e-12


def test_tensor_equals_spin_mixing_f1():  # test/test_analytical_validation.jl:197-241
    g = O.make_grid(O.GridConfig((64,), (10.0,)))
    dV = O.cell_volume(g)
    rng = np.random.default_rng(42)
    psi = (rng.standard_normal((64, 3)) + 1j * rng.standard_normal((64, 3))) / math.sqrt(2)
    psi = np.asfortranarray(psi / math.sqrt(np.sum(np.abs(psi) ** 2) * dV))
    ws = O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(100.0, 10.0),
                          sim_params=O.SimParams(0.001, 1), psi_init=psi)
    e = O.energy_terms(ws)
    cache = O.make_tensor_cache_from_channels(1, O.c0c1_to_gS(1, 100.0, 10.0))
    assert e["c0"] + e["c1"] == pytest.approx(O.tensor_interaction_energy(psi, cache, dV), rel=1e-10)
    ws_sm = O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(0.0, 10.0),
                             sim_params=O.SimParams(0.001, 1), psi_init=psi)
    ws_t = O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(0.0, 0.0),
                            sim_params=O.SimParams(0.001, 1), psi_init=psi)
    ws_t.tensor_cache = O.make_tensor_cache_from_channels(1, O.c0c1_to_gS(1, 0.0, 10.0))
    for _ in range(10):
        O.apply_spin_mixing_step(ws_sm, 0.001, False)
        O.apply_tensor_interaction_step(ws_t, 0.001, False)
    assert np.allclose(ws_sm.psi, ws_t.psi, rtol=1e-4, atol=1e-4 * np.max(np.abs(ws_sm.psi)))


def test_tensor_norm_conservation():  # test/test_tensor_interaction.jl:64-85
    g = O.make_grid(O.GridConfig((32,), (10.0,)))
    dV = O.cell_volume(g)
    rng = np.random.default_rng(5)
    psi = np.asfortranarray(rng.standard_normal((32, 5)) + 1j * rng.standard_normal((32, 5)))
    ws = O.make_workspace(grid=g, atom=O.AtomSpecies("x", 2), interactions=O.InteractionParams(0.0, 0.0, 0.0,
                          (5.0, 0.0, 3.0)), sim_params=O.SimParams(0.01, 1), psi_init=psi)
    assert ws.tensor_cache is not None
    n0 = float(np.sum(np.abs(ws.psi) ** 2)) * dV
    for _ in range(50):
        O.apply_tensor_interaction_step(ws, 0.01, False)
    assert float(np.sum(np.abs(ws.psi) ** 2)) * dV == pytest.approx(n0, rel=1e-8)


def test_workspace_tensor_activation_zeroes_c0_c1():  # test/test_tensor_interaction.jl:238-259
    g = O.make_grid(O.GridConfig((32,), (10.0,)))
    ws = O.make_workspace(grid=g, atom=O.AtomSpecies("x", 2), interactions=O.InteractionParams(100.0, 10.0, 0.0,
                          (0.0, 0.0, 5.0)), sim_params=O.SimParams(0.001, 1))
    assert ws.tensor_cache is not None and ws.interactions.c0 == 0.0 and ws.interactions.c1 == 0.0


@pytest.mark.parametrize("F,target", [(1, 0.5), (6, 3.0)])
def test_constrained_normalisation(F, target):  # test/test_analytical_validation.jl:302-326
    g = O.make_grid(O.GridConfig((64,), (10.0,)))
    dV = O.cell_volume(g)
    n0 = 0.1
    D = 2 * F + 1
    psi = np.zeros((64, D), dtype=np.complex128, order="F")
    if F == 1:
        for c, frac in enumerate((0.7, 0.2, 0.1)):
            psi[:, c] = math.sqrt(n0 * frac)
    else:
        psi[:, :] = math.sqrt(n0 / D)
    O.normalize_psi_constrained(psi, g, target, F)
    Mz = sum((F - c) * float(np.sum(np.abs(psi[:, c]) ** 2)) * dV for c in range(D))
    assert Mz == pytest.approx(target, abs=1e-10)


def test_spin_mixing_conservation_and_identity():  # test/test_spin_mixing.jl:6-81
    for F in (1, 2):
        ws = ws1d(n=64, F=F, c0=0.0, c1=0.5, state="random")
        N0 = O.total_norm(ws.psi, ws.grid)
        M0 = O.magnetization(ws.psi, ws.grid, F)
        for _ in range(10):
            O.apply_spin_mixing_step(ws, 0.01, False)
        assert O.total_norm(ws.psi, ws.grid) == pytest.approx(N0, abs=1e-12)
        assert O.magnetization(ws.psi, ws.grid, F) == pytest.approx(M0, abs=1e-12)
    ws = ws1d(n=64, c0=0.0, c1=0.0, state="random")
    p0 = ws.psi.copy()
    O.apply_spin_mixing_step(ws, 0.01, False)
    assert np.max(np.abs(ws.psi - p0)) < 1e-14
    sm = O.spin_matrices(2)
    sp = np.array([[0.3 + 0.1j, 0.2, 0.5j, 0.1, 0.4]])
    out = O.euler_spin_rotation(sp, np.array([1e-20]), np.array([0.0]), np.array([0.0]), 0.01, sm, False)
    assert np.max(np.abs(out - sp)) < 1e-14


@pytest.mark.parametrize("n,L", [((64,), (20.0,)), ((16, 32), (8.0, 12.0))])
def test_batched_kinetic_equals_per_component(n, L):  # test/test_batched_kinetic.jl:2-40
    g = O.make_grid(O.GridConfig(n, L))
    psi = O.init_psi(g, 1, "random", seed=2)
    ws = O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(1.0, 0.0),
                          sim_params=O.SimParams(0.01, 1), psi_init=psi)
    ref = psi.copy()
    ax = tuple(range(len(n)))
    for c in range(3):
        ref[..., c] = sfft.ifftn(sfft.fftn(psi[..., c], axes=ax) * ws.kinetic_phase, axes=ax)
    O.apply_kinetic_step_batched(ws)
    assert np.allclose(ws.psi, ref, rtol=1e-12, atol=1e-14)


def test_free_gaussian_spreads_and_itp_phase_bounds():  # test/test_propagators.jl:5-43
    ws = ws1d(n=128, c0=0.0, c1=0.0, dt=0.01)
    x = ws.grid.x[0]
    dV = O.cell_volume(ws.grid)

    def width(p):
        d = np.sum(np.abs(p) ** 2, axis=-1)
        return math.sqrt(float(np.sum(d * x ** 2) * dV))

    w0 = width(ws.psi)
    for _ in range(50):
        O.apply_kinetic_step_batched(ws)
    assert O.total_norm(ws.psi, ws.grid) == pytest.approx(1.0, abs=1e-10)
    assert width(ws.psi) > w0
    ph = O.prepare_kinetic_phase(ws.grid, 0.01, True)
    assert np.all(ph.real >= 0) and np.all(ph.real <= 1) and np.all(ph.imag == 0)


def test_ground_states_f1():  # test/test_simulation.jl:6-48, test/test_analytic_ground_states.jl:8-69
    g = O.make_grid(O.GridConfig((64,), (10.0,)))
    dV = O.cell_volume(g)
    V = O.harmonic_potential(g, (1.0,))
    r = O.find_ground_state(grid=g, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                            zeeman=O.ZeemanParams(1.0, 0.0), V=V, dt=0.005, n_steps=2000,
                            initial_state="ferromagnetic")
    pops = [float(np.sum(np.abs(r["workspace"].psi[:, c]) ** 2)) * dV for c in range(3)]
    assert pops[0] > 0.9
    r = O.find_ground_state(grid=g, atom=O.Na23, interactions=O.InteractionParams(10.0, 0.5), V=V, dt=0.005,
                            n_steps=2000, initial_state="polar")
    assert float(np.sum(np.abs(r["workspace"].psi[:, 1]) ** 2)) * dV > 0.9
    ef = O.find_ground_state(grid=g, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5), V=V, dt=0.005,
                             n_steps=1500, initial_state="ferromagnetic")["energy"]
    ep = O.find_ground_state(grid=g, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5), V=V, dt=0.005,
                             n_steps=1500, initial_state="polar")["energy"]
    assert ef < ep


def test_itp_validation_and_nan_detection():  # test/test_analytical_validation.jl:260-300
    with pytest.raises(ValueError):
        O.validate_itp_interactions(O.InteractionParams(1e6, 0.0), 1, 0.01)
    O.validate_itp_interactions(O.InteractionParams(100.0, 10.0), 1, 0.001)
    with pytest.raises(ValueError):
        O.validate_itp_interactions(O.InteractionParams(1.0, 0.0), 6, 0.01, c_dd=1e5)
    O.validate_itp_interactions(O.InteractionParams(100.0, 10.0), 1, 0.001, c_dd=10.0)
    g = O.make_grid(O.GridConfig((16,), (10.0,)))
    psi = np.zeros((16, 3), dtype=np.complex128, order="F")
    psi[0, 0] = np.nan
    ws = O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(100.0, 0.0),
                          sim_params=O.SimParams(0.001, 1, True), psi_init=psi)
    with pytest.raises(ValueError):
        O.check_itp_overflow(ws, 1)
