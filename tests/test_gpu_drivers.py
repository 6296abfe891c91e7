"""GPU parity of the drivers (FP64 plain form) against the oracle: the ITP
ground-state loop, the leapfrog real-time loop with snapshots, the adaptive
Strang loops (step-change with FSAL, Richardson) and the adaptive Yoshida loop."""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from oracle.spinorbec_oracle import _gaussian
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, make_pair, rel_psi_err

pytestmark = pytest.mark.gpu


def test_ground_state_quickstart_1d(gpu):
    """The 1-D spin-1 Rb87 ITP ground state of the reference README (64 points, box 20)."""
    og = O.make_grid(O.GridConfig((64,), (20.0,)))
    hg = S.make_grid(S.GridConfig((64,), (20.0,)))
    ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                             V=O.harmonic_potential(og, (1.0,)), dt=0.005, n_steps=5000, tol=1e-10)
    rg = S.find_ground_state(grid=hg, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                             potential=S.HarmonicTrap(1.0), dt=0.005, n_steps=5000, tol=1e-10)
    assert rg["converged"] == ro["converged"]
    assert rg["steps"] == ro["steps"]
    assert abs(rg["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * abs(ro["energy"])
    assert rel_psi_err(rg["workspace"].psi, ro["workspace"].psi) < PSI_TOL_FP64


@pytest.mark.parametrize("state", ["ferromagnetic", "random"])
def test_ground_state_2d_zeeman(gpu, state):
    n, L = (32, 32), (16.0, 16.0)
    og = O.make_grid(O.GridConfig(n, L))
    hg = S.make_grid(S.GridConfig(n, L))
    psi0 = O.init_psi(og, 1, state, seed=5)
    kw = dict(dt=0.005, n_steps=400, tol=1e-9, psi_init=psi0)
    ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                             zeeman=O.ZeemanParams(0.5, 0.05), V=O.harmonic_potential(og, (1.0, 1.0)), **kw)
    rg = S.find_ground_state(grid=hg, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                             zeeman=S.ZeemanParams(0.5, 0.05), potential=S.HarmonicTrap(1.0, 1.0), **kw)
    assert abs(rg["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * abs(ro["energy"])
    assert rel_psi_err(rg["workspace"].psi, ro["workspace"].psi) < PSI_TOL_FP64


def test_ground_state_constrained_magnetization(gpu):
    n, L = (64,), (16.0,)
    og = O.make_grid(O.GridConfig(n, L))
    hg = S.make_grid(S.GridConfig(n, L))
    kw = dict(dt=0.005, n_steps=200, tol=1e-9, initial_state="uniform", target_magnetization=0.5)
    ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                             V=O.harmonic_potential(og, (1.0,)), **kw)
    rg = S.find_ground_state(grid=hg, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                             potential=S.HarmonicTrap(1.0), **kw)
    assert abs(S.magnetization(rg["workspace"]) - 0.5) < 1e-10
    assert abs(rg["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * abs(ro["energy"])
    assert rel_psi_err(rg["workspace"].psi, ro["workspace"].psi) < PSI_TOL_FP64


def test_ground_state_tensor_f2(gpu):
    n, L = (32,), (12.0,)
    og = O.make_grid(O.GridConfig(n, L))
    hg = S.make_grid(S.GridConfig(n, L))
    psi0 = O.init_psi(og, 2, "random", seed=3)
    kw = dict(dt=0.005, n_steps=300, tol=1e-9, psi_init=psi0)
    ro = O.find_ground_state(grid=og, atom=O.AtomSpecies("f2", 2),
                             interactions=O.InteractionParams(20.0, 1.0, 0.0, (0.0, 0.0, 2.0)),
                             V=O.harmonic_potential(og, (1.0,)), **kw)
    rg = S.find_ground_state(grid=hg, atom=S.AtomSpecies("f2", 2),
                             interactions=S.InteractionParams(20.0, 1.0, 0.0, (0.0, 0.0, 2.0)),
                             potential=S.HarmonicTrap(1.0), **kw)
    assert abs(rg["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * abs(ro["energy"])
    assert rel_psi_err(rg["workspace"].psi, ro["workspace"].psi) < PSI_TOL_FP64


def test_run_simulation_leapfrog_snapshots(gpu):
    n, L = (32, 32), (16.0, 16.0)
    ws_o, ws_g = make_pair(n, L, 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), zeeman=(0.0, 0.1), dt=1e-3)
    ws_o.sim_params = O.SimParams(1e-3, 45, False, None, 10)
    ws_g.sim_params = S.SimParams(1e-3, 45, False, None, 10)
    calls = []
    ro = O.run_simulation(ws_o)
    rg = S.run_simulation(ws_g, callback=lambda ws, step: calls.append(step))
    assert calls == [10, 20, 30, 40]
    assert len(rg.times) == len(ro.times) == 5
    np.testing.assert_allclose(rg.times, ro.times, rtol=0, atol=1e-15)
    np.testing.assert_allclose(rg.energies, ro.energies, rtol=ENERGY_TOL_FP64 * 10)
    np.testing.assert_allclose(rg.norms, ro.norms, rtol=1e-13)
    np.testing.assert_allclose(rg.magnetizations, ro.magnetizations, atol=1e-12)
    for a, b in zip(rg.psi_snapshots, ro.psi_snapshots):
        assert rel_psi_err(a, b) < PSI_TOL_FP64
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64


def test_run_simulation_itp_standard_loop(gpu):
    ws_o, ws_g = make_pair((64,), (20.0,), 1, c0=10.0, c1=-0.5, omega=(1.0,), dt=5e-3, itp=True)
    ws_o.sim_params = O.SimParams(5e-3, 30, True, None, 10)
    ws_g.sim_params = S.SimParams(5e-3, 30, True, None, 10)
    ro = O.run_simulation(ws_o)
    rg = S.run_simulation(ws_g)
    np.testing.assert_allclose(rg.energies, ro.energies, rtol=ENERGY_TOL_FP64 * 10)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64


@pytest.mark.parametrize("mode", ["step_change", "richardson"])
def test_run_simulation_adaptive(gpu, mode):
    ws_o, ws_g = make_pair((64,), (20.0,), 1, c0=10.0, c1=-0.5, omega=(1.0,), zeeman=(0.1, 0.0),
                           state="ferromagnetic")
    ad_o = O.AdaptiveDtParams(dt_init=0.005, dt_min=1e-4, dt_max=0.05, tol=1e-4, error_mode=mode)
    ad_g = S.AdaptiveDtParams(dt_init=0.005, dt_min=1e-4, dt_max=0.05, tol=1e-4, error_mode=mode)
    ro = O.run_simulation_adaptive(ws_o, ad_o, 0.3, 0.1)
    rg = S.run_simulation_adaptive(ws_g, ad_g, t_end=0.3, save_interval=0.1)
    assert (rg["n_accepted"], rg["n_rejected"]) == (ro["n_accepted"], ro["n_rejected"])
    assert abs(rg["final_dt"] - ro["final_dt"]) <= 1e-9 * ro["final_dt"]
    np.testing.assert_allclose(rg["result"].times, ro["result"].times, rtol=0, atol=1e-12)
    np.testing.assert_allclose(rg["result"].energies, ro["result"].energies, rtol=ENERGY_TOL_FP64 * 10)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64


@pytest.mark.parametrize("ddi", [False, True])
def test_run_simulation_yoshida(gpu, ddi):
    kw = dict(ddi=True, c_dd=20.0) if ddi else {}
    ws_o, ws_g = make_pair((64,), (20.0,), 1, c0=1.0, c1=0.0, omega=(1.0,), zeeman=(0.1, 0.0),
                           state="ferromagnetic", **kw)
    ad_o = O.AdaptiveDtParams(dt_init=0.005, dt_min=1e-4, dt_max=0.05, tol=0.01)
    ad_g = S.AdaptiveDtParams(dt_init=0.005, dt_min=1e-4, dt_max=0.05, tol=0.01)
    ro = O.run_simulation_yoshida(ws_o, ad_o, 0.5, 0.1)
    rg = S.run_simulation_yoshida(ws_g, ad_g, t_end=0.5, save_interval=0.1)
    assert (rg["n_accepted"], rg["n_rejected"]) == (ro["n_accepted"], ro["n_rejected"])
    np.testing.assert_allclose(rg["result"].norms, ro["result"].norms, rtol=1e-13)
    np.testing.assert_allclose(rg["result"].energies, ro["result"].energies, rtol=ENERGY_TOL_FP64 * 10)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    N0, N1 = rg["result"].norms[0], rg["result"].norms[-1]
    assert abs(N1 - N0) / N0 < 1e-6  # test/test_split_step.jl:184-187


def test_yoshida_3d_f6_tensor_ddi_padded(gpu):
    """A scaled-down Eu151-like case: 3-D F=6, tensor couplings (c4), zero-padded DDI, adaptive Yoshida."""
    ip = O.interaction_params_from_constraint(c_total=4689.0, c1_ratio=1 / 36, F=6, c_extra=(0.0, 0.0, 50.0))
    og = O.make_grid(O.GridConfig((8, 8, 8), (24.0, 24.0, 24.0)))
    psi = np.zeros((8, 8, 8, 13), dtype=np.complex128, order="F")
    g = _gaussian(og, (3.0, 3.0, 3.0))
    rng = np.random.Generator(np.random.PCG64(11))
    psi[..., 0] = g * np.exp(1j * 0.01 * rng.standard_normal(g.shape))
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * O.cell_volume(og))
    ws_o, ws_g = make_pair((8, 8, 8), (24.0, 24.0, 24.0), 6, c0=ip.c0, c1=ip.c1, c_extra=ip.c_extra,
                           omega=(1.0, 1.0, 1.2), ddi=True, c_dd=100.0, padded=True, psi=psi)
    ad = dict(dt_init=1e-3, dt_min=1e-5, dt_max=0.01, tol=1e-3)
    ro = O.run_simulation_yoshida(ws_o, O.AdaptiveDtParams(**ad), 0.02, 0.01)
    rg = S.run_simulation_yoshida(ws_g, S.AdaptiveDtParams(**ad), t_end=0.02, save_interval=0.01)
    assert (rg["n_accepted"], rg["n_rejected"]) == (ro["n_accepted"], ro["n_rejected"])
    np.testing.assert_allclose(rg["result"].energies, ro["result"].energies, rtol=ENERGY_TOL_FP64 * 10)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64


def test_multistart_picks_lowest(gpu):
    og = O.make_grid(O.GridConfig((32,), (12.0,)))
    hg = S.make_grid(S.GridConfig((32,), (12.0,)))
    kw = dict(dt=0.005, n_steps=200, tol=1e-8, n_random=2, seed=4)
    ro = O.find_ground_state_multistart(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                                        V=O.harmonic_potential(og, (1.0,)),
                                        initial_states=("polar", "ferromagnetic", "random"), **kw)
    rg = S.find_ground_state_multistart(grid=hg, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                                        potential=S.HarmonicTrap(1.0),
                                        initial_states=("polar", "ferromagnetic", "random"), **kw)
    assert rg["initial_state"] == ro["initial_state"]
    assert abs(rg["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * abs(ro["energy"])
    for a, b in zip(rg["all_results"], ro["all_results"]):
        assert abs(a["energy"] - b["energy"]) <= ENERGY_TOL_FP64 * abs(b["energy"])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ground_state_steps_not_multiple_of_check(gpu, precision):
    """n_steps = 53 with checks every 5 steps: the last block ends at n_steps (no check)."""
    og = O.make_grid(O.GridConfig((64,), (20.0,)))
    hg = S.make_grid(S.GridConfig((64,), (20.0,)))
    kw = dict(dt=0.005, n_steps=53, tol=1e-14)
    ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                             V=O.harmonic_potential(og, (1.0,)), **kw)
    rg = S.find_ground_state(grid=hg, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                             potential=S.HarmonicTrap(1.0), precision=precision, **kw)
    assert rg["steps"] == ro["steps"] == 53
    tol = ENERGY_TOL_FP64 if precision == "fp64" else 1e-6
    assert abs(rg["energy"] - ro["energy"]) <= tol * abs(ro["energy"])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_long_lines_1d_2048(gpu, precision):
    """1-D lines of 2048 points: the fused row pass needs more than the default 48 KB of shared memory."""
    ws_o, ws_g = make_pair((2048,), (40.0,), 1, c0=10.0, c1=0.5, omega=(1.0,), zeeman=(0.0, 0.1), dt=1e-3,
                           precision=precision, state="polar")
    for _ in range(20):
        O.split_step(ws_o)
    S.split_step(ws_g, 20)
    tol = PSI_TOL_FP64 if precision == "fp64" else 5e-5
    assert rel_psi_err(ws_g.psi, ws_o.psi) < tol
