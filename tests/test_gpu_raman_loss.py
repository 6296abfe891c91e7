"""GPU parity of the Raman coupling (src/raman.jl:8-31, inside the half potential around the
DDI step, src/split_step.jl:77-103) and the density-dependent losses (src/losses.jl:25-97,
after each real-time step: split_step.jl:21-23, simulation.jl:74-76, adaptive.jl:151-153,
262-264, yoshida.jl:64-66) against the oracle, which is pinned to test/test_raman.jl and
test/test_losses.jl."""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, make_pair, rel_psi_err

pytestmark = pytest.mark.gpu

RAMAN_1D = (2.0, 0.3, (1.7,))
RAMAN_2D = (2.0, -0.2, (1.3, 0.4))


@pytest.mark.parametrize("n,L,F,raman,kw", [
    ((64,), (16.0,), 1, RAMAN_1D, dict(c0=10.0, c1=-0.5)),
    ((32, 32), (12.0, 12.0), 1, RAMAN_2D, dict(c0=10.0, c1=0.5, zeeman=(0.1, 0.05))),
    ((64,), (16.0,), 2, RAMAN_1D, dict(c0=10.0, c1=0.4)),
    ((16, 16), (10.0, 10.0), 1, RAMAN_2D, dict(c0=10.0, c1=0.3, ddi=True, c_dd=30.0)),
    ((8, 8, 8), (8.0, 8.0, 8.0), 6, (1.5, 0.1, (0.9, 0.0, 0.5)),
     dict(c0=4689.0 / 2, c1=4689.0 / 72, c_extra=(0.0, 0.0, 50.0), ddi=True, c_dd=100.0, padded=True)),
])
@pytest.mark.parametrize("itp", [False, True])
def test_split_steps_with_raman(gpu, n, L, F, raman, kw, itp):
    ws_o, ws_g = make_pair(n, L, F, omega=(1.0,) * len(n), raman=raman, itp=itp, dt=1e-3, **kw)
    for _ in range(10):
        O.split_step(ws_o)
    S.split_step(ws_g, 10)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    Eo = O.total_energy(ws_o)
    assert abs(S.total_energy(ws_g) - Eo) <= ENERGY_TOL_FP64 * 10 * abs(Eo)
    assert abs(S.energy_terms(ws_g)["raman"] - O.energy_terms(ws_o)["raman"]) <= 1e-12 * max(1.0, abs(Eo))
    ws_g.close()


def test_raman_fp32(gpu):
    ws_o, ws_g = make_pair((32, 32), (12.0, 12.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), raman=RAMAN_2D,
                           precision="fp32", dt=1e-3)
    for _ in range(50):
        O.split_step(ws_o)
    S.split_step(ws_g, 50)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < 5e-5
    ws_g.close()


def test_ground_state_with_raman(gpu):
    og = O.make_grid(O.GridConfig((64,), (16.0,)))
    hg = S.make_grid(S.GridConfig((64,), (16.0,)))
    psi0 = O.init_psi(og, 1, "random", seed=2)
    ro_ws = O.make_workspace(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                             V=O.harmonic_potential(og, (1.0,)), sim_params=O.SimParams(0.005, 200, True),
                             psi_init=psi0, raman=O.RamanCoupling(*RAMAN_1D))
    rg_ws = S.make_workspace(grid=hg, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                             potential=S.HarmonicTrap(1.0), sim_params=S.SimParams(0.005, 200, True, 1, 20),
                             psi_init=psi0, raman=S.RamanCoupling(*RAMAN_1D))
    for _ in range(200):
        O.split_step(ro_ws)
    S.split_step(rg_ws, 200)
    assert rel_psi_err(rg_ws.psi, ro_ws.psi) < PSI_TOL_FP64
    assert abs(S.total_energy(rg_ws) - O.total_energy(ro_ws)) <= ENERGY_TOL_FP64 * 10 * abs(O.total_energy(ro_ws))
    rg_ws.close()


@pytest.mark.parametrize("F,loss", [(1, (0.5, 0.0)), (1, (0.0, 0.2)), (2, (0.3, 0.05)), (6, (0.4, 0.0))])
def test_leapfrog_with_losses(gpu, F, loss):
    n, L = ((32, 32), (12.0, 12.0)) if F < 6 else ((8, 8, 8), (8.0, 8.0, 8.0))
    kw = dict(c0=10.0, c1=0.5) if F < 6 else dict(c0=4689.0 / 2, c1=4689.0 / 72, c_extra=(0.0, 0.0, 50.0))
    ws_o, ws_g = make_pair(n, L, F, omega=(1.0,) * len(n), zeeman=(0.0, 0.1), loss=loss, dt=1e-3, **kw)
    ws_o.sim_params = O.SimParams(1e-3, 30, False, None, 10)
    ws_g.sim_params = S.SimParams(1e-3, 30, False, None, 10)
    ro = O.run_simulation(ws_o)
    rg = S.run_simulation(ws_g)
    np.testing.assert_allclose(rg.norms, ro.norms, rtol=1e-13)
    assert rg.norms[-1] < rg.norms[0] * (1 - 1e-6)  # atoms are lost
    np.testing.assert_allclose(rg.energies, ro.energies, rtol=ENERGY_TOL_FP64 * 10)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    ws_g.close()


def test_split_steps_with_losses_and_raman(gpu):
    ws_o, ws_g = make_pair((64,), (16.0,), 1, c0=10.0, c1=0.5, omega=(1.0,), raman=RAMAN_1D, loss=(0.5, 0.1),
                           dt=1e-3)
    for _ in range(20):
        O.split_step(ws_o)
    S.split_step(ws_g, 20)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    ws_g.close()


@pytest.mark.parametrize("driver", ["step_change", "richardson", "yoshida"])
def test_adaptive_drivers_with_losses(gpu, driver):
    ws_o, ws_g = make_pair((64,), (20.0,), 1, c0=10.0, c1=-0.5, omega=(1.0,), zeeman=(0.1, 0.0), loss=(0.5, 0.1),
                           state="ferromagnetic")
    ad = dict(dt_init=0.005, dt_min=1e-4, dt_max=0.05, tol=1e-4 if driver != "yoshida" else 0.01)
    if driver == "yoshida":
        ro = O.run_simulation_yoshida(ws_o, O.AdaptiveDtParams(**ad), 0.3, 0.1)
        rg = S.run_simulation_yoshida(ws_g, S.AdaptiveDtParams(**ad), t_end=0.3, save_interval=0.1)
    else:
        ro = O.run_simulation_adaptive(ws_o, O.AdaptiveDtParams(error_mode=driver, **ad), 0.3, 0.1)
        rg = S.run_simulation_adaptive(ws_g, S.AdaptiveDtParams(error_mode=driver, **ad), t_end=0.3,
                                       save_interval=0.1)
    assert (rg["n_accepted"], rg["n_rejected"]) == (ro["n_accepted"], ro["n_rejected"])
    np.testing.assert_allclose(rg["result"].norms, ro["result"].norms, rtol=1e-13)
    assert rg["result"].norms[-1] < rg["result"].norms[0]
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    ws_g.close()


def test_loss_fp32(gpu):
    ws_o, ws_g = make_pair((32, 32), (12.0, 12.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), loss=(0.5, 0.1),
                           precision="fp32", dt=1e-3)
    for _ in range(50):
        O.split_step(ws_o)
    S.split_step(ws_g, 50)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < 5e-5
    assert abs(S.total_norm(ws_g) - O.total_norm(ws_o.psi, ws_o.grid)) < 1e-6
    ws_g.close()
