"""GPU parity of a time-dependent Zeeman term (TimeDependentZeeman, src/types.jl:172-178;
zeeman_at(z, t), src/zeeman.jl:20-21) through the whole-run drivers: the library evaluates the
host function at the state time before every half potential, as _half_potential_step! does
(src/split_step.jl:49), including the leapfrog's merged V(dt) at the start of its step
(src/simulation.jl:66-72) and the adaptive loops' deferred closing half steps."""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, make_pair, rel_psi_err

pytestmark = pytest.mark.gpu


def ramp_o(t):
    return O.ZeemanParams(0.2 - 1.5 * t, 0.1 + 2.0 * t)


def ramp_s(t):
    return S.ZeemanParams(0.2 - 1.5 * t, 0.1 + 2.0 * t)


def _pair(n, L, **kw):
    ws_o, ws_g = make_pair(n, L, 1, c0=10.0, c1=0.5, omega=(1.0,) * len(n), **kw)
    ws_o.zeeman = ramp_o
    ws_g.set_zeeman_function(ramp_s)
    return ws_o, ws_g


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_leapfrog_with_zeeman_ramp(gpu, precision):
    ws_o, ws_g = _pair((32, 32), (12.0, 12.0), dt=2e-3, state="random", precision=precision)
    ws_o.sim_params = O.SimParams(2e-3, 40, False, None, 10)
    ws_g.sim_params = S.SimParams(2e-3, 40, False, None, 10)
    ro = O.run_simulation(ws_o)
    rg = S.run_simulation(ws_g)
    tol = PSI_TOL_FP64 if precision == "fp64" else 5e-5
    etol = ENERGY_TOL_FP64 * 10 if precision == "fp64" else 1e-6
    np.testing.assert_allclose(rg.energies, ro.energies, rtol=etol)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < tol
    # the ramp changes the state: the same run with the t=0 Zeeman term differs
    ws_s = make_pair((32, 32), (12.0, 12.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), dt=2e-3, state="random",
                     zeeman=(0.2, 0.1))[0]
    ws_s.sim_params = O.SimParams(2e-3, 40, False, None, 10)
    O.run_simulation(ws_s, keep_psi=False)
    assert rel_psi_err(ws_s.psi, ws_o.psi) > 1e-6
    ws_g.close()


def test_split_steps_with_zeeman_ramp(gpu):
    ws_o, ws_g = _pair((64,), (16.0,), dt=2e-3, state="random")
    for _ in range(25):
        O.split_step(ws_o)
    S.split_step(ws_g, 25)
    assert abs(ws_g.t - ws_o.t) < 1e-14
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    ws_g.close()


@pytest.mark.parametrize("driver", ["step_change", "richardson", "yoshida"])
def test_adaptive_drivers_with_zeeman_ramp(gpu, driver):
    ws_o, ws_g = _pair((64,), (20.0,), state="ferromagnetic")
    ad = dict(dt_init=0.005, dt_min=1e-4, dt_max=0.05, tol=1e-4 if driver != "yoshida" else 0.01)
    if driver == "yoshida":
        ro = O.run_simulation_yoshida(ws_o, O.AdaptiveDtParams(**ad), 0.3, 0.1)
        rg = S.run_simulation_yoshida(ws_g, S.AdaptiveDtParams(**ad), t_end=0.3, save_interval=0.1)
    else:
        ro = O.run_simulation_adaptive(ws_o, O.AdaptiveDtParams(error_mode=driver, **ad), 0.3, 0.1)
        rg = S.run_simulation_adaptive(ws_g, S.AdaptiveDtParams(error_mode=driver, **ad), t_end=0.3,
                                       save_interval=0.1)
    assert (rg["n_accepted"], rg["n_rejected"]) == (ro["n_accepted"], ro["n_rejected"])
    np.testing.assert_allclose(rg["result"].energies, ro["result"].energies, rtol=ENERGY_TOL_FP64 * 10)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    ws_g.close()
