"""The experiment runner (src/experiment_runner.jl:54-155) as one device-resident pipeline,
against the oracle's restatement on the same parsed configuration: a ground state, a hold with
seeded noise, a linear quadratic-Zeeman ramp, an adaptive phase with a linear-Zeeman ramp and a
change of trap, and losses on every phase."""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, rel_psi_err

pytestmark = pytest.mark.gpu

CONFIG = {"experiment": {
    "name": "quench",
    "system": {"atom": "Rb87", "grid": {"n_points": [64], "box_size": [20.0]},
               "interactions": {"c0": 10.0, "c1": -0.5}, "losses": {"gamma_dr": 0.05, "L3": 0.01}},
    "ground_state": {"dt": 0.005, "n_steps": 400, "tol": 1e-9, "initial_state": "polar",
                     "zeeman": {"p": 0.0, "q": 0.3}, "potential": {"type": "harmonic", "omega": [1.0]}},
    "sequence": [
        {"name": "hold", "duration": 0.05, "dt": 0.001, "save_every": 10, "zeeman": {"q": 0.3},
         "noise_amplitude": 0.01},
        {"name": "ramp", "duration": 0.1, "dt": 0.002, "save_every": 10, "zeeman": {"q": {"from": 0.3, "to": -0.2}}},
        {"name": "adaptive", "duration": 0.1, "dt": 0.002, "save_every": 10,
         "zeeman": {"p": {"from": 0.0, "to": 0.2}, "q": -0.2},
         "potential": {"type": "harmonic", "omega": [1.5]},
         "adaptive_dt": {"dt_init": 0.002, "dt_min": 1e-4, "dt_max": 0.01, "tol": 1e-4}},
    ]}}


def test_run_experiment_against_oracle(gpu):
    ro = O.run_experiment(CONFIG, seed=7)
    rg = S.run_experiment(CONFIG, seed=7)
    assert rg.ground_state_converged == ro["ground_state_converged"]
    assert abs(rg.ground_state_energy - ro["ground_state_energy"]) <= ENERGY_TOL_FP64 * abs(ro["ground_state_energy"])
    assert rg.phase_names == ["hold", "ramp", "adaptive"]
    for a, b in zip(rg.phase_results, ro["phase_results"]):
        np.testing.assert_allclose(a.times, b.times, rtol=0, atol=1e-12)
        np.testing.assert_allclose(a.energies, b.energies, rtol=ENERGY_TOL_FP64 * 10)
        np.testing.assert_allclose(a.norms, b.norms, rtol=1e-13)
    assert rel_psi_err(rg.phase_results[-1].psi_snapshots[-1], ro["psi"]) < PSI_TOL_FP64
    # the ramps and losses act: energy and norm move within the phases
    assert rg.phase_results[1].energies[-1] != rg.phase_results[1].energies[0]
    assert rg.phase_results[-1].norms[-1] < rg.phase_results[0].norms[0]
