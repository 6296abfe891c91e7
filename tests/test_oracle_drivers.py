"""Pins of the oracle's driver-level behaviour to the reference's own tests: resuming a
leapfrog run from a saved state gives the continuous run's result (test/test_checkpoint.jl:
21-54, to 1e-10), and the adaptive loops' L2 change estimator (test/test_adaptive_dt.jl:
84-106)."""

import cmath
import math

import numpy as np
import pytest

import oracle as O


def _ws(n_steps, save_every, psi=None):
    g = O.make_grid(O.GridConfig((16,), (10.0,)))
    return O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(1.0, 0.0),
                            sim_params=O.SimParams(0.01, n_steps, False, None, save_every), psi_init=psi)


def test_resume_equals_continuous_run():
    full = _ws(100, 100)
    psi0 = full.psi.copy()
    O.run_simulation(full, keep_psi=False)
    first = _ws(50, 50, psi0)
    O.run_simulation(first, keep_psi=False)
    rest = _ws(50, 50, first.psi)
    rest.t, rest.step = first.t, first.step
    O.run_simulation(rest, keep_psi=False)
    assert float(np.max(np.abs(rest.psi - full.psi))) < 1e-10
    assert rest.t == pytest.approx(full.t, abs=1e-12)


def test_l2_change_estimator():
    a = np.array([1.0, 2.0, 3.0], dtype=np.complex128)
    c = np.array([1.1, 2.0, 3.0], dtype=np.complex128)
    assert O.wavefunction_l2_change(a, a) == 0.0
    assert O.wavefunction_l2_change(c, a) > 0.0
    phase = a * cmath.exp(0.5j)
    assert O.wavefunction_l2_change(phase, a) > 0.01      # a phase rotation is a change
    g = a * cmath.exp(0.1j)
    assert O.wavefunction_l2_change(g, a) == pytest.approx(2 * (1 - math.cos(0.1)), rel=1e-10)
