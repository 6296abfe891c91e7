"""Pins the oracle's Raman coupling (src/raman.jl, energy term src/energy.jl:123-135) to the
reference's own tests (test/test_raman.jl): identity at zero Rabi frequency, norm kept over
Rabi cycling and with a wave vector, a spatially varying phase from k_eff, a workspace with
the coupling in split_step!, and the Raman term in the total energy."""

import math

import numpy as np
import pytest

import oracle as O


def _uniform_m0(n, L):
    g = O.make_grid(O.GridConfig((n,), (L,)))
    dV = O.cell_volume(g)
    psi = np.zeros((n, 3), dtype=np.complex128, order="F")
    psi[:, 1] = 1.0 / math.sqrt(n * dV)
    return g, psi, dV


def test_zero_rabi_frequency_no_effect():
    g, psi, _ = _uniform_m0(64, 10.0)
    ref = psi.copy()
    O.raman_step_psi(psi, O.spin_matrices(1), O.RamanCoupling(0.0, 0.0, (0.0,)), g, 0.01, False)
    assert np.max(np.abs(psi - ref)) <= 1e-14


def test_rabi_oscillation_keeps_total_population():
    g = O.make_grid(O.GridConfig((32,), (10.0,)))
    dV = O.cell_volume(g)
    psi = np.zeros((32, 3), dtype=np.complex128, order="F")
    psi[:, 0] = 1.0 / math.sqrt(32 * dV)
    sm = O.spin_matrices(1)
    rc = O.RamanCoupling(1.0, 0.0, (0.0,))
    for _ in range(1000):
        O.raman_step_psi(psi, sm, rc, g, 0.01, False)
    assert float(np.sum(np.abs(psi) ** 2)) * dV == pytest.approx(1.0, rel=1e-6)


def test_raman_preserves_norm():
    g, psi, dV = _uniform_m0(32, 10.0)
    sm = O.spin_matrices(1)
    rc = O.RamanCoupling(2.0, 0.3, (1.0,))
    n0 = float(np.sum(np.abs(psi) ** 2)) * dV
    for _ in range(100):
        O.raman_step_psi(psi, sm, rc, g, 0.01, False)
    assert float(np.sum(np.abs(psi) ** 2)) * dV == pytest.approx(n0, rel=1e-10)


def test_wave_vector_changes_result_and_imprints_phase():
    g, psi0, _ = _uniform_m0(64, 20.0)
    sm = O.spin_matrices(1)
    a = psi0.copy()
    b = psi0.copy()
    for _ in range(100):
        O.raman_step_psi(a, sm, O.RamanCoupling(2.0, 0.0, (0.0,)), g, 0.01, False)
        O.raman_step_psi(b, sm, O.RamanCoupling(2.0, 0.0, (2 * math.pi / 5.0,)), g, 0.01, False)
    assert np.max(np.abs(a - b)) > 1e-6
    ph = np.angle(b[:, 0])
    assert ph.max() - ph.min() > 0.1


def _ws(raman, psi=None):
    g = O.make_grid(O.GridConfig((32,), (10.0,)))
    return O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(1.0, 0.1),
                            sim_params=O.SimParams(0.001, 10), raman=raman, psi_init=psi)


def test_workspace_with_raman_split_steps_keep_norm():
    ws = _ws(O.RamanCoupling(0.5, 0.0, (0.0,)))
    for _ in range(10):
        O.split_step(ws)
    assert O.total_norm(ws.psi, ws.grid) == pytest.approx(1.0, rel=0.01)


def test_raman_energy_in_total_energy():
    g = O.make_grid(O.GridConfig((32,), (10.0,)))
    psi = O.init_psi(g, 1, "uniform")
    E = O.total_energy(_ws(O.RamanCoupling(2.0, 0.5, (1.0,)), psi))
    E_no = O.total_energy(_ws(None, psi))
    assert math.isfinite(E) and math.isfinite(E_no) and E != E_no
