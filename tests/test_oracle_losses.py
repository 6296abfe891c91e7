"""Pins the oracle's density-dependent losses (src/losses.jl) to the reference's own tests
(test/test_losses.jl): no loss keeps the norm, the m-dependent dipolar-relaxation decay
(m = -F stable, the top components fastest), the rate table's properties, density
dependence, m-independent 3-body loss, and the loss in split_step!, in the leapfrog run and
not in imaginary time."""

import numpy as np
import pytest

import oracle as O


def _grid():
    return O.make_grid(O.GridConfig((64,), (20.0,)))


def _pops(psi):
    return [float(np.sum(np.abs(psi[:, c]) ** 2)) for c in range(psi.shape[-1])]


def test_no_loss_preserves_norm():
    g = _grid()
    psi = O.init_psi(g, 1, "uniform")
    n0 = O.total_norm(psi, g)
    O.apply_loss_step_psi(psi, O.LossParams(0.0, 0.0), 1, 0.01)
    assert O.total_norm(psi, g) == pytest.approx(n0, rel=1e-14)


def test_m_dependent_decay_spin1():
    psi = O.init_psi(_grid(), 1, "uniform")
    before = _pops(psi)
    for _ in range(100):
        O.apply_loss_step_psi(psi, O.LossParams(0.1, 0.0), 1, 0.01)
    after = _pops(psi)
    assert after[2] == pytest.approx(before[2], rel=1e-14)   # m = -1 stable
    assert after[0] < before[0] and after[1] < before[1]
    assert after[0] < after[1]                               # m = +1: two channels


def test_m_dependent_decay_spin2():
    psi = O.init_psi(_grid(), 2, "uniform")
    before = _pops(psi)
    for _ in range(50):
        O.apply_loss_step_psi(psi, O.LossParams(0.1, 0.0), 2, 0.01)
    after = _pops(psi)
    assert after[4] == pytest.approx(before[4], rel=1e-14)   # m = -2 stable
    for c in range(4):
        assert after[c] < before[c]
    assert after[0] < after[1] and after[0] < after[2]


@pytest.mark.parametrize("F", [1, 2, 3, 6])
def test_rate_table_properties(F):
    r = O.dipolar_relaxation_rates(F, 1.0)
    D = 2 * F + 1
    assert len(r) == D
    assert abs(r[D - 1]) <= 1e-15
    assert np.sum(r) / D == pytest.approx(1.0, rel=1e-12)
    assert np.all(r >= -1e-15)


def test_rate_table_f6_all_nonterminal_positive():
    r = O.dipolar_relaxation_rates(6, 0.5)
    assert np.all(r[:12] > 0.01) and abs(r[12]) <= 1e-15


def test_density_dependence():
    psi = np.zeros((64, 3), dtype=np.complex128)
    psi[:32, 1] = 2.0
    psi[32:, 1] = 0.5
    left0, right0 = float(np.sum(np.abs(psi[:32, 1]) ** 2)), float(np.sum(np.abs(psi[32:, 1]) ** 2))
    O.apply_loss_step_psi(psi, O.LossParams(0.05, 0.0), 1, 0.01)
    left1, right1 = float(np.sum(np.abs(psi[:32, 1]) ** 2)), float(np.sum(np.abs(psi[32:, 1]) ** 2))
    assert (left0 - left1) / left0 > (right0 - right1) / right0


def test_three_body_uniform_across_m():
    psi = O.init_psi(_grid(), 1, "uniform")
    for _ in range(50):
        O.apply_loss_step_psi(psi, O.LossParams(0.0, 0.1), 1, 0.01)
    p = _pops(psi)
    assert p[0] == pytest.approx(p[1], rel=1e-10) and p[1] == pytest.approx(p[2], rel=1e-10)


def _ws(loss, itp=False, n_steps=100, save_every=None):
    g = _grid()
    sp = O.SimParams(0.01, n_steps, itp, None, save_every if save_every is not None else n_steps)
    return O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(1.0, 0.0),
                            V=O.harmonic_potential(g, (1.0,)) if itp else None, sim_params=sp, loss=loss)


def test_split_step_with_loss_decreases_norm():
    ws = _ws(O.LossParams(0.5, 0.0))
    n0 = O.total_norm(ws.psi, ws.grid)
    for _ in range(100):
        O.split_step(ws)
    assert O.total_norm(ws.psi, ws.grid) < n0


def test_leapfrog_with_loss_decreases_norm():
    ws = _ws(O.LossParams(0.5, 0.0))
    n0 = O.total_norm(ws.psi, ws.grid)
    O.run_simulation(ws, keep_psi=False)
    assert O.total_norm(ws.psi, ws.grid) < n0


def test_loss_skipped_in_imaginary_time():
    ws = _ws(O.LossParams(100.0, 100.0), itp=True, n_steps=10)
    for _ in range(10):
        O.split_step(ws)
    assert O.total_norm(ws.psi, ws.grid) == pytest.approx(1.0, rel=1e-6)
