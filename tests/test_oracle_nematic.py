"""Pins the oracle's singlet-pair (nematic) step and amplitude to the reference's own
known-answer and invariant tests (test/test_nematic.jl): the |A00|^2 values of the polar
and ferromagnetic states, identity at c2 = 0 and on ferromagnetic states, norm
conservation in real time, the small-dt limit of the GP equation, and the m <-> -m
symmetry in real and imaginary time."""

import cmath

import numpy as np
import pytest

import oracle as O


def _grid1(n=64, L=20.0):
    return O.make_grid(O.GridConfig((n,), (L,)))


@pytest.mark.parametrize("F,den", [(1, 3.0), (2, 5.0)])
def test_polar_pair_amplitude(F, den):
    g = _grid1()
    psi = O.init_psi(g, F, "polar")
    A = O.singlet_pair_amplitude(psi, F)
    n = O.total_density(psi)
    assert np.sum(np.abs(A) ** 2) == pytest.approx(np.sum(n ** 2) / den, rel=1e-12)


def test_ferromagnetic_pair_amplitude_zero():
    psi = O.init_psi(_grid1(), 1, "ferromagnetic")
    assert np.sum(np.abs(O.singlet_pair_amplitude(psi, 1)) ** 2) < 1e-28


def test_uniform_pair_amplitude_nonzero_and_2d_shape():
    assert np.sum(np.abs(O.singlet_pair_amplitude(O.init_psi(_grid1(), 1, "uniform"), 1)) ** 2) > 0
    g2 = O.make_grid(O.GridConfig((32, 32), (10.0, 10.0)))
    A = O.singlet_pair_amplitude(O.init_psi(g2, 1, "polar"), 1)
    assert A.shape == (32, 32) and np.sum(np.abs(A) ** 2) > 0


def test_identity_at_c2_zero_and_on_ferromagnetic():
    psi = O.init_psi(_grid1(), 1, "uniform")
    ref = psi.copy()
    O.nematic_step_psi(psi, 0.0, 0.01, False)
    assert np.max(np.abs(psi - ref)) <= 1e-15
    psi = O.init_psi(_grid1(), 1, "ferromagnetic")
    ref = psi.copy()
    O.nematic_step_psi(psi, 50.0, 0.01, False)
    assert np.max(np.abs(psi - ref)) <= 1e-14


@pytest.mark.parametrize("F,c2,n", [(1, 50.0, (64,)), (2, 30.0, (64,)), (1, 50.0, (32, 32))])
def test_norm_conserved(F, c2, n):
    g = O.make_grid(O.GridConfig(n, tuple(20.0 if len(n) == 1 else 10.0 for _ in n)))
    psi = O.init_psi(g, F, "uniform")
    n0 = O.total_norm(psi, g)
    O.nematic_step_psi(psi, c2, 0.01, False)
    assert abs(O.total_norm(psi, g) - n0) / n0 < 1e-12


def _point(vals):
    psi = np.zeros((1, len(vals)), dtype=np.complex128)
    psi[0, :] = vals
    return psi


F1 = [0.5 * cmath.exp(0.7j), 0.3 + 0.2j, 0.4 * cmath.exp(-0.3j)]
F2 = [0.4 * cmath.exp(0.5j), 0.3 * cmath.exp(-0.8j), 0.2 + 0.1j, 0.35 * cmath.exp(1.2j), 0.25 * cmath.exp(-0.3j)]


@pytest.mark.parametrize("vals,c2", [(F1, 50.0), (F2, 30.0)])
def test_complex_state_total_norm_50_steps(vals, c2):
    psi = _point(vals)
    before = np.sum(np.abs(psi) ** 2)
    for _ in range(50):
        O.nematic_step_psi(psi, c2, 0.01, False)
    assert np.sum(np.abs(psi) ** 2) == pytest.approx(before, rel=1e-6)


def test_small_dt_matches_gp_equation():
    psi0 = _point(F1)
    psi = psi0.copy()
    c2, dt = 50.0, 1e-6
    O.nematic_step_psi(psi, c2, dt, False)
    signs = (1.0, -1.0, 1.0)
    isd = 1.0 / np.sqrt(3.0)
    A00 = sum(signs[c] * psi0[0, c] * psi0[0, 2 - c] for c in range(3)) * isd
    for c in range(3):
        V = c2 * signs[c] * A00 * isd
        expected = psi0[0, c] - 1j * V * dt * np.conj(psi0[0, 2 - c])
        assert psi[0, c] == pytest.approx(expected, rel=1e-4)


@pytest.mark.parametrize("itp", [False, True])
def test_m_minus_m_symmetry(itp):
    psi = _point(F1)
    swapped = _point([F1[2], F1[1], F1[0]])
    O.nematic_step_psi(psi, 50.0, 0.05, itp)
    O.nematic_step_psi(swapped, 50.0, 0.05, itp)
    assert abs(psi[0, 0] - swapped[0, 2]) <= 1e-14
    assert abs(psi[0, 2] - swapped[0, 0]) <= 1e-14


def test_itp_norm_bounded():
    g = _grid1()
    psi = O.init_psi(g, 1, "polar")
    n0 = O.total_norm(psi, g)
    O.nematic_step_psi(psi, 50.0, 0.001, True)
    n1 = O.total_norm(psi, g)
    assert 0.0 < n1 < 2 * n0
