"""The oracle's grid, spin matrices, 3-D support and LHY term against the reference's own tests
(ports of test/test_grid.jl, test/test_spin_matrices.jl, test/test_3d.jl and the hot-path parts
of test/test_lhy.jl).  CPU only: the oracle is the checker of the GPU path, so it is pinned to
the reference's tests first."""

import math

import numpy as np
import pytest

import oracle as O


def test_grid_construction_1d_2d():  # test/test_grid.jl:4-26
    g = O.make_grid(O.GridConfig((128,), (20.0,)))
    assert len(g.x[0]) == 128 and len(g.k[0]) == 128
    assert g.dx[0] == pytest.approx(20.0 / 128)
    assert g.dk[0] == pytest.approx(2 * math.pi / 20.0)
    assert g.k_squared.shape == (128,) and abs(g.k_squared[0]) < 1e-14
    g2 = O.make_grid(O.GridConfig((64, 64), (10.0, 10.0)))
    assert len(g2.x[0]) == 64 and len(g2.x[1]) == 64
    assert g2.k_squared.shape == (64, 64) and abs(g2.k_squared[0, 0]) < 1e-14


@pytest.mark.parametrize("n,L", [((0,), (10.0,)), ((127,), (10.0,)), ((128,), (-1.0,))])
def test_grid_validation(n, L):  # test/test_grid.jl:28-32
    with pytest.raises(ValueError):
        O.GridConfig(n, L)


def test_cell_volume():  # test/test_grid.jl:40-47
    assert O.cell_volume(O.make_grid(O.GridConfig((128,), (20.0,)))) == pytest.approx(20.0 / 128)
    assert O.cell_volume(O.make_grid(O.GridConfig((64, 32), (10.0, 8.0)))) == pytest.approx((10.0 / 64) * (8.0 / 32))


def test_spin1_basics_and_fz():  # test/test_spin_matrices.jl:6-11, 45-48
    sm = O.spin_matrices(1)
    assert sm.F == 1 and sm.D == 3
    assert list(sm.m_values) == [1, 0, -1]
    assert np.allclose(np.real(np.diag(sm.Fz)), [1.0, 0.0, -1.0])


@pytest.mark.parametrize("F", [1, 2, 3])
def test_hermiticity_and_commutators(F):  # test/test_spin_matrices.jl:13-36
    sm = O.spin_matrices(F)
    for M in (sm.Fx, sm.Fy, sm.Fz):
        assert np.allclose(M, M.conj().T, atol=1e-14)
    assert np.allclose(sm.Fx @ sm.Fy - sm.Fy @ sm.Fx, 1j * sm.Fz, atol=1e-12)
    assert np.allclose(sm.Fy @ sm.Fz - sm.Fz @ sm.Fy, 1j * sm.Fx, atol=1e-12)
    assert np.allclose(sm.Fz @ sm.Fx - sm.Fx @ sm.Fz, 1j * sm.Fy, atol=1e-12)


@pytest.mark.parametrize("F", [1, 2, 3, 6])
def test_casimir(F):  # test/test_spin_matrices.jl:38-44
    sm = O.spin_matrices(F)
    FF = sm.Fx @ sm.Fx + sm.Fy @ sm.Fy + sm.Fz @ sm.Fz
    assert np.allclose(FF, F * (F + 1) * np.eye(2 * F + 1), atol=1e-12)


def test_spin6_components():  # test/test_spin_matrices.jl:49-54
    sm = O.spin_matrices(6)
    assert sm.D == 13 and list(sm.m_values) == list(range(6, -7, -1))


def test_3d_grid_trap_and_gaussian():  # test/test_3d.jl:2-40
    g = O.make_grid(O.GridConfig((16, 16, 16), (10.0, 10.0, 10.0)))
    assert len(g.x) == 3 and len(g.k) == 3 and g.k_squared.shape == (16, 16, 16)
    assert abs(g.k_squared[0, 0, 0]) < 1e-14
    assert g.dx == (10.0 / 16,) * 3 and O.cell_volume(g) == pytest.approx(np.prod(g.dx))
    V = O.harmonic_potential(g, (1.0, 2.0, 3.0))
    assert V.shape == (16, 16, 16) and V[7, 7, 7] > 0.0
    assert V.min() < V[0, 0, 0]
    g2 = O.make_grid(O.GridConfig((16, 16, 16), (20.0, 20.0, 20.0)))
    psi = O.init_psi(g2, 1, "polar")
    assert psi.shape == (16, 16, 16, 3) and O.total_norm(psi, g2) == pytest.approx(1.0, abs=1e-10)


def test_3d_free_particle_norm():  # test/test_3d.jl:42-56
    g = O.make_grid(O.GridConfig((16, 16, 16), (20.0, 20.0, 20.0)))
    ws = O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(0.0, 0.0),
                          sim_params=O.SimParams(0.001, 20, False, 0, 20))
    n0 = O.total_norm(ws.psi, g)
    for _ in range(20):
        O.split_step(ws)
    assert abs(O.total_norm(ws.psi, g) - n0) / n0 < 1e-10


def test_3d_ground_state_norm():  # test/test_3d.jl:58-73 (contact couplings c0=10, c1=-0.5 stand in
    # for compute_interaction_params(Rb87; N_atoms=100), whose unit system is outside the oracle)
    g = O.make_grid(O.GridConfig((16, 16, 16), (20.0, 20.0, 20.0)))
    r = O.find_ground_state(grid=g, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                            V=O.harmonic_potential(g, (1.0, 1.0, 1.0)), dt=0.001, n_steps=500, tol=1e-8,
                            initial_state="ferromagnetic")
    assert O.total_norm(r["workspace"].psi, g) == pytest.approx(1.0, abs=1e-8)


def _lhy_ws(c_lhy, dt=0.01, n_steps=50):
    g = O.make_grid(O.GridConfig((64,), (20.0,)))
    return O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5, c_lhy),
                            V=O.harmonic_potential(g, (1.0,)), sim_params=O.SimParams(dt, n_steps))


def test_lhy_zero_regression_and_norm():  # test/test_lhy.jl:2-20, 72-87
    for c_lhy, dt, n in ((0.0, 0.01, 50), (50.0, 0.005, 100)):
        ws = _lhy_ws(c_lhy, dt, n)
        n0 = O.total_norm(ws.psi, ws.grid)
        for _ in range(n):
            O.split_step(ws)
        assert O.total_norm(ws.psi, ws.grid) == pytest.approx(n0, rel=1e-6)


def test_lhy_energy_sign_and_effect():  # test/test_lhy.jl:22-70
    e1 = O.energy_terms(_lhy_ws(1.0))
    assert e1["lhy"] > 0.0
    assert O.energy_terms(_lhy_ws(0.0))["lhy"] == 0.0
    assert O.total_energy(_lhy_ws(100.0, n_steps=10)) > O.total_energy(_lhy_ws(0.0, n_steps=10))
