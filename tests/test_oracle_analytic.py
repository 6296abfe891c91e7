"""The oracle against the analytic propagator and spin-dynamics tests of the reference
(ports of test/test_physics_level0.jl and test/test_physics_level3.jl): free Gaussian spreading,
Larmor precession, spin-mixing eigenstates, magnetisation conservation under spin mixing with a
quadratic Zeeman term, the ferromagnetic / polar ground states by the sign of c1, and norm and
magnetisation conservation of a spin-6 gas with dipolar coupling.  CPU only; the same cases run
on the device in tests/test_gpu_analytic.py."""

import math

import numpy as np
import pytest

import oracle as O


def _gaussian_m0(grid, sigma0):
    psi = np.zeros(grid.config.n_points + (3,), dtype=np.complex128, order="F")
    psi[..., 1] = np.exp(-grid.x[0] ** 2 / (2 * sigma0 ** 2))
    psi /= math.sqrt(np.sum(np.abs(psi) ** 2) * O.cell_volume(grid))
    return psi


def test_free_gaussian_spreading():  # test/test_physics_level0.jl:7-48
    sigma0, T, dt = 2.0, 3.0, 0.01
    n = round(T / dt)
    g = O.make_grid(O.GridConfig((256,), (40.0,)))
    ws = O.make_workspace(grid=g, atom=O.AtomSpecies("scalar", 1), interactions=O.InteractionParams(0.0, 0.0),
                          sim_params=O.SimParams(dt, n, False, None, n), psi_init=_gaussian_m0(g, sigma0))
    for _ in range(n):
        O.split_step(ws)
    dens = np.abs(ws.psi[:, 1]) ** 2
    x = g.x[0]
    dV = O.cell_volume(g)
    N = dens.sum() * dV
    xm = (x * dens).sum() * dV / N
    var = ((x - xm) ** 2 * dens).sum() * dV / N
    exact = sigma0 ** 2 / 2 + T ** 2 / (2 * sigma0 ** 2)
    assert abs(var - exact) / exact < 1e-3


def _larmor_psi(grid, L):
    zeta = np.array([0.5, 1 / math.sqrt(2), 0.5], dtype=np.complex128)
    return np.asfortranarray(np.tile(zeta / math.sqrt(L), grid.config.n_points + (1,)))


def test_larmor_precession_checkpoints():  # test/test_physics_level0.jl:50-95, test_physics_level3.jl:7-56
    p, dt, L = 1.0, 0.005, 10.0
    g = O.make_grid(O.GridConfig((32,), (L,)))
    cps = [math.pi / 4, math.pi / 2, math.pi, 3 * math.pi / 2, 2 * math.pi]
    steps = [round(t / dt) for t in cps]
    ws = O.make_workspace(grid=g, atom=O.AtomSpecies("s1", 1), interactions=O.InteractionParams(0.0, 0.0),
                          zeeman=O.ZeemanParams(p, 0.0), sim_params=O.SimParams(dt, steps[-1], False, None, steps[-1]),
                          psi_init=_larmor_psi(g, L))
    dV = O.cell_volume(g)
    done = 0
    for t, s in zip(cps, steps):
        for _ in range(s - done):
            O.split_step(ws)
        done = s
        fx, fy, fz = O.spin_density(ws.psi, 1)
        assert abs(fx.sum() * dV - math.cos(p * t)) < 5e-3
        assert abs(fy.sum() * dV + math.sin(p * t)) < 5e-3
        assert abs(fz.sum() * dV) < 1e-10


@pytest.mark.parametrize("comp,c1", [(1, 10.0), (0, -0.5)])
def test_spin_mixing_eigenstates(comp, c1):  # test/test_physics_level0.jl:97-142
    g = O.make_grid(O.GridConfig((64,), (10.0,)))
    psi = np.zeros((64, 3), dtype=np.complex128, order="F")
    psi[:, comp] = np.exp(-g.x[0] ** 2 / 4.0)
    psi /= math.sqrt(np.sum(np.abs(psi) ** 2) * O.cell_volume(g))
    ws = O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(0.0, c1),
                          sim_params=O.SimParams(1.0, 1), psi_init=psi)
    before = np.abs(ws.psi[:, comp]) ** 2
    O.apply_spin_mixing_step(ws, 1.0, False)
    assert np.max(np.abs(np.abs(ws.psi[:, comp]) ** 2 - before)) < 1e-14
    if comp == 0:
        assert np.max(np.abs(ws.psi[:, 1]) ** 2) < 1e-28


def test_magnetization_conserved_under_spin_mixing():  # test/test_physics_level3.jl:58-87
    g = O.make_grid(O.GridConfig((64,), (15.0,)))
    ws = O.make_workspace(grid=g, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                          zeeman=O.ZeemanParams(0.0, 0.5), V=O.harmonic_potential(g, (1.0,)),
                          sim_params=O.SimParams(0.005, 1000, False, None, 100),
                          psi_init=O.init_psi(g, 1, "ferromagnetic"))
    m0 = O.magnetization(ws.psi, g, 1)
    for step in range(1, 1001):
        O.split_step(ws)
        if step % 100 == 0:
            assert abs(O.magnetization(ws.psi, g, 1) - m0) < 1e-8


@pytest.mark.parametrize("c1,state,comp", [(-0.5, "ferromagnetic", 0), (0.5, "polar", 1)])
def test_ground_state_phase_by_c1_sign(c1, state, comp):  # test/test_physics_level3.jl:89-133
    g = O.make_grid(O.GridConfig((128,), (20.0,)))
    r = O.find_ground_state(grid=g, atom=O.Rb87, interactions=O.InteractionParams(10.0, c1),
                            V=O.harmonic_potential(g, (1.0,)), dt=0.005, n_steps=5000, initial_state=state)
    psi = r["workspace"].psi
    pops = [float(np.sum(np.abs(psi[:, c]) ** 4)) for c in range(3)]  # sum |n_c|^2, as the reference sums abs2 of densities
    assert pops[comp] / sum(pops) > 0.95


def test_spin6_ddi_norm_and_magnetization_1d():  # test/test_physics_level3.jl:180-214
    g = O.make_grid(O.GridConfig((32,), (20.0,)))
    ip = O.interaction_params_from_constraint(c_total=200.0, c1_ratio=1.0 / 36.0, F=6)
    ws = O.make_workspace(grid=g, atom=O.AtomSpecies("f6", 6), interactions=ip, zeeman=O.ZeemanParams(0.1, 0.0),
                          V=O.harmonic_potential(g, (1.0,)), sim_params=O.SimParams(1e-4, 200, False, None, 50),
                          psi_init=O.init_psi(g, 6, "ferromagnetic"), enable_ddi=True, c_dd=100.0)
    n0 = O.total_norm(ws.psi, g)
    m0 = O.magnetization(ws.psi, g, 6)
    for step in range(1, 201):
        O.split_step(ws)
        if step % 50 == 0:
            assert abs(O.total_norm(ws.psi, g) - n0) / n0 < 1e-6
            assert abs(O.magnetization(ws.psi, g, 6) - m0) < 1e-4


def _tf_density(V, g, dV):
    """thomas_fermi_density(V, g, dV; N_target=1) (src/thomas_fermi.jl:5-45): n = max(0, (mu - V)/g)
    with mu found by bisection so that sum(n) dV = 1."""
    def norm(mu):
        return float(np.sum(np.maximum(mu - V, 0.0)) / g * dV)
    lo, hi = float(V.min()), float(V.min() + 2.0 * (V.max() - V.min()))
    while norm(hi) < 1.0 and hi < V.max() * 100:
        hi *= 2.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        nm = norm(mid)
        if abs(nm - 1.0) < 1e-12:
            lo = hi = mid
            break
        if nm < 1.0:
            lo = mid
        else:
            hi = mid
    mu = 0.5 * (lo + hi)
    return np.maximum(mu - V, 0.0) / g, mu


def test_thomas_fermi_1d():  # test/test_physics_level2.jl:6-47
    c0 = 200.0
    g = O.make_grid(O.GridConfig((256,), (20.0,)))
    r = O.find_ground_state(grid=g, atom=O.AtomSpecies("t", 1), interactions=O.InteractionParams(c0, 0.0),
                            V=O.harmonic_potential(g, (1.0,)), dt=0.005, n_steps=10000, tol=1e-10,
                            initial_state="polar")
    assert r["converged"]
    dV = O.cell_volume(g)
    x = g.x[0]
    n_num = np.abs(r["workspace"].psi[:, 1]) ** 2
    mu = (3 * c0 / (4 * math.sqrt(2))) ** (2 / 3)
    n_tf = np.maximum(0.0, (mu - x ** 2 / 2) / c0)
    n_tf /= n_tf.sum() * dV
    assert np.sum(np.abs(n_num - n_tf)) * dV < 0.05
    peak = n_num.max()
    R_num = max(abs(x[i]) for i in range(len(x)) if n_num[i] > 0.01 * peak)
    assert abs(R_num - math.sqrt(2 * mu)) / math.sqrt(2 * mu) < 0.1


def test_thomas_fermi_2d():  # test/test_physics_level2.jl:49-83
    c0 = 200.0
    g = O.make_grid(O.GridConfig((64, 64), (15.0, 15.0)))
    V = O.harmonic_potential(g, (1.0, 1.0))
    r = O.find_ground_state(grid=g, atom=O.AtomSpecies("t", 1), interactions=O.InteractionParams(c0, 0.0), V=V,
                            dt=0.005, n_steps=10000, tol=1e-10, initial_state="polar")
    assert r["converged"]
    dV = O.cell_volume(g)
    n_num = np.abs(r["workspace"].psi[..., 1]) ** 2
    n_tf, mu = _tf_density(V, c0, dV)
    assert np.sum(np.abs(n_num - n_tf)) * dV < 0.10
    peak = n_num.max()
    X, Y = np.meshgrid(g.x[0], g.x[1], indexing="ij")
    R_num = float(np.sqrt(X ** 2 + Y ** 2)[n_num > 0.01 * peak].max())
    assert abs(R_num - math.sqrt(2 * mu)) / math.sqrt(2 * mu) < 0.15
