"""The analytic propagator and spin-dynamics tests of the reference (test/test_physics_level0.jl,
test/test_physics_level3.jl) on the device path, through the C ABI, with the reference's own
tolerances: free Gaussian spreading, Larmor precession at checkpoints, spin-mixing eigenstates,
magnetisation conservation under spin mixing with a quadratic Zeeman term, the ferromagnetic /
polar ground states by the sign of c1, and a spin-6 gas with dipolar coupling.  The oracle
passes the same cases (tests/test_oracle_analytic.py)."""

import math

import numpy as np
import pytest

import spinorbec as S

pytestmark = pytest.mark.gpu


def _gaussian_m0(grid, sigma0):
    psi = np.zeros(tuple(grid.config.n_points) + (3,), dtype=np.complex128, order="F")
    psi[..., 1] = np.exp(-grid.x[0] ** 2 / (2 * sigma0 ** 2))
    psi /= math.sqrt(np.sum(np.abs(psi) ** 2) * S.cell_volume(grid))
    return psi


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_free_gaussian_spreading(gpu, precision):  # test/test_physics_level0.jl:7-48
    sigma0, T, dt = 2.0, 3.0, 0.01
    n = round(T / dt)
    g = S.make_grid(S.GridConfig((256,), (40.0,)))
    ws = S.make_workspace(grid=g, atom=S.AtomSpecies("scalar", 1), interactions=S.InteractionParams(0.0, 0.0),
                          sim_params=S.SimParams(dt, n, False, None, n), psi_init=_gaussian_m0(g, sigma0),
                          precision=precision)
    S.split_step(ws, n)
    dens = np.abs(ws.psi[:, 1]) ** 2
    ws.close()
    x = g.x[0]
    dV = S.cell_volume(g)
    N = dens.sum() * dV
    xm = (x * dens).sum() * dV / N
    var = ((x - xm) ** 2 * dens).sum() * dV / N
    exact = sigma0 ** 2 / 2 + T ** 2 / (2 * sigma0 ** 2)
    assert abs(var - exact) / exact < 1e-3


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_larmor_precession_checkpoints(gpu, precision):  # test/test_physics_level0.jl:50-95, level3:7-56
    p, dt, L = 1.0, 0.005, 10.0
    g = S.make_grid(S.GridConfig((32,), (L,)))
    zeta = np.array([0.5, 1 / math.sqrt(2), 0.5], dtype=np.complex128)
    psi = np.asfortranarray(np.tile(zeta / math.sqrt(L), (32, 1)))
    cps = [math.pi / 4, math.pi / 2, math.pi, 3 * math.pi / 2, 2 * math.pi]
    steps = [round(t / dt) for t in cps]
    ws = S.make_workspace(grid=g, atom=S.AtomSpecies("s1", 1), interactions=S.InteractionParams(0.0, 0.0),
                          zeeman=S.ZeemanParams(p, 0.0), sim_params=S.SimParams(dt, steps[-1], False, None, steps[-1]),
                          psi_init=psi, precision=precision)
    dV = S.cell_volume(g)
    done = 0
    for t, s in zip(cps, steps):
        S.split_step(ws, s - done)
        done = s
        fx, fy, fz = S.spin_density_vector(ws)
        assert abs(fx.sum() * dV - math.cos(p * t)) < 5e-3
        assert abs(fy.sum() * dV + math.sin(p * t)) < 5e-3
        assert abs(fz.sum() * dV) < (1e-10 if precision == "fp64" else 1e-6)
    ws.close()


@pytest.mark.parametrize("comp,c1", [(1, 10.0), (0, -0.5)])
def test_spin_mixing_eigenstates(gpu, comp, c1):  # test/test_physics_level0.jl:97-142
    # a half potential step of dt_half = 2 applies spin mixing for a time of 1 (two steps of 1/2)
    # around diagonal steps that are the identity here (c0 = 0, no trap, no Zeeman term)
    g = S.make_grid(S.GridConfig((64,), (10.0,)))
    psi = np.zeros((64, 3), dtype=np.complex128, order="F")
    psi[:, comp] = np.exp(-g.x[0] ** 2 / 4.0)
    psi /= math.sqrt(np.sum(np.abs(psi) ** 2) * S.cell_volume(g))
    ws = S.make_workspace(grid=g, atom=S.Rb87, interactions=S.InteractionParams(0.0, c1),
                          sim_params=S.SimParams(1.0, 1), psi_init=psi)
    before = np.abs(psi[:, comp]) ** 2
    S.half_potential_step(ws, 2.0, False)
    out = ws.psi
    ws.close()
    assert np.max(np.abs(np.abs(out[:, comp]) ** 2 - before)) < 1e-14
    if comp == 0:
        assert np.max(np.abs(out[:, 1]) ** 2) < 1e-28


def test_magnetization_conserved_under_spin_mixing(gpu):  # test/test_physics_level3.jl:58-87
    g = S.make_grid(S.GridConfig((64,), (15.0,)))
    ws = S.make_workspace(grid=g, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                          zeeman=S.ZeemanParams(0.0, 0.5), potential=S.HarmonicTrap(1.0),
                          sim_params=S.SimParams(0.005, 1000, False, None, 100),
                          psi_init=S.init_psi(g, 1, "ferromagnetic"))
    m0 = S.magnetization(ws)
    for _ in range(10):
        S.split_step(ws, 100)
        assert abs(S.magnetization(ws) - m0) < 1e-8
    ws.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("c1,state,comp", [(-0.5, "ferromagnetic", 0), (0.5, "polar", 1)])
def test_ground_state_phase_by_c1_sign(gpu, c1, state, comp, precision):  # test/test_physics_level3.jl:89-133
    g = S.make_grid(S.GridConfig((128,), (20.0,)))
    r = S.find_ground_state(grid=g, atom=S.Rb87, interactions=S.InteractionParams(10.0, c1),
                            potential=S.HarmonicTrap(1.0), dt=0.005, n_steps=5000, initial_state=state,
                            precision=precision)
    psi = r["workspace"].psi
    r["workspace"].close()
    pops = [float(np.sum(np.abs(psi[:, c]) ** 4)) for c in range(3)]
    assert pops[comp] / sum(pops) > 0.95


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_spin6_ddi_norm_and_magnetization_1d(gpu, precision):  # test/test_physics_level3.jl:180-214
    g = S.make_grid(S.GridConfig((32,), (20.0,)))
    ip = S.interaction_params_from_constraint(c_total=200.0, c1_ratio=1.0 / 36.0, F=6)
    ws = S.make_workspace(grid=g, atom=S.AtomSpecies("f6", 6), interactions=ip, zeeman=S.ZeemanParams(0.1, 0.0),
                          potential=S.HarmonicTrap(1.0), sim_params=S.SimParams(1e-4, 200, False, None, 50),
                          psi_init=S.init_psi(g, 6, "ferromagnetic"), enable_ddi=True, c_dd=100.0,
                          precision=precision)
    n0 = S.total_norm(ws)
    m0 = S.magnetization(ws)
    for _ in range(4):
        S.split_step(ws, 50)
        assert abs(S.total_norm(ws) - n0) / n0 < 1e-6
        assert abs(S.magnetization(ws) - m0) < 1e-4
    ws.close()


def _tf_density(V, g, dV):
    """thomas_fermi_density(V, g, dV; N_target=1) (src/thomas_fermi.jl:5-45), by bisection on mu."""
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


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_thomas_fermi_1d(gpu, precision):  # test/test_physics_level2.jl:6-47
    c0 = 200.0
    g = S.make_grid(S.GridConfig((256,), (20.0,)))
    r = S.find_ground_state(grid=g, atom=S.AtomSpecies("t", 1), interactions=S.InteractionParams(c0, 0.0),
                            potential=S.HarmonicTrap(1.0), dt=0.005, n_steps=10000, tol=1e-10,
                            initial_state="polar", precision=precision)
    if precision == "fp64":
        assert r["converged"]
    n_num = np.abs(r["workspace"].psi[:, 1]) ** 2
    r["workspace"].close()
    dV = S.cell_volume(g)
    x = g.x[0]
    mu = (3 * c0 / (4 * math.sqrt(2))) ** (2 / 3)
    n_tf = np.maximum(0.0, (mu - x ** 2 / 2) / c0)
    n_tf /= n_tf.sum() * dV
    assert np.sum(np.abs(n_num - n_tf)) * dV < 0.05
    peak = n_num.max()
    R_num = max(abs(x[i]) for i in range(len(x)) if n_num[i] > 0.01 * peak)
    assert abs(R_num - math.sqrt(2 * mu)) / math.sqrt(2 * mu) < 0.1


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_thomas_fermi_2d(gpu, precision):  # test/test_physics_level2.jl:49-83
    c0 = 200.0
    g = S.make_grid(S.GridConfig((64, 64), (15.0, 15.0)))
    r = S.find_ground_state(grid=g, atom=S.AtomSpecies("t", 1), interactions=S.InteractionParams(c0, 0.0),
                            potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, n_steps=10000, tol=1e-10,
                            initial_state="polar", precision=precision)
    if precision == "fp64":
        assert r["converged"]
    n_num = np.abs(r["workspace"].psi[..., 1]) ** 2
    r["workspace"].close()
    dV = S.cell_volume(g)
    X, Y = np.meshgrid(g.x[0], g.x[1], indexing="ij")
    V = 0.5 * (X ** 2 + Y ** 2)
    n_tf, mu = _tf_density(V, c0, dV)
    assert np.sum(np.abs(n_num - n_tf)) * dV < 0.10
    peak = n_num.max()
    R_num = float(np.sqrt(X ** 2 + Y ** 2)[n_num > 0.01 * peak].max())
    assert abs(R_num - math.sqrt(2 * mu)) / math.sqrt(2 * mu) < 0.15
