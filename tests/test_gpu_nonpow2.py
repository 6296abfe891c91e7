"""Grids whose axes are not powers of two (the reference accepts any even n, src/types.jl:12):
the GPU path transforms such an axis by Bluestein's identity on power-of-two lines of length
>= 2n - 1 (k_blue_*), with the kinetic phase applied between the forward and inverse
transforms of all axes.  Parity against the oracle (numpy FFTs of the same sizes) at the plain
form's bars, the FP32-bulk form with its error stated."""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, make_pair, rel_psi_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,L,F", [((24,), (10.0,), 1), ((100,), (20.0,), 1), ((1000,), (40.0,), 2),
                                   ((48, 40), (12.0, 10.0), 1), ((30, 64), (12.0, 16.0), 2),
                                   ((12, 10, 6), (8.0, 8.0, 6.0), 1), ((10, 12, 8), (8.0, 8.0, 8.0), 6)])
@pytest.mark.parametrize("itp", [False, True])
def test_split_steps_non_pow2(gpu, n, L, F, itp):
    kw = dict(c0=10.0, c1=0.4)
    if F == 6:
        kw = dict(c0=4689.0 / 2, c1=4689.0 / 72, c_extra=(0.0, 0.0, 50.0))
    ws_o, ws_g = make_pair(n, L, F, omega=(1.0,) * len(n), zeeman=(0.1, 0.05), itp=itp, dt=1e-3, **kw)
    for _ in range(10):
        O.split_step(ws_o)
    S.split_step(ws_g, 10)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    Eo = O.total_energy(ws_o)
    assert abs(S.total_energy(ws_g) - Eo) <= ENERGY_TOL_FP64 * 10 * abs(Eo)
    ws_g.close()


def test_leapfrog_non_pow2_snapshots(gpu):
    ws_o, ws_g = make_pair((48, 40), (12.0, 10.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), zeeman=(0.0, 0.1),
                           dt=1e-3)
    ws_o.sim_params = O.SimParams(1e-3, 30, False, None, 10)
    ws_g.sim_params = S.SimParams(1e-3, 30, False, None, 10)
    ro = O.run_simulation(ws_o)
    rg = S.run_simulation(ws_g)
    np.testing.assert_allclose(rg.energies, ro.energies, rtol=ENERGY_TOL_FP64 * 10)
    np.testing.assert_allclose(rg.norms, ro.norms, rtol=1e-13)
    for a, b in zip(rg.psi_snapshots, ro.psi_snapshots):
        assert rel_psi_err(a, b) < PSI_TOL_FP64
    ws_g.close()


def test_ground_state_non_pow2(gpu):
    og = O.make_grid(O.GridConfig((96, 80), (16.0, 14.0)))
    hg = S.make_grid(S.GridConfig((96, 80), (16.0, 14.0)))
    psi0 = O.init_psi(og, 1, "random", seed=8)
    kw = dict(dt=0.005, n_steps=200, tol=1e-9, psi_init=psi0)
    ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                             V=O.harmonic_potential(og, (1.0, 1.0)), **kw)
    rg = S.find_ground_state(grid=hg, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                             potential=S.HarmonicTrap(1.0, 1.0), **kw)
    assert rg["steps"] == ro["steps"]
    assert abs(rg["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * abs(ro["energy"])
    assert rel_psi_err(rg["workspace"].psi, ro["workspace"].psi) < PSI_TOL_FP64
    rg["workspace"].close()


def test_non_pow2_fp32(gpu):
    ws_o, ws_g = make_pair((48, 40), (12.0, 10.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), zeeman=(0.0, 0.1),
                           dt=1e-3, precision="fp32")
    for _ in range(50):
        O.split_step(ws_o)
    S.split_step(ws_g, 50)
    e = rel_psi_err(ws_g.psi, ws_o.psi)
    print(f"FP32 48x40, 50 steps: psi {e:.2e}")
    assert e < 5e-5
    assert abs(S.total_norm(ws_g) - O.total_norm(ws_o.psi, ws_o.grid)) < 1e-6
    ws_g.close()
