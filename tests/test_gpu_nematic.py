"""GPU parity of the singlet-pair (nematic) step (src/nematic.jl: c2 without a higher even
c_k) against the oracle: the fused row passes (leapfrog run with save points, ITP ground
state), the general path with DDI, the FP32-bulk form, and the nematic energy term.
(The operator-level cases are in tests/test_gpu_operators.py: f1_nematic, f2_nematic,
f1_nematic_ddi.)"""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, make_pair, rel_psi_err

pytestmark = pytest.mark.gpu


def test_leapfrog_with_nematic_against_oracle(gpu):
    ws_o, ws_g = make_pair((32, 32), (16.0, 16.0), 1, c0=10.0, c1=-0.5, c_extra=(50.0,), omega=(1.0, 1.0),
                           zeeman=(0.0, 0.1), dt=1e-3, state="uniform")
    ws_o.sim_params = O.SimParams(1e-3, 45, False, None, 10)
    ws_g.sim_params = S.SimParams(1e-3, 45, False, None, 10)
    ro = O.run_simulation(ws_o)
    rg = S.run_simulation(ws_g)
    np.testing.assert_allclose(rg.energies, ro.energies, rtol=ENERGY_TOL_FP64 * 10)
    np.testing.assert_allclose(rg.norms, ro.norms, rtol=1e-13)
    for a, b in zip(rg.psi_snapshots, ro.psi_snapshots):
        assert rel_psi_err(a, b) < PSI_TOL_FP64
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    ws_g.close()


def test_ground_state_with_nematic_against_oracle(gpu):
    n, L = (64,), (16.0,)
    og = O.make_grid(O.GridConfig(n, L))
    hg = S.make_grid(S.GridConfig(n, L))
    psi0 = O.init_psi(og, 2, "random", seed=5)
    kw = dict(dt=0.005, n_steps=300, tol=1e-9, psi_init=psi0)
    ro = O.find_ground_state(grid=og, atom=O.AtomSpecies("f2", 2),
                             interactions=O.InteractionParams(30.0, 1.0, 0.0, (-20.0,)),
                             V=O.harmonic_potential(og, (1.0,)), **kw)
    rg = S.find_ground_state(grid=hg, atom=S.AtomSpecies("f2", 2),
                             interactions=S.InteractionParams(30.0, 1.0, 0.0, (-20.0,)),
                             potential=S.HarmonicTrap(1.0), **kw)
    assert abs(rg["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * abs(ro["energy"])
    assert rel_psi_err(rg["workspace"].psi, ro["workspace"].psi) < PSI_TOL_FP64
    rg["workspace"].close()


def test_split_steps_nematic_ddi_against_oracle(gpu):
    ws_o, ws_g = make_pair((16, 16), (10.0, 10.0), 1, c0=10.0, c1=0.3, c_extra=(20.0,), omega=(1.0, 1.0),
                           ddi=True, c_dd=40.0, dt=2e-3, state="uniform")
    for _ in range(20):
        O.split_step(ws_o)
    S.split_step(ws_g, 20)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    assert abs(S.total_energy(ws_g) - O.total_energy(ws_o)) <= ENERGY_TOL_FP64 * 10 * abs(O.total_energy(ws_o))
    ws_g.close()


@pytest.mark.parametrize("F,c2", [(1, 50.0), (2, 30.0)])
def test_fp32_nematic_against_oracle(gpu, F, c2):
    ws_o, ws_g = make_pair((64, 64), (20.0, 20.0), F, c0=10.0, c1=0.5, c_extra=(c2,), omega=(1.0, 1.0),
                           zeeman=(0.0, 0.1), dt=1e-3, precision="fp32", state="uniform")
    for _ in range(50):
        O.split_step(ws_o)
    S.split_step(ws_g, 50)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < 5e-5
    Eo = O.total_energy(ws_o)
    assert abs(S.total_energy(ws_g) - Eo) / abs(Eo) < 1e-5
    assert abs(S.energy_terms(ws_g)["tensor"] - O.energy_terms(ws_o)["tensor"]) <= 1e-5 * abs(Eo)
    ws_g.close()


def test_batch_nematic_needs_one_shared_c2(gpu):
    """The batch takes the nematic c2 as one value for every solve; per-solve c2 values and
    couplings that switch on the tensor step stay on find_ground_state."""
    g = S.make_grid(S.GridConfig((32, 32), (16.0, 16.0)))
    psis = [S.init_psi(g, 2, "polar") for _ in range(2)]
    f2 = S.AtomSpecies("f2", 2)
    with pytest.raises(S.UnsupportedError):
        S.find_ground_states_batched(grid=g, atom=f2, interactions=[S.InteractionParams(10.0, 0.5, 0.0, (5.0,)),
                                                                    S.InteractionParams(10.0, 0.5, 0.0, (4.0,))],
                                     psi_inits=psis, potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, n_steps=10,
                                     tol=1e-12, precision="fp32")
    with pytest.raises(S.UnsupportedError):
        S.find_ground_states_batched(grid=g, atom=f2, interactions=[S.InteractionParams(10.0, 0.5, 0.0,
                                                                                        (0.5, 0.0, 0.3))] * 2,
                                     psi_inits=psis, potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, n_steps=10,
                                     tol=1e-12, precision="fp32")
