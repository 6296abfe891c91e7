"""GPU parity of the single operators (FP64 plain form) against the oracle.

Each case feeds identical seeded inputs to the oracle and to the CUDA engine
through the C ABI; tolerances: max|Δψ|/max|ψ| <= 1e-10, energies <= 1e-12 rel.
"""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, make_pair, rel_psi_err

pytestmark = pytest.mark.gpu

GRIDS = [
    ((64,), (20.0,)),
    ((32, 16), (12.0, 8.0)),
    ((16, 8, 32), (8.0, 6.0, 10.0)),
    ((4096,), (80.0,)),
    ((8, 512), (4.0, 40.0)),
]


@pytest.mark.parametrize("n,L", GRIDS)
@pytest.mark.parametrize("itp", [False, True])
def test_kinetic_step(gpu, n, L, itp):
    ws_o, ws_g = make_pair(n, L, 1, itp=itp, dt=0.01)
    if itp:
        ws_o.kinetic_phase = O.prepare_kinetic_phase(ws_o.grid, 0.01, True)
    else:
        O.update_batched_kinetic_phase(ws_o, 0.01)
    O.apply_kinetic_step_batched(ws_o)
    S.kinetic_step(ws_g, 0.01, itp)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64


CASES = {
    "f1_sm_zeeman_lhy": dict(F=1, c0=10.0, c1=-0.5, zeeman=(0.3, 0.1), c_lhy=0.7),
    "f1_afm": dict(F=1, c0=10.0, c1=0.5, zeeman=(0.0, 0.1)),
    "f2_euler": dict(F=2, c0=30.0, c1=2.0, zeeman=(0.2, -0.05)),
    "f6_euler": dict(F=6, c0=50.0, c1=3.0, zeeman=(0.1, 0.02)),
    "f2_tensor": dict(F=2, c0=30.0, c1=1.0, c_extra=(0.0, 0.0, 5.0)),
    "f6_tensor": dict(F=6, c0=200.0, c1=200.0 / 36, c_extra=(0.0, 0.0, 50.0), zeeman=(0.4, 0.0)),
    "f1_ddi": dict(F=1, c0=10.0, c1=0.3, ddi=True, c_dd=40.0),
    "f1_ddi_pad": dict(F=1, c0=10.0, c1=0.3, ddi=True, c_dd=40.0, padded=True),
    "f6_ddi_pad_sec": dict(F=6, c0=50.0, c1=0.5, ddi=True, c_dd=60.0, padded=True, secular=True),
    "f6_tensor_ddi_pad": dict(F=6, c0=200.0, c1=200.0 / 36, c_extra=(0.0, 0.0, 50.0), ddi=True, c_dd=100.0,
                              padded=True),
    # singlet-pair (nematic) step: c2 without a higher even c_k (src/nematic.jl)
    "f1_nematic": dict(F=1, c0=10.0, c1=-0.5, c_extra=(50.0,), zeeman=(0.1, 0.05)),
    "f2_nematic": dict(F=2, c0=30.0, c1=2.0, c_extra=(30.0,), zeeman=(0.2, -0.05)),
    "f1_nematic_ddi": dict(F=1, c0=10.0, c1=0.3, c_extra=(20.0,), ddi=True, c_dd=40.0),
}

CASE_GRIDS = [((64,), (20.0,)), ((16, 32), (8.0, 12.0)), ((8, 16, 8), (6.0, 8.0, 6.0))]


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("n,L", CASE_GRIDS)
@pytest.mark.parametrize("itp", [False, True])
def test_half_potential(gpu, case, n, L, itp):
    kw = dict(CASES[case])
    F = kw.pop("F")
    ws_o, ws_g = make_pair(n, L, F, omega=tuple(1.0 + 0.1 * d for d in range(len(n))), itp=itp, **kw)
    for tau in (2e-3, 5e-3):
        O.half_potential_step(ws_o, tau, itp)
        S.half_potential_step(ws_g, tau, itp)
    err = rel_psi_err(ws_g.psi, ws_o.psi)
    assert err < PSI_TOL_FP64, err


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("n,L", CASE_GRIDS)
def test_energy_terms(gpu, case, n, L):
    kw = dict(CASES[case])
    F = kw.pop("F")
    ws_o, ws_g = make_pair(n, L, F, omega=tuple(1.0 + 0.1 * d for d in range(len(n))), **kw)
    eo = O.energy_terms(ws_o)
    eg = S.energy_terms(ws_g)
    Eo = O.total_energy(ws_o)
    scale = max(abs(Eo), max(abs(v) for v in eo.values()))
    for k in eo:
        assert abs(eg[k] - eo[k]) <= ENERGY_TOL_FP64 * scale * 10, (k, eg[k], eo[k])
    assert abs(S.total_energy(ws_g) - Eo) <= ENERGY_TOL_FP64 * abs(Eo) * 10
    assert abs(S.total_norm(ws_g) - O.total_norm(ws_o.psi, ws_o.grid)) < 1e-13
    assert abs(S.magnetization(ws_g) - O.magnetization(ws_o.psi, ws_o.grid, F)) < 1e-12


@pytest.mark.parametrize("padded", [False, True])
@pytest.mark.parametrize("secular", [False, True])
@pytest.mark.parametrize("n,L", CASE_GRIDS)
def test_ddi_potential_fields(gpu, padded, secular, n, L):
    ws_o, ws_g = make_pair(n, L, 2, c0=5.0, ddi=True, c_dd=30.0, padded=padded, secular=secular)
    po = O.ddi_potential(ws_o, padded)
    pg = S.ddi_potential(ws_g, padded)
    scale = max(float(np.max(np.abs(p))) for p in po)
    for a, b in zip(pg, po):
        assert float(np.max(np.abs(a - b))) <= 1e-12 * scale
    so = O.spin_density(ws_o.psi, 2)
    sg = S.spin_density_vector(ws_g)
    for a, b in zip(sg, so):
        assert float(np.max(np.abs(a - b))) <= 1e-14 * max(1.0, float(np.max(np.abs(b))))


@pytest.mark.parametrize("n,L", CASE_GRIDS)
@pytest.mark.parametrize("case", ["f1_sm_zeeman_lhy", "f2_tensor", "f1_ddi_pad", "f1_nematic", "f2_nematic"])
def test_split_step_rt(gpu, n, L, case):
    kw = dict(CASES[case])
    F = kw.pop("F")
    ws_o, ws_g = make_pair(n, L, F, omega=tuple(1.0 for _ in n), dt=2e-3, **kw)
    for _ in range(5):
        O.split_step(ws_o)
    S.split_step(ws_g, 5)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    assert abs(ws_g.t - ws_o.t) < 1e-15 and ws_g.step == ws_o.step


@pytest.mark.parametrize("n,L", CASE_GRIDS)
def test_split_step_itp_normalises(gpu, n, L):
    ws_o, ws_g = make_pair(n, L, 1, c0=10.0, c1=-0.5, omega=tuple(1.0 for _ in n), dt=5e-3, itp=True)
    for _ in range(7):
        O.split_step(ws_o)
    S.split_step(ws_g, 7)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    assert abs(S.total_norm(ws_g) - 1.0) < 1e-13


@pytest.mark.parametrize("case", ["f1_sm_zeeman_lhy", "f6_tensor", "f1_ddi", "f6_tensor_ddi_pad"])
def test_strang_and_yoshida_core(gpu, case):
    kw = dict(CASES[case])
    F = kw.pop("F")
    n, L = ((16, 8, 8), (8.0, 6.0, 6.0)) if F == 6 else ((32, 16), (10.0, 8.0))
    ws_o, ws_g = make_pair(n, L, F, omega=tuple(1.0 for _ in n), **kw)
    O.strang_core(ws_o, 3e-3)
    S.strang_core(ws_g, 3e-3)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    O.yoshida_core(ws_o, 4e-3)
    S.yoshida_core(ws_g, 4e-3)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64


def test_tensor_channels_activation(gpu):
    # src/initialization.jl:164-185: c4 != 0 activates the tensor path with g = c0c1 base + 6j(c4)
    ip = O.interaction_params_from_constraint(c_total=4689.0, c1_ratio=1 / 36, F=6, c_extra=(0.0, 0.0, 50.0))
    ws_o, ws_g = make_pair((16,), (8.0,), 6, c0=ip.c0, c1=ip.c1, c_extra=ip.c_extra)
    active, g = ws_g.tensor_channels()
    assert active
    tc = ws_o.tensor_cache
    assert sorted(g) == sorted(tc.active_channels)
    for S_, gv in zip(tc.active_channels, tc.g_values):
        assert abs(g[S_] - gv) <= 1e-12 * abs(gv)


def test_unsupported_and_invalid(gpu):
    og = S.make_grid(S.GridConfig((2050,), (10.0,)))  # even, not a power of two, above 2048
    with pytest.raises(S.UnsupportedError):
        S.make_workspace(grid=og, atom=S.AtomSpecies("x", 1), interactions=S.InteractionParams(1.0, 0.0),
                         sim_params=S.SimParams(1e-3, 1))
    g2 = S.make_grid(S.GridConfig((16,), (10.0,)))
    with pytest.raises(S.UnsupportedError):  # spin F > 6
        S.make_workspace(grid=g2, atom=S.AtomSpecies("x", 7), interactions=S.InteractionParams(1.0, 0.0),
                         sim_params=S.SimParams(1e-3, 1))
    with pytest.raises(S.ArgumentError):
        S.make_workspace(grid=g2, atom=S.AtomSpecies("x", 1), interactions=S.InteractionParams(1.0, 0.0),
                         sim_params=S.SimParams(1e-3, 1), precision="fp16")
