"""FP32-bulk form: FFTs and pointwise phases in FP32, reductions in FP64.
Each result states its error against the FP64 oracle; the bars are the chosen
form's targets (ground-state energy within 1e-6 relative, norm kept to 1e-7 per
renormalised ITP step and to ~1e-6 over real-time runs)."""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import make_pair, rel_psi_err

pytestmark = pytest.mark.gpu


def test_fp32_ground_state_energy(gpu):
    og = O.make_grid(O.GridConfig((64, 64), (20.0, 20.0)))
    hg = S.make_grid(S.GridConfig((64, 64), (20.0, 20.0)))
    kw = dict(dt=0.005, n_steps=1000, tol=1e-8, initial_state="ferromagnetic")
    ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                             V=O.harmonic_potential(og, (1.0, 1.0)), **kw)
    rg = S.find_ground_state(grid=hg, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                             potential=S.HarmonicTrap(1.0, 1.0), precision="fp32", **kw)
    err = abs(rg["energy"] - ro["energy"]) / abs(ro["energy"])
    assert err < 1e-6, err
    assert abs(S.total_norm(rg["workspace"]) - 1.0) < 1e-7


@pytest.mark.parametrize("case", ["f1", "f6_tensor_ddi"])
def test_fp32_real_time_error_bounded(gpu, case):
    if case == "f1":
        ws_o, ws_g = make_pair((64, 64), (20.0, 20.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), zeeman=(0.0, 0.1),
                               dt=1e-3, precision="fp32", state="polar")
        steps = 200
    else:
        ip = O.interaction_params_from_constraint(c_total=4689.0, c1_ratio=1 / 36, F=6, c_extra=(0.0, 0.0, 50.0))
        ws_o, ws_g = make_pair((8, 8, 8), (24.0, 24.0, 24.0), 6, c0=ip.c0, c1=ip.c1, c_extra=ip.c_extra,
                               omega=(1.0, 1.0, 1.2), ddi=True, c_dd=100.0, padded=True, dt=1e-3,
                               precision="fp32", state="ferromagnetic")
        steps = 20
    N0 = S.total_norm(ws_g)
    E0 = O.total_energy(ws_o)
    for _ in range(steps):
        O.split_step(ws_o)
    S.split_step(ws_g, steps)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < 5e-5
    assert abs(S.total_norm(ws_g) - N0) / N0 < 2e-6
    assert abs(S.total_energy(ws_g) - O.total_energy(ws_o)) / abs(E0) < 1e-5


@pytest.mark.parametrize("F,lanes", [(2, "1"), (6, "1"), (6, "0"), (2, "2"), (3, "2"), (4, "2"), (5, "2"), (6, "2"),
                                     (2, "3"), (4, "3"), (5, "3"), (6, "3"), (2, "-1"), (5, "-1"), (6, "-1")])
def test_fp32_tensor_step_kernels(gpu, F, lanes):
    """The FP32 general-F tensor step against the FP64 oracle, each kernel form by
    SBEC_TENSOR_LANES: 1 the lane-group kernel, 0 one thread per point, 2 rows of h in
    registers, 3 lane groups with two rows per lane, -1 the default choice by D."""
    import os

    ip = O.interaction_params_from_constraint(c_total=600.0, c1_ratio=1 / 36, F=F,
                                              c_extra=(0.0, 0.0, 50.0) if F == 6 else (0.0, 0.0, 20.0))
    old = os.environ.get("SBEC_TENSOR_LANES")
    os.environ["SBEC_TENSOR_LANES"] = lanes
    try:
        ws_o, ws_g = make_pair((16, 16, 16), (12.0, 12.0, 12.0), F, c0=ip.c0, c1=ip.c1, c_extra=ip.c_extra,
                               omega=(1.0, 1.0, 1.2), dt=1e-3, precision="fp32", state="random", seed=9)
    finally:
        if old is None:
            os.environ.pop("SBEC_TENSOR_LANES")
        else:
            os.environ["SBEC_TENSOR_LANES"] = old
    assert ws_g.tensor_channels()[0]
    for _ in range(10):
        O.split_step(ws_o)
    S.split_step(ws_g, 10)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < 5e-5
    assert abs(S.total_energy(ws_g) - O.total_energy(ws_o)) / abs(O.total_energy(ws_o)) < 1e-5
    ws_g.close()


def test_fp32_long_leapfrog_norm_from_real_ground_state(gpu):
    """2000 leapfrog steps from the (real) polar ground state in its trap: FP32 norm within
    1e-6 of FP64.  Round-to-nearest of small rotations of a near-real state gains norm
    at ~3.5e-9 per step; the unbiased rounding of the diagonal and kinetic phases
    leaves a zero-mean error."""
    n, L = (128, 128), (30.0, 30.0)
    hg = S.make_grid(S.GridConfig(n, L))
    gs = S.find_ground_state(grid=hg, atom=S.Na23, interactions=S.InteractionParams(10.0, 0.5),
                             zeeman=S.ZeemanParams(0.0, 0.1), potential=S.HarmonicTrap(1.0, 1.0), dt=0.005,
                             n_steps=400, tol=1e-9, initial_state="polar")
    psi0 = gs["workspace"].psi
    gs["workspace"].close()
    norms = {}
    for prec in ("fp32", "fp64"):
        ws = S.make_workspace(grid=hg, atom=S.Na23, interactions=S.InteractionParams(10.0, 0.5),
                              zeeman=S.ZeemanParams(0.0, 0.1), potential=S.HarmonicTrap(1.0, 1.0),
                              sim_params=S.SimParams(1e-3, 2000, False, None, 2000), psi_init=psi0, precision=prec)
        S.run_simulation(ws, keep_psi=False)
        norms[prec] = S.total_norm(ws)
        ws.close()
    assert abs(norms["fp32"] - norms["fp64"]) / norms["fp64"] < 1e-6


@pytest.mark.parametrize("n,L,F", [((64, 64), (20.0, 20.0), 2), ((32, 32, 32), (16.0,) * 3, 2), ((256,), (40.0,), 2),
                                   ((64, 64), (20.0, 20.0), 1)])
def test_fp32_leapfrog_norm_and_energy_with_zeeman_phases(gpu, n, L, F):
    """2000 real-time steps of a populated m != 0 component under a quadratic Zeeman term
    (q = 0.1: 2e-4 rad per half step at m = +-2): FP32 norm and energy within 4e-6 of the
    FP64 run (measured: about 1.2e-6 on these grids).  A Zeeman factor applied as its own
    rounded product drops the radial part of the small rotation at every call: the norm grew
    by ~4e-8 per step, 8e-5 over this run."""
    hg = S.make_grid(S.GridConfig(n, L))
    psi0 = S.init_psi(hg, F, "ferromagnetic" if F > 1 else "polar")
    res = {}
    for prec in ("fp32", "fp64"):
        ws = S.make_workspace(grid=hg, atom=S.AtomSpecies("x", F), interactions=S.InteractionParams(10.0, -0.3),
                              zeeman=S.ZeemanParams(0.0, 0.1), potential=S.HarmonicTrap(*([1.0] * len(n))),
                              sim_params=S.SimParams(1e-3, 2000, False, None, 2000), psi_init=psi0, precision=prec)
        r = S.run_simulation(ws, keep_psi=False)
        res[prec] = (S.total_norm(ws), r.energies[-1])
        ws.close()
    (n32, e32), (n64, e64) = res["fp32"], res["fp64"]
    assert abs(n32 - n64) / n64 < 4e-6, (n32, n64)
    assert abs(e32 - e64) / abs(e64) < 4e-6, (e32, e64)
