"""GPU parity of the ground-state sweeps and diagnostics against the oracle:

* classify_phase on the device (src/diagnostics.jl:166-206) for spin-1, spin-2 and spin-6
  states, through a workspace and through a batch;
* scan_continuation (src/ground_state.jl:328-378) on a sweep whose energy jumps trigger the
  multistart fallback (:357-360), each point labelled by classify_phase (:363);
* the adaptive-dt ground state (src/ground_state.jl:172-237) with the same dt decisions;
* the ITP NaN guard (src/ground_state.jl:4-29, :142, :193) on a NaN planted in the host psi
  before upload, for the fixed-dt and the adaptive loop;
* find_phase_boundary (src/phase_boundary.jl:9-60): bisection on the device phase labels.
"""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, make_pair, rel_psi_err

pytestmark = pytest.mark.gpu


def _check_phase(rg, ro):
    assert rg["phase"] == ro["phase"]
    assert abs(rg["spin_order"] - ro["spin_order"]) <= 1e-12 * max(1.0, abs(ro["spin_order"]))
    assert abs(rg["nematic_order"] - ro["nematic_order"]) <= 1e-12 * max(1.0, abs(ro["nematic_order"]))
    assert abs(rg["magnetization_density"] - ro["magnetization_density"]) <= 1e-12
    assert set(rg["channel_weights"]) == set(ro["channel_weights"])
    for S_, w in ro["channel_weights"].items():
        assert abs(rg["channel_weights"][S_] - w) <= 1e-12


@pytest.mark.parametrize("n,L,F,state", [((64,), (10.0,), 1, "polar"), ((64,), (10.0,), 1, "ferromagnetic"),
                                         ((32, 32), (10.0, 10.0), 1, "random"),
                                         ((32,), (10.0,), 2, "ferromagnetic"), ((16, 16), (8.0, 8.0), 2, "random"),
                                         ((8, 8, 8), (6.0, 6.0, 6.0), 6, "random"),
                                         ((8, 8, 8), (6.0, 6.0, 6.0), 6, "uniform")])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_classify_phase(gpu, n, L, F, state, precision):
    og = O.make_grid(O.GridConfig(n, L))
    psi = O.init_psi(og, F, state, seed=9)
    _, ws = make_pair(n, L, F, c0=1.0, psi=psi, precision=precision)
    psi_dev = ws.psi  # the FP32 form classifies its own (rounded) state
    rg = S.classify_phase(ws)
    ws.close()
    _check_phase(rg, O.classify_phase(psi_dev, F, og))


def test_classify_phase_batch(gpu):
    og = O.make_grid(O.GridConfig((32, 32), (12.0, 12.0)))
    hg = S.make_grid(S.GridConfig((32, 32), (12.0, 12.0)))
    psis = [O.init_psi(og, 1, st, seed=3) for st in ("polar", "ferromagnetic", "random")]
    b = S.GroundStateBatch(grid=hg, atom=S.Rb87, c0s=[10.0] * 3, c1s=[0.5, -0.5, 0.1], psi_inits=psis,
                           potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, precision="fp64")
    b.ground_state(40, 1e-12)
    for i in range(3):
        _check_phase(b.classify_phase(i), O.classify_phase(b.psi(i), 1, og))
    b.close()


def test_scan_continuation_with_multistart_fallback(gpu):
    og = O.make_grid(O.GridConfig((32,), (16.0,)))
    hg = S.make_grid(S.GridConfig((32,), (16.0,)))
    vals = [5.0, 10.0, 10.5, 20.0]
    kw = dict(n_steps_continuation=100, n_steps_fresh=500, dt=0.005, tol=1e-8)
    ro = O.scan_continuation(param_values=vals, make_interactions=lambda v: O.InteractionParams(v, -0.5), grid=og,
                             atom=O.Rb87, V=O.harmonic_potential(og, (1.0,)), zeeman=O.ZeemanParams(0.05, 0.0), **kw)
    rg = S.scan_continuation(param_values=vals, make_interactions=lambda v: S.InteractionParams(v, -0.5), grid=hg,
                             atom=S.Rb87, potential=S.HarmonicTrap(1.0), zeeman=S.ZeemanParams(0.05, 0.0), **kw)
    assert [r["multistart"] for r in ro] == [False, True, False, True]  # the sweep exercises the fallback
    assert len(rg) == len(ro)
    for a, b in zip(rg, ro):
        assert a["param"] == b["param"]
        assert a["multistart"] == b["multistart"]
        assert a["phase"] == b["phase"]
        assert a["converged"] == b["converged"]
        assert abs(a["energy"] - b["energy"]) <= ENERGY_TOL_FP64 * 10 * abs(b["energy"])
        assert rel_psi_err(a["psi"], b["psi"]) < PSI_TOL_FP64


@pytest.mark.parametrize("batched", [None, False])
def test_find_phase_boundary(gpu, batched):
    """find_phase_boundary (src/phase_boundary.jl:9-60) on the device: the same probes, phases,
    evaluation count and boundary as the oracle; the endpoint solves as one batch (default) or
    one at a time."""
    og = O.make_grid(O.GridConfig((32,), (16.0,)))
    hg = S.make_grid(S.GridConfig((32,), (16.0,)))
    kw = dict(tol=0.05, max_bisections=10, dt=0.01, n_steps=600, initial_state="uniform")
    ro = O.find_phase_boundary(param_range=(-0.7, 0.4), make_interactions=lambda v: O.InteractionParams(10.0, v),
                               grid=og, atom=O.Rb87, V=O.harmonic_potential(og, (1.0,)), **kw)
    rg = S.find_phase_boundary(param_range=(-0.7, 0.4), make_interactions=lambda v: S.InteractionParams(10.0, v),
                               grid=hg, atom=S.Rb87, potential=S.HarmonicTrap(1.0), batched=batched, **kw)
    assert rg == ro


def test_adaptive_ground_state(gpu):
    og = O.make_grid(O.GridConfig((64,), (15.0,)))
    hg = S.make_grid(S.GridConfig((64,), (15.0,)))
    kw = dict(dt=0.001, n_steps=1000, tol=1e-7, adaptive_dt=True, dt_max=0.01)
    ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                             V=O.harmonic_potential(og, (1.0,)), **kw)
    rg = S.find_ground_state(grid=hg, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                             potential=S.HarmonicTrap(1.0), **kw)
    assert rg["converged"] == ro["converged"] and rg["steps"] == ro["steps"]
    assert abs(rg["final_dt"] - ro["final_dt"]) <= 1e-12 * ro["final_dt"]
    assert abs(rg["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * abs(ro["energy"])
    assert rel_psi_err(rg["workspace"].psi, ro["workspace"].psi) < PSI_TOL_FP64
    rg["workspace"].close()


@pytest.mark.parametrize("adaptive", [False, True])
def test_itp_nan_planted_before_upload(gpu, adaptive):
    og = O.make_grid(O.GridConfig((32, 32), (12.0, 12.0)))
    hg = S.make_grid(S.GridConfig((32, 32), (12.0, 12.0)))
    psi = O.init_psi(og, 1, "polar")
    psi[7, 9, 1] = complex(np.nan, 0.0)
    kw = dict(dt=0.005, n_steps=200, tol=1e-8, psi_init=psi, adaptive_dt=adaptive)
    with pytest.raises(ValueError, match="NaN detected in ITP at step 1"):
        O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                            V=O.harmonic_potential(og, (1.0, 1.0)), **kw)
    with pytest.raises(S.NumericError, match="NaN detected in ITP at step 1"):
        S.find_ground_state(grid=hg, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5),
                            potential=S.HarmonicTrap(1.0, 1.0), **kw)
