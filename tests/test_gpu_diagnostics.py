"""``estimate_splitting_error`` and ``validate_conservation`` (src/diagnostics.jl:214-293) on
the device against the oracle: the same splitting-error estimate and conservation drifts, with
the workspace's psi, time and step restored exactly."""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import make_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,L,F,itp", [((64,), (10.0,), 1, False), ((32, 32), (12.0, 12.0), 2, False),
                                       ((32, 32), (12.0, 12.0), 1, True), ((48, 40), (12.0, 10.0), 1, False)])
def test_splitting_error_matches_oracle_and_restores(gpu, n, L, F, itp):
    ws_o, ws_g = make_pair(n, L, F, c0=10.0, c1=-0.5, omega=(1.0,) * len(n), zeeman=(0.0, 0.1), dt=0.01, itp=itp)
    for _ in range(3):
        O.split_step(ws_o)
    S.split_step(ws_g, 3)
    psi_before = ws_g.psi
    t_before = ws_g.t
    eo = O.estimate_splitting_error(ws_o)
    eg = S.estimate_splitting_error(ws_g)
    assert eg > 0
    assert abs(eg - eo) <= 1e-6 * eo, (eg, eo)
    assert np.array_equal(ws_g.psi, psi_before) and ws_g.t == t_before
    # the workspace steps on at its own dt afterwards
    O.split_step(ws_o)
    S.split_step(ws_g, 1)
    assert np.abs(ws_g.psi - ws_o.psi).max() / np.abs(ws_o.psi).max() < 1e-10
    ws_g.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_validate_conservation_matches_oracle(gpu, precision):
    ws_o, ws_g = make_pair((64,), (10.0,), 1, c0=10.0, c1=-0.5, omega=(1.0,), dt=0.001, precision=precision,
                           state="polar")
    ro = O.validate_conservation(ws_o, n_steps=50)
    psi_before = ws_g.psi
    rg = S.validate_conservation(ws_g, n_steps=50)
    assert np.array_equal(ws_g.psi, psi_before)
    assert ro["passed"]
    if precision == "fp64":
        assert rg["passed"] == ro["passed"]
        assert rg["norm_drift"] < 1e-12
        assert abs(rg["energy_drift"] - ro["energy_drift"]) < 1e-10
        assert abs(rg["magnetization_drift"] - ro["magnetization_drift"]) < 1e-10
    else:
        # FP32 bulk: drifts at its rounding level (the default 1e-12 norm bar is an FP64 bar)
        assert rg["norm_drift"] < 1e-5 and rg["energy_drift"] < 1e-3
    ws_g.close()
