"""Step blocks in CUDA-graph chunks: split_step! x n on the fused path (renormalisation
carried across chunks) and on the general path (DDI, tensor), and the general path's
leapfrog segments, replay graphs of up to 16 steps.  A replay runs the same kernels with
the same arguments as the eager launches (SBEC_GRAPHS=0), so the states are
bit-identical; the leapfrog with save points on the general path is also checked against
the oracle."""

import os

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, make_pair, rel_psi_err

pytestmark = pytest.mark.gpu


class _env:
    def __init__(self, **kv):
        self.kv = kv

    def __enter__(self):
        self.old = {k: os.environ.get(k) for k in self.kv}
        os.environ.update({k: str(v) for k, v in self.kv.items()})

    def __exit__(self, *a):
        for k, v in self.old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


CASES = {
    "fused_2d_f1": dict(n=(32, 32), L=(16.0, 16.0), F=1, c0=10.0, c1=0.5, omega=(1.0, 1.0)),
    "fused_1d_f2": dict(n=(64,), L=(16.0,), F=2, c0=20.0, c1=1.0, omega=(1.0,)),
    "ddi_2d_f1": dict(n=(32, 32), L=(16.0, 16.0), F=1, c0=10.0, c1=0.5, omega=(1.0, 1.0), ddi=True, c_dd=3.0),
    "tensor_1d_f2": dict(n=(64,), L=(16.0,), F=2, c0=20.0, c1=1.0, omega=(1.0,), c_extra=(0.0, 0.0, 2.0)),
    "tensor_ddi_2d_f2": dict(n=(16, 16), L=(12.0, 12.0), F=2, c0=20.0, c1=1.0, omega=(1.0, 1.0),
                             c_extra=(0.0, 0.0, 2.0), ddi=True, c_dd=2.0, padded=True),
}


def _pair(case, precision, itp, graphs):
    kw = dict(CASES[case])
    n, L, F, c0, c1 = kw.pop("n"), kw.pop("L"), kw.pop("F"), kw.pop("c0"), kw.pop("c1")
    with _env(SBEC_GRAPHS=int(graphs)):
        return make_pair(n, L, F, c0=c0, c1=c1, dt=1e-3 if not itp else 5e-3, itp=itp, precision=precision,
                         zeeman=(0.0, 0.1), **kw)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_graph_chunks_bit_identical(gpu, case, precision):
    out = {}
    for graphs in (1, 0):
        _, ws = _pair(case, precision, itp=True, graphs=graphs)
        S.split_step(ws, 37)         # two 16-step chunks and a 5-step one
        S.split_step(ws, 37)         # replayed
        a = ws.psi
        ws.close()
        _, ws = _pair(case, precision, itp=False, graphs=graphs)
        ws.sim_params = S.SimParams(1e-3, 45, False, None, 20)
        res = S.run_simulation(ws)
        out[graphs] = (a, ws.psi, res.energies)
        ws.close()
    assert np.array_equal(out[1][0], out[0][0])
    assert np.array_equal(out[1][1], out[0][1])
    assert out[1][2] == out[0][2]


def test_general_path_leapfrog_against_oracle(gpu):
    ws_o, ws_g = _pair("ddi_2d_f1", "fp64", itp=False, graphs=1)
    ws_o.sim_params = O.SimParams(1e-3, 45, False, None, 10)
    ws_g.sim_params = S.SimParams(1e-3, 45, False, None, 10)
    calls = []
    ro = O.run_simulation(ws_o)
    rg = S.run_simulation(ws_g, callback=lambda ws, step: calls.append(step))
    assert calls == [10, 20, 30, 40]
    np.testing.assert_allclose(rg.energies, ro.energies, rtol=ENERGY_TOL_FP64 * 10)
    for a, b in zip(rg.psi_snapshots, ro.psi_snapshots):
        assert rel_psi_err(a, b) < PSI_TOL_FP64
    assert rel_psi_err(ws_g.psi, ws_o.psi) < PSI_TOL_FP64
    ws_g.close()


def test_graph_mode_off_bit_identical(gpu):
    """sbec_set_graph_mode(ws, 0) (the serving workspaces' mode) gives the same state."""
    out = []
    for graphs in (True, False):
        _, ws = _pair("ddi_2d_f1", "fp32", itp=True, graphs=1)
        ws.set_graph_mode(graphs)
        S.split_step(ws, 37)
        S.split_step(ws, 37)
        out.append(ws.psi)
        ws.close()
    assert np.array_equal(out[0], out[1])
