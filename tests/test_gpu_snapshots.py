"""Pipelined save points of run_simulation (sbec_set_snapshot_mode): the snapshots and
the final state are bit-identical to synchronous delivery, and a stop request leaves
psi, t and step exactly at the save point that asked for it."""

import ctypes as C

import numpy as np
import pytest

import spinorbec as S
from parity_util import make_pair

pytestmark = pytest.mark.gpu


def _ws(precision):
    return make_pair((64, 64), (20.0, 20.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), zeeman=(0.0, 0.1), dt=1e-3,
                     precision=precision, state="polar", seed=5)[1]


def _set_run(ws, n_steps, save_every):
    ws.sim_params = S.SimParams(1e-3, n_steps, False, None, save_every)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_pipelined_equals_synchronous(gpu, precision):
    a, b = _ws(precision), _ws(precision)
    for w in (a, b):
        _set_run(w, 230, 40)  # last segment ends without a save point
    ra = S.run_simulation(a)                                     # pipelined (no user callback)
    rb = S.run_simulation(b, callback=lambda ws, step: None)     # synchronous
    assert ra.times == rb.times and ra.energies == rb.energies
    assert ra.norms == rb.norms and ra.magnetizations == rb.magnetizations
    assert len(ra.psi_snapshots) == len(rb.psi_snapshots) == 230 // 40 + 1
    for x, y in zip(ra.psi_snapshots, rb.psi_snapshots):
        assert np.array_equal(x, y)
    assert np.array_equal(a.psi, b.psi)
    assert (a.t, a.step) == (b.t, b.step)
    a.close()
    b.close()


def test_pipelined_stop_restores_save_point(gpu):
    lib = S._lib.load()
    seen = []

    def run(ws, mode):
        seen.clear()

        def cb(user, snap_p):
            s = snap_p.contents
            n = int(np.prod(ws.grid.config.n_points)) * ws.D
            seen.append((s.t, s.step, np.ctypeslib.as_array(s.psi, shape=(2 * n,)).copy()))
            return 1 if len(seen) == 3 else 0

        f = S._lib.CALLBACK(cb)
        S._lib.check(lib.sbec_set_snapshot_mode(ws.handle, mode))
        st = lib.sbec_run_simulation(ws.handle, 200, 25, f, None)
        with pytest.raises(S.CallbackStop):
            S._lib.check(st)
        return seen[-1]

    a, b = _ws("fp32"), _ws("fp32")
    ta, sa, pa = run(a, 1)
    tb, sb, pb = run(b, 0)
    assert (ta, sa) == (tb, sb) == (pytest.approx(0.05), 50)
    assert np.array_equal(pa, pb)
    for w, p in ((a, pa), (b, pb)):
        assert w.step == 50 and w.t == ta
        assert np.array_equal(S.to_interleaved(w.psi), p)
    a.close()
    b.close()
