"""Persistent leapfrog segments (k_lf_segment, opt-in with SBEC_SEGMENT=1: one cooperative
launch per run of merged steps, grid-wide barriers between the column and row passes).

Each block does the per-line work of the separate row and column kernels with the same
FFT plan, so with the line kernels pinned to that plan (SBEC_TUNE_FORCE=0) the state
after a run is bit-identical with and without segments (SBEC_SEGMENT, read when a
workspace is created), save points included.  The segment path is also checked against
the oracle directly, with save points between segments and a user callback."""

import os

import numpy as np
import pytest

import oracle as O
import spinorbec as S

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


def _run(n, F, steps, save_every, segment, seed=3):
    L = (24.0, 24.0)
    g = S.make_grid(S.GridConfig((n, n), L))
    og = O.make_grid(O.GridConfig((n, n), L))
    psi0 = O.init_psi(og, F, "random", seed=seed)
    with _env(SBEC_SEGMENT=int(segment), SBEC_TUNE_FORCE=0):
        ws = S.make_workspace(grid=g, atom=S.AtomSpecies("x", F), interactions=S.InteractionParams(10.0, 0.5),
                              zeeman=S.ZeemanParams(0.0, 0.1), potential=S.HarmonicTrap(1.0, 1.0),
                              sim_params=S.SimParams(1e-3, steps, False, None, save_every), psi_init=psi0,
                              precision="fp32")
    res = S.run_simulation(ws, keep_psi=True)
    out = ws.psi
    ws.close()
    return out, res


@pytest.mark.parametrize("n,F", [(64, 1), (128, 1), (256, 1), (512, 1), (64, 0), (256, 0)])
def test_segment_bit_identical_to_line_kernels(gpu, n, F):
    steps = 60 if n < 512 else 24
    a, ra = _run(n, F, steps, 20 if n < 512 else 8, True)
    b, rb = _run(n, F, steps, 20 if n < 512 else 8, False)
    assert np.array_equal(a, b)
    assert len(ra.psi_snapshots) == len(rb.psi_snapshots)
    for x, y in zip(ra.psi_snapshots, rb.psi_snapshots):
        assert np.array_equal(x, y)
    assert ra.energies == rb.energies


def test_segment_against_oracle(gpu):
    n, L = (128, 128), (20.0, 20.0)
    og = O.make_grid(O.GridConfig(n, L))
    hg = S.make_grid(S.GridConfig(n, L))
    psi0 = O.init_psi(og, 1, "polar")
    ws_o = O.make_workspace(grid=og, atom=O.Na23, interactions=O.InteractionParams(10.0, 0.5),
                            zeeman=O.ZeemanParams(0.0, 0.1), V=O.harmonic_potential(og, (1.0, 1.0)),
                            sim_params=O.SimParams(1e-3, 40), psi_init=psi0)
    with _env(SBEC_SEGMENT=1):
        ws_g = S.make_workspace(grid=hg, atom=S.Na23, interactions=S.InteractionParams(10.0, 0.5),
                                zeeman=S.ZeemanParams(0.0, 0.1), potential=S.HarmonicTrap(1.0, 1.0),
                                sim_params=S.SimParams(1e-3, 40, False, None, 10), psi_init=psi0, precision="fp32")
    for _ in range(40):
        O.split_step(ws_o)
    seen = []
    S.run_simulation(ws_g, callback=lambda ws, step: seen.append(step), keep_psi=False)
    err = float(np.max(np.abs(ws_g.psi - ws_o.psi)) / np.max(np.abs(ws_o.psi)))
    dE = abs(S.total_energy(ws_g) - O.total_energy(ws_o)) / abs(O.total_energy(ws_o))
    ws_g.close()
    assert seen == [10, 20, 30, 40]
    assert err < 5e-5 and dE < 1e-5


def test_segment_barrier_timeout_reports_error_and_recovers(gpu):
    """Fault injected on the host (SBEC_FAULT_SEGMENT_STALL): the barrier's arrival counter
    starts beyond the block count, so every wait of the first segment runs out (bounded
    polling), the remaining segments of the run leave at once, and the run reports
    SBEC_ERR_DEVICE.  The context and the workspace stay usable: the next run, from the
    same initial state, matches a clean run bit for bit."""
    n, F = 64, 1
    L = (24.0, 24.0)
    g = S.make_grid(S.GridConfig((n, n), L))
    og = O.make_grid(O.GridConfig((n, n), L))
    psi0 = O.init_psi(og, F, "random", seed=3)

    def make(**env):
        with _env(SBEC_SEGMENT=1, SBEC_TUNE_FORCE=0, **env):
            return S.make_workspace(grid=g, atom=S.AtomSpecies("x", F), interactions=S.InteractionParams(10.0, 0.5),
                                    zeeman=S.ZeemanParams(0.0, 0.1), potential=S.HarmonicTrap(1.0, 1.0),
                                    sim_params=S.SimParams(1e-3, 30, False, None, 10), psi_init=psi0,
                                    precision="fp32")

    ws = make(SBEC_FAULT_SEGMENT_STALL=1)
    with pytest.raises(Exception, match="grid barrier"):
        S.run_simulation(ws, keep_psi=False)
    ws.psi = psi0
    ws.set_time(0.0, 0)
    S.run_simulation(ws, keep_psi=False)
    recovered = ws.psi
    ws.close()
    clean = make()
    S.run_simulation(clean, keep_psi=False)
    assert np.array_equal(recovered, clean.psi)
    clean.close()
