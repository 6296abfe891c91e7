"""FFT line-kernel variants and their autotuner.

Every compiled variant (plan family x tile scale x stage form) must give the FP32-form result
on its own: each is forced in turn (SBEC_TUNE_FORCE, read when a workspace is
created) and checked against the FP64 oracle on the fused row/column path, the
batched ground state and the unfused x-line path (3-D with DDI).  With tuning on,
the decisions are reported and two workspaces of one shape give identical
results.  The ping-pong stage form (variants 4-7) does the arithmetic of the in-place
form (variants 0-3) in the same order, so the two give bit-identical states; so does the
register-resident row pass and strided lines (variants 12-15) against the tile forms of
the same plan and tile scale (variants 4-7)."""

import os

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import make_pair, rel_psi_err

pytestmark = pytest.mark.gpu

VARIANTS = list(range(8)) + [12, 13, 14, 15]


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


@pytest.mark.parametrize("v", VARIANTS)
def test_forced_variant_fused_2d(gpu, v):
    with _env(SBEC_TUNE_FORCE=v):
        ws_o, ws_g = make_pair((64, 64), (20.0, 20.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), zeeman=(0.0, 0.1),
                               dt=1e-3, precision="fp32", state="polar")
    for _ in range(50):
        O.split_step(ws_o)
    S.split_step(ws_g, 50)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < 5e-5
    assert "forced" in ws_g.tuning_report
    ws_g.close()


_GS_N, _GS_L = (128, 128), (20.0, 20.0)
_GS_C1 = [-0.5, 0.5, 0.2]
_GS_KW = dict(dt=0.005, n_steps=400, tol=1e-12)


@pytest.fixture(scope="module")
def gs_oracle():
    """Initial states and oracle ground-state energies, shared by every forced variant."""
    og = O.make_grid(O.GridConfig(_GS_N, _GS_L))
    psis = [O.init_psi(og, 1, st, seed=3) for st in ("polar", "ferromagnetic", "random")]
    energies = [O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, c1),
                                    V=O.harmonic_potential(og, (1.0, 1.0)), psi_init=p0, **_GS_KW)["energy"]
                for c1, p0 in zip(_GS_C1, psis)]
    return psis, energies


@pytest.mark.parametrize("v", VARIANTS)
def test_forced_variant_batched_ground_state(gpu, gs_oracle, v):
    psis, energies = gs_oracle
    hg = S.make_grid(S.GridConfig(_GS_N, _GS_L))
    with _env(SBEC_TUNE_FORCE=v):
        res = S.find_ground_states_batched(grid=hg, atom=S.Rb87, interactions=[S.InteractionParams(10.0, c)
                                                                               for c in _GS_C1],
                                           psi_inits=psis, potential=S.HarmonicTrap(1.0, 1.0), precision="fp32",
                                           **_GS_KW)
    for e_o, r in zip(energies, res):
        assert abs(r["energy"] - e_o) / abs(e_o) < 1e-6


@pytest.mark.parametrize("v", VARIANTS)
def test_forced_variant_unfused_3d_ddi(gpu, v):
    with _env(SBEC_TUNE_FORCE=v):
        ws_o, ws_g = make_pair((32, 32, 32), (16.0, 16.0, 16.0), 1, c0=5.0, c1=0.3, omega=(1.0, 1.0, 1.2),
                               ddi=True, c_dd=2.0, dt=1e-3, precision="fp32", state="ferromagnetic")
    for _ in range(5):
        O.split_step(ws_o)
    S.split_step(ws_g, 5)
    assert rel_psi_err(ws_g.psi, ws_o.psi) < 5e-5
    assert abs(S.total_energy(ws_g) - O.total_energy(ws_o)) / abs(O.total_energy(ws_o)) < 1e-5
    ws_g.close()


@pytest.mark.parametrize("v", [0, 1, 2, 3])
def test_ping_pong_stages_bit_identical(gpu, v):
    psis = []
    for form in (v, v + 4):
        with _env(SBEC_TUNE_FORCE=form):
            ws_g = make_pair((128, 64), (20.0, 20.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), zeeman=(0.0, 0.1),
                             dt=1e-3, precision="fp32", state="random", seed=5)[1]
        S.split_step(ws_g, 30)
        psis.append(ws_g.psi.copy())
        ws_g.close()
    assert np.array_equal(psis[0], psis[1])


@pytest.mark.parametrize("v", [4, 5, 6, 7])
@pytest.mark.parametrize("shape", [((128, 64), (20.0, 20.0), 1), ((256,), (20.0,), 1), ((64, 32), (16.0, 8.0), 2),
                                   ((32, 64, 32), (16.0, 16.0, 16.0), 1)])
def test_register_row_pass_bit_identical(gpu, v, shape):
    n, L, F = shape
    psis = []
    for form in (v, v + 8):
        with _env(SBEC_TUNE_FORCE=form):
            ws_g = make_pair(n, L, F, c0=10.0, c1=0.5, omega=(1.0,) * len(n), zeeman=(0.0, 0.1), dt=1e-3,
                             precision="fp32", state="random", seed=5)[1]
        S.split_step(ws_g, 30)
        assert f"row variant {form} (forced)" in ws_g.tuning_report
        psis.append(ws_g.psi.copy())
        ws_g.close()
    assert np.array_equal(psis[0], psis[1])


@pytest.mark.parametrize("v", [4, 5, 6, 7])
def test_register_row_pass_itp_matches_tile_form(gpu, v):
    # imaginary time: the renormalisation sums (FP64) are added in another order, so the
    # states agree to the last bits rather than bit for bit
    psis = []
    for form in (v, v + 8):
        with _env(SBEC_TUNE_FORCE=form):
            ws_g = make_pair((64, 64), (20.0, 20.0), 1, c0=10.0, c1=-0.5, omega=(1.0, 1.0), dt=5e-3,
                             itp=True, precision="fp32", state="random", seed=7)[1]
        S.split_step(ws_g, 40)
        psis.append(ws_g.psi.copy())
        ws_g.close()
    assert rel_psi_err(psis[1], psis[0]) < 1e-6


def test_tuning_reports_and_is_shared(gpu):
    with _env(SBEC_TUNE=1):
        # a shape no other test uses, so this process has not tuned it yet
        ws = [make_pair((128, 32), (20.0, 10.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), dt=1e-3, precision="fp32",
                        state="polar", seed=11)[1] for _ in range(2)]
    for w in ws:
        S.split_step(w, 20)
    rep = ws[0].tuning_report + ws[1].tuning_report
    assert "row" in rep and "chosen v" in rep
    # the second workspace reuses the first one's decisions: same kernels, same result
    assert np.array_equal(ws[0].psi, ws[1].psi)
    for w in ws:
        w.close()
