"""Batched ground states (multistart / continuation callers of find_ground_state):
every solve of a batch must give the same result as its own find_ground_state
run on the oracle (FP64), and stay within 1e-6 in energy in the FP32-bulk form."""

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, rel_psi_err

pytestmark = pytest.mark.gpu


def _starts(og, F, c1s):
    states = ["polar", "ferromagnetic", "uniform", "antiferromagnetic", "random"]
    psis, inter = [], []
    for i, c1 in enumerate(c1s):
        st = states[i % len(states)]
        psis.append(O.init_psi(og, F, st, seed=100 + i))
        inter.append((10.0, c1))
    return psis, inter


@pytest.mark.parametrize("n,L", [((64,), (16.0,)), ((32, 32), (16.0, 16.0))])
def test_batch_matches_individual_fp64(gpu, n, L):
    og = O.make_grid(O.GridConfig(n, L))
    hg = S.make_grid(S.GridConfig(n, L))
    c1s = [-1.0, -0.5, -0.1, 0.0, 0.3, 0.7, 1.0]
    psis, inter = _starts(og, 1, c1s)
    kw = dict(dt=0.005, n_steps=600, tol=1e-9)
    res = S.find_ground_states_batched(grid=hg, atom=S.Rb87, interactions=[S.InteractionParams(a, b) for a, b in inter],
                                       psi_inits=psis, zeeman=S.ZeemanParams(0.2, 0.05), potential=S.HarmonicTrap(*([1.0] * len(n))),
                                       precision="fp64", **kw)
    for (c0, c1), p0, r in zip(inter, psis, res):
        ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(c0, c1),
                                 zeeman=O.ZeemanParams(0.2, 0.05), V=O.harmonic_potential(og, (1.0,) * len(n)),
                                 psi_init=p0, **kw)
        assert r["converged"] == ro["converged"] and r["steps"] == ro["steps"]
        assert abs(r["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * abs(ro["energy"]) * 10
        assert rel_psi_err(r["psi"], ro["workspace"].psi) < PSI_TOL_FP64


def test_batch_fp32_energy(gpu):
    n, L = (64, 64), (20.0, 20.0)
    og = O.make_grid(O.GridConfig(n, L))
    hg = S.make_grid(S.GridConfig(n, L))
    c1s = [-0.5, 0.5]
    psis, inter = _starts(og, 1, c1s)
    kw = dict(dt=0.005, n_steps=1000, tol=1e-8)
    res = S.find_ground_states_batched(grid=hg, atom=S.Rb87, interactions=[S.InteractionParams(a, b) for a, b in inter],
                                       psi_inits=psis, potential=S.HarmonicTrap(1.0, 1.0), precision="fp32", **kw)
    for (c0, c1), p0, r in zip(inter, psis, res):
        ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(c0, c1),
                                 V=O.harmonic_potential(og, (1.0, 1.0)), psi_init=p0, **kw)
        assert abs(r["energy"] - ro["energy"]) / abs(ro["energy"]) < 1e-6


def test_batch_fp32_merged_step_energy(gpu):
    """SBEC_BATCH_MERGED=1: two passes per ITP step with a predicted renormalisation; the
    same ground state as the reference order (energy within 1e-6)."""
    import os

    n, L = (64, 64), (20.0, 20.0)
    og = O.make_grid(O.GridConfig(n, L))
    hg = S.make_grid(S.GridConfig(n, L))
    psis = [O.init_psi(og, 1, st, seed=5) for st in ("polar", "ferromagnetic")]
    c1s = [-0.5, 0.5]
    kw = dict(dt=0.005, n_steps=1000, tol=1e-8)
    old = os.environ.get("SBEC_BATCH_MERGED")
    os.environ["SBEC_BATCH_MERGED"] = "1"
    try:
        res = S.find_ground_states_batched(grid=hg, atom=S.Rb87, interactions=[S.InteractionParams(10.0, c)
                                                                               for c in c1s],
                                           psi_inits=psis, potential=S.HarmonicTrap(1.0, 1.0), precision="fp32", **kw)
    finally:
        if old is None:
            os.environ.pop("SBEC_BATCH_MERGED")
        else:
            os.environ["SBEC_BATCH_MERGED"] = old
    for c1, p0, r in zip(c1s, psis, res):
        ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, c1),
                                 V=O.harmonic_potential(og, (1.0, 1.0)), psi_init=p0, **kw)
        assert abs(r["energy"] - ro["energy"]) / abs(ro["energy"]) < 1e-6


def test_batch_on_mixed_grids_matches_per_grid_batches(gpu):
    """One batch object over solves on three grids (sbec_batch_create_grids: grouped by grid,
    the groups advance concurrently) gives each solve the result of a batch of its own grid,
    and the FP64 results match the oracle's find_ground_state per solve."""
    sizes = [32, 16, 32, 64, 16, 64]
    grids_o = {n: O.make_grid(O.GridConfig((n, n), (16.0, 16.0))) for n in set(sizes)}
    grids_s = {n: S.make_grid(S.GridConfig((n, n), (16.0, 16.0))) for n in set(sizes)}
    states = ["polar", "ferromagnetic", "random", "uniform", "random", "antiferromagnetic"]
    c1s = [-0.5, 0.3, 0.1, -0.2, 0.6, 0.0]
    psis = [O.init_psi(grids_o[n], 1, st, seed=40 + i) for i, (n, st) in enumerate(zip(sizes, states))]
    kw = dict(zeeman=S.ZeemanParams(0.1, 0.05), potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, precision="fp64")
    mixed = S.GroundStateBatch(grids=[grids_s[n] for n in sizes], atom=S.Rb87, c0s=[10.0] * 6, c1s=c1s,
                               psi_inits=psis, **kw)
    rm = mixed.ground_state(200, 1e-9)
    pm = [mixed.psi(i) for i in range(6)]
    mixed.close()
    for n in set(sizes):
        idx = [i for i, m in enumerate(sizes) if m == n]
        b = S.GroundStateBatch(grid=grids_s[n], atom=S.Rb87, c0s=[10.0] * len(idx), c1s=[c1s[i] for i in idx],
                               psi_inits=[psis[i] for i in idx], **kw)
        rb = b.ground_state(200, 1e-9)
        for k, i in enumerate(idx):
            assert rb[k] == rm[i]
            assert np.array_equal(b.psi(k), pm[i])
        b.close()
    for i, n in enumerate(sizes):
        ro = O.find_ground_state(grid=grids_o[n], atom=O.Rb87, interactions=O.InteractionParams(10.0, c1s[i]),
                                 zeeman=O.ZeemanParams(0.1, 0.05), V=O.harmonic_potential(grids_o[n], (1.0, 1.0)),
                                 psi_init=psis[i], dt=0.005, n_steps=200, tol=1e-9)
        assert rm[i]["steps"] == ro["steps"] and rm[i]["converged"] == ro["converged"]
        assert abs(rm[i]["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * 10 * abs(ro["energy"])
        assert rel_psi_err(pm[i], ro["workspace"].psi) < PSI_TOL_FP64


def test_batch_of_mixed_spins_matches_per_spin_batches(gpu):
    """One batch object over spin-1 and spin-2 solves on two grids (sbec_batch_create_mixed:
    grouped by grid and F) gives each solve the result of a batch of its own grid and F, and
    the spin-2 results match the oracle's find_ground_state."""
    F2 = S.AtomSpecies("87Rb-F2", 2)
    sizes = [32, 32, 16, 32, 16]
    Fs = [1, 2, 2, 1, 1]
    grids_o = {n: O.make_grid(O.GridConfig((n, n), (16.0, 16.0))) for n in set(sizes)}
    grids_s = {n: S.make_grid(S.GridConfig((n, n), (16.0, 16.0))) for n in set(sizes)}
    states = ["polar", "ferromagnetic", "random", "random", "uniform"]
    c1s = [-0.5, 0.3, 0.1, -0.2, 0.6]
    psis = [O.init_psi(grids_o[n], F, st, seed=60 + i) for i, (n, F, st) in enumerate(zip(sizes, Fs, states))]
    kw = dict(zeeman=S.ZeemanParams(0.1, 0.05), potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, precision="fp64")
    atoms = [S.Rb87 if F == 1 else F2 for F in Fs]
    mixed = S.GroundStateBatch(grids=[grids_s[n] for n in sizes], atoms=atoms, c0s=[10.0] * 5, c1s=c1s,
                               psi_inits=psis, **kw)
    rm = mixed.ground_state(150, 1e-9)
    pm = [mixed.psi(i) for i in range(5)]
    mixed.close()
    assert [p.shape[-1] for p in pm] == [2 * F + 1 for F in Fs]
    for key in set(zip(sizes, Fs)):
        idx = [i for i in range(5) if (sizes[i], Fs[i]) == key]
        b = S.GroundStateBatch(grid=grids_s[key[0]], atom=atoms[idx[0]], c0s=[10.0] * len(idx),
                               c1s=[c1s[i] for i in idx], psi_inits=[psis[i] for i in idx], **kw)
        rb = b.ground_state(150, 1e-9)
        for k, i in enumerate(idx):
            assert rb[k] == rm[i]
            assert np.array_equal(b.psi(k), pm[i])
        b.close()
    for i in (1, 2):
        n = sizes[i]
        ro = O.find_ground_state(grid=grids_o[n], atom=O.AtomSpecies("87Rb-F2", 2),
                                 interactions=O.InteractionParams(10.0, c1s[i]), zeeman=O.ZeemanParams(0.1, 0.05),
                                 V=O.harmonic_potential(grids_o[n], (1.0, 1.0)), psi_init=psis[i], dt=0.005,
                                 n_steps=150, tol=1e-9)
        assert rm[i]["steps"] == ro["steps"] and rm[i]["converged"] == ro["converged"]
        assert abs(rm[i]["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * 10 * abs(ro["energy"])
        assert rel_psi_err(pm[i], ro["workspace"].psi) < PSI_TOL_FP64


def test_batch_spin2_fp64_against_oracle(gpu):
    """Spin-2 solves (five components, spin mixing by the Euler rotation) in one batch."""
    og = O.make_grid(O.GridConfig((32, 32), (16.0, 16.0)))
    hg = S.make_grid(S.GridConfig((32, 32), (16.0, 16.0)))
    states = ["polar", "ferromagnetic", "random", "uniform"]
    c1s = [0.5, -0.5, 0.2, -0.1]
    psis = [O.init_psi(og, 2, st, seed=70 + i) for i, st in enumerate(states)]
    b = S.GroundStateBatch(grid=hg, atom=S.AtomSpecies("f2", 2), c0s=[10.0] * 4, c1s=c1s, psi_inits=psis,
                           potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, precision="fp64")
    res = b.ground_state(200, 1e-9)
    for i, (p0, c1, r) in enumerate(zip(psis, c1s, res)):
        ro = O.find_ground_state(grid=og, atom=O.AtomSpecies("f2", 2), interactions=O.InteractionParams(10.0, c1),
                                 V=O.harmonic_potential(og, (1.0, 1.0)), psi_init=p0, dt=0.005, n_steps=200, tol=1e-9)
        assert r["steps"] == ro["steps"] and r["converged"] == ro["converged"]
        assert abs(r["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * 10 * abs(ro["energy"])
        assert rel_psi_err(b.psi(i), ro["workspace"].psi) < PSI_TOL_FP64
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_spin2_nematic_against_oracle(gpu, precision):
    """Spin-2 solves with the nematic (singlet-pair) c2 shared by the batch: the pair step in
    both potential stages of the fused passes and the pair energy in the convergence test."""
    og = O.make_grid(O.GridConfig((32, 32), (16.0, 16.0)))
    hg = S.make_grid(S.GridConfig((32, 32), (16.0, 16.0)))
    states = ["polar", "ferromagnetic", "random", "uniform"]
    c1s = [0.5, -0.5, 0.2, -0.1]
    c2 = -0.4
    psis = [O.init_psi(og, 2, st, seed=80 + i) for i, st in enumerate(states)]
    n_steps = 200 if precision == "fp64" else 800
    b = S.GroundStateBatch(grid=hg, atom=S.AtomSpecies("f2", 2), c0s=[10.0] * 4, c1s=c1s, psi_inits=psis,
                           potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, c2=c2, precision=precision)
    res = b.ground_state(n_steps, 1e-9)
    for i, (p0, c1, r) in enumerate(zip(psis, c1s, res)):
        ro = O.find_ground_state(grid=og, atom=O.AtomSpecies("f2", 2),
                                 interactions=O.InteractionParams(10.0, c1, 0.0, (c2,)),
                                 V=O.harmonic_potential(og, (1.0, 1.0)), psi_init=p0, dt=0.005, n_steps=n_steps,
                                 tol=1e-9)
        if precision == "fp64":
            assert r["steps"] == ro["steps"] and r["converged"] == ro["converged"]
            assert abs(r["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * 10 * abs(ro["energy"])
            assert rel_psi_err(b.psi(i), ro["workspace"].psi) < PSI_TOL_FP64
        else:
            # FP32 bulk: the energy bar of the batched form against the FP64 oracle
            assert abs(r["energy"] - ro["energy"]) / abs(ro["energy"]) < 1e-6
    b.close()


def test_multistart_spin2_nematic_runs_batched(gpu):
    """find_ground_state_multistart takes the batch for spin-2 contact couplings with c2 and
    gives the one-at-a-time results."""
    hg = S.make_grid(S.GridConfig((32, 32), (16.0, 16.0)))
    kw = dict(grid=hg, atom=S.AtomSpecies("f2", 2), interactions=S.InteractionParams(10.0, 0.3, 0.0, (0.5,)),
              potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, n_steps=300, tol=1e-9, n_random=2, precision="fp64")
    rb = S.find_ground_state_multistart(batched=None, **kw)
    rs = S.find_ground_state_multistart(batched=False, **kw)
    assert rb["initial_state"] == rs["initial_state"]
    for a, c in zip(rb["all_results"], rs["all_results"]):
        assert a["steps"] == c["steps"] and a["converged"] == c["converged"]
        assert abs(a["energy"] - c["energy"]) <= 1e-11 * abs(c["energy"])
    rb["workspace"].close()
    for a in rs["all_results"]:
        a["workspace"].close()


def test_tune_table_import_fixes_the_variant(gpu):
    """A shape found in an imported tune table is not timed again: the workspace reports the
    table's variant, and an exported table loads back unchanged."""
    g = S.make_grid(S.GridConfig((64, 64), (16.0, 16.0)))
    ws = S.make_workspace(grid=g, atom=S.Rb87, interactions=S.InteractionParams(10.0, 0.5),
                          potential=S.HarmonicTrap(1.0, 1.0), sim_params=S.SimParams(1e-3, 20, False, None, 10),
                          precision="fp32")
    S.run_simulation(ws, keep_psi=False)
    table = S.tune_table_export()
    ws.close()
    assert "fp32 row" in table
    S.tune_table_import(table)
    ws2 = S.make_workspace(grid=g, atom=S.Rb87, interactions=S.InteractionParams(10.0, 0.5),
                           potential=S.HarmonicTrap(1.0, 1.0), sim_params=S.SimParams(1e-3, 20, False, None, 10),
                           precision="fp32")
    S.run_simulation(ws2, keep_psi=False)
    assert "from the process table" in ws2.tuning_report
    assert " chosen v" not in ws2.tuning_report  # nothing was timed
    ws2.close()


def test_batch_per_solve_limits_match_single_solves_fp64(gpu):
    """sbec_batch_ground_state_each: every solve with its own step limit and check interval
    (find_ground_state's max(1, n // 10)) follows the one-at-a-time find_ground_state."""
    g = S.make_grid(S.GridConfig((32, 32), (12.0, 12.0)))
    psi0 = S.init_psi(g, 1, "polar")
    c0s, c1s, steps = [10.0, 12.0, 8.0], [0.5, -0.5, 0.1], [300, 470, 120]
    b = S.GroundStateBatch(grid=g, atom=S.Rb87, c0s=c0s, c1s=c1s, psi_inits=[psi0] * 3,
                           potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, precision="fp64")
    rb = b.ground_state(steps, 1e-9)
    for i in range(3):
        rs = S.find_ground_state(grid=g, atom=S.Rb87, interactions=S.InteractionParams(c0s[i], c1s[i]),
                                 potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, n_steps=steps[i], tol=1e-9,
                                 initial_state="polar", precision="fp64")
        assert rb[i]["steps"] == rs["steps"] and rb[i]["converged"] == rs["converged"]
        assert abs(rb[i]["energy"] - rs["energy"]) <= 1e-12 * abs(rs["energy"])
        assert rel_psi_err(b.psi(i), rs["workspace"].psi) < 1e-11
        rs["workspace"].close()
    b.close()


def test_tune_freeze_takes_default_variants_untimed(gpu):
    """With the table frozen, a shape met for the first time is not timed: it takes its
    default variant, recorded in the table."""
    g = S.make_grid(S.GridConfig((32, 256), (8.0, 16.0)))  # a shape no other test tunes
    S.tune_freeze(True)
    try:
        ws = S.make_workspace(grid=g, atom=S.Rb87, interactions=S.InteractionParams(10.0, 0.5),
                              potential=S.HarmonicTrap(1.0, 1.0), sim_params=S.SimParams(1e-3, 20, False, None, 10),
                              precision="fp32")
        S.run_simulation(ws, keep_psi=False)
        rep = ws.tuning_report
        ws.close()
    finally:
        S.tune_freeze(False)
    assert "frozen table: default" in rep
    assert " chosen v" not in rep
