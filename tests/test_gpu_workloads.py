"""GPU parity at the benchmark workloads' own configurations, not at scaled-down grids.

* 2-D spin-1 256x256 real-time leapfrog (box 30, c0=10, c1=0.5, trap (1,1), q=0.1, dt=1e-3,
  save_every=50): 100 steps against the oracle's run_simulation (src/simulation.jl:49-94),
  FP64 at psi 1e-10 / energy 1e-12, the FP32-bulk form with its error stated.
* 3-D spin-6 Eu151 operator set (c_total=4689, c1_ratio=1/36, c4=50: all seven channels;
  zero-padded DDI c_dd=100; trap (1,1,1.2)): three accepted adaptive Yoshida steps
  (src/yoshida.jl:11-98) on 32^3 against the oracle with the same accept/reject counts; the
  FP32-bulk form on 32^3 against the oracle and on 64^3 against the FP64 form.
* Batched 2-D spin-1 ground states on 256x256 (box 20, c0=10, dt=0.005): eight solves
  (polar, ferromagnetic, uniform, antiferromagnetic, four random) against the oracle's
  find_ground_state per solve (src/ground_state.jl:80-170) over 30 steps with checks every 3
  (the oracle's spin-1 rotation costs ~0.2 s per step at this size); at convergence the FP32
  batch against the FP64 batch at 1e-6 in energy.
"""

import math

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from oracle.spinorbec_oracle import _gaussian
from parity_util import ENERGY_TOL_FP64, PSI_TOL_FP64, make_pair, rel_psi_err

pytestmark = pytest.mark.gpu

# FP32-bulk bars (errors against the FP64 oracle after the runs below)
PSI_TOL_FP32 = 5e-5
ENERGY_TOL_FP32 = 1e-6


def _noisy_polar(og, seed=20261203):
    """Polar state plus seeded complex Gaussian noise 1e-3 (N(0,1)+iN(0,1))/sqrt2 on m=+-1, normalised."""
    psi = O.init_psi(og, 1, "polar")
    rng = np.random.Generator(np.random.PCG64(seed))
    shp = og.config.n_points
    for c in (0, 2):
        psi[..., c] += 1e-3 * (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)) / math.sqrt(2.0)
    psi /= math.sqrt(float(np.sum(np.abs(psi) ** 2)) * O.cell_volume(og))
    return psi


# ---------------------------------------------------------------- 2-D 256^2 leapfrog

N2, L2 = (256, 256), (30.0, 30.0)


@pytest.fixture(scope="module")
def leapfrog_256_oracle():
    og = O.make_grid(O.GridConfig(N2, L2))
    psi0 = _noisy_polar(og)
    ws = O.make_workspace(grid=og, atom=O.Na23, interactions=O.InteractionParams(10.0, 0.5),
                          zeeman=O.ZeemanParams(0.0, 0.1), V=O.harmonic_potential(og, (1.0, 1.0)),
                          sim_params=O.SimParams(1e-3, 100, False, None, 50), psi_init=psi0)
    res = O.run_simulation(ws)
    return psi0, res, ws.psi.copy()


def _leapfrog_256_gpu(psi0, precision):
    hg = S.make_grid(S.GridConfig(N2, L2))
    ws = S.make_workspace(grid=hg, atom=S.Na23, interactions=S.InteractionParams(10.0, 0.5),
                          zeeman=S.ZeemanParams(0.0, 0.1), potential=S.HarmonicTrap(1.0, 1.0),
                          sim_params=S.SimParams(1e-3, 100, False, None, 50), psi_init=psi0, precision=precision)
    res = S.run_simulation(ws)
    psi = ws.psi
    ws.close()
    return res, psi


def test_leapfrog_256_fp64(gpu, leapfrog_256_oracle):
    psi0, ro, psi_o = leapfrog_256_oracle
    rg, psi_g = _leapfrog_256_gpu(psi0, "fp64")
    assert len(rg.times) == len(ro.times) == 3
    np.testing.assert_allclose(rg.times, ro.times, rtol=0, atol=1e-15)
    np.testing.assert_allclose(rg.energies, ro.energies, rtol=ENERGY_TOL_FP64)
    np.testing.assert_allclose(rg.norms, ro.norms, rtol=1e-13)
    np.testing.assert_allclose(rg.magnetizations, ro.magnetizations, atol=1e-12)
    for a, b in zip(rg.psi_snapshots, ro.psi_snapshots):
        assert rel_psi_err(a, b) < PSI_TOL_FP64
    assert rel_psi_err(psi_g, psi_o) < PSI_TOL_FP64


def test_leapfrog_256_fp32(gpu, leapfrog_256_oracle):
    psi0, ro, psi_o = leapfrog_256_oracle
    rg, psi_g = _leapfrog_256_gpu(psi0, "fp32")
    e_psi = rel_psi_err(psi_g, psi_o)
    e_E = max(abs(a - b) / abs(b) for a, b in zip(rg.energies, ro.energies))
    e_N = max(abs(a - b) / b for a, b in zip(rg.norms, ro.norms))
    print(f"FP32 256^2 leapfrog, 100 steps: psi {e_psi:.2e}, energy {e_E:.2e}, norm {e_N:.2e}")
    assert e_psi < PSI_TOL_FP32
    assert e_E < ENERGY_TOL_FP32
    assert e_N < 1e-6


# ---------------------------------------------------------------- 3-D spin-6 tensor + padded DDI

EU_IP = O.interaction_params_from_constraint(c_total=4689.0, c1_ratio=1 / 36, F=6, c_extra=(0.0, 0.0, 50.0))
AD = dict(dt_init=1e-3, dt_min=1e-5, dt_max=0.01, tol=1e-3)


def _eu_psi(n):
    og = O.make_grid(O.GridConfig((n,) * 3, (24.0,) * 3))
    psi = np.zeros((n,) * 3 + (13,), dtype=np.complex128, order="F")
    g = _gaussian(og, (3.0, 3.0, 3.0))
    rng = np.random.Generator(np.random.PCG64(11))
    psi[..., 0] = g * np.exp(1j * 0.01 * rng.standard_normal(g.shape))
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * O.cell_volume(og))
    return psi


def _eu_pair(n, precision):
    return make_pair((n,) * 3, (24.0,) * 3, 6, c0=EU_IP.c0, c1=EU_IP.c1, c_extra=EU_IP.c_extra,
                     omega=(1.0, 1.0, 1.2), ddi=True, c_dd=100.0, padded=True, psi=_eu_psi(n), precision=precision)


@pytest.fixture(scope="module")
def eu_32_oracle():
    og = O.make_grid(O.GridConfig((32,) * 3, (24.0,) * 3))
    ws_o = O.make_workspace(grid=og, atom=O.AtomSpecies("x", 6), interactions=EU_IP, zeeman=O.ZeemanParams(0.0, 0.0),
                            V=O.harmonic_potential(og, (1.0, 1.0, 1.2)), sim_params=O.SimParams(1e-3, 10, False),
                            psi_init=_eu_psi(32), enable_ddi=True, c_dd=100.0, ddi_padding=True)
    ro = O.run_simulation_yoshida(ws_o, O.AdaptiveDtParams(**AD), 1.0, 1.0, keep_psi=False, max_accepted=3)
    return ro, ws_o.psi.copy()


def _eu_gpu(n, precision):
    _, ws_g = _eu_pair(n, precision)
    rg = S.run_simulation_yoshida(ws_g, S.AdaptiveDtParams(**AD), t_end=1.0, save_interval=1.0, keep_psi=False,
                                  max_accepted=3)
    psi = ws_g.psi
    ws_g.close()
    return rg, psi


def test_eu151_yoshida_32_fp64(gpu, eu_32_oracle):
    ro, psi_o = eu_32_oracle
    rg, psi_g = _eu_gpu(32, "fp64")
    assert (rg["n_accepted"], rg["n_rejected"]) == (ro["n_accepted"], ro["n_rejected"]) == (3, ro["n_rejected"])
    assert abs(rg["final_dt"] - ro["final_dt"]) <= 1e-9 * ro["final_dt"]
    np.testing.assert_allclose(rg["result"].energies, ro["result"].energies, rtol=ENERGY_TOL_FP64 * 10)
    np.testing.assert_allclose(rg["result"].norms, ro["result"].norms, rtol=1e-13)
    assert rel_psi_err(psi_g, psi_o) < PSI_TOL_FP64


def test_eu151_yoshida_32_fp32(gpu, eu_32_oracle):
    ro, psi_o = eu_32_oracle
    rg, psi_g = _eu_gpu(32, "fp32")
    assert rg["n_accepted"] == 3
    e_psi = rel_psi_err(psi_g, psi_o)
    e_E = abs(rg["result"].energies[-1] - ro["result"].energies[-1]) / abs(ro["result"].energies[-1])
    print(f"FP32 32^3 spin-6 Yoshida, 3 steps: psi {e_psi:.2e}, energy {e_E:.2e}")
    assert e_psi < PSI_TOL_FP32
    assert e_E < ENERGY_TOL_FP32


def test_eu151_yoshida_64_fp32_vs_fp64(gpu):
    r64, p64 = _eu_gpu(64, "fp64")
    r32, p32 = _eu_gpu(64, "fp32")
    assert r64["n_accepted"] == r32["n_accepted"] == 3
    e_psi = rel_psi_err(p32, p64)
    e_E = abs(r32["result"].energies[-1] - r64["result"].energies[-1]) / abs(r64["result"].energies[-1])
    e_N = abs(r32["result"].norms[-1] - r64["result"].norms[-1]) / r64["result"].norms[-1]
    print(f"FP32 vs FP64 64^3 spin-6 Yoshida, 3 steps: psi {e_psi:.2e}, energy {e_E:.2e}, norm {e_N:.2e}")
    assert e_psi < PSI_TOL_FP32
    assert e_E < ENERGY_TOL_FP32
    assert e_N < 1e-7


# ---------------------------------------------------------------- batched 256^2 ground states

NB, LB = (256, 256), (20.0, 20.0)
BATCH_STARTS = [("polar", -1.0), ("ferromagnetic", -0.5), ("uniform", -0.1), ("antiferromagnetic", 0.2),
                ("random", 0.5), ("random", 0.75), ("random", 1.0), ("random", -0.75)]


def _batch_inputs(og):
    psis, c1s = [], []
    for i, (st, c1) in enumerate(BATCH_STARTS):
        psis.append(O.init_psi(og, 1, st, seed=4242 + i))
        c1s.append(c1)
    return psis, c1s


def _run_batch(psis, c1s, precision, n_steps, tol):
    hg = S.make_grid(S.GridConfig(NB, LB))
    b = S.GroundStateBatch(grid=hg, atom=S.Rb87, c0s=[10.0] * len(psis), c1s=c1s, psi_inits=psis,
                           potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, precision=precision)
    res = b.ground_state(n_steps, tol)
    for i, r in enumerate(res):
        r["psi"] = b.psi(i)
    b.close()
    return res


def test_batch_256_fp64_against_oracle(gpu):
    og = O.make_grid(O.GridConfig(NB, LB))
    psis, c1s = _batch_inputs(og)
    res = _run_batch(psis, c1s, "fp64", 30, 1e-8)
    for p0, c1, r in zip(psis, c1s, res):
        ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, c1),
                                 V=O.harmonic_potential(og, (1.0, 1.0)), psi_init=p0, dt=0.005, n_steps=30, tol=1e-8)
        assert r["converged"] == ro["converged"] and r["steps"] == ro["steps"]
        assert abs(r["energy"] - ro["energy"]) <= ENERGY_TOL_FP64 * 10 * abs(ro["energy"])
        assert rel_psi_err(r["psi"], ro["workspace"].psi) < PSI_TOL_FP64


def test_batch_256_fp32_converged_energy(gpu):
    og = O.make_grid(O.GridConfig(NB, LB))
    psis, c1s = _batch_inputs(og)
    r64 = _run_batch(psis, c1s, "fp64", 10000, 1e-8)
    r32 = _run_batch(psis, c1s, "fp32", 10000, 1e-8)
    # The 1e-8 test on max|psi - psi_prev| / max|psi| is below the FP32 resolution of psi
    # unless the FP32 map reaches a fixed point bit for bit, so FP32 solves may run all 10000
    # steps (50 time units); by then the energy has settled, and the bar is on the energy of
    # both forms at the end of their runs.
    worst = max(abs(a["energy"] - b["energy"]) / abs(b["energy"]) for a, b in zip(r32, r64))
    n32, n64 = sum(a["converged"] for a in r32), sum(b["converged"] for b in r64)
    for a, b in zip(r32, r64):
        print(f"  fp32 steps {a['steps']} dE {a['dE']:.2e} dpsi {a['dpsi']:.2e} | "
              f"fp64 steps {b['steps']} dE {b['dE']:.2e} dpsi {b['dpsi']:.2e}")
    print(f"FP32 vs FP64 batched 256^2 ground states: converged {n32} (FP32) / {n64} (FP64) of 8, "
          f"max energy error {worst:.2e}")
    assert worst < ENERGY_TOL_FP32
