"""Shared builders for the parity tests: the same seeded inputs go to the oracle
(CPU FP64 restatement) and to the GPU engine through the C ABI."""

from __future__ import annotations

import numpy as np

import oracle as O
import spinorbec as S

PSI_TOL_FP64 = 1e-10      # max |Δψ| / max |ψ| (parity bar of the plain FP64 form)
ENERGY_TOL_FP64 = 1e-12   # relative energy


def rel_psi_err(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def make_pair(n, L, F, c0=0.0, c1=0.0, *, omega=None, zeeman=(0.0, 0.0), dt=1e-3, itp=False, c_extra=(),
              c_lhy=0.0, ddi=False, c_dd=0.0, padded=False, secular=False, psi=None, seed=7,
              precision="fp64", state="random", normalize_every=None, gS=None, raman=None, loss=None):
    """raman = (Omega_R, delta, k_eff), loss = (gamma_dr, L3): the same RamanCoupling /
    LossParams on both sides."""
    n = tuple(n)
    L = tuple(L)
    og = O.make_grid(O.GridConfig(n, L))
    hg = S.make_grid(S.GridConfig(n, L))
    V = O.harmonic_potential(og, omega) if omega is not None else None
    if psi is None:
        psi = O.init_psi(og, F, state, seed=seed)
    sp_o = O.SimParams(dt, 10, itp, normalize_every)
    sp_h = S.SimParams(dt, 10, itp, normalize_every)
    ws_o = O.make_workspace(grid=og, atom=O.AtomSpecies("x", F), interactions=O.InteractionParams(c0, c1, c_lhy,
                            tuple(c_extra)), zeeman=O.ZeemanParams(*zeeman), V=V, sim_params=sp_o, psi_init=psi,
                            enable_ddi=ddi, c_dd=c_dd, secular_ddi=secular, ddi_padding=padded,
                            raman=O.RamanCoupling(*raman) if raman else None,
                            loss=O.LossParams(*loss) if loss else None)
    if gS is not None:
        ws_o.tensor_cache = O.make_tensor_cache_from_channels(F, gS)
        ws_o.interactions = O.InteractionParams(0.0, 0.0, c_lhy, ())
    ws_g = S.make_workspace(grid=hg, atom=S.AtomSpecies("x", F), interactions=S.InteractionParams(c0, c1, c_lhy,
                            tuple(c_extra)), zeeman=S.ZeemanParams(*zeeman), potential=V, sim_params=sp_h,
                            psi_init=psi, enable_ddi=ddi, c_dd=c_dd, secular_ddi=secular, ddi_padding=padded,
                            precision=precision, gS=gS, raman=S.RamanCoupling(*raman) if raman else None,
                            loss=S.LossParams(*loss) if loss else None)
    return ws_o, ws_g
