"""numpy / scipy.fft FP64 restatement of SpinorBEC.jl's split-step hot path.

TEST INFRASTRUCTURE ONLY (the checker, never the product): see the package
docstring in ``oracle/__init__.py``.

Conventions (identical to the reference, ``src/types.jl:239-244``):

* ``psi`` has shape ``n_points + (D,)`` in Fortran (column-major) order, so
  its flat memory is the reference's ``psi[x, (y, (z,)) c]`` layout: x fastest,
  one planar block of ``prod(n_points)`` complex values per component.
* component index ``c`` (0-based here) carries ``m = F - c``
  (``src/types.jl:43-48``).
* FFTs over the spatial axes: forward unnormalised, inverse normalised by
  ``1/prod(n_points)`` (FFTW's ``fft!`` / ``ifft!``, ``src/propagators.jl:121-135``).

Every function cites the reference file:line it restates.  Arithmetic is
written in the reference's evaluation order where the order is visible in the
Julia source, so that the restatement agrees with the reference to rounding.
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np
import scipy.fft as sfft

_WORKERS = max(1, os.cpu_count() or 1)


def set_fft_workers(n: int) -> None:
    """Number of threads pocketfft may use (the reference's FFTW runs single-threaded)."""
    global _WORKERS
    _WORKERS = max(1, int(n))


# ----------------------------------------------------------------------------
# Grid  (src/types.jl:7-20, src/grid.jl:1-53)
# ----------------------------------------------------------------------------

def fftfreq(n: int, fs: float) -> np.ndarray:
    """FFTW.jl ``fftfreq(n, fs)``: index × (fs/n), indices 0..ceil(n/2)-1, -floor(n/2)..-1."""
    mult = fs / n
    idx = np.concatenate([np.arange(0, (n + 1) // 2), np.arange(-(n // 2), 0)]).astype(np.float64)
    return idx * mult


def rfftfreq(n: int, fs: float) -> np.ndarray:
    """FFTW.jl ``rfftfreq(n, fs)``: index × (fs/n), indices 0..n÷2."""
    mult = fs / n
    return np.arange(0, n // 2 + 1).astype(np.float64) * mult


@dataclass(frozen=True)
class GridConfig:
    """``GridConfig`` (src/types.jl:7-20): even, positive point counts; positive box sizes."""

    n_points: tuple
    box_size: tuple

    def __post_init__(self):
        n = tuple(int(v) for v in self.n_points)
        L = tuple(float(v) for v in self.box_size)
        if len(n) != len(L) or not (1 <= len(n) <= 3):
            raise ValueError("n_points and box_size must have the same length (1..3)")
        if not all(v > 0 and v % 2 == 0 for v in n):
            raise ValueError("n_points must be positive even integers")
        if not all(v > 0 for v in L):
            raise ValueError("box_size must be positive")
        object.__setattr__(self, "n_points", n)
        object.__setattr__(self, "box_size", L)

    @property
    def ndim(self) -> int:
        return len(self.n_points)


@dataclass
class Grid:
    config: GridConfig
    x: tuple
    dx: tuple
    k: tuple
    dk: tuple
    k_squared: np.ndarray


def make_grid(config: GridConfig) -> Grid:
    """``make_grid`` (src/grid.jl:1-23) and ``_compute_k_squared`` (src/grid.jl:25-35)."""
    xs, dxs, ks, dks = [], [], [], []
    for n, L in zip(config.n_points, config.box_size):
        dx = L / n
        xs.append(np.linspace(-L / 2 + dx / 2, L / 2 - dx / 2, n))
        dxs.append(dx)
        dk = 2 * math.pi / L
        ks.append(fftfreq(n, n * dk))
        dks.append(dk)
    ksq = np.zeros(config.n_points, dtype=np.float64, order="F")
    for d, kd in enumerate(ks):
        shape = [1] * config.ndim
        shape[d] = -1
        ksq = ksq + (kd ** 2).reshape(shape)
    return Grid(config, tuple(xs), tuple(dxs), tuple(ks), tuple(dks), np.asfortranarray(ksq))


def cell_volume(grid: Grid) -> float:
    """``cell_volume`` (src/grid.jl:55-57)."""
    v = 1.0
    for d in grid.dx:
        v *= d
    return v


def rfft_output_shape(n_pts: Sequence[int]) -> tuple:
    """``rfft_output_shape`` (src/grid.jl:44): the first axis is halved."""
    return (n_pts[0] // 2 + 1,) + tuple(n_pts[1:])


# ----------------------------------------------------------------------------
# Spin matrices  (src/spin_matrices.jl:1-50)
# ----------------------------------------------------------------------------

@dataclass
class SpinMatrices:
    F: int
    D: int
    m_values: np.ndarray
    Fx: np.ndarray
    Fy: np.ndarray
    Fz: np.ndarray
    Fp: np.ndarray
    Fm: np.ndarray
    Fy_eigvecs: np.ndarray
    Fy_eigvecs_adj: np.ndarray
    Fy_eigvals: np.ndarray


def spin_matrices(F: int) -> SpinMatrices:
    """``spin_matrices`` (src/spin_matrices.jl:1-50); Fy eigen-decomposition in ascending order."""
    if F < 0:
        raise ValueError("F must be non-negative")
    D = 2 * F + 1
    m = np.array([F - c for c in range(D)], dtype=np.int64)
    Fp = np.zeros((D, D), dtype=np.complex128)
    for j in range(D):
        for i in range(D):
            if m[i] == m[j] + 1:
                Fp[i, j] = math.sqrt(F * (F + 1) - m[j] * (m[j] + 1))
    Fm = Fp.conj().T.copy()
    Fx = (Fp + Fm) / 2
    Fy = (Fp - Fm) / 2j
    Fz = np.diag(m.astype(np.float64)).astype(np.complex128)
    vals, vecs = np.linalg.eigh(Fy, UPLO="U")
    if D > 1 and not np.all(np.abs(np.diff(vals) - 1.0) < 1e-10):
        raise AssertionError(f"Fy eigenvalues not uniformly spaced: {vals}")
    return SpinMatrices(F, D, m.astype(np.float64), Fx, Fy, Fz, Fp, Fm,
                        vecs.copy(), vecs.conj().T.copy(), vals.copy())


# ----------------------------------------------------------------------------
# Clebsch-Gordan / Wigner symbols  (src/clebsch_gordan.jl:1-180)
# ----------------------------------------------------------------------------

def _log_factorial(n: int) -> float:
    """``_log_factorial`` (src/clebsch_gordan.jl:4-12)."""
    if n < 0:
        return -math.inf
    s = 0.0
    for i in range(2, n + 1):
        s += math.log(i)
    return s


def _log_triangle_coeff(a: int, b: int, c: int) -> float:
    """``_log_triangle_coeff`` (src/clebsch_gordan.jl:18-24)."""
    ab, ac, bc = a + b - c, a - b + c, -a + b + c
    if ab < 0 or ac < 0 or bc < 0:
        return -math.inf
    return (_log_factorial(ab) + _log_factorial(ac) + _log_factorial(bc)
            - _log_factorial(a + b + c + 1))


def wigner_3j(j1, j2, j3, m1, m2, m3) -> float:
    """``wigner_3j`` Racah formula in log space (src/clebsch_gordan.jl:33-63)."""
    if m1 + m2 + m3 != 0:
        return 0.0
    log_tri = _log_triangle_coeff(j1, j2, j3)
    if log_tri == -math.inf:
        return 0.0
    log_num = (_log_factorial(j1 + m1) + _log_factorial(j1 - m1) + _log_factorial(j2 + m2)
               + _log_factorial(j2 - m2) + _log_factorial(j3 + m3) + _log_factorial(j3 - m3))
    t_min = max(0, j2 - j3 - m1, j1 - j3 + m2)
    t_max = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    if t_min > t_max:
        return 0.0
    s = 0.0
    for t in range(t_min, t_max + 1):
        log_den = (_log_factorial(t) + _log_factorial(j1 + j2 - j3 - t) + _log_factorial(j1 - m1 - t)
                   + _log_factorial(j2 + m2 - t) + _log_factorial(j3 - j2 + m1 + t)
                   + _log_factorial(j3 - j1 - m2 + t))
        sign = 1.0 if t % 2 == 0 else -1.0
        s += sign * math.exp(-log_den)
    phase = 1.0 if (j1 - j2 - m3) % 2 == 0 else -1.0
    return phase * math.exp(0.5 * (log_tri + log_num)) * s


def clebsch_gordan(j1, m1, j2, m2, J, M) -> float:
    """``clebsch_gordan`` via the 3j symbol (src/clebsch_gordan.jl:69-74)."""
    if m1 + m2 != M:
        return 0.0
    phase = 1.0 if (j1 - j2 + M) % 2 == 0 else -1.0
    return phase * math.sqrt(2 * J + 1) * wigner_3j(j1, j2, J, m1, m2, -M)


def wigner_6j(j1, j2, j3, j4, j5, j6) -> float:
    """``wigner_6j`` Racah formula in log space (src/clebsch_gordan.jl:80-110)."""
    t1 = _log_triangle_coeff(j1, j2, j3)
    t2 = _log_triangle_coeff(j1, j5, j6)
    t3 = _log_triangle_coeff(j4, j2, j6)
    t4 = _log_triangle_coeff(j4, j5, j3)
    if -math.inf in (t1, t2, t3, t4):
        return 0.0
    log_tri_sum = 0.5 * (t1 + t2 + t3 + t4)
    t_min = max(j1 + j2 + j3, j1 + j5 + j6, j4 + j2 + j6, j4 + j5 + j3)
    t_max = min(j1 + j2 + j4 + j5, j2 + j3 + j5 + j6, j1 + j3 + j4 + j6)
    if t_min > t_max:
        return 0.0
    s = 0.0
    for t in range(t_min, t_max + 1):
        log_num = _log_factorial(t + 1)
        log_den = (_log_factorial(t - j1 - j2 - j3) + _log_factorial(t - j1 - j5 - j6)
                   + _log_factorial(t - j4 - j2 - j6) + _log_factorial(t - j4 - j5 - j3)
                   + _log_factorial(j1 + j2 + j4 + j5 - t) + _log_factorial(j2 + j3 + j5 + j6 - t)
                   + _log_factorial(j1 + j3 + j4 + j6 - t))
        sign = 1.0 if t % 2 == 0 else -1.0
        s += sign * math.exp(log_num - log_den)
    return math.exp(log_tri_sum) * s


def _build_6j_matrix(F: int):
    """``_build_6j_matrix`` (src/clebsch_gordan.jl:118-128)."""
    even = list(range(0, 2 * F + 1, 2))
    W = np.zeros((len(even), len(even)))
    for i, S in enumerate(even):
        for j, k in enumerate(even):
            W[i, j] = (2 * k + 1) * wigner_6j(F, F, k, F, F, S)
    return W, even


def cn_to_gS(F: int, c_dict: dict) -> dict:
    """``_cn_to_gS``: g_S = Σ_k (2k+1){F F k; F F S} c_k (src/clebsch_gordan.jl:135-141)."""
    W, even = _build_6j_matrix(F)
    c_vec = np.array([c_dict.get(k, 0.0) for k in even])
    g_vec = W @ c_vec
    return {S: float(g_vec[i]) for i, S in enumerate(even)}


def gS_to_cn(F: int, g_dict: dict) -> dict:
    """``_gS_to_cn`` inverse 6j transform (src/clebsch_gordan.jl:148-154)."""
    W, even = _build_6j_matrix(F)
    g_vec = np.array([g_dict.get(S, 0.0) for S in even])
    c_vec = np.linalg.solve(W, g_vec)
    return {k: float(c_vec[j]) for j, k in enumerate(even)}


def precompute_cg_table(F: int) -> dict:
    """``precompute_cg_table``: even l only, |val| < 1e-15 dropped (src/clebsch_gordan.jl:166-180)."""
    table = {}
    for l in range(0, 2 * F + 1, 2):
        for M in range(-l, l + 1):
            for m1 in range(-F, F + 1):
                m2 = M - m1
                if abs(m2) > F:
                    continue
                val = clebsch_gordan(F, m1, F, m2, l, M)
                if abs(val) < 1e-15:
                    continue
                table[(l, M, m1, m2)] = val
    return table


# ----------------------------------------------------------------------------
# Interaction parameters  (src/types.jl:145-170, src/interactions.jl:123-190)
# ----------------------------------------------------------------------------

@dataclass
class InteractionParams:
    """``InteractionParams(c0, c1, c_lhy, c_extra)``; ``c_extra[n-2]`` = c_n (src/types.jl:145-162)."""

    c0: float
    c1: float
    c_lhy: float = 0.0
    c_extra: tuple = ()


def get_cn(ip: InteractionParams, n: int) -> float:
    """``get_cn`` (src/types.jl:164-170)."""
    if n == 0:
        return ip.c0
    if n == 1:
        return ip.c1
    idx = n - 1
    return float(ip.c_extra[idx - 1]) if idx <= len(ip.c_extra) else 0.0


def c0c1_to_gS(F: int, c0: float, c1: float) -> dict:
    """``_c0c1_to_gS``: g_S = c0 + c1 (S(S+1) - 2F(F+1))/2 (src/interactions.jl:123-128)."""
    return {S: c0 + c1 * (S * (S + 1) - 2 * F * (F + 1)) / 2 for S in range(0, 2 * F + 1, 2)}


def c_extra_to_delta_gS(F: int, c_extra: Sequence[float]) -> dict:
    """``_c_extra_to_delta_gS`` (src/interactions.jl:140-155): even ranks 2..2F via 6j."""
    c_dict = {}
    for idx, val in enumerate(c_extra, start=1):
        k = idx + 1
        if abs(val) > 1e-30 and k % 2 == 0 and k <= 2 * F:
            c_dict[k] = float(val)
    if not c_dict:
        return {}
    return cn_to_gS(F, c_dict)


def interaction_params_from_constraint(*, c_total: float, c1_ratio: float = 0.0, F: int,
                                       c_extra: Sequence[float] = ()) -> InteractionParams:
    """``interaction_params_from_constraint``: c0 + F² c1 = c_total (src/interactions.jl:182-188)."""
    c0 = c_total / (1.0 + F ** 2 * c1_ratio)
    c1 = c1_ratio * c0
    return InteractionParams(c0, c1, 0.0, tuple(float(v) for v in c_extra))


# ----------------------------------------------------------------------------
# Tensor interaction cache  (src/tensor_interaction.jl:1-128, 165-193, 278-305)
# ----------------------------------------------------------------------------

@dataclass
class TensorCache:
    F: int
    D: int
    cg_table: dict
    active_channels: list
    g_values: list


def make_tensor_cache_from_channels(F: int, g_dict: dict) -> Optional[TensorCache]:
    """``_make_tensor_cache_from_channels`` (src/tensor_interaction.jl:106-118)."""
    active, g = [], []
    for S in range(0, 2 * F + 1, 2):
        gS = g_dict.get(S, 0.0)
        if abs(gS) > 1e-30:
            active.append(S)
            g.append(float(gS))
    if not active:
        return None
    return TensorCache(F, 2 * F + 1, precompute_cg_table(F), active, g)


def make_tensor_interaction_cache(F: int, interactions: InteractionParams,
                                  basis: str = "coupling") -> Optional[TensorCache]:
    """``make_tensor_interaction_cache(F, interactions; basis)`` (src/tensor_interaction.jl:61-99)."""
    c_dict = {}
    for k in range(0, 2 * F + 1, 2):
        ck = get_cn(interactions, k)
        if abs(ck) > 1e-30:
            c_dict[k] = ck
    if not c_dict:
        return None
    if not any(k > 2 for k in c_dict):
        return None
    if basis == "coupling":
        g_dict = cn_to_gS(F, c_dict)
    elif basis == "channel":
        g_dict = c_dict
    else:
        raise ValueError(f"basis must be :coupling or :channel, got :{basis}")
    return make_tensor_cache_from_channels(F, g_dict)


def precompute_hf_entries(cache: TensorCache):
    """``_precompute_hf_entries`` (src/tensor_interaction.jl:165-193), 0-based component indices.

    Returns arrays (ch_idx, c_m, c_mp, c_mu, c_nu, cg_prod) in the reference's loop order.
    """
    F = cache.F
    out = []
    for si, S in enumerate(cache.active_channels):
        for m in range(-F, F + 1):
            for mu in range(-F, F + 1):
                M = m + mu
                if abs(M) > S:
                    continue
                cg1 = cache.cg_table.get((S, M, m, mu), 0.0)
                if abs(cg1) < 1e-15:
                    continue
                for mp in range(-F, F + 1):
                    nu = M - mp
                    if abs(nu) > F:
                        continue
                    cg2 = cache.cg_table.get((S, M, mp, nu), 0.0)
                    if abs(cg2) < 1e-15:
                        continue
                    out.append((si, F - m, F - mp, F - mu, F - nu, cg1 * cg2))
    if not out:
        return tuple(np.zeros(0, dtype=np.int64) for _ in range(5)) + (np.zeros(0),)
    a = list(zip(*out))
    return (np.array(a[0]), np.array(a[1]), np.array(a[2]), np.array(a[3]), np.array(a[4]),
            np.array(a[5], dtype=np.float64))


def precompute_pair_entries(cache: TensorCache):
    """``_precompute_pair_entries`` (src/tensor_interaction.jl:285-305), 0-based indices."""
    F = cache.F
    out = []
    offset = 0
    for si, S in enumerate(cache.active_channels):
        for M in range(-S, S + 1):
            a_idx = offset + M + S
            for m1 in range(-F, F + 1):
                m2 = M - m1
                if abs(m2) > F:
                    continue
                cg = cache.cg_table.get((S, M, m1, m2), 0.0)
                if abs(cg) < 1e-15:
                    continue
                out.append((a_idx, F - m1, F - m2, cg))
        offset += 2 * S + 1
    return out


# ----------------------------------------------------------------------------
# Potentials, Zeeman  (src/potentials.jl:1-32, src/zeeman.jl:1-21)
# ----------------------------------------------------------------------------

def harmonic_potential(grid: Grid, omega: Sequence[float]) -> np.ndarray:
    """``evaluate_potential(::HarmonicTrap)``: V = ½ Σ_d ω_d² x_d² (src/potentials.jl:5-15)."""
    s = np.zeros(grid.config.n_points, order="F")
    for d, (w, xd) in enumerate(zip(omega, grid.x)):
        shape = [1] * grid.config.ndim
        shape[d] = -1
        s = s + (w ** 2 * xd ** 2).reshape(shape)
    return np.asfortranarray(0.5 * s)


@dataclass
class ZeemanParams:
    p: float = 0.0
    q: float = 0.0


def zeeman_diagonal(z: ZeemanParams, F: int) -> np.ndarray:
    """``zeeman_diagonal``: E_c = -p m + q m², m = F - c (src/zeeman.jl:15-18)."""
    D = 2 * F + 1
    return np.array([-z.p * (F - c) + z.q * (F - c) ** 2 for c in range(D)], dtype=np.float64)


def zeeman_at(z, t: float) -> ZeemanParams:
    """``zeeman_at`` (src/zeeman.jl:20-21): a callable is a time-dependent Zeeman field."""
    return z(t) if callable(z) else z


# ----------------------------------------------------------------------------
# Simulation parameters, DDI parameters, workspace
# (src/types.jl:217-244, src/ddi.jl:7-102, src/ddi_padded.jl:6-49, src/initialization.jl:86-191)
# ----------------------------------------------------------------------------

@dataclass
class SimParams:
    """``SimParams`` (src/types.jl:217-237)."""

    dt: float
    n_steps: int
    imaginary_time: bool = False
    normalize_every: Optional[int] = None
    save_every: Optional[int] = None

    def __post_init__(self):
        if not self.dt > 0:
            raise ValueError("dt must be positive")
        if not self.n_steps > 0:
            raise ValueError("n_steps must be positive")
        if self.normalize_every is None:
            self.normalize_every = 1 if self.imaginary_time else 0
        if self.save_every is None:
            self.save_every = max(1, self.n_steps // 100)


@dataclass
class AtomSpecies:
    """The fields of ``AtomSpecies`` (src/types.jl:80-130) that the hot path reads."""

    name: str
    F: int
    mu_mag: float = 0.0


Rb87 = AtomSpecies("87Rb", 1)
Na23 = AtomSpecies("23Na", 1)
Eu151 = AtomSpecies("151Eu", 6, 7.0 * 9.2740100783e-24)


@dataclass
class DDIParams:
    C_dd: float
    Q: dict  # keys 'xx','xy','xz','yy','yz','zz' at the rfft half shape


def build_q_tensor(kx, ky, kz, rk_shape, secular=False) -> dict:
    """``_build_q_tensor!`` (src/ddi.jl:7-40): Q = k̂k̂ - δ/3, Q(0)=0; secular variant."""
    N = len(rk_shape)
    grids = np.meshgrid(*([kx] + ([ky] if N >= 2 else []) + ([kz] if N >= 3 else [])), indexing="ij")
    kvx = grids[0]
    kvy = grids[1] if N >= 2 else np.zeros(rk_shape)
    kvz = grids[2] if N >= 3 else np.zeros(rk_shape)
    k2 = kvx ** 2
    if N >= 2:
        k2 = k2 + kvy ** 2
    if N >= 3:
        k2 = k2 + kvz ** 2
    zero = k2 == 0.0
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.where(zero, 0.0, 1.0 / np.where(zero, 1.0, k2))
    Q = {}
    if secular:
        qzz = kvz * kvz * inv - 1.0 / 3.0
        Q["zz"] = qzz
        Q["xx"] = -qzz / 2.0
        Q["yy"] = -qzz / 2.0
        Q["xy"] = np.zeros(rk_shape)
        Q["xz"] = np.zeros(rk_shape)
        Q["yz"] = np.zeros(rk_shape)
    else:
        Q["xx"] = kvx * kvx * inv - 1.0 / 3.0
        Q["yy"] = kvy * kvy * inv - 1.0 / 3.0
        Q["zz"] = kvz * kvz * inv - 1.0 / 3.0
        Q["xy"] = kvx * kvy * inv
        Q["xz"] = kvx * kvz * inv
        Q["yz"] = kvy * kvz * inv
    for key in Q:
        Q[key] = np.asfortranarray(np.where(zero, 0.0, Q[key]))
    return Q


def make_ddi_params(grid: Grid, c_dd: float, secular: bool = False) -> DDIParams:
    """``make_ddi_params`` (src/ddi.jl:51-82): Q on the rfft half-grid of the simulation grid."""
    n = grid.config.n_points
    N = len(n)
    kx_r = rfftfreq(n[0], n[0] * grid.dk[0])
    ky = grid.k[1] if N >= 2 else np.zeros(0)
    kz = grid.k[2] if N >= 3 else np.zeros(0)
    return DDIParams(c_dd, build_q_tensor(kx_r, ky, kz, rfft_output_shape(n), secular))


@dataclass
class DDIPadded:
    padded_shape: tuple
    Q: dict


def make_ddi_padded(grid: Grid, c_dd: float, secular: bool = False) -> DDIPadded:
    """``make_ddi_padded`` (src/ddi_padded.jl:6-49): 2n per axis, same dx, padded-grid k."""
    n = grid.config.n_points
    N = len(n)
    ps = tuple(2 * v for v in n)
    dx = grid.dx
    kx_r = rfftfreq(ps[0], ps[0] * 2 * math.pi / (ps[0] * dx[0]))
    kfull = [fftfreq(ps[d], ps[d] * (2 * math.pi / (ps[d] * dx[d]))) for d in range(N)]
    ky = kfull[1] if N >= 2 else np.zeros(0)
    kz = kfull[2] if N >= 3 else np.zeros(0)
    return DDIPadded(ps, build_q_tensor(kx_r, ky, kz, rfft_output_shape(ps), secular))


@dataclass
class Workspace:
    """The fields of ``Workspace`` (src/types.jl:387-407) the hot path reads or writes."""

    psi: np.ndarray
    t: float
    step: int
    grid: Grid
    sm: SpinMatrices
    interactions: InteractionParams
    zeeman: object
    V: np.ndarray
    sim_params: SimParams
    kinetic_phase: np.ndarray
    ddi: Optional[DDIParams] = None
    ddi_padded: Optional[DDIPadded] = None
    tensor_cache: Optional[TensorCache] = None
    # last unpadded Φ, for the ITP overflow check (src/ground_state.jl:12-17)
    last_phi: Optional[tuple] = None
    loss: Optional["LossParams"] = None  # real-time losses (src/losses.jl)
    raman: Optional["RamanCoupling"] = None  # Raman coupling (src/raman.jl)

    @property
    def F(self) -> int:
        return self.sm.F

    @property
    def D(self) -> int:
        return self.sm.D

    @property
    def ndim(self) -> int:
        return self.grid.config.ndim


def prepare_kinetic_phase(grid: Grid, dt: float, imaginary_time: bool = False) -> np.ndarray:
    """``prepare_kinetic_phase`` (src/propagators.jl:1-7)."""
    if imaginary_time:
        return np.exp(-0.5 * grid.k_squared * dt).astype(np.complex128)
    return cis(-0.5 * grid.k_squared * dt)


def cis(x):
    return np.cos(x) + 1j * np.sin(x)


def make_workspace(*, grid: Grid, atom: AtomSpecies, interactions: InteractionParams,
                   zeeman=None, V: Optional[np.ndarray] = None, sim_params: SimParams,
                   psi_init: Optional[np.ndarray] = None, enable_ddi: bool = False,
                   c_dd: float = float("nan"), secular_ddi: bool = False,
                   ddi_padding: bool = False, loss: Optional["LossParams"] = None,
                   raman: Optional["RamanCoupling"] = None) -> Workspace:
    """``make_workspace`` (src/initialization.jl:86-191), including tensor-path activation (:164-185)."""
    F = atom.F
    sm = spin_matrices(F)
    zeeman = ZeemanParams() if zeeman is None else zeeman
    if psi_init is None:
        psi = init_psi(grid, F)
    else:
        psi = np.array(psi_init, dtype=np.complex128, order="F", copy=True)
    if V is None:
        V = np.zeros(grid.config.n_points, order="F")
    V = np.asfortranarray(np.asarray(V, dtype=np.float64))
    kin = prepare_kinetic_phase(grid, sim_params.dt, sim_params.imaginary_time)
    ddi = None
    ddi_pad = None
    if enable_ddi:
        if math.isnan(c_dd) and atom.mu_mag > 0.0:
            raise ValueError(f"enable_ddi=true for dipolar atom {atom.name} but c_dd not specified.")
        c_dd_val = 0.0 if math.isnan(c_dd) else c_dd
        ddi = make_ddi_params(grid, c_dd_val, secular_ddi)
        if ddi_padding:
            ddi_pad = make_ddi_padded(grid, c_dd_val, secular_ddi)
    has_higher = any((i + 1) % 2 == 0 and (i + 1) >= 4 and (i + 1) <= 2 * F and abs(v) > 1e-30
                     for i, v in enumerate(interactions.c_extra, start=1))
    if has_higher:
        g_base = c0c1_to_gS(F, interactions.c0, interactions.c1)
        g_delta = c_extra_to_delta_gS(F, interactions.c_extra)
        g_total = dict(g_base)
        for S, v in g_delta.items():
            g_total[S] = g_total.get(S, 0.0) + v
        tc = make_tensor_cache_from_channels(F, g_total)
        ws_int = InteractionParams(0.0, 0.0, interactions.c_lhy, ())
    else:
        tc = make_tensor_interaction_cache(F, interactions)
        if tc is not None and (abs(interactions.c0) > 1e-30 or abs(interactions.c1) > 1e-30):
            raise ValueError("tensor_cache active with non-zero c0/c1; set c0=c1=0 to avoid double-counting")
        ws_int = interactions
    return Workspace(psi=psi, t=0.0, step=0, grid=grid, sm=sm, interactions=ws_int, zeeman=zeeman,
                     V=V, sim_params=sim_params, kinetic_phase=kin, ddi=ddi, ddi_padded=ddi_pad,
                     tensor_cache=tc, loss=loss, raman=raman)


# ----------------------------------------------------------------------------
# Initial states  (src/initialization.jl:1-79)
# ----------------------------------------------------------------------------

def _gaussian(grid: Grid, sigma) -> np.ndarray:
    """``_gaussian`` (src/initialization.jl:69-79)."""
    s = np.zeros(grid.config.n_points, order="F")
    for d in range(grid.config.ndim):
        shape = [1] * grid.config.ndim
        shape[d] = -1
        s = s + (grid.x[d] ** 2 / (2 * sigma[d] ** 2)).reshape(shape)
    return np.asfortranarray(np.exp(-s))


def init_psi(grid: Grid, F: int, state: str = "polar", seed: int = 42,
             helix_k: Optional[Sequence[float]] = None) -> np.ndarray:
    """``init_psi`` (src/initialization.jl:1-67).

    ``:random`` draws from numpy's PCG64(seed) instead of Julia's MersenneTwister
    (whose stream cannot be reproduced outside Julia): psi = (N(0,1) + iN(0,1))/√2
    per entry, times the Gaussian envelope, then normalised.
    """
    n_pts = grid.config.n_points
    N = grid.config.ndim
    D = 2 * F + 1
    psi = np.zeros(n_pts + (D,), dtype=np.complex128, order="F")
    sigma = tuple(L / 8 for L in grid.config.box_size)
    gauss = _gaussian(grid, sigma)
    if state == "polar":
        psi[..., (D + 1) // 2 - 1] = gauss
    elif state == "ferromagnetic":
        psi[..., 0] = gauss
    elif state == "uniform":
        for c in range(D):
            psi[..., c] = gauss / math.sqrt(D)
    elif state == "antiferromagnetic":
        for c in range(D):
            m = F - c
            sign = 1.0 if (F - m) % 2 == 0 else -1.0
            psi[..., c] = sign * gauss / math.sqrt(D)
    elif state == "random":
        rng = np.random.Generator(np.random.PCG64(seed))
        re = rng.standard_normal(psi.shape)
        im = rng.standard_normal(psi.shape)
        psi[...] = (re + 1j * im) / math.sqrt(2.0)
        for c in range(D):
            psi[..., c] *= gauss
    elif state == "spin_helix":
        sm = spin_matrices(F)
        hk = tuple(helix_k) if helix_k is not None else (0.0,) * N
        theta = np.zeros(n_pts, order="F")
        for d in range(N):
            shape = [1] * N
            shape[d] = -1
            theta = theta + (hk[d] * grid.x[d]).reshape(shape)
        lam, vec = sm.Fy_eigvals, sm.Fy_eigvecs
        # first column of exp(-iθ Fy) = V diag(e^{-iθλ}) V^† e_1
        ph = np.exp(-1j * theta[..., None] * lam)            # (..., D)
        col = (ph * vec[0, :].conj()) @ vec.T                # (..., D)
        psi[...] = col * gauss[..., None]
    else:
        raise ValueError(f"Unknown initial state: {state}")
    dV = cell_volume(grid)
    norm = math.sqrt(float(np.sum(np.abs(psi) ** 2)) * dV)
    psi /= norm
    return psi


# ----------------------------------------------------------------------------
# Kinetic step  (src/propagators.jl:121-145)
# ----------------------------------------------------------------------------

def _axes(ws_or_ndim) -> tuple:
    n = ws_or_ndim if isinstance(ws_or_ndim, int) else ws_or_ndim.ndim
    return tuple(range(n))


def apply_kinetic_step_batched(ws: Workspace) -> None:
    """``apply_kinetic_step_batched!``: fft! over spatial dims, × phase, ifft! (src/propagators.jl:130-135)."""
    ax = _axes(ws)
    a = sfft.fftn(ws.psi, axes=ax, workers=_WORKERS)
    a *= ws.kinetic_phase[..., None]
    ws.psi[...] = sfft.ifftn(a, axes=ax, workers=_WORKERS)


def update_batched_kinetic_phase(ws: Workspace, dt: float) -> None:
    """``_update_batched_kinetic_phase!``: real-time phase cis(-½k²dt) (src/propagators.jl:137-145)."""
    ws.kinetic_phase = cis(-0.5 * ws.grid.k_squared * dt)


# ----------------------------------------------------------------------------
# Diagonal step  (src/propagators.jl:82-119)
# ----------------------------------------------------------------------------

def total_density(psi: np.ndarray) -> np.ndarray:
    """Σ_c |ψ_c|² in component order (src/propagators.jl:86-92)."""
    D = psi.shape[-1]
    s = np.zeros(psi.shape[:-1], order="F")
    for c in range(D):
        s = s + (psi[..., c].real ** 2 + psi[..., c].imag ** 2)
    return s


def diagonal_step(ws: Workspace, dt_frac: float, zeeman_diag: np.ndarray, imaginary_time: bool) -> None:
    """``_diagonal_step_svec!`` (src/propagators.jl:82-119)."""
    psi = ws.psi
    D = ws.D
    n = total_density(psi)
    c0 = ws.interactions.c0
    c_lhy = ws.interactions.c_lhy
    V_int = c0 * n + c_lhy * n * np.sqrt(n)
    if imaginary_time:
        shift = float(np.min(zeeman_diag))
        zee = np.exp(-((zeeman_diag - shift) * dt_frac))
        base = np.exp(-(ws.V + V_int) * dt_frac)
        for c in range(D):
            psi[..., c] *= base * zee[c]
    else:
        zee = cis(-(zeeman_diag * dt_frac))
        base = cis(-(ws.V + V_int) * dt_frac)
        for c in range(D):
            psi[..., c] *= base * zee[c]


# ----------------------------------------------------------------------------
# Spin rotations  (src/spin_mixing.jl:1-98, src/spinor_utils.jl:82-166)
# ----------------------------------------------------------------------------

def _fp_coeffs(F: int) -> np.ndarray:
    """f₊(m_c) = √(F(F+1) - m_c(m_c+1)) for c ≥ 1 (src/spin_mixing.jl:37-38)."""
    D = 2 * F + 1
    out = np.zeros(D)
    Ff1 = float(F * (F + 1))
    for c in range(1, D):
        m = float(F - c)
        out[c] = math.sqrt(Ff1 - m * (m + 1.0))
    return out


def spin_density(psi: np.ndarray, F: int):
    """``_compute_spin_density!`` (src/observables.jl:61-86): (Fx, Fy, Fz) real fields."""
    D = 2 * F + 1
    fp = _fp_coeffs(F)
    fz = np.zeros(psi.shape[:-1], order="F")
    for c in range(D):
        fz = fz + float(F - c) * (psi[..., c].real ** 2 + psi[..., c].imag ** 2)
    fx = np.zeros(psi.shape[:-1], order="F")
    fy = np.zeros(psi.shape[:-1], order="F")
    for c in range(1, D):
        prod = np.conj(psi[..., c - 1]) * psi[..., c]
        fx = fx + fp[c] * prod.real
        fy = fy + fp[c] * prod.imag
    return fx, fy, fz


def euler_spin_rotation(spinor: np.ndarray, phi_x, phi_y, phi_z, dt: float, sm: SpinMatrices,
                        imaginary_time: bool) -> np.ndarray:
    """``_apply_euler_spin_rotation`` (src/spinor_utils.jl:82-166), vectorised over points.

    ``spinor`` has shape (P, D); phi_* have shape (P,).  Returns the rotated spinors.
    """
    F = sm.F
    D = sm.D
    V = sm.Fy_eigvecs
    Vt = sm.Fy_eigvecs_adj
    out = spinor.copy()
    phi_mag = np.sqrt(phi_x ** 2 + phi_y ** 2 + phi_z ** 2)
    act = phi_mag * abs(dt) >= 1e-14
    if not np.any(act):
        return out
    s = spinor[act]
    px, py, pz, pm = phi_x[act], phi_y[act], phi_z[act], phi_mag[act]
    beta = np.arccos(np.clip(pz / pm, -1.0, 1.0))
    alpha = np.arctan2(py, px)
    theta = pm * dt
    z_neg_alpha = cis(-alpha)
    z_beta = cis(beta)
    rz_phase = cis(F * alpha)
    ry_phase = cis(-F * beta)
    P = s.shape[0]
    v = np.empty((P, D), dtype=np.complex128)
    w = np.empty((P, D), dtype=np.complex128)
    phase = rz_phase.copy()
    for c in range(D):
        v[:, c] = phase * s[:, c]
        phase = phase * z_neg_alpha
    phase = ry_phase.copy()
    for i in range(D):
        acc = np.zeros(P, dtype=np.complex128)
        for j in range(D):
            acc = acc + Vt[i, j] * v[:, j]
        w[:, i] = phase * acc
        phase = phase * z_beta
    for i in range(D):
        acc = np.zeros(P, dtype=np.complex128)
        for j in range(D):
            acc = acc + V[i, j] * w[:, j]
        v[:, i] = acc
    if imaginary_time:
        dz_r = np.exp(-F * theta)
        dz_step = np.exp(theta)
        for c in range(D):
            v[:, c] = v[:, c] * dz_r
            dz_r = dz_r * dz_step
    else:
        dz_phase = cis(-F * theta)
        z_theta = cis(theta)
        for c in range(D):
            v[:, c] = v[:, c] * dz_phase
            dz_phase = dz_phase * z_theta
    phase = np.conj(ry_phase)
    z_neg_beta = np.conj(z_beta)
    for i in range(D):
        acc = np.zeros(P, dtype=np.complex128)
        for j in range(D):
            acc = acc + Vt[i, j] * v[:, j]
        w[:, i] = phase * acc
        phase = phase * z_neg_beta
    phase = np.conj(rz_phase)
    z_alpha = np.conj(z_neg_alpha)
    for i in range(D):
        acc = np.zeros(P, dtype=np.complex128)
        for j in range(D):
            acc = acc + V[i, j] * w[:, j]
        v[:, i] = phase * acc
        phase = phase * z_alpha
    out[act] = v
    return out


def _rodrigues(spinor: np.ndarray, sm: SpinMatrices, c1: float, dt_frac: float,
               imaginary_time: bool) -> np.ndarray:
    """``_apply_rodrigues_rotation`` (src/spin_mixing.jl:71-98), vectorised over points: the
    same U = I - i sin(θ) n·F + (cos θ - 1)(n·F)^2 (sinh / cosh in imaginary time) built
    entry by entry, then U ψ."""
    Fs = (sm.Fx, sm.Fy, sm.Fz)
    sc = spinor.conj()
    f = []
    for Fm in Fs:
        acc = np.zeros(spinor.shape[0], dtype=np.complex128)
        for i in range(3):
            row = Fm[i, 0] * spinor[:, 0] + Fm[i, 1] * spinor[:, 1] + Fm[i, 2] * spinor[:, 2]
            acc = acc + sc[:, i] * row
        f.append(acc.real)
    fx, fy, fz = f
    f_mag = np.sqrt(fx ** 2 + fy ** 2 + fz ** 2)
    out = spinor.copy()
    act = f_mag >= 1e-30
    if not np.any(act):
        return out
    fx, fy, fz, fm, s = fx[act], fy[act], fz[act], f_mag[act], spinor[act]
    nF = [[(fx * sm.Fx[i, j] + fy * sm.Fy[i, j] + fz * sm.Fz[i, j]) / fm for j in range(3)] for i in range(3)]
    nF2 = [[nF[i][0] * nF[0][k] + nF[i][1] * nF[1][k] + nF[i][2] * nF[2][k] for k in range(3)] for i in range(3)]
    theta = c1 * fm * dt_frac
    if imaginary_time:
        a, b = -np.sinh(theta), np.cosh(theta) - 1
    else:
        a, b = -1j * np.sin(theta), np.cos(theta) - 1
    res = np.empty_like(s)
    for i in range(3):
        acc = np.zeros(s.shape[0], dtype=np.complex128)
        for j in range(3):
            U = (1.0 if i == j else 0.0) + a * nF[i][j] + b * nF2[i][j]
            acc = acc + U * s[:, j]
        res[:, i] = acc
    out[act] = res
    return out


def _flat_spinors(psi: np.ndarray) -> np.ndarray:
    D = psi.shape[-1]
    return psi.reshape(-1, D, order="F")


def _set_flat_spinors(psi: np.ndarray, flat: np.ndarray) -> None:
    psi[...] = flat.reshape(psi.shape, order="F")


def apply_spin_mixing_step(ws: Workspace, dt_frac: float, imaginary_time: bool) -> None:
    """``apply_spin_mixing_step!`` (src/spin_mixing.jl:1-66)."""
    c1 = ws.interactions.c1
    if abs(c1) < 1e-30:
        return
    sm = ws.sm
    flat = _flat_spinors(ws.psi)
    if sm.D == 3:
        new = _rodrigues(flat, sm, c1, dt_frac, imaginary_time)
    else:
        F = sm.F
        fp = _fp_coeffs(F)
        fz = np.zeros(flat.shape[0])
        for c in range(sm.D):
            fz = fz + float(F - c) * (flat[:, c].real ** 2 + flat[:, c].imag ** 2)
        fre = np.zeros(flat.shape[0])
        fim = np.zeros(flat.shape[0])
        for c in range(1, sm.D):
            prod = np.conj(flat[:, c - 1]) * flat[:, c]
            fre = fre + fp[c] * prod.real
            fim = fim + fp[c] * prod.imag
        new = euler_spin_rotation(flat, c1 * fre, c1 * fim, c1 * fz, dt_frac, sm, imaginary_time)
    _set_flat_spinors(ws.psi, new)


# ----------------------------------------------------------------------------
# Raman coupling  (src/raman.jl:1-31, src/spinor_utils.jl:27-38, src/energy.jl:123-135)
# ----------------------------------------------------------------------------

@dataclass
class RamanCoupling:
    """``RamanCoupling{N}(Omega_R, delta, k_eff)`` (src/types.jl:179-183)."""

    Omega_R: float
    delta: float
    k_eff: tuple


def _raman_hamiltonians(sm: SpinMatrices, raman: RamanCoupling, grid: Grid) -> np.ndarray:
    """H_R(r) = delta Fz + (Omega_R/2)(e^{i k.r} F+ + e^{-i k.r} F-) at every point, as an array
    (points in column-major order, D, D)."""
    shape = grid.config.n_points
    kr = np.zeros(shape, order="F")
    for d in range(len(shape)):
        sl = [None] * len(shape)
        sl[d] = slice(None)
        kr = kr + raman.k_eff[d] * np.asarray(grid.x[d])[tuple(sl)]
    ph = np.exp(1j * kr).ravel(order="F")
    return (raman.delta * sm.Fz[None, :, :]
            + (raman.Omega_R / 2) * (ph[:, None, None] * sm.Fp[None, :, :] + np.conj(ph)[:, None, None] * sm.Fm[None, :, :]))


def raman_step_psi(psi: np.ndarray, sm: SpinMatrices, raman: RamanCoupling, grid: Grid, dt: float,
                   imaginary_time: bool) -> None:
    """``apply_raman_step!`` (src/raman.jl:8-31) on psi[..., D] in place: per point
    psi <- V exp(-i Lambda dt) V^dagger psi (exp(-Lambda dt) in imaginary time) from the
    eigen-decomposition of H_R (``_exp_i_hermitian``, src/spinor_utils.jl:27-38)."""
    H = _raman_hamiltonians(sm, raman, grid)
    lam, V = np.linalg.eigh(H)
    e = np.exp(-lam * dt) if imaginary_time else np.exp(-1j * lam * dt)
    flat = _flat_spinors(psi)
    y = np.einsum("pji,pj->pi", np.conj(V), flat)          # V^dagger psi
    out = np.einsum("pij,pj->pi", V, e * y)
    _set_flat_spinors(psi, out)


def raman_energy(psi: np.ndarray, sm: SpinMatrices, raman: RamanCoupling, grid: Grid) -> float:
    """``_raman_energy`` (src/energy.jl:123-135): sum over points of Re(psi^dagger H_R psi) dV."""
    H = _raman_hamiltonians(sm, raman, grid)
    flat = _flat_spinors(psi)
    return float(np.sum(np.einsum("pi,pij,pj->p", np.conj(flat), H, flat).real)) * cell_volume(grid)


# ----------------------------------------------------------------------------
# Density-dependent losses  (src/losses.jl:1-97)
# ----------------------------------------------------------------------------

@dataclass
class LossParams:
    """``LossParams(gamma_dr, L3)`` (src/types.jl): dipolar-relaxation rate and 3-body rate."""

    gamma_dr: float
    L3: float = 0.0


def dipolar_relaxation_rates(F: int, gamma_dr: float) -> np.ndarray:
    """``_dipolar_relaxation_rates`` (src/losses.jl:68-97): gamma_m = gamma_dr raw_m / Z with
    raw_m = sum over q in (-1, -2), |m + q| <= F, of CG(F,m; 2,q | F,m+q)^2 and Z = sum raw / D."""
    D = 2 * F + 1
    raw = np.zeros(D)
    for c in range(D):
        m = F - c
        s = 0.0
        for q in (-1, -2):
            mp = m + q
            if abs(mp) > F:
                continue
            cg = clebsch_gordan(F, m, 2, q, F, mp)
            s += cg * cg
        raw[c] = s
    if raw.sum() < 1e-30:
        return np.zeros(D)
    Z = raw.sum() / D
    return np.array([gamma_dr * raw[c] / Z for c in range(D)])


def apply_loss_step_psi(psi: np.ndarray, loss: Optional["LossParams"], F: int, dt: float) -> None:
    """``apply_loss_step!`` (src/losses.jl:25-45) on psi[..., D] in place:
    psi_m *= exp(-(gamma_m + L3) n dt / 2), n the total density before the step; components
    with a rate below 1e-30 (and everything when both rates are below 1e-30) are untouched."""
    if loss is None or (loss.gamma_dr < 1e-30 and loss.L3 < 1e-30):
        return
    n = total_density(psi)
    rates = dipolar_relaxation_rates(F, loss.gamma_dr)
    for c in range(psi.shape[-1]):
        rate = rates[c] + loss.L3
        if rate < 1e-30:
            continue
        psi[..., c] *= np.exp(-rate * n * dt / 2)


# ----------------------------------------------------------------------------
# Singlet-pair (nematic) step  (src/nematic.jl:1-119, src/observables.jl:94-111)
# ----------------------------------------------------------------------------

def _pair_signs(D: int) -> np.ndarray:
    """(-1)^(F-m) for component c (m = F - c): +1 for even c, -1 for odd c."""
    return np.array([1.0 if c % 2 == 0 else -1.0 for c in range(D)])


def singlet_pair_amplitude(psi: np.ndarray, F: int) -> np.ndarray:
    """``singlet_pair_amplitude`` (src/observables.jl:94-111):
    A00 = sum_c (-1)^(F-m) psi_c psi_(D-1-c) / sqrt(D)."""
    D = 2 * F + 1
    sg = _pair_signs(D)
    s = np.zeros(psi.shape[:-1], dtype=np.complex128)
    for c in range(D):
        s = s + sg[c] * psi[..., c] * psi[..., D - 1 - c]
    return s * (1.0 / math.sqrt(float(D)))


def apply_nematic_step(ws: Workspace, dt: float, imaginary_time: bool) -> None:
    """``apply_nematic_step!`` (src/nematic.jl:34-51) on a workspace."""
    nematic_step_psi(ws.psi, get_cn(ws.interactions, 2), dt, imaginary_time)


def nematic_step_psi(psi: np.ndarray, c2: float, dt: float, imaginary_time: bool) -> None:
    """``_nematic_loop!`` (src/nematic.jl:53-119) on psi[..., D] in place: each (m, -m) pair
    turned by the exact solution of i d psi_m/dt = V psi*_(-m), V = c2 A00 (-1)^(F-m) / sqrt(D),
    with A00 from the state before the step; skipped where |V| < 1e-30 (and entirely for
    |c2| < 1e-30)."""
    if abs(c2) < 1e-30:
        return
    D = psi.shape[-1]
    flat = _flat_spinors(psi)
    inv_sqrt_D = 1.0 / math.sqrt(float(D))
    sg = _pair_signs(D)
    A00 = np.zeros(flat.shape[0], dtype=np.complex128)
    for c in range(D):
        A00 = A00 + sg[c] * flat[:, c] * flat[:, D - 1 - c]
    A00 = A00 * inv_sqrt_D
    V_base = c2 * A00 * inv_sqrt_D
    new = flat.copy()
    for c in range((D + 1) // 2):
        cp = D - 1 - c
        V = V_base * sg[c]
        absV = np.abs(V)
        act = absV >= 1e-30
        phase = np.where(act, V / np.where(act, absV, 1.0), 0.0)
        if imaginary_time:
            a = np.cosh(absV * dt)
            b = -phase * np.sinh(absV * dt)
        else:
            a = np.cos(absV * dt)
            b = -1j * phase * np.sin(absV * dt)
        vm, vn = flat[:, c], flat[:, cp]
        new[:, c] = np.where(act, a * vm + b * np.conj(vn), vm)
        if cp != c:
            new[:, cp] = np.where(act, a * vn + b * np.conj(vm), vn)
    _set_flat_spinors(psi, new)


# ----------------------------------------------------------------------------
# General-F tensor interaction  (src/tensor_interaction.jl:130-276)
# ----------------------------------------------------------------------------

def apply_tensor_interaction_step(ws: Workspace, dt: float, imaginary_time: bool) -> None:
    """``apply_tensor_interaction_step!`` / ``_tensor_step_point!`` (src/tensor_interaction.jl:130-240)."""
    cache = ws.tensor_cache
    D = cache.D
    ch, cm, cmp, cmu, cnu, cgp = precompute_hf_entries(cache)
    g = np.array(cache.g_values)
    flat = _flat_spinors(ws.psi)
    n_local = np.sum(flat.real ** 2 + flat.imag ** 2, axis=1)
    act = n_local >= 1e-20
    if not np.any(act):
        return
    s = flat[act]
    P = s.shape[0]
    # h[m, m'] = sum_e coef_e conj(psi_mu) psi_nu over the HFEntry terms e targeting (m, m'):
    # one product matrix (conj(psi_mu) psi_nu for every (mu, nu)) times a fixed (D^2 x D^2)
    # coefficient map, the same sum as the reference's entry loop in another order.
    W = getattr(cache, "_h_map", None)
    if W is None:
        W = np.zeros((D * D, D * D))
        coef = g[ch] * cgp
        np.add.at(W, (cmu * D + cnu, cm * D + cmp), coef)
        cache._h_map = W
    prod = (np.conj(s)[:, :, None] * s[:, None, :]).reshape(P, D * D)
    h = (prod @ W).reshape(P, D, D)
    vals, vecs = np.linalg.eigh(h, UPLO="U")
    proj = np.einsum("pjk,pj->pk", vecs.conj(), s)
    if imaginary_time:
        ex = np.exp(-vals * dt)
    else:
        ex = cis(-vals * dt)
    tmp = ex * proj
    new = np.einsum("pik,pk->pi", vecs, tmp)
    flat = flat.copy()
    flat[act] = new
    _set_flat_spinors(ws.psi, flat)


def tensor_interaction_energy(psi: np.ndarray, cache: TensorCache, dV: float) -> float:
    """``_tensor_interaction_energy``: ½ Σ_S g_S Σ_M |A_SM|² (src/tensor_interaction.jl:247-276)."""
    entries = precompute_pair_entries(cache)
    flat = _flat_spinors(psi)
    nA = sum(2 * S + 1 for S in cache.active_channels)
    A = np.zeros((flat.shape[0], nA), dtype=np.complex128)
    for a_idx, c1, c2, cg in entries:
        A[:, a_idx] += cg * flat[:, c1] * flat[:, c2]
    E = 0.0
    offset = 0
    for si, S in enumerate(cache.active_channels):
        for mi in range(2 * S + 1):
            E += 0.5 * cache.g_values[si] * float(np.sum(np.abs(A[:, offset + mi]) ** 2))
        offset += 2 * S + 1
    return E * dV


# ----------------------------------------------------------------------------
# Dipolar interaction  (src/ddi.jl:108-201, src/ddi_padded.jl:55-124)
# ----------------------------------------------------------------------------

def _rfftn(a: np.ndarray) -> np.ndarray:
    """FFTW ``rfft`` over all dims, halving the FIRST dim (src/grid.jl:46-53)."""
    N = a.ndim
    axes = tuple(range(1, N)) + (0,)
    return sfft.rfftn(a, axes=axes, workers=_WORKERS)


def _irfftn(a: np.ndarray, shape) -> np.ndarray:
    N = a.ndim
    axes = tuple(range(1, N)) + (0,)
    s = tuple(shape[1:]) + (shape[0],)
    return sfft.irfftn(a, s=s, axes=axes, workers=_WORKERS)


def _convolve_q(fx, fy, fz, Q: dict, C: float):
    """Spectral contraction Φ_α = C Σ_β Q_αβ F̂_β (src/ddi.jl:120-129)."""
    shape = fx.shape
    fkx, fky, fkz = _rfftn(fx), _rfftn(fy), _rfftn(fz)
    px = C * (Q["xx"] * fkx + Q["xy"] * fky + Q["xz"] * fkz)
    py = C * (Q["xy"] * fkx + Q["yy"] * fky + Q["yz"] * fkz)
    pz = C * (Q["xz"] * fkx + Q["yz"] * fky + Q["zz"] * fkz)
    return _irfftn(px, shape), _irfftn(py, shape), _irfftn(pz, shape)


def ddi_potential(ws: Workspace, padded: bool):
    """``_compute_and_convolve_ddi!`` / ``_compute_and_convolve_ddi_padded!`` → (Φx, Φy, Φz) on the grid."""
    fx, fy, fz = spin_density(ws.psi, ws.F)
    C = ws.ddi.C_dd
    if not padded:
        return _convolve_q(fx, fy, fz, ws.ddi.Q, C)
    ps = ws.ddi_padded.padded_shape
    n = ws.grid.config.n_points
    corner = tuple(slice(0, v) for v in n)
    pads = []
    for f in (fx, fy, fz):
        p = np.zeros(ps, order="F")
        p[corner] = f
        pads.append(p)
    ox, oy, oz = _convolve_q(*pads, ws.ddi_padded.Q, C)
    return ox[corner], oy[corner], oz[corner]


def apply_ddi_step(ws: Workspace, dt_frac: float, imaginary_time: bool) -> None:
    """``apply_ddi_step!`` (src/ddi.jl:168-201; padded src/ddi_padded.jl:90-124)."""
    padded = ws.ddi_padded is not None
    phix, phiy, phiz = ddi_potential(ws, padded)
    if not padded:
        ws.last_phi = (phix, phiy, phiz)
    flat = _flat_spinors(ws.psi)
    new = euler_spin_rotation(flat, phix.ravel(order="F"), phiy.ravel(order="F"), phiz.ravel(order="F"),
                              dt_frac, ws.sm, imaginary_time)
    _set_flat_spinors(ws.psi, new)


# ----------------------------------------------------------------------------
# Integrators  (src/split_step.jl:10-195)
# ----------------------------------------------------------------------------

YOSHIDA_W1 = 1.0 / (2.0 - 2.0 ** (1 / 3))
YOSHIDA_W0 = 1.0 - 2.0 * YOSHIDA_W1


def half_potential_step(ws: Workspace, dt_half: float, imaginary_time: bool) -> None:
    """``_half_potential_step!`` (src/split_step.jl:48-133): symmetric inner splitting
    diag, spin mixing, nematic | tensor, [Raman], [DDI], [Raman], nematic | tensor, spin
    mixing, diag."""
    zee = zeeman_at(ws.zeeman, ws.t)
    zd = zeeman_diagonal(zee, ws.F)
    diagonal_step(ws, dt_half / 2, zd, imaginary_time)
    if ws.tensor_cache is not None:
        apply_tensor_interaction_step(ws, dt_half / 2, imaginary_time)
    else:
        apply_spin_mixing_step(ws, dt_half / 2, imaginary_time)
        apply_nematic_step(ws, dt_half / 2, imaginary_time)
    if ws.raman is not None:
        raman_step_psi(ws.psi, ws.sm, ws.raman, ws.grid, dt_half / 2, imaginary_time)
    if ws.ddi is not None:
        apply_ddi_step(ws, dt_half, imaginary_time)
    if ws.raman is not None:
        raman_step_psi(ws.psi, ws.sm, ws.raman, ws.grid, dt_half / 2, imaginary_time)
    if ws.tensor_cache is not None:
        apply_tensor_interaction_step(ws, dt_half / 2, imaginary_time)
    else:
        apply_nematic_step(ws, dt_half / 2, imaginary_time)
        apply_spin_mixing_step(ws, dt_half / 2, imaginary_time)
    diagonal_step(ws, dt_half / 2, zd, imaginary_time)


def normalize_psi(psi: np.ndarray, grid: Grid) -> None:
    """``_normalize_psi!`` (src/split_step.jl:185-195): per-component Σ|ψ|²·dV, summed."""
    dV = cell_volume(grid)
    norm_sq = 0.0
    for c in range(psi.shape[-1]):
        norm_sq += float(np.sum(np.abs(psi[..., c]) ** 2)) * dV
    psi /= math.sqrt(norm_sq)


def split_step(ws: Workspace) -> None:
    """``split_step!`` (src/split_step.jl:10-35): V(dt/2) K(dt) V(dt/2) (+ ITP renormalisation)."""
    dt = ws.sim_params.dt
    it = ws.sim_params.imaginary_time
    half_potential_step(ws, dt / 2, it)
    apply_kinetic_step_batched(ws)
    half_potential_step(ws, dt / 2, it)
    if not it and ws.loss is not None:  # src/split_step.jl:21-23
        apply_loss_step_psi(ws.psi, ws.loss, ws.F, dt)
    ws.t += 0.0 if it else dt
    ws.step += 1
    ne = ws.sim_params.normalize_every
    if it and ne > 0 and ws.step % ne == 0:
        normalize_psi(ws.psi, ws.grid)


def strang_core(ws: Workspace, dt: float) -> None:
    """``_strang_core!`` (src/split_step.jl:146-152)."""
    half_potential_step(ws, dt / 2, False)
    update_batched_kinetic_phase(ws, dt)
    apply_kinetic_step_batched(ws)
    half_potential_step(ws, dt / 2, False)


def yoshida_core(ws: Workspace, dt: float) -> None:
    """``_yoshida_core!``: 4V + 3K with merged boundary V (src/split_step.jl:161-183)."""
    w1, w0 = YOSHIDA_W1, YOSHIDA_W0
    wm = (w1 + w0) / 2
    half_potential_step(ws, w1 * dt / 2, False)
    update_batched_kinetic_phase(ws, w1 * dt)
    apply_kinetic_step_batched(ws)
    half_potential_step(ws, wm * dt, False)
    update_batched_kinetic_phase(ws, w0 * dt)
    apply_kinetic_step_batched(ws)
    half_potential_step(ws, wm * dt, False)
    update_batched_kinetic_phase(ws, w1 * dt)
    apply_kinetic_step_batched(ws)
    half_potential_step(ws, w1 * dt / 2, False)


# ----------------------------------------------------------------------------
# Observables and energy  (src/observables.jl:1-31, src/energy.jl:6-135)
# ----------------------------------------------------------------------------

def total_norm(psi: np.ndarray, grid: Grid) -> float:
    """``total_norm`` (src/observables.jl:13-17)."""
    return float(np.sum(total_density(psi))) * cell_volume(grid)


def magnetization(psi: np.ndarray, grid: Grid, F: int) -> float:
    """``magnetization`` (src/observables.jl:22-31)."""
    dV = cell_volume(grid)
    Mz = 0.0
    for c in range(psi.shape[-1]):
        Mz += (F - c) * float(np.sum(np.abs(psi[..., c]) ** 2)) * dV
    return Mz


def pair_amplitude(psi: np.ndarray, F: int, S: int, M: int, cg_table: dict) -> np.ndarray:
    """``pair_amplitude`` (src/observables.jl:118-142):
    A_SM = sum_m1 CG(F,m1;F,M-m1|S,M) psi_m1 psi_(M-m1), pairs with |CG| < 1e-15 skipped."""
    A = np.zeros(psi.shape[:-1], dtype=np.complex128)
    for m1 in range(-F, F + 1):
        m2 = M - m1
        if abs(m2) > F:
            continue
        cg = cg_table.get((S, M, m1, m2), 0.0)
        if abs(cg) < 1e-15:
            continue
        A = A + cg * psi[..., F - m1] * psi[..., F - m2]
    return A


def pair_amplitude_spectrum(psi: np.ndarray, F: int, grid: Grid) -> dict:
    """``pair_amplitude_spectrum`` (src/observables.jl:227-246): (S, M) -> int |A_SM|^2 dV and
    S -> sum over M, for every even S <= 2F."""
    cg_table = precompute_cg_table(F)
    dV = cell_volume(grid)
    amplitudes, weights = {}, {}
    for S in range(0, 2 * F + 1, 2):
        w = 0.0
        for M in range(-S, S + 1):
            val = float(np.sum(np.abs(pair_amplitude(psi, F, S, M, cg_table)) ** 2)) * dV
            amplitudes[(S, M)] = val
            w += val
        weights[S] = w
    return dict(amplitudes=amplitudes, channel_weights=weights)


def classify_phase(psi: np.ndarray, F: int, grid: Grid) -> dict:
    """``classify_phase`` (src/diagnostics.jl:166-206): spin order |<F>|^2 / (F^2 n^2), nematic
    order (S = 0 pair weight over n^2 / D), normalised channel weights, the phase label and
    Mz / N.  Thresholds 0.9 / 0.9 / 0.5 and the label order are the reference's."""
    D = 2 * F + 1
    dV = cell_volume(grid)
    n = total_density(psi)
    n_sum = float(np.sum(n)) * dV
    n_sq_sum = float(np.sum(n ** 2)) * dV
    if n_sum < 1e-30:
        return dict(spin_order=0.0, nematic_order=0.0, channel_weights={}, phase="vacuum",
                    magnetization_density=0.0)
    fx, fy, fz = spin_density(psi, F)
    f_sq = float(np.sum(fx ** 2 + fy ** 2 + fz ** 2)) * dV
    spin_order = f_sq / (float(F) ** 2 * n_sq_sum)
    spec = pair_amplitude_spectrum(psi, F, grid)
    total_w = sum(spec["channel_weights"].values())
    cw = {S: (w / total_w if total_w > 0 else 0.0) for S, w in spec["channel_weights"].items()}
    nematic_order = spec["channel_weights"].get(0, 0.0) / (n_sq_sum / D)
    Mz = magnetization(psi, grid, F) / n_sum
    if spin_order > 0.9:
        phase = "ferromagnetic"
    elif nematic_order > 0.9:
        phase = "polar" if F == 1 else "nematic"
    elif cw.get(2 * F, 0.0) > 0.5:
        phase = "cyclic"
    else:
        phase = "mixed"
    return dict(spin_order=spin_order, nematic_order=nematic_order, channel_weights=cw, phase=phase,
                magnetization_density=Mz)


def energy_terms(ws: Workspace) -> dict:
    """The terms of ``total_energy`` (src/energy.jl:6-135)."""
    psi = ws.psi
    grid = ws.grid
    D = ws.D
    dV = cell_volume(grid)
    N = int(np.prod(grid.config.n_points))
    ax = _axes(ws)
    E_kin = 0.0
    for c in range(D):
        b = sfft.fftn(psi[..., c], axes=ax, workers=_WORKERS)
        E_kin += float(np.sum(grid.k_squared * (b.real ** 2 + b.imag ** 2))) * dV / N
    E_kin *= 0.5
    E_trap = 0.0
    for c in range(D):
        E_trap += float(np.sum(ws.V * np.abs(psi[..., c]) ** 2)) * dV
    zd = zeeman_diagonal(zeeman_at(ws.zeeman, ws.t), ws.F)
    E_zee = 0.0
    for c in range(D):
        E_zee += zd[c] * float(np.sum(np.abs(psi[..., c]) ** 2)) * dV
    n = total_density(psi)
    E_c0 = E_c1 = 0.0
    if ws.tensor_cache is None:
        E_c0 = 0.5 * ws.interactions.c0 * float(np.sum(n ** 2)) * dV
        fx, fy, fz = spin_density(psi, ws.F)
        E_c1 = 0.5 * ws.interactions.c1 * float(np.sum(fx ** 2 + fy ** 2 + fz ** 2)) * dV
    E_ddi = 0.0
    if ws.ddi is not None:
        fx, fy, fz = spin_density(psi, ws.F)
        px, py, pz = _convolve_q(fx, fy, fz, ws.ddi.Q, ws.ddi.C_dd)
        E_ddi = 0.5 * float(np.sum(px * fx + py * fy + pz * fz)) * dV
    E_lhy = 0.0
    if ws.interactions.c_lhy != 0.0:
        E_lhy = (2.0 / 5.0) * ws.interactions.c_lhy * float(np.sum(n * n * np.sqrt(n))) * dV
    E_tensor = 0.0
    if ws.tensor_cache is not None:
        E_tensor = tensor_interaction_energy(psi, ws.tensor_cache, dV)
    else:
        c2 = get_cn(ws.interactions, 2)
        if c2 != 0.0:  # _nematic_energy (src/energy.jl:106-109)
            E_tensor = 0.5 * c2 * float(np.sum(np.abs(singlet_pair_amplitude(psi, ws.F)) ** 2)) * dV
    terms = dict(kinetic=E_kin, trap=E_trap, zeeman=E_zee, c0=E_c0, c1=E_c1, ddi=E_ddi,
                 lhy=E_lhy, tensor=E_tensor)
    if ws.raman is not None:  # the Raman term only where the workspace has a coupling
        terms["raman"] = raman_energy(psi, ws.sm, ws.raman, grid)
    return terms


def total_energy(ws: Workspace) -> float:
    """``total_energy`` (src/energy.jl:6-54): the terms summed in the reference's order."""
    e = energy_terms(ws)
    return (e["kinetic"] + e["trap"] + e["zeeman"] + e["c0"] + e["c1"] + e["ddi"] + e["lhy"]
            + e["tensor"] + e.get("raman", 0.0))


# ----------------------------------------------------------------------------
# Simulation drivers  (src/simulation.jl:1-94, src/simulation_utils.jl:1-26)
# ----------------------------------------------------------------------------

@dataclass
class SimulationResult:
    times: list = field(default_factory=list)
    energies: list = field(default_factory=list)
    norms: list = field(default_factory=list)
    magnetizations: list = field(default_factory=list)
    psi_snapshots: list = field(default_factory=list)


def _record_snapshot(res: SimulationResult, ws: Workspace, keep_psi: bool = True) -> None:
    """``_record_snapshot!`` (src/simulation_utils.jl:9-15)."""
    res.times.append(ws.t)
    res.energies.append(total_energy(ws))
    res.norms.append(total_norm(ws.psi, ws.grid))
    res.magnetizations.append(magnetization(ws.psi, ws.grid, ws.F))
    if keep_psi:
        res.psi_snapshots.append(ws.psi.copy(order="F"))


def run_simulation(ws: Workspace, callback: Optional[Callable] = None,
                   keep_psi: bool = True) -> SimulationResult:
    """``run_simulation!`` (src/simulation.jl:1-22): standard loop for ITP, leapfrog for real time."""
    sp = ws.sim_params
    res = SimulationResult()
    _record_snapshot(res, ws, keep_psi)
    if sp.imaginary_time:
        for step in range(1, sp.n_steps + 1):
            split_step(ws)
            if step % sp.save_every == 0:
                _record_snapshot(res, ws, keep_psi)
                if callback is not None:
                    callback(ws, step)
        return res
    _run_leapfrog(ws, sp, res, callback, keep_psi)
    return res


def _run_leapfrog(ws, sp, res, callback, keep_psi) -> None:
    """``_run_simulation_leapfrog!``: merged V(dt) except at save/last steps (src/simulation.jl:49-94)."""
    dt = sp.dt
    half_potential_step(ws, dt / 2, False)
    for step in range(1, sp.n_steps + 1):
        apply_kinetic_step_batched(ws)
        is_save = step % sp.save_every == 0
        is_last = step == sp.n_steps
        need_split = is_save or is_last
        if need_split:
            half_potential_step(ws, dt / 2, False)
        else:
            half_potential_step(ws, dt, False)
        apply_loss_step_psi(ws.psi, ws.loss, ws.F, dt)  # src/simulation.jl:75-77
        ws.t += dt
        ws.step += 1
        if is_save:
            _record_snapshot(res, ws, keep_psi)
            if callback is not None:
                callback(ws, step)
        if need_split and not is_last:
            half_potential_step(ws, dt / 2, False)


# ----------------------------------------------------------------------------
# Adaptive drivers  (src/adaptive.jl:1-296, src/yoshida.jl:11-98, src/types.jl:343-361)
# ----------------------------------------------------------------------------

@dataclass
class AdaptiveDtParams:
    dt_init: float = 0.001
    dt_min: float = 1e-5
    dt_max: float = 0.01
    tol: float = 1e-3
    error_mode: str = "step_change"

    def __post_init__(self):
        if not self.dt_init > 0:
            raise ValueError("dt_init must be positive")
        if not self.dt_min > 0:
            raise ValueError("dt_min must be positive")
        if not self.dt_max >= self.dt_min:
            raise ValueError("dt_max must be >= dt_min")
        if not self.tol > 0:
            raise ValueError("tol must be positive")
        if self.error_mode not in ("step_change", "richardson"):
            raise ValueError(f"error_mode must be :step_change or :richardson, got :{self.error_mode}")


def wavefunction_l2_change(psi_new: np.ndarray, psi_old: np.ndarray) -> float:
    """``_wavefunction_l2_change``: ‖ψ_new-ψ_old‖²/‖ψ_old‖² (src/adaptive.jl:42-50)."""
    d = psi_new - psi_old
    diff_sq = float(np.sum(d.real ** 2 + d.imag ** 2))
    old_sq = float(np.sum(psi_old.real ** 2 + psi_old.imag ** 2))
    return diff_sq / max(old_sq, 1e-300)


def _save_point(res, ws, keep_psi):
    res.times.append(ws.t)
    res.energies.append(total_energy(ws))
    res.norms.append(total_norm(ws.psi, ws.grid))
    res.magnetizations.append(magnetization(ws.psi, ws.grid, ws.F))
    if keep_psi:
        res.psi_snapshots.append(ws.psi.copy(order="F"))


def run_simulation_adaptive(ws: Workspace, adaptive: AdaptiveDtParams, t_end: float,
                            save_interval: float, callback=None, keep_psi: bool = True):
    """``run_simulation_adaptive!`` (src/adaptive.jl:57-67)."""
    if adaptive.error_mode == "richardson":
        return _adaptive_richardson(ws, adaptive, t_end, save_interval, callback, keep_psi)
    return _adaptive_step_change(ws, adaptive, t_end, save_interval, callback, keep_psi)


def _adaptive_step_change(ws, adaptive, t_end, save_interval, callback, keep_psi):
    """``_adaptive_step_change_loop!`` with FSAL deferral (src/adaptive.jl:69-195)."""
    dt = min(max(adaptive.dt_init, adaptive.dt_min), adaptive.dt_max)
    current_kinetic_dt = float("nan")
    res = SimulationResult()
    _record_snapshot(res, ws, keep_psi)
    psi_old = np.empty_like(ws.psi)
    next_save = ws.t + save_interval
    n_acc = n_rej = 0
    fsal_deferred = False
    fsal_dt = 0.0
    while ws.t < t_end - 1e-14:
        dt_step = min(dt, t_end - ws.t)
        rem = next_save - ws.t
        if rem > 1e-14 and rem < dt_step:
            dt_step = rem
        dt_step = max(dt_step, adaptive.dt_min)
        is_clamped = dt_step < dt * 0.99
        may_reject = (not is_clamped) and dt_step > adaptive.dt_min * 1.01
        if dt_step != current_kinetic_dt:
            update_batched_kinetic_phase(ws, dt_step)
            current_kinetic_dt = dt_step
        need_err = not is_clamped
        if need_err:
            psi_old[...] = ws.psi
        prev_fd, prev_fdt = fsal_deferred, fsal_dt
        if fsal_deferred and abs(fsal_dt - dt_step) < 1e-14:
            half_potential_step(ws, dt_step, False)
        elif fsal_deferred:
            half_potential_step(ws, fsal_dt / 2, False)
            half_potential_step(ws, dt_step / 2, False)
        else:
            half_potential_step(ws, dt_step / 2, False)
        fsal_deferred = False
        apply_kinetic_step_batched(ws)
        rel = 0.0
        if may_reject:
            rel = wavefunction_l2_change(ws.psi, psi_old)
            if rel > adaptive.tol:
                ws.psi[...] = psi_old
                fsal_deferred, fsal_dt = prev_fd, prev_fdt
                factor = max(0.5, 0.9 * math.sqrt(adaptive.tol / rel))
                dt = max(dt_step * factor, adaptive.dt_min)
                current_kinetic_dt = float("nan")
                n_rej += 1
                continue
        fsal_deferred = True
        fsal_dt = dt_step
        apply_loss_step_psi(ws.psi, ws.loss, ws.F, dt_step)  # src/adaptive.jl:151-153
        ws.t += dt_step
        ws.step += 1
        n_acc += 1
        if not is_clamped:
            if not may_reject:
                rel = wavefunction_l2_change(ws.psi, psi_old)
            factor = min(2.0, 0.9 * math.sqrt(adaptive.tol / rel)) if rel > 1e-300 else 2.0
            dt = min(max(dt * factor, adaptive.dt_min), adaptive.dt_max)
        if ws.t >= next_save - 1e-14:
            half_potential_step(ws, fsal_dt / 2, False)
            fsal_deferred = False
            _save_point(res, ws, keep_psi)
            if callback is not None:
                callback(ws, n_acc)
            next_save += save_interval
    if fsal_deferred:
        half_potential_step(ws, fsal_dt / 2, False)
    if not res.times or abs(res.times[-1] - ws.t) > 1e-12:
        _record_snapshot(res, ws, keep_psi)
    return dict(result=res, n_accepted=n_acc, n_rejected=n_rej, final_dt=dt)


def _full_strang_step(ws, dt_step):
    half_potential_step(ws, dt_step / 2, False)
    apply_kinetic_step_batched(ws)
    half_potential_step(ws, dt_step / 2, False)


def _adaptive_richardson(ws, adaptive, t_end, save_interval, callback, keep_psi):
    """``_adaptive_richardson_loop!`` (src/adaptive.jl:204-296)."""
    dt = min(max(adaptive.dt_init, adaptive.dt_min), adaptive.dt_max)
    res = SimulationResult()
    _record_snapshot(res, ws, keep_psi)
    next_save = ws.t + save_interval
    n_acc = n_rej = 0
    while ws.t < t_end - 1e-14:
        dt_step = min(dt, t_end - ws.t)
        rem = next_save - ws.t
        if rem > 1e-14 and rem < dt_step:
            dt_step = rem
        dt_step = max(dt_step, adaptive.dt_min)
        is_clamped = dt_step < dt * 0.99
        may_reject = (not is_clamped) and dt_step > adaptive.dt_min * 1.01
        psi_saved = ws.psi.copy(order="F")
        update_batched_kinetic_phase(ws, dt_step)
        _full_strang_step(ws, dt_step)
        psi_full = ws.psi.copy(order="F")
        ws.psi[...] = psi_saved
        dt_half = dt_step / 2
        update_batched_kinetic_phase(ws, dt_half)
        _full_strang_step(ws, dt_half)
        _full_strang_step(ws, dt_half)
        err = wavefunction_l2_change(psi_full, ws.psi)
        if may_reject and err > adaptive.tol:
            ws.psi[...] = psi_saved
            factor = max(0.5, 0.9 * (adaptive.tol / err) ** (1 / 3))
            dt = max(dt_step * factor, adaptive.dt_min)
            n_rej += 1
            continue
        apply_loss_step_psi(ws.psi, ws.loss, ws.F, dt_step)  # src/adaptive.jl:262-264
        ws.t += dt_step
        ws.step += 1
        n_acc += 1
        if not is_clamped:
            factor = min(2.0, 0.9 * (adaptive.tol / err) ** (1 / 3)) if err > 1e-300 else 2.0
            dt = min(max(dt * factor, adaptive.dt_min), adaptive.dt_max)
        if ws.t >= next_save - 1e-14:
            _save_point(res, ws, keep_psi)
            if callback is not None:
                callback(ws, n_acc)
            next_save += save_interval
    if not res.times or abs(res.times[-1] - ws.t) > 1e-12:
        _record_snapshot(res, ws, keep_psi)
    return dict(result=res, n_accepted=n_acc, n_rejected=n_rej, final_dt=dt)


def run_simulation_yoshida(ws: Workspace, adaptive: AdaptiveDtParams, t_end: float,
                           save_interval: float, callback=None, keep_psi: bool = True,
                           max_accepted: Optional[int] = None):
    """``run_simulation_yoshida!``: adaptive S4 with embedded S2 error (src/yoshida.jl:11-98).

    ``max_accepted`` (not in the reference) stops the loop after that many accepted
    steps; it is used only to bound long runs.
    """
    dt = min(max(adaptive.dt_init, adaptive.dt_min), adaptive.dt_max)
    res = SimulationResult()
    _record_snapshot(res, ws, keep_psi)
    next_save = ws.t + save_interval
    n_acc = n_rej = 0
    while ws.t < t_end - 1e-14:
        if max_accepted is not None and n_acc >= max_accepted:
            break
        dt_step = min(dt, t_end - ws.t)
        rem = next_save - ws.t
        if rem > 1e-14 and rem < dt_step:
            dt_step = rem
        dt_step = max(dt_step, adaptive.dt_min)
        is_clamped = dt_step < dt * 0.99
        psi_old = ws.psi.copy(order="F")
        strang_core(ws, dt_step)
        psi_strang = ws.psi.copy(order="F")
        ws.psi[...] = psi_old
        yoshida_core(ws, dt_step)
        err = wavefunction_l2_change(ws.psi, psi_strang)
        if (not is_clamped) and err > adaptive.tol and dt_step > adaptive.dt_min * 1.01:
            ws.psi[...] = psi_old
            factor = max(0.3, 0.9 * (adaptive.tol / err) ** 0.2)
            dt = max(dt_step * factor, adaptive.dt_min)
            n_rej += 1
            continue
        apply_loss_step_psi(ws.psi, ws.loss, ws.F, dt_step)  # src/yoshida.jl:64-66
        ws.t += dt_step
        ws.step += 1
        n_acc += 1
        if not is_clamped:
            factor = min(3.0, 0.9 * (adaptive.tol / err) ** 0.2) if err > 1e-300 else 3.0
            dt = min(max(dt * factor, adaptive.dt_min), adaptive.dt_max)
        if ws.t >= next_save - 1e-14:
            _save_point(res, ws, keep_psi)
            if callback is not None:
                callback(ws, n_acc)
            next_save += save_interval
    if not res.times or abs(res.times[-1] - ws.t) > 1e-12:
        _record_snapshot(res, ws, keep_psi)
    return dict(result=res, n_accepted=n_acc, n_rejected=n_rej, final_dt=dt)


# ----------------------------------------------------------------------------
# Ground-state drivers  (src/ground_state.jl:1-392)
# ----------------------------------------------------------------------------

ITP_EXPONENT_LIMIT = 50.0


def check_itp_overflow(ws: Workspace, step: int) -> None:
    """``_check_itp_overflow`` (src/ground_state.jl:4-29)."""
    if np.any(np.isnan(ws.psi)):
        raise ValueError(f"NaN detected in ITP at step {step}. Likely DDI potential overflow. Reduce dt.")
    if ws.ddi is None or ws.last_phi is None:
        return
    phi_max = max(float(np.max(np.abs(p))) for p in ws.last_phi)
    exponent = phi_max * ws.sim_params.dt / 2
    if exponent > ITP_EXPONENT_LIMIT:
        raise ValueError(f"DDI potential overflow in ITP at step {step}: exponent={exponent:.1f} > 50")


def validate_itp_zeeman(zeeman, F: int, dt: float) -> None:
    """``_validate_itp_zeeman`` (src/ground_state.jl:31-42)."""
    if callable(zeeman):
        return
    max_zee = float(np.max(np.abs(zeeman_diagonal(zeeman, F))))
    if max_zee * dt / 4 > ITP_EXPONENT_LIMIT:
        raise ValueError(f"Zeeman p={zeeman.p} with F={F} and dt={dt} causes overflow in imaginary time")


def validate_itp_interactions(interactions: InteractionParams, F: int, dt: float,
                              psi: Optional[np.ndarray] = None, c_dd: float = 0.0) -> None:
    """``_validate_itp_interactions`` (src/ground_state.jl:46-78)."""
    n_peak = float(np.max(total_density(psi))) if psi is not None else 1.0
    max_c = max(abs(interactions.c0), abs(interactions.c1))
    if max_c > 1e-30 and max_c * n_peak * dt / 4 > ITP_EXPONENT_LIMIT:
        raise ValueError("Spin interaction may cause overflow in imaginary time")
    if c_dd > 0 and c_dd * F * n_peak * dt / 2 > ITP_EXPONENT_LIMIT:
        raise ValueError("DDI may cause overflow in imaginary time")


def normalize_psi_constrained(psi: np.ndarray, grid: Grid, target_Mz: float, F: int) -> None:
    """``_normalize_psi_constrained!``: Newton for λ with weights e^{λm} (src/ground_state.jl:279-320)."""
    dV = cell_volume(grid)
    D = psi.shape[-1]
    normalize_psi(psi, grid)
    lam = 0.0
    for _ in range(20):
        norms = np.empty(D)
        for c in range(D):
            m = F - c
            w = math.exp(lam * m)
            norms[c] = float(np.sum(np.abs(psi[..., c]) ** 2)) * dV * w ** 2
        total = float(np.sum(norms))
        if total < 1e-30:
            break
        Mz = sum((F - c) * norms[c] for c in range(D)) / total
        if abs(Mz - target_Mz) < 1e-12:
            break
        dMz = 0.0
        for c in range(D):
            m = F - c
            dMz += 2 * m * (m - Mz) * norms[c] / total
        if abs(dMz) < 1e-30:
            break
        lam -= (Mz - target_Mz) / dMz
        lam = min(max(lam, -10.0), 10.0)
    for c in range(D):
        psi[..., c] *= math.exp(lam * (F - c))
    normalize_psi(psi, grid)


def find_ground_state(*, grid: Grid, atom: AtomSpecies, interactions: InteractionParams, zeeman=None,
                      V=None, dt: float = 0.001, n_steps: int = 10000, tol: float = 1e-10,
                      initial_state: str = "polar", psi_init=None, enable_ddi: bool = False,
                      c_dd: float = float("nan"), secular_ddi: bool = False,
                      adaptive_dt: bool = False, dt_max: Optional[float] = None,
                      target_magnetization: Optional[float] = None) -> dict:
    """``find_ground_state`` (src/ground_state.jl:80-170); adaptive variant (:172-237)."""
    zeeman = ZeemanParams() if zeeman is None else zeeman
    psi0 = init_psi(grid, atom.F, initial_state) if psi_init is None else np.array(psi_init, order="F", copy=True)
    validate_itp_zeeman(zeeman, atom.F, dt)
    eff_cdd = c_dd if (enable_ddi and not math.isnan(c_dd)) else 0.0
    validate_itp_interactions(interactions, atom.F, dt, psi=psi0, c_dd=eff_cdd)
    if adaptive_dt:
        return _find_ground_state_adaptive(grid=grid, atom=atom, interactions=interactions, zeeman=zeeman,
                                           V=V, dt=dt, n_steps=n_steps, tol=tol, psi0=psi0,
                                           enable_ddi=enable_ddi, c_dd=c_dd, secular_ddi=secular_ddi,
                                           dt_max=10.0 * dt if dt_max is None else dt_max)
    use_c = target_magnetization is not None
    sp = SimParams(dt, n_steps, True, 0 if use_c else 1, max(1, n_steps // 10))
    ws = make_workspace(grid=grid, atom=atom, interactions=interactions, zeeman=zeeman, V=V, sim_params=sp,
                        psi_init=psi0, enable_ddi=enable_ddi, c_dd=c_dd, secular_ddi=secular_ddi)
    if use_c:
        normalize_psi_constrained(ws.psi, ws.grid, target_magnetization, atom.F)
    E_prev = total_energy(ws)
    converged = False
    psi_prev = ws.psi.copy(order="F")
    final_dE = final_dpsi = float("nan")
    steps_done = 0
    for step in range(1, n_steps + 1):
        split_step(ws)
        steps_done = step
        if step <= 10:
            check_itp_overflow(ws, step)
        if use_c:
            normalize_psi_constrained(ws.psi, ws.grid, target_magnetization, atom.F)
        if step % sp.save_every == 0:
            E = total_energy(ws)
            dE = abs(E - E_prev)
            pmax = float(np.max(np.abs(ws.psi)))
            dpsi = float(np.max(np.abs(ws.psi - psi_prev))) / pmax if pmax > 0 else 0.0
            final_dE, final_dpsi = dE, dpsi
            if dE < tol and dpsi < tol:
                converged = True
                break
            E_prev = E
            psi_prev[...] = ws.psi
    return dict(workspace=ws, converged=converged, energy=total_energy(ws), dE=final_dE,
                dpsi=final_dpsi, steps=steps_done)


def _find_ground_state_adaptive(*, grid, atom, interactions, zeeman, V, dt, n_steps, tol, psi0,
                                enable_ddi, c_dd, secular_ddi, dt_max):
    """``_find_ground_state_adaptive`` (src/ground_state.jl:172-237)."""
    current_dt = dt
    check_every = max(1, n_steps // 100)
    sp = SimParams(current_dt, check_every, True, 1, check_every)
    ws = make_workspace(grid=grid, atom=atom, interactions=interactions, zeeman=zeeman, V=V, sim_params=sp,
                        psi_init=psi0, enable_ddi=enable_ddi, c_dd=c_dd, secular_ddi=secular_ddi)
    E_prev = total_energy(ws)
    converged = False
    total_steps = 0
    final_dE = final_dpsi = float("nan")
    while total_steps < n_steps:
        psi_backup = ws.psi.copy(order="F")
        for i in range(1, check_every + 1):
            split_step(ws)
            if i == 1 and total_steps == 0:
                check_itp_overflow(ws, 1)
        total_steps += check_every
        E = total_energy(ws)
        if math.isnan(E) or E > E_prev:
            ws.psi[...] = psi_backup
            current_dt = max(current_dt * 0.5, 1e-8)
            _rebuild_with_dt(ws, current_dt)
        else:
            dE = abs(E - E_prev)
            pmax = float(np.max(np.abs(ws.psi)))
            dpsi = float(np.max(np.abs(ws.psi - psi_backup))) / pmax if pmax > 0 else 0.0
            final_dE, final_dpsi = dE, dpsi
            if dE < tol and dpsi < tol:
                converged = True
                break
            E_prev = E
            new_dt = min(current_dt * 1.1, dt_max)
            if new_dt != current_dt:
                current_dt = new_dt
                _rebuild_with_dt(ws, current_dt)
    return dict(workspace=ws, converged=converged, energy=total_energy(ws), dE=final_dE,
                dpsi=final_dpsi, steps=total_steps, final_dt=current_dt)


def _rebuild_with_dt(ws: Workspace, new_dt: float) -> None:
    """``_rebuild_workspace_with_dt`` (src/ground_state.jl:380-392): ITP phase for the new dt."""
    sp = ws.sim_params
    ws.sim_params = SimParams(new_dt, sp.n_steps, True, sp.normalize_every, sp.save_every)
    ws.kinetic_phase = prepare_kinetic_phase(ws.grid, new_dt, True)


def find_ground_state_multistart(*, initial_states=("polar", "ferromagnetic", "uniform", "antiferromagnetic"),
                                 n_random: int = 3, seed: int = 42, grid, atom, interactions, **kw) -> dict:
    """``find_ground_state_multistart`` (src/ground_state.jl:239-277); random seeds are seed+i."""
    results = []
    for state in initial_states:
        if state == "random":
            for i in range(1, n_random + 1):
                psi0 = init_psi(grid, atom.F, "random", seed=seed + i)
                r = find_ground_state(grid=grid, atom=atom, interactions=interactions, psi_init=psi0, **kw)
                results.append(dict(initial_state="random", idx=i, **r))
        else:
            r = find_ground_state(grid=grid, atom=atom, interactions=interactions, initial_state=state, **kw)
            results.append(dict(initial_state=state, idx=0, **r))
    best = min(results, key=lambda r: r["energy"])
    return dict(workspace=best["workspace"], converged=best["converged"], energy=best["energy"],
                initial_state=best["initial_state"], all_results=results)


def scan_continuation(*, param_values, make_interactions: Callable, grid, atom, initial_state="polar",
                      energy_jump_threshold=0.1, n_steps_continuation=500, n_steps_fresh=5000, **kw) -> list:
    """``scan_continuation`` (src/ground_state.jl:328-378), each point labelled by
    ``classify_phase`` (:363)."""
    results = []
    prev_psi = None
    prev_E = float("nan")
    for val in param_values:
        inter = make_interactions(val)
        if prev_psi is not None:
            r = find_ground_state(grid=grid, atom=atom, interactions=inter, psi_init=prev_psi.copy(order="F"),
                                  n_steps=n_steps_continuation, **kw)
        else:
            r = find_ground_state(grid=grid, atom=atom, interactions=inter, initial_state=initial_state,
                                  n_steps=n_steps_fresh, **kw)
        if not math.isnan(prev_E) and abs(r["energy"] - prev_E) / max(abs(prev_E), 1e-30) > energy_jump_threshold:
            r = find_ground_state_multistart(grid=grid, atom=atom, interactions=inter, n_steps=n_steps_fresh, **kw)
        psi = r["workspace"].psi
        phase = classify_phase(psi, atom.F, grid)["phase"]
        results.append(dict(param=val, energy=r["energy"], converged=r["converged"], phase=phase,
                            psi=psi.copy(order="F"), multistart=r.get("initial_state") is not None))
        prev_psi = psi.copy(order="F")
        prev_E = r["energy"]
    return results


# ----------------------------------------------------------------------------
# Host-buffer helpers (the C-ABI layout: interleaved re/im, x fastest)
# ----------------------------------------------------------------------------



def estimate_splitting_error(ws: Workspace) -> float:
    """``estimate_splitting_error`` (src/diagnostics.jl:214-251): one split step of dt against
    two of dt/2 (kinetic phase prepared for dt/2) from the same state, max|psi_1 - psi_2| /
    max|psi|; psi, t and step restored."""
    psi_save, t_save, step_save = ws.psi.copy(), ws.t, ws.step
    kin_save, sp = ws.kinetic_phase, ws.sim_params
    psi_norm = float(np.abs(psi_save).max())
    split_step(ws)
    psi_full = ws.psi.copy()
    ws.psi[...] = psi_save
    ws.t, ws.step = t_save, step_save
    dt_half = sp.dt / 2
    ws.kinetic_phase = prepare_kinetic_phase(ws.grid, dt_half, sp.imaginary_time)
    ws.sim_params = SimParams(dt_half, sp.n_steps, sp.imaginary_time, sp.normalize_every, sp.save_every)
    try:
        split_step(ws)
        split_step(ws)
        psi_half = ws.psi.copy()
    finally:
        ws.kinetic_phase, ws.sim_params = kin_save, sp
    ws.psi[...] = psi_save
    ws.t, ws.step = t_save, step_save
    return float(np.abs(psi_full - psi_half).max()) / psi_norm


def validate_conservation(ws: Workspace, *, n_steps: int = 100, tol_norm: float = 1e-12, tol_energy: float = 1e-3,
                          tol_magnetization: float = 1e-6) -> dict:
    """``validate_conservation`` (src/diagnostics.jl:259-293): drifts of N, E and Mz over
    n_steps split steps (the state restored), passed when all are below their tolerances."""
    psi_save, t_save, step_save = ws.psi.copy(), ws.t, ws.step
    N0, E0, M0 = total_norm(ws.psi, ws.grid), total_energy(ws), magnetization(ws.psi, ws.grid, ws.F)
    for _ in range(n_steps):
        split_step(ws)
    N1, E1, M1 = total_norm(ws.psi, ws.grid), total_energy(ws), magnetization(ws.psi, ws.grid, ws.F)
    ws.psi[...] = psi_save
    ws.t, ws.step = t_save, step_save
    nd = abs(N1 - N0) / max(N0, 1e-30)
    ed = abs(E1 - E0) / max(abs(E0), 1e-30)
    md = abs(M1 - M0) / max(abs(M0), 1e-10)
    return dict(passed=nd < tol_norm and ed < tol_energy and md < tol_magnetization, norm_drift=nd,
                energy_drift=ed, magnetization_drift=md)

def find_phase_boundary(*, param_range, make_interactions: Callable, grid, atom, tol: float = 0.01,
                        max_bisections: int = 20, **kw) -> dict:
    """``find_phase_boundary`` (src/phase_boundary.jl:9-60): bisection on the ``classify_phase``
    label of ``find_ground_state`` at each probe; the interval keeps the left endpoint's phase
    on its left (a midpoint of that phase moves a, any other moves b and its phase)."""
    def classify_at(val):
        r = find_ground_state(grid=grid, atom=atom, interactions=make_interactions(val), **kw)
        return classify_phase(r["workspace"].psi, atom.F, grid)["phase"]

    a, b = param_range
    phase_a, phase_b = classify_at(a), classify_at(b)
    n_eval = 2
    if phase_a == phase_b:
        return dict(boundary_value=(a + b) / 2, phase_left=phase_a, phase_right=phase_b, n_evaluations=n_eval)
    for _ in range(max_bisections):
        if abs(b - a) < tol:
            break
        mid = (a + b) / 2
        phase_mid = classify_at(mid)
        n_eval += 1
        if phase_mid == phase_a:
            a = mid
        else:
            b = mid
            phase_b = phase_mid
    return dict(boundary_value=(a + b) / 2, phase_left=phase_a, phase_right=phase_b, n_evaluations=n_eval)

def psi_to_interleaved(psi: np.ndarray) -> np.ndarray:
    flat = np.ascontiguousarray(psi.ravel(order="F"))
    return flat.view(np.float64)


def interleaved_to_psi(buf: np.ndarray, n_points: Sequence[int], D: int) -> np.ndarray:
    c = np.asarray(buf, dtype=np.float64).view(np.complex128)
    return np.asfortranarray(c.reshape(tuple(n_points) + (D,), order="F"))


# ----------------------------------------------------------------------------
# Experiment runner  (src/experiment.jl, src/experiment_runner.jl:36-168)
# ----------------------------------------------------------------------------

def _exp_ramp(v):
    """``_parse_ramp_or_constant`` (src/experiment.jl:201-209): (from, to) or a constant."""
    if isinstance(v, dict):
        return (float(v["from"]), float(v["to"])) if "to" in v else (float(v["from"]), float(v["from"]))
    return (float(v), float(v))


def _exp_potential(pc: dict, grid: Grid):
    t = str(pc.get("type", "none"))
    if t == "none":
        return None
    return harmonic_potential(grid, tuple(float(w) for w in pc["omega"]))


def run_experiment(d: dict, seed: int = 42) -> dict:
    """``run_experiment`` (src/experiment_runner.jl:54-155) on the parsed YAML mapping: an optional
    ground state, then each phase in a new workspace that starts from the previous psi at the
    running time offset, with ``_build_zeeman`` ramps (:36-52) and ``_add_noise!`` (:157-168,
    noise from PCG64(seed + phase index), complex normal of unit variance)."""
    d = d.get("experiment", d)
    sd = d["system"]
    atom = {"Rb87": Rb87, "Na23": Na23, "Eu151": Eu151}[str(sd["atom"])]
    npts = tuple(int(v) for v in sd["grid"]["n_points"])
    box = tuple(float(v) for v in sd["grid"]["box_size"])
    grid = make_grid(GridConfig(npts, box))
    inter = sd["interactions"]
    ks = [int(k[1:]) for k in inter if k[0] == "c" and k[1:].isdigit() and int(k[1:]) >= 2]
    c_extra = tuple(float(inter.get(f"c{n}", 0.0)) for n in range(2, max(ks) + 1)) if ks else ()
    ip = InteractionParams(float(inter["c0"]), float(inter["c1"]), float(inter.get("c_lhy", 0.0)), c_extra)
    loss = None
    if "losses" in sd:
        loss = LossParams(float(sd["losses"].get("gamma_dr", 0.0)), float(sd["losses"].get("L3", 0.0)))
    psi = None
    gs_E = gs_conv = None
    prev_pot = None
    if "ground_state" in d:
        g = d["ground_state"]
        z = g.get("zeeman", {})
        prev_pot = g.get("potential", {"type": "none"})
        r = find_ground_state(grid=grid, atom=atom, interactions=ip,
                              zeeman=ZeemanParams(float(z.get("p", 0.0)), float(z.get("q", 0.0))),
                              V=_exp_potential(prev_pot, grid), dt=float(g["dt"]), n_steps=int(g["n_steps"]),
                              tol=float(g["tol"]), initial_state=str(g.get("initial_state", "polar")))
        gs_E, gs_conv = r["energy"], r["converged"]
        psi = r["workspace"].psi.copy(order="F")
    results = []
    t_offset = 0.0
    for i, ph in enumerate(d.get("sequence", [])):
        pc = ph.get("potential", prev_pot)
        prev_pot = pc
        dt, duration = float(ph["dt"]), float(ph["duration"])
        save_every = int(ph.get("save_every", 1))
        z = ph.get("zeeman", {})
        (p0, p1), (q0, q1) = _exp_ramp(z.get("p", 0.0)), _exp_ramp(z.get("q", 0.0))
        if p0 == p1 and q0 == q1:
            zee = ZeemanParams(p0, q0)
        else:
            def zee(t, t0=t_offset, dur=duration, p0=p0, p1=p1, q0=q0, q1=q1):
                f = min(max((t - t0) / dur if dur > 0 else 0.0, 0.0), 1.0)
                return ZeemanParams(p0 + (p1 - p0) * f, q0 + (q1 - q0) * f)
        n_steps = int(round(duration / dt))
        ws = make_workspace(grid=grid, atom=atom, interactions=ip, zeeman=zee, V=_exp_potential(pc, grid),
                            sim_params=SimParams(dt, n_steps, False, None, save_every), psi_init=psi, loss=loss)
        ws.t = t_offset
        amp = ph.get("noise_amplitude")
        if amp is not None and float(amp) > 0:
            D = ws.psi.shape[-1]
            dom = int(np.argmax([float(np.sum(np.abs(ws.psi[..., c]) ** 2)) for c in range(D)]))
            rng = np.random.Generator(np.random.PCG64(seed + i))
            shp = ws.psi.shape[:-1]
            for c in range(D):
                if c != dom:
                    ws.psi[..., c] += float(amp) * (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)) / math.sqrt(2.0)
            ws.psi /= math.sqrt(float(np.sum(np.abs(ws.psi) ** 2)) * cell_volume(grid))
        if "adaptive_dt" in ph:
            a = ph["adaptive_dt"]
            ad = AdaptiveDtParams(dt_init=float(a.get("dt_init", dt)), dt_min=float(a.get("dt_min", 1e-5)),
                                  dt_max=float(a.get("dt_max", 10 * dt)), tol=float(a.get("tol", 1e-3)),
                                  error_mode=str(a.get("error_mode", "step_change")))
            res = run_simulation_adaptive(ws, ad, t_offset + duration, dt * save_every)["result"]
        else:
            res = run_simulation(ws)
        psi = ws.psi.copy(order="F")
        t_offset += duration
        results.append(res)
    return dict(ground_state_energy=gs_E, ground_state_converged=gs_conv, phase_results=results, psi=psi)
