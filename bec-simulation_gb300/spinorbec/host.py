"""Host-side setup that stays on the caller's side of the C ABI.

In the reference these run in Julia before any hot-path call: the grid
(src/grid.jl:1-35), potentials (src/potentials.jl:1-32), initial states
(src/initialization.jl:1-79) and the interaction parameter containers
(src/types.jl:145-178, src/interactions.jl:182-188).  They produce the host
buffers that ``sbec_ws_create`` copies to the device.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np


def _fftfreq(n: int, fs: float) -> np.ndarray:
    mult = fs / n
    idx = np.concatenate([np.arange(0, (n + 1) // 2), np.arange(-(n // 2), 0)]).astype(np.float64)
    return idx * mult


@dataclass(frozen=True)
class GridConfig:
    """``GridConfig(n_points, box_size)`` (src/types.jl:7-20)."""

    n_points: tuple
    box_size: tuple

    def __post_init__(self):
        n = tuple(int(v) for v in (self.n_points if isinstance(self.n_points, (tuple, list)) else (self.n_points,)))
        L = tuple(float(v) for v in (self.box_size if isinstance(self.box_size, (tuple, list)) else (self.box_size,)))
        if len(n) != len(L) or not 1 <= len(n) <= 3:
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


def make_grid(config: GridConfig) -> Grid:
    """``make_grid`` (src/grid.jl:1-23)."""
    xs, dxs, ks = [], [], []
    for n, L in zip(config.n_points, config.box_size):
        dx = L / n
        xs.append(np.linspace(-L / 2 + dx / 2, L / 2 - dx / 2, n))
        dxs.append(dx)
        ks.append(_fftfreq(n, n * (2 * math.pi / L)))
    return Grid(config, tuple(xs), tuple(dxs), tuple(ks))


def cell_volume(grid: Grid) -> float:
    v = 1.0
    for d in grid.dx:
        v *= d
    return v


@dataclass
class HarmonicTrap:
    """``HarmonicTrap(omega...)`` (src/types.jl:190-198)."""

    omega: tuple

    def __init__(self, *omega):
        if len(omega) == 1 and isinstance(omega[0], (tuple, list)):
            omega = tuple(omega[0])
        self.omega = tuple(float(w) for w in omega)


@dataclass
class NoPotential:
    pass


def evaluate_potential(pot, grid: Grid) -> np.ndarray:
    """``evaluate_potential`` for NoPotential / HarmonicTrap / an explicit array (src/potentials.jl:1-15)."""
    shape = grid.config.n_points
    if pot is None or isinstance(pot, NoPotential):
        return np.zeros(shape, order="F")
    if isinstance(pot, np.ndarray):
        return np.asfortranarray(pot, dtype=np.float64)
    if isinstance(pot, HarmonicTrap):
        s = np.zeros(shape, order="F")
        for d, (w, xd) in enumerate(zip(pot.omega, grid.x)):
            sh = [1] * grid.config.ndim
            sh[d] = -1
            s = s + (w ** 2 * xd ** 2).reshape(sh)
        return np.asfortranarray(0.5 * s)
    raise TypeError(f"unsupported potential {type(pot).__name__}: pass its values as an array")


@dataclass
class InteractionParams:
    """``InteractionParams(c0, c1, c_lhy, c_extra)``; ``c_extra[n-2]`` = c_n (src/types.jl:145-162)."""

    c0: float
    c1: float
    c_lhy: float = 0.0
    c_extra: tuple = ()


def interaction_params_from_constraint(*, c_total: float, c1_ratio: float = 0.0, F: int,
                                       c_extra: Sequence[float] = ()) -> InteractionParams:
    """c0 + F² c1 = c_total (src/interactions.jl:182-188)."""
    c0 = c_total / (1.0 + F ** 2 * c1_ratio)
    return InteractionParams(c0, c1_ratio * c0, 0.0, tuple(float(v) for v in c_extra))


@dataclass
class ZeemanParams:
    p: float = 0.0
    q: float = 0.0


@dataclass
class RamanCoupling:
    """``RamanCoupling{N}(Omega_R, delta, k_eff)`` (src/types.jl:179-183)."""

    Omega_R: float
    delta: float
    k_eff: tuple


@dataclass
class LossParams:
    """``LossParams(gamma_dr, L3)`` (src/types.jl:291-296)."""

    gamma_dr: float
    L3: float = 0.0


@dataclass
class AtomSpecies:
    name: str
    F: int
    mu_mag: float = 0.0


Rb87 = AtomSpecies("87Rb", 1)
Na23 = AtomSpecies("23Na", 1)
Eu151 = AtomSpecies("151Eu", 6, 7.0 * 9.2740100783e-24)


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
class AdaptiveDtParams:
    """``AdaptiveDtParams`` (src/types.jl:343-361)."""

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


def _gaussian(grid: Grid, sigma) -> np.ndarray:
    s = np.zeros(grid.config.n_points, order="F")
    for d in range(grid.config.ndim):
        sh = [1] * grid.config.ndim
        sh[d] = -1
        s = s + (grid.x[d] ** 2 / (2 * sigma[d] ** 2)).reshape(sh)
    return np.asfortranarray(np.exp(-s))


def _fy_eig(F: int):
    D = 2 * F + 1
    Fp = np.zeros((D, D), dtype=np.complex128)
    for c in range(1, D):
        m = F - c
        Fp[c - 1, c] = math.sqrt(F * (F + 1) - m * (m + 1))
    Fy = (Fp - Fp.conj().T) / 2j
    return np.linalg.eigh(Fy)


def init_psi(grid: Grid, F: int, state: str = "polar", seed: int = 42,
             helix_k: Optional[Sequence[float]] = None) -> np.ndarray:
    """``init_psi`` (src/initialization.jl:1-67); ``:random`` uses numpy PCG64(seed)."""
    n_pts = grid.config.n_points
    N = grid.config.ndim
    D = 2 * F + 1
    psi = np.zeros(n_pts + (D,), dtype=np.complex128, order="F")
    gauss = _gaussian(grid, tuple(L / 8 for L in grid.config.box_size))
    if state == "polar":
        psi[..., (D + 1) // 2 - 1] = gauss
    elif state == "ferromagnetic":
        psi[..., 0] = gauss
    elif state == "uniform":
        for c in range(D):
            psi[..., c] = gauss / math.sqrt(D)
    elif state == "antiferromagnetic":
        for c in range(D):
            psi[..., c] = (1.0 if c % 2 == 0 else -1.0) * gauss / math.sqrt(D)
    elif state == "random":
        rng = np.random.Generator(np.random.PCG64(seed))
        re = rng.standard_normal(psi.shape)
        im = rng.standard_normal(psi.shape)
        psi[...] = (re + 1j * im) / math.sqrt(2.0)
        for c in range(D):
            psi[..., c] *= gauss
    elif state == "spin_helix":
        lam, vec = _fy_eig(F)
        hk = tuple(helix_k) if helix_k is not None else (0.0,) * N
        theta = np.zeros(n_pts, order="F")
        for d in range(N):
            sh = [1] * N
            sh[d] = -1
            theta = theta + (hk[d] * grid.x[d]).reshape(sh)
        ph = np.exp(-1j * theta[..., None] * lam)
        psi[...] = ((ph * vec[0, :].conj()) @ vec.T) * gauss[..., None]
    else:
        raise ValueError(f"Unknown initial state: {state}")
    psi /= math.sqrt(float(np.sum(np.abs(psi) ** 2)) * cell_volume(grid))
    return psi


def to_interleaved(psi: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(psi, dtype=np.complex128).ravel(order="F")).view(np.float64)


def from_interleaved(buf: np.ndarray, n_points, D: int) -> np.ndarray:
    c = np.asarray(buf, dtype=np.float64).view(np.complex128)
    return np.asfortranarray(c.reshape(tuple(n_points) + (D,), order="F"))


@dataclass
class SimulationResult:
    """``SimulationResult`` (src/simulation_utils.jl:1-7)."""

    times: list = field(default_factory=list)
    energies: list = field(default_factory=list)
    norms: list = field(default_factory=list)
    magnetizations: list = field(default_factory=list)
    psi_snapshots: list = field(default_factory=list)
