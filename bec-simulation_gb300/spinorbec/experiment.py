"""The experiment runner (src/experiment.jl, src/experiment_runner.jl:54-155) over the device
drivers: a ground state followed by a sequence of real-time phases with constant or linearly
ramped Zeeman terms, run as one device-resident pipeline.

The configuration is the reference's YAML schema as a parsed mapping (any YAML loader gives
it; the keys are those of src/experiment.jl:92-230).  The ground state runs in its own
imaginary-time workspace; every phase then reuses one real-time workspace (dt, potential,
Zeeman function and clock set per phase), so psi stays on the device from phase to phase
instead of being copied into a new workspace as the reference does.  Noise
(``noise_amplitude``) is drawn from numpy's PCG64(seed + phase index) with the reference's
distribution (complex normal, unit variance) — Julia's global RNG stream cannot be reproduced.
"""

from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _lib
from .api import (find_ground_state, make_workspace, run_simulation, run_simulation_adaptive)
from .host import (AdaptiveDtParams, AtomSpecies, Eu151, GridConfig, HarmonicTrap, InteractionParams,
                   LossParams, Na23, NoPotential, Rb87, SimParams, ZeemanParams, cell_volume,
                   interaction_params_from_constraint, make_grid)


@dataclass
class ConstantValue:
    """``ConstantValue`` (src/experiment.jl:3-5)."""

    value: float


@dataclass
class LinearRamp:
    """``LinearRamp`` (src/experiment.jl:7-10)."""

    start: float
    stop: float


def interpolate_value(v, t_frac: float) -> float:
    """``interpolate_value`` (src/experiment.jl:14-15): the ramp clamps t_frac to [0, 1]."""
    if isinstance(v, ConstantValue):
        return v.value
    return v.start + (v.stop - v.start) * min(max(t_frac, 0.0), 1.0)


@dataclass
class PhaseConfig:
    name: str
    duration: float
    dt: float
    save_every: int
    zeeman_p: object
    zeeman_q: object
    potential: Optional[dict]
    noise_amplitude: Optional[float]
    adaptive_dt: Optional[AdaptiveDtParams]


@dataclass
class GroundStateConfig:
    dt: float
    n_steps: int
    tol: float
    initial_state: str
    zeeman: ZeemanParams
    potential: dict
    enable_ddi: bool


@dataclass
class SystemConfig:
    atom: AtomSpecies
    grid_n_points: tuple
    grid_box_size: tuple
    interactions: InteractionParams
    ddi_enabled: bool = False
    c_dd: Optional[float] = None
    secular: bool = False
    loss: Optional[LossParams] = None


@dataclass
class ExperimentConfig:
    name: str
    system: SystemConfig
    ground_state: Optional[GroundStateConfig]
    sequence: list = field(default_factory=list)


@dataclass
class ExperimentResult:
    config: ExperimentConfig
    ground_state_energy: Optional[float]
    ground_state_converged: Optional[bool]
    phase_results: list
    phase_names: list


ATOMS = {"Rb87": Rb87, "Na23": Na23, "Eu151": Eu151}


def resolve_atom(name: str) -> AtomSpecies:
    """``resolve_atom`` (src/experiment.jl:79-89)."""
    if name not in ATOMS:
        raise _lib.ArgumentError(f"Unknown atom: {name}. Available: {sorted(ATOMS)}")
    return ATOMS[name]


def _vec(v, typ):
    return tuple(typ(x) for x in v) if isinstance(v, (list, tuple)) else (typ(v),)


def _c_extra(inter: dict) -> tuple:
    """``_parse_c_extra`` (src/experiment.jl:221-238): c2, c3, ... filled with zeros."""
    ns = [int(m.group(1)) for k in inter for m in [re.match(r"^c(\d+)$", str(k))] if m and int(m.group(1)) >= 2]
    if not ns:
        return ()
    return tuple(float(inter.get(f"c{n}", 0.0)) for n in range(2, max(ns) + 1))


def _ramp(v):
    """``_parse_ramp_or_constant`` (src/experiment.jl:201-209)."""
    if isinstance(v, dict):
        if "to" in v:
            return LinearRamp(float(v["from"]), float(v["to"]))
        return ConstantValue(float(v["from"]))
    return ConstantValue(float(v))


def parse_experiment(d: dict) -> ExperimentConfig:
    """``_parse_experiment`` and friends (src/experiment.jl:104-199) on a parsed mapping; an
    ``experiment`` top-level key is unwrapped as in load_experiment."""
    d = d.get("experiment", d)
    sd = d["system"]
    atom = resolve_atom(str(sd["atom"]))
    g = sd["grid"]
    inter = sd["interactions"]
    if "c_total" in inter:
        ip = interaction_params_from_constraint(c_total=float(inter["c_total"]),
                                                c1_ratio=float(inter.get("c1_ratio", 0.0)), F=atom.F,
                                                c_extra=_c_extra(inter))
    else:
        ip = InteractionParams(float(inter["c0"]), float(inter["c1"]), float(inter.get("c_lhy", 0.0)), _c_extra(inter))
    dd = sd.get("ddi", {})
    loss = None
    if "losses" in sd:
        loss = LossParams(float(sd["losses"].get("gamma_dr", 0.0)), float(sd["losses"].get("L3", 0.0)))
    system = SystemConfig(atom, _vec(g["n_points"], int), _vec(g["box_size"], float), ip,
                          bool(dd.get("enabled", False)), float(dd["c_dd"]) if "c_dd" in dd else None,
                          bool(dd.get("secular", False)), loss)
    gs = None
    if "ground_state" in d:
        gd = d["ground_state"]
        z = gd.get("zeeman", {})
        gs = GroundStateConfig(float(gd["dt"]), int(gd["n_steps"]), float(gd["tol"]),
                               str(gd.get("initial_state", "polar")),
                               ZeemanParams(float(z.get("p", 0.0)), float(z.get("q", 0.0))),
                               gd.get("potential", {"type": "none"}), bool(gd.get("enable_ddi", False)))
    seq = []
    for pd in d.get("sequence", []):
        dt = float(pd["dt"])
        z = pd.get("zeeman", {})
        ad = None
        if "adaptive_dt" in pd:
            a = pd["adaptive_dt"]
            ad = AdaptiveDtParams(dt_init=float(a.get("dt_init", dt)), dt_min=float(a.get("dt_min", 1e-5)),
                                  dt_max=float(a.get("dt_max", 10 * dt)), tol=float(a.get("tol", 1e-3)),
                                  error_mode=str(a.get("error_mode", "step_change")))
        nz = pd.get("noise_amplitude")
        seq.append(PhaseConfig(str(pd.get("name", "unnamed")), float(pd["duration"]), dt, int(pd.get("save_every", 1)),
                               _ramp(z.get("p", 0.0)), _ramp(z.get("q", 0.0)), pd.get("potential"),
                               None if nz is None else float(nz), ad))
    return ExperimentConfig(str(d.get("name", "unnamed")), system, gs, seq)


def build_potential(pc: dict, ndim: int):
    """``_build_potential`` (src/experiment_runner.jl:1-26) for the none and harmonic types;
    the others (gravity, crossed dipole, composite) are evaluated by the Julia side and passed
    as a potential array."""
    t = str(pc.get("type", "none"))
    if t == "none":
        return NoPotential()
    if t == "harmonic":
        om = pc.get("omega")
        if om is None:
            raise _lib.ArgumentError("Harmonic potential requires omega")
        om = _vec(om, float)
        if len(om) != ndim:
            raise _lib.ArgumentError(f"omega length must match grid dimensions ({ndim})")
        return HarmonicTrap(*om)
    raise _lib.UnsupportedError(f"potential type {t} is not built by this runner; pass its values as an array")


def zeeman_function(phase: PhaseConfig, t_offset: float):
    """``_build_zeeman`` (src/experiment_runner.jl:36-52): a constant ZeemanParams, or
    t -> interpolated (p, q) over the phase's duration."""
    if isinstance(phase.zeeman_p, ConstantValue) and isinstance(phase.zeeman_q, ConstantValue):
        return ZeemanParams(phase.zeeman_p.value, phase.zeeman_q.value)

    def f(t: float) -> ZeemanParams:
        frac = (t - t_offset) / phase.duration if phase.duration > 0 else 0.0
        return ZeemanParams(interpolate_value(phase.zeeman_p, frac), interpolate_value(phase.zeeman_q, frac))

    return f


def add_noise(psi: np.ndarray, amplitude: float, grid, seed: int) -> np.ndarray:
    """``_add_noise!`` (src/experiment_runner.jl:157-168): complex normal noise of the given
    amplitude on every component but the most populated one, then renormalised; PCG64(seed)."""
    psi = np.array(psi, dtype=np.complex128, order="F", copy=True)
    D = psi.shape[-1]
    dom = int(np.argmax([float(np.sum(np.abs(psi[..., c]) ** 2)) for c in range(D)]))
    rng = np.random.Generator(np.random.PCG64(seed))
    shp = psi.shape[:-1]
    for c in range(D):
        if c == dom:
            continue
        psi[..., c] += amplitude * (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)) / math.sqrt(2.0)
    psi /= math.sqrt(float(np.sum(np.abs(psi) ** 2)) * cell_volume(grid))
    return psi


def run_experiment(config, *, seed: int = 42, precision: str = "fp64", verbose: bool = False) -> ExperimentResult:
    """``run_experiment`` (src/experiment_runner.jl:54-155); config: an ExperimentConfig or
    the parsed YAML mapping."""
    if isinstance(config, dict):
        config = parse_experiment(config)
    sc = config.system
    ndim = len(sc.grid_n_points)
    grid = make_grid(GridConfig(sc.grid_n_points, sc.grid_box_size))
    c_dd = float("nan") if sc.c_dd is None else sc.c_dd
    gs_E = gs_conv = None
    psi = None
    pot_cfg = None
    if config.ground_state is not None:
        gs = config.ground_state
        pot_cfg = gs.potential
        r = find_ground_state(grid=grid, atom=sc.atom, interactions=sc.interactions, zeeman=gs.zeeman,
                              potential=build_potential(gs.potential, ndim), dt=gs.dt, n_steps=gs.n_steps, tol=gs.tol,
                              initial_state=gs.initial_state, enable_ddi=gs.enable_ddi, c_dd=c_dd,
                              secular_ddi=sc.secular, precision=precision)
        gs_E, gs_conv = r["energy"], r["converged"]
        psi = r["workspace"].psi
        r["workspace"].close()
        if verbose:
            print(f"ground state: converged={gs_conv}, E={gs_E}")
    results, names = [], []
    t_offset = 0.0
    ws = None
    try:
        for i, ph in enumerate(config.sequence):
            pc = ph.potential if ph.potential is not None else pot_cfg
            if pc is None:
                raise _lib.ArgumentError(f"Phase '{ph.name}' has no potential and nothing to inherit")
            pot = build_potential(pc, ndim)
            zee = zeeman_function(ph, t_offset)
            n_steps = int(round(ph.duration / ph.dt))
            sp = SimParams(ph.dt, n_steps, False, None, ph.save_every)
            if ws is None:
                ws = make_workspace(grid=grid, atom=sc.atom, interactions=sc.interactions, zeeman=zee,
                                    potential=pot, sim_params=sp, psi_init=psi, enable_ddi=sc.ddi_enabled, c_dd=c_dd,
                                    secular_ddi=sc.secular, loss=sc.loss, precision=precision)
            else:
                ws.set_dt(ph.dt)
                ws.sim_params = sp
                from .host import evaluate_potential
                V = np.ascontiguousarray(evaluate_potential(pot, grid).ravel(order="F"))
                _lib.check(ws._lib.sbec_set_potential(ws.handle, _lib.dptr(V)))
                if callable(zee):
                    ws.set_zeeman_function(zee)
                else:
                    ws.set_zeeman_function(None)
                    ws.set_zeeman(zee.p, zee.q)
                    ws.zeeman = zee
            pot_cfg = pc
            ws.set_time(t_offset, 0)
            if ph.noise_amplitude is not None and ph.noise_amplitude > 0:
                ws.psi = add_noise(ws.psi, ph.noise_amplitude, grid, seed + i)
            if ph.adaptive_dt is not None:
                out = run_simulation_adaptive(ws, ph.adaptive_dt, t_end=t_offset + ph.duration,
                                              save_interval=ph.dt * ph.save_every)
                res = out["result"]
            else:
                res = run_simulation(ws)
            t_offset += ph.duration
            results.append(res)
            names.append(ph.name)
            if verbose:
                print(f"phase {i + 1} {ph.name}: t={ws.t}, E={res.energies[-1]}")
    finally:
        if ws is not None:
            ws.close()
    return ExperimentResult(config, gs_E, gs_conv, results, names)
