"""The experiment runner's configuration side against the reference's own tests
(test/test_experiment.jl:2-295, the YAML cases as parsed mappings — the runner takes the
mapping any YAML loader gives): ramp interpolation with clamping, the full schema with a
ground state and a three-phase sequence, DDI, the minimal form, noise amplitudes, the c_extra
fill rule, the Zeeman function of a ramped phase and the harmonic potential builder.  CPU only."""

import pytest

from spinorbec import _lib
from spinorbec import experiment as X
from spinorbec.host import HarmonicTrap, NoPotential, ZeemanParams


def test_interpolate_value():  # test/test_experiment.jl:2-14
    c = X.ConstantValue(3.0)
    assert [X.interpolate_value(c, t) for t in (0.0, 0.5, 1.0)] == [3.0, 3.0, 3.0]
    r = X.LinearRamp(1.0, 5.0)
    assert X.interpolate_value(r, 0.0) == 1.0
    assert X.interpolate_value(r, 0.5) == 3.0
    assert X.interpolate_value(r, 1.0) == 5.0
    assert X.interpolate_value(r, -0.1) == 1.0
    assert X.interpolate_value(r, 1.5) == 5.0


FULL = {"experiment": {
    "name": "test experiment",
    "system": {"atom": "Rb87", "grid": {"n_points": [64], "box_size": [20.0]},
               "interactions": {"c0": 10.0, "c1": -0.5}},
    "ground_state": {"dt": 0.005, "n_steps": 100, "tol": 1.0e-8, "initial_state": "polar",
                     "zeeman": {"p": 0.0, "q": 0.1}, "potential": {"type": "harmonic", "omega": [1.0]}},
    "sequence": [
        {"name": "ramp", "duration": 1.0, "dt": 0.01, "save_every": 10,
         "zeeman": {"p": {"from": 0.0, "to": 0.5}, "q": 0.0}, "potential": {"type": "harmonic", "omega": [1.0]}},
        {"name": "hold", "duration": 2.0, "dt": 0.01, "save_every": 20, "zeeman": {"p": 0.5, "q": 0.0}},
        {"name": "release", "duration": 0.5, "dt": 0.005, "save_every": 10, "zeeman": {"p": 0.0, "q": 0.0},
         "potential": {"type": "none"}},
    ]}}


def test_full_schema():  # test/test_experiment.jl:16-112
    cfg = X.parse_experiment(FULL)
    assert cfg.name == "test experiment"
    assert cfg.system.atom.name == X.Rb87.name
    assert cfg.system.grid_n_points == (64,) and cfg.system.grid_box_size == (20.0,)
    assert cfg.system.interactions.c0 == 10.0 and cfg.system.interactions.c1 == -0.5
    assert cfg.system.ddi_enabled is False
    gs = cfg.ground_state
    assert gs is not None and gs.dt == 0.005 and gs.n_steps == 100 and gs.tol == 1.0e-8
    assert gs.initial_state == "polar" and gs.zeeman == ZeemanParams(0.0, 0.1)
    assert gs.potential["type"] == "harmonic" and gs.potential["omega"] == [1.0]
    assert len(cfg.sequence) == 3
    ramp, hold, release = cfg.sequence
    assert (ramp.name, ramp.duration, ramp.dt, ramp.save_every) == ("ramp", 1.0, 0.01, 10)
    assert isinstance(ramp.zeeman_p, X.LinearRamp) and (ramp.zeeman_p.start, ramp.zeeman_p.stop) == (0.0, 0.5)
    assert isinstance(ramp.zeeman_q, X.ConstantValue) and ramp.zeeman_q.value == 0.0
    assert ramp.potential is not None
    assert hold.name == "hold" and hold.potential is None  # inherits the previous potential
    assert release.name == "release" and release.potential["type"] == "none"


def test_ddi_and_minimal():  # test/test_experiment.jl:114-158
    ddi = X.parse_experiment({"experiment": {
        "name": "ddi test",
        "system": {"atom": "Eu151", "grid": {"n_points": [32], "box_size": [10.0]},
                   "interactions": {"c0": 5.0, "c1": 0.0}, "ddi": {"enabled": True, "c_dd": 1.5e-5}},
        "sequence": []}})
    assert ddi.system.ddi_enabled is True and ddi.system.c_dd == 1.5e-5
    assert ddi.system.atom.name == X.Eu151.name
    mini = X.parse_experiment({"experiment": {
        "name": "minimal",
        "system": {"atom": "Na23", "grid": {"n_points": 32, "box_size": 10.0},
                   "interactions": {"c0": 1.0, "c1": 0.1}},
        "sequence": []}})
    assert mini.system.atom.name == X.Na23.name
    assert mini.system.grid_n_points == (32,)
    assert mini.ground_state is None and mini.sequence == []


def test_noise_amplitude():  # test/test_experiment.jl:261-294
    cfg = X.parse_experiment({"experiment": {
        "name": "noise test",
        "system": {"atom": "Rb87", "grid": {"n_points": [32], "box_size": [10.0]},
                   "interactions": {"c0": 1.0, "c1": 0.0}},
        "sequence": [
            {"name": "noisy", "duration": 1.0, "dt": 0.01, "noise_amplitude": 0.05,
             "zeeman": {"p": 0.0, "q": 0.0}, "potential": {"type": "harmonic", "omega": [1.0]}},
            {"name": "quiet", "duration": 1.0, "dt": 0.01, "zeeman": {"p": 0.0, "q": 0.0}}]}})
    assert cfg.sequence[0].noise_amplitude == 0.05
    assert cfg.sequence[1].noise_amplitude is None


def test_c_extra_fill_and_unknown_atom():  # src/experiment.jl:79-89, 221-238
    assert X._c_extra({"c0": 1.0, "c1": 0.0, "c4": 2.0}) == (0.0, 0.0, 2.0)
    assert X._c_extra({"c0": 1.0, "c1": 0.0}) == ()
    with pytest.raises(_lib.ArgumentError):
        X.resolve_atom("K39")


def test_zeeman_function_and_potentials():  # src/experiment_runner.jl:1-52
    cfg = X.parse_experiment(FULL)
    ramp, hold, _ = cfg.sequence
    f = X.zeeman_function(ramp, 2.0)
    assert callable(f)
    assert f(2.0) == ZeemanParams(0.0, 0.0)
    assert f(2.5) == ZeemanParams(0.25, 0.0)
    assert f(3.5) == ZeemanParams(0.5, 0.0)  # clamped after the phase
    assert X.zeeman_function(hold, 0.0) == ZeemanParams(0.5, 0.0)
    assert isinstance(X.build_potential({"type": "none"}, 1), NoPotential)
    assert isinstance(X.build_potential({"type": "harmonic", "omega": [1.0]}, 1), HarmonicTrap)
    with pytest.raises(_lib.ArgumentError):
        X.build_potential({"type": "harmonic", "omega": [1.0, 2.0]}, 1)
    with pytest.raises(_lib.UnsupportedError):
        X.build_potential({"type": "gravity"}, 1)
