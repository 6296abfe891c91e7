"""CPU checks of the C-ABI library: it builds, loads, exports every entry point
that include/sbec.h declares, and fails loudly (no CPU fallback) without a GPU."""

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_functions():
    text = (ROOT / "include" / "sbec.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(sbec_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = header_functions()
    for must in ("sbec_ws_create", "sbec_split_step", "sbec_run_yoshida", "sbec_ground_state", "sbec_total_energy"):
        assert must in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(libsbec):
    lib = ctypes.CDLL(str(ROOT / "bec-simulation_gb300" / "lib" / "libsbec.so"))
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(libsbec):
    from spinorbec import _lib

    assert set(header_functions()) <= set(_lib._PROTOS)


def test_no_device_fails_loudly(libsbec):
    import spinorbec as S

    if S.device_count() > 0:
        pytest.skip("a GPU is visible: the no-device path is exercised only on CPU hosts")
    g = S.make_grid(S.GridConfig((16,), (8.0,)))
    with pytest.raises(S.DeviceError):
        S.make_workspace(grid=g, atom=S.Rb87, interactions=S.InteractionParams(1.0, 0.0),
                         sim_params=S.SimParams(1e-3, 1))


def test_invalid_config_rejected_before_device(libsbec):
    import spinorbec as S

    g = S.make_grid(S.GridConfig((24,), (8.0,)))
    kw = dict(atom=S.Rb87, interactions=S.InteractionParams(1.0, 0.0), sim_params=S.SimParams(1e-3, 1))
    with pytest.raises(S.UnsupportedError):  # the dipolar convolution needs power-of-two axes
        S.make_workspace(grid=g, enable_ddi=True, c_dd=1.0, **kw)
    with pytest.raises(S.UnsupportedError):  # Bluestein axes beyond 512 points (y, z)
        S.make_workspace(grid=S.make_grid(S.GridConfig((8, 600), (8.0, 8.0))), **kw)
    if S.device_count() == 0:  # a non-power-of-two even n is on the GPU path
        with pytest.raises(S.DeviceError):
            S.make_workspace(grid=g, **kw)
    g2 = S.make_grid(S.GridConfig((16,), (8.0,)))
    with pytest.raises(S.UnsupportedError):  # spin F > 6
        S.make_workspace(grid=g2, atom=S.AtomSpecies("x", 7), interactions=S.InteractionParams(1.0, 0.0),
                         sim_params=S.SimParams(1e-3, 1))


def test_host_layout_roundtrip():
    import spinorbec as S

    rng = np.random.default_rng(0)
    psi = np.asfortranarray(rng.standard_normal((4, 6, 3)) + 1j * rng.standard_normal((4, 6, 3)))
    buf = S.to_interleaved(psi)
    assert buf[0] == psi[0, 0, 0].real and buf[1] == psi[0, 0, 0].imag
    assert buf[2] == psi[1, 0, 0].real  # x fastest (column-major, src/types.jl:239-244)
    assert np.array_equal(S.from_interleaved(buf, (4, 6), 3), psi)


def test_snapshot_store_blocks():
    """Save-point copies land in disjoint views of shared host blocks, same values and
    layout as a plain copy, a new block started when one is full."""
    from spinorbec.api import _SnapshotStore
    import spinorbec as S

    rng = np.random.default_rng(1)
    store = _SnapshotStore((4, 6), 3)
    store.per_block = 2
    outs, refs = [], []
    for _ in range(5):
        src = rng.standard_normal(2 * 4 * 6 * 3)
        outs.append(store.take(src.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        refs.append(S.from_interleaved(src.copy(), (4, 6), 3))
        src[:] = 0.0  # the source slot is reused by the next save point
    for o, r in zip(outs, refs):
        assert np.array_equal(o, r) and o.flags["F_CONTIGUOUS"]
    outs[0][...] = 0.0
    assert np.array_equal(outs[1], refs[1])
    assert outs[0].base is outs[1].base and outs[2].base is not outs[0].base


@pytest.mark.parametrize("case", ["zeeman", "interaction", "ddi"])
def test_itp_overflow_guards_before_device(case):
    """find_ground_state rejects parameters whose imaginary-time exponents would overflow
    (src/ground_state.jl:31-78) before any device work, with the reference's message."""
    import spinorbec as S

    g = S.make_grid(S.GridConfig((32,), (10.0,)))
    kw = dict(grid=g, atom=S.AtomSpecies("x", 1), dt=0.01, n_steps=10)
    if case == "zeeman":
        kw.update(interactions=S.InteractionParams(1.0, 0.0), zeeman=S.ZeemanParams(50000.0, 0.0))
        match = "Zeeman p=50000.0 with F=1 and dt=0.01 causes overflow"
    elif case == "interaction":
        kw.update(interactions=S.InteractionParams(1e7, 0.0))
        match = "Spin interaction c0=10000000.0"
    else:
        kw.update(interactions=S.InteractionParams(1.0, 0.0), enable_ddi=True, c_dd=1e7)
        match = "DDI c_dd=10000000.0 with F=1"
    with pytest.raises(S.ArgumentError, match=match):
        S.find_ground_state(**kw)


def test_raman_and_loss_options_reach_the_library():
    """RamanCoupling and LossParams are carried to sbec_ws_create (no UnsupportedError); a
    k_eff of the wrong length is an ArgumentError before any device work, and on a host
    without a GPU the workspace fails with DeviceError (no CPU fallback)."""
    import spinorbec as S

    g = S.make_grid(S.GridConfig((32,), (10.0,)))
    kw = dict(grid=g, atom=S.Rb87, interactions=S.InteractionParams(1.0, 0.0), sim_params=S.SimParams(1e-3, 1))
    with pytest.raises(S.ArgumentError, match="k_eff"):
        S.make_workspace(raman=S.RamanCoupling(1.0, 0.0, (0.0, 1.0)), **kw)
    if S.device_count() > 0:
        pytest.skip("a GPU is visible: the no-device path is exercised only on CPU hosts")
    with pytest.raises(S.DeviceError):
        S.make_workspace(raman=S.RamanCoupling(1.0, 0.1, (2.0,)), loss=S.LossParams(0.1, 0.01), **kw)


def test_tune_table_import_export(libsbec):
    """The autotuner's process table round-trips through its text form (host only), and a
    malformed line is refused with SBEC_ERR_INVALID."""
    import spinorbec as S

    S.tune_table_import("fp32 test-shape D=3 grid=8x8x1 solves=1\t5\n")
    text = S.tune_table_export()
    assert "fp32 test-shape D=3 grid=8x8x1 solves=1\t5\n" in text
    with pytest.raises(S.ArgumentError):
        S.tune_table_import("no tab here\n")
    with pytest.raises(S.ArgumentError):
        S.tune_table_import("shape\tx\n")


def test_batch_refuses_unsupported_configs_before_device(libsbec):
    """sbec_batch_create / _grids / _mixed refuse what the fused passes cannot run (a tensor
    step, D = 7) with SBEC_ERR_UNSUPPORTED before any device work, on every host; a supported
    configuration (spin 2 with a nematic c2) gets as far as the device check."""
    import ctypes as C

    import numpy as np

    import spinorbec as S
    from spinorbec import _lib, api

    g = S.make_grid(S.GridConfig((32, 32), (16.0, 16.0)))
    lib = S.load()

    def create(F, c_extra):
        cfg = api._config(g, F, S.ZeemanParams(), S.SimParams(0.005, 1, True, 1, 1), "fp64",
                          S.InteractionParams(0.0, 0.0, 0.0, c_extra))
        psi = np.zeros(2 * 32 * 32 * (2 * F + 1))
        c0 = np.array([10.0]); c1 = np.array([0.1])
        V = np.zeros(32 * 32)
        h = C.c_void_p()
        st = lib.sbec_batch_create(C.byref(cfg), 1, api.dptr(c0), api.dptr(c1), api.dptr(psi), api.dptr(V),
                                   C.byref(h))
        if st == _lib.SBEC_OK:
            lib.sbec_batch_destroy(h)
        return st

    assert create(2, (0.5, 0.0, 0.3)) == _lib.SBEC_ERR_UNSUPPORTED  # c4 switches on the tensor step
    assert create(3, ()) == _lib.SBEC_ERR_UNSUPPORTED               # D = 7 has no fused passes
    st = create(2, (0.5,))                                           # nematic c2: supported
    assert st == (_lib.SBEC_ERR_DEVICE if S.device_count() == 0 else _lib.SBEC_OK)
    with pytest.raises(S.UnsupportedError):
        S.GroundStateBatch(grids=[g], atoms=[S.AtomSpecies("f3", 3)], c0s=[10.0], c1s=[0.1],
                           psi_inits=[S.init_psi(g, 3, "polar")], dt=0.005, precision="fp64")
