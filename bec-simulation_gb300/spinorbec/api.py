"""SpinorBEC.jl's hot-path API over the C ABI (names follow the Julia API).

=====================================  =================================================
Julia (reference)                      here (every call runs on the GPU through libsbec)
=====================================  =================================================
make_workspace (initialization.jl:86)  make_workspace(...) -> Workspace
split_step! (split_step.jl:10)         split_step(ws, n=1)
_half_potential_step! (:48)            half_potential_step(ws, dt_half, imaginary_time)
apply_kinetic_step_batched! (prop:130) kinetic_step(ws, dt, imaginary_time)
_strang_core! / _yoshida_core!         strang_core(ws, dt) / yoshida_core(ws, dt)
run_simulation! (simulation.jl:1)      run_simulation(ws, callback=None)
run_simulation_adaptive! (adaptive:57) run_simulation_adaptive(ws, ...)
run_simulation_yoshida! (yoshida:11)   run_simulation_yoshida(ws, ...)
find_ground_state (ground_state:80)    find_ground_state(...)
find_ground_state_multistart (:239)    find_ground_state_multistart(...)
scan_continuation (:328)               scan_continuation(...)
total_energy / total_norm / magnet.    total_energy(ws) / total_norm(ws) / magnetization(ws)
=====================================  =================================================
"""

from __future__ import annotations

import ctypes as C
import math
from typing import Callable, Optional

import numpy as np

from . import _lib
from ._lib import check, dptr, load
from .host import (AdaptiveDtParams, AtomSpecies, Grid, InteractionParams, SimParams, SimulationResult,
                   ZeemanParams, cell_volume, evaluate_potential, from_interleaved, init_psi, to_interleaved)

PRECISIONS = {"fp64": _lib.SBEC_FP64, "fp32": _lib.SBEC_FP32_BULK, "fp32_bulk": _lib.SBEC_FP32_BULK}


class Workspace:
    """A device-resident workspace (``Workspace``, src/types.jl:387-407)."""

    def __init__(self, handle, grid: Grid, F: int, sim_params: SimParams, precision: str, zeeman):
        self._h = handle
        self.grid = grid
        self.F = F
        self.D = 2 * F + 1
        self.sim_params = sim_params
        self.precision = precision
        self.zeeman = zeeman
        self._lib = load()

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("workspace has been closed")
        return self._h

    def close(self) -> None:
        if self._h is not None:
            check(self._lib.sbec_ws_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state
    @property
    def psi(self) -> np.ndarray:
        n = int(np.prod(self.grid.config.n_points)) * self.D
        buf = np.empty(2 * n, dtype=np.float64)
        check(self._lib.sbec_get_psi(self.handle, dptr(buf)))
        return from_interleaved(buf, self.grid.config.n_points, self.D)

    @psi.setter
    def psi(self, value: np.ndarray) -> None:
        buf = to_interleaved(value)
        check(self._lib.sbec_set_psi(self.handle, dptr(buf)))

    @property
    def t(self) -> float:
        t = C.c_double()
        s = C.c_int64()
        check(self._lib.sbec_get_time(self.handle, C.byref(t), C.byref(s)))
        return t.value

    @property
    def step(self) -> int:
        t = C.c_double()
        s = C.c_int64()
        check(self._lib.sbec_get_time(self.handle, C.byref(t), C.byref(s)))
        return s.value

    def set_time(self, t: float, step: int) -> None:
        check(self._lib.sbec_set_time(self.handle, float(t), int(step)))

    def set_zeeman(self, p: float, q: float) -> None:
        check(self._lib.sbec_set_zeeman(self.handle, float(p), float(q)))

    def set_zeeman_function(self, fn) -> None:
        """TimeDependentZeeman: fn(t) -> ZeemanParams is evaluated by the library at the state
        time before every half potential (sbec_set_zeeman_fn); None restores the static term."""
        if fn is None:
            check(self._lib.sbec_set_zeeman_fn(self.handle, _lib.ZEEMAN_FN(), None))
            self._zfn = None
            self.zeeman = ZeemanParams() if not isinstance(self.zeeman, ZeemanParams) else self.zeeman
            return

        def _cb(user, t, pp, qp):
            try:
                z = fn(t)
                pp[0], qp[0] = float(z.p), float(z.q)
            except Exception:  # reported by the library as a non-finite Zeeman term
                pp[0] = qp[0] = float("nan")

        self._zfn = _lib.ZEEMAN_FN(_cb)
        check(self._lib.sbec_set_zeeman_fn(self.handle, self._zfn, None))
        self.zeeman = fn

    def set_dt(self, dt: float) -> None:
        check(self._lib.sbec_set_dt(self.handle, float(dt)))
        self.sim_params = SimParams(dt, self.sim_params.n_steps, self.sim_params.imaginary_time,
                                    self.sim_params.normalize_every, self.sim_params.save_every)

    # ---- tracing
    def profile(self, enable: bool = True) -> None:
        check(self._lib.sbec_profile_enable(self.handle, int(bool(enable))))

    def profile_read(self) -> dict:
        buf = (_lib.sbec_kernel_stat * 64)()
        n = C.c_int32()
        check(self._lib.sbec_profile_read(self.handle, buf, 64, C.byref(n)))
        return {buf[i].name.decode(): dict(launches=buf[i].launches, ms=buf[i].ms, bytes=buf[i].bytes)
                for i in range(min(n.value, 64))}

    @property
    def launch_count(self) -> int:
        n = C.c_int64()
        check(self._lib.sbec_launch_count(self.handle, C.byref(n)))
        return n.value

    @property
    def tuning_report(self) -> str:
        """Autotuner decisions (line-kernel variant per call shape, with every variant's time)."""
        return _report(self._lib.sbec_tuning_report, self.handle)

    def set_graph_mode(self, graphs: bool) -> None:
        """Replay repeated step blocks from CUDA graphs (default) or launch every kernel
        eagerly (sbec_set_graph_mode); same kernels, same results."""
        check(self._lib.sbec_set_graph_mode(self.handle, 1 if graphs else 0))

    @property
    def stream_ptr(self) -> int:
        p = C.c_void_p()
        check(self._lib.sbec_ws_stream(self.handle, C.byref(p)))
        return int(p.value or 0)

    def tensor_channels(self):
        act = C.c_int32()
        n = C.c_int32()
        S = (C.c_int32 * 32)()
        g = (C.c_double * 32)()
        check(self._lib.sbec_tensor_channels(self.handle, C.byref(act), C.byref(n), S, g))
        return bool(act.value), {int(S[i]): float(g[i]) for i in range(n.value)}


def make_workspace(*, grid: Grid, atom: AtomSpecies, interactions: InteractionParams, zeeman=None, potential=None,
                   sim_params: SimParams, psi_init: Optional[np.ndarray] = None, enable_ddi: bool = False,
                   c_dd: float = float("nan"), secular_ddi: bool = False, ddi_padding: bool = False,
                   gS: Optional[dict] = None, precision: str = "fp64", graphs: bool = True,
                   raman=None, loss=None) -> Workspace:
    """``make_workspace`` (src/initialization.jl:86-191) with a device-resident state.
    graphs=False: the workspace launches every kernel eagerly (see Workspace.set_graph_mode).
    ``raman`` (RamanCoupling: a per-point spin rotation inside the half potential,
    src/raman.jl) and ``loss`` (LossParams: a pointwise decay after each real-time step,
    src/losses.jl) run on the device."""
    lib = load()
    zeeman = ZeemanParams() if zeeman is None else zeeman
    if callable(zeeman):
        z0 = zeeman(0.0)
    else:
        z0 = zeeman
    F = atom.F
    if enable_ddi and math.isnan(c_dd) and atom.mu_mag > 0.0:
        raise _lib.ArgumentError(
            f"enable_ddi=true for dipolar atom {atom.name} but c_dd not specified. Pass c_dd in dimensionless units.")
    cfg = _lib.sbec_config()
    nd = grid.config.ndim
    cfg.ndim = nd
    for d in range(nd):
        cfg.n[d] = grid.config.n_points[d]
        cfg.L[d] = grid.config.box_size[d]
    cfg.F = F
    cfg.c0, cfg.c1, cfg.c_lhy = interactions.c0, interactions.c1, interactions.c_lhy
    ce = tuple(interactions.c_extra)
    if len(ce) > _lib.SBEC_MAX_C_EXTRA:
        raise _lib.ArgumentError("too many c_extra entries")
    cfg.n_c_extra = len(ce)
    for i, v in enumerate(ce):
        cfg.c_extra[i] = float(v)
    if gS is not None:
        cfg.gS_direct = 1
        for S in range(0, 2 * F + 1, 2):
            cfg.gS[S // 2] = float(gS.get(S, 0.0))
    cfg.zeeman_p, cfg.zeeman_q = z0.p, z0.q
    cfg.enable_ddi = int(bool(enable_ddi))
    cfg.c_dd = 0.0 if math.isnan(c_dd) else float(c_dd)
    cfg.secular_ddi = int(bool(secular_ddi))
    cfg.ddi_padding = int(bool(ddi_padding))
    cfg.dt = sim_params.dt
    cfg.imaginary_time = int(bool(sim_params.imaginary_time))
    cfg.normalize_every = int(sim_params.normalize_every)
    if precision not in PRECISIONS:
        raise _lib.ArgumentError(f"unknown precision {precision!r}")
    cfg.precision = PRECISIONS[precision]
    if raman is not None:
        k = tuple(float(v) for v in raman.k_eff)
        if len(k) != nd:
            raise _lib.ArgumentError("RamanCoupling.k_eff must have one entry per grid axis")
        cfg.raman = 1
        cfg.raman_omega, cfg.raman_delta = float(raman.Omega_R), float(raman.delta)
        for d in range(nd):
            cfg.raman_k[d] = k[d]
    if loss is not None:
        cfg.loss_gamma_dr, cfg.loss_L3 = float(loss.gamma_dr), float(loss.L3)
    psi = init_psi(grid, F) if psi_init is None else psi_init
    pbuf = to_interleaved(psi)
    if pbuf.size != 2 * int(np.prod(grid.config.n_points)) * (2 * F + 1):
        raise _lib.ArgumentError("psi_init has the wrong shape")
    V = np.ascontiguousarray(evaluate_potential(potential, grid).ravel(order="F"))
    h = C.c_void_p()
    check(lib.sbec_ws_create(C.byref(cfg), dptr(pbuf), dptr(V), C.byref(h)))
    ws = Workspace(h, grid, F, sim_params, precision, zeeman)
    ws.atom, ws.interactions = atom, interactions
    ws.c_dd = 0.0 if not enable_ddi or math.isnan(c_dd) else float(c_dd)
    if callable(zeeman):
        ws.set_zeeman_function(zeeman)
    if not graphs:
        ws.set_graph_mode(False)
    return ws


# ---- operators ---------------------------------------------------------------

def half_potential_step(ws: Workspace, dt_half: float, imaginary_time: bool = False) -> None:
    """``_half_potential_step!`` (src/split_step.jl:48-133); a time-dependent Zeeman term is
    evaluated by the library at the workspace time."""
    check(ws._lib.sbec_half_potential(ws.handle, float(dt_half), int(bool(imaginary_time))))


def kinetic_step(ws: Workspace, dt: float, imaginary_time: bool = False) -> None:
    check(ws._lib.sbec_kinetic(ws.handle, float(dt), int(bool(imaginary_time))))


def split_step(ws: Workspace, n: int = 1) -> None:
    """``split_step!`` repeated ``n`` times (src/split_step.jl:10-35)."""
    check(ws._lib.sbec_split_step(ws.handle, int(n)))


def strang_core(ws: Workspace, dt: float) -> None:
    check(ws._lib.sbec_strang_core(ws.handle, float(dt)))


def yoshida_core(ws: Workspace, dt: float) -> None:
    check(ws._lib.sbec_yoshida_core(ws.handle, float(dt)))


def normalize(ws: Workspace) -> None:
    check(ws._lib.sbec_normalize(ws.handle))


def normalize_constrained(ws: Workspace, target_Mz: float) -> None:
    check(ws._lib.sbec_normalize_constrained(ws.handle, float(target_Mz)))


# ---- reductions ----------------------------------------------------------------

def total_energy(ws: Workspace) -> float:
    E = C.c_double()
    check(ws._lib.sbec_total_energy(ws.handle, C.byref(E)))
    return E.value


def energy_terms(ws: Workspace) -> dict:
    t = _lib.sbec_energy_terms()
    check(ws._lib.sbec_energy_breakdown(ws.handle, C.byref(t)))
    return {k: getattr(t, k) for k, _ in t._fields_}


def total_norm(ws: Workspace) -> float:
    v = C.c_double()
    check(ws._lib.sbec_total_norm(ws.handle, C.byref(v)))
    return v.value


def magnetization(ws: Workspace) -> float:
    v = C.c_double()
    check(ws._lib.sbec_magnetization(ws.handle, C.byref(v)))
    return v.value


def spin_density_vector(ws: Workspace):
    n = int(np.prod(ws.grid.config.n_points))
    out = np.empty(3 * n)
    check(ws._lib.sbec_spin_density(ws.handle, dptr(out)))
    shp = ws.grid.config.n_points
    return tuple(out[i * n:(i + 1) * n].reshape(shp, order="F") for i in range(3))


def ddi_potential(ws: Workspace, padded: bool = False):
    n = int(np.prod(ws.grid.config.n_points))
    out = np.empty(3 * n)
    check(ws._lib.sbec_ddi_potential(ws.handle, int(bool(padded)), dptr(out)))
    shp = ws.grid.config.n_points
    return tuple(out[i * n:(i + 1) * n].reshape(shp, order="F") for i in range(3))


def _phase_dict(info) -> dict:
    nch = int(info.n_channels)
    return dict(spin_order=info.spin_order, nematic_order=info.nematic_order,
                channel_weights={2 * k: info.channel_weights[k] for k in range(nch)} if info.phase else {},
                phase=_lib.PHASE_LABELS[info.phase], magnetization_density=info.magnetization_density,
                raw_channel_weights={2 * k: info.raw_channel_weights[k] for k in range(nch)})


def classify_phase(ws: Workspace) -> dict:
    """``classify_phase`` (src/diagnostics.jl:166-206) of the device-resident psi: spin order,
    nematic order, normalised pair-channel weights, the phase label and Mz/N, reduced on the
    device in FP64 (no psi round trip)."""
    info = _lib.sbec_phase_info()
    check(ws._lib.sbec_classify_phase(ws.handle, C.byref(info)))
    return _phase_dict(info)


# ---- drivers -------------------------------------------------------------------

class _SnapshotStore:
    """Host storage for psi snapshots: each snapshot is a view into a 64 MiB block (or one
    snapshot, if larger).  A block that size is backed by huge pages where the kernel offers
    them, so filling it faults far fewer pages than one fresh array per save point, and the
    copy keeps pace with the device's next segment."""

    BLOCK_BYTES = 64 << 20

    def __init__(self, n_points, D: int):
        self.n_points = tuple(n_points)
        self.D = D
        self.n = int(np.prod(self.n_points)) * D          # complex values per snapshot
        self.per_block = max(1, self.BLOCK_BYTES // (16 * self.n))
        self.block = None
        self.used = 0

    def take(self, src_ptr) -> np.ndarray:
        if self.block is None or self.used == self.per_block:
            self.block = np.empty(2 * self.n * self.per_block, dtype=np.float64)
            self.used = 0
        dst = self.block[2 * self.n * self.used:2 * self.n * (self.used + 1)]
        self.used += 1
        dst[:] = np.ctypeslib.as_array(src_ptr, shape=(2 * self.n,))
        return from_interleaved(dst, self.n_points, self.D)


class _Recorder:
    def __init__(self, ws: Workspace, callback, keep_psi: bool, use_count_arg: bool):
        self.ws = ws
        self.res = SimulationResult()
        self.callback = callback
        self.keep_psi = keep_psi
        self.first = True
        self.step0 = 0
        self.count = 0
        self.err = None
        store = _SnapshotStore(ws.grid.config.n_points, ws.D) if keep_psi else None

        def _cb(user, snap_p):
            try:
                s = snap_p.contents
                self.res.times.append(s.t)
                self.res.energies.append(s.energy)
                self.res.norms.append(s.norm)
                self.res.magnetizations.append(s.magnetization)
                if self.keep_psi:
                    self.res.psi_snapshots.append(store.take(s.psi))
                if self.first:
                    self.first = False
                    self.step0 = s.step
                elif self.callback is not None:
                    self.count += 1
                    self.callback(ws, s.step - self.step0 if not use_count_arg else self.count)
                return 0
            except Exception as e:  # surface Python errors after the C call returns
                self.err = e
                return 1

        self.cfunc = _lib.CALLBACK(_cb)

    def raise_pending(self):
        if self.err is not None:
            raise self.err


def run_simulation(ws: Workspace, callback: Optional[Callable] = None, keep_psi: bool = True) -> SimulationResult:
    """``run_simulation!`` (src/simulation.jl:1-94): leapfrog real time or the standard ITP loop.

    Without a user callback the save points are recorded from pinned snapshots while the
    device runs the next segment (sbec_set_snapshot_mode); a user callback, which may read or
    change the workspace, gets synchronous save points as in the reference."""
    sp = ws.sim_params
    rec = _Recorder(ws, callback, keep_psi, use_count_arg=False)
    check(ws._lib.sbec_set_snapshot_mode(ws.handle, 1 if callback is None else 0))
    st = ws._lib.sbec_run_simulation(ws.handle, sp.n_steps, sp.save_every, rec.cfunc, None)
    rec.raise_pending()
    check(st)
    return rec.res


def save_state(filename: str, ws: Workspace) -> None:
    """``save_state`` (src/io.jl:1-28): psi, t, step and the parameters that define the run, in
    a NumPy .npz archive with the reference's field names (JLD2 is the Julia side's format)."""
    z = ws.zeeman if isinstance(ws.zeeman, ZeemanParams) else None
    ip = getattr(ws, "interactions", None)
    np.savez(filename, psi=ws.psi, t=ws.t, step=ws.step,
             grid_n_points=np.array(ws.grid.config.n_points), grid_box_size=np.array(ws.grid.config.box_size),
             atom_name=getattr(getattr(ws, "atom", None), "name", ""),
             c0=ip.c0 if ip else np.nan, c1=ip.c1 if ip else np.nan, c_lhy=ip.c_lhy if ip else np.nan,
             c_extra=np.array(ip.c_extra if ip else (), dtype=np.float64),
             zeeman_p=z.p if z else np.nan, zeeman_q=z.q if z else np.nan, c_dd=getattr(ws, "c_dd", 0.0),
             dt=ws.sim_params.dt, imaginary_time=bool(ws.sim_params.imaginary_time))


def load_state(filename: str) -> dict:
    """``load_state`` (src/io.jl): the fields written by save_state."""
    with np.load(filename) as d:
        out = {k: d[k] for k in d.files}
    for k in ("t", "c0", "c1", "c_lhy", "zeeman_p", "zeeman_q", "c_dd", "dt"):
        out[k] = float(out[k])
    out["step"] = int(out["step"])
    out["imaginary_time"] = bool(out["imaginary_time"])
    out["atom_name"] = str(out["atom_name"])
    out["psi"] = np.asfortranarray(out["psi"])
    return out


def run_simulation_checkpointed(ws: Workspace, checkpoint_dir: str = "checkpoints", checkpoint_every: int = 1000,
                                callback: Optional[Callable] = None, resume: bool = False) -> SimulationResult:
    """``run_simulation_checkpointed!`` (src/simulation.jl:96-148): with resume, psi, t and step
    come from the latest step_*.npz in checkpoint_dir; the remaining n_steps - step steps run
    through run_simulation, and every save point whose global step is a multiple of
    checkpoint_every writes step_<8-digit step>.npz before the user's callback runs."""
    import os

    os.makedirs(checkpoint_dir, exist_ok=True)
    if resume:
        existing = sorted(f for f in os.listdir(checkpoint_dir) if f.startswith("step_") and f.endswith(".npz"))
        if existing:
            data = load_state(os.path.join(checkpoint_dir, existing[-1]))
            ws.psi = data["psi"]
            ws.set_time(data["t"], data["step"])
    start_step = ws.step
    remaining = ws.sim_params.n_steps - start_step
    if remaining <= 0:
        return run_simulation(ws, callback=callback)

    def checkpoint_cb(ws_cb, step):
        global_step = start_step + step
        if global_step % checkpoint_every == 0:
            save_state(os.path.join(checkpoint_dir, f"step_{global_step:08d}.npz"), ws_cb)
        if callback is not None:
            callback(ws_cb, step)

    sp = ws.sim_params
    ws.sim_params = SimParams(sp.dt, remaining, sp.imaginary_time, sp.normalize_every, sp.save_every)
    try:
        return run_simulation(ws, callback=checkpoint_cb)
    finally:
        ws.sim_params = sp


def _adaptive_params(adaptive: AdaptiveDtParams) -> _lib.sbec_adaptive_params:
    p = _lib.sbec_adaptive_params()
    p.dt_init, p.dt_min, p.dt_max, p.tol = adaptive.dt_init, adaptive.dt_min, adaptive.dt_max, adaptive.tol
    p.error_mode = 0 if adaptive.error_mode == "step_change" else 1
    return p


def run_simulation_adaptive(ws: Workspace, adaptive: AdaptiveDtParams = None, *, t_end: float,
                            save_interval: float, callback=None, keep_psi: bool = True) -> dict:
    """``run_simulation_adaptive!`` (src/adaptive.jl:57-296)."""
    adaptive = AdaptiveDtParams() if adaptive is None else adaptive
    rec = _Recorder(ws, callback, keep_psi, use_count_arg=True)
    out = _lib.sbec_adaptive_result()
    st = ws._lib.sbec_run_adaptive(ws.handle, C.byref(_adaptive_params(adaptive)), float(t_end),
                                   float(save_interval), rec.cfunc, None, C.byref(out))
    rec.raise_pending()
    check(st)
    _final_snapshot(ws, rec)
    return dict(result=rec.res, n_accepted=out.n_accepted, n_rejected=out.n_rejected, final_dt=out.final_dt)


def run_simulation_yoshida(ws: Workspace, adaptive: AdaptiveDtParams = None, *, t_end: float,
                           save_interval: float, callback=None, keep_psi: bool = True,
                           max_accepted: Optional[int] = None) -> dict:
    """``run_simulation_yoshida!`` (src/yoshida.jl:11-98)."""
    adaptive = AdaptiveDtParams() if adaptive is None else adaptive
    rec = _Recorder(ws, callback, keep_psi, use_count_arg=True)
    out = _lib.sbec_adaptive_result()
    st = ws._lib.sbec_run_yoshida(ws.handle, C.byref(_adaptive_params(adaptive)), float(t_end), float(save_interval),
                                  int(max_accepted or 0), rec.cfunc, None, C.byref(out))
    rec.raise_pending()
    check(st)
    _final_snapshot(ws, rec)
    return dict(result=rec.res, n_accepted=out.n_accepted, n_rejected=out.n_rejected, final_dt=out.final_dt)


def _final_snapshot(ws: Workspace, rec: _Recorder) -> None:
    """Closing `_record_snapshot!` when the last save time differs from t (src/yoshida.jl:93-95)."""
    t = ws.t
    if not rec.res.times or abs(rec.res.times[-1] - t) > 1e-12:
        rec.res.times.append(t)
        rec.res.energies.append(total_energy(ws))
        rec.res.norms.append(total_norm(ws))
        rec.res.magnetizations.append(magnetization(ws))
        if rec.keep_psi:
            rec.res.psi_snapshots.append(ws.psi)


ITP_EXPONENT_LIMIT = 50.0


def _zeeman_energies(z: ZeemanParams, F: int) -> np.ndarray:
    return np.array([-z.p * (F - c) + z.q * (F - c) ** 2 for c in range(2 * F + 1)])


def _validate_itp(zeeman, interactions: InteractionParams, F: int, dt: float, psi, c_dd: float) -> None:
    """``_validate_itp_zeeman`` / ``_validate_itp_interactions`` (src/ground_state.jl:31-78)."""
    lim = ITP_EXPONENT_LIMIT
    if not callable(zeeman):
        e = float(np.max(np.abs(_zeeman_energies(zeeman, F)))) * dt / 4
        if e > lim:
            raise _lib.ArgumentError(
                f"Zeeman p={zeeman.p} with F={F} and dt={dt} causes overflow in imaginary time "
                f"(exponent={e:.1f} > {lim}). Reduce p or dt. For ferromagnetic ground state, p=10 suffices.")
    n_peak = float(np.max(np.sum(np.abs(psi) ** 2, axis=-1))) if psi is not None else 1.0
    max_c = max(abs(interactions.c0), abs(interactions.c1))
    if max_c > 1e-30 and max_c * n_peak * dt / 4 > lim:
        raise _lib.ArgumentError(
            f"Spin interaction c0={interactions.c0}, c1={interactions.c1} with n_peak≈{n_peak:.3g} and dt={dt} "
            f"may cause overflow in imaginary time (estimated exponent={max_c * n_peak * dt / 4:.1f} > {lim}). "
            "Reduce c0/c1 magnitude or dt.")
    if c_dd > 0 and c_dd * F * n_peak * dt / 2 > lim:
        raise _lib.ArgumentError(
            f"DDI c_dd={c_dd} with F={F}, n_peak≈{n_peak:.3g} and dt={dt} may cause overflow in imaginary "
            f"time (estimated exponent={c_dd * F * n_peak * dt / 2:.1f} > {lim}). Reduce c_dd or dt.")


def find_ground_state(*, grid: Grid, atom: AtomSpecies, interactions: InteractionParams, zeeman=None,
                      potential=None, dt: float = 0.001, n_steps: int = 10000, tol: float = 1e-10,
                      initial_state: str = "polar", psi_init=None, enable_ddi: bool = False,
                      c_dd: float = float("nan"), secular_ddi: bool = False, adaptive_dt: bool = False,
                      dt_max: Optional[float] = None, target_magnetization: Optional[float] = None,
                      precision: str = "fp64", graphs: bool = True) -> dict:
    """``find_ground_state`` (src/ground_state.jl:80-237).  graphs as in make_workspace."""
    zeeman = ZeemanParams() if zeeman is None else zeeman
    psi0 = init_psi(grid, atom.F, initial_state) if psi_init is None else np.array(psi_init, order="F", copy=True)
    eff_cdd = c_dd if (enable_ddi and not math.isnan(c_dd)) else 0.0
    _validate_itp(zeeman, interactions, atom.F, dt, psi0, eff_cdd)
    if adaptive_dt:
        return _find_ground_state_adaptive(grid, atom, interactions, zeeman, potential, dt, n_steps, tol, psi0,
                                           enable_ddi, c_dd, secular_ddi, 10.0 * dt if dt_max is None else dt_max,
                                           precision, graphs)
    use_c = target_magnetization is not None
    sp = SimParams(dt, n_steps, True, 0 if use_c else 1, max(1, n_steps // 10))
    ws = make_workspace(grid=grid, atom=atom, interactions=interactions, zeeman=zeeman, potential=potential,
                        sim_params=sp, psi_init=psi0, enable_ddi=enable_ddi, c_dd=c_dd, secular_ddi=secular_ddi,
                        precision=precision, graphs=graphs)
    r = _lib.sbec_gs_result()
    check(ws._lib.sbec_ground_state(ws.handle, n_steps, float(tol), sp.save_every,
                                    float(target_magnetization) if use_c else float("nan"), C.byref(r)))
    return dict(workspace=ws, converged=bool(r.converged), energy=r.energy, dE=r.dE, dpsi=r.dpsi, steps=r.steps)


def _find_ground_state_adaptive(grid, atom, interactions, zeeman, potential, dt, n_steps, tol, psi0, enable_ddi,
                                c_dd, secular_ddi, dt_max, precision, graphs=True):
    """``_find_ground_state_adaptive`` (src/ground_state.jl:172-237), run by the library's
    driver (sbec_ground_state_adaptive): the backup of psi stays on the device, and the
    NaN / DDI-overflow guard after the first step raises NumericError as the reference
    raises ArgumentError."""
    check_every = max(1, n_steps // 100)
    sp = SimParams(dt, check_every, True, 1, check_every)
    ws = make_workspace(grid=grid, atom=atom, interactions=interactions, zeeman=zeeman, potential=potential,
                        sim_params=sp, psi_init=psi0, enable_ddi=enable_ddi, c_dd=c_dd, secular_ddi=secular_ddi,
                        precision=precision, graphs=graphs)
    r = _lib.sbec_gs_result()
    final_dt = C.c_double()
    check(ws._lib.sbec_ground_state_adaptive(ws.handle, int(n_steps), float(tol), float(dt_max), C.byref(r),
                                             C.byref(final_dt)))
    ws.sim_params = SimParams(final_dt.value, sp.n_steps, True, sp.normalize_every, sp.save_every)
    return dict(workspace=ws, converged=bool(r.converged), energy=r.energy, dE=r.dE, dpsi=r.dpsi, steps=r.steps,
                final_dt=final_dt.value)


def _nematic_c2(interactions: InteractionParams):
    """The nematic c2 of contact couplings (c_extra[0]), or None when c_extra holds a higher
    coupling (c3 and up: the tensor path or terms the batch does not take)."""
    extra = [float(v) for v in interactions.c_extra]
    if any(abs(v) > 1e-30 for v in extra[1:]):
        return None
    return extra[0] if extra else 0.0


def _batch_eligible(atom: AtomSpecies, interactions: InteractionParams, kw: dict) -> bool:
    """Whether every start of a multistart search can run as one GroundStateBatch: the batch
    takes contact couplings (c0, c1, c_lhy and the nematic c2) with a static Zeeman term and
    the plain find_ground_state loop (no DDI, adaptive dt or magnetisation constraint)."""
    if atom.F > 2 or _nematic_c2(interactions) is None:
        return False
    if kw.get("enable_ddi") or kw.get("adaptive_dt") or kw.get("target_magnetization") is not None:
        return False
    if callable(kw.get("zeeman")) or kw.get("psi_init") is not None:
        return False
    return True


def find_ground_state_multistart(*, initial_states=("polar", "ferromagnetic", "uniform", "antiferromagnetic"),
                                 n_random: int = 3, seed: int = 42, grid, atom, interactions, batched=None,
                                 **kw) -> dict:
    """``find_ground_state_multistart`` (src/ground_state.jl:239-277); random seeds are seed+i.

    batched=None (default) runs all starts as one GroundStateBatch when they are eligible
    (contact couplings, static Zeeman, plain ITP loop); each solve follows find_ground_state's
    loop and convergence test, so the results are those of the one-at-a-time loop.  Only the
    lowest-energy start gets a workspace (rebuilt from its psi); every entry of all_results
    carries its psi."""
    starts = []
    for state in initial_states:
        if state == "random":
            for i in range(1, n_random + 1):
                starts.append(("random", i, init_psi(grid, atom.F, "random", seed=seed + i)))
        else:
            starts.append((state, 0, init_psi(grid, atom.F, state)))
    use_batch = _batch_eligible(atom, interactions, kw) if batched is None else bool(batched)
    if use_batch and len(starts) > 1:
        dt = kw.get("dt", 0.001)
        zeeman = ZeemanParams() if kw.get("zeeman") is None else kw["zeeman"]
        for _, _, p0 in starts:
            _validate_itp(zeeman, interactions, atom.F, dt, p0, 0.0)
        b = GroundStateBatch(grid=grid, atom=atom, c0s=[interactions.c0] * len(starts),
                             c1s=[interactions.c1] * len(starts), psi_inits=[p for _, _, p in starts],
                             zeeman=zeeman, potential=kw.get("potential"), dt=dt, c_lhy=interactions.c_lhy,
                             c2=_nematic_c2(interactions), precision=kw.get("precision", "fp64"))
        n_steps = kw.get("n_steps", 10000)
        res = b.ground_state(n_steps, kw.get("tol", 1e-10))
        results = []
        for (state, idx, _), r in zip(starts, res):
            results.append(dict(initial_state=state, idx=idx, workspace=None, psi=None, **r))
        ib = min(range(len(results)), key=lambda i: results[i]["energy"])
        for i, r in enumerate(results):
            r["psi"] = b.psi(i)
        b.close()
        best = results[ib]
        sp = SimParams(dt, n_steps, True, 1, max(1, n_steps // 10))
        best["workspace"] = make_workspace(grid=grid, atom=atom, interactions=interactions, zeeman=zeeman,
                                           potential=kw.get("potential"), sim_params=sp, psi_init=best["psi"],
                                           precision=kw.get("precision", "fp64"), graphs=kw.get("graphs", True))
    else:
        results = []
        for state, idx, p0 in starts:
            r = find_ground_state(grid=grid, atom=atom, interactions=interactions, psi_init=p0, **kw)
            results.append(dict(initial_state=state, idx=idx, **r))
        best = min(results, key=lambda r: r["energy"])
    return dict(workspace=best["workspace"], converged=best["converged"], energy=best["energy"],
                initial_state=best["initial_state"], all_results=results)


def scan_continuation(*, param_values, make_interactions: Callable, grid, atom, initial_state="polar",
                      energy_jump_threshold=0.1, n_steps_continuation=500, n_steps_fresh=5000, **kw) -> list:
    """``scan_continuation`` (src/ground_state.jl:328-378): each point warm-starts from the
    previous ground state, an energy jump above the threshold falls back to a multistart search
    (batched when eligible), and each point is labelled by ``classify_phase`` on the device."""
    results = []
    prev_psi = None
    prev_E = float("nan")
    for val in param_values:
        inter = make_interactions(val)
        if prev_psi is not None:
            r = find_ground_state(grid=grid, atom=atom, interactions=inter, psi_init=prev_psi,
                                  n_steps=n_steps_continuation, **kw)
        else:
            r = find_ground_state(grid=grid, atom=atom, interactions=inter, initial_state=initial_state,
                                  n_steps=n_steps_fresh, **kw)
        multistart = False
        if not math.isnan(prev_E) and abs(r["energy"] - prev_E) / max(abs(prev_E), 1e-30) > energy_jump_threshold:
            r["workspace"].close()
            r = find_ground_state_multistart(grid=grid, atom=atom, interactions=inter, n_steps=n_steps_fresh, **kw)
            multistart = True
        ws = r["workspace"]
        phase = classify_phase(ws)["phase"]
        psi = ws.psi
        results.append(dict(param=val, energy=r["energy"], converged=r["converged"], phase=phase, psi=psi,
                            multistart=multistart))
        ws.close()
        prev_psi = psi
        prev_E = r["energy"]
    return results


def estimate_splitting_error(ws: Workspace) -> float:
    """``estimate_splitting_error`` (src/diagnostics.jl:214-251): one split step of dt against
    two of dt/2 from the current state (restored afterwards, the saved copy on the device);
    max|psi_1 - psi_2| / max|psi|."""
    err = C.c_double()
    check(ws._lib.sbec_estimate_splitting_error(ws.handle, C.byref(err)))
    return err.value


def validate_conservation(ws: Workspace, *, n_steps: int = 100, tol_norm: float = 1e-12, tol_energy: float = 1e-3,
                          tol_magnetization: float = 1e-6) -> dict:
    """``validate_conservation`` (src/diagnostics.jl:259-293): the drifts of N, E and Mz over
    n_steps split steps on the device (the state restored), passed when all are below their
    tolerances."""
    nd, ed, md = C.c_double(), C.c_double(), C.c_double()
    check(ws._lib.sbec_conservation_drift(ws.handle, int(n_steps), C.byref(nd), C.byref(ed), C.byref(md)))
    return dict(passed=nd.value < tol_norm and ed.value < tol_energy and md.value < tol_magnetization,
                norm_drift=nd.value, energy_drift=ed.value, magnetization_drift=md.value)


def find_phase_boundary(*, param_range, make_interactions: Callable, grid, atom, tol: float = 0.01,
                        max_bisections: int = 20, batched=None, **kw) -> dict:
    """``find_phase_boundary`` (src/phase_boundary.jl:9-60): bisection on the phase label
    (``classify_phase`` on the device) of ``find_ground_state`` at each probe.  The two
    endpoint solves are independent and run as one GroundStateBatch when eligible (contact
    couplings, plain ITP loop; batched=None decides, True/False forces), with
    find_ground_state's loop, check interval and initial state per solve; the bisection
    probes depend on each other and run one at a time."""
    def classify_at(val):
        r = find_ground_state(grid=grid, atom=atom, interactions=make_interactions(val), **kw)
        ws = r["workspace"]
        phase = classify_phase(ws)["phase"]
        ws.close()
        return phase

    a, b = param_range
    ia, ib = make_interactions(a), make_interactions(b)
    use_batch = (_batch_eligible(atom, ia, kw) and _batch_eligible(atom, ib, kw) and ia.c_lhy == ib.c_lhy
                 and _nematic_c2(ia) == _nematic_c2(ib) if batched is None else bool(batched))
    if use_batch:
        dt = kw.get("dt", 0.001)
        zeeman = ZeemanParams() if kw.get("zeeman") is None else kw["zeeman"]
        p0 = init_psi(grid, atom.F, kw.get("initial_state", "polar"))
        for inter in (ia, ib):
            _validate_itp(zeeman, inter, atom.F, dt, p0, 0.0)
        bt = GroundStateBatch(grid=grid, atom=atom, c0s=[ia.c0, ib.c0], c1s=[ia.c1, ib.c1], psi_inits=[p0, p0],
                              zeeman=zeeman, potential=kw.get("potential"), dt=dt, c_lhy=ia.c_lhy,
                              c2=_nematic_c2(ia) or 0.0, precision=kw.get("precision", "fp64"))
        bt.ground_state(kw.get("n_steps", 10000), kw.get("tol", 1e-10))
        phase_a, phase_b = bt.classify_phase(0)["phase"], bt.classify_phase(1)["phase"]
        bt.close()
    else:
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


def _config(grid: Grid, F: int, zeeman, sim_params: SimParams, precision: str, interactions=None) -> _lib.sbec_config:
    cfg = _lib.sbec_config()
    cfg.ndim = grid.config.ndim
    for d in range(grid.config.ndim):
        cfg.n[d] = grid.config.n_points[d]
        cfg.L[d] = grid.config.box_size[d]
    cfg.F = F
    if interactions is not None:
        cfg.c0, cfg.c1, cfg.c_lhy = interactions.c0, interactions.c1, interactions.c_lhy
        ce = tuple(interactions.c_extra)
        if len(ce) > _lib.SBEC_MAX_C_EXTRA:
            raise _lib.ArgumentError("too many c_extra entries")
        cfg.n_c_extra = len(ce)
        for i, v in enumerate(ce):
            cfg.c_extra[i] = float(v)
    z = zeeman(0.0) if callable(zeeman) else zeeman
    cfg.zeeman_p, cfg.zeeman_q = z.p, z.q
    cfg.dt = sim_params.dt
    cfg.imaginary_time = int(bool(sim_params.imaginary_time))
    cfg.normalize_every = int(sim_params.normalize_every)
    if precision not in PRECISIONS:
        raise _lib.ArgumentError(f"unknown precision {precision!r}")
    cfg.precision = PRECISIONS[precision]
    return cfg


class GroundStateBatch:
    """Independent ITP solves that share F, dt and Zeeman, stepped together.

    Each solve follows ``find_ground_state``'s loop and convergence test
    (src/ground_state.jl:116-169) with its own c0, c1 and initial psi; solves leave
    the batch at the check where they converge.  ``grid`` puts every solve on one grid;
    ``grids`` gives one grid per solve (sbec_batch_create_grids: solves are grouped by grid
    and the groups advance concurrently), with ``potential`` evaluated on each grid.
    ``atoms`` (one AtomSpecies per solve, with ``grids``) mixes spins: solves are grouped by
    grid and F (sbec_batch_create_mixed).  ``c_lhy`` and the nematic ``c2`` (the reference's
    c_extra[0], src/nematic.jl:34-51) are shared by every solve.
    """

    def __init__(self, *, grid: Optional[Grid] = None, atom: Optional[AtomSpecies] = None, c0s, c1s, psi_inits,
                 zeeman=None, potential=None, dt: float = 0.005, c_lhy: float = 0.0, c2: float = 0.0,
                 precision: str = "fp32", grids=None, atoms=None):
        lib = load()
        if (grid is None) == (grids is None):
            raise _lib.ArgumentError("give either grid (one grid for every solve) or grids (one per solve)")
        if (atom is None) == (atoms is None):
            raise _lib.ArgumentError("give either atom (one spin for every solve) or atoms (one per solve)")
        if atoms is not None and grids is None:
            raise _lib.ArgumentError("atoms (one spin per solve) goes with grids (one grid per solve)")
        self.n = len(psi_inits)
        self.atoms = [atom] * self.n if atoms is None else list(atoms)
        if len(self.atoms) != self.n:
            raise _lib.ArgumentError("atoms and psi_inits must have the same length")
        atom = self.atoms[0]
        self.F, self.D = atom.F, 2 * atom.F + 1
        if len(c0s) != self.n or len(c1s) != self.n:
            raise _lib.ArgumentError("c0s, c1s and psi_inits must have the same length")
        self.grids = [grid] * self.n if grids is None else list(grids)
        if len(self.grids) != self.n:
            raise _lib.ArgumentError("grids and psi_inits must have the same length")
        self.grid = grid if grid is not None else self.grids[0]
        zeeman = ZeemanParams() if zeeman is None else zeeman
        cfg = _config(self.grid, atom.F, zeeman, SimParams(dt, 1, True, 1, 1), precision,
                      InteractionParams(0.0, 0.0, c_lhy, (float(c2),) if abs(float(c2)) > 1e-30 else ()))
        c0 = np.ascontiguousarray(c0s, dtype=np.float64)
        c1 = np.ascontiguousarray(c1s, dtype=np.float64)
        h = C.c_void_p()
        if grids is None:
            psi = np.concatenate([to_interleaved(p) for p in psi_inits])
            V = np.ascontiguousarray(evaluate_potential(potential, grid).ravel(order="F"))
            check(lib.sbec_batch_create(C.byref(cfg), self.n, dptr(c0), dptr(c1), dptr(psi), dptr(V), C.byref(h)))
        else:
            nd = self.grid.config.ndim
            n = np.ones(3 * self.n, dtype=np.int32)
            L = np.ones(3 * self.n, dtype=np.float64)
            keep, Vs = [], {}
            psi_p = (C.POINTER(C.c_double) * self.n)()
            V_p = (C.POINTER(C.c_double) * self.n)()
            for i, (g, p) in enumerate(zip(self.grids, psi_inits)):
                if g.config.ndim != nd:
                    raise _lib.ArgumentError("every grid of a batch has the same number of axes")
                n[3 * i:3 * i + nd] = g.config.n_points
                L[3 * i:3 * i + nd] = g.config.box_size
                buf = to_interleaved(p)
                keep.append(buf)
                psi_p[i] = dptr(buf)
                key = (tuple(g.config.n_points), tuple(g.config.box_size))
                if key not in Vs:
                    Vs[key] = np.ascontiguousarray(evaluate_potential(potential, g).ravel(order="F"))
                V_p[i] = dptr(Vs[key])
            if atoms is None:
                check(lib.sbec_batch_create_grids(C.byref(cfg), self.n, n.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  dptr(L), dptr(c0), dptr(c1), psi_p, V_p, C.byref(h)))
            else:
                Fs = np.ascontiguousarray([a.F for a in self.atoms], dtype=np.int32)
                check(lib.sbec_batch_create_mixed(C.byref(cfg), self.n, Fs.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  n.ctypes.data_as(C.POINTER(C.c_int32)), dptr(L), dptr(c0),
                                                  dptr(c1), psi_p, V_p, C.byref(h)))
        self._h = h
        self._lib = lib

    def close(self) -> None:
        if self._h is not None:
            check(self._lib.sbec_batch_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ground_state(self, n_steps, tol: float, check_every=None) -> list:
        """find_ground_state's loop for every solve.  n_steps (and check_every) is one value for
        all solves or one per solve; check_every defaults to find_ground_state's max(1, n // 10)."""
        out = (_lib.sbec_gs_result * self.n)()
        if np.ndim(n_steps) == 0 and np.ndim(check_every) == 0:
            ce = max(1, int(n_steps) // 10) if check_every is None else check_every
            check(self._lib.sbec_batch_ground_state(self._h, int(n_steps), float(tol), int(ce), out))
        else:
            ns = np.broadcast_to(np.asarray(n_steps, dtype=np.int64), (self.n,)).copy()
            if check_every is None:
                ce = np.maximum(1, ns // 10)
            else:
                ce = np.broadcast_to(np.asarray(check_every, dtype=np.int64), (self.n,)).copy()
            check(self._lib.sbec_batch_ground_state_each(self._h, ns.ctypes.data_as(C.POINTER(C.c_int64)),
                                                         float(tol), ce.ctypes.data_as(C.POINTER(C.c_int64)), out))
        return [dict(converged=bool(r.converged), energy=r.energy, dE=r.dE, dpsi=r.dpsi, steps=r.steps) for r in out]

    def set_graph_mode(self, graphs: bool) -> None:
        """As Workspace.set_graph_mode, for every group of the batch."""
        check(self._lib.sbec_batch_set_graph_mode(self._h, 1 if graphs else 0))

    def psi(self, i: int) -> np.ndarray:
        g = self.grids[int(i)]
        D = 2 * self.atoms[int(i)].F + 1
        n = int(np.prod(g.config.n_points)) * D
        buf = np.empty(2 * n)
        check(self._lib.sbec_batch_get_psi(self._h, int(i), dptr(buf)))
        return from_interleaved(buf, g.config.n_points, D)

    def energies(self) -> np.ndarray:
        E = np.empty(self.n)
        check(self._lib.sbec_batch_energies(self._h, dptr(E)))
        return E

    def classify_phase(self, i: int) -> dict:
        """``classify_phase`` (src/diagnostics.jl:166-206) of solve i, reduced on the device."""
        info = _lib.sbec_phase_info()
        check(self._lib.sbec_batch_classify_phase(self._h, int(i), C.byref(info)))
        return _phase_dict(info)

    @property
    def tuning_report(self) -> str:
        return _report(self._lib.sbec_batch_tuning_report, self._h)


def batch_supported(grid: Grid, F: int, precision: str = "fp32", c_lhy: float = 0.0, c2: float = 0.0) -> bool:
    """Whether solves of spin F with contact couplings (and the nematic c2) on `grid` can run as
    a GroundStateBatch (sbec_batch_supported: power-of-two axes, D in {1, 3, 5}, a row pass that
    fits the first axis).  Needs no device."""
    cfg = _config(grid, F, ZeemanParams(), SimParams(0.005, 1, True, 1, 1), precision,
                  InteractionParams(0.0, 0.0, c_lhy, (float(c2),) if abs(float(c2)) > 1e-30 else ()))
    ok = C.c_int32()
    check(load().sbec_batch_supported(C.byref(cfg), C.byref(ok)))
    return bool(ok.value)


def tune_table_export() -> str:
    """The autotuner's process-wide decisions (shape<TAB>variant lines), for saving."""
    lib = load()
    n = C.c_int64()
    check(lib.sbec_tune_table_export(None, 0, C.byref(n)))
    buf = C.create_string_buffer(n.value + 1)
    check(lib.sbec_tune_table_export(buf, n.value + 1, C.byref(n)))
    return buf.value.decode()


def tune_table_import(text: str) -> None:
    """Load saved autotuner decisions: shapes found there are not timed again, so FP32 results
    are the same in every process that loads the same table."""
    check(load().sbec_tune_table_import(text.encode()))


def tune_freeze(frozen: bool = True) -> None:
    """frozen=True: call shapes missing from the autotuner's table take their default variant
    instead of being timed, so no later result depends on a timing race; False: time new
    shapes again (default)."""
    check(load().sbec_tune_freeze(1 if frozen else 0))


def _report(fn, handle) -> str:
    n = C.c_int64()
    check(fn(handle, None, 0, C.byref(n)))
    buf = C.create_string_buffer(n.value + 1)
    check(fn(handle, buf, n.value + 1, C.byref(n)))
    return buf.value.decode()


def find_ground_states_batched(*, grid: Grid, atom: AtomSpecies, interactions: list, psi_inits: list, zeeman=None,
                               potential=None, dt: float = 0.005, n_steps: int = 10000, tol: float = 1e-10,
                               precision: str = "fp32") -> list:
    """``find_ground_state`` for many (interactions, psi0) pairs at once; one result per pair.
    The batch takes per-solve c0 and c1 and a shared c_lhy and nematic c2; higher couplings in
    c_extra (the tensor path) are not on the batched path."""
    c2s = {_nematic_c2(ip) for ip in interactions}
    if None in c2s:
        raise _lib.UnsupportedError("batched solves take c0, c1, c_lhy and c2 only; higher c_extra needs "
                                    "find_ground_state")
    if len(c2s) > 1:
        raise _lib.UnsupportedError("the solves of a batch share one nematic c2")
    b = GroundStateBatch(grid=grid, atom=atom, c0s=[ip.c0 for ip in interactions], c1s=[ip.c1 for ip in interactions],
                         psi_inits=psi_inits, zeeman=zeeman, potential=potential, dt=dt,
                         c_lhy=interactions[0].c_lhy if interactions else 0.0, c2=c2s.pop() if c2s else 0.0,
                         precision=precision)
    res = b.ground_state(n_steps, tol)
    for i, r in enumerate(res):
        r["psi"] = b.psi(i)
    b.close()
    return res


__all__ = [n for n in dir() if not n.startswith("_")]
