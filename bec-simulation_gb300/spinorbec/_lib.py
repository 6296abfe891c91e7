"""ctypes binding of ``include/sbec.h`` (libsbec.so, built in-tree).

The library is the product path: every operator runs as CUDA kernels.  There is
no CPU fallback — loading fails loudly when ``libsbec.so`` is missing, and
workspace creation fails with :class:`DeviceError` when no GPU is present.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_ROOT / "lib" / "libsbec.so"

SBEC_MAX_C_EXTRA = 32
SBEC_MAX_CHANNELS = 32

SBEC_OK, SBEC_ERR_INVALID, SBEC_ERR_UNSUPPORTED, SBEC_ERR_OOM, SBEC_ERR_NUMERIC, SBEC_ERR_DEVICE, \
    SBEC_ERR_CALLBACK = range(7)
SBEC_FP64, SBEC_FP32_BULK = 0, 1


class SbecError(RuntimeError):
    status = -1


class ArgumentError(SbecError, ValueError):
    """Invalid argument (the reference's ``ArgumentError``)."""
    status = SBEC_ERR_INVALID


class UnsupportedError(SbecError, NotImplementedError):
    status = SBEC_ERR_UNSUPPORTED


class OutOfMemoryError(SbecError, MemoryError):
    status = SBEC_ERR_OOM


class NumericError(SbecError, ArithmeticError):
    """NaN / imaginary-time overflow detected (src/ground_state.jl:4-29)."""
    status = SBEC_ERR_NUMERIC


class DeviceError(SbecError):
    status = SBEC_ERR_DEVICE


class CallbackStop(SbecError):
    status = SBEC_ERR_CALLBACK


_ERRORS = {c.status: c for c in (ArgumentError, UnsupportedError, OutOfMemoryError, NumericError, DeviceError,
                                 CallbackStop)}


class sbec_config(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32),
        ("n", C.c_int32 * 3),
        ("L", C.c_double * 3),
        ("F", C.c_int32),
        ("c0", C.c_double),
        ("c1", C.c_double),
        ("c_lhy", C.c_double),
        ("n_c_extra", C.c_int32),
        ("c_extra", C.c_double * SBEC_MAX_C_EXTRA),
        ("gS_direct", C.c_int32),
        ("gS", C.c_double * SBEC_MAX_CHANNELS),
        ("zeeman_p", C.c_double),
        ("zeeman_q", C.c_double),
        ("enable_ddi", C.c_int32),
        ("c_dd", C.c_double),
        ("secular_ddi", C.c_int32),
        ("ddi_padding", C.c_int32),
        ("dt", C.c_double),
        ("imaginary_time", C.c_int32),
        ("normalize_every", C.c_int32),
        ("precision", C.c_int32),
        ("raman", C.c_int32),
        ("raman_omega", C.c_double),
        ("raman_delta", C.c_double),
        ("raman_k", C.c_double * 3),
        ("loss_gamma_dr", C.c_double),
        ("loss_L3", C.c_double),
    ]


class sbec_snapshot(C.Structure):
    _fields_ = [("t", C.c_double), ("step", C.c_int64), ("energy", C.c_double), ("norm", C.c_double),
                ("magnetization", C.c_double), ("psi", C.POINTER(C.c_double))]


class sbec_adaptive_params(C.Structure):
    _fields_ = [("dt_init", C.c_double), ("dt_min", C.c_double), ("dt_max", C.c_double), ("tol", C.c_double),
                ("error_mode", C.c_int32)]


class sbec_adaptive_result(C.Structure):
    _fields_ = [("n_accepted", C.c_int64), ("n_rejected", C.c_int64), ("final_dt", C.c_double)]


class sbec_gs_result(C.Structure):
    _fields_ = [("converged", C.c_int32), ("energy", C.c_double), ("dE", C.c_double), ("dpsi", C.c_double),
                ("steps", C.c_int64)]


class sbec_energy_terms(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("kinetic", "trap", "zeeman", "c0", "c1", "ddi", "lhy", "tensor", "raman")]


class sbec_phase_info(C.Structure):
    _fields_ = [("spin_order", C.c_double), ("nematic_order", C.c_double), ("magnetization_density", C.c_double),
                ("phase", C.c_int32), ("n_channels", C.c_int32),
                ("channel_weights", C.c_double * SBEC_MAX_CHANNELS),
                ("raw_channel_weights", C.c_double * SBEC_MAX_CHANNELS)]


PHASE_LABELS = ("vacuum", "ferromagnetic", "polar", "nematic", "cyclic", "mixed")


class sbec_kernel_stat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_int64), ("ms", C.c_double), ("bytes", C.c_double)]


CALLBACK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(sbec_snapshot))
ZEEMAN_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double))

_P = C.c_void_p
_D = C.POINTER(C.c_double)
_PROTOS = {
    "sbec_last_error": (C.c_char_p, []),
    "sbec_version": (C.c_char_p, []),
    "sbec_device_count": (C.c_int, []),
    "sbec_ws_create": (C.c_int, [C.POINTER(sbec_config), _D, _D, C.POINTER(_P)]),
    "sbec_ws_destroy": (C.c_int, [_P]),
    "sbec_set_psi": (C.c_int, [_P, _D]),
    "sbec_get_psi": (C.c_int, [_P, _D]),
    "sbec_set_time": (C.c_int, [_P, C.c_double, C.c_int64]),
    "sbec_get_time": (C.c_int, [_P, _D, C.POINTER(C.c_int64)]),
    "sbec_set_zeeman": (C.c_int, [_P, C.c_double, C.c_double]),
    "sbec_set_zeeman_fn": (C.c_int, [_P, ZEEMAN_FN, C.c_void_p]),
    "sbec_set_potential": (C.c_int, [_P, _D]),
    "sbec_set_dt": (C.c_int, [_P, C.c_double]),
    "sbec_tensor_channels": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), _D]),
    "sbec_half_potential": (C.c_int, [_P, C.c_double, C.c_int32]),
    "sbec_kinetic": (C.c_int, [_P, C.c_double, C.c_int32]),
    "sbec_normalize": (C.c_int, [_P]),
    "sbec_normalize_constrained": (C.c_int, [_P, C.c_double]),
    "sbec_split_step": (C.c_int, [_P, C.c_int64]),
    "sbec_strang_core": (C.c_int, [_P, C.c_double]),
    "sbec_yoshida_core": (C.c_int, [_P, C.c_double]),
    "sbec_run_simulation": (C.c_int, [_P, C.c_int64, C.c_int64, CALLBACK, C.c_void_p]),
    "sbec_run_adaptive": (C.c_int, [_P, C.POINTER(sbec_adaptive_params), C.c_double, C.c_double, CALLBACK,
                                    C.c_void_p, C.POINTER(sbec_adaptive_result)]),
    "sbec_run_yoshida": (C.c_int, [_P, C.POINTER(sbec_adaptive_params), C.c_double, C.c_double, C.c_int64,
                                   CALLBACK, C.c_void_p, C.POINTER(sbec_adaptive_result)]),
    "sbec_ground_state": (C.c_int, [_P, C.c_int64, C.c_double, C.c_int64, C.c_double, C.POINTER(sbec_gs_result)]),
    "sbec_ground_state_adaptive": (C.c_int, [_P, C.c_int64, C.c_double, C.c_double, C.POINTER(sbec_gs_result), _D]),
    "sbec_total_energy": (C.c_int, [_P, _D]),
    "sbec_energy_breakdown": (C.c_int, [_P, C.POINTER(sbec_energy_terms)]),
    "sbec_total_norm": (C.c_int, [_P, _D]),
    "sbec_magnetization": (C.c_int, [_P, _D]),
    "sbec_spin_density": (C.c_int, [_P, _D]),
    "sbec_ddi_potential": (C.c_int, [_P, C.c_int32, _D]),
    "sbec_classify_phase": (C.c_int, [_P, C.POINTER(sbec_phase_info)]),
    "sbec_batch_classify_phase": (C.c_int, [_P, C.c_int32, C.POINTER(sbec_phase_info)]),
    "sbec_profile_enable": (C.c_int, [_P, C.c_int32]),
    "sbec_profile_read": (C.c_int, [_P, C.POINTER(sbec_kernel_stat), C.c_int32, C.POINTER(C.c_int32)]),
    "sbec_launch_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "sbec_ws_stream": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "sbec_set_snapshot_mode": (C.c_int, [_P, C.c_int32]),
    "sbec_set_graph_mode": (C.c_int, [_P, C.c_int32]),
    "sbec_tuning_report": (C.c_int, [_P, C.c_char_p, C.c_int64, C.POINTER(C.c_int64)]),
    "sbec_batch_tuning_report": (C.c_int, [_P, C.c_char_p, C.c_int64, C.POINTER(C.c_int64)]),
    "sbec_tune_table_export": (C.c_int, [C.c_char_p, C.c_int64, C.POINTER(C.c_int64)]),
    "sbec_tune_freeze": (C.c_int, [C.c_int32]),
    "sbec_estimate_splitting_error": (C.c_int, [_P, _D]),
    "sbec_conservation_drift": (C.c_int, [_P, C.c_int64, _D, _D, _D]),
    "sbec_tune_table_import": (C.c_int, [C.c_char_p]),
    "sbec_batch_create": (C.c_int, [C.POINTER(sbec_config), C.c_int32, _D, _D, _D, _D, C.POINTER(_P)]),
    "sbec_batch_create_grids": (C.c_int, [C.POINTER(sbec_config), C.c_int32, C.POINTER(C.c_int32), _D, _D, _D,
                                          C.POINTER(_D), C.POINTER(_D), C.POINTER(_P)]),
    "sbec_batch_create_mixed": (C.c_int, [C.POINTER(sbec_config), C.c_int32, C.POINTER(C.c_int32),
                                          C.POINTER(C.c_int32), _D, _D, _D, C.POINTER(_D), C.POINTER(_D),
                                          C.POINTER(_P)]),
    "sbec_batch_destroy": (C.c_int, [_P]),
    "sbec_batch_ground_state": (C.c_int, [_P, C.c_int64, C.c_double, C.c_int64, C.POINTER(sbec_gs_result)]),
    "sbec_batch_ground_state_each": (C.c_int, [_P, C.POINTER(C.c_int64), C.c_double, C.POINTER(C.c_int64),
                                               C.POINTER(sbec_gs_result)]),
    "sbec_batch_set_graph_mode": (C.c_int, [_P, C.c_int32]),
    "sbec_batch_supported": (C.c_int, [C.POINTER(sbec_config), C.POINTER(C.c_int32)]),
    "sbec_batch_get_psi": (C.c_int, [_P, C.c_int32, _D]),
    "sbec_batch_energies": (C.c_int, [_P, _D]),
    "sbec_measure_fma_peak": (C.c_int, [C.c_int32, _D]),
    "sbec_component_norms_noalloc": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p]),
}

_lib = None


def lib_path() -> Path:
    return Path(os.environ.get("SBEC_LIB", str(LIB_PATH)))


def load() -> C.CDLL:
    """Load libsbec.so (raises if it has not been built — there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not p.exists():
        raise ImportError(f"libsbec.so not found at {p}; build it with bec-simulation_gb300/build.py")
    L = C.CDLL(str(p))
    for name, (res, args) in _PROTOS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status == SBEC_OK:
        return
    msg = load().sbec_last_error().decode(errors="replace")
    raise _ERRORS.get(status, SbecError)(msg)


def dptr(a):
    return a.ctypes.data_as(_D)
