"""ctypes declarations of libsunnygb300.so (include/sunny_gb300.h).

The library must be built in-tree (``sunny.jl_gb300/libsunnygb300.so``); there is no CPU
fallback, so loading fails loudly if it is missing.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libsunnygb300.so"

SGB_OK = 0
SGB_ERR_ARG = -1
SGB_ERR_CUDA = -2
SGB_ERR_NOCONVERGE = -3
SGB_ERR_TIMEOUT = -4
SGB_ERR_STATE = -5
SGB_ERR_NOMEM = -6

MODE_DIPOLE = 0
MODE_DIPOLE_UNCORRECTED = 1
MODE_SUN = 2
FP64 = 0
FP32 = 1


class Desc(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("natoms", C.c_int32), ("N", C.c_int32),
                ("mode", C.c_int32), ("precision", C.c_int32), ("device", C.c_int32)]


class BondC(C.Structure):
    _fields_ = [("i", C.c_int32), ("j", C.c_int32), ("n", C.c_int32 * 3), ("scalar", C.c_double),
                ("bilin", C.c_double * 9), ("biquad_kind", C.c_int32), ("biquad", C.c_double * 25)]


class SiteBondC(C.Structure):
    _fields_ = [("cell", C.c_int32 * 3), ("pad", C.c_int32), ("bond", BondC)]


class Proposal(C.Structure):
    _fields_ = [("n", C.c_int32), ("kind", C.c_int32 * 4), ("weight", C.c_double * 4), ("magnitude", C.c_double * 4)]


PROPOSE_UNIFORM, PROPOSE_FLIP, PROPOSE_DELTA = 0, 1, 2


class CorrDesc(C.Structure):
    _fields_ = [("nobs", C.c_int32), ("obs", C.POINTER(C.c_double)), ("ncorr", C.c_int32),
                ("pairs", C.POINTER(C.c_int32)), ("n_all_omega", C.c_int32), ("measperiod", C.c_int32),
                ("dt", C.c_double), ("damping", C.c_double), ("tol", C.c_double), ("max_iters", C.c_int32),
                ("calculate_errors", C.c_int32)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I32 = C.c_int32
_I64 = C.c_int64
_U64 = C.c_uint64

# name -> (restype, argtypes)
SIGNATURES = {
    "sgb_create": (C.c_int, [C.POINTER(Desc), C.POINTER(_P)]),
    "sgb_destroy": (None, [_P]),
    "sgb_last_error": (C.c_char_p, [_P]),
    "sgb_nsites": (_I64, [_P]),
    "sgb_set_sites": (C.c_int, [_P, _D, _D, _D]),
    "sgb_set_onsite": (C.c_int, [_P, _I32, _D]),
    "sgb_set_bonds": (C.c_int, [_P, C.POINTER(BondC), _I32]),
    "sgb_set_bonds_at": (C.c_int, [_P, C.POINTER(SiteBondC), _I64]),
    "sgb_set_general": (C.c_int, [_P, C.POINTER(_I32), _I32, _D, _D]),
    "sgb_set_onsite_at": (C.c_int, [_P, _D]),
    "sgb_set_state": (C.c_int, [_P, _D, _D]),
    "sgb_get_state": (C.c_int, [_P, _D, _D]),
    "sgb_set_midpoint_predictor": (C.c_int, [_P, _I32]),
    "sgb_energy_grad": (C.c_int, [_P, _D]),
    "sgb_energy_grad_static": (C.c_int, [_P, _D]),
    "sgb_energy": (C.c_int, [_P, _D, _D]),
    "sgb_langevin": (C.c_int, [_P, C.c_double, C.c_double, C.c_double, _U64, _U64, _I32, _D]),
    "sgb_langevin_noise": (C.c_int, [_P, _U64, _U64, _D]),
    "sgb_midpoint": (C.c_int, [_P, C.c_double, C.c_double, C.c_double, _I32, _I32, C.POINTER(_I64)]),
    "sgb_set_langevin_cluster": (C.c_int, [_P, _I32]),
    "sgb_langevin_kernel": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "sgb_local_sweeps": (C.c_int, [_P, C.c_double, C.c_double, C.POINTER(Proposal), _U64, _U64, _D, _D, _D]),
    "sgb_local_colors": (C.c_int, [_P, C.POINTER(_I32), C.POINTER(_I32)]),
    "sgb_local_energy_change": (C.c_int, [_P, _I64, _D, _D]),
    "sgb_set_dipole_dipole": (C.c_int, [_P, C.c_double, _D, _D, _D]),
    "sgb_minimize_energy": (C.c_int, [_P, _I32, C.c_double, _U64, C.POINTER(_I32), C.POINTER(_I32), _D]),
    "sgb_corr_create": (C.c_int, [_P, C.POINTER(CorrDesc), C.POINTER(_P)]),
    "sgb_corr_destroy": (None, [_P]),
    "sgb_corr_add_sample": (C.c_int, [_P, _I32]),
    "sgb_corr_data": (C.c_int, [_P, _D, _D, C.POINTER(_I64)]),
    "sgb_corr_intensities": (C.c_int, [_P, _I32, C.POINTER(_I32), _D, _D, _I32, C.POINTER(_I32), _I32, _D]),
    "sgb_corr_merge": (C.c_int, [_P, _P]),
    "sgb_corr_compare": (C.c_int, [_P, _P, _D]),
    "sgb_corr_set_time_transform": (C.c_int, [_P, _I32]),
    "sgb_corr_time_transform": (C.c_int, [_P]),
    "sgb_corr_cross": (C.c_int, [_P, _P, _P, _P, _D]),
    "sgb_corr_profile": (C.c_int, [_P, _I32]),
    "sgb_corr_phase_times": (C.c_int, [_P, _D, C.POINTER(_I64), C.POINTER(_I64)]),
    "sgb_batch_create": (C.c_int, [C.POINTER(Desc), _I32, C.POINTER(_I32), C.POINTER(_P)]),
    "sgb_batch_create_group": (C.c_int, [C.POINTER(_P), _I32, C.POINTER(_P)]),
    "sgb_batch_destroy": (None, [_P]),
    "sgb_batch_last_error": (C.c_char_p, [_P]),
    "sgb_batch_nsites": (_I64, [_P, _I32]),
    "sgb_batch_set_couplings": (C.c_int, [_P, _D, _D, _D, _D, C.POINTER(BondC), _I32]),
    "sgb_batch_set_state": (C.c_int, [_P, _I32, _D]),
    "sgb_batch_get_state": (C.c_int, [_P, _I32, _D]),
    "sgb_batch_set_kT": (C.c_int, [_P, _D]),
    "sgb_batch_get_kT": (C.c_int, [_P, _D]),
    "sgb_batch_langevin": (C.c_int, [_P, C.c_double, C.c_double, _U64, _U64, _I32]),
    "sgb_batch_energy": (C.c_int, [_P, _D]),
    "sgb_batch_exchange": (C.c_int, [_P, _I32, _U64, _U64, _D, C.POINTER(_I64)]),
    "sgb_batch_step_ensemble": (C.c_int, [_P, C.c_double, C.c_double, _U64, _I32, _I32, C.POINTER(_I64)]),
    "sgb_batch_graph_active": (C.c_int, [_P]),
    "sgb_batch_langevin_noise": (C.c_int, [_P, _I32, _U64, _U64, _D]),
    "sgb_batch_corr_create": (C.c_int, [_P, C.POINTER(CorrDesc), C.POINTER(_P)]),
    "sgb_batch_set_midpoint_predictor": (C.c_int, [_P, _I32]),
    "sgb_batch_midpoint_shapes": (C.c_int, [_P, _I32, C.POINTER(_I32), C.POINTER(C.c_float), C.POINTER(_I32)]),
    "sgb_batch_langevin_shapes": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(_I32)]),
    "sgb_batch_set_midpoint_first_accept": (C.c_int, [_P, _I32]),
    "sgb_batch_set_midpoint_chunk": (C.c_int, [_P, _I32]),
    "sgb_batch_select_midpoint_shape": (C.c_int, [_P, _I32]),
    "sgb_adjoint_create": (C.c_int, [_P, C.POINTER(CorrDesc), _I32, _P, C.POINTER(_I32), _D, C.POINTER(_P)]),
    "sgb_adjoint_destroy": (None, [_P]),
    "sgb_adjoint_last_error": (C.c_char_p, [_P]),
    "sgb_adjoint_set_target": (C.c_int, [_P, _D]),
    "sgb_adjoint_loss_grad": (C.c_int, [_P, _D, _I32, _D, _D, _D, _D]),
    "sgb_adjoint_loss": (C.c_int, [_P, _D, _D, _D]),
    "sgb_event_record": (C.c_int, [_P, _I32]),
    "sgb_event_elapsed": (C.c_int, [_P, _I32, _I32, C.POINTER(C.c_float)]),
    "sgb_batch_event_record": (C.c_int, [_P, _I32]),
    "sgb_batch_event_elapsed": (C.c_int, [_P, _I32, _I32, C.POINTER(C.c_float)]),
    "sgb_synchronize": (C.c_int, [_P]),
    "sgb_kernel_launches": (_I64, [_P]),
    "sgb_batch_kernel_launches": (_I64, [_P]),
    "sgb_flush_l2": (C.c_int, [_P]),
    "sgb_set_wait_limit": (C.c_int, [_P, C.c_double]),
    "sgb_batch_set_wait_limit": (C.c_int, [_P, C.c_double]),
    "sgb_wait_probe": (C.c_int, [_P]),
    "sgb_version": (C.c_char_p, []),
}

_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load libsunnygb300.so and declare every entry point. Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                           " (there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_D)


class SunnyGPUError(RuntimeError):
    """Raised for a non-zero status of the C ABI; `code` holds the SGB_ERR_* value."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def check(rc: int, lib: C.CDLL, handle=None, batch: bool = False) -> None:
    if rc != SGB_OK:
        if batch:
            msg = lib.sgb_batch_last_error(handle)
        else:
            msg = lib.sgb_last_error(handle)
        raise SunnyGPUError(rc, (msg or b"").decode("utf-8", "replace") or f"error {rc}")
