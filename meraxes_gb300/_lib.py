"""Loader of the in-tree CUDA library (libmxreion.so) through its C ABI.

The product path has no CPU fallback: if the library cannot be built or
loaded, `load()` raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from .params import MxGalaxies, MxGlobals, MxGrids, MxParams

_LOCK = threading.Lock()
_LIB = None

MX_OK = 0
ERRORS = {-1: "MX_EINVAL", -2: "MX_ENOMEM", -3: "MX_ECUDA", -4: "MX_ETABLE", -5: "MX_ESTATE", -6: "MX_ENOTSUP"}

# every entry point declared in include/mx_reion.h
EXPORTS = [
    "mx_create", "mx_destroy", "mx_last_error", "mx_set_redshifts", "mx_n_sfr_histories", "mx_filter_radii",
    "mx_find_HII_bubbles", "mx_ComputeTs", "mx_ComputeBrightnessTemperatureBox", "mx_step",
    "mx_find_HII_bubbles_device", "mx_ComputeTs_device", "mx_ComputeBrightnessTemperatureBox_device",
    "mx_step_device", "mx_profile_enable", "mx_profile_read", "mx_build_info",
    "mx_brightness_temperature_noalloc", "mx_ps_length", "mx_Compute_PS", "mx_Compute_PS_device",
    "mx_lightcone_init", "mx_ConstructLightcone", "mx_ConstructLightcone_device",
    "mx_construct_baryon_grids", "mx_construct_baryon_grids_device", "mx_calculate_Mvir_crit",
    "mx_calculate_Mvir_crit_device", "mx_set_xray_params", "mx_ps_loss_device", "mx_adjoint_device",
    "mx_create_limited", "mx_fft_block_sizes", "mx_zpass_blocks_per_sm", "mx_set_step_graph", "mx_batch_create", "mx_batch_run",
    "mx_batch_run_graph", "mx_batch_destroy",
    "mx_batch_last_error",
]


class MxBatchItem(ctypes.Structure):
    """ctypes image of `mx_batch_item` (include/mx_reion.h)."""

    _fields_ = [("params", ctypes.POINTER(MxParams)), ("redshifts", ctypes.POINTER(ctypes.c_double)),
                ("n_snaps", ctypes.c_int32), ("snapshot", ctypes.c_int32), ("grids", ctypes.POINTER(MxGrids)),
                ("out", ctypes.POINTER(MxGlobals)), ("status", ctypes.c_int32)]


class MxKernelStat(ctypes.Structure):
    """ctypes image of `mx_kernel_stat` (include/mx_reion.h)."""

    _fields_ = [("name", ctypes.c_char * 40), ("launches", ctypes.c_int32), ("ms", ctypes.c_double),
                ("bytes", ctypes.c_double)]


class MxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def lib_path() -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libmxreion.so")


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = lib_path()
        if build_if_missing:
            from .build import build

            build()
        if not os.path.exists(path):
            raise RuntimeError(f"CUDA library missing: {path} (run meraxes_gb300/build.py)")
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.mx_create.argtypes = [ctypes.POINTER(MxParams), ctypes.c_char_p, ctypes.POINTER(P)]
        L.mx_create.restype = ctypes.c_int
        L.mx_destroy.argtypes = [P]
        L.mx_destroy.restype = None
        L.mx_last_error.argtypes = [P]
        L.mx_last_error.restype = ctypes.c_char_p
        L.mx_set_redshifts.argtypes = [P, ctypes.POINTER(ctypes.c_double), ctypes.c_int32]
        L.mx_set_redshifts.restype = ctypes.c_int
        L.mx_n_sfr_histories.argtypes = [P]
        L.mx_n_sfr_histories.restype = ctypes.c_int32
        L.mx_fft_block_sizes.argtypes = [P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
        L.mx_fft_block_sizes.restype = ctypes.c_int
        L.mx_zpass_blocks_per_sm.argtypes = [P]
        L.mx_zpass_blocks_per_sm.restype = ctypes.c_int32
        L.mx_set_step_graph.argtypes = [P, ctypes.c_int32]
        L.mx_set_step_graph.restype = ctypes.c_int
        L.mx_filter_radii.argtypes = [P, ctypes.POINTER(ctypes.c_double), ctypes.c_int32]
        L.mx_filter_radii.restype = ctypes.c_int32
        for fn in ("mx_find_HII_bubbles", "mx_ComputeTs", "mx_ComputeBrightnessTemperatureBox", "mx_step"):
            getattr(L, fn).argtypes = [P, ctypes.c_int32, ctypes.POINTER(MxGrids), ctypes.POINTER(MxGlobals)]
            getattr(L, fn).restype = ctypes.c_int
        for fn in ("mx_find_HII_bubbles_device", "mx_ComputeTs_device", "mx_ComputeBrightnessTemperatureBox_device",
                   "mx_step_device"):
            getattr(L, fn).argtypes = [P, ctypes.c_int32, ctypes.POINTER(MxGrids), ctypes.POINTER(MxGlobals), P]
            getattr(L, fn).restype = ctypes.c_int
        L.mx_profile_enable.argtypes = [P, ctypes.c_int32]
        L.mx_profile_enable.restype = ctypes.c_int
        L.mx_profile_read.argtypes = [P, ctypes.POINTER(MxKernelStat), ctypes.c_int32]
        L.mx_profile_read.restype = ctypes.c_int32
        L.mx_build_info.argtypes = []
        L.mx_build_info.restype = ctypes.c_char_p
        L.mx_brightness_temperature_noalloc.argtypes = [ctypes.POINTER(MxParams), ctypes.c_double, P, P, P, P, P, P,
                                                        ctypes.c_char_p, ctypes.c_size_t]
        L.mx_brightness_temperature_noalloc.restype = ctypes.c_int
        L.mx_ps_length.argtypes = [P]
        L.mx_ps_length.restype = ctypes.c_int32
        L.mx_Compute_PS.argtypes = [P, P, P, P, P, ctypes.c_int32]
        L.mx_Compute_PS.restype = ctypes.c_int
        L.mx_Compute_PS_device.argtypes = [P, P, P, P, P, ctypes.c_int32, P]
        L.mx_Compute_PS_device.restype = ctypes.c_int
        L.mx_lightcone_init.argtypes = [P, ctypes.c_double, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
        L.mx_lightcone_init.restype = ctypes.c_int64
        L.mx_ConstructLightcone.argtypes = [P, ctypes.c_int32, P, P, P, P]
        L.mx_ConstructLightcone.restype = ctypes.c_int
        L.mx_ConstructLightcone_device.argtypes = [P, ctypes.c_int32, P, P, P, P, P]
        L.mx_ConstructLightcone_device.restype = ctypes.c_int
        gal = [P, ctypes.c_int32, ctypes.POINTER(MxGalaxies), ctypes.c_int32, ctypes.c_double, ctypes.c_double,
               ctypes.POINTER(MxGrids)]
        L.mx_construct_baryon_grids.argtypes = gal
        L.mx_construct_baryon_grids.restype = ctypes.c_int
        L.mx_construct_baryon_grids_device.argtypes = gal + [P]
        L.mx_construct_baryon_grids_device.restype = ctypes.c_int
        mvir = [P, ctypes.c_double, ctypes.POINTER(ctypes.c_double), P, P, P]
        L.mx_calculate_Mvir_crit.argtypes = mvir
        L.mx_calculate_Mvir_crit.restype = ctypes.c_int
        L.mx_calculate_Mvir_crit_device.argtypes = mvir + [P]
        L.mx_calculate_Mvir_crit_device.restype = ctypes.c_int
        L.mx_create_limited.argtypes = [ctypes.POINTER(MxParams), ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(P)]
        L.mx_create_limited.restype = ctypes.c_int
        L.mx_batch_create.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_size_t, ctypes.POINTER(P)]
        L.mx_batch_create.restype = ctypes.c_int
        L.mx_batch_run.argtypes = [P, ctypes.POINTER(MxBatchItem), ctypes.c_int32]
        L.mx_batch_run.restype = ctypes.c_int
        L.mx_batch_run_graph.argtypes = [P, ctypes.POINTER(MxBatchItem), ctypes.c_int32]
        L.mx_batch_run_graph.restype = ctypes.c_int
        L.mx_batch_destroy.argtypes = [P]
        L.mx_batch_destroy.restype = None
        L.mx_batch_last_error.argtypes = [P]
        L.mx_batch_last_error.restype = ctypes.c_char_p
        L.mx_set_xray_params.argtypes = [P, ctypes.c_double, ctypes.c_double]
        L.mx_set_xray_params.restype = ctypes.c_int
        L.mx_ps_loss_device.argtypes = [P, P, ctypes.c_int32, ctypes.POINTER(ctypes.c_float),
                                        ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_float), P, P]
        L.mx_ps_loss_device.restype = ctypes.c_int
        L.mx_adjoint_device.argtypes = [P, ctypes.c_int32, ctypes.POINTER(MxGrids), P, P, P,
                                        ctypes.POINTER(ctypes.c_double), P]
        L.mx_adjoint_device.restype = ctypes.c_int
        _LIB = L
        return L
