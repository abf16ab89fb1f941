"""ctypes binding of libkwave_gb300.so (declarations in include/kwave_gb300.h).

The library is built in-tree by ``kwave_gb300.build.build()``.  There is no
CPU fallback: if the shared library is missing or no CUDA device is present,
``lib()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libkwave_gb300.so"

KW_OK, KW_ERR_INVALID, KW_ERR_CUDA, KW_ERR_OOM, KW_ERR_UNSUPPORTED, KW_ERR_STATE = range(6)

# field ids
KW_F_C0, KW_F_RHO0, KW_F_DTRSG0, KW_F_DTRSG1, KW_F_DTRSG2, KW_F_BONA, KW_F_TAU, KW_F_ETA, KW_F_P0 = range(9)
# tables
KW_T_K, KW_T_PML, KW_T_PMLSG, KW_T_OPGRAD, KW_T_OPDIV, KW_T_UNSTAG, KW_T_WCOORD = range(7)
# source modes
KW_SRC_DIRICHLET, KW_SRC_ADDITIVE, KW_SRC_ADDITIVE_NC = range(3)
SRC_MODES = {"dirichlet": KW_SRC_DIRICHLET, "additive": KW_SRC_ADDITIVE, "additive-no-correction": KW_SRC_ADDITIVE_NC}
# series
KW_R_P, KW_R_UX_ST, KW_R_UY_ST, KW_R_UZ_ST, KW_R_UX, KW_R_UY, KW_R_UZ = range(7)
# fields
KW_FLD_P, KW_FLD_U0, KW_FLD_U1, KW_FLD_U2, KW_FLD_RHO0, KW_FLD_RHO1, KW_FLD_RHO2 = range(7)
KW_AGG_MAX, KW_AGG_MIN, KW_AGG_RMS = range(3)
KW_DESC_GENERIC_FFT = 1


class KwGridDesc(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32),
        ("shape", C.c_int32 * 3),
        ("Nt", C.c_int32),
        ("record_start", C.c_int32),
        ("spacing", C.c_double * 3),
        ("dt", C.c_double),
        ("c_ref", C.c_double),
        ("use_sg", C.c_int32),
        ("use_kspace", C.c_int32),
        ("absorb_mode", C.c_int32),
        ("dispersion", C.c_int32),
        ("nonlinear", C.c_int32),
        ("flags", C.c_int32),
        ("alpha_power", C.c_double),
    ]


class KwaveGB300Error(RuntimeError):
    """A failing call of libkwave_gb300 (message from kw_last_error)."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


_lib = None

# exported symbols and their prototypes: (restype, argtypes)
_P = C.c_void_p
_PROTOS = {
    "kw_version": (C.c_int32, []),
    "kw_last_error": (C.c_char_p, []),
    "kw_device_query": (C.c_int32, [C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_uint64)]),
    "kw_plan_create": (C.c_int32, [C.POINTER(KwGridDesc), C.POINTER(_P)]),
    "kw_plan_set_field": (C.c_int32, [_P, C.c_int32, _P, C.c_int64, C.c_float]),
    "kw_plan_set_table": (C.c_int32, [_P, C.c_int32, C.c_int32, _P, C.c_int64]),
    "kw_plan_set_source": (C.c_int32, [_P, C.c_int32, C.c_int32, _P, C.c_int32, _P, C.c_int32, C.c_int32]),
    "kw_plan_set_sensor": (C.c_int32, [_P, _P, C.c_int32, C.c_int32]),
    "kw_plan_set_sensor_interp": (C.c_int32, [_P, C.c_int32, C.c_int32, _P, _P]),
    "kw_plan_set_p0_smoothing": (C.c_int32, [_P, _P, C.c_int32, C.c_double]),
    "kw_plan_derive_medium": (C.c_int32, [_P, C.c_int32, _P, C.c_int64, C.c_double, C.c_double, C.c_int32]),
    "kw_plan_finalize": (C.c_int32, [_P]),
    "kw_plan_run": (C.c_int32, [_P, C.c_int32, _P]),
    "kw_plan_set_graphs": (C.c_int32, [_P, C.c_int32]),
    "kw_plan_adjoint_p0": (C.c_int32, [_P, _P, C.c_int64, _P, _P]),
    "kw_plan_adjoint": (C.c_int32, [_P, _P, C.c_int64, _P, _P, _P]),
    "kw_plan_set_checkpoints": (C.c_int32, [_P, C.c_int32]),
    "kw_plan_update_p0": (C.c_int32, [_P, _P, C.c_int64]),
    "kw_plan_update_source": (C.c_int32, [_P, C.c_int32, _P, C.c_int32, C.c_int32]),
    "kw_plan_set_radix_order": (C.c_int32, [_P, C.c_int32]),
    "kw_batch_autotune_radix": (C.c_int32, [_P, C.c_int32, _P, C.POINTER(C.c_int32)]),
    "kw_batch_set_radix_order": (C.c_int32, [_P, C.c_int32]),
    "kw_batch_set_loops": (C.c_int32, [_P, C.c_int32]),
    "kw_batch_graph_launches": (C.c_int32, [_P, C.POINTER(C.c_int64)]),
    "kw_plan_set_wait_test": (C.c_int32, [_P, C.c_int32]),
    # learned warm start (kw_unet.cu)
    "kw_umma_gemm": (C.c_int32, [_P, _P, _P, C.c_int32, C.c_int32, C.c_int32, _P]),
    "kw_umma_gemm_mn": (C.c_int32, [_P, _P, _P, C.c_int32, C.c_int32, C.c_int32, _P]),
    "kw_conv3x3": (C.c_int32, [_P, C.c_int32, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P, _P, C.c_int32,
                               C.c_int32, _P, _P, _P]),
    "kw_conv3x3_wgrad": (C.c_int32, [_P, C.c_int32, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P, C.c_int32,
                                     _P, _P]),
    "kw_unet_avgpool2": (C.c_int32, [_P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "kw_unet_avgpool2_bwd": (C.c_int32, [_P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P, _P]),
    "kw_unet_relu_grad": (C.c_int32, [_P, _P, _P, C.c_int64, _P]),
    "kw_unet_split_concat_grad": (C.c_int32, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P, _P, _P,
                                              _P]),
    "kw_unet_flip_weights": (C.c_int32, [_P, _P, C.c_int32, C.c_int32, _P]),
    "kw_unet_bias_grad": (C.c_int32, [_P, _P, C.c_int64, C.c_int32, _P]),
    "kw_unet_mse_grad": (C.c_int32, [_P, C.c_int32, _P, C.c_float, _P, _P, C.c_int64, C.c_float, _P, _P]),
    "kw_unet_residual_out": (C.c_int32, [_P, C.c_int32, _P, C.c_float, _P, C.c_int64, _P]),
    "kw_unet_adam": (C.c_int32, [_P, _P, _P, _P, _P, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float,
                                 C.c_int32, _P]),
    "kw_unet_image_to_nhwc": (C.c_int32, [_P, _P, C.c_int64, C.c_int32, C.c_float, _P]),
    "kw_plan_autotune": (C.c_int32, [_P, C.c_int32, _P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "kw_batch_create": (C.c_int32, [_P, C.c_int32, C.POINTER(_P)]),
    "kw_batch_run": (C.c_int32, [_P, C.c_int32, _P]),
    "kw_batch_destroy": (C.c_int32, [_P]),
    "kw_batch_launch_count": (C.c_int32, [_P, C.POINTER(C.c_int64)]),
    "kw_batch_autotune": (C.c_int32, [_P, C.c_int32, _P, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int32)]),
    "kw_plan_sync": (C.c_int32, [_P, _P]),
    "kw_plan_time_index": (C.c_int32, [_P, C.POINTER(C.c_int32)]),
    "kw_plan_read_series": (C.c_int32, [_P, C.c_int32, _P, C.c_int64]),
    "kw_plan_read_aggregate": (C.c_int32, [_P, C.c_int32, C.c_int32, _P, C.c_int64]),
    "kw_plan_read_field": (C.c_int32, [_P, C.c_int32, _P, C.c_int64]),
    "kw_plan_field_device_ptr": (C.c_int32, [_P, C.c_int32, C.POINTER(_P)]),
    "kw_plan_reset": (C.c_int32, [_P]),
    "kw_plan_set_timing": (C.c_int32, [_P, C.c_int32]),
    "kw_plan_read_timing": (C.c_int32, [_P, _P, _P]),
    "kw_plan_launch_count": (C.c_int32, [_P, C.POINTER(C.c_int64)]),
    "kw_gradient_noalloc": (C.c_int32, [_P, _P, C.c_int32, _P, _P, C.c_int32, C.c_double, C.c_int32, _P]),
    "kw_plan_destroy": (C.c_int32, [_P]),
}
KW_K_NAMES = ("axis_ops", "axis_plain", "rows_init", "rows_u", "rows_rho", "rows_eos")

EXPORTED_SYMBOLS = tuple(_PROTOS)


def load(path: os.PathLike | str | None = None):
    """Load the shared library (no device access)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise ImportError(f"libkwave_gb300.so not built at {p}; run kwave_gb300.build.build() (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def lib():
    return load()


def check(rc: int):
    if rc != KW_OK:
        msg = lib().kw_last_error().decode(errors="replace")
        if rc in (KW_ERR_INVALID,):
            raise ValueError(msg)
        if rc == KW_ERR_UNSUPPORTED:
            raise NotImplementedError(msg)
        raise KwaveGB300Error(rc, msg)


def ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def require_device():
    """Fail loudly when no CUDA device is usable (the backend has no CPU path)."""
    sm, ma, mi, fr = C.c_int32(), C.c_int32(), C.c_int32(), C.c_uint64()
    rc = lib().kw_device_query(C.byref(sm), C.byref(ma), C.byref(mi), C.byref(fr))
    if rc != KW_OK:
        raise RuntimeError("kwave_gb300 needs a CUDA GPU: " + lib().kw_last_error().decode(errors="replace"))
    return dict(sm_count=sm.value, cc=(ma.value, mi.value), free_bytes=fr.value)
