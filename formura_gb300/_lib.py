"""ctypes binding of libformura_gb300.so (include/formura_gb300.h).

There is no CPU fallback: if the library is missing or was not built, the
import of the binding raises instead of computing anything another way.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from . import build as _build

c_int, c_size_t, c_void_p, c_double, c_int64 = (
    ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_double, ctypes.c_int64)


class FormuraError(RuntimeError):
    """A C-ABI call returned a non-zero fm_status."""

    def __init__(self, status: int, where: str, message: str):
        super().__init__("%s failed: %s (%s)" % (where, STATUS_NAMES.get(status, status), message))
        self.status = status


STATUS_NAMES = {0: "FM_OK", 1: "FM_ERR_ARG", 2: "FM_ERR_CUDA", 3: "FM_ERR_TIMEOUT",
                4: "FM_ERR_NONFINITE", 5: "FM_ERR_UNSUPPORTED", 6: "FM_ERR_NOMEM"}


class GsParams(ctypes.Structure):
    """fm_gs_params."""
    _fields_ = [("F", c_double), ("k", c_double), ("Du", c_double), ("Dv", c_double),
                ("dt", c_double), ("dx", c_double)]


# name -> (restype, argtypes)
SIGNATURES = {
    "fm_last_error": (ctypes.c_char_p, []),
    "fm_status_name": (ctypes.c_char_p, [c_int]),
    "fm_version": (ctypes.c_char_p, []),
    "fm_device_count": (c_int, []),
    "fm_malloc": (c_int, [ctypes.POINTER(c_void_p), c_size_t]),
    "fm_free": (c_int, [c_void_p]),
    "fm_memset": (c_int, [c_void_p, c_int, c_size_t, c_void_p]),
    "fm_memcpy_h2d": (c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    "fm_memcpy_d2h": (c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    "fm_memcpy_d2d": (c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    "fm_stream_sync": (c_int, [c_void_p]),
    "fm_host_register": (c_int, [c_void_p, c_size_t]),
    "fm_host_unregister": (c_int, [c_void_p]),
    "fm_gs3d_f64_forward": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                    ctypes.POINTER(GsParams), c_int, c_void_p]),
    "fm_gs3d_f32k_forward": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_int, ctypes.POINTER(GsParams), c_void_p]),
    "fm_gs3d_f32k_tb_forward": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_void_p, c_int, c_int,
                                        ctypes.POINTER(GsParams), c_void_p]),
    "fm_diff2d_f64_forward": (c_int, [c_int, c_int, c_void_p, c_void_p, c_double, c_int, c_void_p]),
    "fm_diff2d_f64_forward_noalloc": (c_int, [c_int, c_int, c_void_p, c_double, c_int, c_void_p]),
    "fm_gs2d_f32_forward": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                    ctypes.POINTER(GsParams), c_int, c_void_p]),
    "fm_gs2d_ensemble_create": (c_int, [ctypes.POINTER(c_void_p), c_int, ctypes.POINTER(c_int),
                                        ctypes.POINTER(c_double), ctypes.POINTER(c_double),
                                        c_double, c_double, c_double, c_double, c_int, c_int]),
    "fm_gs2d_ensemble_layout": (c_int, [c_void_p, ctypes.POINTER(c_int64),
                                        ctypes.POINTER(c_int64), ctypes.POINTER(c_int)]),
    "fm_gs2d_ensemble_forward": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                         c_int, c_void_p]),
    "fm_gs2d_ensemble_status": (c_int, [c_void_p, c_void_p]),
    "fm_gs2d_ensemble_destroy": (c_int, [c_void_p]),
    "fm_mhd_forward_f64": (c_int, [c_int, ctypes.POINTER(c_void_p), c_void_p, c_int, c_void_p]),
    "fm_mhd_forward_f32": (c_int, [c_int, ctypes.POINTER(c_void_p), c_void_p, c_int, c_void_p]),
    "fm_mhd_totals_scratch_elems": (c_size_t, [c_int]),
    "fm_mhd_totals": (c_int, [c_int, c_int, ctypes.POINTER(c_void_p), c_void_p, c_void_p,
                              c_void_p]),
    "fm_tc_gemm_bf16": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_void_p]),
    "fm_conv3x3_fwd_bf16": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p]),
    "fm_conv3x3_wgrad_bf16": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p]),
    "fm_sur_pack": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                            c_void_p]),
    "fm_sur_unpack": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, ctypes.c_float,
                              c_void_p]),
    "fm_sur_loss_grad": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_void_p, c_void_p, ctypes.c_float, ctypes.c_float, c_void_p]),
    "fm_sur_bias_grad": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "fm_sur_flip": (c_int, [c_void_p, c_void_p, c_void_p]),
    "fm_sur_adam": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                            c_void_p, c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                            ctypes.c_float, c_int, c_int, c_void_p]),
    "fm_sur_gelu_bwd": (c_int, [ctypes.c_longlong, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fm_sum_f64_scratch_elems": (c_size_t, [c_int64]),
    "fm_snapshot_create": (c_int, [ctypes.POINTER(c_void_p), c_int, ctypes.POINTER(c_int), c_int]),
    "fm_snapshot_plane_elems": (ctypes.c_longlong, [c_void_p, c_int]),
    "fm_snapshot_begin": (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p]),
    "fm_snapshot_wait": (c_int, [c_void_p, c_void_p]),
    "fm_snapshot_destroy": (None, [c_void_p]),
    "fm_sum_f64": (c_int, [c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fm_sum_f32_as_f64": (c_int, [c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fm_tensor_map_3d": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int,
                                 c_int]),
    "fm_tune_set": (c_int, [ctypes.c_char_p, c_int]),
    "fm_tune_get": (c_int, [ctypes.c_char_p, c_int]),
    "fm_tune_clear": (c_int, []),
    "fm_probe_fma": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p]),
}

_lock = threading.Lock()
_lib = None


def library_path() -> Path:
    return _build.LIB


def lib(build_if_missing: bool = True) -> ctypes.CDLL:
    """The loaded libformura_gb300.so with every signature declared."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not path.exists():
            if not build_if_missing:
                raise FileNotFoundError("%s is not built (run __graft_entry__.build())" % path)
            _build.build_library()
        h = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
        return h


def check(status: int, where: str) -> None:
    if status != 0:
        raise FormuraError(status, where, lib().fm_last_error().decode(errors="replace"))
