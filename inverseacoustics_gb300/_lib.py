"""ctypes binding of libia.so (the C ABI declared in include/ia.h).

The shared library is built in-tree by ``inverseacoustics_gb300._build``.
There is no fallback: if the library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# IA_LIBRARY selects another in-tree build, e.g. the bounds-checked
# libia_debug.so (inverseacoustics_gb300._build.build(debug_bounds=True))
LIB_PATH = os.environ.get("IA_LIBRARY") or os.path.join(HERE, "libia.so")

IA_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA runtime error", 3: "allocation failed",
          4: "Jacobi iteration did not converge", 5: "singular matrix", 6: "non-finite value",
          7: "invalid quadrature rule", 8: "size above the entry point's limit",
          9: "workspace would grow during stream capture"}
IA_INFO_NOCONV, IA_INFO_SINGULAR, IA_INFO_NONFINITE, IA_INFO_TIMEOUT = 1, 2, 4, 8
IA_INFO_PRECISION, IA_INFO_UNRESOLVED = 16, 32
IA_GCV_STANDARD, IA_GCV_REFERENCE = 0, 1
IA_PREC_FP64, IA_PREC_MIXED = 0, 1
IA_METHOD_TIKHONOV_GCV, IA_METHOD_TSVD, IA_METHOD_TIKHONOV_FIXED = 0, 1, 2
IA_METHOD_TIKHONOV_LCURVE, IA_METHOD_TIKHONOV_QUASIOPT = 3, 4
IA_METHOD_DSVD_FIXED, IA_METHOD_DSVD_LCURVE, IA_METHOD_DSVD_QUASIOPT = 5, 6, 7


class IAError(RuntimeError):
    def __init__(self, code: int, where: str = ""):
        self.code = code
        super().__init__(f"{where}: {STATUS.get(code, 'unknown status')} (ia_status {code})")


class Config(C.Structure):
    _fields_ = [("c", C.c_double), ("rho", C.c_double), ("method", C.c_int), ("gcv_mode", C.c_int),
                ("gcv_points", C.c_int), ("gcv_lo", C.c_double), ("gcv_hi", C.c_double),
                ("lambda_fixed", C.c_double), ("tsvd_k", C.c_int), ("precision", C.c_int),
                ("svd_max_sweeps", C.c_int), ("refine_steps", C.c_int), ("mode_iters", C.c_int),
                ("mode_oversample", C.c_int), ("gemm_slices", C.c_int),
                ("mixed_guard", C.c_double), ("pipeline_parts", C.c_int), ("mixed_fallback", C.c_int)]


IA_ADMM_L1, IA_ADMM_L2, IA_ADMM_LP = 1, 2, 3


class AdmmConfig(C.Structure):
    _fields_ = [("norm", C.c_int), ("max_iters", C.c_int), ("rho", C.c_double), ("gamma", C.c_double),
                ("epsilon", C.c_double), ("p", C.c_double), ("gst_iters", C.c_int), ("precision", C.c_int)]


class Rules(C.Structure):
    _fields_ = [("nq", C.c_int), ("regular", C.c_void_p), ("nqs", C.c_int), ("singular", C.c_void_p)]


_lib = None

_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_PP = C.POINTER(C.c_void_p)

_SIGS = {
    "ia_config_default": (None, [_P]),
    "ia_admm_config_default": (None, [_P]),
    "ia_admm_batch": (_I, [_P, _I, _I, _I, _P, _I, _P, _P, _P, _P, _P, _P, _P]),
    "ia_config_size": (_I, []),
    "ia_status_string": (C.c_char_p, [_I]),
    "ia_version": (C.c_char_p, []),
    "ia_last_cuda_error": (_I, []),
    "ia_bounds_report": (_I, [C.POINTER(C.c_int), C.POINTER(C.c_ulonglong), C.POINTER(C.c_char_p),
                              C.POINTER(C.c_int), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "ia_free": (None, [_P]),
    "ia_read_msh": (_I, [C.c_char_p, _D, _D, _PP, _PP, _PP, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    "ia_esm": (_I, [_I, _I, _P, _P, _PP, _PP, _D, _D, _P]),
    "ia_ibem": (_I, [_I, _I, _I, _P, _P, _P, _PP, _PP, _D, _I, _P, _P, _P]),
    "ia_invr": (_I, [_I, _I, _I, _P, _P, _P, _PP, _PP, _PP, _D, _I, _P, _I, _P, _P]),
    "ia_hels": (_I, [_I, _I, _P, _P, _PP, _PP, _PP, _D, _I, _P]),
    "ia_csvd": (_I, [_I, _I, _P, _PP, _PP, _PP]),
    "ia_tsvd": (_I, [_I, _I, _I, _I, _P, _P, _P, _P, _PP]),
    "ia_to_pressure": (_I, [_I, _I, _P, _P, _PP]),
    "ia_to_velocity": (_I, [_I, _I, _P, _P, _PP]),
    "ia_sound_power": (_I, [_I, _P, _P, C.POINTER(C.c_double), _D]),
    "ia_create": (_I, [_PP, _I, _P]),
    "ia_destroy": (_I, [_P]),
    "ia_set_stream": (_I, [_P, _P]),
    "ia_synchronize": (_I, [_P]),
    "ia_launch_count": (C.c_longlong, [_P]),
    "ia_tune_table_size": (_I, []),
    "ia_tune_reset": (None, []),
    "ia_last_fallback_bins": (_I, [_P]),
    "ia_capture_begin": (_I, [_P]),
    "ia_capture_end": (_I, [_P, _PP]),
    "ia_graph_launch": (_I, [_P]),
    "ia_graph_kernel_count": (_I, [_P]),
    "ia_graph_destroy": (_I, [_P]),
    "ia_mesh_create": (_I, [_P, _I, _I, _P, _P, _P, _PP]),
    "ia_mesh_destroy": (_I, [_P]),
    "ia_monopole_batch": (_I, [_P, _I, _I, _I, _P, _P, _P, _P]),
    "ia_ibem_assemble_batch": (_I, [_P, _P, _I, _P, _I, _P, _I, _P, _P, _P, _P, _P, _P]),
    "ia_ibem_transfer_batch": (_I, [_P, _P, _I, _P, _I, _P, _P, _P, _P]),
    "ia_hels_batch": (_I, [_P, _I, _P, _I, _I, _P, _P]),
    "ia_svd_batch": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P]),
    "ia_regularize_batch": (_I, [_P, _I, _I, _I, _P, _P, _P, _I, _P, _P, _P, _P]),
    "ia_solve_batch": (_I, [_P, _I, _I, _I, _P, _I, _P, _P, _P, _P, _P, _P]),
    "ia_solve_batch_noalloc": (_I, [_P, _I, _I, _I, _P, _I, _P, _P, _P, _P, _P, _P]),
    "ia_zgemm_batch": (_I, [_P, _I, _I, _I, _I, _I, _D, _P, _I, C.c_longlong, _P, _I, C.c_longlong, _D, _P, _I,
                            C.c_longlong, _I, _I, _I, _P]),
    "ia_ibem_solve_batch": (_I, [_P, _P, _I, _P, _I, _P, _I, _P, _P, _P, _P, _P, _P]),
    "ia_esm_solve_batch": (_I, [_P, _I, _I, _P, _P, _I, _P, _I, _P, _P, _P, _P, _P, _P]),
    "ia_hels_solve_batch": (_I, [_P, _I, _P, _I, _I, _P, _I, _P, _P, _P, _P, _P, _P]),
    "ia_sinc_resistance_batch": (_I, [_P, _I, _P, _I, _P, _D, _P, _P]),
    "ia_radiation_modes_batch": (_I, [_P, _I, _I, _P, _I, _P, _P, _P, _P]),
    "ia_sound_power_batch": (_I, [_P, _I, _I, _P, _I, _P, _P]),
    "ia_bem_modes_batch": (_I, [_P, _P, _I, _P, _I, _P, _I, _P, _I, _P, _P, _P, _P, _P, _P]),
    "ia_bem_modes_complex_batch": (_I, [_P, _P, _I, _P, _I, _P, _I, _P, _I, _P, _P, _P, _P, _P, _P]),
    "ia_esm_design_batch": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
}


def declared_symbols():
    return list(_SIGS)


def lib():
    """Load libia.so (or IA_LIBRARY).  Raises OSError if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"library not built at {LIB_PATH}; run inverseacoustics_gb300._build.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code: int, where: str):
    if code != IA_OK:
        raise IAError(code, where)


def default_config(**kw) -> Config:
    cfg = Config()
    lib().ia_config_default(C.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def default_admm_config(**kw) -> AdmmConfig:
    cfg = AdmmConfig()
    lib().ia_admm_config_default(C.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg
