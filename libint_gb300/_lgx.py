"""ctypes binding of liblgx.so (the C ABI declared in include/lgx.h).

The product path: every call lands in the CUDA library; there is no CPU
fallback.  Loading fails loudly when the shared library is missing.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

LGX_OK = 0
LGX_ERR_INVALID_ARG = 1
LGX_ERR_CUDA = 2
LGX_ERR_LMAX_EXCEEDED = 3
LGX_ERR_NO_BASIS = 4
LGX_ERR_WATCHDOG = 5
LGX_ERR_TOO_LARGE = 6
LGX_ERR_NO_DEVICE = 7

LGX_OP_COULOMB = 0
LGX_OP_ERF_COULOMB = 1
LGX_OP_ERFC_COULOMB = 2

LGX_FP64 = 0
LGX_MIXED = 1
LGX_MIXED_FP32_BOYS = 2
LGX_NOALLOC_MAX_NBF = 768
LGX_SCREEN_ORIGINAL = 0
LGX_SCREEN_CONSERVATIVE = 1

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)


class LgxShell(ctypes.Structure):
    _fields_ = [("l", ctypes.c_int32), ("pure", ctypes.c_int32),
                ("nprim", ctypes.c_int32), ("pad_", ctypes.c_int32),
                ("origin", ctypes.c_double * 3), ("alpha", _dp), ("coeff", _dp)]


class LgxJkStats(ctypes.Structure):
    _fields_ = [("quartets_fp64", ctypes.c_int64), ("quartets_fp32", ctypes.c_int64),
                ("integrals", ctypes.c_int64), ("prim_quartets", ctypes.c_int64),
                ("kernel_ms", ctypes.c_double), ("pass_ms", ctypes.c_double),
                ("flops_fp64", ctypes.c_double), ("flops_fp32", ctypes.c_double),
                ("launches", ctypes.c_int64)]


class LgxLaunchStats(ctypes.Structure):
    _fields_ = [("la", ctypes.c_int32), ("lb", ctypes.c_int32), ("lc", ctypes.c_int32),
                ("ld", ctypes.c_int32), ("fp32", ctypes.c_int32), ("kernel", ctypes.c_int32),
                ("shape", ctypes.c_int32), ("deriv", ctypes.c_int32),
                ("quartets", ctypes.c_int64), ("prim_quartets", ctypes.c_int64),
                ("integrals", ctypes.c_int64), ("flops", ctypes.c_double),
                ("ms", ctypes.c_double), ("flops_fp64", ctypes.c_double)]


LGX_PRIM_MAX_M = 15


class LgxPrimQuartet(ctypes.Structure):
    """lgx_prim_quartet: one primitive quartet of caller-computed VRR inputs."""
    _fields_ = [("PA", ctypes.c_double * 3), ("QC", ctypes.c_double * 3),
                ("WP", ctypes.c_double * 3), ("WQ", ctypes.c_double * 3),
                ("oo2z", ctypes.c_double), ("oo2e", ctypes.c_double),
                ("oo2ze", ctypes.c_double), ("roz", ctypes.c_double), ("roe", ctypes.c_double),
                ("two_alpha", ctypes.c_double * 4),
                ("ss", ctypes.c_double * (LGX_PRIM_MAX_M + 1))]


# numpy view of an lgx_prim_quartet array (same field order, all doubles)
PRIM_DTYPE = None
try:
    import numpy as _np
    PRIM_DTYPE = _np.dtype([("PA", "f8", 3), ("QC", "f8", 3), ("WP", "f8", 3), ("WQ", "f8", 3),
                            ("oo2z", "f8"), ("oo2e", "f8"), ("oo2ze", "f8"), ("roz", "f8"),
                            ("roe", "f8"), ("two_alpha", "f8", 4),
                            ("ss", "f8", LGX_PRIM_MAX_M + 1)])
    assert PRIM_DTYPE.itemsize == ctypes.sizeof(LgxPrimQuartet)
except ImportError:  # numpy is optional for the bare ctypes binding
    pass


# Every symbol include/lgx.h declares, with its ctypes signature.
SIGNATURES = {
    "lgx_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]),
    "lgx_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "lgx_set_operator": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]),
    "lgx_set_watchdog": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64]),
    "lgx_set_fock_precision": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "lgx_boys": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_int64, ctypes.c_int,
                                _dp]),
    "lgx_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "lgx_version": (ctypes.c_char_p, []),
    "lgx_compute_shellset": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(LgxShell),
                                            ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                            _dp, ctypes.c_size_t,
                                            ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int)]),
    "lgx_compute_shellset_pairs": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(LgxShell),
                                                  ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                  _dp, _dp, ctypes.c_size_t,
                                                  ctypes.POINTER(ctypes.c_int),
                                                  ctypes.POINTER(ctypes.c_int),
                                                  ctypes.POINTER(ctypes.c_int)]),
    "lgx_compute_primitive_set": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.POINTER(LgxPrimQuartet), ctypes.c_int,
                                                 _dp, _dp, _dp, ctypes.c_size_t,
                                                 ctypes.POINTER(ctypes.c_int),
                                                 ctypes.POINTER(ctypes.c_int)]),
    "lgx_set_basis": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _ip, _ip, _ip, _ip,
                                     _dp, _dp, _dp]),
    "lgx_basis_nbf": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "lgx_set_pair_subset": (ctypes.c_int, [ctypes.c_void_p, _ip, ctypes.c_int64]),
    "lgx_schwarz": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "lgx_compute_batch": (ctypes.c_int, [ctypes.c_void_p, _ip, ctypes.c_int64, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_double, _i64p, _dp,
                                         ctypes.c_size_t, _ip]),
    "lgx_compute_batch_device": (ctypes.c_int, [ctypes.c_void_p, _ip, ctypes.c_int64, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_double, _i64p,
                                                ctypes.c_void_p, ctypes.c_size_t,
                                                ctypes.c_void_p]),
    "lgx_jk": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_double, ctypes.c_int,
                              ctypes.c_double, ctypes.POINTER(LgxJkStats)]),
    "lgx_jk_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                     ctypes.c_double, ctypes.POINTER(LgxJkStats)]),
    "lgx_jk_device_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_double, ctypes.POINTER(LgxJkStats)]),
    "lgx_last_pass_launches": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(LgxLaunchStats),
                                              ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "lgx_jk_grad": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_int,
                                   ctypes.c_double, ctypes.POINTER(LgxJkStats)]),
    "lgx_enforce_unit_normalization": (ctypes.c_int, [ctypes.c_int]),
    "lgx_shell_normalize": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]),
    "lgx_solid_coeff": (ctypes.c_double, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int]),
    "lgx_basis_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, _ip, _dp,
                                      ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int), _ip, _ip, _ip, _ip, _dp,
                                      _dp, _dp]),
    "lgx_water_cluster": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                         _ip, _dp]),
}

_LIB = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads liblgx.so (building it first when absent and nvcc exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("liblgx.so is not built; run __graft_entry__.build()")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class LgxError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("lgx error %d: %s" % (status, msg))
        self.status = status


def check(status: int, ctx=None, what: str = ""):
    if status != LGX_OK:
        msg = what
        if ctx is not None:
            msg = (what + ": " if what else "") + load().lgx_last_error(ctx).decode()
        raise LgxError(status, msg)


def ptr(a, ct=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(ct))
