"""ctypes binding of libwtgpu.so (declarations: include/wtgpu.h).

The library is the only compute path: if it is missing or cannot be loaded,
every call raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import warnings
from pathlib import Path

# the in-tree build (the only library this package loads)
LIB_PATH = Path(__file__).resolve().parent / "libwtgpu.so"

WTG_OK = 0
WTG_EINVAL = -1
WTG_ENOMEM = -2
WTG_ECUDA = -3
WTG_ENODEV = -4
WTG_EUNSUPPORTED = -6

PT_NOT_CONVERGED = 1
PT_SINGULAR = 2
PT_NONFINITE = 4
PT_TIMEOUT = 8

PREC_FP64 = 0
PREC_MIXED = 1

# test-only switches of wtg_test_option
TEST_FP64_GLOBAL_INVERSE = 1
TEST_MIXED_SPIN_LIMIT = 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i32p = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)
_vp = C.c_void_p

# name -> (restype, argtypes); mirrors include/wtgpu.h
SIGNATURES = {
    "wtg_model_create": (C.c_int, [C.c_int, C.c_int, _ip, _dp, _ip, C.c_int, C.c_int, C.POINTER(_vp)]),
    "wtg_model_destroy": (C.c_int, [_vp]),
    "wtg_model_ndim": (C.c_int, [_vp]),
    "wtg_model_set_loto": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp, C.c_double]),
    "wtg_ham_qlayer2qlayer": (C.c_int, [_vp, _dp, _dp, _dp]),
    "wtg_surfgreen_1985": (C.c_int, [C.c_int, C.c_double, C.c_double, _dp, _dp, C.c_double, C.c_int,
                                      _dp, _dp, _dp, _ip, _ip]),
    "wtg_surface_spectrum": (C.c_int, [_vp, C.c_int, _dp, C.c_int, _dp, C.c_double, C.c_double, C.c_int,
                                        C.c_int, _ip, C.c_int, _ip, C.c_int, C.c_int,
                                        _dp, _dp, _dp, _i32p, _u8p]),
    "wtg_surface_spectrum_device": (C.c_int, [_vp, C.c_int, _vp, C.c_int, _vp, C.c_double, C.c_double,
                                               C.c_int, C.c_int, _ip, C.c_int, _ip, C.c_int, C.c_int,
                                               _vp, _vp, _vp, _vp, _vp, _vp]),
    "wtg_mat_mul": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int]),
    "wtg_inv": (C.c_int, [C.c_int, _dp, C.c_int, _ip]),
    "wtg_surface_spectrum_spin": (C.c_int, [_vp, C.c_int, _dp, C.c_int, _dp, C.c_double, C.c_double,
                                             C.c_int, C.c_int, _ip, C.c_int, _ip, C.c_int, C.c_int,
                                             _dp, _dp, _dp, _dp, _i32p, _u8p]),
    "wtg_model_profile": (C.c_int, [_vp, C.c_int]),
    "wtg_model_profile_read": (C.c_int, [_vp, _dp, _dp, C.POINTER(C.c_longlong), _ip]),
    "wtg_probe_fp64_peak": (C.c_int, [_dp]),
    "wtg_probe_dmma_peak": (C.c_int, [_dp]),
    "wtg_surfgreen_batch_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, _vp, C.c_int, _vp, C.c_double,
                                               C.c_double, C.c_int, C.c_int, _ip, C.c_int, _ip, C.c_int,
                                               _vp, _vp, _vp, _vp, _vp, _vp]),
    "wtg_engine_create": (C.c_int, [C.c_int, C.POINTER(_vp), C.c_int, C.c_int, _ip, _ip, _ip, _ip,
                                     C.POINTER(_vp)]),
    "wtg_engine_destroy": (C.c_int, [_vp]),
    "wtg_engine_info": (C.c_int, [_vp, C.POINTER(C.c_longlong), _ip, C.POINTER(C.c_longlong)]),
    "wtg_engine_set_graphs": (C.c_int, [_vp, C.c_int]),
    "wtg_engine_graph_info": (C.c_int, [_vp, _ip, C.POINTER(C.c_longlong)]),
    "wtg_tile_set": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "wtg_tile_get": (C.c_int, [C.c_int, C.c_int, _ip, _ip]),
    "wtg_engine_run": (C.c_int, [_vp, C.c_int, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                  _dp, _dp, _dp, _i32p, _u8p]),
    "wtg_batch_spectrum": (C.c_int, [C.c_int, C.POINTER(_vp), C.c_int, _ip, _dp, _dp, _dp, C.c_double,
                                      C.c_int, _ip, _ip, _ip, _ip, C.c_int, C.c_int, _dp, _dp, _dp,
                                      _i32p, _u8p]),
    "wtg_jdos_kpath": (C.c_int, [C.c_int, C.c_int, _dp, _dp]),
    "wtg_jdos_kplane": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_double, _dp]),
    "wtg_test_option": (C.c_int, [C.c_int, C.c_int]),
    "wtg_last_error": (C.c_int, [C.c_char_p, C.c_int]),
    "wtg_device_info": (C.c_int, [C.c_char_p, C.c_int]),
}

_lib = None


class WtgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"wtg error {code}: {msg}")
        self.code = code


def load() -> C.CDLL:
    """Load the in-tree library (building it is the caller's step)."""
    global _lib
    if _lib is not None:
        return _lib
    p = LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is not built; call wannier_tools_gb300.build() first "
                           "(there is no CPU fallback for this path)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    if os.environ.get("WTG_TILES", "1") != "0":
        _install_tiles(lib)
    return lib


def _install_tiles(lib) -> None:
    """Put the autotuner's table (tiles.json beside this file) for the current
    device into the library; nothing without a device or without an entry."""
    buf = C.create_string_buffer(256)
    if lib.wtg_device_info(buf, 256) != 0:
        return
    from .autotune import FORMS, TABLE, device_key, entries_for
    if not TABLE.exists():
        return
    table = json.loads(TABLE.read_text())
    for form, ent in entries_for(table, device_key(buf.value.decode())).items():
        for ndim, v in ent.items():
            if lib.wtg_tile_set(FORMS[form], ndim, v) < 0:     # an entry this build rejects
                warnings.warn(f"tiles.json: {form} Ndim {ndim} = {v} rejected: {last_error()}")


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().wtg_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int) -> int:
    """Raise on hard errors (rc < 0); return rc (>= 0: count of flagged points)."""
    if rc < 0:
        raise WtgError(rc, last_error())
    return rc
