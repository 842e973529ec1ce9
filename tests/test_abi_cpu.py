"""The C-ABI library builds, loads and exports every symbol include/*.h
declares; error paths that need no GPU return their codes (no compute)."""
import ctypes as C
import re

import pytest

from wannier_tools_gb300 import _lib

from .conftest import ROOT, has_gpu


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(re.findall(r"\b(wtg_\w+)\s*\(", text))
    return names


def test_header_declares_the_abi():
    names = declared_symbols()
    for required in ("wtg_model_create", "wtg_model_destroy", "wtg_ham_qlayer2qlayer",
                     "wtg_surfgreen_1985", "wtg_surface_spectrum", "wtg_surface_spectrum_device",
                     "wtg_last_error", "wtg_device_info"):
        assert required in names


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in sorted(declared_symbols()) if not hasattr(built_lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    assert declared_symbols() == set(_lib.SIGNATURES)


def test_bad_arguments_without_compute(built_lib):
    lib = built_lib
    assert lib.wtg_surfgreen_1985(0, 0.0, 0.0, None, None, 0.0, 0, None, None, None, None, None) == _lib.WTG_EINVAL
    assert lib.wtg_model_destroy(None) == _lib.WTG_EINVAL
    assert lib.wtg_model_ndim(None) == _lib.WTG_EINVAL
    assert "null model" in _lib.last_error()
    h = C.c_void_p()
    assert lib.wtg_model_create(0, 1, None, None, None, 1, 10, C.byref(h)) == _lib.WTG_EINVAL


@pytest.mark.skipif(has_gpu(), reason="checks the no-device error path")
def test_no_device_is_reported(built_lib):
    import numpy as np
    irv = np.zeros((1, 3), np.int32)
    hr = np.zeros(2, np.float64)
    h = C.c_void_p()
    rc = built_lib.wtg_model_create(1, 1, irv.ctypes.data_as(C.POINTER(C.c_int)),
                                    hr.ctypes.data_as(C.POINTER(C.c_double)), None, 1, 10, C.byref(h))
    assert rc == _lib.WTG_ENODEV
    assert _lib.last_error()
    with pytest.raises(_lib.WtgError):
        _lib.check(rc)
