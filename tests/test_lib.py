"""The C-ABI library loads without a GPU and exports every symbol the public
header declares (no compute calls here)."""
import ctypes as C
import os

from csim_gb300 import _lib


def test_library_exports_every_header_symbol():
    syms = _lib.header_symbols()
    assert len(syms) > 40
    missing = [s for s in syms if not hasattr(_lib.lib, s)]
    assert not missing, missing


def test_bindings_cover_the_header():
    assert set(_lib.header_symbols()) <= set(_lib.SIGNATURES) | {"csg_last_error"}


def test_version_and_errors_without_gpu():
    assert "sm_103a" in _lib.version()
    # a null-argument call fails cleanly with a message, no device needed
    try:
        _lib.call("csg_sync", None)
    except _lib.CsgError as e:
        assert e.code == -1 and "null" in str(e)
    else:
        raise AssertionError("csg_sync(NULL) must fail")


def test_built_for_sm103a():
    lib = _lib.LIB_PATH
    assert os.path.exists(lib)
