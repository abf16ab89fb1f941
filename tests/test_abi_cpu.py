"""C-ABI checks that need no GPU: the library builds, loads, and exports every
entry point that include/kwave_gb300.h declares, with matching ctypes
prototypes in kwave_gb300._lib."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "kwave_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int32_t|const char\*)\s+(kw_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib

    return _lib.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "kw_plan_create" in syms and "kw_plan_run" in syms and "kw_last_error" in syms
    assert len(syms) >= 15


def test_library_exports_every_declared_symbol(lib):
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_ctypes_prototypes_cover_header(lib):
    from kwave_gb300 import _lib

    assert set(declared_symbols()) == set(_lib.EXPORTED_SYMBOLS)


def test_version_and_error_string(lib):
    assert lib.kw_version() == 100
    assert isinstance(lib.kw_last_error(), bytes)


def test_plan_create_rejects_bad_descriptors(lib):
    import ctypes as C

    from kwave_gb300 import _lib

    d = _lib.KwGridDesc()
    d.ndim = 4
    h = C.c_void_p()
    assert lib.kw_plan_create(C.byref(d), C.byref(h)) == _lib.KW_ERR_UNSUPPORTED
    assert b"2-D and 3-D" in lib.kw_last_error()
    d.ndim = 2
    d.shape[0], d.shape[1] = 64, 22  # 22 = 2 * 11: prime factor above 7
    d.Nt = 10
    d.spacing[0] = d.spacing[1] = 1e-4
    d.dt = 1e-8
    assert lib.kw_plan_create(C.byref(d), C.byref(h)) == _lib.KW_ERR_UNSUPPORTED
    assert b"prime factor" in lib.kw_last_error()
    d.shape[1] = 60
    d.Nt = 0
    assert lib.kw_plan_create(C.byref(d), C.byref(h)) == _lib.KW_ERR_INVALID
