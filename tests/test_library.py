"""The C-ABI library builds for sm_103a, loads, and exports every symbol the
public header declares; argument errors map to the reference's exception
kinds without touching a GPU."""
import ctypes
import os
import re

import pytest

import paliwa_gb300 as pg
from paliwa_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"\b(paliwa_gb_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert names, "no declarations found"
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert set(_lib.SIGNATURES) <= names


def test_version_and_wavelets():
    lib = _lib.load()
    assert lib.paliwa_gb_version() >= 100
    for name, wid in (("hat", 0), ("biorthogonal", 1), ("fullweighting", 2)):
        assert pg.wavelet_id(name) == wid
    with pytest.raises(pg.OutOfRange):
        pg.wavelet_id("db4")
    with pytest.raises(KeyError):  # std::out_of_range from map::at
        pg.wavelet_id("")


def test_wavelet_tables_match_reference():
    """paliwa/paliwa_wavelets.hpp:15-28, as served by the library."""
    lib = _lib.load()
    for name in ("hat", "biorthogonal", "fullweighting"):
        for direction, table in (
                (1, pg.lifting_wavelet_filter_offsets_and_coefficients),
                (-1, pg.lifting_wavelet_reconstruct_offsets_and_coefficients)):
            n = ctypes.c_int()
            offs = (ctypes.c_int32 * 8)()
            co = (ctypes.c_double * 24)()
            _lib.check(lib.paliwa_gb_wavelet_filters(
                pg.wavelet_id(name), direction, ctypes.byref(n), offs, co))
            got = [(offs[p], tuple(co[3 * p:3 * p + 3])) for p in range(n.value)]
            assert got == [(o, tuple(c)) for o, c in table[name]]


def test_argument_errors_without_gpu():
    lib = _lib.load()
    lv = _lib.i64([2, 2])
    # null grid
    rc = lib.paliwa_gb_hierarchize(None, 0, 2, lv, _lib.i64([0, 0]), lv, 0,
                                   None)
    assert rc == _lib.INVALID_ARGUMENT
    # lmin > level (paliwa_transform.hpp:359-362 asserts)
    rc = lib.paliwa_gb_hierarchize(None, 0, 2, lv, _lib.i64([3, 0]), lv, 0,
                                   None)
    assert rc == _lib.INVALID_ARGUMENT
    assert lib.paliwa_gb_last_error()
    # unknown dtype
    rc = lib.paliwa_gb_hierarchize(None, 9, 2, lv, _lib.i64([0, 0]), lv, 0,
                                   None)
    assert rc == _lib.INVALID_ARGUMENT


def test_batch_and_ct_null_handles_without_gpu():
    """Entry points taking a handle reject a null one before any CUDA call."""
    lib = _lib.load()
    assert lib.paliwa_gb_batch_set_groups(None, 2) == _lib.INVALID_ARGUMENT
    assert lib.paliwa_gb_batch_hierarchize(None, None) == \
        _lib.INVALID_ARGUMENT
    assert lib.paliwa_gb_ct_combine(None, None, None) == \
        _lib.INVALID_ARGUMENT
    lib.paliwa_gb_batch_destroy(None)  # no-op
    lib.paliwa_gb_ct_destroy(None)
