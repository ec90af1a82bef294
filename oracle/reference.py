"""The reference itself, compiled here -- TEST INFRASTRUCTURE.

``make -C oracle ref`` compiles the unmodified paliwa headers from the
reference checkout (paliwa_transform.hpp, paliwa_domains.hpp,
paliwa_wavelets.hpp, paliwa_dimensions.hpp, paliwa_utils.hpp) against the
serial DDC/Kokkos stand-ins in ``oracle/ref_shim/`` into
``oracle/_ref/libpaliwa_ref.so`` (entry points in ``oracle/ref_driver.cpp``).
Only the CPU tests use it, to hold the oracle's restatement equal to the
reference; the checkout does not exist where the GPU tests run, so
``available()`` is False there and those tests skip.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "libpaliwa_ref.so")
REFERENCE = os.environ.get("PALIWA_REFERENCE", "/root/reference")
_lib = None


def available():
    return os.path.isdir(os.path.join(REFERENCE, "paliwa"))


def build():
    subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF={REFERENCE}"],
                   check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.ref_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _longs(v):
    v = [int(x) for x in v]
    return (ctypes.c_long * max(1, len(v)))(*v)


def _check(rc):
    if rc == 0:
        return
    msg = lib().ref_last_error().decode()
    if rc == 1:
        raise ValueError(msg)
    if rc == 3:
        raise KeyError(msg)
    raise RuntimeError(msg)


def _dtype(a):
    if a.dtype == np.float64:
        return 0
    if a.dtype == np.float32:
        return 1
    raise TypeError("float64 or float32 grids")


def _filters(filters):
    offs = (ctypes.c_int * max(1, len(filters)))(*[int(o) for o, _ in filters])
    co = (ctypes.c_double * max(1, 3 * len(filters)))(
        *[float(c) for _, f in filters for c in f])
    return offs, co


def hierarchize(grid, level, minimum_level, maximum_level, wavelet="hat",
                forward=True):
    """paliwa::hierarchize / dehierarchize on a C-contiguous grid."""
    assert grid.flags.c_contiguous
    _check(lib().ref_hierarchize(
        grid.ctypes.data_as(ctypes.c_void_p), _dtype(grid), len(level),
        _longs(level), _longs(minimum_level), _longs(maximum_level),
        wavelet.encode(), 1 if forward else 0))
    return grid


def dehierarchize(grid, level, minimum_level, maximum_level, wavelet="hat"):
    return hierarchize(grid, level, minimum_level, maximum_level, wavelet,
                       forward=False)


def transform_in(grid, level, maximum_level, dim, levels, filters,
                 front=None, extents=None):
    """paliwa::transform_in<Dim> (full-grid overload) on the whole lattice,
    or on the window (front uids, extents) of it that ``grid`` holds."""
    offs, co = _filters(filters)
    _check(lib().ref_transform_in(
        grid.ctypes.data_as(ctypes.c_void_p), _dtype(grid), len(level),
        _longs(level), _longs(maximum_level),
        None if front is None else _longs(front),
        None if extents is None else _longs(extents), int(dim),
        _longs(levels), len(levels), offs, co, len(filters)))
    return grid


def transform_outputs(grid, level, maximum_level, front, extents, dim, levels,
                      filters, out_front, out_extents, out_strides, mode=0):
    """paliwa::transform_in<Dim> restricted-output overload on a window buffer
    (mode 0 Direct, 1 PackedPasses, 2 PackedPoles)."""
    offs, co = _filters(filters)
    _check(lib().ref_transform_outputs(
        grid.ctypes.data_as(ctypes.c_void_p), _dtype(grid), len(level),
        _longs(level), _longs(maximum_level), _longs(front), _longs(extents),
        int(dim), _longs(levels), len(levels), offs, co, len(filters),
        _longs(out_front), _longs(out_extents), _longs(out_strides),
        int(mode)))
    return grid


def transform_bounds(outputs, level, maximum_level, levels, offsets):
    """paliwa::transform_bounds: (bounds per level 0..level, writes per
    (level index, pass)) as lists of (min, max)."""
    n, nf = len(levels), len(offsets)
    bounds = (ctypes.c_long * (2 * (level + 1)))()
    writes = (ctypes.c_long * max(1, 2 * n * nf))()
    o = (ctypes.c_int * max(1, nf))(*[int(x) for x in offsets])
    _check(lib().ref_transform_bounds(
        ctypes.c_long(outputs[0]), ctypes.c_long(outputs[1]),
        ctypes.c_long(level), ctypes.c_long(maximum_level), _longs(levels),
        n, o, nf, bounds, writes))
    b = [(bounds[2 * i], bounds[2 * i + 1]) for i in range(level + 1)]
    w = [[(writes[2 * (i * nf + p)], writes[2 * (i * nf + p) + 1])
          for p in range(nf)] for i in range(n)]
    return b, w


def covering_periodic_bounds(indices, period):
    out = (ctypes.c_long * 2)()
    _check(lib().ref_covering_periodic_bounds(
        _longs(indices), len(indices), ctypes.c_long(period), out))
    return out[0], out[1]


def pole_pass_segments(writes, origin, level, maximum_level, pass_level):
    n = ctypes.c_int()
    cap = 64
    out = (ctypes.c_int * (5 * cap))()
    _check(lib().ref_pole_pass_segments(
        ctypes.c_long(writes[0]), ctypes.c_long(writes[1]),
        ctypes.c_long(origin), level, maximum_level, pass_level, cap,
        ctypes.byref(n), out))
    return [tuple(out[5 * i:5 * i + 5]) for i in range(min(n.value, cap))]


def level_domain(kind, level, finest_level, lbound=None):
    """kind 0: strided_domain_from_level, 1: the hierarchical subspace
    domain; returns (front, extents, strides)."""
    d = len(level)
    f, e, s = ((ctypes.c_long * d)() for _ in range(3))
    _check(lib().ref_level_domain(
        kind, d, _longs(level), _longs(finest_level),
        _longs(lbound if lbound is not None else [0] * d), f, e, s))
    return tuple(f), tuple(e), tuple(s)


def restrict_strided_with_discrete(domain, box_front, box_extents):
    front, ext, st = domain
    d = len(front)
    out = (ctypes.c_long * (3 * d))()
    _check(lib().ref_restrict_strided_with_discrete(
        d, _longs(front), _longs(ext), _longs(st), _longs(box_front),
        _longs(box_extents), out))
    return tuple(out[:d]), tuple(out[d:2 * d]), tuple(out[2 * d:])


def required_transform_domain(forward, level, minimum_level, maximum_level,
                              local_front, local_extent, wavelet):
    cap = 1 << 16
    out = (ctypes.c_long * cap)()
    n = ctypes.c_long()
    _check(lib().ref_required_transform_domain(
        1 if forward else 0, ctypes.c_long(level), ctypes.c_long(minimum_level),
        ctypes.c_long(maximum_level), ctypes.c_long(local_front),
        ctypes.c_long(local_extent), wavelet.encode(), cap, ctypes.byref(n),
        out))
    return list(out[:n.value])


def periodic_unit_interval(n):
    cap = max(1, int(n))
    out = (ctypes.c_double * cap)()
    cnt = ctypes.c_long()
    _check(lib().ref_periodic_unit_interval(ctypes.c_long(n), cap,
                                            ctypes.byref(cnt), out))
    return list(out[:cnt.value])


def hierarchical_subspaces(nodal_level):
    d = len(nodal_level)
    cap = 1
    for l in nodal_level:
        cap *= int(l) + 1
    out = (ctypes.c_long * (cap * d))()
    cnt = ctypes.c_long()
    _check(lib().ref_hierarchical_subspaces(d, _longs(nodal_level), cap,
                                            ctypes.byref(cnt), out))
    return [tuple(out[i * d:(i + 1) * d]) for i in range(cnt.value)]


def restrict_periodic_bounds_2d(front, extents, strides, bounds, period):
    """paliwa::restrict_periodic_bounds along dimension 0 of a 2D strided
    domain: a list of (front, extents, strides) parts."""
    n = ctypes.c_int()
    out = (ctypes.c_long * 12)()
    _check(lib().ref_restrict_periodic_bounds(
        _longs(front), _longs(extents), _longs(strides),
        ctypes.c_long(bounds[0]), ctypes.c_long(bounds[1]),
        ctypes.c_long(period), ctypes.byref(n), out))
    return [(tuple(out[6 * i:6 * i + 2]), tuple(out[6 * i + 2:6 * i + 4]),
             tuple(out[6 * i + 4:6 * i + 6])) for i in range(n.value)]


def for_each_transform_index(bounds, maximum_level):
    flat = [v for b in bounds for v in b]
    cap = 1 << 16
    out = (ctypes.c_long * cap)()
    n = ctypes.c_long()
    _check(lib().ref_for_each_transform_index(
        _longs(flat), len(bounds), ctypes.c_long(maximum_level), cap,
        ctypes.byref(n), out))
    return list(out[:n.value])
