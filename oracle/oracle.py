"""CPU oracle for the paliwa hierarchization transform -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module. It restates the reference algorithm on
the CPU so that the GPU product can be checked against it; it is never the
path that is measured as the GPU result and never a fallback for it.

Transform arithmetic lives in ``paliwa_oracle.hpp`` (C++, built by the
Makefile beside it into ``_build/liboracle.so``). This module wraps it with
numpy and adds pure-Python restatements of the reference's index maps and of
its combination-technique driver, each citing the reference file:line it
follows. The reference itself cannot be compiled here (DDC, Kokkos, MPI and
GoogleTest are absent); parity is pinned to its tests' known answers and to
its in-test 1D reference loop (see tests/golden/).
"""
from __future__ import annotations

import ctypes
import itertools
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

WAVELETS = {"hat": 0, "biorthogonal": 1, "fullweighting": 2}

# paliwa/paliwa_wavelets.hpp:15-28
FORWARD = {
    "hat": [(1, (-0.5, 1.0, -0.5))],
    "biorthogonal": [(1, (-0.5, 1.0, -0.5)), (0, (0.25, 1.0, 0.25))],
    "fullweighting": [(0, (0.25, 0.5, 0.25)), (1, (-0.5, 1.0, -0.5))],
}
INVERSE = {
    "hat": [(1, (0.5, 1.0, 0.5))],
    "biorthogonal": [(0, (-0.25, 1.0, -0.25)), (1, (0.5, 1.0, 0.5))],
    "fullweighting": [(1, (0.5, 1.0, 0.5)), (0, (-0.5, 2.0, -0.5))],
}


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_last_error.restype = ctypes.c_char_p
        L.oracle_max_threads.restype = ctypes.c_int
        L.oracle_transform_in.restype = ctypes.c_int
        L.oracle_hierarchize.restype = ctypes.c_int
        L.oracle_transform_in_window.restype = ctypes.c_int
        _lib = L
    return _lib


def _longs(v):
    return (ctypes.c_long * len(v))(*[int(x) for x in v])


def _check(rc):
    if rc == 0:
        return
    msg = lib().oracle_last_error().decode()
    if rc == 1:
        raise ValueError(msg)
    if rc == 3:
        raise KeyError(msg)
    raise RuntimeError(msg)


def _dtype_code(a):
    if a.dtype == np.float64:
        return 0
    if a.dtype == np.float32:
        return 1
    raise TypeError("oracle grids are float64 or float32")


def max_threads():
    return lib().oracle_max_threads()


def set_threads(n):
    lib().oracle_set_threads(int(n))


def transform_in(grid, level, maximum_level, dim, levels, filters, mode=0):
    """In-place transform_in along ``dim`` (paliwa_transform.hpp:215-251)."""
    assert grid.flags.c_contiguous
    offs = (ctypes.c_int * max(1, len(filters)))(*[int(o) for o, _ in filters])
    co = (ctypes.c_double * max(1, 3 * len(filters)))(
        *[float(c) for _, f in filters for c in f])
    _check(lib().oracle_transform_in(
        grid.ctypes.data_as(ctypes.c_void_p), _dtype_code(grid), len(level),
        _longs(level), _longs(maximum_level), int(dim), _longs(levels or [0]),
        len(levels), offs, co, len(filters), int(mode)))
    return grid


def transform_in_window(grid, level, maximum_level, front, dim, levels,
                        filters):
    """transform_in along ``dim`` on a chunk holding the window of the level
    lattice whose front uids are ``front`` and whose extents are
    ``grid.shape`` (the reference's checked lifting passes,
    paliwa_transform.hpp:24-51 with CheckBounds, :224-247)."""
    assert grid.flags.c_contiguous
    offs = (ctypes.c_int * max(1, len(filters)))(*[int(o) for o, _ in filters])
    co = (ctypes.c_double * max(1, 3 * len(filters)))(
        *[float(c) for _, f in filters for c in f])
    _check(lib().oracle_transform_in_window(
        grid.ctypes.data_as(ctypes.c_void_p), _dtype_code(grid), len(level),
        _longs(level), _longs(maximum_level), _longs(front),
        _longs(grid.shape), int(dim), _longs(levels or [0]), len(levels),
        offs, co, len(filters)))
    return grid


def hierarchize(grid, level, minimum_level, maximum_level, wavelet="hat",
                forward=True, mode=0):
    """In-place (de)hierarchize over all dims (paliwa_transform.hpp:401-431)."""
    assert grid.flags.c_contiguous
    if wavelet not in WAVELETS:
        raise KeyError(wavelet)  # std::map::at -> std::out_of_range
    assert grid.shape == tuple(1 << int(l) for l in level)
    _check(lib().oracle_hierarchize(
        grid.ctypes.data_as(ctypes.c_void_p), _dtype_code(grid), len(level),
        _longs(level), _longs(minimum_level), _longs(maximum_level),
        WAVELETS[wavelet], 1 if forward else 0, int(mode)))
    return grid


def dehierarchize(grid, level, minimum_level, maximum_level, wavelet="hat",
                  mode=0):
    return hierarchize(grid, level, minimum_level, maximum_level, wavelet,
                       forward=False, mode=mode)


# --------------------------------------------------------------------------
# Index maps (paliwa/paliwa_domains.hpp), as (front, extents, strides) tuples
# in finest-level uid coordinates.


def strided_domain_from_level(level, finest_level, lbound=None):
    """paliwa_domains.hpp:33-49: extents 2^l, strides 2^(L-l), front lbound."""
    d = len(level)
    front = tuple(lbound) if lbound is not None else (0,) * d
    extents = tuple(1 << int(l) for l in level)
    strides = tuple(1 << (int(L) - int(l)) for l, L in zip(level, finest_level))
    return front, extents, strides


def strided_hierarchical_domain_from_level(level, finest_level, lbound=None):
    """paliwa_domains.hpp:51-83: 2^(l-1) odd points, start 2^(L-l), stride
    2^(L-l+1); level 0 is the single point at the origin."""
    d = len(level)
    lb = tuple(lbound) if lbound is not None else (0,) * d
    front, ext, st = [], [], []
    for l, L, b in zip(level, finest_level, lb):
        l, L = int(l), int(L)
        if l == 0:
            ext.append(1)
            front.append(b)
        else:
            ext.append(1 << (l - 1))
            front.append(b + (1 << (L - l)))
        st.append(1 << (L - l + 1))
    return tuple(front), tuple(ext), tuple(st)


def odd_strided_domain_from_domain(domain, dim):
    """paliwa_domains.hpp:85-98 (lbound defaults to the origin)."""
    front, ext, st = (list(x) for x in domain)
    new_front = [0] * len(front)
    new_front[dim] = st[dim]
    st[dim] *= 2
    ext[dim] //= 2
    return tuple(new_front), tuple(ext), tuple(st)


def even_strided_domain_from_domain(domain, dim):
    """paliwa_domains.hpp:100-111 (lbound defaults to the origin)."""
    front, ext, st = (list(x) for x in domain)
    st[dim] *= 2
    ext[dim] //= 2
    return (0,) * len(front), tuple(ext), tuple(st)


def domain_points(domain):
    front, ext, st = domain
    axes = [range(f, f + e * s, s) for f, e, s in zip(front, ext, st)]
    return list(itertools.product(*axes))


# --------------------------------------------------------------------------
# Combination technique driver, restated from the reference's test driver
# test/test_paliwa_combination_technique.cpp:77-340 and paliwa_utils.hpp:9-26.


def iterate_hierarchical_subspaces(nodal_level):
    """paliwa_utils.hpp:9-26: every s with 0 <= s_i <= l_i, lexicographic."""
    return list(itertools.product(*[range(int(l) + 1) for l in nodal_level]))


def subspace_counts(all_levels):
    """test_paliwa_combination_technique.cpp:177-192."""
    counts = {}
    for lv in all_levels:
        for s in iterate_hierarchical_subspaces(lv):
            counts[s] = counts.get(s, 0) + 1
    return counts


def kept_subspaces(all_levels):
    """Only subspaces present in more than one component grid are kept
    (test_paliwa_combination_technique.cpp:212-225), in std::map order
    (lexicographic on the level tuple)."""
    return sorted(s for s, c in subspace_counts(all_levels).items() if c > 1)


def subspace_size(s):
    return math.prod(1 if l == 0 else 1 << (l - 1) for l in s)


def combine(grids, all_levels, coefficients, maximum_level, subspaces):
    """test_paliwa_combination_technique.cpp:256-290: for every grid and every
    kept subspace contained in it, subspace += coefficient * grid on the
    subspace's points. Returns one float64 array per subspace (in the order of
    ``subspaces``), in the subspace domain's row-major order."""
    out = []
    for s in subspaces:
        acc = np.zeros([1 if l == 0 else 1 << (l - 1) for l in s])
        for g, lv, c in zip(grids, all_levels, coefficients):
            if any(si > li for si, li in zip(s, lv)):
                continue
            acc += c * g[subspace_slices(s, lv)]
        out.append(acc)
    return out


def subspace_slices(s, lv):
    """Slices selecting hierarchical subspace s inside a grid at level lv:
    along each dim, compact indices start 2^(lv-s) (0 at s=0), step 2^(lv-s+1)."""
    sl = []
    for si, li in zip(s, lv):
        if si == 0:
            sl.append(slice(0, 1))
        else:
            sl.append(slice(1 << (li - si), None, 1 << (li - si + 1)))
    return tuple(sl)


def scatter(subspace_values, subspaces, maximum_level):
    """test_paliwa_combination_technique.cpp:293-318: add every kept subspace
    into a zeroed full grid at the maximum level."""
    full = np.zeros([1 << int(L) for L in maximum_level])
    for v, s in zip(subspace_values, subspaces):
        full[subspace_slices(s, maximum_level)] += v
    return full


# --------------------------------------------------------------------------
# The same combine and restriction, vectorised per grid, for full-size
# schemes (thousands of grids): every point of a grid at level lv belongs to
# exactly one hierarchical subspace s <= lv; along an axis, compact index
# i > 0 lies in s = lv - ctz(i) at position i >> (lv - s + 1), and i = 0 in
# s = 0. The sparse grid is laid out as the library lays it out: the kept
# subspaces in lexicographic order, each dense over the extents of
# strided_hierarchical_domain_from_level(s, L) (paliwa_domains.hpp:51-83),
# concatenated.


def sparse_offsets(subspaces):
    """First sparse point of each subspace (in the given order) and the total."""
    offsets, total = {}, 0
    for s in subspaces:
        offsets[tuple(s)] = total
        total += subspace_size(s)
    return offsets, total


def _axis_subspace(l):
    i = np.arange(1 << l, dtype=np.int64)
    s = np.zeros_like(i)
    pos = np.zeros_like(i)
    nz = i > 0
    ctz = np.zeros_like(i)
    v = i[nz]
    c = np.zeros_like(v)
    while True:
        odd = (v & 1) == 1
        if odd.all():
            break
        c += ~odd
        v = np.where(odd, v, v >> 1)
    ctz[nz] = c
    s[nz] = l - ctz[nz]
    pos[nz] = i[nz] >> (l - s[nz] + 1)
    ext = np.where(s == 0, 1, 1 << np.maximum(s - 1, 0))
    return s, pos, ext


def grid_sparse_index(lv, offsets):
    """Sparse index of every point of a grid at level ``lv`` (row-major,
    int64), -1 where the point's subspace is not kept."""
    d = len(lv)
    axes = [_axis_subspace(int(l)) for l in lv]
    shape = [1 << int(l) for l in lv]
    # Local subspace table: multi-index s (0 <= s_k <= lv_k) -> offset or -1.
    dims = [int(l) + 1 for l in lv]
    table = np.full(math.prod(dims), -1, dtype=np.int64)
    for flat, s in enumerate(itertools.product(*[range(n) for n in dims])):
        table[flat] = offsets.get(s, -1)
    def bcast(a, k):
        sh = [1] * d
        sh[k] = a.shape[0]
        return a.reshape(sh)
    local = np.zeros(shape, dtype=np.int64)
    for k in range(d):
        local = local * dims[k] + bcast(axes[k][0], k)
    base = table[local]
    inner = np.zeros(shape, dtype=np.int64)
    stride = np.ones(shape, dtype=np.int64)
    for k in reversed(range(d)):
        inner = inner + bcast(axes[k][1], k) * stride
        stride = stride * bcast(axes[k][2], k)
    return np.where(base >= 0, base + inner, -1)


def combine_sparse(grids, all_levels, coefficients, offsets, total):
    """test_paliwa_combination_technique.cpp:256-290, as one flat float64
    vector: grids in order, sparse += coefficient * grid on every kept point
    (the product rounded, then the sum, as ``acc += c * g``)."""
    sparse = np.zeros(total)
    for g, lv, c in zip(grids, all_levels, coefficients):
        idx = grid_sparse_index(lv, offsets).ravel()
        keep = idx >= 0
        sparse[idx[keep]] += float(c) * np.asarray(g, np.float64).ravel()[keep]
    return sparse


def restrict_sparse(grid, lv, sparse, offsets):
    """The restriction of the combined sparse grid back into one component
    grid: every kept point takes the combined value (rounded to the grid's
    storage type); the other points are left as they are."""
    idx = grid_sparse_index(lv, offsets).ravel()
    keep = idx >= 0
    flat = grid.reshape(-1)
    flat[keep] = sparse[idx[keep]].astype(grid.dtype)
    return grid
