"""CPU oracle of the restricted-output transform -- TEST INFRASTRUCTURE.

Only ``tests/`` may import this module: it checks the GPU product and the
library's host planner, and is never the measured or shipped path.

Pure-Python / numpy restatement of the reference's restricted-output
transform along one axis:

* ``transform_bounds``      paliwa/paliwa_domains.hpp:316-452
* ``transform_indices``     paliwa/paliwa_domains.hpp:454-486
* ``covering_periodic_bounds`` paliwa/paliwa_domains.hpp:488-503
* ``pole_pass_segments``    paliwa/paliwa_domains.hpp:505-538
* ``restrict_periodic_bounds`` paliwa/paliwa_domains.hpp:540-567 (one axis)
* ``transform_outputs``     paliwa/paliwa_transform.hpp:258-331 (Direct
  execution of ``detail::transform_with_remote`` with grid == remote) and the
  lifting pass :24-51, over a periodic window buffer (below).

Bounds are ``None`` (empty) or a pair ``(min, max)`` of finest-level uids,
``min > max`` wrapping around the period.

Window buffers: the grid is given as a dense row-major array whose axis d
holds the uids ``(front[d] + k * spacing[d]) mod 2^L[d]`` for
``k < shape[d]``, ``spacing[d] = 2^(L[d] - level[d])``. A full grid is the
window with front 0 and 2^level points; a window may wrap around the period,
so one buffer can hold outputs and the periodic halo they need.
"""
from __future__ import annotations

import numpy as np


class _Interval:
    """Unwrapped inclusive interval; empty when lo > hi
    (detail::LevelInterval, paliwa_domains.hpp:324-356)."""

    __slots__ = ("lo", "hi")

    def __init__(self, lo=1, hi=0):
        self.lo, self.hi = lo, hi

    def empty(self):
        return self.lo > self.hi

    def aligned(self, stride, offset):
        if self.empty():
            return _Interval()
        return _Interval(self.lo + (offset - self.lo) % stride,
                         self.hi - (self.hi - offset) % stride)

    def include(self, other):
        if other.empty():
            return
        if self.empty():
            self.lo, self.hi = other.lo, other.hi
        else:
            self.lo = min(self.lo, other.lo)
            self.hi = max(self.hi, other.hi)

    def periodic(self, period, stride, offset):
        if self.empty():
            return None
        if (self.hi - self.lo) // stride + 1 >= period // stride:
            return (offset, period - stride + offset)
        return (self.lo % period, self.hi % period)


def transform_bounds(outputs, level, maximum_level, levels, filters,
                     visit=None):
    """Exact write set of every (level index, pass) and the required input
    bounds per hierarchical level 0..level (paliwa_domains.hpp:357-452).
    ``filters`` is a list of (offset, coefficients); coefficients are not
    read. Raises ValueError where the reference throws std::invalid_argument.
    """
    levels = [int(l) for l in levels]
    if len(levels) > 1:
        step = levels[1] - levels[0]
        if step not in (1, -1):
            raise ValueError("Transform levels must be consecutive")
        for a, b in zip(levels, levels[1:]):
            if b - a != step:
                raise ValueError(
                    "Transform levels must be monotone and consecutive")
    period = 1 << maximum_level

    def lstride(h):
        return period if h == 0 else 2 << (maximum_level - h)

    def loffset(h):
        return 0 if h == 0 else 1 << (maximum_level - h)

    out = _Interval()
    if outputs is not None:
        lo, hi = outputs
        out = _Interval(lo, hi + (period if lo > hi else 0))
    req = [out.aligned(lstride(h), loffset(h)) for h in range(level + 1)]
    for i in reversed(range(len(levels))):
        l = levels[i]
        if l < 1 or l > level:
            raise ValueError("Invalid transform level")
        s = 1 << (maximum_level - l)
        for p in reversed(range(len(filters))):
            off = int(filters[p][0])
            if off not in (0, 1):
                raise ValueError("Filter offset not supported")
            if off == 0:
                writes = _Interval()
                for h in range(l):
                    writes.include(req[h])
            else:
                writes = _Interval(req[l].lo, req[l].hi)
            if visit is not None:
                visit(i, p, writes.periodic(period, 2 * s, off * s))
            if writes.empty():
                continue
            nb = _Interval(writes.lo - s, writes.hi + s)
            if off == 0:
                req[l].include(nb.aligned(2 * s, s))
            else:
                for h in range(l):
                    req[h].include(nb.aligned(lstride(h), loffset(h)))
    return [req[h].periodic(period, lstride(h), loffset(h))
            for h in range(level + 1)]


def transform_indices(bounds, maximum_level):
    """Every uid of the per-level bounds (for_each_transform_index,
    paliwa_domains.hpp:454-469), in visiting order."""
    period = 1 << maximum_level
    out = []
    for h, b in enumerate(bounds):
        if b is None:
            continue
        stride = period if h == 0 else 2 << (maximum_level - h)
        last = b[1] + (period if b[0] > b[1] else 0)
        out.extend(x % period for x in range(b[0], last + 1, stride))
    return out


def covering_periodic_bounds(indices, period):
    """paliwa_domains.hpp:488-503."""
    if not indices:
        return None
    res = (indices[0], indices[-1])
    widest = indices[0] + period - indices[-1]
    for a, b in zip(indices, indices[1:]):
        if b - a > widest:
            widest = b - a
            res = (b, a)
    return res


def pole_pass_segments(writes, origin, level, maximum_level, pass_level):
    """paliwa_domains.hpp:505-538: runs (first, count, stride, lower, upper)
    of packed-pencil slots. Raises ValueError for the reference's
    std::invalid_argument."""
    if writes is None:
        return []
    if (level < 1 or level >= 31 or maximum_level < level or
            maximum_level >= 64 or pass_level < 1 or pass_level > level):
        raise ValueError("Invalid levels for packed-pole indexing")
    n = 1 << level
    dist = 1 << (level - pass_level)
    step = 2 * dist
    shift = maximum_level - level
    gperiod = 1 << maximum_level
    a, b = writes
    span = b - a if b >= a else gperiod - (a - b)
    left = (span >> shift) // step + 1
    x = ((a - origin) if a >= origin else gperiod - (origin - a)) >> shift
    runs = []
    while left > 0:
        lower = n - (dist - x) if x < dist else x - dist
        upper = x - (n - dist) if x >= n - dist else x + dist
        end = dist - 1 if x < dist else (n - dist - 1 if x < n - dist
                                         else n - 1)
        cnt = min(left, (end - x) // step + 1)
        runs.append((x, cnt, step, lower, upper))
        left -= cnt
        adv = cnt * step
        x = adv - (n - x) if adv >= n - x else x + adv
    return runs


def restrict_periodic_bounds(first, count, stride, bounds, period):
    """One axis of paliwa_domains.hpp:540-567: the points first + k * stride
    (k < count) inside periodic bounds, as at most two (first, count) runs."""
    if bounds is None or count == 0:
        return []
    last = first + (count - 1) * stride
    runs = []

    def append(lower, upper):
        lower = max(lower, first)
        upper = min(upper, last)
        begin = first + ((lower - first + stride - 1) // stride) * stride
        if begin > upper:
            return
        runs.append((begin, (upper - begin) // stride + 1))

    lo, hi = bounds
    if lo <= hi:
        append(lo, hi)
    else:
        append(lo, period - 1)
        append(0, hi)
    return runs


def _window_index(uids, front, spacing, period, extent):
    off = (np.asarray(uids, dtype=np.int64) - front) % period
    if np.any(off % spacing) or np.any(off // spacing >= extent):
        raise RuntimeError("Transform domain is missing required input values")
    return off // spacing


def transform_outputs(buf, front, level, maximum_level, dim, levels, filters,
                      out_front, out_extents, out_strides):
    """In-place restricted-output transform of a window buffer along ``dim``
    (transform_with_remote, Direct execution, paliwa_transform.hpp:258-331).

    Writes exactly the reference's write sets: per (level, pass) the points of
    that parity whose uid along ``dim`` lies in the planned bounds, at the
    outputs' points in the other dimensions. Arithmetic is the lifting pass
    (c0*lo + c1*me) + c2*up in the buffer's dtype, one rounding per
    operation (numpy does not contract)."""
    nd = buf.ndim
    L = [int(x) for x in maximum_level]
    lv = [int(x) for x in level]
    spacing = [1 << (L[d] - lv[d]) for d in range(nd)]
    periods = [1 << L[d] for d in range(nd)]
    if any(int(e) == 0 for e in out_extents):
        return buf
    period = periods[dim]
    o_first = int(out_front[dim])
    o_last = o_first + (int(out_extents[dim]) - 1) * int(out_strides[dim])
    outputs = (o_first % period, o_last % period)
    writes_by = {}

    def visit(i, p, w):
        writes_by[(i, p)] = w

    bounds = transform_bounds(outputs, lv[dim], L[dim], levels, filters, visit)
    # Every required input along dim must be in the window (:282-289).
    _window_index(transform_indices(bounds, L[dim]), int(front[dim]),
                  spacing[dim], period, buf.shape[dim])
    # Buffer indices of the outputs in the other dimensions.
    other = []
    for d in range(nd):
        if d == dim:
            other.append(None)
            continue
        uids = int(out_front[d]) + np.arange(int(out_extents[d]),
                                             dtype=np.int64) * int(out_strides[d])
        other.append(_window_index(uids % periods[d], int(front[d]),
                                   spacing[d], periods[d], buf.shape[d]))
    T = buf.dtype.type
    for i, l in enumerate(int(x) for x in levels):
        s = 1 << (L[dim] - l)
        for p, (off, f) in enumerate(filters):
            b = writes_by[(i, p)]
            first = off * s  # even / odd lattice of level l along dim
            count = 1 << (l - 1)
            for begin, cnt in restrict_periodic_bounds(first, count, 2 * s, b,
                                                       period):
                x = begin + 2 * s * np.arange(cnt, dtype=np.int64)
                lo = np.where(x == 0, period - s, x - s)
                up = np.where(x + s == period, 0, x + s)
                fr, sp, ext = int(front[dim]), spacing[dim], buf.shape[dim]
                ix = [_window_index(v, fr, sp, period, ext) for v in (x, lo, up)]
                sel = [other[d] if d != dim else None for d in range(nd)]

                def take(k):
                    idx = list(sel)
                    idx[dim] = k
                    return buf[np.ix_(*idx)]

                c0, c1, c2 = (T(c) for c in f)
                val = (c0 * take(ix[1]) + c1 * take(ix[0])) + c2 * take(ix[2])
                idx = list(sel)
                idx[dim] = ix[0]
                buf[np.ix_(*idx)] = val
    return buf
