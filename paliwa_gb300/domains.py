"""Level-strided index maps of paliwa (paliwa/paliwa_domains.hpp,
paliwa/paliwa_dimensions.hpp) on the host.

A ``StridedDomain`` is the (front, extents, strides) triple of a
``ddc::StridedDiscreteDomain`` in finest-level uid coordinates. On the device
the same maps are compact-index arithmetic inside the lifting kernels
(distance 2^(level - l) and parity ``offset``); these host versions build
plans, describe grids to callers and are checked bit-exactly against the
reference's known answers.
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass


@dataclass(frozen=True)
class StridedDomain:
    front: tuple
    extents: tuple
    strides: tuple

    def size(self):
        return math.prod(self.extents)

    def empty(self):
        return self.size() == 0

    def back(self):
        return tuple(f + (e - 1) * s
                     for f, e, s in zip(self.front, self.extents, self.strides))

    def contains(self, uid):
        for x, f, e, s in zip(uid, self.front, self.extents, self.strides):
            if x < f or (x - f) % s != 0 or (x - f) // s >= e:
                return False
        return True

    def points(self):
        axes = [range(f, f + e * s, s)
                for f, e, s in zip(self.front, self.extents, self.strides)]
        return itertools.product(*axes)


def strided_domain_from_level(level, finest_level, lbound=None):
    """paliwa_domains.hpp:33-49. The reference shifts a 32-bit ``1 << l``
    (:41, :45), so levels are valid below 31."""
    for l, L in zip(level, finest_level):
        if not 0 <= int(l) <= int(L) < 31:
            raise ValueError("requires 0 <= level <= finest_level < 31")
    d = len(level)
    front = tuple(int(x) for x in lbound) if lbound is not None else (0,) * d
    return StridedDomain(front, tuple(1 << int(l) for l in level),
                         tuple(1 << (int(L) - int(l))
                               for l, L in zip(level, finest_level)))


def strided_hierarchical_domain_from_level(level, finest_level, lbound=None):
    """paliwa_domains.hpp:51-83: the hierarchical subspace of level vector
    ``level``: 2^(l-1) points per dimension starting at 2^(L-l) with stride
    2^(L-l+1); level 0 is the single point at the front."""
    d = len(level)
    lb = tuple(int(x) for x in lbound) if lbound is not None else (0,) * d
    front, ext, st = [], [], []
    for l, L, b in zip(level, finest_level, lb):
        l, L = int(l), int(L)
        if not 0 <= l <= L:
            raise ValueError("requires 0 <= level <= finest_level")
        ext.append(1 if l == 0 else 1 << (l - 1))
        front.append(b if l == 0 else b + (1 << (L - l)))
        st.append(1 << (L - l + 1))
    return StridedDomain(tuple(front), tuple(ext), tuple(st))


def odd_strided_domain_from_domain(domain, dim, lbound=None):
    """paliwa_domains.hpp:85-98: points of odd parity along ``dim``."""
    d = len(domain.front)
    lb = list(lbound) if lbound is not None else [0] * d
    lb[dim] += domain.strides[dim]
    st = list(domain.strides)
    st[dim] *= 2
    ext = list(domain.extents)
    ext[dim] //= 2
    return StridedDomain(tuple(lb), tuple(ext), tuple(st))


def even_strided_domain_from_domain(domain, dim, lbound=None):
    """paliwa_domains.hpp:100-111: points of even parity along ``dim``."""
    d = len(domain.front)
    lb = tuple(lbound) if lbound is not None else (0,) * d
    st = list(domain.strides)
    st[dim] *= 2
    ext = list(domain.extents)
    ext[dim] //= 2
    return StridedDomain(tuple(lb), tuple(ext), tuple(st))


def get_strided_domains(all_levels, maximum_level, lbound=None):
    """paliwa_domains.hpp:113-128: one strided domain per component grid."""
    return [strided_domain_from_level(l, maximum_level, lbound)
            for l in all_levels]


def restrict_strided_with_discrete(domain, other_front, other_back):
    """paliwa_domains.hpp:141-214: the points of ``domain`` inside the box
    [other_front, other_back] (both inclusive). Dimensions the box does not
    constrain are passed as None and keep the strided extent (:149-151,
    :175-182). The first point uses the reference's ceil of a float quotient
    (:152-157)."""
    front, ext = [], []
    for f, e, s, of, ob in zip(domain.front, domain.extents, domain.strides,
                               other_front, other_back):
        if of is None:
            nf = f
        else:
            import numpy as np
            q = np.float32(of - f) / np.float32(s)
            nf = f + int(np.float32(math.ceil(float(q))) * np.float32(s))
        front.append(nf)
        if ob is None:
            ext.append(e)
        else:
            ext.append((ob - nf) // s + 1 if ob >= nf else
                       -((nf - ob) // s) + 1)
    return StridedDomain(tuple(front), tuple(ext), tuple(domain.strides))


def periodic_unit_interval_coordinates(level, finest_level):
    """paliwa_dimensions.hpp:71-79: coordinate x = uid / 2^L of each point
    of a grid at ``level`` (uid = k * 2^(L - l)) on [0, 1) without the
    periodic end point."""
    return [[(k << (int(L) - int(l))) / float(1 << int(L))
             for k in range(1 << int(l))]
            for l, L in zip(level, finest_level)]
