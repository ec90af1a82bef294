"""Bit-exact CPU model of the FP32-compensated transform -- TEST INFRASTRUCTURE.

Only ``tests/`` may import this module. The FP32-compensated mode is this
project's own precision scheme (the reference has FP64 only), so its model is
not a restatement of the reference: it restates, with numpy float32
operations, the arithmetic the GPU kernels perform, so that every kernel
variant can be checked bit for bit. The level and pass order are the
reference's (paliwa/paliwa_transform.hpp:346-431 drives levels fine to coarse
for hierarchize_in and coarse to fine for dehierarchize_in; each pass updates
the points k = offset*s mod 2s from their neighbours k +- s, periodic, as in
detail::lifting_pass :24-51).

A value is an unevaluated pair h + l of float32. Loading a stored float gives
(x, 0); storing gives fl(h + l), once per axis. With symmetric exact-scaler
filters (c0 == c2 and every coefficient a power of two, true for all paliwa
wavelet tables) an update is

    s  = TwoSum(lo.h, up.h)                  (Knuth, 6 operations)
    e1 = s.l + (lo.l + up.l)
    t  = c0 * s.h                            (exact: c0 is a power of two)
    m  = me.h          if c1 == 1 else c1 * me.h        (exact)
    r  = TwoSum(m, t)
    l  = c0 * e1 + r.l                       (the GPU's fma; c0*e1 is exact)
    l  = l + me.l      if c1 == 1 else c1 * me.l + l    (fma; product exact)
    result (r.h, l)

Every product is exact, so numpy's separately rounded float32 multiply and
add give the same bits as the GPU's fused multiply-add.
"""
from __future__ import annotations

import numpy as np

from oracle import FORWARD, INVERSE

_f = np.float32


def _two_sum(a, b):
    s = a + b
    bb = s - a
    e = (a - (s - bb)) + (b - bb)
    return s, e


def _update(coeffs, lo, me, up):
    c0, c1, c2 = (_f(c) for c in coeffs)
    assert c0 == c2, "model covers symmetric filters only"
    lo_h, lo_l = lo
    me_h, me_l = me
    up_h, up_l = up
    s_h, s_l = _two_sum(lo_h, up_h)
    e1 = s_l + (lo_l + up_l)
    t = c0 * s_h
    m = me_h if c1 == 1 else c1 * me_h
    r_h, r_l = _two_sum(m, t)
    l = c0 * e1 + r_l
    l = l + me_l if c1 == 1 else c1 * me_l + l
    return r_h, l


def _axis(x, dim, level, lmin, filters, forward):
    """One axis, in place on a float32 array (levels lmin+1 .. level)."""
    n = x.shape[dim]
    v = np.moveaxis(x, dim, 0)
    h = v.copy()
    lo_part = np.zeros_like(h)
    ls = list(range(lmin + 1, level + 1))
    if forward:
        ls.reverse()  # hierarchize_in: fine to coarse
    with np.errstate(all="ignore"):
        for lv in ls:
            s = 1 << (level - lv)
            for offset, coeffs in filters:
                k = np.arange(offset * s, n, 2 * s)
                km, kp = (k - s) % n, (k + s) % n
                r_h, r_l = _update(coeffs, (h[km], lo_part[km]),
                                   (h[k], lo_part[k]), (h[kp], lo_part[kp]))
                h[k] = r_h
                lo_part[k] = r_l
        v[...] = h + lo_part


def hierarchize(x, level, lmin, wavelet="hat", forward=True):
    """Compensated transform of every axis in order (dims 0 .. d-1, as the
    reference's hierarchize/dehierarchize); returns a new float32 array."""
    y = np.array(x, dtype=np.float32, copy=True)
    filters = (FORWARD if forward else INVERSE)[wavelet]
    for d in range(y.ndim):
        _axis(y, d, int(level[d]), int(lmin[d]), filters, forward)
    return y
