"""Restricted-output planning and transform on the CPU.

Pins the oracle's restatement (oracle/restricted.py) to the reference's own
checks in test/test_paliwa_plan.cpp, re-expressed here:
  * exact_access_sets / longer_filter_sequences (:29-112): write and read
    sets against an independent reverse walk of the stencil graph;
  * multipass_sparse_values (:114-197): restricted outputs equal the in-test
    1D reference loop;
  * nonconsecutive_levels_are_rejected, periodic_pole_cover,
    packed_pass_exact_accesses, packed_pass_large_coordinates,
    packed_pass_index_range (:199-429);
  * remote_only_complex_poles (:286-362) with real values: slabs of a 2D
    grid, including the periodic edges, against the full transform.
Then checks the library's host planner (paliwa_gb_transform_bounds, the
same code as the drop-in header include/paliwa/paliwa_plan.hpp) against the
oracle bound for bound.
"""
import itertools
import random

import numpy as np
import pytest

import oracle
import restricted as R
from paliwa_gb300 import _lib, transform as T


def points(b, stride, period):
    if b is None:
        return set()
    last = b[1] + (period if b[0] > b[1] else 0)
    return {i % period for i in range(b[0], last + 1, stride)}


def reverse_stencil(level, maximum, start, count, levels, filters):
    """Independent reference of test_paliwa_plan.cpp:29-69: walk the
    stencil graph backwards over explicit point sets."""
    period = 1 << maximum
    spacing = 1 << (maximum - level)
    output = None
    if count:
        output = (start * spacing, ((start + count - 1) * spacing) % period)
    required = points(output, spacing, period)
    expected = [[set() for _ in filters] for _ in levels]
    for li in reversed(range(len(levels))):
        stride = 1 << (maximum - levels[li])
        for p in reversed(range(len(filters))):
            for i in required:
                if i % (2 * stride) == filters[p][0] * stride:
                    expected[li][p].add(i)
            for i in expected[li][p]:
                required.add((i + period - stride) % period)
                required.add((i + stride) % period)
    return output, expected, required


def check_plan(level, maximum, start, count, levels, filters):
    period = 1 << maximum
    output, expected, required = reverse_stencil(level, maximum, start,
                                                 count, levels, filters)
    seen = {}
    bounds = R.transform_bounds(output, level, maximum, levels, filters,
                                lambda i, p, w: seen.__setitem__((i, p), w))
    for li, l in enumerate(levels):
        for p in range(len(filters)):
            got = points(seen[(li, p)], 2 << (maximum - l), period)
            assert got == expected[li][p], (li, p)
    assert len(bounds) == level + 1
    actual = set()
    for h in range(level + 1):
        actual |= points(bounds[h], period if h == 0 else 2 << (maximum - h),
                         period)
    assert actual == required
    return output, bounds, seen


LEVEL_LISTS = [[4, 3, 2, 1], [1, 2, 3, 4], [4, 3], [3, 4], [4], []]


def test_exact_access_sets():
    """Every parity sequence of up to five passes, every ordinary and wrapped
    output interval, both directions, partial levels and a coarser grid
    (test_paliwa_plan.cpp:71-91)."""
    for maximum in (4, 6):
        for passes in range(1, 6):
            for mask in range(1 << passes):
                filters = [((mask >> p) & 1, (0.0, 1.0, 0.0))
                           for p in range(passes)]
                for levels in LEVEL_LISTS:
                    for start in range(16):
                        for count in range(17):
                            check_plan(4, maximum, start, count, levels,
                                       filters)


def test_longer_filter_sequences():
    rng = random.Random(20260928)
    for _ in range(300):
        level = 1 + rng.randrange(8)
        minimum = rng.randrange(level + 1)
        levels = list(range(minimum + 1, level + 1))
        if rng.randrange(2):
            levels.reverse()
        filters = [(rng.randrange(2), (0.0, 0.0, 0.0))
                   for _ in range(6 + rng.randrange(7))]
        check_plan(level, level + 2, rng.randrange(1 << level),
                   rng.randrange((1 << level) + 1), levels, filters)


def test_library_planner_matches_oracle():
    rng = random.Random(7)
    for _ in range(400):
        level = 1 + rng.randrange(9)
        maximum = level + rng.randrange(3)
        minimum = rng.randrange(level + 1)
        levels = list(range(minimum + 1, level + 1))
        if rng.randrange(2):
            levels.reverse()
        filters = [(rng.randrange(2), (0.0, 0.0, 0.0))
                   for _ in range(1 + rng.randrange(5))]
        period = 1 << maximum
        if rng.randrange(8) == 0:
            outputs = None
        else:
            outputs = (rng.randrange(period), rng.randrange(period))
        seen = {}
        want = R.transform_bounds(outputs, level, maximum, levels, filters,
                                  lambda i, p, w: seen.__setitem__((i, p), w))
        bounds, writes = T.transform_bounds(outputs, level, maximum, levels,
                                            filters)
        assert bounds == want
        for i in range(len(levels)):
            for p in range(len(filters)):
                assert writes[i][p] == seen[(i, p)]


def test_nonconsecutive_levels_are_rejected():
    filters = [(1, (0.0, 1.0, 0.0))]
    for levels in ([4, 1], [1, 4], [1, 2, 1]):
        with pytest.raises(ValueError):
            R.transform_bounds((0, 0), 4, 4, levels, filters)
        with pytest.raises(_lib.InvalidArgument):
            T.transform_bounds((0, 0), 4, 4, levels, filters)
    with pytest.raises(_lib.InvalidArgument):
        T.transform_bounds((0, 0), 4, 4, [5], filters)
    with pytest.raises(_lib.InvalidArgument):
        T.transform_bounds((0, 0), 4, 4, [4], [(2, (0.0, 1.0, 0.0))])


def test_periodic_pole_cover():
    cases = [([], None), ([12], (12, 12)), ([8, 12, 16], (8, 16)),
             ([0, 4, 56, 60], (56, 4)), ([0, 16, 32, 48], (0, 48))]
    for idx, want in cases:
        assert R.covering_periodic_bounds(idx, 64) == want


def test_packed_pass_exact_accesses():
    assert R.pole_pass_segments(None, 0, 3, 5, 2) == []
    spacing = 4
    for level in range(1, 6):
        period = 1 << level
        for pas in range(1, level + 1):
            dist = 1 << (level - pas)
            for origin in range(period):
                for parity in (0, 1):
                    for start in range(parity * dist, period, 2 * dist):
                        for count in range(1, period // (2 * dist) + 1):
                            last = (start + (count - 1) * 2 * dist) % period
                            runs = R.pole_pass_segments(
                                (start * spacing, last * spacing),
                                origin * spacing, level, level + 2, pas)
                            got = [(a + k * st, lo + k * st, up + k * st)
                                   for a, n, st, lo, up in runs
                                   for k in range(n)]

                            def slot(x):
                                return (x - origin + 2 * period) % period

                            want = []
                            for i in range(count):
                                x = (start + i * 2 * dist) % period
                                want.append((slot(x), slot(x - dist),
                                             slot(x + dist)))
                            assert got == want


def test_packed_pass_large_coordinates():
    maximum = 63
    spacing = 1 << (maximum - 3)
    runs = R.pole_pass_segments((spacing, 5 * spacing), 6 * spacing, 3,
                                maximum, 3)
    got = [(a + k * st, lo + k * st, up + k * st)
           for a, n, st, lo, up in runs for k in range(n)]
    assert got == [(3, 2, 4), (5, 4, 6), (7, 6, 0)]
    with pytest.raises(ValueError):
        R.pole_pass_segments((0, 0), 0, 31, 31, 1)


def reference_loop(inp, levels, filters, maximum):
    """test_paliwa_plan.cpp:128-139: the 1D periodic reference loop."""
    ref = inp.copy()
    period = ref.size
    for l in levels:
        stride = 1 << (maximum - l)
        for off, f in filters:
            for i in range(off * stride, period, 2 * stride):
                ref[i] = (f[0] * ref[(i + period - stride) % period] +
                          f[1] * ref[i]) + f[2] * ref[(i + stride) % period]
    return ref


def test_multipass_sparse_values():
    maximum, level, spacing, period = 6, 4, 4, 64
    inp = 1.0 + np.sin(np.arange(period) * 0.7)
    for passes in range(1, 6):
        for mask in range(1 << passes):
            filters = [((mask >> p) & 1,
                        (0.0, 1.0, 0.25) if p % 2 else (-0.5, 1.0, 0.125))
                       for p in range(passes)]
            for levels in ([4, 3, 2, 1], [1, 2, 3, 4]):
                ref = reference_loop(inp, levels, filters, maximum)
                for start in (0, 3, 12, 15):
                    count = min(4, 16 - start)
                    outputs = (start * spacing,
                               (start + count - 1) * spacing)
                    bounds = R.transform_bounds(outputs, level, maximum,
                                                levels, filters)
                    need = sorted(R.transform_indices(bounds, maximum))
                    cover = R.covering_periodic_bounds(need, period)
                    ext = ((cover[1] - cover[0]) % period) // spacing + 1
                    uids = (cover[0] + spacing * np.arange(ext)) % period
                    buf = inp[uids].copy()
                    R.transform_outputs(buf, (cover[0],), (level,),
                                        (maximum,), 0, levels, filters,
                                        (start * spacing,), (count,),
                                        (spacing,))
                    for k in range(count):
                        u = (start + k) * spacing
                        j = ((u - cover[0]) % period) // spacing
                        assert abs(buf[j] - ref[u]) <= 1e-12


FIVE_PASSES = [(1, (-0.5, 1.0, 0.125)), (0, (0.0, 1.0, 0.25)),
               (0, (0.125, 1.0, 0.125)), (1, (0.0, 1.0, 0.25)),
               (1, (-0.25, 1.0, 0.125))]


def full_axis_transform(x, dim, level, maximum, levels, filters):
    y = np.ascontiguousarray(x.copy())
    oracle.transform_in(y, level, maximum, dim, levels, filters)
    return y


def slab_case(dim, start, count, forward, dtype=np.float64):
    """A slab of `count` points from `start` along `dim` of a (4, 3) grid at
    maximum (6, 5), with its periodic halo in one window buffer."""
    level, maximum = (4, 3), (6, 5)
    shape = tuple(1 << l for l in level)
    u0 = np.arange(shape[0])[:, None] * (1 << (maximum[0] - level[0]))
    u1 = np.arange(shape[1])[None, :] * (1 << (maximum[1] - level[1]))
    x = (np.sin(u0 + 0.3 * u1) + np.cos(0.7 * u0 - u1)).astype(dtype)
    n = level[dim]
    levels = list(range(n, 0, -1))
    if not forward:
        levels.reverse()
    ref = full_axis_transform(x, dim, level, maximum, levels, FIVE_PASSES)
    sp = 1 << (maximum[dim] - level[dim])
    period = 1 << maximum[dim]
    ofront = [0, 0]
    oext = list(shape)
    ostr = [1 << (maximum[d] - level[d]) for d in range(2)]
    ofront[dim] = start * sp
    oext[dim] = count
    bounds = R.transform_bounds(
        (start * sp, ((start + count - 1) * sp) % period), n, maximum[dim],
        levels, FIVE_PASSES)
    need = sorted(set(R.transform_indices(bounds, maximum[dim])) |
                  {((start + k) * sp) % period for k in range(count)})
    cover = R.covering_periodic_bounds(need, period)
    ext = ((cover[1] - cover[0]) % period) // sp + 1
    idx = ((cover[0] + sp * np.arange(ext)) % period) // sp
    buf = np.ascontiguousarray(np.take(x, idx, axis=dim))
    front = [0, 0]
    front[dim] = cover[0]
    return dict(x=x, ref=ref, buf=buf, front=tuple(front), level=level,
                maximum=maximum, dim=dim, levels=levels,
                outputs=(tuple(ofront), tuple(oext), tuple(ostr)),
                idx=idx, start=start, count=count)


def slab_outputs(c, buf):
    """Output values of a slab case's buffer, in grid order along dim."""
    sp = 1 << (c["maximum"][c["dim"]] - c["level"][c["dim"]])
    n = 1 << c["level"][c["dim"]]
    rows = []
    for k in range(c["count"]):
        g = (c["start"] + k) % n
        j = int(np.nonzero(c["idx"] == g)[0][0])
        rows.append(np.take(buf, j, axis=c["dim"]))
    want = [np.take(c["ref"], (c["start"] + k) % n, axis=c["dim"])
            for k in range(c["count"])]
    del sp
    return rows, want


@pytest.mark.parametrize("dim", [0, 1])
@pytest.mark.parametrize("forward", [True, False])
def test_slabs_match_full_transform(dim, forward):
    size = 1 << (4, 3)[dim]
    for start, count in ((0, size // 2), (size // 2, size // 2), (0, size),
                         (size - 3, 3)):
        c = slab_case(dim, start, count, forward)
        buf = c["buf"].copy()
        o = c["outputs"]
        R.transform_outputs(buf, c["front"], c["level"], c["maximum"], dim,
                            c["levels"], FIVE_PASSES, *o)
        rows, want = slab_outputs(c, buf)
        for r, w in zip(rows, want):
            assert np.max(np.abs(r - w)) <= 1e-12


def test_missing_input_is_an_error():
    c = slab_case(0, 4, 4, True)
    buf = c["buf"][1:].copy()  # drop the window's first point
    front = (c["front"][0] + (1 << 2), 0)
    with pytest.raises(RuntimeError):
        R.transform_outputs(buf, front, c["level"], c["maximum"], 0,
                            c["levels"], FIVE_PASSES, *c["outputs"])


def test_library_argument_errors_without_gpu():
    """paliwa_gb_transform_outputs validates everything on the host before
    any launch: shapes and levels (std::invalid_argument), a required input
    outside the window (std::runtime_error, paliwa_transform.hpp:282-289),
    and returns at once for empty outputs. The grid pointer is never
    dereferenced on these paths."""
    lib = _lib.load()
    fake = 256  # an aligned address that is never touched here
    hat = [(1, (-0.5, 1.0, -0.5))]

    def call(dtype=_lib.F64, level=(4,), maximum=(4,), front=(0,),
             extents=(16,), levels=(4, 3, 2, 1), filters=hat,
             outputs=((4,), (4,), (1,)), grid=fake):
        of, oe, os_ = outputs
        return lib.paliwa_gb_transform_outputs(
            grid, dtype, len(level), _lib.i64(level), _lib.i64(maximum),
            _lib.i64(front), _lib.i64(extents), 0, _lib.i64(levels),
            len(levels), _lib.i32([o for o, _ in filters]),
            _lib.f64([c for _, f in filters for c in f]), len(filters),
            _lib.i64(of), _lib.i64(oe), _lib.i64(os_), None)

    assert call(outputs=((4,), (0,), (1,)), grid=None) == _lib.OK
    assert call(dtype=_lib.F32C) == _lib.INVALID_ARGUMENT
    assert call(grid=None) == _lib.INVALID_ARGUMENT
    assert call(extents=(17,)) == _lib.INVALID_ARGUMENT
    assert call(level=(3,), maximum=(4,), front=(1,), extents=(8,),
                levels=(3, 2, 1), outputs=((2,), (1,), (2,))) == \
        _lib.INVALID_ARGUMENT  # front off the level-3 lattice
    assert call(levels=(4, 2)) == _lib.INVALID_ARGUMENT  # not consecutive
    assert call(filters=[(2, (0.0, 1.0, 0.0))]) == _lib.INVALID_ARGUMENT
    # Outputs 4..7 need inputs around the whole axis; the window holds
    # uids 0..7 only.
    assert call(extents=(8,)) == _lib.RUNTIME_ERROR
    assert b"missing required input" in lib.paliwa_gb_last_error()
    # A second dimension whose outputs leave the window.
    assert call(level=(4, 2), maximum=(4, 2), front=(0, 0), extents=(16, 2),
                outputs=((4, 0), (4, 4), (1, 1))) == _lib.INVALID_ARGUMENT
