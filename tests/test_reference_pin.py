"""The oracle pinned to the reference itself (CPU).

``oracle/_ref/libpaliwa_ref.so`` is the reference's own headers
(paliwa_transform.hpp, paliwa_domains.hpp, paliwa_wavelets.hpp,
paliwa_dimensions.hpp, paliwa_utils.hpp), compiled unmodified from the
reference checkout against the serial DDC/Kokkos stand-ins of
``oracle/ref_shim``. These tests hold every oracle function that the GPU
tests use as their checker -- and the library's host-side planner and index
maps -- equal to it: bit for bit for values, exactly for index sets. They
need the reference checkout and skip where it is absent.
"""
import itertools
import math
import os

import numpy as np
import pytest

import oracle as O
import reference as R

pytestmark = pytest.mark.skipif(not R.available(),
                                reason="reference checkout not present")

WAVELETS = ["hat", "biorthogonal", "fullweighting"]
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "plan_multipass.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    O.build()
    R.build()


def both_ways(x, level, lmin, lmax, wavelet):
    """(forward, inverse-of-forward) from the reference and from the oracle
    in both of its execution modes."""
    ref_f = R.hierarchize(x.copy(), level, lmin, lmax, wavelet)
    ref_b = R.dehierarchize(ref_f.copy(), level, lmin, lmax, wavelet)
    outs = []
    for mode in (0, 1):  # Direct, packed poles
        f = O.hierarchize(x.copy(), level, lmin, lmax, wavelet, mode=mode)
        b = O.dehierarchize(f.copy(), level, lmin, lmax, wavelet, mode=mode)
        outs.append((f, b))
    return (ref_f, ref_b), outs


def assert_same(x, level, lmin, lmax, wavelet):
    (rf, rb), outs = both_ways(x, level, lmin, lmax, wavelet)
    for f, b in outs:
        assert np.array_equal(f, rf), (level, lmin, wavelet)
        assert np.array_equal(b, rb), (level, lmin, wavelet)


@pytest.mark.parametrize("wavelet", WAVELETS)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_c1_2d(wavelet, dtype):
    """C1: the 64 x 64 grid, sin(2 pi x) cos(3 pi y) + U[-0.01, 0.01]."""
    x = np.arange(64) / 64.0
    f = np.multiply.outer(np.sin(2 * np.pi * x), np.cos(3 * np.pi * x))
    f = f + np.random.default_rng(20261204).uniform(-0.01, 0.01, f.shape)
    for lmin in ((0, 0), (1, 3), (6, 2)):
        assert_same(f.astype(dtype), (6, 6), lmin, (6, 6), wavelet)


@pytest.mark.parametrize("wavelet", WAVELETS)
def test_c2_slice_3d(wavelet):
    """A 64^3 grid of the C2 input family (8 Gaussians plus noise)."""
    import bench
    w = bench.Workload("3d-biorthogonal-999")
    w.levels = [(6, 6, 6)]
    x = np.ascontiguousarray(w.grid_values(0))
    assert_same(x, (6, 6, 6), (0, 0, 0), (6, 6, 6), wavelet)
    assert_same(x, (6, 6, 6), (2, 0, 5), (7, 6, 8), wavelet)


@pytest.mark.parametrize("wavelet", WAVELETS)
def test_reduced_c3_6d(wavelet):
    """C3's family at levels (3, 3, 3, 3, 2, 2): products of cosines + noise,
    FP64 and FP32."""
    import bench
    w = bench.Workload("6d-hat-555544")
    w.levels = [(3, 3, 3, 3, 2, 2)]
    x = np.ascontiguousarray(w.grid_values(0))
    lvl = w.levels[0]
    assert_same(x, lvl, (0,) * 6, lvl, wavelet)
    assert_same(x.astype(np.float32), lvl, (1, 0, 2, 0, 1, 0), lvl, wavelet)


def test_fifty_ct_grids():
    """Fifty grids of the 4D combination scheme |l|_1 = 12 - q (lmin 1, the
    CT driver's wavelet) with the C4 input function, plus every wavelet on
    ten of them."""
    import bench
    from paliwa_gb300 import ct as pct
    w = bench.Workload("4d-ct-20")
    levels, _ = pct.combination_scheme(4, 12, 3, 1)
    rng = np.random.default_rng(5)
    pick = sorted(rng.choice(len(levels), 50, replace=False))
    w.levels = [levels[i] for i in pick]
    lmax = (9,) * 4
    for i, lv in enumerate(w.levels):
        x = np.ascontiguousarray(w.grid_values(i))
        wavelets = WAVELETS if i < 10 else ["biorthogonal"]
        for wav in wavelets:
            assert_same(x, lv, (1,) * 4, lmax, wav)


def test_transform_in_level_lists_and_filters():
    """transform_in with explicit level orders and general filter tables
    (non-power-of-two coefficients, repeated parities), FP64 and FP32."""
    rng = np.random.default_rng(11)
    for trial in range(60):
        nd = int(rng.integers(1, 4))
        level = [int(rng.integers(1, 7)) for _ in range(nd)]
        lmax = [l + int(rng.integers(0, 3)) for l in level]
        dim = int(rng.integers(0, nd))
        lv = [int(v) for v in rng.permutation(np.arange(1, level[dim] + 1))]
        npass = int(rng.integers(1, 4))
        filt = [(int(rng.integers(0, 2)),
                 tuple(float(c) for c in rng.uniform(-1, 1, 3)))
                for _ in range(npass)]
        dtype = np.float64 if trial % 2 == 0 else np.float32
        x = rng.standard_normal([1 << l for l in level]).astype(dtype)
        a = R.transform_in(x.copy(), level, lmax, dim, lv, filt)
        b = O.transform_in(x.copy(), level, lmax, dim, lv, filt)
        assert np.array_equal(a, b), trial


def test_transform_in_on_windows_checks_bounds():
    """The full-grid transform_in on a chunk that holds only a window of the
    lattice (lifting_pass with CheckBounds): the oracle's restatement equals
    the reference on random windows, every wavelet, both directions."""
    rng = np.random.default_rng(0)
    for trial in range(300):
        nd = int(rng.integers(1, 4))
        level = [int(rng.integers(1, 6)) for _ in range(nd)]
        lmax = [l + int(rng.integers(0, 3)) for l in level]
        sp = [1 << (L - l) for l, L in zip(level, lmax)]
        front = [int(rng.integers(0, 1 << l)) * s for l, s in zip(level, sp)]
        ext = [int(rng.integers(1, (1 << l) - f // s + 1))
               for l, s, f in zip(level, sp, front)]
        dim = int(rng.integers(0, nd))
        lv = (list(range(level[dim], 0, -1)) if trial % 2
              else list(range(1, level[dim] + 1)))
        wav = WAVELETS[trial % 3]
        filt = O.FORWARD[wav] if trial % 4 < 2 else O.INVERSE[wav]
        x = rng.standard_normal(ext)
        a = R.transform_in(x.copy(), level, lmax, dim, lv, filt, front, ext)
        b = O.transform_in_window(x.copy(), level, lmax, front, dim, lv, filt)
        assert np.array_equal(a, b), trial


def test_golden_multipass_vectors_from_the_reference():
    """The committed vectors of tests/golden/plan_multipass.npz (the
    reference test's 1D reference loop, test/test_paliwa_plan.cpp:114-139)
    are what the reference's transform_in computes, bit for bit: a level-4
    grid inside maximum level 6 holds every fourth uid of the loop's
    period-64 array."""
    g = np.load(GOLDEN)
    inp = g["input"]
    for (passes, mask, order), want in zip(g["cases"], g["output"]):
        filt = []
        for p in range(passes):
            off = 1 if mask & (1 << p) else 0
            filt.append((off, (0.0, 1.0, 0.25) if p % 2 else
                         (-0.5, 1.0, 0.125)))
        levels = [4, 3, 2, 1] if order == 0 else [1, 2, 3, 4]
        got = R.transform_in(inp[::4].copy(), (4,), (6,), 0, levels, filt)
        assert np.array_equal(got, want[::4]), (passes, mask, order)


def random_window(rng, nd):
    level = [int(rng.integers(1, 6)) for _ in range(nd)]
    lmax = [l + int(rng.integers(0, 3)) for l in level]
    sp = [1 << (L - l) for l, L in zip(level, lmax)]
    front = [int(rng.integers(0, 1 << l)) * s for l, s in zip(level, sp)]
    ext = [int(rng.integers(1, (1 << l) - f // s + 1))
           for l, s, f in zip(level, sp, front)]
    return level, lmax, sp, front, ext


def test_restricted_outputs_every_pole_execution():
    """The restricted-output transform_in (outputs overload) on window
    buffers: the oracle's restatement (oracle/restricted.py) equals the
    reference's Direct, PackedPasses and PackedPoles executions, and the
    reference's "missing required input values" error where it throws."""
    import restricted as RS
    rng = np.random.default_rng(4)
    checked = errors = 0
    for trial in range(400):
        nd = int(rng.integers(1, 4))
        level, lmax, sp, front, ext = random_window(rng, nd)
        dim = int(rng.integers(0, nd))
        lv = (list(range(level[dim], 0, -1)) if trial % 2
              else list(range(1, level[dim] + 1)))
        lv = lv[:int(rng.integers(1, len(lv) + 1))]
        wav = WAVELETS[trial % 3]
        filt = O.FORWARD[wav] if trial % 4 < 2 else O.INVERSE[wav]
        # outputs: a sub-box of the window (points of the lattice)
        of, oe = [], []
        for d in range(nd):
            a = int(rng.integers(0, ext[d]))
            b = int(rng.integers(a, ext[d]))
            of.append(front[d] + a * sp[d])
            oe.append(b - a + 1)
        x = rng.standard_normal(ext)
        try:
            want = RS.transform_outputs(x.copy(), front, level, lmax, dim, lv,
                                        filt, of, oe, sp)
        except RuntimeError:
            want = None
        for mode in (0, 1, 2):
            try:
                got = R.transform_outputs(x.copy(), level, lmax, front, ext,
                                          dim, lv, filt, of, oe, sp, mode)
            except RuntimeError as e:
                assert "missing required input" in str(e)
                got = None
            if want is None:
                assert got is None, (trial, mode)
                errors += 1
            else:
                assert got is not None, (trial, mode)
                if mode < 2:
                    assert np.array_equal(got, want), (trial, mode)
                else:
                    # Packed poles gathers the inputs once, runs every pass
                    # in scratch and scatters back only the outputs
                    # (paliwa_transform.hpp:115-185): those equal Direct's,
                    # every other point keeps its input value.
                    sel = tuple(slice((f - w) // s, (f - w) // s + e)
                                for f, w, s, e in zip(of, front, sp, oe))
                    assert np.array_equal(got[sel], want[sel]), trial
                    rest = np.ones(x.shape, bool)
                    rest[sel] = False
                    assert np.array_equal(got[rest], x[rest]), trial
                checked += 1
    assert checked > 300 and errors > 30


def test_planner_known_answers_and_random_bounds():
    """transform_bounds, covering_periodic_bounds and pole_pass_segments:
    the oracle's planner and the library's host planner (C ABI) against the
    reference, on every parity sequence of up to three passes, ordinary and
    wrapped outputs, both level orders, partial level lists."""
    import restricted as RS
    from paliwa_gb300 import transform as T
    rng = np.random.default_rng(9)
    for trial in range(1500):
        L = int(rng.integers(1, 8))
        level = int(rng.integers(1, L + 1))
        period = 1 << L
        lv = list(range(1, level + 1))
        if trial % 2:
            lv.reverse()
        lv = lv[:int(rng.integers(1, len(lv) + 1))]
        npass = int(rng.integers(1, 4))
        offs = [int(v) for v in rng.integers(0, 2, npass)]
        filt = [(o, (0.0, 1.0, 0.0)) for o in offs]
        if trial % 10 == 0:
            outputs = (-1, -1)
        else:
            outputs = (int(rng.integers(0, period)),
                       int(rng.integers(0, period)))
        rb, rw = R.transform_bounds(outputs, level, L, lv, offs)
        ow = {}
        ob = RS.transform_bounds(None if outputs[0] < 0 else outputs, level,
                                 L, lv, filt,
                                 lambda i, p, w: ow.__setitem__((i, p), w))
        norm = lambda b: (-1, -1) if b is None else tuple(b)
        assert [norm(b) for b in ob] == rb, trial
        assert [[norm(ow[(i, p)]) for p in range(npass)]
                for i in range(len(lv))] == rw, trial
        lb, lw = T.transform_bounds(None if outputs[0] < 0 else outputs,
                                    level, L, lv, filt)
        assert [norm(b) for b in lb] == rb, trial
        assert [[norm(w) for w in row] for row in lw] == rw, trial
    for trial in range(300):
        period = 1 << int(rng.integers(1, 8))
        n = int(rng.integers(1, period + 1))
        idx = sorted(int(v) for v in rng.choice(period, n, replace=False))
        assert tuple(RS.covering_periodic_bounds(idx, period)) == \
            R.covering_periodic_bounds(idx, period)
    for trial in range(600):
        L = int(rng.integers(1, 9))
        level = int(rng.integers(1, L + 1))
        pl = int(rng.integers(1, level + 1))
        step = 1 << (L - pl + 1)
        first = ((int(rng.integers(0, 1 << L)) // step) * step +
                 int(rng.integers(0, 2)) * (step // 2)) % (1 << L)
        last = ((first + int(rng.integers(0, 1 << L)) // step * step)
                % (1 << L))
        origin = int(rng.integers(0, 1 << level)) << (L - level)
        want = R.pole_pass_segments((first, last), origin, level, L, pl)
        got = [tuple(s) for s in RS.pole_pass_segments((first, last), origin,
                                                       level, L, pl)]
        assert got == want, trial


def test_index_maps_and_enumeration():
    """strided_domain_from_level, strided_hierarchical_domain_from_level,
    restrict_strided_with_discrete, initialize_dim_periodic_unit_interval and
    iterate_hierarchical_subspaces: the oracle's and the library's Python
    mirrors (paliwa_gb300.domains) against the reference."""
    from paliwa_gb300 import domains as D
    rng = np.random.default_rng(2)
    for trial in range(300):
        nd = int(rng.integers(1, 6))
        level = [int(rng.integers(0, 7)) for _ in range(nd)]
        lmax = [l + int(rng.integers(0, 4)) for l in level]
        lb = [int(rng.integers(0, 5)) for _ in range(nd)]
        want0 = R.level_domain(0, level, lmax, lb)
        want1 = R.level_domain(1, level, lmax, lb)
        assert O.strided_domain_from_level(level, lmax, lb) == want0
        assert O.strided_hierarchical_domain_from_level(level, lmax, lb) \
            == want1
        d0 = D.strided_domain_from_level(level, lmax, lb)
        d1 = D.strided_hierarchical_domain_from_level(level, lmax, lb)
        assert (tuple(d0.front), tuple(d0.extents), tuple(d0.strides)) == want0
        assert (tuple(d1.front), tuple(d1.extents), tuple(d1.strides)) == want1
        # the points of the strided domain inside a box
        dom = D.strided_domain_from_level(level, lmax)
        bf = [int(rng.integers(0, 1 << L)) for L in lmax]
        be = [int(rng.integers(1, (1 << L) - f + 1)) for f, L in zip(bf, lmax)]
        want = R.restrict_strided_with_discrete(
            (tuple(dom.front), tuple(dom.extents), tuple(dom.strides)), bf, be)
        got = D.restrict_strided_with_discrete(
            dom, bf, [f + e - 1 for f, e in zip(bf, be)])
        assert (tuple(got.front), tuple(got.extents),
                tuple(got.strides)) == want, trial
    for n in (1, 2, 3, 8, 64, 1000):
        want = R.periodic_unit_interval(n)
        if n & (n - 1) == 0:
            l = n.bit_length() - 1
            got = D.periodic_unit_interval_coordinates((l,), (l,))[0]
            assert got == want
        assert want == [k * (1.0 / n) for k in range(n)] or \
            np.allclose(want, np.arange(n) / n, rtol=0, atol=1e-15)
    for level in ((2, 1), (0, 3, 1), (1, 1, 1, 2), (3,)):
        assert R.hierarchical_subspaces(level) == \
            [tuple(s) for s in O.iterate_hierarchical_subspaces(level)]
