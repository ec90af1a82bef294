"""The CPU oracle against the reference's own tests (no GPU needed)."""
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "plan_multipass.npz")


def golden_filters(passes, mask):
    # test/test_paliwa_plan.cpp:121-125
    return [((1 if mask & (1 << p) else 0),
             (0.0, 1.0, 0.25) if p % 2 else (-0.5, 1.0, 0.125))
            for p in range(passes)]


def test_oracle_matches_reference_test_loop(oracle_mod):
    """test/test_paliwa_plan.cpp:114-163: the transform of the level-4 grid
    inside maximum level 6 equals the reference's own 1D periodic loop."""
    g = np.load(GOLDEN)
    inp, cases, out = g["input"], g["cases"], g["output"]
    for (passes, mask, order), expected in zip(cases, out):
        levels = [4, 3, 2, 1] if order == 0 else [1, 2, 3, 4]
        grid = inp[::4].copy()  # uids 0, 4, ..., 60: the level-4 grid
        for mode in (0, 1):
            got = oracle_mod.transform_in(grid.copy(), [4], [6], 0, levels,
                                          golden_filters(passes, mask), mode)
            assert np.array_equal(got, expected[::4]), (passes, mask, order)
        # points off the level-4 lattice are never written by the loop
        others = np.ones(64, bool)
        others[::4] = False
        assert np.array_equal(expected[others], inp[others])


def seeded_grid(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.random(shape)


@pytest.mark.parametrize("lmin", [(0, 0), (0, 1), (0, 3), (1, 0), (1, 1),
                                  (1, 3), (3, 0), (3, 1), (3, 3)])
def test_hat_stays_same_2d(oracle_mod, lmin):
    """test/test_paliwa_transform.cpp:17-79 (level (3,3) in (4,4)): points of
    the lmin grid keep their values (1e-14), every other point changes, and
    dehierarchize undoes hierarchize (1e-13). The reference draws its input
    from Kokkos' XorShift64 pool (seed 12345), which is not reproducible
    without Kokkos; the input here has the same form (1 + ix + iy) * (1 + u)
    with u from a seeded numpy generator."""
    level, lmax = (3, 3), (4, 4)
    ix = np.arange(8)[:, None] * 2
    iy = np.arange(8)[None, :] * 2
    x = (1 + ix + iy) * (1 + seeded_grid((8, 8), 12345))
    y = x.copy()
    oracle_mod.hierarchize(y, level, lmin, lmax, "hat")
    sx, sy = 1 << (level[0] - lmin[0]), 1 << (level[1] - lmin[1])
    on_lmin = np.zeros((8, 8), bool)
    on_lmin[::sx, ::sy] = True
    assert np.all(np.abs(y[on_lmin] - x[on_lmin]) <= 1e-14)
    assert np.all(y[~on_lmin] != x[~on_lmin])
    oracle_mod.dehierarchize(y, level, lmin, lmax, "hat")
    assert np.max(np.abs(y - x)) <= 1e-13


@pytest.mark.parametrize("wavelet", ["biorthogonal", "fullweighting"])
def test_mass_conservation_2d(oracle_mod, wavelet):
    """test/test_paliwa_transform.cpp:81-143: after hierarchization the sum
    over the lmin grid equals mean * count to 1e-13 (every wavelet but hat)."""
    level, lmax = (3, 3), (4, 4)
    ix = np.arange(8)[:, None] * 2
    iy = np.arange(8)[None, :] * 2
    for lmin in [(a, b) for a in (0, 1, 3) for b in (0, 1, 3)]:
        x = (1 + ix + iy) * (1 + seeded_grid((8, 8), 12345))
        avg = x.sum() / x.size
        y = oracle_mod.hierarchize(x.copy(), level, lmin, lmax, wavelet)
        sx, sy = 1 << (level[0] - lmin[0]), 1 << (level[1] - lmin[1])
        sub = y[::sx, ::sy]
        assert abs(sub.sum() - avg * sub.size) <= 1e-13


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("wavelet", ["hat", "biorthogonal", "fullweighting"])
def test_direct_and_packed_poles_agree(oracle_mod, dtype, wavelet):
    """Both reference execution modes (PoleExecution::Direct and
    PackedPoles, paliwa/paliwa_transform.hpp:21) compute identical values."""
    for level, lmin in [((5,), (0,)), ((3, 4), (1, 0)), ((2, 3, 4), (0, 1, 2)),
                        ((4, 1, 3, 2), (2, 0, 0, 1))]:
        lmax = tuple(l + 1 for l in level)
        x = seeded_grid([1 << l for l in level], 7).astype(dtype)
        for fwd in (True, False):
            a = oracle_mod.hierarchize(x.copy(), level, lmin, lmax, wavelet,
                                       forward=fwd, mode=0)
            b = oracle_mod.hierarchize(x.copy(), level, lmin, lmax, wavelet,
                                       forward=fwd, mode=1)
            assert np.array_equal(a, b)


def test_round_trip_all_wavelets(oracle_mod):
    for wavelet in ("hat", "biorthogonal", "fullweighting"):
        level, lmin, lmax = (6, 5, 4), (0, 2, 1), (7, 5, 6)
        x = seeded_grid([64, 32, 16], 3)
        y = oracle_mod.hierarchize(x.copy(), level, lmin, lmax, wavelet)
        oracle_mod.dehierarchize(y, level, lmin, lmax, wavelet)
        assert np.max(np.abs(y - x)) <= 1e-13


def test_oracle_errors(oracle_mod):
    x = np.zeros((4, 4))
    with pytest.raises(KeyError):
        oracle_mod.hierarchize(x, (2, 2), (0, 0), (2, 2), "db4")
    with pytest.raises(ValueError):
        oracle_mod.hierarchize(x, (2, 2), (3, 0), (2, 2), "hat")
    with pytest.raises(RuntimeError):  # paliwa_transform.hpp:239-240
        oracle_mod.transform_in(x, (2, 2), (2, 2), 0, [2], [(2, (0, 1, 0))])


@pytest.mark.parametrize("wavelet", ["hat", "biorthogonal", "fullweighting"])
def test_compensated_model_close_to_fp64(oracle_mod, wavelet):
    """The FP32-compensated model stays within 1e-6 (normwise max) of the
    FP64 oracle on the same FP32 inputs, and well inside plain FP32's error:
    it is a faithful model of a compensated scheme, not of plain FP32."""
    from compensated import hierarchize as model
    level, lmin = (6, 5, 4), (0, 1, 0)
    rng = np.random.default_rng(3)
    x = rng.uniform(-1.0, 1.0, [1 << l for l in level]).astype(np.float32)
    for forward in (True, False):
        ref = oracle_mod.hierarchize(x.astype(np.float64), level, lmin, level,
                                     wavelet, forward=forward)
        got = model(x, level, lmin, wavelet, forward).astype(np.float64)
        plain = oracle_mod.hierarchize(x.copy(), level, lmin, level, wavelet,
                                       forward=forward).astype(np.float64)
        scale = np.max(np.abs(ref))
        err = np.max(np.abs(got - ref)) / scale
        err_plain = np.max(np.abs(plain - ref)) / scale
        assert err <= 1e-6, err
        # One rounding per axis and point: at most 3 ulps-scale errors.
        assert err <= 3 * 2.0 ** -24 * 1.01 + 1e-12 or err < err_plain


def test_c1_configuration_round_trip(oracle_mod):
    """C1, the reference's CPU-sized case: 2D hat at (6, 6) on
    sin(2 pi x) cos(3 pi y) + noise; the forward keeps the lmin = 0 point
    (hat, paliwa test_paliwa_transform.cpp:57-73 style) and the round trip
    returns the input to 1e-13."""
    x = np.arange(64) / 64.0
    f = np.multiply.outer(np.sin(2 * np.pi * x), np.cos(3 * np.pi * x))
    f = f + np.random.default_rng(20261204).uniform(-0.01, 0.01, f.shape)
    h = oracle_mod.hierarchize(f.copy(), (6, 6), (0, 0), (6, 6), "hat")
    assert h[0, 0] == f[0, 0]
    back = oracle_mod.dehierarchize(h, (6, 6), (0, 0), (6, 6), "hat")
    assert np.max(np.abs(back - f)) <= 1e-13 * np.max(np.abs(f))


def test_vectorised_combine_and_restrict_match_the_driver_restatement():
    """The per-grid vectorised combine (used for full-size schemes) equals the
    subspace-by-subspace restatement of the reference driver
    (test/test_paliwa_combination_technique.cpp:256-290) bit for bit, and
    the restriction writes exactly the kept points."""
    import itertools
    import oracle as O
    for d, top in ((2, 9), (3, 7), (4, 7)):
        levels = [l for q in range(d) for l in itertools.product(
            range(1, top + 1), repeat=d) if sum(l) == top - q]
        coeffs = [(-1) ** (top - sum(l)) * math.comb(d - 1, top - sum(l))
                  for l in levels]
        rng = np.random.default_rng(d)
        grids = [rng.standard_normal([1 << x for x in l]) for l in levels]
        subs = O.kept_subspaces(levels)
        slow = O.combine(grids, levels, coeffs, None, subs)
        offs, total = O.sparse_offsets(subs)
        fast = O.combine_sparse(grids, levels, coeffs, offs, total)
        assert np.array_equal(np.concatenate([a.ravel() for a in slow]), fast)
        for g, lv in zip(grids[:5], levels[:5]):
            r = O.restrict_sparse(g.copy(), lv, fast, offs)
            for s, v in zip(subs, slow):
                if all(si <= li for si, li in zip(s, lv)):
                    assert np.array_equal(r[O.subspace_slices(s, lv)], v)
            changed = r != g
            idx = O.grid_sparse_index(lv, offs)
            assert not changed[idx < 0].any()
