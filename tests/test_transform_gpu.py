"""GPU parity: the sm_103a kernels against the CPU oracle, through the C ABI.

FP64 and plain FP32 are bit-identical to the oracle (the reference's
arithmetic with its evaluation order). FP32-compensated is checked against
the FP64 oracle with a normwise tolerance of 1e-6 (max |err| / max |ref|).
"""
import numpy as np
import pytest

import paliwa_gb300 as pg

pytestmark = pytest.mark.gpu

WAVELETS = ["hat", "biorthogonal", "fullweighting"]
F32C_TOL = 1e-6


def torch_dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def gpu_transform(x, level, lmin, lmax, wavelet, forward, compensated=False):
    t = torch_dev(x)
    fn = pg.hierarchize if forward else pg.dehierarchize
    fn(t, level, lmin, lmax, wavelet, compensated=compensated)
    return host(t)


def random_input(level, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, [1 << l for l in level])


SHAPES = [
    ((1,), (0,)), ((2,), (0,)), ((5,), (1,)), ((9,), (0,)), ((12,), (3,)),
    ((13,), (0,)),
    ((6, 6), (0, 0)), ((3, 3), (1, 3)), ((4, 9), (2, 0)), ((10, 2), (0, 1)),
    ((1, 12), (0, 5)),
    ((5, 4, 3), (0, 1, 2)), ((2, 7, 5), (1, 0, 0)), ((3, 1, 8), (0, 0, 0)),
    ((2, 2, 3, 4), (1, 0, 2, 0)), ((3, 2, 1, 2, 1, 2), (0, 0, 0, 1, 0, 0)),
]


@pytest.mark.parametrize("wavelet", WAVELETS)
@pytest.mark.parametrize("level,lmin", SHAPES)
def test_f64_bit_exact(level, lmin, wavelet):
    lmax = tuple(l + 2 for l in level)
    x = random_input(level, sum(level) + 11)
    for forward in (True, False):
        want = import_oracle().hierarchize(x.copy(), level, lmin, lmax,
                                           wavelet, forward=forward)
        got = gpu_transform(x, level, lmin, lmax, wavelet, forward)
        assert np.array_equal(got, want), (level, lmin, wavelet, forward)


@pytest.mark.parametrize("wavelet", WAVELETS)
@pytest.mark.parametrize("level,lmin", SHAPES[::2])
def test_f32_plain_bit_exact(level, lmin, wavelet):
    lmax = tuple(level)
    x = random_input(level, 5).astype(np.float32)
    for forward in (True, False):
        want = import_oracle().hierarchize(x.copy(), level, lmin, lmax,
                                           wavelet, forward=forward)
        got = gpu_transform(x, level, lmin, lmax, wavelet, forward)
        assert np.array_equal(got, want)


@pytest.mark.parametrize("wavelet", WAVELETS)
@pytest.mark.parametrize("level,lmin", SHAPES)
def test_f32_compensated_error(level, lmin, wavelet):
    lmax = tuple(level)
    x = random_input(level, 9)
    for forward in (True, False):
        want = import_oracle().hierarchize(x.copy(), level, lmin, lmax,
                                           wavelet, forward=forward)
        got = gpu_transform(x.astype(np.float32), level, lmin, lmax, wavelet,
                            forward, compensated=True).astype(np.float64)
        scale = max(np.max(np.abs(want)), 1e-300)
        err = np.max(np.abs(got - want)) / scale
        assert err <= F32C_TOL, (level, wavelet, forward, err)


# Partly filled warps and tiles of the wide kernel: strided pencils of 32 or
# 64 points with one or two column groups, last-axis pencils with fewer
# pencils than a warp holds, narrow inner extents.
WIDE_EDGE = [((5, 1), (0, 0)), ((6, 1), (1, 0)), ((1, 5), (0, 0)),
             ((2, 6), (0, 1)), ((1, 9), (0, 0)), ((3, 4), (0, 0)),
             ((4, 2, 1), (0, 0, 0)), ((2, 2, 5), (0, 0, 0)),
             ((6, 3, 2), (1, 0, 0)), ((3, 7, 1), (0, 2, 0))]


@pytest.mark.parametrize("wavelet", WAVELETS)
@pytest.mark.parametrize(
    "level,lmin", [s for s in SHAPES + WIDE_EDGE if max(s[0]) <= 12])
def test_f32_compensated_bit_exact_model(level, lmin, wavelet):
    """Every kernel's FP32-compensated arithmetic, bit for bit, against the
    numpy model of the same operations (one rounding to FP32 per axis).
    Pencils longer than 4096 points run in several stages per axis (windowed
    fine levels, sub-lattice coarse levels), each ending in a rounding to
    FP32; those shapes are held to the FP64 tolerance instead."""
    from compensated import hierarchize as model
    x = random_input(level, 13).astype(np.float32)
    for forward in (True, False):
        want = model(x, level, lmin, wavelet, forward)
        got = gpu_transform(x, level, lmin, tuple(level), wavelet, forward,
                            compensated=True)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (
            level, lmin, wavelet, forward)


@pytest.mark.parametrize("wavelet", WAVELETS)
@pytest.mark.parametrize("level,lmin", WIDE_EDGE)
def test_wide_edges_bit_exact(level, lmin, wavelet):
    """FP64 and FP32 through the wide kernel's partly filled warps."""
    for dt in (np.float64, np.float32):
        x = random_input(level, 17).astype(dt)
        for forward in (True, False):
            want = import_oracle().hierarchize(x.copy(), level, lmin,
                                               tuple(level), wavelet,
                                               forward=forward)
            got = gpu_transform(x, level, lmin, tuple(level), wavelet,
                                forward)
            assert np.array_equal(got, want), (level, dt, wavelet, forward)


# Strided pencils of 128 to 4096 points on the tile kernel: chunks exchanged
# by shuffle (G <= 32) and through shared memory (G > 32), 8- and 16-byte
# copy pieces, inner extents narrower than a tile row, partial tiles.
TILE_SHAPES = [((7, 3), (0, 0)), ((8, 2), (1, 0)), ((9, 4), (0, 1)),
               ((10, 2), (0, 1)), ((11, 3), (2, 0)), ((12, 2), (0, 0)),
               ((2, 10, 3), (0, 1, 0)), ((8, 1, 2), (0, 0, 0)),
               ((9, 6), (3, 0))]


@pytest.mark.parametrize("wavelet", WAVELETS)
@pytest.mark.parametrize("level,lmin", TILE_SHAPES)
def test_tile_shapes_exact(level, lmin, wavelet):
    """FP64 and FP32 bit-identical to the oracle, FP32c bit-identical to
    the compensated model, forward and inverse."""
    from compensated import hierarchize as model
    O = import_oracle()
    for dt in (np.float64, np.float32):
        x = random_input(level, 23).astype(dt)
        for forward in (True, False):
            want = O.hierarchize(x.copy(), level, lmin, tuple(level), wavelet,
                                 forward=forward)
            got = gpu_transform(x, level, lmin, tuple(level), wavelet,
                                forward)
            assert np.array_equal(got, want), (level, dt, wavelet, forward)
    x = random_input(level, 29).astype(np.float32)
    for forward in (True, False):
        want = model(x, level, lmin, wavelet, forward)
        got = gpu_transform(x, level, lmin, tuple(level), wavelet, forward,
                            compensated=True)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


LONG = [((14,), (0,)), ((15,), (2,)), ((17,), (0,)), ((16, 1), (3, 0)),
        ((2, 15), (0, 0)), ((14, 2), (0, 1)), ((1, 1, 1, 17), (1, 1, 1, 1))]


@pytest.mark.parametrize("wavelet", WAVELETS)
@pytest.mark.parametrize("level,lmin", LONG)
def test_long_pencils_bit_exact(level, lmin, wavelet):
    """Pencils longer than one CTA holds: fine levels on windows with halos,
    coarse levels on the strided sub-lattice."""
    lmax = tuple(level)
    x = random_input(level, 21)
    for forward in (True, False):
        want = import_oracle().hierarchize(x.copy(), level, lmin, lmax,
                                           wavelet, forward=forward)
        got = gpu_transform(x, level, lmin, lmax, wavelet, forward)
        assert np.array_equal(got, want), (level, wavelet, forward)


def golden_filters(passes, mask):
    return [((1 if mask & (1 << p) else 0),
             (0.0, 1.0, 0.25) if p % 2 else (-0.5, 1.0, 0.125))
            for p in range(passes)]


def test_transform_in_reference_loop_golden():
    """transform_in with the generic filter lists of
    test/test_paliwa_plan.cpp:114-163 matches the committed golden vectors of
    the reference's own 1D loop, bit for bit."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden",
                             "plan_multipass.npz"))
    for (passes, mask, order), expected in zip(g["cases"], g["output"]):
        levels = [4, 3, 2, 1] if order == 0 else [1, 2, 3, 4]
        t = torch_dev(g["input"][::4].copy())
        pg.transform_in(t, 0, (4,), (6,), levels, golden_filters(passes, mask))
        assert np.array_equal(host(t), expected[::4]), (passes, mask, order)


@pytest.mark.parametrize("level,dim", [((6, 5), 0), ((6, 5), 1), ((3, 14), 1),
                                       ((15, 2), 0)])
def test_transform_in_general_coefficients(level, dim):
    """Coefficients that are not powers of two use separately rounded
    products and sums: still bit-identical to the oracle. Levels in any
    order, repeated levels included."""
    filters = [(1, (-0.3, 1.1, 0.7)), (0, (0.2, 0.9, -0.15)),
               (1, (0.1, 1.0, 0.1))]
    lev = level[dim]
    levels = [lev, 1, 2, lev - 1, 2]
    lmax = tuple(l + 1 for l in level)
    x = random_input(level, 4)
    want = import_oracle().transform_in(x.copy(), level, lmax, dim, levels,
                                        filters)
    t = torch_dev(x)
    pg.transform_in(t, dim, level, lmax, levels, filters)
    assert np.array_equal(host(t), want)


def test_per_dimension_calls_compose():
    level, lmin, lmax = (4, 5, 3), (1, 0, 2), (4, 5, 3)
    x = random_input(level, 8)
    want = import_oracle().hierarchize(x.copy(), level, lmin, lmax,
                                       "biorthogonal")
    t = torch_dev(x)
    for d in range(3):
        assert pg.hierarchize_in(t, d, level, lmin, lmax, "biorthogonal")
    assert np.array_equal(host(t), want)
    for d in range(3):
        pg.dehierarchize_in(t, d, level, lmin, lmax, "biorthogonal")
    assert np.max(np.abs(host(t) - x)) <= 1e-13


def test_errors_on_gpu():
    import torch
    t = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(pg.PaliwaError, match="Filter offset not supported"):
        pg.transform_in(t, 0, (4,), (4,), [4], [(2, (0.0, 1.0, 0.0))])
    with pytest.raises(pg.OutOfRange):
        pg.hierarchize(t, (4,), (0,), (4,), "nope")
    with pytest.raises(pg.InvalidArgument):
        pg.hierarchize(t, (4,), (5,), (4,), "hat")
    with pytest.raises(pg.InvalidArgument):
        pg.hierarchize(t, (3,), (0,), (4,), "hat")  # wrong size
    with pytest.raises(pg.InvalidArgument):
        pg.hierarchize(t.cpu(), (4,), (0,), (4,), "hat")


def import_oracle():
    import oracle
    oracle.build()
    return oracle


CT_SHAPES = [(17, 1, 1, 1), (1, 17, 1, 1), (1, 1, 17, 1), (1, 1, 1, 17),
             (12, 2, 3, 3), (3, 12, 2, 3), (2, 3, 12, 3), (5, 5, 5, 5),
             (1, 1, 9, 9), (14, 1, 2, 3)]


@pytest.mark.parametrize("level", CT_SHAPES)
def test_ct_shapes_f64_exact_and_f32c_error(level):
    """Component-grid shapes of the 4D combination technique (|l|_1 = 17..20,
    l >= 1), lmin = 1: FP64 bit-exact, FP32c within 1e-6 of FP64, single grid
    and in one batch."""
    from paliwa_gb300 import ct as pct
    lmin = (1, 1, 1, 1)
    lmax = (17, 17, 17, 17)
    x = random_input(level, 31)
    O = import_oracle()
    for forward in (True, False):
        want = O.hierarchize(x.copy(), level, lmin, lmax, "biorthogonal",
                             forward=forward)
        got = gpu_transform(x, level, lmin, lmax, "biorthogonal", forward)
        assert np.array_equal(got, want)
        got32 = gpu_transform(x.astype(np.float32), level, lmin, lmax,
                              "biorthogonal", forward, compensated=True)
        err = np.max(np.abs(got32 - want)) / np.max(np.abs(want))
        assert err <= F32C_TOL, (level, forward, err)


def test_ct_shapes_in_one_batch_f32c():
    import torch
    from paliwa_gb300 import ct as pct
    lmin, lmax = (1, 1, 1, 1), (17, 17, 17, 17)
    xs = [random_input(l, i) for i, l in enumerate(CT_SHAPES)]
    O = import_oracle()
    wants = [O.hierarchize(x.copy(), l, lmin, lmax, "biorthogonal")
             for x, l in zip(xs, CT_SHAPES)]
    buf, gs = pct.packed_grids(CT_SHAPES, torch.float32)
    for g, x in zip(gs, xs):
        g.copy_(torch.from_numpy(x.astype(np.float32).reshape(-1)))
    torch.cuda.synchronize()
    b = pct.Batch(gs, CT_SHAPES, lmin, lmax, "biorthogonal", compensated=True)
    s = torch.cuda.Stream()
    b.hierarchize(s)
    s.synchronize()
    for g, w, l in zip(gs, wants, CT_SHAPES):
        got = g.double().cpu().numpy().reshape(w.shape)
        err = np.max(np.abs(got - w)) / np.max(np.abs(w))
        assert err <= F32C_TOL, (l, err)


@pytest.mark.parametrize("level", [(18, 4), (3, 17, 2)])
def test_long_pencils_many_tiles(level):
    """Grids large enough that persistent CTAs process many windows each."""
    lmin = (0,) * len(level)
    x = random_input(level, 12)
    O = import_oracle()
    for forward in (True, False):
        want = O.hierarchize(x.copy(), level, lmin, level, "biorthogonal",
                             forward=forward)
        got = gpu_transform(x, level, lmin, level, "biorthogonal", forward)
        assert np.array_equal(got, want), (level, forward)
        got32 = gpu_transform(x.astype(np.float32), level, lmin, level,
                              "biorthogonal", forward, compensated=True)
        err = np.max(np.abs(got32 - want)) / np.max(np.abs(want))
        assert err <= F32C_TOL
