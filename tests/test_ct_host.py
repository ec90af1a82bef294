"""Host-side combination-technique logic (no GPU)."""
import math

from paliwa_gb300 import ct as pct


def test_classical_scheme_counts_4d():
    """|l|_1 = 20 - q, l_i >= 1, q = 0..3: 969 + 816 + 680 + 560 grids."""
    levels, coeffs = pct.combination_scheme(4, 20, 3, 1)
    for q, n in enumerate([969, 816, 680, 560]):
        sel = [c for l, c in zip(levels, coeffs) if sum(l) == 20 - q]
        assert len(sel) == n
        assert set(sel) == {(-1) ** q * math.comb(3, q)}
    assert sum(1 << sum(l) for l in levels) == 1695547392


def test_classical_scheme_counts_6d():
    levels, _ = pct.combination_scheme(6, 16, 5, 1)
    assert len(levels) == 7798
    assert sum(1 << sum(l) for l in levels) == 292388864


def test_subspace_count_matches_oracle(oracle_mod):
    levels, _ = pct.combination_scheme(3, 9, 2, 1)
    assert pct.subspace_count(levels) == oracle_mod.subspace_counts(levels)


def test_group_ranges_cover_in_order():
    from paliwa_gb300.ct import group_ranges
    for sizes, groups in (([5, 1, 1, 1, 8, 2, 2], 3), ([1] * 10, 4),
                          ([3], 8), ([1, 1], 5), ([7, 7, 7, 7], 2),
                          (list(range(1, 40)), 8)):
        r = group_ranges(sizes, groups)
        assert r[0][0] == 0 and r[-1][1] == len(sizes)
        assert all(a < b for a, b in r)
        assert all(r[i][1] == r[i + 1][0] for i in range(len(r) - 1))
        assert len(r) <= max(1, min(groups, len(sizes)))
    r = group_ranges([1] * 64, 8)
    assert [b - a for a, b in r] == [8] * 8


def test_launch_code_names():
    """Batch.profile's launch codes (include/paliwa_gb300.h): staged, direct,
    wide, tile, halo and slab kernels, and the TMA wide kernel's forms
    (2048 + R, plus 32 / 64 / 96 / 128 / 160 for the chunked, long, last
    axis, inner extent 2 and long last-axis forms)."""
    from paliwa_gb300 import ct as pct
    names = {
        32: "lift_kernel staged R=32", -16: "lift_kernel direct R=16",
        64 + 8: "wide_kernel R=8", 128 + 16: "wide_kernel last axis R=16",
        192 + 16: "tile_kernel R=16", 256 + 16: "tile_kernel long R=16",
        512: "halo_kernel", 1024: "slab_kernel",
        2048 + 16: "twide_kernel R=16",
        2048 + 32 + 16: "twide_kernel chunked R=16",
        2048 + 64 + 16: "twide_kernel long R=16",
        2048 + 96 + 4: "twide_kernel last axis R=4",
        2048 + 128 + 8: "twide_kernel inner 2 R=8",
        2048 + 160 + 16: "twide_kernel long last axis R=16",
    }
    for code, name in names.items():
        assert pct.kernel_name(code) == name, (code, pct.kernel_name(code))
