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
