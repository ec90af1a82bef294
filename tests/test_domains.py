"""Index maps (paliwa_domains.hpp) and combination-technique sizes against
the reference's known answers (no GPU needed)."""
import itertools

import numpy as np
import pytest

import paliwa_gb300 as pg


def test_restrict_strided_domain_known_answers():
    """test/test_paliwa_restrict.cpp:19-47."""
    full = pg.strided_domain_from_level((3, 3), (4, 4))  # indices 0, 2, .. 14
    r = pg.restrict_strided_with_discrete(full, (1, 4), (5, 12))
    assert r.front == (2, 4)
    assert r.back() == (4, 12)
    r2 = pg.restrict_strided_with_discrete(full, (None, 4), (None, 11))
    assert r2.front == (0, 4)
    assert r2.back() == (14, 10)


def test_strided_domain_from_level_matches_oracle(oracle_mod):
    rng = np.random.default_rng(1)
    for _ in range(200):
        d = int(rng.integers(1, 7))
        L = rng.integers(0, 20, size=d)
        l = [int(rng.integers(0, x + 1)) for x in L]
        dom = pg.strided_domain_from_level(l, L)
        assert (dom.front, dom.extents, dom.strides) == \
            oracle_mod.strided_domain_from_level(l, L)
        h = pg.strided_hierarchical_domain_from_level(l, L)
        assert (h.front, h.extents, h.strides) == \
            oracle_mod.strided_hierarchical_domain_from_level(l, L)
        for dim in range(d):
            if dom.extents[dim] < 2:
                continue
            ev = pg.even_strided_domain_from_domain(dom, dim)
            od = pg.odd_strided_domain_from_domain(dom, dim)
            t = (dom.front, dom.extents, dom.strides)
            assert (ev.front, ev.extents, ev.strides) == \
                oracle_mod.even_strided_domain_from_domain(t, dim)
            assert (od.front, od.extents, od.strides) == \
                oracle_mod.odd_strided_domain_from_domain(t, dim)


def test_hierarchical_subspaces_partition_the_grid():
    """Every point of the level-l grid lies in exactly one hierarchical
    subspace 0 <= s <= l (paliwa_domains.hpp:51-83, paliwa_utils.hpp:9-26)."""
    level, L = (3, 2), (4, 5)
    grid = pg.strided_domain_from_level(level, L)
    seen = {}
    for s in itertools.product(*[range(x + 1) for x in level]):
        for p in pg.strided_hierarchical_domain_from_level(s, L).points():
            seen[p] = seen.get(p, 0) + 1
    assert sorted(seen) == sorted(grid.points())
    assert set(seen.values()) == {1}


CT_SCHEMES = {
    # test/test_paliwa_combination_technique.cpp:105-122
    2: [(2, 11), (3, 10), (4, 9), (5, 8), (6, 7), (7, 6), (8, 5), (9, 4),
        (10, 3), (2, 10), (3, 9), (4, 8), (5, 7), (6, 6), (7, 5), (8, 4),
        (9, 3)],
    3: [(4, 6, 7), (5, 5, 7), (5, 6, 6), (4, 5, 6)],
    4: [(2, 2, 4, 4), (3, 2, 3, 4), (1, 4, 3, 4), (1, 2, 5, 4), (2, 3, 3, 4),
        (1, 3, 4, 4), (2, 2, 3, 5), (1, 3, 3, 5), (1, 2, 3, 6), (1, 2, 4, 5),
        (1, 2, 4, 4), (2, 2, 3, 4), (1, 3, 3, 4), (1, 2, 3, 5), (1, 2, 3, 4)],
}
CT_MAX = {2: (10, 11), 3: (5, 6, 7), 4: (3, 4, 5, 6)}


@pytest.mark.parametrize("d,full,sparse", [(2, 106496, 18432),
                                           (3, 425984, 131072),
                                           (4, 50176, 5120)])
def test_combination_sizes_known_answers(oracle_mod, d, full, sparse):
    """test/test_paliwa_combination_technique.cpp:139-145 and :226-232."""
    levels = CT_SCHEMES[d]
    doms = pg.get_strided_domains(levels, CT_MAX[d])
    assert sum(x.size() for x in doms) == full
    kept = oracle_mod.kept_subspaces(levels)
    assert sum(oracle_mod.subspace_size(s) for s in kept) == sparse
    assert sum(pg.strided_hierarchical_domain_from_level(s, CT_MAX[d]).size()
               for s in kept) == sparse
