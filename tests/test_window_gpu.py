"""transform_in on chunks that hold only a box of the level lattice (GPU).

The reference runs bounds-checked lifting passes whenever a chunk's domain is
not the complete lattice (paliwa/paliwa_transform.hpp:24-51, :224-247): a
point is updated only when it and both periodic neighbours lie in the
chunk. paliwa_gb_transform_in_window does the same on the GPU; these tests
hold it to the oracle's restatement (itself pinned to the reference compiled
here) bit for bit, and fold it over every dimension as hierarchize and
dehierarchize do for such chunks.
"""
import numpy as np
import pytest

import paliwa_gb300 as pg
from paliwa_gb300 import _lib

pytestmark = pytest.mark.gpu

WAVELETS = ["hat", "biorthogonal", "fullweighting"]


def oracle():
    import oracle as O
    O.build()
    return O


def random_window(rng, nd, top=7):
    level = [int(rng.integers(1, top)) for _ in range(nd)]
    lmax = [l + int(rng.integers(0, 3)) for l in level]
    sp = [1 << (L - l) for l, L in zip(level, lmax)]
    front = [int(rng.integers(0, 1 << l)) * s for l, s in zip(level, sp)]
    ext = [int(rng.integers(1, (1 << l) - f // s + 1))
           for l, s, f in zip(level, sp, front)]
    if rng.random() < 0.25:  # the whole axis 0 (its wrapped points are in)
        front[0], ext[0] = 0, 1 << level[0]
    return level, lmax, front, ext


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_windows_match_the_oracle(dtype):
    import torch
    O = oracle()
    rng = np.random.default_rng(17 if dtype == np.float64 else 18)
    for trial in range(150):
        nd = int(rng.integers(1, 4))
        level, lmax, front, ext = random_window(rng, nd)
        dim = int(rng.integers(0, nd))
        lv = list(range(1, level[dim] + 1))
        if trial % 2:
            lv.reverse()
        if trial % 5 == 0:
            filt = [(int(rng.integers(0, 2)),
                     tuple(float(c) for c in rng.uniform(-1, 1, 3)))
                    for _ in range(int(rng.integers(1, 4)))]
        else:
            wav = WAVELETS[trial % 3]
            filt = O.FORWARD[wav] if trial % 4 < 2 else O.INVERSE[wav]
        x = rng.standard_normal(ext).astype(dtype)
        g = torch.from_numpy(x.copy()).cuda()
        pg.transform_in_window(g, dim, level, lmax, lv, filt, front)
        torch.cuda.synchronize()
        want = O.transform_in_window(x.copy(), level, lmax, front, dim, lv,
                                     filt)
        assert np.array_equal(g.cpu().numpy(), want), (trial, level, front,
                                                       ext, dim)


def test_hierarchize_fold_on_windows():
    """hierarchize / dehierarchize of a box: every dimension in order, the
    wavelet's table, levels lmin+1..level (paliwa_transform.hpp:346-431)."""
    import torch
    O = oracle()
    rng = np.random.default_rng(23)
    for trial in range(60):
        nd = int(rng.integers(1, 4))
        level, lmax, front, ext = random_window(rng, nd)
        lmin = [int(rng.integers(0, l + 1)) for l in level]
        wav = WAVELETS[trial % 3]
        x = rng.standard_normal(ext)
        g = torch.from_numpy(x.copy()).cuda()
        want = x.copy()
        for forward in (True, False):
            table = O.FORWARD[wav] if forward else O.INVERSE[wav]
            for d in range(nd):
                lv = list(range(lmin[d] + 1, level[d] + 1))
                if forward:
                    lv.reverse()
                if lv:
                    pg.transform_in_window(g, d, level, lmax, lv, table,
                                           front)
                    O.transform_in_window(want, level, lmax, front, d, lv,
                                          table)
            torch.cuda.synchronize()
            assert np.array_equal(g.cpu().numpy(), want), trial


def test_window_argument_errors():
    import torch
    g = torch.zeros(4, dtype=torch.float64, device="cuda")
    hat = [(1, (-0.5, 1.0, -0.5))]
    with pytest.raises(_lib.InvalidArgument):  # wraps around the period
        pg.transform_in_window(g, 0, (3,), (3,), [3], hat, (6,))
    with pytest.raises(_lib.InvalidArgument):  # off the lattice
        pg.transform_in_window(g, 0, (2,), (3,), [2], hat, (1,))
    with pytest.raises(_lib.InvalidArgument):  # level beyond the grid's
        pg.transform_in_window(g, 0, (3,), (3,), [4], hat, (0,))
    with pytest.raises(_lib.PaliwaError, match="Filter offset"):
        pg.transform_in_window(g, 0, (3,), (3,), [3], [(2, (0, 1, 0))], (0,))
