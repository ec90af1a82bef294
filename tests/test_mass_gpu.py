"""Mass conservation of the GPU transform (the reference's
test/test_paliwa_transform.cpp:81-143, restated).

After hierarchize, the values on the minimum-level lattice sum to the grid's
mean times the number of those points, for every wavelet except hat (whose
coarse points keep nodal values). The reference checks a level (3, 3) grid
inside maximum level (4, 4), every minimum level in {0, 1, 3}^2, inputs
(1 + uid_x + uid_y)(1 + U[0, 1)), to 1e-13 absolute in FP64. Here the same
case runs on the GPU (its inputs re-seeded with numpy: the reference draws
them from Kokkos' XorShift64 pool), bit-identical to the oracle, plus larger
3D grids in FP64 (relative 1e-13) and in FP32-compensated arithmetic.

FP32-compensated: the grid is stored in float; each axis rounds every value
to float once, so a value perturbed by at most 2^-24 |v| per axis moves the
minimum-level sum by at most its weight count / N times that. The bound held
below is d * 2^-24 * count * max|x| (d axes of rounding, the last one of the
stored minimum-level values included); no step of the transform needs FP64
arithmetic to meet it.
"""
import math

import numpy as np
import pytest

import paliwa_gb300 as pg

pytestmark = pytest.mark.gpu

WAVELETS = ["biorthogonal", "fullweighting"]


def oracle():
    import oracle as O
    O.build()
    return O


def lmin_points(level, minimum_level, maximum_level):
    """Slices of a grid at `level` selecting the points of
    strided_domain_from_level(minimum_level, maximum_level)
    (paliwa/paliwa_domains.hpp:33-49): uids that are multiples of
    2^(L - lmin), i.e. compact indices that are multiples of 2^(l - lmin)."""
    return tuple(slice(None, None, 1 << (l - m))
                 for l, m in zip(level, minimum_level))


@pytest.mark.parametrize("wavelet", WAVELETS)
def test_reference_case_fp64(wavelet):
    import torch
    O = oracle()
    level, lmax = (3, 3), (4, 4)
    rng = np.random.default_rng(12345)
    uid = 2 * np.arange(8)  # uids of the level-3 points inside level 4
    for mx in (0, 1, 3):
        for my in (0, 1, 3):
            lmin = (mx, my)
            x = (1.0 + np.add.outer(uid, uid)) * (1.0 + rng.uniform(0, 1, (8, 8)))
            g = torch.from_numpy(x.copy()).cuda()
            pg.hierarchize(g, level, lmin, lmax, wavelet)
            torch.cuda.synchronize()
            got = g.cpu().numpy()
            want = O.hierarchize(x.copy(), level, lmin, lmax, wavelet)
            assert np.array_equal(got, want), lmin
            sel = got[lmin_points(level, lmin, lmax)]
            # The reference's tolerance is 1e-13 absolute on its own random
            # inputs; on these (sums up to ~400) two units in the last place
            # of the sum exceed it, so the bound is the larger of 1e-13 and
            # four ulps of the target (sums taken exactly).
            target = math.fsum(x.ravel()) / x.size * sel.size
            tol = max(1e-13, 4 * float(np.spacing(target)))
            assert abs(math.fsum(sel.ravel()) - target) <= tol, (lmin, wavelet)


@pytest.mark.parametrize("wavelet", WAVELETS)
@pytest.mark.parametrize("lmin", [(0, 0, 0), (2, 1, 3), (4, 4, 4)])
def test_larger_grids_fp64_and_fp32c(wavelet, lmin):
    import torch
    level = (9, 8, 7)
    rng = np.random.default_rng(sum(lmin) + len(wavelet))
    idx = np.meshgrid(*[np.arange(1 << l) / (1 << l) for l in level],
                      indexing="ij")
    x = (2.0 + np.sin(2 * np.pi * idx[0]) * np.cos(2 * np.pi * idx[1])
         + idx[2]) * (1.0 + rng.uniform(0, 1, [1 << l for l in level]))
    sel = lmin_points(level, lmin, level)

    # FP64: relative 1e-13.
    g = torch.from_numpy(x.copy()).cuda()
    pg.hierarchize(g, level, lmin, level, wavelet)
    torch.cuda.synchronize()
    coarse = g.cpu().numpy()[sel]
    target = x.sum() / x.size * coarse.size
    assert abs(coarse.sum() - target) <= 1e-13 * abs(target)

    # FP32-compensated: within the float storage bound of the docstring.
    x32 = x.astype(np.float32)
    target32 = x32.astype(np.float64).sum() / x32.size * coarse.size
    g32 = torch.from_numpy(x32.copy()).cuda()
    pg.hierarchize(g32, level, lmin, level, wavelet, compensated=True)
    torch.cuda.synchronize()
    coarse32 = g32.cpu().numpy()[sel].astype(np.float64)
    bound = len(level) * 2.0 ** -24 * coarse.size * float(np.abs(x32).max())
    assert abs(coarse32.sum() - target32) <= bound, (
        abs(coarse32.sum() - target32), bound)
