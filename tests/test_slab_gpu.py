"""The slab kernel: every level of a grid's trailing axes in one pass
(paliwa_gb300/csrc/slab.cuh), in batches.

Its results are the per-axis plan's bits (the same updates in the same
order), so every case compares a batch planned with slab launches against
the same batch planned axis by axis -- FP64, FP32 and FP32-compensated,
both directions -- and FP64 also against the oracle. The bounded waits of
the kernel report no timeout.
"""
import itertools

import numpy as np
import pytest

from paliwa_gb300 import ct as pct

pytestmark = pytest.mark.gpu

WAVELETS = ["hat", "biorthogonal", "fullweighting"]


def oracle():
    import oracle as O
    O.build()
    return O


def scheme(ndim, top, qmax, lmin=1):
    return [l for q in range(qmax + 1)
            for l in itertools.product(range(lmin, top + 1), repeat=ndim)
            if sum(l) == top - q]


def run_pair(levels, lmin, lmax, wavelet, dtype, compensated, seed):
    import torch
    rng = np.random.default_rng(seed)
    host = [rng.uniform(-1, 1, 1 << sum(l)) for l in levels]
    out = []
    for slabs in (True, False):
        buf, views = pct.packed_grids(levels, dtype)
        for v, h in zip(views, host):
            v.copy_(torch.from_numpy(h.astype(np.float64)).to(dtype))
        torch.cuda.synchronize()
        s = torch.cuda.Stream()
        bt = pct.Batch(views, levels, lmin, lmax, wavelet,
                       compensated=compensated, slabs=slabs)
        bt.hierarchize(s)
        s.synchronize()
        f = buf.clone()
        bt.dehierarchize(s)
        s.synchronize()
        bt.status()
        esz = buf.element_size()
        starts = [(v.data_ptr() - buf.data_ptr()) // esz for v in views]
        out.append((f, buf.clone(), starts))
        # The kernels of the forward plan (this runs it once more, after
        # the results were taken).
        _, _, kernels = bt.profile(forward=True, stream=s)
        s.synchronize()
        bt.status()
        out[-1] += (kernels,)
        bt.close()
    return host, out


@pytest.mark.parametrize("dtype_name", ["f64", "f32", "f32c"])
@pytest.mark.parametrize("case", [(3, 10, 2), (4, 12, 3), (5, 11, 2),
                                  (6, 12, 2), (2, 14, 2)])
def test_slab_plan_equals_per_axis_plan(dtype_name, case):
    import torch
    ndim, top, qmax = case
    levels = scheme(ndim, top, qmax)
    lmin, lmax = (1,) * ndim, (top,) * ndim
    dtype = torch.float64 if dtype_name == "f64" else torch.float32
    for w, wavelet in enumerate(WAVELETS):
        host, ((f1, b1, v1, k1), (f2, b2, _, k2)) = run_pair(
            levels, lmin, lmax, wavelet, dtype, dtype_name == "f32c",
            100 * ndim + top + w)
        assert pct.SLAB_KERNEL in k1 and pct.SLAB_KERNEL not in k2
        assert torch.equal(f1, f2), (case, wavelet)
        assert torch.equal(b1, b2), (case, wavelet)
        if dtype_name == "f64" and w == 1:
            O = oracle()
            for i in range(0, len(levels), max(1, len(levels) // 40)):
                lv = levels[i]
                off = v1[i]  # the grid's first element in the buffer
                got = f1[off:off + (1 << sum(lv))].cpu().numpy()
                want = O.hierarchize(
                    host[i].reshape([1 << l for l in lv]).copy(), lv, lmin,
                    lmax, wavelet).reshape(-1)
                assert np.array_equal(got, want), (case, lv)


def test_slab_lmin_zero_and_single_tile_grids():
    """Grids of one tile or less (down to 1 KB), minimum level 0 and axes
    of a single point."""
    import torch
    levels = [(0, 3, 5), (2, 0, 6), (1, 1, 7), (3, 4, 1), (5, 5, 0),
              (2, 2, 4), (4, 6, 2), (1, 7, 7)]
    lmin, lmax = (0, 0, 0), (7, 7, 7)
    for dtype, comp in ((torch.float64, False), (torch.float32, True)):
        host, ((f1, b1, _, k1), (f2, b2, _, _)) = run_pair(
            levels, lmin, lmax, "biorthogonal", dtype, comp, 5)
        assert pct.SLAB_KERNEL in k1
        assert torch.equal(f1, f2)
        assert torch.equal(b1, b2)
