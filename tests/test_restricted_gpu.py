"""Restricted-output transform on the GPU (paliwa_gb_transform_outputs)
against the oracle's restatement (oracle/restricted.py), bit for bit over
the whole window buffer: outputs, the intermediate values left in their
dependency cone, and every untouched point."""
import random

import numpy as np
import pytest

import oracle
import restricted as R
from paliwa_gb300 import _lib, transform as T

pytestmark = pytest.mark.gpu

WAVELET_PASSES = [
    oracle.FORWARD["hat"], oracle.INVERSE["hat"],
    oracle.FORWARD["biorthogonal"], oracle.INVERSE["biorthogonal"],
    oracle.FORWARD["fullweighting"], oracle.INVERSE["fullweighting"],
]


def random_case(rng, dtype, max_dims=3):
    nd = rng.randint(1, max_dims)
    level = [rng.randint(1, 7 if nd == 1 else (5 if nd <= 3 else 3))
             for _ in range(nd)]
    maximum = [l + rng.randint(0, 2) for l in level]
    dim = rng.randrange(nd)
    lmin = rng.randrange(level[dim])
    levels = list(range(lmin + 1, level[dim] + 1))
    if rng.randrange(2):
        levels.reverse()
    kind = rng.randrange(3)
    if kind == 0:
        filters = rng.choice(WAVELET_PASSES)
    elif kind == 1:  # powers of two: the fused (exact-product) arithmetic
        filters = [(rng.randrange(2),
                    tuple(rng.choice([0.0, 0.25, -0.5, 1.0, 0.125, 2.0])
                          for _ in range(3)))
                   for _ in range(rng.randint(1, 5))]
    else:  # general coefficients: separately rounded products and sums
        filters = [(rng.randrange(2),
                    tuple(rng.uniform(-1.0, 1.0) for _ in range(3)))
                   for _ in range(rng.randint(1, 5))]
    sp = [1 << (maximum[d] - level[d]) for d in range(nd)]
    per = [1 << maximum[d] for d in range(nd)]
    n = [1 << level[d] for d in range(nd)]
    # Outputs: an interval along dim (may wrap), strided boxes elsewhere.
    ofront, oext, ostr = [], [], []
    for d in range(nd):
        if d == dim:
            cnt = rng.randint(1, n[d])
            ofront.append(rng.randrange(n[d]) * sp[d])
            oext.append(cnt)
            ostr.append(sp[d])
        else:
            step = rng.choice([1, 1, 2])
            cnt = rng.randint(1, max(1, n[d] // step))
            ofront.append(rng.randrange(n[d]) * sp[d])
            oext.append(cnt)
            ostr.append(step * sp[d])
    # Window: covers the required inputs along dim (plus a random margin,
    # wrapping where it falls), and the outputs elsewhere.
    first = ofront[dim]
    last = (first + (oext[dim] - 1) * ostr[dim]) % per[dim]
    bounds = R.transform_bounds((first, last), level[dim], maximum[dim],
                                levels, filters)
    need = sorted(set(R.transform_indices(bounds, maximum[dim])) |
                  {(first + k * ostr[dim]) % per[dim]
                   for k in range(oext[dim])})
    wfront, wext = [], []
    for d in range(nd):
        if d == dim:
            cov = R.covering_periodic_bounds(need, per[d])
            ext = ((cov[1] - cov[0]) % per[d]) // sp[d] + 1
            before = rng.randint(0, n[d] - ext)
            after = rng.randint(0, n[d] - ext - before)
            wfront.append((cov[0] - before * sp[d]) % per[d])
            wext.append(ext + before + after)
        else:
            span = (oext[d] - 1) * (ostr[d] // sp[d]) + 1
            before = rng.randint(0, n[d] - span)
            wfront.append((ofront[d] - before * sp[d]) % per[d])
            wext.append(span + before + rng.randint(0, n[d] - span - before))
    buf = np.asarray(
        np.random.default_rng(rng.randrange(1 << 30)).uniform(-1, 1, wext),
        dtype=dtype)
    return dict(buf=buf, front=wfront, level=level, maximum=maximum,
                dim=dim, levels=levels, filters=filters,
                outputs=(ofront, oext, ostr))


def run_gpu(c):
    import torch
    g = torch.from_numpy(c["buf"].copy()).cuda()
    T.transform_outputs(g, c["dim"], c["level"], c["maximum"], c["levels"],
                        c["filters"], c["outputs"], window_front=c["front"])
    torch.cuda.synchronize()
    return g.cpu().numpy()


def run_oracle(c):
    b = c["buf"].copy()
    R.transform_outputs(b, c["front"], c["level"], c["maximum"], c["dim"],
                        c["levels"], c["filters"], *c["outputs"])
    return b


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_random_windows_match_oracle(dtype):
    rng = random.Random(20261203 if dtype == np.float64 else 17)
    for trial in range(120):
        c = random_case(rng, dtype)
        got, want = run_gpu(c), run_oracle(c)
        assert np.array_equal(got, want), (trial, c["level"], c["dim"],
                                           c["levels"], c["outputs"],
                                           c["front"], c["buf"].shape)


def test_random_windows_up_to_5d():
    rng = random.Random(5)
    for trial in range(60):
        c = random_case(rng, np.float64, max_dims=5)
        got, want = run_gpu(c), run_oracle(c)
        assert np.array_equal(got, want), (trial, c["level"], c["dim"])


@pytest.mark.parametrize("wavelet", ["hat", "biorthogonal", "fullweighting"])
def test_full_outputs_equal_full_transform(wavelet):
    """Outputs = the whole grid: the restricted transform is transform_in."""
    import torch
    level, maximum = (5, 4, 6), (6, 4, 7)
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, [1 << l for l in level])
    for dim in range(3):
        for filters, levels in (
                (oracle.FORWARD[wavelet], list(range(level[dim], 0, -1))),
                (oracle.INVERSE[wavelet], list(range(1, level[dim] + 1)))):
            want = x.copy()
            oracle.transform_in(want, level, maximum, dim, levels, filters)
            g = torch.from_numpy(x.copy()).cuda()
            sp = [1 << (m - l) for l, m in zip(level, maximum)]
            T.transform_outputs(g, dim, level, maximum, levels, filters,
                                ((0, 0, 0), [1 << l for l in level], sp))
            torch.cuda.synchronize()
            assert np.array_equal(g.cpu().numpy(), want)


def test_slab_with_periodic_halo():
    """A slab at the periodic edge of a 2D grid in one wrapped window
    buffer, forward and inverse, equals the full transform on the slab."""
    import torch
    level, maximum = (7, 5), (7, 6)
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, [1 << l for l in level])
    dim, start, count = 0, 120, 16  # points 120..127, 0..7
    period = 1 << maximum[0]
    filters = oracle.FORWARD["biorthogonal"]
    levels = list(range(level[0], 0, -1))
    full = x.copy()
    oracle.transform_in(full, level, maximum, dim, levels, filters)
    bounds = R.transform_bounds((start, (start + count - 1) % period),
                                level[0], maximum[0], levels, filters)
    need = sorted(set(R.transform_indices(bounds, maximum[0])) |
                  {(start + k) % period for k in range(count)})
    cov = R.covering_periodic_bounds(need, period)
    ext = (cov[1] - cov[0]) % period + 1
    idx = (cov[0] + np.arange(ext)) % period
    buf = np.ascontiguousarray(x[idx])
    g = torch.from_numpy(buf.copy()).cuda()
    T.transform_outputs(g, dim, level, maximum, levels, filters,
                        ((start, 0), (count, 1 << level[1]), (1, 2)),
                        window_front=(cov[0], 0))
    torch.cuda.synchronize()
    got = g.cpu().numpy()
    for k in range(count):
        u = (start + k) % period
        j = (u - cov[0]) % period
        assert np.array_equal(got[j], full[u])


def test_errors():
    import torch
    level, maximum = (4,), (4,)
    filters = oracle.FORWARD["hat"]
    g = torch.zeros(8, dtype=torch.float64, device="cuda")
    # The window holds uids 0..7; outputs 4..7 need inputs beyond it.
    with pytest.raises(_lib.PaliwaError):
        T.transform_outputs(g, 0, level, maximum, [4, 3, 2, 1], filters,
                            ((4,), (4,), (1,)))
    with pytest.raises(_lib.InvalidArgument):  # levels not consecutive
        T.transform_outputs(g, 0, level, maximum, [4, 2], filters,
                            ((0,), (1,), (1,)))
    with pytest.raises(_lib.InvalidArgument):  # front off the grid
        T.transform_outputs(torch.zeros(8, dtype=torch.float64,
                                        device="cuda"), 0, (3,), (4,),
                            [3], filters, ((0,), (1,), (2,)),
                            window_front=(1,))
    # Compensated FP32 is not available for restricted outputs.
    lib = _lib.load()
    rc = lib.paliwa_gb_transform_outputs(
        g.data_ptr(), _lib.F32C, 1, _lib.i64(level), _lib.i64(maximum),
        _lib.i64([0]), _lib.i64([8]), 0, _lib.i64([4]), 1, _lib.i32([1]),
        _lib.f64([-0.5, 1.0, -0.5]), 1, _lib.i64([0]), _lib.i64([1]),
        _lib.i64([1]), None)
    assert rc == _lib.INVALID_ARGUMENT
    # Empty outputs return at once, whatever the window.
    T.transform_outputs(g, 0, level, maximum, [4, 3, 2, 1], filters,
                        ((4,), (0,), (1,)))


@pytest.mark.parametrize("wavelet", ["hat", "biorthogonal", "fullweighting"])
@pytest.mark.parametrize("slabs", [2, 4])
def test_slab_decomposition_equals_serial(wavelet, slabs):
    """The single-GPU form of the reference's distributed-vs-serial tests
    (test/test_paliwa_distributed.cpp:240-273, 455-461): the grid is cut
    into `slabs` slabs along each axis in turn; every slab is transformed on
    its own in a window buffer holding it and its periodic halo (what the
    reference exchanges between ranks), and the slabs' outputs, put back
    together after each axis, equal the serial hierarchize (and, after the
    inverse, dehierarchize) bit for bit."""
    import torch
    level, lmin, maximum = (6, 5, 4), (1, 0, 2), (6, 5, 4)
    rng = np.random.default_rng(slabs)
    x = rng.uniform(-1, 1, [1 << l for l in level])
    for forward in (True, False):
        table = oracle.FORWARD if forward else oracle.INVERSE
        filters = table[wavelet]
        want = x.copy()
        oracle.hierarchize(want, level, lmin, maximum, wavelet,
                           forward=forward)
        state = x.copy()
        for dim in range(3):
            n = 1 << level[dim]
            levels = list(range(lmin[dim] + 1, level[dim] + 1))
            if forward:
                levels.reverse()
            if not levels:
                continue
            out = state.copy()
            size = n // slabs
            for sl in range(slabs):
                start = sl * size
                bounds = R.transform_bounds(
                    (start, start + size - 1), level[dim], maximum[dim],
                    levels, filters)
                need = sorted(set(R.transform_indices(bounds, maximum[dim])) |
                              set(range(start, start + size)))
                cov = R.covering_periodic_bounds(need, n)
                ext = (cov[1] - cov[0]) % n + 1
                idx = (cov[0] + np.arange(ext)) % n
                buf = np.ascontiguousarray(np.take(state, idx, axis=dim))
                g = torch.from_numpy(buf).cuda()
                front = [0, 0, 0]
                front[dim] = cov[0]
                ofront = [0, 0, 0]
                ofront[dim] = start
                oext = [1 << l for l in level]
                oext[dim] = size
                T.transform_outputs(g, dim, level, maximum, levels, filters,
                                    (ofront, oext, (1, 1, 1)),
                                    window_front=front)
                torch.cuda.synchronize()
                res = g.cpu().numpy()
                for k in range(size):
                    j = (start + k - cov[0]) % n
                    dst = [slice(None)] * 3
                    src = [slice(None)] * 3
                    dst[dim] = start + k
                    src[dim] = j
                    out[tuple(dst)] = res[tuple(src)]
            state = out
        assert np.array_equal(state, want), (wavelet, slabs, forward)
        x = want if forward else x
