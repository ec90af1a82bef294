"""Parity on the benchmark configurations at their full sizes.

C1 (2D hat, 64 x 64, the reference's CPU-sized case) and C2 (3D CDF
biorthogonal, 512^3) and C3 (6D hat, 32^4 x 16^2) are compared with the CPU
oracle point for point in FP64 (bit-identical), forward and inverse, on the
bench's seeded inputs; FP32c is held to the normwise 1e-6 target on C3. C4
(the batched 4D combination technique, 3,025 grids, 1.7 G points) is
compared with the oracle grid by grid in FP64, forward and inverse
(bit-identical), and checked through size-independent properties: the FP64
round trip, exact linearity, and the FP32c forward against the FP64 forward
within the target. C5 (the 6D scheme, 7,798 grids) runs its whole FP64
pipeline -- forward, combine, restrict, inverse -- against the oracle's
restatement of the reference driver (bit-identical at every stage), and its
FP32c pipeline against the FP64 one per q.
"""
import math

import numpy as np
import pytest

import paliwa_gb300 as pg

pytestmark = pytest.mark.gpu


def oracle():
    import oracle as O
    O.build()
    return O


def c1_input():
    """f(x, y) = sin(2 pi x) cos(3 pi y) + U[-0.01, 0.01] on the 64 x 64
    periodic grid x = i / 64 (the C1 configuration, seeded)."""
    x = np.arange(64) / 64.0
    f = np.multiply.outer(np.sin(2 * np.pi * x), np.cos(3 * np.pi * x))
    return f + np.random.default_rng(20261204).uniform(-0.01, 0.01, f.shape)


def to_gpu(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def test_c1_2d_hat_bit_exact_and_round_trip():
    import torch
    O = oracle()
    x = c1_input()
    level, lmin = (6, 6), (0, 0)
    t = to_gpu(x)
    pg.hierarchize(t, level, lmin, level, "hat")
    torch.cuda.synchronize()
    want = O.hierarchize(x.copy(), level, lmin, level, "hat")
    assert np.array_equal(t.cpu().numpy(), want)
    pg.dehierarchize(t, level, lmin, level, "hat")
    torch.cuda.synchronize()
    back = t.cpu().numpy()
    assert np.max(np.abs(back - x)) <= 1e-13 * np.max(np.abs(x))


@pytest.mark.parametrize("name", ["3d-biorthogonal-999", "6d-hat-555544"])
def test_c2_c3_full_size_bit_exact(name):
    import torch
    import bench
    O = oracle()
    w = bench.Workload(name)
    x = w.grid_values(0)
    level, lmin = w.levels[0], w.lmin
    t = to_gpu(x)
    pg.hierarchize(t, level, lmin, w.lmax, w.wavelet)
    torch.cuda.synchronize()
    want = O.hierarchize(x.copy(), level, lmin, w.lmax, w.wavelet)
    got = t.cpu().numpy()
    assert np.array_equal(got, want), name
    pg.dehierarchize(t, level, lmin, w.lmax, w.wavelet)
    torch.cuda.synchronize()
    back = O.dehierarchize(want.copy(), level, lmin, w.lmax, w.wavelet)
    assert np.array_equal(t.cpu().numpy(), back), name
    assert np.max(np.abs(back - x)) <= 1e-13 * np.max(np.abs(x))
    if name.startswith("6d"):
        # C3 also runs in FP32c: normwise error against the FP64 oracle.
        t32 = to_gpu(x.astype(np.float32))
        pg.hierarchize(t32, level, lmin, w.lmax, w.wavelet, compensated=True)
        torch.cuda.synchronize()
        e = np.max(np.abs(t32.cpu().numpy().astype(np.float64) - want))
        assert e / np.max(np.abs(want)) <= 1e-6


def test_c4_full_size_round_trip_and_fp32c_error():
    import torch
    import bench
    from paliwa_gb300 import ct as pct
    w = bench.Workload("4d-ct-20")
    b64, v64 = pct.packed_grids(w.levels, torch.float64)
    for i, v in enumerate(v64):
        v.copy_(torch.from_numpy(np.ascontiguousarray(
            w.grid_values(i)).reshape(-1)))
    b32, v32 = pct.packed_grids(w.levels, torch.float32)
    b32.copy_(b64)
    pristine = b64.clone()
    # The copies above ran on the default stream; the batches run on `s`.
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    bt64 = pct.Batch(v64, w.levels, w.lmin, w.lmax, w.wavelet)
    bt32 = pct.Batch(v32, w.levels, w.lmin, w.lmax, w.wavelet,
                     compensated=True)
    bt64.hierarchize(s)
    bt32.hierarchize(s)
    s.synchronize()
    # FP32c forward against FP64 forward, normwise over the batch.
    err = float((b32.double() - b64).abs().max())
    assert err / float(b64.abs().max()) <= 1e-6
    # FP64 round trip.
    bt64.dehierarchize(s)
    s.synchronize()
    rt = float((b64 - pristine).abs().max())
    assert rt <= 1e-13 * float(pristine.abs().max())
    # Linearity of the forward transform: T(2x) == 2 T(x) exactly (scaling
    # by 2 commutes with every rounding).
    b64.copy_(pristine)
    torch.cuda.synchronize()
    bt64.hierarchize(s)
    s.synchronize()
    once = b64.clone()
    b64.copy_(pristine * 2)
    torch.cuda.synchronize()
    bt64.hierarchize(s)
    s.synchronize()
    assert torch.equal(b64, once * 2)
    bt64.close()
    bt32.close()
    assert math.isfinite(err)


def test_c5_ct_pipeline_per_q_error():
    """C5: the 6D CDF (2,2) scheme |l|_1 = 16 - q, q = 0..5 (7,798 grids,
    292 M points): forward transform of every grid, FP64 combine into the
    sparse grid, restrict back, inverse of every grid. The FP32-compensated
    pipeline (FP32 grids, combine still in FP64) is compared per q with the
    FP64 pipeline, normwise (max |e| / max |ref| over the grids of that q).

    The combination adds grids with coefficients up to C(5, 2) = 10, which
    amplifies the rounding of the inputs to FP32 storage: the FP64 pipeline
    run on the FP32-rounded inputs is already 1.5e-6 to 2.4e-6 away (the
    storage floor), above 1e-6. The FP32c pipeline (measured 3.0e-6 to
    3.8e-6, 1.6 to 2.1 times the floor) is held to three times that floor
    per q; its forward transform alone to 1e-6."""
    import torch
    import bench
    from paliwa_gb300 import ct as pct
    w = bench.Workload("6d-ct-16")
    b64, v64 = pct.packed_grids(w.levels, torch.float64)
    for i, v in enumerate(v64):
        v.copy_(torch.from_numpy(np.ascontiguousarray(
            w.grid_values(i)).reshape(-1)))
    pristine = b64.clone()
    b32, v32 = pct.packed_grids(w.levels, torch.float32)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    bt64 = pct.Batch(v64, w.levels, w.lmin, w.lmax, w.wavelet)
    ct64 = pct.CombinationTechnique(v64, w.levels, w.coeffs, w.lmax)
    bt32 = pct.Batch(v32, w.levels, w.lmin, w.lmax, w.wavelet,
                     compensated=True)
    ct32 = pct.CombinationTechnique(v32, w.levels, w.coeffs, w.lmax)

    def pipeline(bt, ct, buf, inputs, forward_only=False):
        buf.copy_(inputs)
        torch.cuda.synchronize()
        bt.hierarchize(s)
        if not forward_only:
            sparse = ct.combine(stream=s)
            ct.restrict(sparse, stream=s)
            bt.dehierarchize(s)
        s.synchronize()
        return buf.double().clone()

    ref = pipeline(bt64, ct64, b64, pristine)
    floor = pipeline(bt64, ct64, b64, pristine.float().double())
    got = pipeline(bt32, ct32, b32, pristine)
    starts = [(v.data_ptr() - b64.data_ptr()) // 8 for v in v64]

    def per_q(a, q):
        idx = [i for i, qq in enumerate(w.q) if qq == q]
        x = torch.cat([a[starts[i]:starts[i] + v64[i].numel()] for i in idx])
        y = torch.cat([ref[starts[i]:starts[i] + v64[i].numel()]
                       for i in idx])
        return float((x - y).abs().max()) / float(y.abs().max())

    for q in sorted(set(w.q)):
        e, f = per_q(got, q), per_q(floor, q)
        assert math.isfinite(e) and e <= 3 * f, (q, e, f)
    fwd = pipeline(bt32, ct32, b32, pristine, forward_only=True)
    ref_fwd = pipeline(bt64, ct64, b64, pristine, forward_only=True)
    rel = float((fwd - ref_fwd).abs().max()) / float(ref_fwd.abs().max())
    assert rel <= 1e-6, rel
    for h in (ct64, ct32, bt64, bt32):
        h.close()


def test_c4_fp64_full_size_bit_exact_against_oracle():
    """C4 at full size (3,025 grids, 1.7 G points) in FP64: the batched
    forward and inverse transforms of every grid are bit-identical to the
    CPU oracle's hierarchize and dehierarchize of the same grid."""
    import torch
    import bench
    from paliwa_gb300 import ct as pct
    O = oracle()
    w = bench.Workload("4d-ct-20")
    b64, v64 = pct.packed_grids(w.levels, torch.float64)
    for i, v in enumerate(v64):
        v.copy_(torch.from_numpy(np.ascontiguousarray(
            w.grid_values(i)).reshape(-1)))
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    bt = pct.Batch(v64, w.levels, w.lmin, w.lmax, w.wavelet)

    def expected(i, forward):
        x = np.ascontiguousarray(w.grid_values(i))
        y = O.hierarchize(x, w.levels[i], w.lmin, w.lmax, w.wavelet)
        if not forward:
            y = O.dehierarchize(y, w.levels[i], w.lmin, w.lmax, w.wavelet)
        return y

    for forward in (True, False):
        (bt.hierarchize if forward else bt.dehierarchize)(s)
        s.synchronize()
        host = b64.cpu().numpy()
        starts = [(v.data_ptr() - b64.data_ptr()) // 8 for v in v64]
        bad = [i for i, lv in enumerate(w.levels) if not np.array_equal(
            host[starts[i]:starts[i] + (1 << sum(lv))],
            expected(i, forward).reshape(-1))]
        assert not bad, (forward, len(bad), bad[:5])
    bt.close()


def test_c5_fp64_pipeline_bit_exact_against_oracle():
    """C5 at full size (6D, 7,798 grids) in FP64: forward transform of every
    grid, combine into the kept sparse-grid subspaces, restrict back into the
    grids, inverse transform -- each stage bit-identical to the oracle's
    restatement of the reference driver (hierarchize per grid,
    test/test_paliwa_combination_technique.cpp:256-290 for the combine)."""
    import torch
    import bench
    from paliwa_gb300 import ct as pct
    O = oracle()
    w = bench.Workload("6d-ct-16")
    b64, v64 = pct.packed_grids(w.levels, torch.float64)
    inputs = [np.ascontiguousarray(w.grid_values(i)) for i in
              range(len(w.levels))]
    for v, x in zip(v64, inputs):
        v.copy_(torch.from_numpy(x.reshape(-1)))
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    bt = pct.Batch(v64, w.levels, w.lmin, w.lmax, w.wavelet)
    ct = pct.CombinationTechnique(v64, w.levels, w.coeffs, w.lmax)
    starts = [(v.data_ptr() - b64.data_ptr()) // 8 for v in v64]

    def grids_of(host):
        return [host[a:a + (1 << sum(lv))].reshape([1 << l for l in lv])
                for a, lv in zip(starts, w.levels)]

    bt.hierarchize(s)
    s.synchronize()
    want = [O.hierarchize(x.copy(), lv, w.lmin, w.lmax, w.wavelet)
            for x, lv in zip(inputs, w.levels)]
    got = grids_of(b64.cpu().numpy())
    assert all(np.array_equal(a, b) for a, b in zip(got, want))

    sparse = ct.combine(stream=s)
    s.synchronize()
    subs, offs_lib = ct.subspaces()
    assert subs == O.kept_subspaces(w.levels)
    offs, total = O.sparse_offsets(subs)
    assert total == ct.npoints
    assert [offs[sb] for sb in subs] == offs_lib
    want_sparse = O.combine_sparse(want, w.levels, w.coeffs, offs, total)
    assert np.array_equal(sparse.cpu().numpy(), want_sparse)

    ct.restrict(sparse, stream=s)
    bt.dehierarchize(s)
    s.synchronize()
    for g, lv in zip(want, w.levels):
        O.restrict_sparse(g, lv, want_sparse, offs)
        O.dehierarchize(g, lv, w.lmin, w.lmax, w.wavelet)
    got = grids_of(b64.cpu().numpy())
    bad = [i for i, (a, b) in enumerate(zip(got, want))
           if not np.array_equal(a, b)]
    assert not bad, (len(bad), bad[:5])
    ct.close()
    bt.close()
