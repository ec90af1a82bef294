"""Batched transforms and the combination technique on the GPU, against the
oracle restatement of the reference's test driver
(test/test_paliwa_combination_technique.cpp)."""
import math

import numpy as np
import pytest

import paliwa_gb300 as pg
from paliwa_gb300 import ct as pct

pytestmark = pytest.mark.gpu

# test/test_paliwa_combination_technique.cpp:84-125
SCHEMES = {
    2: dict(lmax=(10, 11), lmin=(2, 3),
            levels=[(2, 11), (3, 10), (4, 9), (5, 8), (6, 7), (7, 6), (8, 5),
                    (9, 4), (10, 3), (2, 10), (3, 9), (4, 8), (5, 7), (6, 6),
                    (7, 5), (8, 4), (9, 3)],
            coeffs=[1] * 9 + [-1] * 8, full=106496, sparse=18432),
    3: dict(lmax=(5, 6, 7), lmin=(4, 5, 6),
            levels=[(4, 6, 7), (5, 5, 7), (5, 6, 6), (4, 5, 6)],
            coeffs=[1, 1, 1, -2], full=425984, sparse=131072),
    4: dict(lmax=(3, 4, 5, 6), lmin=(1, 2, 3, 4),
            levels=[(2, 2, 4, 4), (3, 2, 3, 4), (1, 4, 3, 4), (1, 2, 5, 4),
                    (2, 3, 3, 4), (1, 3, 4, 4), (2, 2, 3, 5), (1, 3, 3, 5),
                    (1, 2, 3, 6), (1, 2, 4, 5), (1, 2, 4, 4), (2, 2, 3, 4),
                    (1, 3, 3, 4), (1, 2, 3, 5), (1, 2, 3, 4)],
            coeffs=[1] * 10 + [-3] * 4 + [3], full=50176, sparse=5120),
}


def oracle():
    import oracle as o
    o.build()
    return o


def sine_grid(level, lmax):
    """prod_i sin(pi x_i) at x = uid / 2^L (:61-71 with
    paliwa_dimensions.hpp:71-79)."""
    f = None
    for d, (l, L) in enumerate(zip(level, lmax)):
        x = (np.arange(1 << l) << (L - l)) / float(1 << L)
        shape = [1] * len(level)
        shape[d] = len(x)
        v = np.sin(math.pi * x).reshape(shape)
        f = v if f is None else f * v
    return np.ascontiguousarray(np.broadcast_to(f, [1 << l for l in level]))


def upload(arrays):
    import torch
    return [torch.from_numpy(a.copy()).cuda().reshape(-1) for a in arrays]


@pytest.mark.parametrize("d", [2, 3, 4])
@pytest.mark.parametrize("wavelet", ["hat", "biorthogonal", "fullweighting"])
def test_batch_matches_oracle_per_grid(d, wavelet):
    sc = SCHEMES[d]
    rng = np.random.default_rng(d)
    xs = [rng.uniform(-1, 1, [1 << l for l in lv]) for lv in sc["levels"]]
    gs = upload(xs)
    b = pct.Batch(gs, sc["levels"], sc["lmin"], sc["lmax"], wavelet)
    import torch
    b.hierarchize(torch.cuda.current_stream())
    torch.cuda.synchronize()
    O = oracle()
    for g, x, lv in zip(gs, xs, sc["levels"]):
        want = O.hierarchize(x.copy(), lv, sc["lmin"], sc["lmax"], wavelet)
        assert np.array_equal(g.cpu().numpy().reshape(want.shape), want)
    b.dehierarchize()  # legacy default stream: direct launches
    torch.cuda.synchronize()
    for g, x in zip(gs, xs):
        assert np.max(np.abs(g.cpu().numpy().reshape(x.shape) - x)) <= 1e-13
    b.close()


def test_batch_graph_replay_and_compensated():
    import torch
    sc = SCHEMES[4]
    rng = np.random.default_rng(5)
    xs = [rng.uniform(-1, 1, [1 << l for l in lv]) for lv in sc["levels"]]
    O = oracle()
    wants = [O.hierarchize(x.copy(), lv, sc["lmin"], sc["lmax"], "biorthogonal")
             for x, lv in zip(xs, sc["levels"])]
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        g32 = [t.float() for t in upload(xs)]
        b = pct.Batch(g32, sc["levels"], sc["lmin"], sc["lmax"],
                      "biorthogonal", compensated=True)
        for rep in range(3):  # capture once, replay; inverse in between
            b.hierarchize(s)
            s.synchronize()
            for g, w in zip(g32, wants):
                got = g.double().cpu().numpy().reshape(w.shape)
                assert np.max(np.abs(got - w)) / np.max(np.abs(w)) <= 1e-6
            b.dehierarchize(s)
        b.close()


def test_long_pencils_in_batch():
    """Grids whose pencils exceed one CTA mix windowed and sub-lattice stages
    with ordinary jobs in one plan."""
    import torch
    levels = [(17, 1), (1, 16), (13, 4), (9, 8), (2, 2)]
    lmin, lmax = (1, 1), (17, 16)
    rng = np.random.default_rng(1)
    xs = [rng.uniform(-1, 1, [1 << l for l in lv]) for lv in levels]
    buf, gs = pct.packed_grids(levels, torch.float64)
    for g, x in zip(gs, xs):
        g.copy_(torch.from_numpy(x.reshape(-1)))
    b = pct.Batch(gs, levels, lmin, lmax, "biorthogonal")
    s = torch.cuda.Stream()
    b.hierarchize(s)
    s.synchronize()
    O = oracle()
    for g, x, lv in zip(gs, xs, levels):
        want = O.hierarchize(x.copy(), lv, lmin, lmax, "biorthogonal")
        assert np.array_equal(g.cpu().numpy().reshape(want.shape), want)


@pytest.mark.parametrize("d", [2, 3, 4])
def test_combination_technique_reference_driver(d):
    """The reference driver end to end (:77-340): sizes, FP64 combine
    (bit-exact against the oracle restatement), scatter, full-grid
    dehierarchize and the integral check mean ~ (2/pi)^d within 0.031."""
    import torch
    sc = SCHEMES[d]
    O = oracle()
    xs = [sine_grid(lv, sc["lmax"]) for lv in sc["levels"]]
    assert sum(x.size for x in xs) == sc["full"]
    gs = upload(xs)
    b = pct.Batch(gs, sc["levels"], sc["lmin"], sc["lmax"], "biorthogonal")
    b.hierarchize()
    ct = pct.CombinationTechnique(gs, sc["levels"], sc["coeffs"], sc["lmax"])
    assert ct.npoints == sc["sparse"]
    subs, offs = ct.subspaces()
    assert subs == O.kept_subspaces(sc["levels"])
    sparse = ct.combine()
    torch.cuda.synchronize()
    hier = [O.hierarchize(x.copy(), lv, sc["lmin"], sc["lmax"], "biorthogonal")
            for x, lv in zip(xs, sc["levels"])]
    want = O.combine(hier, sc["levels"], sc["coeffs"], sc["lmax"], subs)
    got = sparse.cpu().numpy()
    for w, off in zip(want, offs):
        assert np.array_equal(got[off:off + w.size], w.reshape(-1))
    full = ct.scatter(sparse)
    torch.cuda.synchronize()
    want_full = O.scatter(want, subs, sc["lmax"])
    assert np.array_equal(full.cpu().numpy(), want_full)
    pg.dehierarchize(full, sc["lmax"], sc["lmin"], sc["lmax"], "biorthogonal")
    mean = float(full.mean())
    assert abs(mean - (2 / math.pi) ** d) <= 0.031
    O.dehierarchize(want_full, sc["lmax"], sc["lmin"], sc["lmax"],
                    "biorthogonal")
    assert np.array_equal(full.cpu().numpy(), want_full)
    ct.close()


def test_restrict_writes_combined_values():
    import torch
    sc = SCHEMES[2]
    rng = np.random.default_rng(3)
    xs = [rng.uniform(-1, 1, [1 << l for l in lv]) for lv in sc["levels"]]
    gs = upload(xs)
    ct = pct.CombinationTechnique(gs, sc["levels"], sc["coeffs"], sc["lmax"])
    sparse = ct.combine()
    ct.restrict(sparse)
    torch.cuda.synchronize()
    O = oracle()
    subs, offs = ct.subspaces()
    sp = sparse.cpu().numpy()
    for g, lv, x in zip(gs, sc["levels"], xs):
        arr = g.cpu().numpy().reshape(x.shape)
        written = np.zeros(x.shape, bool)
        for s, off in zip(subs, offs):
            if any(si > li for si, li in zip(s, lv)):
                continue
            sl = O.subspace_slices(s, lv)
            n = O.subspace_size(s)
            assert np.array_equal(arr[sl].reshape(-1), sp[off:off + n])
            written[sl] = True
        assert np.array_equal(arr[~written], x[~written])


def test_classical_scheme_sizes():
    levels, coeffs = pct.combination_scheme(4, 20, 3, 1)
    counts = [sum(1 for l in levels if sum(l) == 20 - q) for q in range(4)]
    assert counts == [969, 816, 680, 560]
    assert sum(1 << sum(l) for l in levels) == 1695547392
    assert set(coeffs) == {1, -3, 3, -1}


def test_full_scheme_batch_deterministic_and_exact():
    """A whole 4D scheme (|l|_1 = 18 - q, q = 0..3, 2059 grids, ~0.25 G
    points) in one batch: persistent CTAs loop over many tiles, and windowed
    stages of long pencils run next to each other. Two runs give identical
    bits (no race between overlapping windows), and every grid with a pencil
    longer than one CTA matches the oracle bit for bit in FP64."""
    import torch
    levels, _ = pct.combination_scheme(4, 18, 3, 1)
    lmin, lmax = (1, 1, 1, 1), (15, 15, 15, 15)
    rng = np.random.default_rng(7)
    buf, gs = pct.packed_grids(levels, torch.float64)
    buf.copy_(torch.from_numpy(rng.uniform(-1, 1, buf.numel())))
    pristine = buf.clone()
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    b = pct.Batch(gs, levels, lmin, lmax, "biorthogonal")
    b.hierarchize(s)
    s.synchronize()
    first = buf.clone()
    buf.copy_(pristine)
    torch.cuda.synchronize()
    b.hierarchize(s)
    s.synchronize()
    assert torch.equal(first, buf)
    O = oracle()
    long = [i for i, l in enumerate(levels) if max(l) > 12]
    assert long
    for i in long[::3]:
        lv = levels[i]
        x = pristine.narrow(0, gs[i].data_ptr() // 8 - buf.data_ptr() // 8,
                            gs[i].numel()).cpu().numpy().reshape(
                                [1 << l for l in lv])
        want = O.hierarchize(x.copy(), lv, lmin, lmax, "biorthogonal")
        assert np.array_equal(gs[i].cpu().numpy().reshape(want.shape), want), lv
    b.dehierarchize(s)
    s.synchronize()
    assert torch.max(torch.abs(buf - pristine)) <= 1e-12
    b.close()


def test_batch_compensated_bit_exact_model():
    """FP32-compensated batch of a whole 4D scheme (|l|_1 = 14 - q, 791
    grids of uneven shapes, one job list per launch): every kernel variant
    the plan picks, bit for bit against the numpy model of the compensated
    arithmetic, forward and inverse."""
    import torch
    from compensated import hierarchize as model
    levels, _ = pct.combination_scheme(4, 14, 3, 1)
    lmin, lmax = (1, 1, 1, 1), (11, 11, 11, 11)
    rng = np.random.default_rng(11)
    buf, gs = pct.packed_grids(levels, torch.float32)
    buf.copy_(torch.from_numpy(rng.uniform(-1, 1, buf.numel())))
    pristine = buf.cpu().numpy().copy()
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    b = pct.Batch(gs, levels, lmin, lmax, "biorthogonal", compensated=True)
    base = buf.data_ptr() // 4
    for forward in (True, False):
        buf.copy_(torch.from_numpy(pristine))
        torch.cuda.synchronize()
        (b.hierarchize if forward else b.dehierarchize)(s)
        s.synchronize()
        out = buf.cpu().numpy()
        for i in range(0, len(levels), 3):
            lv = levels[i]
            o = gs[i].data_ptr() // 4 - base
            shape = [1 << l for l in lv]
            x = pristine[o:o + gs[i].numel()].reshape(shape)
            want = model(x, lv, lmin, "biorthogonal", forward)
            got = out[o:o + gs[i].numel()].reshape(shape)
            assert np.array_equal(got.view(np.uint32),
                                  want.view(np.uint32)), (lv, forward)
    b.close()


def test_host_batch_matches_device_batch():
    """HostBatch (grids in pinned host memory, copies overlapped with the
    transforms of other groups) gives the device Batch's bits."""
    import torch
    levels, _ = pct.combination_scheme(4, 13, 3, 1)
    lmin, lmax = (1, 1, 1, 1), (10, 10, 10, 10)
    hb = pct.HostBatch(levels, lmin, lmax, "biorthogonal", torch.float32,
                       compensated=True, groups=5)
    assert len(hb.batches) == 5
    rng = np.random.default_rng(13)
    host_in = torch.from_numpy(
        rng.uniform(-1, 1, hb.numel()).astype(np.float32)).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    for steps in (("hierarchize",), ("hierarchize", "dehierarchize")):
        hb.run(host_in, host_out, steps)
        torch.cuda.synchronize()
        buf, gs = pct.packed_grids(levels, torch.float32)
        buf.copy_(host_in)
        b = pct.Batch(gs, levels, lmin, lmax, "biorthogonal",
                      compensated=True)
        for name in steps:
            getattr(b, name)()
        torch.cuda.synchronize()
        assert torch.equal(buf.cpu(), host_out), steps
        b.close()
    hb.close()


def test_autotune_keeps_results_exact():
    """After the autotuner has re-planned (any kernel per class of stages),
    FP64 stays bit-identical to the oracle and FP32c to the compensated
    model; the tuning report names an applicable kernel for every class."""
    import torch
    from compensated import hierarchize as model
    levels, _ = pct.combination_scheme(4, 13, 3, 1)
    lmin, lmax = (1, 1, 1, 1), (10, 10, 10, 10)
    rng = np.random.default_rng(17)
    O = oracle()
    for dt, comp in ((torch.float64, False), (torch.float32, True)):
        buf, gs = pct.packed_grids(levels, dt)
        x = rng.uniform(-1, 1, buf.numel())
        buf.copy_(torch.from_numpy(x))
        pristine = buf.clone()
        s = torch.cuda.Stream()
        b = pct.Batch(gs, levels, lmin, lmax, "biorthogonal", compensated=comp)
        b.autotune(reps=1, stream=s)
        for fwd in (True, False):
            rep = b.tuning(fwd)
            assert rep
            for _, desc, names, chosen in rep:
                assert chosen in names, (desc, names, chosen)
        buf.copy_(pristine)
        torch.cuda.synchronize()
        b.hierarchize(s)
        s.synchronize()
        for i in range(0, len(levels), 7):
            lv = levels[i]
            shape = [1 << l for l in lv]
            o = (gs[i].data_ptr() - buf.data_ptr()) // buf.element_size()
            xi = pristine[o:o + gs[i].numel()].cpu().numpy().reshape(shape)
            got = gs[i].cpu().numpy().reshape(shape)
            if comp:
                want = model(xi, lv, lmin, "biorthogonal", True)
                assert np.array_equal(got.view(np.uint32),
                                      want.view(np.uint32)), lv
            else:
                want = O.hierarchize(xi.copy(), lv, lmin, lmax, "biorthogonal")
                assert np.array_equal(got, want), lv
        b.close()


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("coefficients", ["integer", "fraction"])
def test_combine_restrict_subspaces_in_many_grids(dtype, coefficients):
    """1100 small 4D grids (levels 1..3 per dimension, repeated level
    vectors allowed): the sums over the grids run in grid order, so they
    equal the oracle's bit for bit. Integer coefficients on FP32 grids take
    the fused multiply-add (exact products), fractions the separately
    rounded form. The coarsest subspaces lie in more than 1024 grids and are
    restricted one warp per point, the rest one thread per point; restrict
    writes every grid's copy of every subspace."""
    import torch
    rng = np.random.default_rng(11)
    levels = [tuple(int(x) for x in rng.integers(1, 4, 4))
              for _ in range(1100)]
    if coefficients == "integer":
        coeffs = [float(c) for c in rng.integers(-3, 4, len(levels))]
    else:
        coeffs = [float(c) for c in rng.uniform(-1, 1, len(levels))]
    lmax = (3, 3, 3, 3)
    xs = [rng.uniform(-1, 1, [1 << l for l in lv]).astype(dtype)
          for lv in levels]
    gs = upload(xs)
    ct = pct.CombinationTechnique(gs, levels, coeffs, lmax)
    O = oracle()
    subs, offs = ct.subspaces()
    counts = O.subspace_counts(levels)
    assert max(counts[s] for s in subs) > 1024
    assert any(counts[s] <= 1024 for s in subs)
    sparse = ct.combine()
    torch.cuda.synchronize()
    want = O.combine([x.astype(np.float64) for x in xs], levels, coeffs,
                     lmax, subs)
    got = sparse.cpu().numpy()
    for w, off in zip(want, offs):
        assert np.array_equal(got[off:off + w.size], w.reshape(-1))
    ct.restrict(sparse)
    torch.cuda.synchronize()
    sp = sparse.cpu().numpy().astype(dtype)
    for g, lv, x in zip(gs, levels, xs):
        arr = g.cpu().numpy().reshape(x.shape)
        for s, off in zip(subs, offs):
            if any(si > li for si, li in zip(s, lv)):
                continue
            n = O.subspace_size(s)
            assert np.array_equal(arr[O.subspace_slices(s, lv)].reshape(-1),
                                  sp[off:off + n])
    ct.close()


@pytest.mark.parametrize("groups", [1, 2, 3, 7, 20])
def test_batch_groups_give_identical_results(groups):
    """Grids dealt into groups run on parallel branches (forked streams,
    joined into the caller's stream, captured into one graph); every group
    count gives the oracle's values bit for bit, through a graph on a
    non-default stream and through direct launches on the legacy stream,
    including long pencils with halo passes in every group."""
    import torch
    levels = [(14, 2), (2, 14), (13, 3), (3, 13), (8, 8), (9, 7), (7, 9),
              (12, 4), (4, 12), (6, 6), (5, 5), (1, 1)]
    lmin, lmax = (1, 1), (14, 14)
    rng = np.random.default_rng(groups)
    xs = [rng.uniform(-1, 1, [1 << l for l in lv]) for lv in levels]
    gs = upload(xs)
    b = pct.Batch(gs, levels, lmin, lmax, "biorthogonal", groups=groups)
    O = oracle()
    s = torch.cuda.Stream()
    for _ in range(2):  # capture, then replay
        for g, x in zip(gs, xs):
            g.copy_(torch.from_numpy(x).reshape(-1))
        b.hierarchize(s)
        s.synchronize()
        for g, x, lv in zip(gs, xs, levels):
            want = O.hierarchize(x.copy(), lv, lmin, lmax, "biorthogonal")
            assert np.array_equal(g.cpu().numpy().reshape(want.shape), want)
    b.dehierarchize()  # legacy default stream: forked direct launches
    torch.cuda.synchronize()
    for g, x in zip(gs, xs):
        assert np.max(np.abs(g.cpu().numpy().reshape(x.shape) - x)) <= 1e-13
    b.close()


@pytest.mark.parametrize("ctas", [1, 3])
def test_ctas_per_sm_cap_gives_identical_results(ctas):
    """A cap on the CTAs per SM of every launch changes only how many CTAs
    walk the tiles: FP64 results equal the oracle's bit for bit, long
    pencils (halo passes and windows) and slab launches included."""
    import torch
    levels = [(14, 2), (2, 14), (13, 3), (8, 8), (6, 6), (5, 5), (3, 4)]
    lmin, lmax = (1, 1), (14, 14)
    rng = np.random.default_rng(40 + ctas)
    xs = [rng.uniform(-1, 1, [1 << l for l in lv]) for lv in levels]
    buf, gs = pct.packed_grids(levels, torch.float64)
    for g, x in zip(gs, xs):
        g.copy_(torch.from_numpy(x).reshape(-1))
    b = pct.Batch(gs, levels, lmin, lmax, "biorthogonal")
    b.set_ctas_per_sm(ctas)
    s = torch.cuda.Stream()
    b.hierarchize(s)
    s.synchronize()
    b.status()
    O = oracle()
    for g, x, lv in zip(gs, xs, levels):
        want = O.hierarchize(x.copy(), lv, lmin, lmax, "biorthogonal")
        assert np.array_equal(g.cpu().numpy().reshape(want.shape), want), lv
    b.close()


def test_tma_wide_kernel_gives_the_wide_kernels_bits():
    """FP32-compensated strided stages of up to 64 points run on the TMA
    wide kernel by default; the per-thread-copy wide kernel gives the same
    bits, forward and inverse, for every wavelet. The scheme mixes inner
    extents of 2 columns (left on the wide kernel), 4 to 2^10 columns, grids
    smaller than one tile and sub-lattice stages of long pencils."""
    import torch
    levels = [(6, 1, 3), (5, 2, 2), (4, 6, 1), (3, 3, 5), (6, 6, 2), (2, 5, 7),
              (1, 4, 9), (6, 2, 1), (2, 2, 2), (14, 2, 1), (5, 5, 5),
              (4, 1, 10)]
    lmin, lmax = (1, 1, 1), (14, 14, 14)
    rng = np.random.default_rng(77)
    host = [rng.uniform(-1, 1, 1 << sum(l)).astype(np.float32)
            for l in levels]
    for wavelet in ("hat", "biorthogonal", "fullweighting"):
        out = []
        for tma in (True, False):
            buf, gs = pct.packed_grids(levels, torch.float32)
            for g, h in zip(gs, host):
                g.copy_(torch.from_numpy(h))
            b = pct.Batch(gs, levels, lmin, lmax, wavelet, compensated=True)
            if not tma:
                b.use_tma(False)
            s = torch.cuda.Stream()
            kernels = b.profile(True, stream=s)[2]
            if tma:
                assert any(k > pct.TWIDE_KERNEL for k in kernels)
            else:
                assert not any(k > pct.TWIDE_KERNEL for k in kernels)
            for g, h in zip(gs, host):
                g.copy_(torch.from_numpy(h))
            b.hierarchize(s)
            s.synchronize()
            fwd = buf.clone()
            b.dehierarchize(s)
            s.synchronize()
            b.status()
            out.append((fwd, buf.clone()))
            b.close()
        assert torch.equal(out[0][0], out[1][0]), wavelet
        assert torch.equal(out[0][1], out[1][1]), wavelet


def test_every_tma_wide_class_gives_the_wide_kernels_bits():
    """Chunks of 2, 4, 8 and 16 points, up to 128 chunks per pencil: every
    class of stages that the TMA wide kernel applies to, set to it through
    set_tuning, gives the bits of the same classes set to the per-thread-copy
    wide kernel (or, for pencils of 128 to 2048 points, the tile or staged
    kernel), forward and inverse, for every wavelet. A kernel that does not
    apply, or a class the plan lacks, is refused with nothing changed."""
    import torch
    levels = [(6, 1, 3), (5, 2, 2), (4, 6, 1), (3, 3, 5), (6, 6, 2), (2, 5, 7),
              (1, 4, 9), (6, 2, 1), (2, 2, 2), (5, 5, 5), (4, 1, 10),
              (3, 2, 8), (2, 3, 6), (7, 4, 3), (8, 5, 1), (2, 8, 4),
              (7, 2, 2), (13, 2, 1), (9, 3, 2), (2, 9, 4), (10, 2, 3),
              (3, 11, 2), (11, 1, 4), (2, 6, 1), (3, 4, 1), (2, 2, 11),
              (2, 1, 12)]
    lmin, lmax = (1, 1, 1), (14, 14, 14)
    rng = np.random.default_rng(78)
    host = [rng.uniform(-1, 1, 1 << sum(l)).astype(np.float32)
            for l in levels]
    seen, seen_last, seen_pairs = set(), set(), set()
    for wavelet in ("hat", "biorthogonal", "fullweighting"):
        out = []
        for kernel in ("twide", "other"):
            buf, gs = pct.packed_grids(levels, torch.float32)
            # no slabs: the small grids' axes would go to the slab kernel
            b = pct.Batch(gs, levels, lmin, lmax, wavelet, compensated=True,
                          slabs=False)
            for forward in (True, False):
                # the other kernel: the wide kernel, else the tile or the
                # staged kernel
                cls = {c: kernel if kernel == "twide" else
                       next(k for k in ("wide", "tile", "staged32", "staged")
                            if k in names)
                       for c, _, names, _ in b.tuning(forward)
                       if "twide" in names}
                assert cls, "no class of the scheme takes the TMA wide kernel"
                b.set_tuning(cls, forward)
                assert all(ch == cls[c] for c, _, _, ch in b.tuning(forward)
                           if c in cls)
                if kernel == "twide":
                    seen.update(d["log2_n"] for c, d, _, _ in
                                b.tuning(forward) if c in cls)
                    seen_last.update(d["log2_n"] for c, d, _, _ in
                                     b.tuning(forward)
                                     if c in cls and d["last"])
                    seen_pairs.update(d["log2_n"] for c, d, _, _ in
                                      b.tuning(forward)
                                      if c in cls and not d["last"] and
                                      d["log2_inner_bytes"] == 3)
            s = torch.cuda.Stream()
            kernels = b.profile(True, stream=s)[2]
            assert any(k > pct.TWIDE_KERNEL for k in kernels) == \
                (kernel == "twide")
            if kernel == "twide":  # pencils of 64 and 128 chunks
                assert any(k > pct.TWIDE_KERNEL + pct.TWIDE_LONG
                           for k in kernels)
            for g, h in zip(gs, host):
                g.copy_(torch.from_numpy(h))
            b.hierarchize(s)
            s.synchronize()
            fwd = buf.clone()
            b.dehierarchize(s)
            s.synchronize()
            b.status()
            out.append((fwd, buf.clone()))
            if kernel == "other":
                c0 = b.tuning(True)[0][0]
                with pytest.raises(ValueError):
                    b.set_tuning({c0: "twide", 1 << 20: "wide"})
                with pytest.raises(ValueError):
                    b.set_tuning({c0: 99})
            b.close()
        assert torch.equal(out[0][0], out[1][0]), wavelet
        assert torch.equal(out[0][1], out[1][1]), wavelet
    # pencils of 4 to 2048 points (axes at level 1 = lmin have nothing to
    # do), strided and along the last axis
    assert {2, 3, 4, 5, 6, 7, 8, 9, 10, 11} <= seen, seen
    assert {2, 3, 4, 5, 6, 10, 11, 12} <= seen_last, seen_last
    # strided axes of inner extent 2 (8 bytes per row)
    assert {2, 4, 5, 6} <= seen_pairs, seen_pairs
