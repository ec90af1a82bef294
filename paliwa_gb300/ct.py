"""Batched transforms and the sparse-grid combination technique.

The reference ships the combination technique only as a test driver
(test/test_paliwa_combination_technique.cpp:77-340): hierarchize every
component grid, combine the hierarchical surpluses with the scheme's
coefficients into the sparse-grid subspaces (FP64), scatter them onto a full
grid and dehierarchize it. This module exposes those steps over the CUDA
library:

* ``Batch``: one plan (and one CUDA graph per direction) that transforms every
  component grid, replacing the per-grid ``hierarchize`` calls on
  ``instances[i % n]`` (:164-174).
* ``CombinationTechnique``: subspace enumeration and the FP64 combine
  (:176-290), the restriction of the combined subspaces back onto each
  component grid, and the scatter onto a full grid (:293-318).
* ``combination_scheme``: the classical level sets |l|_1 = n - q with
  coefficients (-1)^q * C(d-1, q).
"""
from __future__ import annotations

import ctypes
import itertools
import math

from . import _lib
from .transform import _dtype_code, _stream_handle, wavelet_id


def combination_scheme(ndim, level_sum, qmax=None, minimum_level=1):
    """Classical combination technique: every level vector l with
    l_i >= minimum_level and |l|_1 = level_sum - q for q = 0..qmax, with
    coefficient (-1)^q * C(ndim - 1, q). Level vectors are listed in
    q-major, then lexicographic order."""
    if qmax is None:
        qmax = ndim - 1
    lmin = ([minimum_level] * ndim if isinstance(minimum_level, int)
            else list(minimum_level))
    levels, coeffs = [], []
    for q in range(qmax + 1):
        m = level_sum - q
        for l in _compositions(m, lmin):
            levels.append(tuple(l))
            coeffs.append((-1) ** q * math.comb(ndim - 1, q))
    return levels, coeffs


def _compositions(total, lmin):
    if len(lmin) == 1:
        if total >= lmin[0]:
            yield (total,)
        return
    rest_min = sum(lmin[1:])
    for first in range(lmin[0], total - rest_min + 1):
        for tail in _compositions(total - first, lmin[1:]):
            yield (first,) + tail


def packed_grids(levels, dtype, device="cuda", align=64):
    """One device allocation holding every grid (each start aligned to
    ``align`` elements); returns (buffer, list of flat views)."""
    import torch
    sizes = [1 << sum(int(x) for x in l) for l in levels]
    offsets, off = [], 0
    for s in sizes:
        offsets.append(off)
        off += (s + align - 1) // align * align
    buf = torch.empty(off, dtype=dtype, device=device)
    return buf, [buf.narrow(0, o, s) for o, s in zip(offsets, sizes)]


# Launch codes of the slab kernel and (plus the chunk size, plus 32 for
# pencils of 8 to 32 chunks, 64 for more, 96 for the last axis, 160 for its
# pencils of more than 32 chunks and 128 for strided axes of inner extent 2)
# of the TMA wide kernel in Batch.profile.
SLAB_KERNEL = 1024
TWIDE_KERNEL = 2048
TWIDE_CHUNKED = 32
TWIDE_LONG = 64
TWIDE_CONTIG = 96
TWIDE_PAIRS = 128
TWIDE_LONG_CONTIG = 160


def kernel_name(code):
    """Name of the lifting kernel behind a launch code of Batch.profile."""
    if code > TWIDE_KERNEL + TWIDE_LONG_CONTIG:
        return ("twide_kernel long last axis "
                f"R={code - TWIDE_KERNEL - TWIDE_LONG_CONTIG}")
    if code > TWIDE_KERNEL + TWIDE_PAIRS:
        return ("twide_kernel inner 2 "
                f"R={code - TWIDE_KERNEL - TWIDE_PAIRS}")
    if code > TWIDE_KERNEL + TWIDE_CONTIG:
        return ("twide_kernel last axis "
                f"R={code - TWIDE_KERNEL - TWIDE_CONTIG}")
    if code > TWIDE_KERNEL + TWIDE_LONG:
        return f"twide_kernel long R={code - TWIDE_KERNEL - TWIDE_LONG}"
    if code > TWIDE_KERNEL + TWIDE_CHUNKED:
        return f"twide_kernel chunked R={code - TWIDE_KERNEL - TWIDE_CHUNKED}"
    if code > TWIDE_KERNEL:
        return f"twide_kernel R={code - TWIDE_KERNEL}"
    if code == SLAB_KERNEL:
        return "slab_kernel"
    if code == 512:
        return "halo_kernel"
    if code > 256:
        return f"tile_kernel long R={code - 256}"
    if code > 192:
        return f"tile_kernel R={code - 192}"
    if code > 128:
        return f"wide_kernel last axis R={code - 128}"
    if code > 64:
        return f"wide_kernel R={code - 64}"
    if code < 0:
        return f"lift_kernel direct R={-code}"
    return f"lift_kernel staged R={code}"


def _ptr_array(grids):
    arr = (ctypes.c_void_p * len(grids))()
    for i, g in enumerate(grids):
        arr[i] = g.data_ptr()
    return arr


def _check_grids(grids, levels):
    if len(grids) != len(levels):
        raise _lib.InvalidArgument("one level vector per grid")
    dt = grids[0].dtype
    for g, l in zip(grids, levels):
        if not g.is_cuda or not g.is_contiguous() or g.dtype != dt:
            raise _lib.InvalidArgument(
                "grids must be contiguous CUDA tensors of one dtype")
        if g.numel() != 1 << sum(int(x) for x in l):
            raise _lib.InvalidArgument("grid size does not match its level")


class Batch:
    """Forward / inverse transform of many grids with one plan.

    ``grids`` are CUDA tensors (bound by address at construction),
    ``levels[i]`` the level vector of grid i; ``minimum_level`` and
    ``maximum_level`` are shared, as in the reference's driver. ``groups``
    (default: the library's, 4) is the number of groups of grids run on
    parallel branches (see :meth:`set_groups`)."""

    def __init__(self, grids, levels, minimum_level, maximum_level,
                 wavelet_name="hat", compensated=False, groups=None,
                 slabs=True):
        _check_grids(grids, levels)
        self.grids = list(grids)
        self.levels = [tuple(int(x) for x in l) for l in levels]
        ndim = len(self.levels[0])
        flat = [x for l in self.levels for x in l]
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        _lib.check(self._lib.paliwa_gb_batch_create(
            ndim, len(grids), _lib.i64(flat), _lib.i64(minimum_level),
            _lib.i64(maximum_level), _dtype_code(grids[0], compensated),
            wavelet_id(wavelet_name), _ptr_array(grids),
            ctypes.byref(self._h)))
        self.points = sum(g.numel() for g in grids)
        if not slabs:
            self.use_slabs(False)
        if groups is not None:
            self.set_groups(groups)

    def use_slabs(self, enable):
        """Plan the trailing axes of grids whose slabs fit a tile as one
        slab launch (default), or every axis on its own (the same bits).
        Synchronizes the device."""
        _lib.check(self._lib.paliwa_gb_batch_use_slabs(self._h, int(enable)))

    def use_tma(self, enable):
        """Run FP32c strided stages of up to 16 chunks per pencil on the TMA
        wide kernel where the plan chose it (default), or on the wide and
        tile kernels' per-thread copies (the same bits). Synchronizes the
        device."""
        _lib.check(self._lib.paliwa_gb_batch_use_tma(self._h, int(enable)))

    def set_ctas_per_sm(self, ctas):
        """Cap every launch of the batch at ``ctas`` CTAs per SM, leaving
        room on each SM for the other groups' launches (0: as many as fit,
        the default). Synchronizes the device."""
        _lib.check(self._lib.paliwa_gb_batch_set_ctas_per_sm(self._h,
                                                             int(ctas)))

    def status(self):
        """Raises DeviceTimeout if a slab launch gave up a bounded wait for
        its tile copies since the last call. Synchronizes the device."""
        _lib.check(self._lib.paliwa_gb_batch_status(self._h))

    def set_groups(self, ngroups):
        """Split the grids into ``ngroups`` groups of about equal size, each
        planned on its own and run on its own branch (forked from and joined
        into the caller's stream) so that their launches overlap; 1 runs
        every launch on the caller's stream. Synchronizes the device."""
        _lib.check(self._lib.paliwa_gb_batch_set_groups(self._h,
                                                        int(ngroups)))

    def hierarchize(self, stream=None):
        _lib.check(self._lib.paliwa_gb_batch_hierarchize(
            self._h, _stream_handle(self.grids[0], stream)))

    def dehierarchize(self, stream=None):
        _lib.check(self._lib.paliwa_gb_batch_dehierarchize(
            self._h, _stream_handle(self.grids[0], stream)))

    def use_graphs(self, enable):
        _lib.check(self._lib.paliwa_gb_batch_use_graphs(self._h, int(enable)))

    def launches(self):
        p, f, i = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(self._lib.paliwa_gb_batch_info(
            self._h, ctypes.byref(p), ctypes.byref(f), ctypes.byref(i)))
        return f.value, i.value

    def profile(self, forward=True, stream=None):
        """Per-launch (milliseconds, algorithmic bytes, kernel) of one
        direction, launched without a graph and bracketed by CUDA events.
        kernel: R > 0 staged with chunks of R points, -R direct, 64 + R
        wide (see :func:`kernel_name`)."""
        n = ctypes.c_int()
        s = _stream_handle(self.grids[0], stream)
        _lib.check(self._lib.paliwa_gb_batch_profile(
            self._h, int(forward), s, 0, ctypes.byref(n), None, None, None))
        ms = (ctypes.c_float * max(1, n.value))()
        by = (ctypes.c_int64 * max(1, n.value))()
        kd = (ctypes.c_int32 * max(1, n.value))()
        _lib.check(self._lib.paliwa_gb_batch_profile(
            self._h, int(forward), s, n.value, ctypes.byref(n), ms, by, kd))
        return (list(ms[:n.value]), list(by[:n.value]), list(kd[:n.value]))

    def autotune(self, reps=2, stream=None):
        """Pick the fastest kernel per class of stages by timing each
        direction (see paliwa_gb_batch_autotune); returns the number of
        classes whose kernel changed. The grids' contents come back up to
        rounding."""
        n = ctypes.c_int()
        _lib.check(self._lib.paliwa_gb_batch_autotune(
            self._h, _stream_handle(self.grids[0], stream), int(reps),
            ctypes.byref(n)))
        return n.value

    KERNELS = ("staged", "direct", "wide", "tile", "staged32", "twide")

    def tuning(self, forward=True):
        """[(class, {last, sub, log2_n, log2_inner_bytes}, applicable kernel
        names, chosen kernel name)] of one direction's plan."""
        n = ctypes.c_int()
        _lib.check(self._lib.paliwa_gb_batch_tuning(
            self._h, int(forward), 0, ctypes.byref(n), None, None, None))
        cl = (ctypes.c_int32 * max(1, n.value))()
        ks = (ctypes.c_int32 * max(1, n.value))()
        ch = (ctypes.c_int32 * max(1, n.value))()
        _lib.check(self._lib.paliwa_gb_batch_tuning(
            self._h, int(forward), n.value, ctypes.byref(n), cl, ks, ch))
        out = []
        for c, k, x in zip(cl[:n.value], ks[:n.value], ch[:n.value]):
            desc = {"last": c & 1, "sub": (c >> 1) & 1,
                    "log2_n": (c >> 2) & 63, "log2_inner_bytes": c >> 8}
            names = [self.KERNELS[i] for i in range(len(self.KERNELS))
                     if (k >> i) & 1]
            out.append((c, desc, names, self.KERNELS[x]))
        return out

    def set_tuning(self, choices, forward=True):
        """Set the kernel of classes of one direction's plan: `choices` maps
        class codes (as tuning() reports them) to kernel names or numbers.
        Raises ValueError, changing nothing, for a class the plan lacks or a
        kernel that does not apply to it."""
        items = list(choices.items())
        cl = (ctypes.c_int32 * max(1, len(items)))()
        ch = (ctypes.c_int32 * max(1, len(items)))()
        for i, (c, k) in enumerate(items):
            cl[i] = int(c)
            ch[i] = self.KERNELS.index(k) if isinstance(k, str) else int(k)
        _lib.check(self._lib.paliwa_gb_batch_set_tuning(
            self._h, int(forward), len(items), cl, ch))

    def close(self):
        if self._h:
            self._lib.paliwa_gb_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def group_ranges(sizes, groups):
    """Split consecutive items of the given sizes into at most ``groups``
    consecutive, non-empty ranges [a, b) of about equal total size."""
    total = sum(sizes)
    groups = max(1, min(int(groups), len(sizes)))
    out, a, acc = [], 0, 0
    for i, s in enumerate(sizes):
        acc += s
        left = len(sizes) - (i + 1)
        want = len(out) + 1
        if want < groups and (acc * groups >= total * want
                              or left == groups - want):
            out.append((a, i + 1))
            a = i + 1
    out.append((a, len(sizes)))
    return out


class HostBatch:
    """Transforms of a batch of grids held in host memory, with the copies
    to and from the device overlapped with the transforms.

    The grids are packed into one device buffer (the layout of
    :func:`packed_grids`, which is also the layout of the host buffers) and
    split into ``groups`` consecutive groups of about equal size, each with
    its own plan (:class:`Batch`). :meth:`run` copies group g in on one copy
    stream, transforms it on the compute stream once it has landed, and
    copies it out on a second copy stream once transformed, so that group
    g + 1 arrives and group g - 1 leaves while group g is transformed. Host
    buffers should be pinned (``pin_memory()``) for the copies to be
    asynchronous. ``batch_groups`` is passed to every group's
    :class:`Batch` (its parallel branches); ``copy_streams`` streams per
    direction carry the copies (groups dealt round-robin), so that copies
    of neighbouring groups in one direction may run at once."""

    def __init__(self, levels, minimum_level, maximum_level,
                 wavelet_name="hat", dtype=None, compensated=False, groups=8,
                 device=None, align=64, batch_groups=None, copy_streams=1):
        import torch
        dtype = torch.float32 if dtype is None else dtype
        self.levels = [tuple(int(x) for x in l) for l in levels]
        self.buf, self.grids = packed_grids(self.levels, dtype,
                                            device or "cuda", align)
        base = self.buf.data_ptr()
        esz = self.buf.element_size()
        starts = [(g.data_ptr() - base) // esz for g in self.grids]
        ends = starts[1:] + [self.buf.numel()]
        self.ranges = group_ranges([e - s for s, e in zip(starts, ends)],
                                   groups)
        self.spans = [(starts[a], ends[b - 1]) for a, b in self.ranges]
        self.batches = [Batch(self.grids[a:b], self.levels[a:b],
                              minimum_level, maximum_level, wavelet_name,
                              compensated, batch_groups)
                        for a, b in self.ranges]
        dev = self.buf.device
        k = max(1, int(copy_streams))
        self._in = [torch.cuda.Stream(dev) for _ in range(k)]
        self._out = [torch.cuda.Stream(dev) for _ in range(k)]
        self._run = torch.cuda.Stream(dev)
        self._streams = self._in + [self._run] + self._out
        self.points = sum(g.numel() for g in self.grids)

    def numel(self):
        """Elements of the packed host (and device) buffers."""
        return self.buf.numel()

    def run(self, host_in, host_out, steps=("hierarchize", "dehierarchize"),
            stream=None):
        """Copy ``host_in`` in, apply the ``steps`` (method names of
        :class:`Batch`, in order) to every grid, copy the result to
        ``host_out``. Ordered after the current (or given) stream, which
        waits for the last copy out."""
        import torch
        if host_in.numel() != self.buf.numel() or \
                host_out.numel() != self.buf.numel():
            raise _lib.InvalidArgument("host buffers must hold numel() "
                                       "elements in the packed layout")
        cur = stream or torch.cuda.current_stream(self.buf.device)
        s_run = self._run
        start = torch.cuda.Event()
        start.record(cur)
        for s in self._streams:
            s.wait_event(start)
        landed, done = [], []
        for i, (a, b) in enumerate(self.spans):
            s_in = self._in[i % len(self._in)]
            with torch.cuda.stream(s_in):
                self.buf[a:b].copy_(host_in[a:b], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(s_in)
                landed.append(ev)
        for bt, ev in zip(self.batches, landed):
            s_run.wait_event(ev)
            for name in steps:
                getattr(bt, name)(s_run)
            ev2 = torch.cuda.Event()
            ev2.record(s_run)
            done.append(ev2)
        for i, ((a, b), ev) in enumerate(zip(self.spans, done)):
            s_out = self._out[i % len(self._out)]
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev)
                host_out[a:b].copy_(self.buf[a:b], non_blocking=True)
        for s_out in self._out:
            end = torch.cuda.Event()
            end.record(s_out)
            cur.wait_event(end)

    def close(self):
        for bt in self.batches:
            bt.close()
        self.batches = []


class CombinationTechnique:
    """Sparse-grid combine / restrict / scatter of a combination scheme."""

    def __init__(self, grids, levels, coefficients, maximum_level,
                 keep_all=False):
        _check_grids(grids, levels)
        self.grids = list(grids)
        self.levels = [tuple(int(x) for x in l) for l in levels]
        self.maximum_level = tuple(int(x) for x in maximum_level)
        self.ndim = len(self.levels[0])
        flat = [x for l in self.levels for x in l]
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        dtype = _lib.F64 if grids[0].dtype.itemsize == 8 else _lib.F32
        _lib.check(self._lib.paliwa_gb_ct_create(
            self.ndim, len(grids), _lib.i64(flat), _lib.f64(coefficients),
            _lib.i64(self.maximum_level), dtype, _ptr_array(grids),
            int(keep_all), ctypes.byref(self._h)))
        n, ns = ctypes.c_int64(), ctypes.c_int64()
        _lib.check(self._lib.paliwa_gb_ct_info(self._h, ctypes.byref(n),
                                               ctypes.byref(ns)))
        self.npoints, self.nsubspaces = n.value, ns.value

    def subspaces(self):
        """(level vectors, first sparse point of each), lexicographic."""
        lv = (ctypes.c_int64 * max(1, self.nsubspaces * self.ndim))()
        off = (ctypes.c_int64 * max(1, self.nsubspaces))()
        _lib.check(self._lib.paliwa_gb_ct_subspaces(self._h, lv, off))
        levels = [tuple(lv[i * self.ndim:(i + 1) * self.ndim])
                  for i in range(self.nsubspaces)]
        return levels, list(off[:self.nsubspaces])

    def combine(self, sparse=None, stream=None):
        import torch
        if sparse is None:
            sparse = torch.empty(self.npoints, dtype=torch.float64,
                                 device=self.grids[0].device)
        self._check_sparse(sparse)
        _lib.check(self._lib.paliwa_gb_ct_combine(
            self._h, sparse.data_ptr(), _stream_handle(self.grids[0], stream)))
        return sparse

    def restrict(self, sparse, stream=None):
        self._check_sparse(sparse)
        _lib.check(self._lib.paliwa_gb_ct_restrict(
            self._h, sparse.data_ptr(), _stream_handle(self.grids[0], stream)))

    def scatter(self, sparse, full=None, stream=None):
        import torch
        self._check_sparse(sparse)
        shape = [1 << l for l in self.maximum_level]
        if full is None:
            full = torch.empty(shape, dtype=torch.float64,
                               device=self.grids[0].device)
        if (full.dtype != torch.float64 or not full.is_contiguous()
                or full.numel() != math.prod(shape)):
            raise _lib.InvalidArgument("full grid must be float64 at lmax")
        _lib.check(self._lib.paliwa_gb_ct_scatter(
            self._h, sparse.data_ptr(), full.data_ptr(),
            _stream_handle(self.grids[0], stream)))
        return full

    def _check_sparse(self, sparse):
        import torch
        if (sparse.dtype != torch.float64 or not sparse.is_cuda
                or not sparse.is_contiguous()
                or sparse.numel() != self.npoints):
            raise _lib.InvalidArgument(
                f"sparse grid must be a float64 CUDA tensor of {self.npoints}")

    def close(self):
        if self._h:
            self._lib.paliwa_gb_ct_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def subspace_count(levels):
    """Host restatement of the subspace counting, for planning and tests
    (paliwa_utils.hpp:9-26)."""
    counts = {}
    for lv in levels:
        for s in itertools.product(*[range(int(x) + 1) for x in lv]):
            counts[s] = counts.get(s, 0) + 1
    return counts
