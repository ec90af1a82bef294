"""The allocation-free transform (paliwa_gb_transform_noalloc) gives the same
results as the allocating entry points.

It exists for callers that cannot let a library allocate device memory
(graph captures that must replay without allocation nodes, processes whose
own allocator holds the device memory, solver loops that cannot afford
allocator latency). Grids with pencils longer than 4096 points use its 64 MiB
static scratch array; the cases below do, and each is checked on two calls in
a row, since the array keeps the previous call's contents. This file sorts
last so that a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

from paliwa_gb300 import _lib

pytestmark = pytest.mark.gpu

# (dtype code, numpy dtype, level, wavelet id)
CASES = [
    (_lib.F64, np.float64, (16, 3), _lib.BIORTHOGONAL),
    (_lib.F64, np.float64, (2, 14, 2), _lib.HAT),
    (_lib.F32C, np.float32, (17, 2), _lib.BIORTHOGONAL),
    (_lib.F32, np.float32, (3, 15), _lib.FULLWEIGHTING),
]


def run(fn, dev, dtype_code, level, lmin, wavelet, direction, stream):
    lib = _lib.load()
    n = len(level)
    if fn == "noalloc":
        rc = lib.paliwa_gb_transform_noalloc(
            dev.data_ptr(), dtype_code, n, _lib.i64(level), _lib.i64(lmin),
            _lib.i64(level), wavelet, direction, stream)
    else:
        f = (lib.paliwa_gb_hierarchize if direction > 0
             else lib.paliwa_gb_dehierarchize)
        rc = f(dev.data_ptr(), dtype_code, n, _lib.i64(level), _lib.i64(lmin),
               _lib.i64(level), wavelet, stream)
    _lib.check(rc)


@pytest.mark.parametrize("case", CASES)
def test_noalloc_matches_allocating_entry_points(case):
    import torch
    code, npdt, level, wavelet = case
    lmin = (1,) * len(level)
    rng = np.random.default_rng(sum(level))
    s = torch.cuda.Stream()
    for call in range(2):  # two calls in a row share the static scratch
        direction = 1 if call == 0 else -1
        x = torch.from_numpy(
            rng.uniform(-1, 1, [1 << l for l in level]).astype(npdt)).cuda()
        a, b = x.clone(), x.clone()
        torch.cuda.synchronize()
        run("noalloc", a, code, level, lmin, wavelet, direction, s.cuda_stream)
        run("alloc", b, code, level, lmin, wavelet, direction, s.cuda_stream)
        s.synchronize()
        # FP64 and FP32 are bit-exact in every test; FP32c is deterministic,
        # so the two entry points agree exactly as well.
        assert torch.equal(a, b), (level, call)
        assert not torch.equal(a, x)


def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch
    level = (20, 4)  # 2^24 doubles = 128 MiB > 64 MiB, pencil of 2^20 points
    g = torch.zeros(16, dtype=torch.float64, device="cuda")  # never touched
    lib = _lib.load()
    rc = lib.paliwa_gb_transform_noalloc(
        g.data_ptr(), _lib.F64, 2, _lib.i64(level), _lib.i64((0, 0)),
        _lib.i64(level), _lib.HAT, 1, None)
    assert rc == _lib.INVALID_ARGUMENT
    assert b"64 MiB" in lib.paliwa_gb_last_error()
