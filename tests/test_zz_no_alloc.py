"""The allocation-free transform (paliwa_gb_transform_noalloc).

Who needs it: programs whose own allocator already holds the GPU's memory (a
framework's caching pool, a solver's arena), where a library allocation can
fail or fragment that memory, and time-step loops that cannot pay for
allocator calls or for the device synchronization that cudaFree implies.
The allocating entry points take the scratch of grids with pencils longer
than 4096 points from the stream-ordered allocator; this entry point takes
it from one 64 MiB array in device memory instead.

Checked here, through the C ABI: the same results as the allocating entry
point (bit for bit) and as the CPU oracle, on two calls in a row (the array
keeps the previous call's contents); no allocation from the device's memory
pool and no change of the free device memory during those calls; grids
needing more than 64 MiB of scratch are rejected before any work is queued.
This file sorts last so that a run stopping at the first failure has run
every other test first.
"""
import ctypes

import numpy as np
import pytest

from paliwa_gb300 import _lib

pytestmark = pytest.mark.gpu

# (dtype code, numpy dtype, level, wavelet id): every case has a pencil of
# more than 4096 points, so it uses the scratch array.
CASES = [
    (_lib.F64, np.float64, (16, 3), _lib.BIORTHOGONAL),
    (_lib.F64, np.float64, (2, 14, 2), _lib.HAT),
    (_lib.F32C, np.float32, (17, 2), _lib.BIORTHOGONAL),
    (_lib.F32, np.float32, (3, 15), _lib.FULLWEIGHTING),
]
WAVELET_NAMES = {_lib.HAT: "hat", _lib.BIORTHOGONAL: "biorthogonal",
                 _lib.FULLWEIGHTING: "fullweighting"}

# cuda.h: CUmemPool_attribute CU_MEMPOOL_ATTR_USED_MEM_HIGH (cuuint64_t).
_USED_MEM_HIGH = 8


class DevicePool:
    """High watermark of the current memory pool of device 0 (the pool the
    stream-ordered allocator draws from), through the driver API."""

    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        assert self.cu.cuDeviceGet(ctypes.byref(dev), 0) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetMemPool(ctypes.byref(self.pool), dev) == 0

    def reset(self):
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(
            self.pool, _USED_MEM_HIGH, ctypes.byref(zero)) == 0

    def high(self):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(
            self.pool, _USED_MEM_HIGH, ctypes.byref(v)) == 0
        return v.value


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


def oracle_result(x, level, lmin, wavelet, direction):
    import oracle
    oracle.build()
    y = np.array(x, dtype=np.float64 if x.dtype == np.float64 else x.dtype)
    return oracle.hierarchize(y, level, lmin, level, WAVELET_NAMES[wavelet],
                              forward=direction > 0)


@pytest.mark.parametrize("case", CASES)
def test_noalloc_matches_allocating_entry_point_and_oracle(case):
    import torch
    code, npdt, level, wavelet = case
    lmin = (1,) * len(level)
    rng = np.random.default_rng(sum(level))
    s = torch.cuda.Stream()
    for call in range(2):  # two calls in a row share the static scratch
        direction = 1 if call == 0 else -1
        host = rng.uniform(-1, 1, [1 << l for l in level]).astype(npdt)
        x = torch.from_numpy(host).cuda()
        a, b = x.clone(), x.clone()
        torch.cuda.synchronize()
        run("noalloc", a, code, level, lmin, wavelet, direction, s.cuda_stream)
        run("alloc", b, code, level, lmin, wavelet, direction, s.cuda_stream)
        s.synchronize()
        # Every path gives the same bits (FP32c is deterministic too).
        assert torch.equal(a, b), (level, call)
        assert not torch.equal(a, x)
        got = a.cpu().numpy()
        if code == _lib.F32C:
            # Compensated arithmetic against the FP64 oracle, normwise.
            want = oracle_result(host.astype(np.float64), level, lmin,
                                 wavelet, direction)
            err = np.max(np.abs(got.astype(np.float64) - want))
            assert err <= 1e-6 * np.max(np.abs(want)), (level, call, err)
        else:
            want = oracle_result(host, level, lmin, wavelet, direction)
            assert np.array_equal(got, want), (level, call)


def test_noalloc_allocates_nothing():
    import torch
    code, npdt, level, wavelet = CASES[0]
    lmin = (1,) * len(level)
    rng = np.random.default_rng(7)
    x = torch.from_numpy(
        rng.uniform(-1, 1, [1 << l for l in level]).astype(npdt)).cuda()
    s = torch.cuda.Stream()
    pool = DevicePool()
    # Warm-up: the first call on a device loads the library's device code
    # (and with it the array) and looks up the array's address.
    run("noalloc", x, code, level, lmin, wavelet, 1, s.cuda_stream)
    run("noalloc", x, code, level, lmin, wavelet, -1, s.cuda_stream)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    pool.reset()
    for direction in (1, -1):
        run("noalloc", x, code, level, lmin, wavelet, direction,
            s.cuda_stream)
    s.synchronize()
    assert pool.high() == 0
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    # The check can see an allocation: the allocating entry point takes the
    # same grid's scratch from that pool.
    pool.reset()
    run("alloc", x, code, level, lmin, wavelet, 1, s.cuda_stream)
    s.synchronize()
    assert pool.high() >= x.numel() * x.element_size()


def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch
    level = (20, 4)  # 2^24 doubles = 128 MiB > 64 MiB, pencil of 2^20 points
    # A buffer of the grid's full size, so that a regression of the size
    # check shows up as a wrong return code or a changed buffer.
    g = torch.full((1 << 20, 1 << 4), 3.0, dtype=torch.float64,
                   device="cuda")
    torch.cuda.synchronize()
    lib = _lib.load()
    rc = lib.paliwa_gb_transform_noalloc(
        g.data_ptr(), _lib.F64, 2, _lib.i64(level), _lib.i64((0, 0)),
        _lib.i64(level), _lib.HAT, 1, None)
    torch.cuda.synchronize()
    assert rc == _lib.INVALID_ARGUMENT
    assert b"64 MiB" in lib.paliwa_gb_last_error()
    assert bool((g == 3.0).all())
