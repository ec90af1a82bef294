"""One host thread driving two GPUs: each kernel's shared-memory opt-in and
occupancy are set up per device, so the staged and tile kernels (which need
the opt-in for more than 48 KB of dynamic shared memory) launch on the
second device after running on the first. Skipped with fewer than two GPUs.
"""
import numpy as np
import pytest

import paliwa_gb300 as pg

pytestmark = pytest.mark.gpu


def test_same_thread_two_devices():
    import torch
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    import oracle as O
    O.build()
    # (12, 3): the last axis of 8 points and a strided 4096-point axis (the
    # staged kernel, 32-point chunks for FP32c, tile kernel for FP64/FP32).
    level, lmin = (12, 3), (0, 0)
    x = np.random.default_rng(3).uniform(-1, 1, [1 << l for l in level])
    want = O.hierarchize(x.copy(), level, lmin, level, "biorthogonal")
    for dev in (0, 1, 0):
        with torch.cuda.device(dev):
            g = torch.from_numpy(x.copy()).to(f"cuda:{dev}")
            pg.hierarchize(g, level, lmin, level, "biorthogonal")
            g32 = torch.from_numpy(x.astype(np.float32)).to(f"cuda:{dev}")
            pg.hierarchize(g32, level, lmin, level, "biorthogonal",
                           compensated=True)
            torch.cuda.synchronize(dev)
            assert np.array_equal(g.cpu().numpy(), want)
            err = np.abs(g32.cpu().numpy().astype(np.float64) - want).max()
            assert err <= 1e-6 * np.abs(want).max()
