"""Raw dump of device grids (paliwa/paliwa_io.hpp:13-23): the file holds the
grid's values in storage order with no header, so numpy.fromfile -- what
paliwa/postprocess.py does -- reads the grid back bit for bit."""
import os

import numpy as np
import pytest

from paliwa_gb300 import _lib
from paliwa_gb300 import io as pio


def test_reference_file_names():
    # paliwa/postprocess.py:25-33, 37-50
    assert pio.raw_grid_filename((6, 6)) == "strided_grid_6_6_2d.raw"
    assert (pio.raw_grid_filename((5, 4, 3), "distributed_grid", 2) ==
            "distributed_grid_5_4_3_3d_rank2.raw")


def test_unwritable_file_is_a_runtime_error(tmp_path):
    lib = _lib.load()
    bad = str(tmp_path / "no_such_dir" / "grid.raw").encode()
    rc = lib.paliwa_gb_dump_to_binary_file(None, 0, bad, None)
    assert rc == _lib.RUNTIME_ERROR
    assert b"cannot open" in lib.paliwa_gb_last_error()
    rc = lib.paliwa_gb_dump_to_binary_file(None, 8, bad, None)
    assert rc == _lib.INVALID_ARGUMENT


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,level", [("float64", (6, 6)),
                                         ("float32", (5, 4, 3)),
                                         ("float64", (12, 12))])
def test_dump_reads_back_with_fromfile(tmp_path, dtype, level):
    """(12, 12) in float64 is 128 MiB: four pieces through the two pinned
    buffers."""
    import torch
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, [1 << l for l in level]).astype(dtype)
    g = torch.from_numpy(x).cuda()
    # Work queued before the dump on the same stream is in the file.
    g.mul_(2.0)
    path = tmp_path / pio.raw_grid_filename(level)
    pio.dump_chunk_span_to_binary_file(g, path)
    got = np.fromfile(path, dtype=dtype).reshape(x.shape)
    assert np.array_equal(got, x * 2)
    # An existing file is truncated.
    pio.dump_chunk_span_to_binary_file(g[:1].contiguous(), path)
    assert os.path.getsize(path) == g[:1].numel() * g.element_size()
