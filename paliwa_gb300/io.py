"""Raw dump of device grids (paliwa/paliwa_io.hpp:13-23).

``dump_chunk_span_to_binary_file(grid, filename)`` writes a CUDA tensor's
values in storage order (row-major, native byte order, no header), the raw
format that paliwa/postprocess.py reads with ``numpy.fromfile``; the copy to
the host runs in the CUDA library through pinned buffers, overlapped with the
file write. ``raw_grid_filename`` gives the reference's file names.
"""
from __future__ import annotations

from . import _lib


def raw_grid_filename(level, prefix="strided_grid", rank=None):
    """paliwa/postprocess.py:25-33 (serial) and :37-50 (per rank):
    ``{prefix}_{l0}_{l1}..._{d}d.raw`` or ``..._rank{r}.raw``."""
    name = "_".join(str(int(l)) for l in level) + f"_{len(level)}d"
    if rank is None:
        return f"{prefix}_{name}.raw"
    return f"{prefix}_{name}_rank{int(rank)}.raw"


def dump_chunk_span_to_binary_file(grid, filename, stream=None):
    """Write ``grid`` (a contiguous CUDA tensor) to ``filename``, ordered
    after the work queued on ``stream`` (default: the current torch stream
    of the grid's device)."""
    import torch
    if not isinstance(grid, torch.Tensor) or not grid.is_cuda:
        raise _lib.InvalidArgument("grid must be a CUDA tensor")
    if not grid.is_contiguous():
        raise _lib.InvalidArgument("grid must be C-contiguous")
    lib = _lib.load()
    with torch.cuda.device(grid.device):
        s = torch.cuda.current_stream(grid.device) if stream is None else stream
        h = s.cuda_stream if hasattr(s, "cuda_stream") else int(s)
        _lib.check(lib.paliwa_gb_dump_to_binary_file(
            grid.data_ptr(), grid.numel() * grid.element_size(),
            str(filename).encode(), h))
