"""Host-side mirror of paliwa's transform API (paliwa/paliwa_transform.hpp).

Same names, argument meaning and error behaviour as the reference's
header-only templates, over CUDA tensors instead of DDC chunk spans:

* ``hierarchize(grid, level, minimum_level, maximum_level, wavelet_name)``
  -- paliwa_transform.hpp:401-415
* ``dehierarchize(...)`` -- :417-431
* ``hierarchize_in(grid, dim, level, minimum_level, maximum_level, ...)``
  and ``dehierarchize_in`` -- :346-399 (``Dim`` becomes ``dim``)
* ``transform_in(grid, dim, level, maximum_level, levels, filters)``
  -- :215-251 (full-grid overload); ``transform_in_window`` for a grid that
  holds only a box of the lattice (the reference's bounds-checked passes)

A grid is a C-contiguous CUDA tensor holding the dense row-major storage of
``strided_domain_from_level(level, maximum_level)``: 2^level[d] points along
dimension d. float64 grids compute in double (the reference's Value =
double); float32 grids compute in float (Value = float) or, with
``compensated=True``, in double-float registers rounded to float once per
dimension. Every call is asynchronous on ``stream`` (default: the current
torch stream of the grid's device), like the reference on an execution-space
instance. All work runs in the CUDA library; there is no CPU path.
"""
from __future__ import annotations

from . import _lib

# paliwa/paliwa_wavelets.hpp:15-28
lifting_wavelet_filter_offsets_and_coefficients = {
    "hat": [(1, (-0.5, 1.0, -0.5))],
    "biorthogonal": [(1, (-0.5, 1.0, -0.5)), (0, (0.25, 1.0, 0.25))],
    "fullweighting": [(0, (0.25, 0.5, 0.25)), (1, (-0.5, 1.0, -0.5))],
}
lifting_wavelet_reconstruct_offsets_and_coefficients = {
    "hat": [(1, (0.5, 1.0, 0.5))],
    "biorthogonal": [(0, (-0.25, 1.0, -0.25)), (1, (0.5, 1.0, 0.5))],
    "fullweighting": [(1, (0.5, 1.0, 0.5)), (0, (-0.5, 2.0, -0.5))],
}


def wavelet_id(name):
    """Wavelet name -> library id; unknown names raise OutOfRange (a
    KeyError), as ``std::map::at`` throws std::out_of_range
    (paliwa_transform.hpp:370, 397)."""
    import ctypes
    out = ctypes.c_int(-1)
    _lib.check(_lib.load().paliwa_gb_wavelet_id(wavelet_name_bytes(name),
                                                 ctypes.byref(out)))
    return out.value


def wavelet_name_bytes(name):
    return name.encode() if isinstance(name, str) else bytes(name)


def _dtype_code(grid, compensated):
    import torch
    if grid.dtype == torch.float64:
        if compensated:
            raise _lib.InvalidArgument(
                "compensated arithmetic applies to float32 grids")
        return _lib.F64
    if grid.dtype == torch.float32:
        return _lib.F32C if compensated else _lib.F32
    raise _lib.InvalidArgument(f"unsupported grid dtype {grid.dtype}")


def _check_grid(grid, level):
    import torch
    if not isinstance(grid, torch.Tensor):
        raise _lib.InvalidArgument("grid must be a torch.Tensor")
    if not grid.is_cuda:
        raise _lib.InvalidArgument("grid must live in CUDA device memory")
    if not grid.is_contiguous():
        raise _lib.InvalidArgument("grid must be C-contiguous")
    expected = 1 << sum(int(l) for l in level)
    if grid.numel() != expected:
        raise _lib.InvalidArgument(
            f"grid has {grid.numel()} points, level {tuple(level)} needs "
            f"{expected}")


def _stream_handle(grid, stream):
    import torch
    if stream is None:
        stream = torch.cuda.current_stream(grid.device)
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


def _call(fn_name, grid, args, stream):
    import torch
    lib = _lib.load()
    with torch.cuda.device(grid.device):
        s = _stream_handle(grid, stream)
        _lib.check(getattr(lib, fn_name)(grid.data_ptr(), *args, s))


def hierarchize(grid, level, minimum_level, maximum_level,
                wavelet_name="hat", stream=None, compensated=False):
    """Forward transform over every dimension, dimension 0 first."""
    _check_grid(grid, level)
    d = len(level)
    _call("paliwa_gb_hierarchize", grid,
          (_dtype_code(grid, compensated), d, _lib.i64(level),
           _lib.i64(minimum_level), _lib.i64(maximum_level),
           wavelet_id(wavelet_name)), stream)
    return grid


def dehierarchize(grid, level, minimum_level, maximum_level,
                  wavelet_name="hat", stream=None, compensated=False):
    """Inverse transform over every dimension, dimension 0 first."""
    _check_grid(grid, level)
    d = len(level)
    _call("paliwa_gb_dehierarchize", grid,
          (_dtype_code(grid, compensated), d, _lib.i64(level),
           _lib.i64(minimum_level), _lib.i64(maximum_level),
           wavelet_id(wavelet_name)), stream)
    return grid


def hierarchize_in(grid, dim, level, minimum_level, maximum_level,
                   wavelet_name="hat", stream=None, compensated=False):
    """Forward transform along one dimension (levels level..lmin+1)."""
    _check_grid(grid, level)
    _call("paliwa_gb_hierarchize_in", grid,
          (_dtype_code(grid, compensated), len(level), _lib.i64(level),
           _lib.i64(minimum_level), _lib.i64(maximum_level), int(dim),
           wavelet_id(wavelet_name)), stream)
    return True


def dehierarchize_in(grid, dim, level, minimum_level, maximum_level,
                     wavelet_name="hat", stream=None, compensated=False):
    """Inverse transform along one dimension (levels lmin+1..level)."""
    _check_grid(grid, level)
    _call("paliwa_gb_dehierarchize_in", grid,
          (_dtype_code(grid, compensated), len(level), _lib.i64(level),
           _lib.i64(minimum_level), _lib.i64(maximum_level), int(dim),
           wavelet_id(wavelet_name)), stream)
    return True


def transform_in(grid, dim, level, maximum_level, levels, filters,
                 stream=None, compensated=False):
    """transform_in<Dim> (full-grid overload): for each level in ``levels``
    (in order) and each ``(offset, (c0, c1, c2))`` in ``filters`` (in order),
    one lifting pass along ``dim``."""
    _check_grid(grid, level)
    filters = list(filters)
    levels = [int(l) for l in levels]
    _call("paliwa_gb_transform_in", grid,
          (_dtype_code(grid, compensated), len(level), _lib.i64(level),
           _lib.i64(maximum_level), int(dim), _lib.i64(levels), len(levels),
           _lib.i32([o for o, _ in filters]),
           _lib.f64([c for _, f in filters for c in f]), len(filters)),
          stream)
    return True


def transform_in_window(grid, dim, level, maximum_level, levels, filters,
                        window_front, stream=None):
    """transform_in<Dim> (full-grid overload) on a grid tensor that holds
    only a box of the level lattice: along dimension d the uids
    ``window_front[d] + k * 2^(maximum_level[d] - level[d])`` for
    ``k < grid.shape[d]``. The reference's bounds-checked passes: a point is
    updated only when it and both periodic neighbours are in the box
    (paliwa_transform.hpp:24-51, :224-247). float64 or float32 grids."""
    if not grid.is_contiguous():
        raise _lib.InvalidArgument("grid must be C-contiguous")
    if grid.dim() != len(level):
        raise _lib.InvalidArgument("grid rank must equal len(level)")
    filters = list(filters)
    levels = [int(l) for l in levels]
    code = _lib.F64 if grid.element_size() == 8 else _lib.F32
    _call("paliwa_gb_transform_in_window", grid,
          (code, len(level), _lib.i64(level), _lib.i64(maximum_level),
           _lib.i64(window_front), _lib.i64(list(grid.shape)), int(dim),
           _lib.i64(levels), len(levels), _lib.i32([o for o, _ in filters]),
           _lib.f64([c for _, f in filters for c in f]), len(filters)),
          stream)
    return True


def transform_bounds(outputs, level, maximum_level, levels, filters):
    """paliwa::transform_bounds (paliwa_domains.hpp:357-452) through the
    library's host planner: ``outputs`` is ``None`` (empty) or ``(min, max)``
    in finest-level uids (min > max wraps). Returns ``(bounds, writes)``:
    the required input bounds per hierarchical level 0..level and the write
    bounds of each (level index, pass), each ``None`` or ``(min, max)``.
    Only the filter offsets are read. Host code; needs no GPU."""
    import ctypes
    levels = [int(l) for l in levels]
    filters = list(filters)
    lo, hi = (-1, -1) if outputs is None else (int(outputs[0]),
                                               int(outputs[1]))
    nb = 2 * (int(level) + 1)
    nw = 2 * max(1, len(levels) * len(filters))
    b = (ctypes.c_int64 * nb)()
    w = (ctypes.c_int64 * nw)()
    _lib.check(_lib.load().paliwa_gb_transform_bounds(
        lo, hi, int(level), int(maximum_level), _lib.i64(levels), len(levels),
        _lib.i32([o for o, _ in filters]), len(filters), b, w))

    def pairs(a, n):
        return [None if a[2 * k] < 0 else (a[2 * k], a[2 * k + 1])
                for k in range(n)]

    bounds = pairs(b, int(level) + 1)
    flat = pairs(w, len(levels) * len(filters))
    writes = [flat[i * len(filters):(i + 1) * len(filters)]
              for i in range(len(levels))]
    return bounds, writes


def transform_outputs(grid, dim, level, maximum_level, levels, filters,
                      outputs, window_front=None, stream=None):
    """transform_in<Dim>(grid, level, maximum_level, levels, filters,
    outputs, ...) (paliwa_transform.hpp:258-344): the lifting sequence along
    ``dim`` restricted to the points the outputs depend on.

    ``grid`` is a C-contiguous float64 or float32 CUDA tensor holding a
    window of the grid: along dimension d its ``grid.shape[d]`` points are
    the uids ``(window_front[d] + k * 2^(L[d] - level[d])) mod 2^L[d]``
    (default front 0; the full grid is front 0 with 2^level points).
    ``outputs`` is ``(front, extents, strides)`` in uids, like a
    ``StridedDiscreteDomain``. A required input outside the window raises
    PaliwaError (the reference's std::runtime_error)."""
    import torch
    if not isinstance(grid, torch.Tensor) or not grid.is_cuda:
        raise _lib.InvalidArgument("grid must be a CUDA tensor")
    if not grid.is_contiguous():
        raise _lib.InvalidArgument("grid must be C-contiguous")
    nd = len(level)
    if grid.dim() != nd:
        raise _lib.InvalidArgument("grid must have one axis per dimension")
    if window_front is None:
        window_front = (0,) * nd
    front, extents, strides = outputs
    filters = list(filters)
    levels = [int(l) for l in levels]
    _call("paliwa_gb_transform_outputs", grid,
          (_dtype_code(grid, False), nd, _lib.i64(level),
           _lib.i64(maximum_level), _lib.i64(window_front),
           _lib.i64(grid.shape), int(dim), _lib.i64(levels), len(levels),
           _lib.i32([o for o, _ in filters]),
           _lib.f64([c for _, f in filters for c in f]), len(filters),
           _lib.i64(front), _lib.i64(extents), _lib.i64(strides)), stream)
    return True
