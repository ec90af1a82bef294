// CPU oracle for the paliwa lifting-wavelet (hierarchization) transform.
//
// TEST INFRASTRUCTURE ONLY. This file restates, on the CPU, the algorithm of
// the reference library paliwa (header-only C++20 over DDC/Kokkos) so that the
// GPU product can be checked against it. Only tests/, the smoke check and the
// CPU-baseline leg of bench.py may load it. It is never the thing measured as
// the GPU path and never a fallback for it.
//
// The reference cannot be compiled in this environment (DDC, Kokkos, MPI and
// GoogleTest are absent), so parity is pinned to the reference's own tests:
// its in-test 1D periodic reference loop (test/test_paliwa_plan.cpp:128-139),
// its property tests (test/test_paliwa_transform.cpp:57-73, 127-131) and its
// known-answer tests for the index maps and the combination technique.
//
// Arithmetic follows paliwa/paliwa_transform.hpp:46-49 exactly:
//   g[i] = (Value)c0 * g[lower] + (Value)c1 * g[i] + (Value)c2 * g[upper]
// evaluated left to right with one rounding per operation. Build with
// -ffp-contract=off so that no fused multiply-add changes the rounding.
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace paliwa_oracle {

using Filters = std::vector<std::pair<int, std::array<double, 3>>>;

// Wavelet tables: paliwa/paliwa_wavelets.hpp:15-28 (forward :17-20, inverse
// :24-27). Index 0 = hat, 1 = biorthogonal, 2 = fullweighting.
inline Filters forward_filters(int wavelet) {
  switch (wavelet) {
  case 0: return {{1, {-0.5, 1.0, -0.5}}};
  case 1: return {{1, {-0.5, 1.0, -0.5}}, {0, {0.25, 1.0, 0.25}}};
  case 2: return {{0, {0.25, 0.5, 0.25}}, {1, {-0.5, 1.0, -0.5}}};
  }
  throw std::out_of_range("unknown wavelet");
}
inline Filters inverse_filters(int wavelet) {
  switch (wavelet) {
  case 0: return {{1, {0.5, 1.0, 0.5}}};
  case 1: return {{0, {-0.25, 1.0, -0.25}}, {1, {0.5, 1.0, 0.5}}};
  case 2: return {{1, {0.5, 1.0, 0.5}}, {0, {-0.5, 2.0, -0.5}}};
  }
  throw std::out_of_range("unknown wavelet");
}

// Dense row-major grid at `level` inside `maximum_level`: 2^level[d] points in
// dimension d, last dimension fastest (paliwa/paliwa_domains.hpp:33-49 for the
// extents/strides, paliwa/postprocess.py:30-35 for the row-major layout).
struct Shape {
  int ndim = 0;
  std::array<long, 16> level{}, maximum_level{};
  long extent(int d) const { return 1L << level[d]; }
  long size() const {
    long s = 1;
    for (int d = 0; d < ndim; ++d) s *= extent(d);
    return s;
  }
  // View as [outer, n, inner] around dimension `dim`.
  void split(int dim, long &outer, long &n, long &inner) const {
    outer = 1;
    inner = 1;
    for (int d = 0; d < dim; ++d) outer *= extent(d);
    for (int d = dim + 1; d < ndim; ++d) inner *= extent(d);
    n = extent(dim);
  }
};

enum class Mode { Direct = 0, PackedPoles = 1 };

// One lifting pass: paliwa/paliwa_transform.hpp:24-51 (detail::lifting_pass)
// over the even or odd half of the operating domain (:238-241). The periodic
// neighbour rule is the reference's, written in uid space at :37-41:
//   lower = x == 0 ? period - stride : x - stride
//   upper = x + stride == period ? 0 : x + stride
// Here uid = k * unit with unit = 2^(L - level), stride = s * unit and
// period = n * unit, so the same rule holds for compact indices k, s, n.
template <typename Value>
void lifting_pass_direct(Value *g, long outer, long n, long inner, long s,
                         int offset, std::array<double, 3> const &f) {
  Value const c0 = static_cast<Value>(f[0]);
  Value const c1 = static_cast<Value>(f[1]);
  Value const c2 = static_cast<Value>(f[2]);
  long const writes = n / (2 * s);
#pragma omp parallel for collapse(2) schedule(static)
  for (long a = 0; a < outer; ++a) {
    for (long m = 0; m < writes; ++m) {
      long const k = offset * s + 2 * s * m;
      long const lo = k == 0 ? n - s : k - s;
      long const up = k + s == n ? 0 : k + s;
      Value *base = g + a * n * inner;
      for (long b = 0; b < inner; ++b) {
        Value const vl = base[lo * inner + b];
        Value const vm = base[k * inner + b];
        Value const vu = base[up * inner + b];
        base[k * inner + b] = c0 * vl + c1 * vm + c2 * vu;
      }
    }
  }
}

// transform_in (full overload) on a chunk that holds only a window of the
// level lattice: the reference's lifting_pass<CheckBounds = true>
// (paliwa/paliwa_transform.hpp:24-51, chosen when the chunk's domain is not
// the complete lattice, :224-228, :242-247). The window holds, along each
// dimension d, the uids front[d] + k * 2^(L[d] - level[d]) for
// k < extents[d] (no wrap: a DDC domain), dense and row-major. A write point
// is updated only when it and both of its periodic neighbours (:37-41) lie
// in the window; every other point keeps its value.
template <typename Value>
void transform_in_window(Value *g, Shape const &shape, long const *front,
                         long const *extents, int dim,
                         std::vector<long> const &levels,
                         Filters const &filters) {
  long outer = 1, inner = 1;
  for (int d = 0; d < dim; ++d) outer *= extents[d];
  for (int d = dim + 1; d < shape.ndim; ++d) inner *= extents[d];
  long const n = extents[dim];
  long const L = shape.maximum_level[dim];
  long const spacing = 1L << (L - shape.level[dim]);
  long const period = 1L << L;
  long const f = front[dim];
  auto index = [&](long uid) -> long {
    long const r = uid - f;
    if (r < 0 || r % spacing != 0) return -1;
    return r / spacing < n ? r / spacing : -1;
  };
  for (long l : levels) {
    if (l < 1 || l > shape.level[dim])
      throw std::invalid_argument("requires 1 <= level <= grid level");
    long const s = 1L << (L - l);
    for (auto const &[offset, c] : filters) {
      if (offset != 0 && offset != 1)
        throw std::runtime_error("Filter offset not supported");
      Value const c0 = static_cast<Value>(c[0]);
      Value const c1 = static_cast<Value>(c[1]);
      Value const c2 = static_cast<Value>(c[2]);
      for (long m = 0; m < (1L << (l - 1)); ++m) {
        long const x = offset * s + 2 * s * m;
        long const k = index(x);
        long const lo = index(x == 0 ? period - s : x - s);
        long const up = index(x + s == period ? 0 : x + s);
        if (k < 0 || lo < 0 || up < 0) continue;
        for (long a = 0; a < outer; ++a) {
          Value *base = g + a * n * inner;
          for (long b = 0; b < inner; ++b) {
            Value const vl = base[lo * inner + b];
            Value const vm = base[k * inner + b];
            Value const vu = base[up * inner + b];
            base[k * inner + b] = c0 * vl + c1 * vm + c2 * vu;
          }
        }
      }
    }
  }
}

// transform_in (full overload), paliwa/paliwa_transform.hpp:215-251: for each
// level in the given order, for each (offset, filter) in table order, one pass.
// `levels` are reference levels l (1 <= l <= level[dim]); the compact stride of
// level l is 2^(level[dim] - l) (:236-237).
template <typename Value>
void transform_in_direct(Value *g, Shape const &shape, int dim,
                         std::vector<long> const &levels,
                         Filters const &filters) {
  long outer, n, inner;
  shape.split(dim, outer, n, inner);
  for (long l : levels) {
    if (l < 1 || l > shape.level[dim])
      throw std::invalid_argument("Invalid transform level");
    long const s = 1L << (shape.level[dim] - l);
    for (auto const &[offset, filter] : filters) {
      if (offset != 0 && offset != 1)
        throw std::runtime_error("Filter offset not supported");
      lifting_pass_direct(g, outer, n, inner, s, offset, filter);
    }
  }
}

// The reference's CPU "pencil in scratch" execution
// (paliwa/paliwa_transform.hpp:53-210, PoleExecution::PackedPoles): gather one
// pole (pencil) into scratch, run every level and pass on it, scatter back.
// The per-point arithmetic is identical to the direct pass, so the results
// are bit-identical; only the memory traffic differs.
template <typename Value>
void transform_in_packed(Value *g, Shape const &shape, int dim,
                         std::vector<long> const &levels,
                         Filters const &filters) {
  long outer, n, inner;
  shape.split(dim, outer, n, inner);
  for (long l : levels)
    if (l < 1 || l > shape.level[dim])
      throw std::invalid_argument("Invalid transform level");
  for (auto const &pass : filters)
    if (pass.first != 0 && pass.first != 1)
      throw std::runtime_error("Filter offset not supported");
  // Pencils are processed in blocks of `width` neighbouring columns so the
  // gather and scatter stay cache friendly for strided dimensions.
  long const width = inner >= 8 ? 8 : inner;
  long const blocks = outer * (inner / width);
#pragma omp parallel
  {
    std::vector<Value> scratch(static_cast<size_t>(n * width));
#pragma omp for schedule(static)
    for (long blk = 0; blk < blocks; ++blk) {
      long const a = blk / (inner / width);
      long const b0 = (blk % (inner / width)) * width;
      Value *base = g + a * n * inner + b0;
      for (long k = 0; k < n; ++k)
        for (long w = 0; w < width; ++w)
          scratch[k * width + w] = base[k * inner + w];
      for (long l : levels) {
        long const s = 1L << (shape.level[dim] - l);
        for (auto const &[offset, f] : filters) {
          Value const c0 = static_cast<Value>(f[0]);
          Value const c1 = static_cast<Value>(f[1]);
          Value const c2 = static_cast<Value>(f[2]);
          for (long k = offset * s; k < n; k += 2 * s) {
            long const lo = k == 0 ? n - s : k - s;
            long const up = k + s == n ? 0 : k + s;
            for (long w = 0; w < width; ++w) {
              Value const vl = scratch[lo * width + w];
              Value const vm = scratch[k * width + w];
              Value const vu = scratch[up * width + w];
              scratch[k * width + w] = c0 * vl + c1 * vm + c2 * vu;
            }
          }
        }
      }
      for (long k = 0; k < n; ++k)
        for (long w = 0; w < width; ++w)
          base[k * inner + w] = scratch[k * width + w];
    }
  }
}

template <typename Value>
void transform_in(Value *g, Shape const &shape, int dim,
                  std::vector<long> const &levels, Filters const &filters,
                  Mode mode) {
  if (mode == Mode::Direct)
    transform_in_direct(g, shape, dim, levels, filters);
  else
    transform_in_packed(g, shape, dim, levels, filters);
}

// hierarchize_in / dehierarchize_in (paliwa/paliwa_transform.hpp:346-399):
// forward levels level..lmin+1 (decreasing, :364-367), inverse lmin+1..level
// (increasing, :392-394). hierarchize / dehierarchize (:401-431) fold over the
// dimensions in declaration order, dimension 0 first.
template <typename Value>
void hierarchize(Value *g, Shape const &shape, long const *minimum_level,
                 int wavelet, bool forward, Mode mode) {
  Filters const filters =
      forward ? forward_filters(wavelet) : inverse_filters(wavelet);
  for (int d = 0; d < shape.ndim; ++d) {
    long const lev = shape.level[d], lmin = minimum_level[d];
    if (lmin < 0 || lmin > lev || lev > shape.maximum_level[d])
      throw std::invalid_argument("requires 0 <= lmin <= level <= lmax");
    std::vector<long> levels;
    for (long l = lmin + 1; l <= lev; ++l) levels.push_back(l);
    if (forward) std::reverse(levels.begin(), levels.end());
    transform_in(g, shape, d, levels, filters, mode);
  }
}

} // namespace paliwa_oracle
