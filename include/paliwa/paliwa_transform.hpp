// Drop-in replacement of paliwa's transform API (paliwa/paliwa_transform.hpp)
// that runs the GB300 kernels of libpaliwa_gb300 through the C ABI in
// paliwa_gb300.h.
//
// Same names, template shapes and error behaviour as the reference:
//   hierarchize / dehierarchize           (paliwa_transform.hpp:401-431)
//   hierarchize_in<Dim> / dehierarchize_in<Dim>           (:346-399)
//   transform_in<Dim> (full-grid overload)               (:215-251)
//   transform_in<Dim> (restricted outputs)               (:258-344)
//   PoleExecution                                        (:21)
// and, through paliwa_domains.hpp, the index maps and planner of
// paliwa/paliwa_domains.hpp. Grids are ChunkSpans whose data_handle() is
// device memory holding the dense row-major storage of their domain: the
// complete lattice strided_domain_from_level(level, maximum_level) runs the
// tiled GPU transform; a chunk holding a box of that lattice runs the
// reference's bounds-checked passes (:24-51, :224-247) on the GPU.
// The last argument stands in for the Kokkos execution-space instance: any
// object with a cuda_stream() member (Kokkos::Cuda has one), a
// paliwa::gb300::Stream, or nothing (the legacy default stream). Calls are
// asynchronous on that stream; callers synchronize, as with the reference.
//
// Errors: std::invalid_argument for level/shape violations (the reference
// asserts or throws it), std::runtime_error for unsupported filter offsets
// (:239-240), std::out_of_range for unknown wavelet names (map::at, :370).
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#if defined(PALIWA_GB300_USE_DDC)
#include <ddc/ddc.hpp>
#else
#include "ddc_compat.hpp"
#endif

#include "../paliwa_gb300.h"
#include "paliwa_domains.hpp"
#include "paliwa_wavelets.hpp"

namespace paliwa {

// Accepted for source compatibility; the device path tiles pencils itself.
enum class PoleExecution { Direct, PackedPasses, PackedPoles };

namespace gb300 {

struct Stream {
  void *handle = nullptr;  // a cudaStream_t
  // Waits for this stream's queued work, like an instance's fence().
  void fence() const;
};

template <class T, class = void> struct has_cuda_stream : std::false_type {};
template <class T>
struct has_cuda_stream<T, std::void_t<decltype(std::declval<T>().cuda_stream())>>
    : std::true_type {};

template <class ExecSpace> void *stream_of(ExecSpace const &instance) {
  if constexpr (std::is_same_v<ExecSpace, Stream>)
    return instance.handle;
  else if constexpr (has_cuda_stream<ExecSpace>::value)
    return static_cast<void *>(instance.cuda_stream());
  else
    return nullptr;
}

inline void check(int rc) {
  if (rc == PALIWA_GB_OK) return;
  std::string const msg = paliwa_gb_last_error();
  switch (rc) {
  case PALIWA_GB_INVALID_ARGUMENT: throw std::invalid_argument(msg);
  case PALIWA_GB_OUT_OF_RANGE: throw std::out_of_range(msg);
  default: throw std::runtime_error(msg);
  }
}

inline void Stream::fence() const { check(paliwa_gb_synchronize(handle)); }

template <class T> constexpr int dtype_of() {
  if constexpr (std::is_same_v<std::remove_cv_t<T>, double>)
    return PALIWA_GB_F64;
  else if constexpr (std::is_same_v<std::remove_cv_t<T>, float>)
    return PALIWA_GB_F32;
  else
    static_assert(sizeof(T) == 0, "grids hold double or float");
}

inline int wavelet_id(std::string const &name) {
  int id = -1;
  check(paliwa_gb_wavelet_id(name.c_str(), &id));
  return id;
}

template <class... DDims>
std::array<int64_t, sizeof...(DDims)>
levels_of(ddc::DiscreteVector<DDims...> const &v) {
  return {static_cast<int64_t>(v.template get<DDims>())...};
}

template <class Dim, class... DDims> constexpr int dim_index() {
  constexpr bool same[] = {std::is_same_v<Dim, DDims>...};
  for (int i = 0; i < static_cast<int>(sizeof...(DDims)); ++i)
    if (same[i]) return i;
  return -1;
}

} // namespace gb300

namespace gb300 {

template <class... DDims>
void check_levels(ddc::DiscreteVector<DDims...> const &level,
                  ddc::DiscreteVector<DDims...> const &maximum_level) {
  auto const l = levels_of(level);
  auto const L = levels_of(maximum_level);
  for (size_t i = 0; i < l.size(); ++i)
    if (l[i] < 0 || L[i] < l[i] || L[i] > 62)
      throw std::invalid_argument("requires 0 <= level <= maximum_level");
}

// Whether the span holds the complete lattice of the level
// (paliwa_transform.hpp:224-228); those grids take the GPU's tiled
// transforms, every other chunk the bounds-checked passes.
template <class ChunkSpanType, class... DDims>
bool is_complete(ChunkSpanType const &grid,
                 ddc::DiscreteVector<DDims...> const &level,
                 ddc::DiscreteVector<DDims...> const &maximum_level) {
  check_levels(level, maximum_level);
  auto const l = levels_of(level);
  auto const L = levels_of(maximum_level);
  std::array<long, sizeof...(DDims)> la{}, La{};
  for (size_t i = 0; i < l.size(); ++i) {
    la[i] = static_cast<long>(l[i]);
    La[i] = static_cast<long>(L[i]);
  }
  return grid.domain() == strided_domain_from_level<DDims...>(la, La);
}

// The box of the level lattice that a partial chunk holds: front uids and
// extents per dimension. Its strides must be the level's spacing.
template <class ChunkSpanType, class... DDims>
void window_of(ChunkSpanType const &grid,
               ddc::DiscreteVector<DDims...> const &level,
               ddc::DiscreteVector<DDims...> const &maximum_level,
               std::array<int64_t, sizeof...(DDims)> &front,
               std::array<int64_t, sizeof...(DDims)> &extents) {
  auto const l = levels_of(level);
  auto const L = levels_of(maximum_level);
  auto const dom = grid.domain();
  size_t i = 0;
  ((front[i] = static_cast<int64_t>(dom.front().template uid<DDims>()),
    extents[i] = static_cast<int64_t>(dom.extents().template get<DDims>()),
    static_cast<int64_t>(dom.strides().template get<DDims>()) ==
            (int64_t{1} << (L[i] - l[i]))
        ? void(++i)
        : throw std::invalid_argument(
              "the chunk's strides must be the level's spacing")),
   ...);
}

// transform_in along dimension `dim` of a partial chunk (C ABI
// paliwa_gb_transform_in_window).
template <class ChunkSpanType, class... DDims>
void transform_window(ChunkSpanType const &grid,
                      ddc::DiscreteVector<DDims...> const &level,
                      ddc::DiscreteVector<DDims...> const &maximum_level,
                      int dim, std::vector<int64_t> const &levels,
                      LiftingPasses const &filters, void *stream) {
  using T = typename ChunkSpanType::element_type;
  constexpr size_t n = sizeof...(DDims);
  std::array<int64_t, n> front{}, extents{};
  window_of(grid, level, maximum_level, front, extents);
  auto const lv = levels_of(level);
  auto const lm = levels_of(maximum_level);
  std::vector<int32_t> offs;
  std::vector<double> co;
  for (auto const &[o, f] : filters) {
    offs.push_back(o);
    co.insert(co.end(), f.begin(), f.end());
  }
  check(paliwa_gb_transform_in_window(
      static_cast<void *>(grid.data_handle()), dtype_of<T>(),
      static_cast<int>(n), lv.data(), lm.data(), front.data(), extents.data(),
      dim, levels.data(), static_cast<int>(levels.size()), offs.data(),
      co.data(), static_cast<int>(offs.size()), stream));
}

// Levels level[dim] .. lmin+1 (forward) or lmin+1 .. level[dim] (inverse)
// of hierarchize_in / dehierarchize_in (paliwa_transform.hpp:346-399).
template <class... DDims>
std::vector<int64_t> level_range(ddc::DiscreteVector<DDims...> const &level,
                                 ddc::DiscreteVector<DDims...> const &minimum,
                                 ddc::DiscreteVector<DDims...> const &maximum,
                                 int dim, bool forward) {
  auto const l = levels_of(level)[dim];
  auto const m = levels_of(minimum)[dim];
  if (m < 0 || m > l || l > levels_of(maximum)[dim])
    throw std::invalid_argument(
        "requires 0 <= minimum_level <= level <= maximum_level");
  std::vector<int64_t> r;
  for (int64_t k = m + 1; k <= l; ++k) r.push_back(k);
  if (forward) std::reverse(r.begin(), r.end());
  return r;
}

} // namespace gb300

// transform_in<Dim> (full-grid overload, paliwa_transform.hpp:215-251):
// every level of `levels` in order, the filters of each in order. A chunk
// holding the complete lattice runs the GPU's tiled transform; any other
// chunk (a box of the lattice) the bounds-checked passes of the reference.
template <class Dim, class ChunkSpanType, class LevelRange,
          class ExecSpace = gb300::Stream, class... Dims>
constexpr bool
transform_in(ChunkSpanType grid, ddc::DiscreteVector<Dims...> const &level,
             ddc::DiscreteVector<Dims...> const &maximum_level,
             LevelRange const &levels, LiftingPasses const &filters,
             ExecSpace instance = ExecSpace()) {
  using T = typename ChunkSpanType::element_type;
  std::vector<int64_t> ls;
  for (auto l : levels) ls.push_back(static_cast<int64_t>(l));
  if (!gb300::is_complete(grid, level, maximum_level)) {
    gb300::transform_window(grid, level, maximum_level,
                            gb300::dim_index<Dim, Dims...>(), ls, filters,
                            gb300::stream_of(instance));
    return true;
  }
  auto const lv = gb300::levels_of(level);
  auto const lm = gb300::levels_of(maximum_level);
  std::vector<int32_t> offs;
  std::vector<double> co;
  for (auto const &[o, f] : filters) {
    offs.push_back(o);
    co.insert(co.end(), f.begin(), f.end());
  }
  gb300::check(paliwa_gb_transform_in(
      static_cast<void *>(grid.data_handle()), gb300::dtype_of<T>(),
      static_cast<int>(lv.size()), lv.data(), lm.data(),
      gb300::dim_index<Dim, Dims...>(), ls.data(),
      static_cast<int>(ls.size()), offs.data(), co.data(),
      static_cast<int>(offs.size()), gb300::stream_of(instance)));
  return true;
}

namespace gb300 {
template <class Dim, bool Forward, class ChunkSpanType, class ExecSpace,
          class... DDims>
bool transform_axis(ChunkSpanType const grid,
                    ddc::DiscreteVector<DDims...> const &level,
                    ddc::DiscreteVector<DDims...> const &minimum_level,
                    ddc::DiscreteVector<DDims...> const &maximum_level,
                    std::string const &wavelet_name, ExecSpace instance) {
  using T = typename ChunkSpanType::element_type;
  int const dim = dim_index<Dim, DDims...>();
  if (!is_complete(grid, level, maximum_level)) {
    auto const &filters =
        (Forward ? lifting_wavelet_filter_offsets_and_coefficients
                 : lifting_wavelet_reconstruct_offsets_and_coefficients)
            .at(wavelet_name);
    auto const ls = level_range(level, minimum_level, maximum_level, dim,
                                Forward);
    transform_window(grid, level, maximum_level, dim, ls, filters,
                     stream_of(instance));
    return true;
  }
  auto const lv = levels_of(level);
  auto const ln = levels_of(minimum_level);
  auto const lm = levels_of(maximum_level);
  check((Forward ? paliwa_gb_hierarchize_in : paliwa_gb_dehierarchize_in)(
      static_cast<void *>(grid.data_handle()), dtype_of<T>(),
      static_cast<int>(lv.size()), lv.data(), ln.data(), lm.data(), dim,
      wavelet_id(wavelet_name), stream_of(instance)));
  return true;
}
} // namespace gb300

// hierarchize_in<Dim> / dehierarchize_in<Dim> (paliwa_transform.hpp:346-399).
template <class DDimInWhichToHierarchize, class ChunkSpanType,
          class ExecSpace = gb300::Stream, class... DDims>
constexpr bool
hierarchize_in(ChunkSpanType const strided_grid,
               ddc::DiscreteVector<DDims...> const &level,
               ddc::DiscreteVector<DDims...> const &minimum_level,
               ddc::DiscreteVector<DDims...> const &maximum_level,
               std::string const &wavelet_name = "hat",
               ExecSpace instance = ExecSpace()) {
  return gb300::transform_axis<DDimInWhichToHierarchize, true>(
      strided_grid, level, minimum_level, maximum_level, wavelet_name,
      instance);
}

template <class DDimInWhichToHierarchize, class ChunkSpanType,
          class ExecSpace = gb300::Stream, class... DDims>
constexpr bool
dehierarchize_in(ChunkSpanType const strided_grid,
                 ddc::DiscreteVector<DDims...> const &level,
                 ddc::DiscreteVector<DDims...> const &minimum_level,
                 ddc::DiscreteVector<DDims...> const &maximum_level,
                 std::string const &wavelet_name = "hat",
                 ExecSpace instance = ExecSpace()) {
  return gb300::transform_axis<DDimInWhichToHierarchize, false>(
      strided_grid, level, minimum_level, maximum_level, wavelet_name,
      instance);
}

// hierarchize / dehierarchize (paliwa_transform.hpp:401-431): every
// dimension in declaration order.
template <class ChunkSpanType, class ExecSpace = gb300::Stream,
          class... DDims>
constexpr void hierarchize(ChunkSpanType const strided_grid,
                           ddc::DiscreteVector<DDims...> const &level,
                           ddc::DiscreteVector<DDims...> const &minimum_level,
                           ddc::DiscreteVector<DDims...> const &maximum_level,
                           std::string const &wavelet_name = "hat",
                           ExecSpace instance = ExecSpace()) {
  using T = typename ChunkSpanType::element_type;
  if (!gb300::is_complete(strided_grid, level, maximum_level)) {
    (hierarchize_in<DDims>(strided_grid, level, minimum_level, maximum_level,
                           wavelet_name, instance),
     ...);
    return;
  }
  auto const lv = gb300::levels_of(level);
  auto const ln = gb300::levels_of(minimum_level);
  auto const lm = gb300::levels_of(maximum_level);
  gb300::check(paliwa_gb_hierarchize(
      static_cast<void *>(strided_grid.data_handle()), gb300::dtype_of<T>(),
      static_cast<int>(lv.size()), lv.data(), ln.data(), lm.data(),
      gb300::wavelet_id(wavelet_name), gb300::stream_of(instance)));
}

template <class ChunkSpanType, class ExecSpace = gb300::Stream,
          class... DDims>
constexpr void dehierarchize(ChunkSpanType const strided_grid,
                             ddc::DiscreteVector<DDims...> const &level,
                             ddc::DiscreteVector<DDims...> const &minimum_level,
                             ddc::DiscreteVector<DDims...> const &maximum_level,
                             std::string const &wavelet_name = "hat",
                             ExecSpace instance = ExecSpace()) {
  using T = typename ChunkSpanType::element_type;
  if (!gb300::is_complete(strided_grid, level, maximum_level)) {
    (dehierarchize_in<DDims>(strided_grid, level, minimum_level,
                             maximum_level, wavelet_name, instance),
     ...);
    return;
  }
  auto const lv = gb300::levels_of(level);
  auto const ln = gb300::levels_of(minimum_level);
  auto const lm = gb300::levels_of(maximum_level);
  gb300::check(paliwa_gb_dehierarchize(
      static_cast<void *>(strided_grid.data_handle()), gb300::dtype_of<T>(),
      static_cast<int>(lv.size()), lv.data(), ln.data(), lm.data(),
      gb300::wavelet_id(wavelet_name), gb300::stream_of(instance)));
}

// Restricted-output transform (paliwa_transform.hpp:333-344): the lifting
// sequence along Dim, writing only what `outputs` depends on. The grid's
// domain is a window of the level's lattice (strides 2^(L - l)) that holds
// every required input; PoleExecution is accepted for source compatibility
// (the device path plans its own work).
template <class Dim, class ChunkSpanType, class LevelRange, class ExecSpace,
          class... Dims>
constexpr bool transform_in(
    ChunkSpanType grid, ddc::DiscreteVector<Dims...> const &level,
    ddc::DiscreteVector<Dims...> const &maximum_level,
    LevelRange const &levels, LiftingPasses const &filters,
    ddc::StridedDiscreteDomain<Dims...> const &outputs, ExecSpace instance,
    PoleExecution = PoleExecution::Direct) {
  using T = typename ChunkSpanType::element_type;
  auto const lv = gb300::levels_of(level);
  auto const lm = gb300::levels_of(maximum_level);
  constexpr size_t n = sizeof...(Dims);
  auto const dom = grid.domain();
  std::array<int64_t, n> wf{}, we{}, of{}, oe{}, os{};
  size_t i = 0;
  ((wf[i] = static_cast<int64_t>(dom.front().template uid<Dims>()),
    we[i] = static_cast<int64_t>(dom.extents().template get<Dims>()),
    of[i] = static_cast<int64_t>(outputs.front().template uid<Dims>()),
    oe[i] = static_cast<int64_t>(outputs.extents().template get<Dims>()),
    os[i] = static_cast<int64_t>(outputs.strides().template get<Dims>()),
    ++i),
   ...);
  i = 0;
  ((static_cast<int64_t>(dom.strides().template get<Dims>()) ==
            (int64_t{1} << (lm[i] - lv[i]))
        ? void(++i)
        : throw std::invalid_argument(
              "the grid's strides must be the level's spacing")),
   ...);
  std::vector<int64_t> ls;
  for (auto l : levels) ls.push_back(static_cast<int64_t>(l));
  std::vector<int32_t> offs;
  std::vector<double> co;
  for (auto const &[o, f] : filters) {
    offs.push_back(o);
    co.insert(co.end(), f.begin(), f.end());
  }
  gb300::check(paliwa_gb_transform_outputs(
      static_cast<void *>(grid.data_handle()), gb300::dtype_of<T>(),
      static_cast<int>(n), lv.data(), lm.data(), wf.data(), we.data(),
      gb300::dim_index<Dim, Dims...>(), ls.data(),
      static_cast<int>(ls.size()), offs.data(), co.data(),
      static_cast<int>(offs.size()), of.data(), oe.data(), os.data(),
      gb300::stream_of(instance)));
  return true;
}

} // namespace paliwa
