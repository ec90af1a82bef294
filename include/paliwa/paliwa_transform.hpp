// Drop-in replacement of paliwa's transform API (paliwa/paliwa_transform.hpp)
// that runs the GB300 kernels of libpaliwa_gb300 through the C ABI in
// paliwa_gb300.h.
//
// Same names, template shapes and error behaviour as the reference:
//   hierarchize / dehierarchize           (paliwa_transform.hpp:401-431)
//   hierarchize_in<Dim> / dehierarchize_in<Dim>           (:346-399)
//   transform_in<Dim> (full-grid overload)               (:215-251)
//   transform_in<Dim> (restricted outputs)               (:258-344)
//   for_each_transform_index<Dim>            (paliwa_domains.hpp:454-469)
//   restrict_periodic_bounds<Dim>            (paliwa_domains.hpp:540-567)
//   transform_bounds, covering_periodic_bounds, pole_pass_segments
//                                  (paliwa_plan.hpp, paliwa_domains.hpp)
//   strided_domain_from_level                (paliwa_domains.hpp:33-49)
// Grids are ChunkSpans whose data_handle() is device memory holding the dense
// row-major storage of strided_domain_from_level(level, maximum_level).
// The last argument stands in for the Kokkos execution-space instance: any
// object with a cuda_stream() member (Kokkos::Cuda has one), a
// paliwa::gb300::Stream, or nothing (the legacy default stream). Calls are
// asynchronous on that stream; callers synchronize, as with the reference.
//
// Errors: std::invalid_argument for level/shape violations (the reference
// asserts or throws it), std::runtime_error for unsupported filter offsets
// (:239-240), std::out_of_range for unknown wavelet names (map::at, :370).
#pragma once

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
#include "paliwa_plan.hpp"
#include "paliwa_wavelets.hpp"

namespace paliwa {

// Accepted for source compatibility; the device path tiles pencils itself.
enum class PoleExecution { Direct, PackedPasses, PackedPoles };

namespace gb300 {

struct Stream {
  void *handle = nullptr;  // a cudaStream_t
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

// paliwa_domains.hpp:33-49: 2^l points per dimension, stride 2^(L - l).
template <class... DDims>
constexpr ddc::StridedDiscreteDomain<DDims...> strided_domain_from_level(
    std::array<long int, sizeof...(DDims)> const &level,
    std::array<long int, sizeof...(DDims)> const &finest_level,
    ddc::DiscreteElement<DDims...> lbound = ddc::DiscreteElement<DDims...>()) {
  std::array<long, sizeof...(DDims)> ext{}, str{};
  for (size_t i = 0; i < sizeof...(DDims); ++i) {
    ext[i] = 1L << level[i];
    str[i] = 1L << (finest_level[i] - level[i]);
  }
  return ddc::StridedDiscreteDomain<DDims...>(
      lbound, ddc::DiscreteVector<DDims...>(ext),
      ddc::DiscreteVector<DDims...>(str));
}

namespace gb300 {
// The device path transforms complete grids: the span's domain must be
// strided_domain_from_level(level, maximum_level) (the reference's
// "complete" case, paliwa_transform.hpp:224-228).
template <class ChunkSpanType, class... DDims>
void check_complete(ChunkSpanType const &grid,
                    ddc::DiscreteVector<DDims...> const &level,
                    ddc::DiscreteVector<DDims...> const &maximum_level) {
  auto const l = levels_of(level);
  auto const L = levels_of(maximum_level);
  for (size_t i = 0; i < l.size(); ++i)
    if (l[i] < 0 || L[i] < l[i] || L[i] > 62)
      throw std::invalid_argument("requires 0 <= level <= maximum_level");
  std::array<long, sizeof...(DDims)> la{}, La{};
  for (size_t i = 0; i < l.size(); ++i) {
    la[i] = static_cast<long>(l[i]);
    La[i] = static_cast<long>(L[i]);
  }
  if (!(grid.domain() == strided_domain_from_level<DDims...>(la, La)))
    throw std::invalid_argument(
        "the GPU transform needs the complete grid of the level");
}
} // namespace gb300

template <class Dim, class ChunkSpanType, class LevelRange,
          class ExecSpace = gb300::Stream, class... Dims>
constexpr bool
transform_in(ChunkSpanType grid, ddc::DiscreteVector<Dims...> const &level,
             ddc::DiscreteVector<Dims...> const &maximum_level,
             LevelRange const &levels, LiftingPasses const &filters,
             ExecSpace instance = ExecSpace()) {
  gb300::check_complete(grid, level, maximum_level);
  using T = typename ChunkSpanType::element_type;
  auto const lv = gb300::levels_of(level);
  auto const lm = gb300::levels_of(maximum_level);
  std::vector<int64_t> ls;
  for (auto l : levels) ls.push_back(static_cast<int64_t>(l));
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

template <class DDimInWhichToHierarchize, class ChunkSpanType,
          class ExecSpace = gb300::Stream, class... DDims>
constexpr bool
hierarchize_in(ChunkSpanType const strided_grid,
               ddc::DiscreteVector<DDims...> const &level,
               ddc::DiscreteVector<DDims...> const &minimum_level,
               ddc::DiscreteVector<DDims...> const &maximum_level,
               std::string const &wavelet_name = "hat",
               ExecSpace instance = ExecSpace()) {
  gb300::check_complete(strided_grid, level, maximum_level);
  using T = typename ChunkSpanType::element_type;
  auto const lv = gb300::levels_of(level);
  auto const ln = gb300::levels_of(minimum_level);
  auto const lm = gb300::levels_of(maximum_level);
  gb300::check(paliwa_gb_hierarchize_in(
      static_cast<void *>(strided_grid.data_handle()), gb300::dtype_of<T>(),
      static_cast<int>(lv.size()), lv.data(), ln.data(), lm.data(),
      gb300::dim_index<DDimInWhichToHierarchize, DDims...>(),
      gb300::wavelet_id(wavelet_name), gb300::stream_of(instance)));
  return true;
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
  gb300::check_complete(strided_grid, level, maximum_level);
  using T = typename ChunkSpanType::element_type;
  auto const lv = gb300::levels_of(level);
  auto const ln = gb300::levels_of(minimum_level);
  auto const lm = gb300::levels_of(maximum_level);
  gb300::check(paliwa_gb_dehierarchize_in(
      static_cast<void *>(strided_grid.data_handle()), gb300::dtype_of<T>(),
      static_cast<int>(lv.size()), lv.data(), ln.data(), lm.data(),
      gb300::dim_index<DDimInWhichToHierarchize, DDims...>(),
      gb300::wavelet_id(wavelet_name), gb300::stream_of(instance)));
  return true;
}

template <class ChunkSpanType, class ExecSpace = gb300::Stream,
          class... DDims>
constexpr void hierarchize(ChunkSpanType const strided_grid,
                           ddc::DiscreteVector<DDims...> const &level,
                           ddc::DiscreteVector<DDims...> const &minimum_level,
                           ddc::DiscreteVector<DDims...> const &maximum_level,
                           std::string const &wavelet_name = "hat",
                           ExecSpace instance = ExecSpace()) {
  gb300::check_complete(strided_grid, level, maximum_level);
  using T = typename ChunkSpanType::element_type;
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
  gb300::check_complete(strided_grid, level, maximum_level);
  using T = typename ChunkSpanType::element_type;
  auto const lv = gb300::levels_of(level);
  auto const ln = gb300::levels_of(minimum_level);
  auto const lm = gb300::levels_of(maximum_level);
  gb300::check(paliwa_gb_dehierarchize(
      static_cast<void *>(strided_grid.data_handle()), gb300::dtype_of<T>(),
      static_cast<int>(lv.size()), lv.data(), ln.data(), lm.data(),
      gb300::wavelet_id(wavelet_name), gb300::stream_of(instance)));
}

// paliwa_domains.hpp:454-469: visit every uid of per-level bounds (level 0:
// multiples of the period; level h: odd points of level h).
template <typename Dim, typename Visit>
void for_each_transform_index(std::vector<PeriodicBounds> const &bounds,
                              long maximum_level, Visit visit) {
  long const period = 1L << maximum_level;
  for (size_t h = 0; h < bounds.size(); ++h) {
    auto const b = bounds[h];
    if (b.empty()) continue;
    long const stride = h == 0 ? period : 2L << (maximum_level - h);
    long const last = b.max + (b.min > b.max ? period : 0);
    for (long x = b.min; x <= last; x += stride)
      visit(ddc::DiscreteElement<Dim>(x % period));
  }
}

// paliwa_domains.hpp:540-567: the points of `domain` whose uid along Dim
// lies in the periodic bounds, as at most two strided domains (a wrapped
// interval splits at the period); the lattice of `domain` is kept.
template <typename Dim, typename... Dims>
std::vector<ddc::StridedDiscreteDomain<Dims...>>
restrict_periodic_bounds(ddc::StridedDiscreteDomain<Dims...> const &domain,
                         PeriodicBounds bounds, long period) {
  std::vector<ddc::StridedDiscreteDomain<Dims...>> parts;
  if (bounds.empty() || domain.size() == 0) return parts;
  long const first = static_cast<long>(domain.front().template uid<Dim>());
  long const stride = static_cast<long>(domain.strides().template get<Dim>());
  long const last =
      first + (static_cast<long>(domain.extents().template get<Dim>()) - 1) *
                  stride;
  auto add = [&](long lo, long hi) {
    lo = std::max(lo, first);
    hi = std::min(hi, last);
    long const begin = first + ((lo - first + stride - 1) / stride) * stride;
    if (begin > hi) return;
    auto f = domain.front();
    f.template uid<Dim>() = begin;
    auto e = domain.extents();
    e.template get<Dim>() = (hi - begin) / stride + 1;
    parts.emplace_back(f, e, domain.strides());
  };
  if (bounds.min <= bounds.max) {
    add(bounds.min, bounds.max);
  } else {
    add(bounds.min, period - 1);
    add(0, bounds.max);
  }
  return parts;
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
