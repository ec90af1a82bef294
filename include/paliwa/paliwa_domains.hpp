// Drop-in for paliwa/paliwa_domains.hpp: the level index maps, domain set
// operations and the restricted-output planner, over DDC types (the real
// DDC when PALIWA_GB300_USE_DDC is defined, else ddc_compat.hpp).
//
// Same names, argument meaning and exception types as the reference:
//   replace_dim                                   (:20-31)
//   strided_domain_from_level                     (:33-49)
//   strided_hierarchical_domain_from_level        (:51-83)
//   odd_/even_strided_domain_from_domain          (:85-111)
//   get_strided_domains                           (:113-128)
//   get_even_and_odd_half_domain_functors         (:130-139)
//   get_intersected_begin / get_intersected_extent (:141-193)
//   restrict_strided_with_discrete                (:195-214)
//   restrict_sparse_with_other_domain, sparse_from_strided_domain,
//   union_of_sparse_domains                       (:216-313)
//   PeriodicBounds, transform_bounds, covering_periodic_bounds,
//   PolePassSegment, pole_pass_segments           (paliwa_plan.hpp)
//   for_each_transform_index                      (:437-450)
//   domain_from_transform_bounds                  (:453-468)
//   restrict_periodic_bounds                      (:539-568)
//   local_pole_domain                             (:571-588)
//   get_required_transform_domain(s)              (:590-673)
// Everything here is host arithmetic on uids; the GPU transforms take the
// resulting shapes through the C ABI.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <functional>
#include <iterator>
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

#include "paliwa_plan.hpp"
#include "paliwa_wavelets.hpp"

namespace paliwa {

namespace domains_detail {
using Uid = ddc::DiscreteElementType;
using Off = ddc::DiscreteVectorElement;

// A one-dimensional sparse domain from a list of uids (sorted, distinct).
template <class Dim>
ddc::SparseDiscreteDomain<Dim> sparse_1d(std::vector<Uid> uids) {
  std::sort(uids.begin(), uids.end());
  uids.erase(std::unique(uids.begin(), uids.end()), uids.end());
  std::vector<ddc::DiscreteElement<Dim>> elements;
  elements.reserve(uids.size());
  for (Uid u : uids) elements.emplace_back(u);
#if defined(PALIWA_GB300_USE_DDC)
  Kokkos::View<ddc::DiscreteElement<Dim> *, Kokkos::SharedSpace> view(
      "paliwa_sparse_elements", elements.size());
  for (std::size_t i = 0; i < elements.size(); ++i) view(i) = elements[i];
  return ddc::SparseDiscreteDomain<Dim>(view);
#else
  return ddc::SparseDiscreteDomain<Dim>(elements);
#endif
}

// Whether a DDC element type has dimension tag T.
template <class T, class Element> struct element_has_tag : std::false_type {};
template <class T, class... Ts>
struct element_has_tag<T, ddc::DiscreteElement<Ts...>>
    : std::bool_constant<(std::is_same_v<T, Ts> || ...)> {};

template <class Dim, class Domain> std::vector<Uid> uids_of(Domain const &d) {
  std::vector<Uid> out;
  ddc::host_for_each(ddc::select<Dim>(d), [&](ddc::DiscreteElement<Dim> e) {
    out.push_back(static_cast<Uid>(e.uid()));
  });
  return out;
}
} // namespace domains_detail

// The element `base` with its DimToReplace component taken from d_elem.
template <typename DimToReplace, typename... DDims>
constexpr ddc::DiscreteElement<DDims...>
replace_dim(ddc::DiscreteElement<DDims...> base,
            ddc::DiscreteElement<DimToReplace> d_elem) {
  base.template uid<DimToReplace>() = d_elem.uid();
  return base;
}

// The grid of a level: 2^l points per dimension at uid stride 2^(L - l).
template <typename... DDims>
constexpr ddc::StridedDiscreteDomain<DDims...> strided_domain_from_level(
    std::array<long int, sizeof...(DDims)> const &level,
    std::array<long int, sizeof...(DDims)> const &finest_level,
    ddc::DiscreteElement<DDims...> lbound = ddc::DiscreteElement<DDims...>()) {
  std::array<long, sizeof...(DDims)> points{}, spacing{};
  for (std::size_t d = 0; d < sizeof...(DDims); ++d) {
    points[d] = 1L << level[d];
    spacing[d] = 1L << (finest_level[d] - level[d]);
  }
  return ddc::StridedDiscreteDomain<DDims...>(
      lbound, ddc::DiscreteVector<DDims...>(points),
      ddc::DiscreteVector<DDims...>(spacing));
}

// The hierarchical subspace of level vector `level`: per dimension the odd
// points of that level, 2^(l-1) of them from uid 2^(L-l) at stride
// 2^(L-l+1); level 0 is the single coarse point (stride 2^(L+1)).
template <typename... DDims>
constexpr ddc::StridedDiscreteDomain<DDims...>
strided_hierarchical_domain_from_level(
    std::array<long int, sizeof...(DDims)> const &level,
    std::array<long int, sizeof...(DDims)> const &finest_level,
    ddc::DiscreteElement<DDims...> lbound = ddc::DiscreteElement<DDims...>()) {
  std::array<long, sizeof...(DDims)> count{}, first{}, stride{};
  for (std::size_t d = 0; d < sizeof...(DDims); ++d) {
    long const gap = finest_level[d] - level[d];
    count[d] = level[d] == 0 ? 1L : 1L << (level[d] - 1);
    first[d] = level[d] == 0 ? 0L : 1L << gap;
    stride[d] = 2L << gap;
  }
  return ddc::StridedDiscreteDomain<DDims...>(
      lbound + ddc::DiscreteVector<DDims...>(first),
      ddc::DiscreteVector<DDims...>(count),
      ddc::DiscreteVector<DDims...>(stride));
}

// Odd and even halves of a domain along one dimension: every second point
// from the domain's stride (odd) or from 0 (even), relative to lbound.
template <typename DDimInWhichItsOdd, typename... DDims>
constexpr ddc::StridedDiscreteDomain<DDims...> odd_strided_domain_from_domain(
    ddc::StridedDiscreteDomain<DDims...> const &domain,
    ddc::DiscreteElement<DDims...> lbound = ddc::DiscreteElement<DDims...>()) {
  auto strides = domain.strides();
  auto extents = domain.extents();
  auto const s = strides.template get<DDimInWhichItsOdd>();
  strides.template get<DDimInWhichItsOdd>() = 2 * s;
  extents.template get<DDimInWhichItsOdd>() /= 2;
  return ddc::StridedDiscreteDomain<DDims...>(
      lbound + ddc::DiscreteVector<DDimInWhichItsOdd>(s), extents, strides);
}

template <typename DDimInWhichItsEven, typename... DDims>
constexpr ddc::StridedDiscreteDomain<DDims...> even_strided_domain_from_domain(
    ddc::StridedDiscreteDomain<DDims...> const &domain,
    ddc::DiscreteElement<DDims...> lbound = ddc::DiscreteElement<DDims...>()) {
  auto strides = domain.strides();
  auto extents = domain.extents();
  strides.template get<DDimInWhichItsEven>() *= 2;
  extents.template get<DDimInWhichItsEven>() /= 2;
  return ddc::StridedDiscreteDomain<DDims...>(lbound, extents, strides);
}

// One grid domain per level vector of a combination scheme.
template <typename... DDims>
std::vector<ddc::StridedDiscreteDomain<DDims...>> get_strided_domains(
    std::vector<std::array<long int, sizeof...(DDims)>> const &all_levels,
    std::array<long int, sizeof...(DDims)> maximum_level,
    ddc::DiscreteElement<DDims...> lbound = ddc::DiscreteElement<DDims...>()) {
  std::vector<ddc::StridedDiscreteDomain<DDims...>> grids;
  grids.reserve(all_levels.size());
  for (auto const &l : all_levels)
    grids.push_back(strided_domain_from_level<DDims...>(l, maximum_level,
                                                        lbound));
  return grids;
}

// (even, odd) half-domain functions along DDimInWhichToTransform, each
// taking a domain (lbound = origin).
template <typename DDimInWhichToTransform, typename... DDims>
constexpr decltype(auto) get_even_and_odd_half_domain_functors() {
  using Domain = ddc::StridedDiscreteDomain<DDims...>;
  auto even = [](Domain const &d) {
    return even_strided_domain_from_domain<DDimInWhichToTransform, DDims...>(
        d, ddc::DiscreteElement<DDims...>());
  };
  auto odd = [](Domain const &d) {
    return odd_strided_domain_from_domain<DDimInWhichToTransform, DDims...>(
        d, ddc::DiscreteElement<DDims...>());
  };
  return std::make_pair(even, odd);
}

// The first point of a strided lattice at or after other_begin, per
// dimension that other_begin has (others keep strided_begin). The quotient
// is rounded up in single precision, as the reference computes it.
template <typename OtherElementType, typename HeadTag, typename... Tags>
constexpr ddc::DiscreteElement<HeadTag, Tags...> get_intersected_begin(
    ddc::DiscreteElement<HeadTag, Tags...> const &strided_begin,
    ddc::DiscreteVector<HeadTag, Tags...> const &strides,
    OtherElementType const &other_begin) {
  ddc::DiscreteElement<HeadTag, Tags...> begin = strided_begin;
  auto one = [&](auto tag) {
    using T = decltype(tag);
    if constexpr (domains_detail::element_has_tag<T, OtherElementType>::value) {
      auto const b = static_cast<domains_detail::Off>(strided_begin.template uid<T>());
      auto const o = static_cast<domains_detail::Off>(other_begin.template uid<T>());
      float const s = static_cast<float>(strides.template get<T>());
      float const steps = std::ceil(static_cast<float>(o - b) / s);
      begin.template uid<T>() = static_cast<domains_detail::Uid>(
          b + static_cast<domains_detail::Off>(steps * s));
    }
  };
  (one(HeadTag{}), ..., one(Tags{}));
  return begin;
}

// Points of the lattice from strided_begin up to other_back, per dimension
// that other_back has (others keep strided_extents).
template <class HeadTag, class... Tags, class... OtherTags>
constexpr ddc::DiscreteVector<HeadTag, Tags...> get_intersected_extent(
    ddc::DiscreteElement<HeadTag, Tags...> const &strided_begin,
    ddc::DiscreteVector<HeadTag, Tags...> const &strides,
    ddc::DiscreteVector<HeadTag, Tags...> const &strided_extents,
    ddc::DiscreteElement<OtherTags...> const &other_back) {
  ddc::DiscreteVector<HeadTag, Tags...> ext = strided_extents;
  auto one = [&](auto tag) {
    using T = decltype(tag);
    if constexpr ((std::is_same_v<T, OtherTags> || ...)) {
      auto const span =
          static_cast<domains_detail::Off>(other_back.template uid<T>()) -
          static_cast<domains_detail::Off>(strided_begin.template uid<T>());
      ext.template get<T>() = span / strides.template get<T>() + 1;
    }
  };
  (one(HeadTag{}), ..., one(Tags{}));
  return ext;
}

// The strided domain's points inside another domain's box.
template <typename DDom, typename... DDims>
constexpr auto restrict_strided_with_discrete(
    ddc::StridedDiscreteDomain<DDims...> const &thisdomain,
    DDom const &odomain) {
  auto const begin = get_intersected_begin(thisdomain.front(),
                                           thisdomain.strides(),
                                           odomain.front());
  return ddc::StridedDiscreteDomain<DDims...>(
      begin,
      get_intersected_extent(begin, thisdomain.strides(), thisdomain.extents(),
                             odomain.back()),
      thisdomain.strides());
}

// The points of a sparse domain (per dimension) that another domain holds.
template <typename... DDims, typename DomainType>
ddc::SparseDiscreteDomain<DDims...> restrict_sparse_with_other_domain(
    ddc::SparseDiscreteDomain<DDims...> const &sparse_domain,
    DomainType const &other_domain) {
  auto keep = [&](auto tag) {
    using T = decltype(tag);
    auto const axis = ddc::select<T>(other_domain);
    std::vector<domains_detail::Uid> kept;
    for (auto u : domains_detail::uids_of<T>(sparse_domain))
      if (axis.contains(ddc::DiscreteElement<T>(u))) kept.push_back(u);
    return domains_detail::sparse_1d<T>(kept);
  };
  return ddc::SparseDiscreteDomain<DDims...>(keep(DDims{})...);
}

// A strided domain as a sparse one (the same points).
template <typename... DDims>
constexpr auto sparse_from_strided_domain(
    ddc::StridedDiscreteDomain<DDims...> const &strided_domain) {
  return ddc::SparseDiscreteDomain<DDims...>(domains_detail::sparse_1d<DDims>(
      domains_detail::uids_of<DDims>(strided_domain))...);
}

// Per dimension, the sorted union of two sparse domains' uids.
template <typename... DDims>
ddc::SparseDiscreteDomain<DDims...> union_of_sparse_domains(
    ddc::SparseDiscreteDomain<DDims...> const &first_sparse_domain,
    ddc::SparseDiscreteDomain<DDims...> const &second_sparse_domain) {
  auto merge = [&](auto tag) {
    using T = decltype(tag);
    auto a = domains_detail::uids_of<T>(first_sparse_domain);
    auto const b = domains_detail::uids_of<T>(second_sparse_domain);
    a.insert(a.end(), b.begin(), b.end());
    return domains_detail::sparse_1d<T>(a);
  };
  return ddc::SparseDiscreteDomain<DDims...>(merge(DDims{})...);
}

// Every uid that per-level bounds name (level 0: multiples of the period,
// level h: odd points of level h), level by level, each from min upwards.
template <typename Dim, typename Visit>
void for_each_transform_index(std::vector<PeriodicBounds> const &bounds,
                              long maximum_level, Visit visit) {
  long const period = 1L << maximum_level;
  for (std::size_t h = 0; h < bounds.size(); ++h) {
    if (bounds[h].empty()) continue;
    long const step = plan::level_stride(static_cast<long>(h), maximum_level);
    long const span = plan::mod_floor(bounds[h].max - bounds[h].min, period);
    for (long k = 0; k <= span / step; ++k)
      visit(ddc::DiscreteElement<Dim>((bounds[h].min + k * step) % period));
  }
}

// The same uids as a sorted one-dimensional sparse domain.
template <typename Dim>
auto domain_from_transform_bounds(std::vector<PeriodicBounds> const &bounds,
                                  long maximum_level) {
  std::vector<domains_detail::Uid> uids;
  for_each_transform_index<Dim>(bounds, maximum_level,
                                [&](ddc::DiscreteElement<Dim> e) {
                                  uids.push_back(e.uid());
                                });
  return domains_detail::sparse_1d<Dim>(uids);
}

// The points of `domain` whose uid along Dim lies in the periodic bounds,
// as at most two strided domains (a wrapped interval becomes its part from
// min to the period's end, then its part from 0); the lattice is kept.
template <typename Dim, typename... Dims>
std::vector<ddc::StridedDiscreteDomain<Dims...>>
restrict_periodic_bounds(ddc::StridedDiscreteDomain<Dims...> const &domain,
                         PeriodicBounds bounds, long period) {
  std::vector<ddc::StridedDiscreteDomain<Dims...>> parts;
  if (bounds.empty() || domain.size() == 0) return parts;
  long const f = static_cast<long>(domain.front().template uid<Dim>());
  long const s = static_cast<long>(domain.strides().template get<Dim>());
  long const n = static_cast<long>(domain.extents().template get<Dim>());
  std::array<std::pair<long, long>, 2> pieces{};
  int npieces = 0;
  if (bounds.min <= bounds.max) {
    pieces[npieces++] = {bounds.min, bounds.max};
  } else {
    pieces[npieces++] = {bounds.min, period - 1};
    pieces[npieces++] = {0, bounds.max};
  }
  for (int i = 0; i < npieces; ++i) {
    // Domain points k with f + k s in [lo, hi], 0 <= k < n.
    long const k0 = std::max(0L, pieces[i].first <= f
                                     ? 0L
                                     : (pieces[i].first - f + s - 1) / s);
    if (pieces[i].second < f) continue;
    long const k1 = std::min(n - 1, (pieces[i].second - f) / s);
    if (k1 < k0) continue;
    auto front = domain.front();
    front.template uid<Dim>() = static_cast<domains_detail::Uid>(f + k0 * s);
    auto extents = domain.extents();
    extents.template get<Dim>() = k1 - k0 + 1;
    parts.emplace_back(front, extents, domain.strides());
  }
  return parts;
}

// `global` along Dim, `local` in every other dimension.
template <typename Dim, typename... Dims>
auto local_pole_domain(ddc::StridedDiscreteDomain<Dims...> const &global,
                       ddc::StridedDiscreteDomain<Dims...> const &local) {
  auto front = local.front();
  auto extents = local.extents();
  auto strides = local.strides();
  front.template uid<Dim>() = global.front().template uid<Dim>();
  extents.template get<Dim>() = global.extents().template get<Dim>();
  strides.template get<Dim>() = global.strides().template get<Dim>();
  return ddc::StridedDiscreteDomain<Dims...>(front, extents, strides);
}

// The inputs along SelectedDim that the local part's transform reads but
// does not hold (its ghosts), as a sorted sparse domain: the restricted
// transform of the local uid interval, levels lmin+1..level (coarse to fine
// for the inverse), planned with transform_bounds. Throws
// std::runtime_error when a required input lies outside the full domain,
// std::out_of_range for an unknown wavelet.
template <typename SelectedDim, typename SDDom, typename DDom>
constexpr ddc::SparseDiscreteDomain<SelectedDim> get_required_transform_domain(
    bool is_for_hierarchization, SDDom const &full_domain,
    DDom const &local_domain, ddc::DiscreteVector<SelectedDim> const &level,
    ddc::DiscreteVector<SelectedDim> const &minimum_level,
    ddc::DiscreteVector<SelectedDim> const &maximum_level,
    std::string const &wavelet_name = "hat") {
  long const l = static_cast<long>(level);
  long const L = static_cast<long>(maximum_level);
  std::vector<long> levels;
  for (long k = static_cast<long>(minimum_level) + 1; k <= l; ++k)
    levels.push_back(k);
  if (is_for_hierarchization) std::reverse(levels.begin(), levels.end());
  auto const &filters =
      (is_for_hierarchization
           ? lifting_wavelet_filter_offsets_and_coefficients
           : lifting_wavelet_reconstruct_offsets_and_coefficients)
          .at(wavelet_name);
  PeriodicBounds outputs;
  if (!local_domain.empty())
    outputs = {static_cast<long>(local_domain.front().template uid<SelectedDim>()),
               static_cast<long>(local_domain.back().template uid<SelectedDim>())};
  auto const bounds = transform_bounds(outputs, l, L, levels, filters,
                                       [](std::size_t, std::size_t,
                                          PeriodicBounds) {});
  std::vector<domains_detail::Uid> ghosts;
  for_each_transform_index<SelectedDim>(
      bounds, L, [&](ddc::DiscreteElement<SelectedDim> e) {
        if (!full_domain.contains(e))
          throw std::runtime_error("Required input outside full domain");
        if (!local_domain.contains(e)) ghosts.push_back(e.uid());
      });
  return domains_detail::sparse_1d<SelectedDim>(ghosts);
}

// The same for every dimension: the product of the per-dimension ghosts.
template <typename DDom, typename... DDims>
constexpr ddc::SparseDiscreteDomain<DDims...> get_required_transform_domains(
    bool is_for_hierarchization,
    ddc::StridedDiscreteDomain<DDims...> const &full_domain,
    DDom const &local_domain, ddc::DiscreteVector<DDims...> const &level,
    ddc::DiscreteVector<DDims...> const &minimum_level,
    ddc::DiscreteVector<DDims...> const &maximum_level,
    std::string const &wavelet_name = "hat") {
  return ddc::SparseDiscreteDomain<DDims...>(
      get_required_transform_domain<DDims>(
          is_for_hierarchization, ddc::select<DDims>(full_domain),
          ddc::select<DDims>(local_domain), ddc::select<DDims>(level),
          ddc::select<DDims>(minimum_level), ddc::select<DDims>(maximum_level),
          wavelet_name)...);
}

} // namespace paliwa
