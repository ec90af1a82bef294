// Drop-in for paliwa/paliwa_dimensions.hpp: the dimension tags and the
// periodic unit-interval coordinates of the grids.
//
// Same names as the reference: the tag structs A..Z (:10-35),
// NumberedType (:37-39), D_Dim (:41-42), DDimA..DDimZ (:44-69),
// initialize_dim_periodic_unit_interval (:71-79),
// optional_initialize_dims_periodic_unit_intervals (:81-97) and
// optional_initialize_dims_periodic_unit_cube (:99-104). A dimension of
// resolution n is the uniform sampling of n + 1 points on [0, 1] with the
// point at 1 removed: uid k sits at x = k / n (the periodic grid; a grid at
// level l inside maximum level L has its points at uids k 2^(L - l)).
#pragma once

#include <cassert>
#include <cstddef>
#include <type_traits>

#if defined(PALIWA_GB300_USE_DDC)
#include <ddc/ddc.hpp>
#else
#include "ddc_compat.hpp"
#endif

namespace paliwa {

// The reference's tag structs: the continuous dimensions of DDimA..DDimZ.
struct A {};
struct B {};
struct C {};
struct D {};
struct E {};
struct F {};
struct G {};
struct H {};
struct I {};
struct J {};
struct K {};
struct L {};
struct M {};
struct N {};
struct O {};
struct P {};
struct Q {};
struct R {};
struct S {};
struct T {};
struct U {};
struct V {};
struct W {};
struct X {};
struct Y {};
struct Z {};

// Distinct types for distinct numbers over the same base.
template <typename Base, size_t type_number> struct NumberedType : Base {
  static constexpr size_t ID = type_number;
};

// A discrete dimension: uniform points along continuous dimension Tag.
template <class Tag, size_t type_number = 0>
struct D_Dim : NumberedType<ddc::UniformPointSampling<Tag>, type_number> {};

using DDimA = D_Dim<A>;
using DDimB = D_Dim<B>;
using DDimC = D_Dim<C>;
using DDimD = D_Dim<D>;
using DDimE = D_Dim<E>;
using DDimF = D_Dim<F>;
using DDimG = D_Dim<G>;
using DDimH = D_Dim<H>;
using DDimI = D_Dim<I>;
using DDimJ = D_Dim<J>;
using DDimK = D_Dim<K>;
using DDimL = D_Dim<L>;
using DDimM = D_Dim<M>;
using DDimN = D_Dim<N>;
using DDimO = D_Dim<O>;
using DDimP = D_Dim<P>;
using DDimQ = D_Dim<Q>;
using DDimR = D_Dim<R>;
using DDimS = D_Dim<S>;
using DDimT = D_Dim<T>;
using DDimU = D_Dim<U>;
using DDimV = D_Dim<V>;
using DDimW = D_Dim<W>;
using DDimX = D_Dim<X>;
using DDimY = D_Dim<Y>;
using DDimZ = D_Dim<Z>;

// Registers DDim's discrete space: resolution points at x = k / resolution
// on [0, 1), and returns their domain.
template <typename DDim>
ddc::DiscreteDomain<DDim> initialize_dim_periodic_unit_interval(
    ddc::DiscreteVector<DDim> const &resolution) {
  using CDim = typename DDim::continuous_dimension_type;
  // resolution + 1 points from 0 to 1, the last one (x = 1 = x = 0) dropped.
  auto const closed = ddc::init_discrete_space<DDim>(
      DDim::template init<DDim>(ddc::Coordinate<CDim>(0.0),
                                ddc::Coordinate<CDim>(1.0), resolution + 1));
  return closed.remove_last(ddc::DiscreteVector<DDim>(1));
}

// The same, unless DDim's space already exists (then it must be the same
// unit interval; an empty domain is returned).
template <typename DDimToInitialize, typename... DDims,
          typename = std::enable_if_t<(sizeof...(DDims) > 1)>>
ddc::DiscreteDomain<DDimToInitialize>
optional_initialize_dims_periodic_unit_intervals(
    ddc::DiscreteVector<DDims...> const &resolution) {
  if (!ddc::is_discrete_space_initialized<DDimToInitialize>())
    return initialize_dim_periodic_unit_interval<DDimToInitialize>(
        ddc::select<DDimToInitialize>(resolution));
  [[maybe_unused]] auto const &space =
      ddc::host_discrete_space<DDimToInitialize>();
  assert(space.origin() == 0.0);
  assert(space.step() == 1.0 / (ddc::select<DDimToInitialize>(resolution)));
  return ddc::DiscreteDomain<DDimToInitialize>();
}

template <typename... DDims>
ddc::DiscreteDomain<DDims...> optional_initialize_dims_periodic_unit_cube(
    ddc::DiscreteVector<DDims...> &resolution) {
  return ddc::DiscreteDomain<DDims...>(
      optional_initialize_dims_periodic_unit_intervals<DDims>(resolution)...);
}

} // namespace paliwa
