// Minimal stand-in for the subset of DDC (discrete-domain containers) that
// paliwa's transform API uses, for builds without DDC.
//
// paliwa passes grids as ddc::ChunkSpan over a ddc::StridedDiscreteDomain and
// levels as ddc::DiscreteVector (paliwa/paliwa_transform.hpp:401-431,
// paliwa/paliwa_domains.hpp:33-49). These types carry exactly that: tagged
// integer vectors, a strided domain (front, extents, strides, row-major) and a
// non-owning span over device memory. When the real DDC is available
// (PALIWA_GB300_USE_DDC), include <ddc/ddc.hpp> instead; the transform
// headers only use data_handle(), domain(), front(), extents(), strides() and
// the per-tag accessors below.
#pragma once

#include <array>
#include <cstddef>
#include <type_traits>

namespace ddc {

// DDC's coordinate types: element uids are unsigned, differences signed.
using DiscreteElementType = std::size_t;
using DiscreteVectorElement = std::ptrdiff_t;

namespace detail {
template <class T, class... Ts> constexpr std::size_t index_of() {
  constexpr bool same[] = {std::is_same_v<T, Ts>...};
  for (std::size_t i = 0; i < sizeof...(Ts); ++i)
    if (same[i]) return i;
  return sizeof...(Ts);
}
} // namespace detail

template <class... Tags> struct DiscreteVector {
  std::array<long, sizeof...(Tags)> v{};
  constexpr DiscreteVector() = default;
  constexpr explicit DiscreteVector(std::array<long, sizeof...(Tags)> a)
      : v(a) {}
  template <class... I,
            class = std::enable_if_t<sizeof...(I) == sizeof...(Tags) &&
                                     sizeof...(Tags) != 1 &&
                                     (std::is_integral_v<I> && ...)>>
  constexpr DiscreteVector(I... i) : v{static_cast<long>(i)...} {}
  template <class I, class = std::enable_if_t<std::is_integral_v<I> &&
                                              sizeof...(Tags) == 1>>
  constexpr explicit DiscreteVector(I i) : v{static_cast<long>(i)} {}
  template <class T> constexpr long &get() {
    return v[detail::index_of<T, Tags...>()];
  }
  template <class T> constexpr long get() const {
    return v[detail::index_of<T, Tags...>()];
  }
  constexpr bool operator==(DiscreteVector const &o) const { return v == o.v; }
};

template <class... Tags> struct DiscreteElement {
  std::array<long, sizeof...(Tags)> uid_{};
  constexpr DiscreteElement() = default;
  constexpr explicit DiscreteElement(std::array<long, sizeof...(Tags)> a)
      : uid_(a) {}
  template <class I, class = std::enable_if_t<std::is_integral_v<I> &&
                                              sizeof...(Tags) == 1>>
  constexpr explicit DiscreteElement(I i) : uid_{static_cast<long>(i)} {}
  template <class T> constexpr long uid() const {
    return uid_[detail::index_of<T, Tags...>()];
  }
  template <class T> constexpr long &uid() {
    return uid_[detail::index_of<T, Tags...>()];
  }
  constexpr bool operator==(DiscreteElement const &o) const {
    return uid_ == o.uid_;
  }
};

template <class... Tags> struct StridedDiscreteDomain {
  using discrete_element_type = DiscreteElement<Tags...>;
  using discrete_vector_type = DiscreteVector<Tags...>;
  DiscreteElement<Tags...> front_{};
  DiscreteVector<Tags...> extents_{}, strides_{};
  constexpr StridedDiscreteDomain() = default;
  constexpr StridedDiscreteDomain(DiscreteElement<Tags...> f,
                                  DiscreteVector<Tags...> e,
                                  DiscreteVector<Tags...> s)
      : front_(f), extents_(e), strides_(s) {}
  constexpr DiscreteElement<Tags...> front() const { return front_; }
  constexpr DiscreteVector<Tags...> extents() const { return extents_; }
  constexpr DiscreteVector<Tags...> strides() const { return strides_; }
  constexpr std::size_t size() const {
    std::size_t s = 1;
    for (long e : extents_.v) s *= static_cast<std::size_t>(e);
    return s;
  }
  constexpr bool operator==(StridedDiscreteDomain const &o) const {
    return front_ == o.front_ && extents_ == o.extents_ &&
           strides_ == o.strides_;
  }
};

// Non-owning view of the dense row-major storage of a domain.
template <class T, class Domain> class ChunkSpan {
 public:
  using element_type = T;
  constexpr ChunkSpan() = default;
  constexpr ChunkSpan(T *data, Domain const &d) : data_(data), domain_(d) {}
  constexpr T *data_handle() const { return data_; }
  constexpr Domain const &domain() const { return domain_; }
  constexpr ChunkSpan span_view() const { return *this; }

 private:
  T *data_ = nullptr;
  Domain domain_{};
};

template <class T, class... Tags> constexpr long get(DiscreteVector<Tags...> const &v) {
  return v.template get<T>();
}

} // namespace ddc
