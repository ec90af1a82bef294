// Subset of DDC (discrete-domain containers) that paliwa's API uses, for
// builds without DDC: discrete elements, vectors and domains (strided, dense
// and sparse), selection by tag, host iteration, a non-owning chunk span and
// uniform point sampling. When the real DDC is available
// (PALIWA_GB300_USE_DDC), the drop-in headers include <ddc/ddc.hpp> instead.
// Written from DDC's documented semantics, which paliwa relies on:
//  * an element holds one unsigned uid per dimension tag, a vector one
//    signed offset per tag; tags are types, and values are matched by tag,
//    not by position, when elements or vectors are combined;
//  * a StridedDiscreteDomain is {front + k * stride : 0 <= k < extent} per
//    dimension; a chunk over it is dense and row-major (last tag fastest),
//    element e at index (uid - front) / stride per dimension (the layout
//    paliwa/paliwa_io.hpp:13-23 and paliwa/postprocess.py:30-35 read);
//  * iteration visits every element of a domain once (row-major here);
//  * a SparseDiscreteDomain is the product of sorted per-dimension uid sets.
// A ChunkSpan's operator() dereferences its pointer on the host: the device
// transforms take data_handle() and never call it.
#pragma once

#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <functional>
#include <numeric>
#include <optional>
#include <stdexcept>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

namespace ddc {

using DiscreteElementType = std::size_t;
using DiscreteVectorElement = std::ptrdiff_t;

namespace detail {
template <class... T> struct TypeSeq {};

// Position of T in Ts..., or -1.
template <class T, class... Ts> constexpr int tag_index() {
  int i = 0, found = -1;
  ((std::is_same_v<T, Ts> ? (found = found < 0 ? i : found, ++i) : ++i), ...);
  return found;
}

template <class T, class Seq> struct in_seq;
template <class T, class... Ts> struct in_seq<T, TypeSeq<Ts...>> {
  static constexpr bool value = (std::is_same_v<T, Ts> || ...);
};

// TypeSeq<Ts...> without Rm.
template <class Rm, class Acc, class... Ts> struct remove_one;
template <class Rm, class... Acc> struct remove_one<Rm, TypeSeq<Acc...>> {
  using type = TypeSeq<Acc...>;
};
template <class Rm, class... Acc, class T, class... Ts>
struct remove_one<Rm, TypeSeq<Acc...>, T, Ts...> {
  using type = typename std::conditional_t<
      std::is_same_v<Rm, T>, remove_one<Rm, TypeSeq<Acc...>, Ts...>,
      remove_one<Rm, TypeSeq<Acc..., T>, Ts...>>::type;
};
} // namespace detail

template <class T, class Seq>
inline constexpr bool in_tags_v = detail::in_seq<T, Seq>::value;

template <class... Tags> class DiscreteVector;
template <class... Tags> class DiscreteElement;

template <class T> struct is_discrete_vector : std::false_type {};
template <class... T>
struct is_discrete_vector<DiscreteVector<T...>> : std::true_type {};
template <class T> struct is_discrete_element : std::false_type {};
template <class... T>
struct is_discrete_element<DiscreteElement<T...>> : std::true_type {};

namespace detail {
// The value of tag T from the first of `parts` (elements or vectors) that
// has it.
template <class T, class V, class First, class... Rest>
constexpr V take_tag(First const &first, Rest const &...rest) {
  if constexpr (First::template has_tag<T>())
    return first.template value_of<T>();
  else {
    static_assert(sizeof...(Rest) > 0, "tag missing from every part");
    return take_tag<T, V>(rest...);
  }
}
} // namespace detail

// ---------------------------------------------------------------- vectors

template <class... Tags> class DiscreteVector {
  std::array<DiscreteVectorElement, sizeof...(Tags)> m_values{};

  template <class... T> friend class DiscreteVector;
  template <class... T>
  friend constexpr std::array<DiscreteVectorElement, sizeof...(T)> &
  detail_array(DiscreteVector<T...> &);
  template <class... T>
  friend constexpr std::array<DiscreteVectorElement, sizeof...(T)> const &
  detail_array(DiscreteVector<T...> const &);

public:
  static constexpr std::size_t rank() { return sizeof...(Tags); }
  template <class T> static constexpr bool has_tag() {
    return (std::is_same_v<T, Tags> || ...);
  }

  constexpr DiscreteVector() = default;

  template <class... V,
            std::enable_if_t<sizeof...(V) == sizeof...(Tags) &&
                                 (sizeof...(V) >= 1) &&
                                 (std::is_arithmetic_v<V> && ...),
                             int> = 0>
  explicit constexpr DiscreteVector(V... v)
      : m_values{static_cast<DiscreteVectorElement>(v)...} {}

  template <class I, std::enable_if_t<std::is_integral_v<I>, int> = 0>
  explicit constexpr DiscreteVector(
      std::array<I, sizeof...(Tags)> const &values) {
    for (std::size_t i = 0; i < sizeof...(Tags); ++i)
      m_values[i] = static_cast<DiscreteVectorElement>(values[i]);
  }

  // From vectors over subsets of the tags, matched by tag.
  template <class... Parts,
            std::enable_if_t<(sizeof...(Parts) >= 1) &&
                                 (is_discrete_vector<Parts>::value && ...),
                             int> = 0>
  explicit constexpr DiscreteVector(Parts const &...parts)
      : m_values{detail::take_tag<Tags, DiscreteVectorElement>(parts...)...} {}

  template <class T> constexpr DiscreteVectorElement &get() {
    static_assert(has_tag<T>(), "tag not in this vector");
    return m_values[detail::tag_index<T, Tags...>()];
  }
  template <class T> constexpr DiscreteVectorElement const &get() const {
    static_assert(has_tag<T>(), "tag not in this vector");
    return m_values[detail::tag_index<T, Tags...>()];
  }
  template <class T> constexpr DiscreteVectorElement value_of() const {
    return get<T>();
  }
  template <class T>
  constexpr DiscreteVectorElement get_or(DiscreteVectorElement d) const {
    if constexpr (has_tag<T>())
      return get<T>();
    else
      return d;
  }

  constexpr DiscreteVectorElement value() const
    requires(sizeof...(Tags) == 1)
  {
    return m_values[0];
  }
  constexpr operator DiscreteVectorElement() const
    requires(sizeof...(Tags) == 1)
  {
    return m_values[0];
  }

  constexpr DiscreteVector &operator+=(DiscreteVector const &o) {
    for (std::size_t i = 0; i < sizeof...(Tags); ++i) m_values[i] += o.m_values[i];
    return *this;
  }
  constexpr DiscreteVector &operator-=(DiscreteVector const &o) {
    for (std::size_t i = 0; i < sizeof...(Tags); ++i) m_values[i] -= o.m_values[i];
    return *this;
  }
  constexpr DiscreteVector &operator*=(DiscreteVectorElement f) {
    for (auto &v : m_values) v *= f;
    return *this;
  }
  friend constexpr DiscreteVector operator+(DiscreteVector a,
                                            DiscreteVector const &b) {
    return a += b;
  }
  friend constexpr DiscreteVector operator-(DiscreteVector a,
                                            DiscreteVector const &b) {
    return a -= b;
  }
  friend constexpr DiscreteVector operator-(DiscreteVector a) {
    for (auto &v : a.m_values) v = -v;
    return a;
  }
  template <class I, std::enable_if_t<std::is_integral_v<I>, int> = 0>
  friend constexpr DiscreteVector operator*(I f, DiscreteVector a) {
    return a *= static_cast<DiscreteVectorElement>(f);
  }
  template <class I, std::enable_if_t<std::is_integral_v<I>, int> = 0>
  friend constexpr DiscreteVector operator*(DiscreteVector a, I f) {
    return a *= static_cast<DiscreteVectorElement>(f);
  }
  // One-dimensional vectors combine with plain integers.
  template <class I, std::size_t N = sizeof...(Tags),
            std::enable_if_t<std::is_integral_v<I> && N == 1, int> = 0>
  friend constexpr DiscreteVector operator+(DiscreteVector a, I b) {
    a.m_values[0] += static_cast<DiscreteVectorElement>(b);
    return a;
  }
  template <class I, std::size_t N = sizeof...(Tags),
            std::enable_if_t<std::is_integral_v<I> && N == 1, int> = 0>
  friend constexpr DiscreteVector operator-(DiscreteVector a, I b) {
    a.m_values[0] -= static_cast<DiscreteVectorElement>(b);
    return a;
  }
  friend constexpr bool operator==(DiscreteVector const &a,
                                   DiscreteVector const &b) {
    return a.m_values == b.m_values;
  }
  friend constexpr bool operator!=(DiscreteVector const &a,
                                   DiscreteVector const &b) {
    return !(a == b);
  }
};

// --------------------------------------------------------------- elements

template <class... Tags> class DiscreteElement {
  std::array<DiscreteElementType, sizeof...(Tags)> m_uids{};

  template <class... T> friend class DiscreteElement;
  template <class... T>
  friend constexpr std::array<DiscreteElementType, sizeof...(T)> &
  detail_array(DiscreteElement<T...> &);
  template <class... T>
  friend constexpr std::array<DiscreteElementType, sizeof...(T)> const &
  detail_array(DiscreteElement<T...> const &);

public:
  static constexpr std::size_t rank() { return sizeof...(Tags); }
  template <class T> static constexpr bool has_tag() {
    return (std::is_same_v<T, Tags> || ...);
  }

  constexpr DiscreteElement() = default;

  template <class... V,
            std::enable_if_t<sizeof...(V) == sizeof...(Tags) &&
                                 (sizeof...(V) >= 1) &&
                                 (std::is_arithmetic_v<V> && ...),
                             int> = 0>
  explicit constexpr DiscreteElement(V... v)
      : m_uids{static_cast<DiscreteElementType>(v)...} {}

  template <class I, std::enable_if_t<std::is_integral_v<I>, int> = 0>
  explicit constexpr DiscreteElement(std::array<I, sizeof...(Tags)> const &u) {
    for (std::size_t i = 0; i < sizeof...(Tags); ++i)
      m_uids[i] = static_cast<DiscreteElementType>(u[i]);
  }

  // From elements over subsets of the tags, matched by tag.
  template <class... Parts,
            std::enable_if_t<(sizeof...(Parts) >= 1) &&
                                 (is_discrete_element<Parts>::value && ...),
                             int> = 0>
  explicit constexpr DiscreteElement(Parts const &...parts)
      : m_uids{detail::take_tag<Tags, DiscreteElementType>(parts...)...} {}

  template <class T> constexpr DiscreteElementType &uid() {
    static_assert(has_tag<T>(), "tag not in this element");
    return m_uids[detail::tag_index<T, Tags...>()];
  }
  template <class T> constexpr DiscreteElementType const &uid() const {
    static_assert(has_tag<T>(), "tag not in this element");
    return m_uids[detail::tag_index<T, Tags...>()];
  }
  constexpr DiscreteElementType uid() const
    requires(sizeof...(Tags) == 1)
  {
    return m_uids[0];
  }
  template <class T> constexpr DiscreteElementType value_of() const {
    return uid<T>();
  }

  // Element +- vector over a subset of the tags: only those dimensions move.
  template <class... VT>
  constexpr DiscreteElement &operator+=(DiscreteVector<VT...> const &v) {
    ((uid<VT>() += static_cast<DiscreteElementType>(v.template get<VT>())),
     ...);
    return *this;
  }
  template <class... VT>
  constexpr DiscreteElement &operator-=(DiscreteVector<VT...> const &v) {
    ((uid<VT>() -= static_cast<DiscreteElementType>(v.template get<VT>())),
     ...);
    return *this;
  }
  template <class... VT>
  friend constexpr DiscreteElement operator+(DiscreteElement e,
                                             DiscreteVector<VT...> const &v) {
    return e += v;
  }
  template <class... VT>
  friend constexpr DiscreteElement operator-(DiscreteElement e,
                                             DiscreteVector<VT...> const &v) {
    return e -= v;
  }
  friend constexpr DiscreteVector<Tags...> operator-(DiscreteElement const &a,
                                                     DiscreteElement const &b) {
    return DiscreteVector<Tags...>(
        (static_cast<DiscreteVectorElement>(a.template uid<Tags>()) -
         static_cast<DiscreteVectorElement>(b.template uid<Tags>()))...);
  }
  friend constexpr bool operator==(DiscreteElement const &a,
                                   DiscreteElement const &b) {
    return a.m_uids == b.m_uids;
  }
  friend constexpr bool operator!=(DiscreteElement const &a,
                                   DiscreteElement const &b) {
    return !(a == b);
  }
  friend constexpr bool operator<(DiscreteElement const &a,
                                  DiscreteElement const &b) {
    return a.m_uids < b.m_uids;
  }
  friend constexpr bool operator>(DiscreteElement const &a,
                                  DiscreteElement const &b) {
    return b < a;
  }
  friend constexpr bool operator<=(DiscreteElement const &a,
                                   DiscreteElement const &b) {
    return !(b < a);
  }
  friend constexpr bool operator>=(DiscreteElement const &a,
                                   DiscreteElement const &b) {
    return !(a < b);
  }
};

template <class... T>
constexpr std::array<DiscreteVectorElement, sizeof...(T)> &
detail_array(DiscreteVector<T...> &v) {
  return v.m_values;
}
template <class... T>
constexpr std::array<DiscreteVectorElement, sizeof...(T)> const &
detail_array(DiscreteVector<T...> const &v) {
  return v.m_values;
}
template <class... T>
constexpr std::array<DiscreteElementType, sizeof...(T)> &
detail_array(DiscreteElement<T...> &e) {
  return e.m_uids;
}
template <class... T>
constexpr std::array<DiscreteElementType, sizeof...(T)> const &
detail_array(DiscreteElement<T...> const &e) {
  return e.m_uids;
}
namespace detail {
template <class X> constexpr auto &array(X &x) { return detail_array(x); }
} // namespace detail

template <class... Sel, class... T>
constexpr DiscreteVector<Sel...> select(DiscreteVector<T...> const &v) {
  return DiscreteVector<Sel...>(v.template get<Sel>()...);
}
template <class... Sel, class... T>
constexpr DiscreteElement<Sel...> select(DiscreteElement<T...> const &e) {
  return DiscreteElement<Sel...>(e.template uid<Sel>()...);
}
template <class Sel, class... T>
constexpr DiscreteElement<Sel> select_or(DiscreteElement<T...> const &e,
                                         DiscreteElement<Sel> const &d) {
  if constexpr ((std::is_same_v<Sel, T> || ...))
    return DiscreteElement<Sel>(e.template uid<Sel>());
  else
    return d;
}

// ---------------------------------------------------------------- domains

namespace detail {
// Row-major walk over per-dimension positions k_i in [0, extent_i).
template <std::size_t N, class F>
void row_major(std::array<DiscreteVectorElement, N> const &extents, F &&f) {
  for (std::size_t i = 0; i < N; ++i)
    if (extents[i] <= 0) return;
  std::array<DiscreteVectorElement, N> k{};
  for (;;) {
    f(k);
    std::size_t d = N;
    while (d > 0) {
      --d;
      if (++k[d] < extents[d]) break;
      k[d] = 0;
      if (d == 0) return;
    }
    if constexpr (N == 0) return;
  }
}
} // namespace detail

template <class... Tags> class StridedDiscreteDomain {
  DiscreteElement<Tags...> m_front;
  DiscreteVector<Tags...> m_extents;
  DiscreteVector<Tags...> m_strides;

public:
  using discrete_element_type = DiscreteElement<Tags...>;
  using discrete_vector_type = DiscreteVector<Tags...>;
  static constexpr std::size_t rank() { return sizeof...(Tags); }
  template <class T> static constexpr bool has_tag() {
    return (std::is_same_v<T, Tags> || ...);
  }

  constexpr StridedDiscreteDomain() = default;
  constexpr StridedDiscreteDomain(DiscreteElement<Tags...> const &front,
                                  DiscreteVector<Tags...> const &extents,
                                  DiscreteVector<Tags...> const &strides)
      : m_front(front), m_extents(extents), m_strides(strides) {}
  // From domains over subsets of the tags, matched by tag.
  template <class... Parts,
            std::enable_if_t<(sizeof...(Parts) >= 1) &&
                                 (Parts::is_strided_domain && ...),
                             int> = 0>
  explicit constexpr StridedDiscreteDomain(Parts const &...parts)
      : m_front(parts.front()...), m_extents(parts.extents()...),
        m_strides(parts.strides()...) {}
  static constexpr bool is_strided_domain = true;

  constexpr DiscreteElement<Tags...> front() const { return m_front; }
  constexpr DiscreteElement<Tags...> back() const {
    DiscreteElement<Tags...> b = m_front;
    ((b.template uid<Tags>() += static_cast<DiscreteElementType>(
          (m_extents.template get<Tags>() - 1) *
          m_strides.template get<Tags>())),
     ...);
    return b;
  }
  constexpr DiscreteVector<Tags...> extents() const { return m_extents; }
  constexpr DiscreteVector<Tags...> strides() const { return m_strides; }
  template <class T> constexpr DiscreteVector<T> extent() const {
    return DiscreteVector<T>(m_extents.template get<T>());
  }
  constexpr std::size_t size() const {
    std::size_t n = 1;
    ((n *= static_cast<std::size_t>(m_extents.template get<Tags>())), ...);
    return n;
  }
  constexpr bool empty() const { return size() == 0; }

  template <class... ET>
  constexpr bool contains(DiscreteElement<ET...> const &e) const {
    auto one = [&](auto tag) {
      using T = decltype(tag);
      auto const x = static_cast<DiscreteVectorElement>(e.template uid<T>());
      auto const f =
          static_cast<DiscreteVectorElement>(m_front.template uid<T>());
      auto const s = m_strides.template get<T>();
      auto const n = m_extents.template get<T>();
      if (n <= 0 || x < f) return false;
      if ((x - f) % s != 0) return false;
      return (x - f) / s < n;
    };
    return (one(Tags{}) && ...);
  }
  // Row-major position of e (every dimension of this domain).
  template <class... ET>
  constexpr std::size_t offset(DiscreteElement<ET...> const &e) const {
    std::size_t off = 0;
    ((off = off * static_cast<std::size_t>(m_extents.template get<Tags>()) +
            static_cast<std::size_t>(
                (static_cast<DiscreteVectorElement>(e.template uid<Tags>()) -
                 static_cast<DiscreteVectorElement>(
                     m_front.template uid<Tags>())) /
                m_strides.template get<Tags>())),
     ...);
    return off;
  }
  template <class F> void for_each(F &&f) const {
    std::array<DiscreteVectorElement, sizeof...(Tags)> ext{
        m_extents.template get<Tags>()...};
    detail::row_major<sizeof...(Tags)>(ext, [&](auto const &k) {
      DiscreteElement<Tags...> e = m_front;
      std::size_t i = 0;
      ((e.template uid<Tags>() += static_cast<DiscreteElementType>(
            k[i] * m_strides.template get<Tags>()),
        ++i),
       ...);
      f(e);
    });
  }
  friend constexpr bool operator==(StridedDiscreteDomain const &a,
                                   StridedDiscreteDomain const &b) {
    if (a.empty() && b.empty()) return true;
    return a.m_front == b.m_front && a.m_extents == b.m_extents &&
           a.m_strides == b.m_strides;
  }
  friend constexpr bool operator!=(StridedDiscreteDomain const &a,
                                   StridedDiscreteDomain const &b) {
    return !(a == b);
  }
};

template <class... Tags> class DiscreteDomain {
  DiscreteElement<Tags...> m_front;
  DiscreteVector<Tags...> m_extents;

public:
  using discrete_element_type = DiscreteElement<Tags...>;
  using discrete_vector_type = DiscreteVector<Tags...>;
  static constexpr bool is_strided_domain = false;

  constexpr DiscreteDomain() = default;
  constexpr DiscreteDomain(DiscreteElement<Tags...> const &front,
                           DiscreteVector<Tags...> const &extents)
      : m_front(front), m_extents(extents) {}
  template <class... Parts,
            std::enable_if_t<(sizeof...(Parts) >= 1) &&
                                 (!Parts::is_strided_domain && ...),
                             int> = 0>
  explicit constexpr DiscreteDomain(Parts const &...parts)
      : m_front(parts.front()...), m_extents(parts.extents()...) {}

  constexpr DiscreteElement<Tags...> front() const { return m_front; }
  constexpr DiscreteElement<Tags...> back() const {
    DiscreteElement<Tags...> b = m_front;
    ((b.template uid<Tags>() += static_cast<DiscreteElementType>(
          m_extents.template get<Tags>() - 1)),
     ...);
    return b;
  }
  constexpr DiscreteVector<Tags...> extents() const { return m_extents; }
  constexpr DiscreteVector<Tags...> strides() const {
    return DiscreteVector<Tags...>((Tags{}, 1)...);
  }
  constexpr std::size_t size() const {
    std::size_t n = 1;
    ((n *= static_cast<std::size_t>(m_extents.template get<Tags>())), ...);
    return n;
  }
  constexpr bool empty() const { return size() == 0; }
  constexpr DiscreteDomain remove_last(DiscreteVector<Tags...> const &n) const {
    return DiscreteDomain(m_front, m_extents - n);
  }
  template <class... ET>
  constexpr bool contains(DiscreteElement<ET...> const &e) const {
    return ((e.template uid<Tags>() >= m_front.template uid<Tags>() &&
             e.template uid<Tags>() - m_front.template uid<Tags>() <
                 static_cast<DiscreteElementType>(
                     m_extents.template get<Tags>())) &&
            ...);
  }
  template <class F> void for_each(F &&f) const {
    StridedDiscreteDomain<Tags...>(m_front, m_extents, strides()).for_each(f);
  }
};

struct SparseTag {};

template <class... Tags> class SparseDiscreteDomain : public SparseTag {
  // Sorted uids per dimension (the domain is their product).
  std::array<std::vector<DiscreteElementType>, sizeof...(Tags)> m_uids;

  template <class... T> friend class SparseDiscreteDomain;

public:
  using discrete_element_type = DiscreteElement<Tags...>;
  static constexpr bool is_strided_domain = false;

  SparseDiscreteDomain() = default;

  // From a list of one-dimensional elements: any container with size() and
  // operator()(i) (a Kokkos view) or operator[](i) (a std::vector).
  template <class Elements,
            std::enable_if_t<sizeof...(Tags) == 1 &&
                                 !std::is_base_of_v<SparseTag, Elements>,
                             int> = 0>
  explicit SparseDiscreteDomain(Elements const &elements) {
    for (std::size_t i = 0; i < elements.size(); ++i) {
      if constexpr (std::is_invocable_v<Elements const &, std::size_t>)
        m_uids[0].push_back(elements(i).uid());
      else
        m_uids[0].push_back(elements[i].uid());
    }
    std::sort(m_uids[0].begin(), m_uids[0].end());
  }
  // From sparse domains over other tag sets: each tag taken from the first
  // part that has it.
  template <class... Parts,
            std::enable_if_t<(sizeof...(Parts) >= 1) &&
                                 (Parts::is_sparse_domain && ...),
                             int> = 0>
  explicit SparseDiscreteDomain(Parts const &...parts)
      : m_uids{take<Tags>(parts...)...} {}
  static constexpr bool is_sparse_domain = true;

  template <class T> static constexpr bool has_tag() {
    return (std::is_same_v<T, Tags> || ...);
  }
  template <class T> std::vector<DiscreteElementType> const &uids() const {
    return m_uids[detail::tag_index<T, Tags...>()];
  }

  std::size_t size() const {
    std::size_t n = 1;
    for (auto const &u : m_uids) n *= u.size();
    return n;
  }
  bool empty() const { return size() == 0; }
  DiscreteVector<Tags...> extents() const {
    return DiscreteVector<Tags...>(
        static_cast<DiscreteVectorElement>(uids<Tags>().size())...);
  }
  DiscreteElement<Tags...> front() const {
    return DiscreteElement<Tags...>(uids<Tags>().front()...);
  }
  DiscreteElement<Tags...> back() const {
    return DiscreteElement<Tags...>(uids<Tags>().back()...);
  }
  template <class... ET> bool contains(DiscreteElement<ET...> const &e) const {
    return (std::binary_search(uids<Tags>().begin(), uids<Tags>().end(),
                               e.template uid<Tags>()) &&
            ...);
  }
  template <class F> void for_each(F &&f) const {
    std::array<DiscreteVectorElement, sizeof...(Tags)> ext{
        static_cast<DiscreteVectorElement>(uids<Tags>().size())...};
    detail::row_major<sizeof...(Tags)>(ext, [&](auto const &k) {
      std::size_t i = 0;
      DiscreteElement<Tags...> e((uids<Tags>()[k[i++]])...);
      f(e);
    });
  }

  // Iteration of one-dimensional sparse domains.
  class iterator {
    std::vector<DiscreteElementType> const *m_u;
    std::size_t m_i;

  public:
    iterator(std::vector<DiscreteElementType> const *u, std::size_t i)
        : m_u(u), m_i(i) {}
    DiscreteElement<Tags...> operator*() const {
      return DiscreteElement<Tags...>((*m_u)[m_i]);
    }
    iterator &operator++() {
      ++m_i;
      return *this;
    }
    bool operator!=(iterator const &o) const { return m_i != o.m_i; }
    bool operator==(iterator const &o) const { return m_i == o.m_i; }
  };
  iterator begin() const { return iterator(&m_uids[0], 0); }
  iterator end() const { return iterator(&m_uids[0], m_uids[0].size()); }

private:
  template <class T, class First, class... Rest>
  static std::vector<DiscreteElementType> take(First const &f,
                                               Rest const &...r) {
    if constexpr (First::template has_tag<T>())
      return f.template uids<T>();
    else
      return take<T>(r...);
  }
};

template <class... Sel, class... T>
constexpr StridedDiscreteDomain<Sel...>
select(StridedDiscreteDomain<T...> const &d) {
  return StridedDiscreteDomain<Sel...>(select<Sel...>(d.front()),
                                       select<Sel...>(d.extents()),
                                       select<Sel...>(d.strides()));
}
template <class... Sel, class... T>
constexpr DiscreteDomain<Sel...> select(DiscreteDomain<T...> const &d) {
  return DiscreteDomain<Sel...>(select<Sel...>(d.front()),
                                select<Sel...>(d.extents()));
}
template <class... Sel, class... T>
SparseDiscreteDomain<Sel...> select(SparseDiscreteDomain<T...> const &d) {
  return SparseDiscreteDomain<Sel...>(d);
}

namespace detail {
template <class Seq> struct strided_of;
template <class... T> struct strided_of<TypeSeq<T...>> {
  using type = StridedDiscreteDomain<T...>;
  template <class... A>
  static constexpr type from(StridedDiscreteDomain<A...> const &d) {
    return select<T...>(d);
  }
};
} // namespace detail

template <class... Rm, class... T>
constexpr auto remove_dims_of(StridedDiscreteDomain<T...> const &d) {
  static_assert(sizeof...(Rm) == 1, "one dimension at a time");
  using Seq = typename detail::remove_one<Rm..., detail::TypeSeq<>, T...>::type;
  return detail::strided_of<Seq>::from(d);
}

// ---------------------------------------------------------- iteration

template <class Domain, class F> void host_for_each(Domain const &d, F &&f) {
  d.for_each(f);
}
template <class Exec, class Domain, class F>
void parallel_for_each(Exec const &, Domain const &d, F &&f) {
  d.for_each(f);
}
template <class Domain, class F,
          std::enable_if_t<!std::is_invocable_v<Domain>, int> = 0>
void parallel_for_each(Domain const &d, F &&f) {
  d.for_each(f);
}

// ------------------------------------------------------------- chunks

// A non-owning dense row-major view of values over a domain.
template <class ElementType, class Support> class ChunkSpan {
  ElementType *m_data = nullptr;
  Support m_domain;

public:
  using element_type = ElementType;
  using value_type = std::remove_cv_t<ElementType>;
  using discrete_domain_type = Support;

  ChunkSpan() = default;
  ChunkSpan(ElementType *data, Support const &domain)
      : m_data(data), m_domain(domain) {}
  Support const &domain() const { return m_domain; }
  ElementType *data_handle() const { return m_data; }
  std::size_t size() const { return m_domain.size(); }
  template <class... ET>
  ElementType &operator()(DiscreteElement<ET...> const &e) const {
    return m_data[m_domain.offset(e)];
  }
  ChunkSpan span_view() const { return *this; }
};

// ------------------------------------------- uniform point sampling

template <class CDim> class Coordinate {
  double m_x = 0.0;

public:
  constexpr Coordinate() = default;
  constexpr explicit Coordinate(double x) : m_x(x) {}
  constexpr operator double() const { return m_x; }
};

// Points origin + uid * step of one continuous dimension CDim.
template <class CDim> class UniformPointSampling {
public:
  using continuous_dimension_type = CDim;

  template <class DDim> class Impl {
    double m_origin = 0.0, m_step = 1.0;

  public:
    Impl() = default;
    Impl(double origin, double step) : m_origin(origin), m_step(step) {}
    Coordinate<CDim> origin() const { return Coordinate<CDim>(m_origin); }
    double step() const { return m_step; }
    DiscreteElement<DDim> front() const { return DiscreteElement<DDim>(0); }
    Coordinate<CDim> coordinate(DiscreteElement<DDim> const &e) const {
      return Coordinate<CDim>(m_origin +
                              static_cast<double>(e.uid()) * m_step);
    }
  };

  // n points from a to b, both included.
  template <class DDim>
  static std::tuple<Impl<DDim>, DiscreteDomain<DDim>>
  init(Coordinate<CDim> a, Coordinate<CDim> b, DiscreteVector<DDim> n) {
    double const step = (double(b) - double(a)) /
                        static_cast<double>(static_cast<DiscreteVectorElement>(n) - 1);
    return {Impl<DDim>(double(a), step),
            DiscreteDomain<DDim>(DiscreteElement<DDim>(0), n)};
  }
};

namespace detail {
template <class DDim> struct DiscreteSpaceSlot {
  static inline std::optional<
      typename DDim::template Impl<DDim>> value;
};
} // namespace detail

template <class DDim, class ImplT, class DomainT>
DomainT init_discrete_space(std::tuple<ImplT, DomainT> const &t) {
  detail::DiscreteSpaceSlot<DDim>::value = std::get<0>(t);
  return std::get<1>(t);
}
template <class DDim> bool is_discrete_space_initialized() {
  return detail::DiscreteSpaceSlot<DDim>::value.has_value();
}
template <class DDim> auto const &host_discrete_space() {
  if (!detail::DiscreteSpaceSlot<DDim>::value)
    throw std::runtime_error("discrete space not initialised");
  return *detail::DiscreteSpaceSlot<DDim>::value;
}
template <class DDim>
auto coordinate(DiscreteElement<DDim> const &e) {
  return host_discrete_space<DDim>().coordinate(e);
}

template <class T, class... Tags>
constexpr DiscreteVectorElement get(DiscreteVector<Tags...> const &v) {
  return v.template get<T>();
}

} // namespace ddc
