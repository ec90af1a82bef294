// Serial stand-in for the part of Kokkos' public API that paliwa's headers
// use -- TEST INFRASTRUCTURE. It lets the unmodified reference headers
// compile into oracle/_ref (see oracle/Makefile, target `ref`), so that the
// CPU oracle can be checked against the reference itself. Kokkos is not in
// this image; nothing here comes from its sources: each name below follows
// its documented meaning, executed serially on the host.
#pragma once

#include <cassert>
#include <cstddef>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define KOKKOS_LAMBDA [=]
#define KOKKOS_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_ASSERT(x) assert(x)

namespace Kokkos {

struct HostSpace {};
using SharedSpace = HostSpace;
using SharedHostPinnedSpace = HostSpace;

// The only execution space: runs every iteration in order on the calling
// thread; fence() has nothing to wait for.
struct Serial {
  using execution_space = Serial;
  using memory_space = HostSpace;
  void fence() const {}
  static int concurrency() { return 1; }
};
using DefaultExecutionSpace = Serial;
using DefaultHostExecutionSpace = Serial;

template <class ExecSpace, class Space> struct SpaceAccessibility {
  static constexpr bool accessible = true;
};

struct LayoutRight {};

struct WithoutInitializing_t {};
inline constexpr WithoutInitializing_t WithoutInitializing{};

struct ViewAllocProp {
  std::string label;
};
namespace detail {
inline void collect(ViewAllocProp &) {}
template <class... R>
void collect(ViewAllocProp &p, std::string const &s, R const &...r) {
  p.label = s;
  collect(p, r...);
}
template <class... R>
void collect(ViewAllocProp &p, char const *s, R const &...r) {
  p.label = s;
  collect(p, r...);
}
template <class T, class... R>
void collect(ViewAllocProp &p, T const &, R const &...r) {
  collect(p, r...);
}
} // namespace detail
template <class... Args> ViewAllocProp view_alloc(Args const &...args) {
  ViewAllocProp p;
  detail::collect(p, args...);
  return p;
}

// Host arrays of rank 1 (T*) and rank 2 (T**, row-major), value-initialised.
// Like Kokkos views, copies are handles to the same storage (shallow): a
// lambda that captures a view by value writes the caller's array.
template <class DataType, class... Props> class View;

template <class T, class... Props> class View<T *, Props...> {
public:
  using value_type = T;
  View() : m_data(std::make_shared<std::vector<T>>()) {}
  View(std::string const &, std::size_t n)
      : m_data(std::make_shared<std::vector<T>>(n)) {}
  View(char const *, std::size_t n)
      : m_data(std::make_shared<std::vector<T>>(n)) {}
  View(ViewAllocProp const &, std::size_t n)
      : m_data(std::make_shared<std::vector<T>>(n)) {}
  T &operator()(std::size_t i) const { return (*m_data)[i]; }
  T *data() const { return m_data->data(); }
  std::size_t size() const { return m_data->size(); }
  std::size_t extent(int) const { return m_data->size(); }
  void resize_to(std::size_t n) { m_data->resize(n); }

private:
  std::shared_ptr<std::vector<T>> m_data;
};

template <class T, class... Props> class View<T **, Props...> {
public:
  using value_type = T;
  View() : m_data(std::make_shared<std::vector<T>>()) {}
  View(ViewAllocProp const &, std::size_t n0, std::size_t n1)
      : m_n1(n1), m_data(std::make_shared<std::vector<T>>(n0 * n1)) {}
  View(std::string const &, std::size_t n0, std::size_t n1)
      : m_n1(n1), m_data(std::make_shared<std::vector<T>>(n0 * n1)) {}
  T &operator()(std::size_t i, std::size_t j) const {
    return (*m_data)[i * m_n1 + j];
  }
  T *data() const { return m_data->data(); }
  std::size_t extent(int r) const {
    return r == 0 ? (m_n1 ? m_data->size() / m_n1 : 0) : m_n1;
  }

private:
  std::size_t m_n1 = 0;
  std::shared_ptr<std::vector<T>> m_data;
};

template <class T, class... Props>
void resize(View<T *, Props...> &v, std::size_t n) {
  v.resize_to(n);
}

namespace Experimental {
// One token per concurrent thread of the space: one for Serial.
template <class ExecSpace> class UniqueToken {
public:
  UniqueToken() = default;
  explicit UniqueToken(ExecSpace const &) {}
  int size() const { return 1; }
  int acquire() const { return 0; }
  void release(int) const {}
};
} // namespace Experimental

inline void fence() {}

} // namespace Kokkos
