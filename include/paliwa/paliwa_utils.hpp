// Drop-in for paliwa/paliwa_utils.hpp: enumeration of hierarchical
// subspaces (:9-26) and fencing a set of execution instances (:27-32).
#pragma once

#include <cassert>
#include <cstddef>
#include <functional>

namespace paliwa {

// Calls callback(tmp_level) for every vector with
// 0 <= tmp_level[d] <= nodal_level[d] in the dimensions d >= current_dim
// (the others keep their values), in lexicographic order, the last
// dimension fastest. T is an indexable sequence such as
// std::array<long, d>. On return tmp_level[d] = nodal_level[d] + 1 for
// d >= current_dim.
template <typename T>
constexpr void
iterate_hierarchical_subspaces(const T &nodal_level, T &tmp_level,
                               size_t current_dim,
                               const std::function<void(const T &)> &callback) {
  assert(tmp_level.size() == nodal_level.size());
  size_t const n = nodal_level.size();
  if (current_dim >= n) {
    callback(tmp_level);
    return;
  }
  for (size_t d = current_dim; d < n; ++d) tmp_level[d] = 0;
  for (;;) {
    callback(tmp_level);
    // Odometer step over dimensions n-1 .. current_dim.
    size_t d = n;
    while (d > current_dim) {
      --d;
      if (tmp_level[d] < nodal_level[d]) {
        ++tmp_level[d];
        break;
      }
      if (d == current_dim) {
        for (size_t e = current_dim; e < n; ++e)
          tmp_level[e] = nodal_level[e] + 1;
        return;
      }
      tmp_level[d] = 0;
    }
  }
}

// Waits for every instance's queued work (instance.fence()).
template <typename InstancesType>
constexpr void fence_all_instances(InstancesType const &instances) {
  for (auto const &instance : instances) instance.fence();
}

} // namespace paliwa
