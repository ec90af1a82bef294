// Host planner of the restricted-output transform: which points of one axis
// every (level, pass) of a lifting sequence must write so that a requested
// output interval comes out exact, and which inputs that reads.
//
// Drop-in for the planner half of paliwa/paliwa_domains.hpp:
//   PeriodicBounds                                   (:316-322)
//   transform_bounds                                 (:357-452)
//   covering_periodic_bounds                         (:488-503)
//   PolePassSegment / pole_pass_segments             (:505-538)
// Same names, argument meaning and exceptions (std::invalid_argument). Plain
// C++17 without DDC, so that the C-ABI library plans with the same code the
// callers see; the DDC-typed helpers (for_each_transform_index,
// restrict_periodic_bounds) live in paliwa_transform.hpp.
#pragma once

#include <algorithm>
#include <array>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <utility>
#include <vector>

namespace paliwa {

// Inclusive bounds on one axis in finest-level uids; min > max wraps around
// the period, min < 0 is the empty set. The stride comes from the level and
// parity the bounds belong to.
struct PeriodicBounds {
  long min = -1;
  long max = -1;
  bool empty() const { return min < 0; }
};

namespace detail {

// An interval on the unwrapped axis (no periodic cases while it grows);
// empty when lo > hi.
struct AxisInterval {
  long lo = 1;
  long hi = 0;
  bool empty() const { return lo > hi; }

  static long floor_mod(long x, long m) {
    long const r = x % m;
    return r < 0 ? r + m : r;
  }

  // The points of the lattice {offset + k * stride} inside the interval,
  // as the tightest interval with lattice end points.
  AxisInterval on_lattice(long stride, long offset) const {
    if (empty()) return {};
    return {lo + floor_mod(offset - lo, stride),
            hi - floor_mod(hi - offset, stride)};
  }

  void merge(AxisInterval const &o) {
    if (o.empty()) return;
    if (empty()) {
      *this = o;
      return;
    }
    lo = std::min(lo, o.lo);
    hi = std::max(hi, o.hi);
  }

  // Back onto the periodic axis. An interval that holds a whole period of
  // its lattice becomes the canonical full range, so that no point is
  // listed twice.
  PeriodicBounds wrap(long period, long stride, long offset) const {
    if (empty()) return {};
    if ((hi - lo) / stride + 1 >= period / stride)
      return {offset, offset + period - stride};
    return {floor_mod(lo, period), floor_mod(hi, period)};
  }
};

} // namespace detail

// Exact access sets of a restricted transform along one axis. The state is
// one interval per hierarchical level: the odd points of level h (h >= 1,
// lattice 2^(L-h) + k 2^(L-h+1)) or the single coarse lattice of level 0
// (multiples of 2^L). Passes are walked last to first; each pass's write set
// is reported through visit_pass(level index, pass index, bounds), and its
// three-point stencil extends the sets it reads. Returns the required input
// bounds per level 0..level. Levels must be consecutive (a gap would leave
// holes in the even points); coefficient values are not inspected.
template <typename LevelRange, typename VisitPass>
std::vector<PeriodicBounds> transform_bounds(
    PeriodicBounds outputs, long level, long maximum_level,
    LevelRange const &levels,
    std::vector<std::pair<int, std::array<double, 3>>> const &filters,
    VisitPass visit_pass) {
  using detail::AxisInterval;
  std::vector<long> const order(levels.begin(), levels.end());
  if (order.size() > 1) {
    long const step = order[1] - order[0];
    if (step != 1 && step != -1)
      throw std::invalid_argument("Transform levels must be consecutive");
    for (size_t i = 1; i < order.size(); ++i)
      if (order[i] - order[i - 1] != step)
        throw std::invalid_argument(
            "Transform levels must be monotone and consecutive");
  }
  long const period = 1L << maximum_level;
  auto lattice_stride = [&](long h) {
    return h == 0 ? period : 2L << (maximum_level - h);
  };
  auto lattice_offset = [&](long h) {
    return h == 0 ? 0L : 1L << (maximum_level - h);
  };
  AxisInterval out;
  if (!outputs.empty())
    out = {outputs.min, outputs.max + (outputs.min > outputs.max ? period : 0)};
  std::vector<AxisInterval> need(static_cast<size_t>(level + 1));
  for (long h = 0; h <= level; ++h)
    need[h] = out.on_lattice(lattice_stride(h), lattice_offset(h));

  for (size_t i = order.size(); i-- > 0;) {
    long const l = order[i];
    if (l < 1 || l > level)
      throw std::invalid_argument("Invalid transform level");
    long const s = 1L << (maximum_level - l);
    for (size_t pass = filters.size(); pass-- > 0;) {
      int const parity = filters[pass].first;
      if (parity != 0 && parity != 1)
        throw std::invalid_argument("Filter offset not supported");
      // Odd points of level l are need[l]; its even points are exactly the
      // points of all coarser levels.
      AxisInterval writes;
      if (parity == 1) {
        writes = need[l];
      } else {
        for (long h = 0; h < l; ++h) writes.merge(need[h]);
      }
      visit_pass(i, pass, writes.wrap(period, 2 * s, parity * s));
      if (writes.empty()) continue;
      AxisInterval const taps{writes.lo - s, writes.hi + s};
      if (parity == 0) {
        need[l].merge(taps.on_lattice(2 * s, s));
      } else {
        for (long h = 0; h < l; ++h)
          need[h].merge(taps.on_lattice(lattice_stride(h), lattice_offset(h)));
      }
    }
  }
  std::vector<PeriodicBounds> bounds(static_cast<size_t>(level + 1));
  for (long h = 0; h <= level; ++h)
    bounds[h] = need[h].wrap(period, lattice_stride(h), lattice_offset(h));
  return bounds;
}

// The smallest periodic interval that holds every index of a sorted list of
// distinct indices: it starts after the largest gap between neighbours.
inline PeriodicBounds covering_periodic_bounds(std::vector<long> const &indices,
                                               long period) {
  if (indices.empty()) return {};
  PeriodicBounds best{indices.front(), indices.back()};
  long widest = indices.front() + period - indices.back();
  for (size_t k = 1; k < indices.size(); ++k) {
    long const gap = indices[k] - indices[k - 1];
    if (gap > widest) {
      widest = gap;
      best = {indices[k], indices[k - 1]};
    }
  }
  return best;
}

// One affine run of a lifting pass in packed-pencil slots: `count` writes
// from slot `first` by `stride`, reading slots lower + k stride and
// upper + k stride. Runs are cut where a neighbour wraps around the pencil.
struct PolePassSegment {
  int first, count, stride;
  int lower, upper;
};

// Runs of one pass over the written interval `writes` (finest uids) of a
// pencil of 2^level points at spacing 2^(maximum_level - level) that starts
// at uid `origin`, for the pass of level `pass_level`. Uids are unsigned
// like DDC's DiscreteElementType (std::size_t); only slots must fit an int.
inline std::vector<PolePassSegment>
pole_pass_segments(PeriodicBounds writes, std::size_t origin, int level,
                   int maximum_level, int pass_level) {
  using Uid = std::size_t;
  std::vector<PolePassSegment> runs;
  if (writes.empty()) return runs;
  if (level < 1 || level >= std::numeric_limits<int>::digits ||
      maximum_level < level ||
      maximum_level >= std::numeric_limits<Uid>::digits ||
      pass_level < 1 || pass_level > level)
    throw std::invalid_argument("Invalid levels for packed-pole indexing");
  int const n = 1 << level;                    // slots in the pencil
  int const dist = 1 << (level - pass_level);  // neighbour distance
  int const step = 2 * dist;
  int const shift = maximum_level - level;
  Uid const uperiod = Uid{1} << maximum_level;
  Uid const a = static_cast<Uid>(writes.min);
  Uid const b = static_cast<Uid>(writes.max);
  Uid const span = b >= a ? b - a : uperiod - (a - b);
  int left = static_cast<int>(span >> shift) / step + 1;
  int x = static_cast<int>((a >= origin ? a - origin : uperiod - (origin - a)) >>
                           shift);
  while (left > 0) {
    int const lo = x < dist ? x + n - dist : x - dist;
    int const hi = x >= n - dist ? x + dist - n : x + dist;
    // Last slot before the lower or upper neighbour changes its wrap.
    int const last = x < dist ? dist - 1 : (x < n - dist ? n - dist - 1 : n - 1);
    int const k = std::min(left, (last - x) / step + 1);
    runs.push_back({x, k, step, lo, hi});
    left -= k;
    int const advance = k * step;
    x = advance >= n - x ? advance - (n - x) : x + advance;
  }
  return runs;
}

} // namespace paliwa
