// Host planner of the restricted-output transform: which points of one axis
// every (level, pass) of a lifting sequence must write so that a requested
// output interval comes out exact, and which inputs that reads.
//
// Interface of the planner half of paliwa/paliwa_domains.hpp:
//   PeriodicBounds                                   (:317-321)
//   transform_bounds                                 (:365-434)
//   covering_periodic_bounds                         (:471-485)
//   PolePassSegment / pole_pass_segments             (:489-535)
// Same names, argument meaning and exception types; plain C++17 without DDC,
// so that the C-ABI library plans with the same code its callers see.
//
// Method. A lifting pass of level l with parity o writes the points
// x = o s + 2 k s (s = 2^(L - l), finest uids) and reads x - s, x, x + s.
// Walking the passes from last to first, the set of points whose values the
// outputs still depend on is kept as a list of arithmetic progressions of
// uids on the unwrapped axis. A pass must write exactly the points of that
// set on its own lattice; for consecutive levels these form one progression
// of the lattice (the property the reference's tests check against a
// brute-force walk of the stencil graph), so its hull is the write set. The
// pass then adds its taps x +- s, which again form one progression. The
// required inputs of hierarchical level h are the set's points on h's
// lattice (odd multiples of 2^(L - h), or multiples of 2^L for h = 0).
#pragma once

#include <algorithm>
#include <array>
#include <cstddef>
#include <cstdint>
#include <iterator>
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

namespace plan {

inline long mod_floor(long x, long m) {
  long const r = x % m;
  return r < 0 ? r + m : r;
}

// {first, first + step, ..., last} on the unwrapped uid axis; step is a
// power of two; empty when last < first.
struct Progression {
  long first = 0;
  long last = -1;
  long step = 1;
  bool empty() const { return last < first; }
};

// The points of p on the lattice {offset + k * stride} (stride a power of
// two, like p.step).
inline Progression on_lattice(Progression const &p, long stride, long offset) {
  if (p.empty()) return {};
  if (p.step >= stride) {
    // Every point of p has the same residue modulo stride.
    if (mod_floor(p.first - offset, stride) != 0) return {};
    return p;
  }
  // p visits every residue modulo stride that is congruent to p.first
  // modulo p.step; the lattice's residue is among them or not.
  if (mod_floor(offset - p.first, p.step) != 0) return {};
  long const lo = p.first + mod_floor(offset - p.first, stride);
  long const hi = p.last - mod_floor(p.last - offset, stride);
  if (hi < lo) return {};
  return {lo, hi, stride};
}

// Smallest progression of the lattice that holds the lattice points of
// every progression in `set`.
inline Progression hull_on_lattice(std::vector<Progression> const &set,
                                   long stride, long offset) {
  Progression h{0, -1, stride};
  bool any = false;
  for (auto const &p : set) {
    Progression const q = on_lattice(p, stride, offset);
    if (q.empty()) continue;
    h.first = any ? std::min(h.first, q.first) : q.first;
    h.last = any ? std::max(h.last, q.last) : q.last;
    any = true;
  }
  return h;
}

// A lattice progression as periodic bounds: the whole lattice (one period
// or more) becomes the canonical range {offset, offset + period - stride},
// so that no point is listed twice.
inline PeriodicBounds to_bounds(Progression const &p, long period,
                                long stride, long offset) {
  if (p.empty()) return {};
  if (p.last - p.first >= period - stride)
    return {offset, offset + period - stride};
  return {mod_floor(p.first, period), mod_floor(p.last, period)};
}

// Lattice of hierarchical level h inside maximum level L.
inline long level_stride(long h, long L) { return h == 0 ? 1L << L : 2L << (L - h); }
inline long level_offset(long h, long L) { return h == 0 ? 0L : 1L << (L - h); }

inline void check_consecutive(std::vector<long> const &levels) {
  if (levels.size() < 2) return;
  long const d = levels[1] - levels[0];
  if (d != 1 && d != -1)
    throw std::invalid_argument("Transform levels must be consecutive");
  for (size_t i = 2; i < levels.size(); ++i)
    if (levels[i] - levels[i - 1] != d)
      throw std::invalid_argument(
          "Transform levels must be monotone and consecutive");
}

} // namespace plan

// Exact access sets of a restricted transform along one axis: calls
// visit_pass(level index, pass index, write bounds) for every pass, last to
// first, and returns the required input bounds per hierarchical level
// 0..level. `levels` must be consecutive and monotone; only the filters'
// parities matter.
template <typename LevelRange, typename VisitPass>
std::vector<PeriodicBounds> transform_bounds(
    PeriodicBounds outputs, long level, long maximum_level,
    LevelRange const &levels,
    std::vector<std::pair<int, std::array<double, 3>>> const &filters,
    VisitPass visit_pass) {
  using plan::Progression;
  std::vector<long> const seq(levels.begin(), levels.end());
  plan::check_consecutive(seq);
  long const L = maximum_level;
  long const period = 1L << L;
  std::vector<Progression> needed;
  if (!outputs.empty()) {
    // The grid's points (the lattice of `level`) inside the outputs.
    long const spacing = 1L << (L - level);
    long const hi = outputs.max + (outputs.max < outputs.min ? period : 0);
    needed.push_back(plan::on_lattice({outputs.min, hi, 1}, spacing, 0));
  }
  for (auto li = seq.rbegin(); li != seq.rend(); ++li) {
    long const l = *li;
    if (l < 1 || l > level)
      throw std::invalid_argument("Invalid transform level");
    long const s = 1L << (L - l);
    size_t const index = static_cast<size_t>(std::distance(li, seq.rend())) - 1;
    for (size_t pass = filters.size(); pass-- > 0;) {
      int const parity = filters[pass].first;
      if (parity != 0 && parity != 1)
        throw std::invalid_argument("Filter offset not supported");
      Progression const w = plan::hull_on_lattice(needed, 2 * s, parity * s);
      visit_pass(index, pass, plan::to_bounds(w, period, 2 * s, parity * s));
      if (!w.empty()) needed.push_back({w.first - s, w.last + s, 2 * s});
    }
  }
  std::vector<PeriodicBounds> required;
  required.reserve(static_cast<size_t>(level + 1));
  for (long h = 0; h <= level; ++h) {
    long const st = plan::level_stride(h, L), off = plan::level_offset(h, L);
    required.push_back(
        plan::to_bounds(plan::hull_on_lattice(needed, st, off), period, st,
                        off));
  }
  return required;
}

// The smallest periodic interval holding every index of a sorted list of
// distinct indices: it starts right after the widest gap between
// neighbours (the gap that wraps from the last index to the first counts,
// and wins ties, then earlier gaps).
inline PeriodicBounds covering_periodic_bounds(std::vector<long> const &indices,
                                               long period) {
  if (indices.empty()) return {};
  std::vector<long> gaps(indices.size());
  gaps[0] = indices.front() + period - indices.back();
  for (size_t k = 1; k < indices.size(); ++k)
    gaps[k] = indices[k] - indices[k - 1];
  size_t const g = static_cast<size_t>(
      std::distance(gaps.begin(), std::max_element(gaps.begin(), gaps.end())));
  if (g == 0) return {indices.front(), indices.back()};
  return {indices[g], indices[g - 1]};
}

// One affine run of a lifting pass in packed-pencil slots: `count` writes
// from slot `first` by `stride`, reading slots lower + k stride and
// upper + k stride.
struct PolePassSegment {
  int first, count, stride;
  int lower, upper;
};

// Runs of one pass over the written interval `writes` (finest uids) of a
// pencil of 2^level slots at spacing 2^(maximum_level - level) whose slot 0
// is uid `origin`, for the pass of level `pass_level`. A run ends where a
// neighbour starts or stops wrapping around the pencil (slots dist and
// n - dist, dist = 2^(level - pass_level)) or where the writes wrap past the
// last slot. Uids are unsigned like DDC's DiscreteElementType; only slots
// must fit an int.
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
  int const n = 1 << level;
  int const dist = 1 << (level - pass_level);
  int const step = 2 * dist;
  int const shift = maximum_level - level;
  Uid const upos = Uid{1} << maximum_level;
  auto slot_of = [&](Uid uid) {
    Uid const rel = uid >= origin ? uid - origin : upos - (origin - uid);
    return static_cast<int>(rel >> shift);
  };
  Uid const a = static_cast<Uid>(writes.min), b = static_cast<Uid>(writes.max);
  Uid const span = b >= a ? b - a : upos - (a - b);
  int remaining = static_cast<int>(span >> shift) / step + 1;
  int const boundaries[3] = {dist, n - dist, n};
  for (int x = slot_of(a); remaining > 0;) {
    int const next = *std::upper_bound(boundaries, boundaries + 3, x);
    int const count = std::min(remaining, (next - x + step - 1) / step);
    int const lower = x - dist < 0 ? x - dist + n : x - dist;
    int const upper = x + dist >= n ? x + dist - n : x + dist;
    runs.push_back({x, count, step, lower, upper});
    remaining -= count;
    x = static_cast<int>((static_cast<long>(x) + static_cast<long>(count) * step) % n);
  }
  return runs;
}

} // namespace paliwa
