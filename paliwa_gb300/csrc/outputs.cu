// Restricted-output transform along one axis: transform_in(grid, level,
// maximum_level, levels, filters, outputs, ...) of the reference
// (paliwa/paliwa_transform.hpp:258-344, Direct execution), which writes only
// the points that the requested outputs depend on.
//
// Planning is host code shared with the drop-in headers
// (include/paliwa/paliwa_plan.hpp: transform_bounds). Every (level, pass)
// then writes one or two runs of its parity lattice along the axis (the
// planned periodic bounds, cut at the period) times the outputs' points in
// the other dimensions; each run is one launch of out_pass_kernel, one thread
// per written point, in the reference's order of levels and passes, so the
// buffer ends bit-identical to the reference's (outputs, and the
// intermediate values it leaves in the dependency cone).
//
// The grid is a window buffer: along dimension d it holds the uids
// (front[d] + k * spacing[d]) mod 2^L[d], k < extents[d], spacing[d] =
// 2^(L[d] - level[d]), dense and row-major. The full grid is the window with
// front 0 and 2^level points; a window may wrap around the period, so one
// buffer holds a slab and the periodic halo it needs (what the reference
// keeps in separate local and remote storage).
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "arith.cuh"
#include "paliwa_gb300.h"
#include "paliwa/paliwa_plan.hpp"
#include "plan.hpp"

namespace pgb {

bool exact_scalers(std::vector<Filter> const &filters);

namespace {

constexpr int kOutMaxDims = 12;
constexpr int kOutThreads = 256;

struct OutPass {
  unsigned long long base;
  int ndim, dim;
  int log2_spacing;                // along dim, uid -> buffer index
  long long period, wfront;        // along dim, in uids
  long long s;                     // neighbour distance in uids
  long long first, step, count;    // written uids first + k step, k < count
  long long total;                 // threads with work
  long long elem[kOutMaxDims];     // element strides of the buffer
  long long obase[kOutMaxDims];    // other dims: buffer index of output 0
  long long ostep[kOutMaxDims];    //   index step between outputs
  long long oext[kOutMaxDims];     //   output count (count along dim)
  Coeffs c;
};

template <typename T, bool Exact>
__global__ void __launch_bounds__(kOutThreads) out_pass_kernel(OutPass const p) {
  using A = Plain<T, Exact>;
  T *g = reinterpret_cast<T *>(p.base);
  long long const nthreads =
      static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x +
                     threadIdx.x;
       t < p.total; t += nthreads) {
    // Row-major decomposition over the written box (last dimension
    // fastest, so neighbouring threads touch neighbouring outputs).
    unsigned long long r = static_cast<unsigned long long>(t);
    long long off = 0, k = 0;
    for (int d = p.ndim - 1; d >= 0; --d) {
      unsigned long long const e = static_cast<unsigned long long>(p.oext[d]);
      long long const j = static_cast<long long>(r % e);
      r /= e;
      if (d == p.dim)
        k = j;
      else
        off += (p.obase[d] + j * p.ostep[d]) * p.elem[d];
    }
    long long const x = p.first + k * p.step;
    long long const lo = x == 0 ? p.period - p.s : x - p.s;
    long long const up = x + p.s == p.period ? 0 : x + p.s;
    long long const m = p.period - 1;
    long long const es = p.elem[p.dim];
    long long const ix = ((x - p.wfront) & m) >> p.log2_spacing;
    long long const il = ((lo - p.wfront) & m) >> p.log2_spacing;
    long long const iu = ((up - p.wfront) & m) >> p.log2_spacing;
    T const vl = g[off + il * es];
    T const vm = g[off + ix * es];
    T const vu = g[off + iu * es];
    g[off + ix * es] =
        A::template update<false>(p.c, vl, vm, vu);
  }
}

int device_sm_count() {
  int dev = 0, sms = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
             "cudaDeviceGetAttribute");
  return sms;
}

void launch_out_pass(int dtype, bool exact, OutPass const &p, cudaStream_t s) {
  // SM count of the current device (a thread may drive several GPUs).
  static thread_local int sms_by_device[64] = {};
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= 64)
    throw StatusError(PALIWA_GB_RUNTIME_ERROR, "device ordinal too large");
  int &sms = sms_by_device[dev];
  if (sms == 0) sms = device_sm_count();
  // Enough CTAs for 8 per SM (the kernel is latency-bound on three
  // scattered loads per thread); larger passes loop.
  long long const want = (p.total + kOutThreads - 1) / kOutThreads;
  long long const cap = 8LL * sms;
  unsigned const blocks = static_cast<unsigned>(want < cap ? want : cap);
  if (dtype == PALIWA_GB_F64) {
    if (exact)
      out_pass_kernel<double, true><<<blocks, kOutThreads, 0, s>>>(p);
    else
      out_pass_kernel<double, false><<<blocks, kOutThreads, 0, s>>>(p);
  } else {
    if (exact)
      out_pass_kernel<float, true><<<blocks, kOutThreads, 0, s>>>(p);
    else
      out_pass_kernel<float, false><<<blocks, kOutThreads, 0, s>>>(p);
  }
  cuda_check(cudaGetLastError(), "out_pass_kernel launch");
}

long long floor_mod(long long x, long long m) {
  long long const r = x % m;
  return r < 0 ? r + m : r;
}

using FilterList = std::vector<std::pair<int, std::array<double, 3>>>;

FilterList filter_list(int nfilters, int32_t const *offsets,
                       double const *coefficients) {
  if (nfilters < 0)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "negative filter count");
  if (nfilters > 0 && (offsets == nullptr || coefficients == nullptr))
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "filters are null");
  FilterList f;
  for (int p = 0; p < nfilters; ++p)
    f.push_back({offsets[p],
                 {coefficients[3 * p], coefficients[3 * p + 1],
                  coefficients[3 * p + 2]}});
  return f;
}

std::vector<long> level_list(int nlevels, int64_t const *levels) {
  if (nlevels < 0)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "negative level count");
  if (nlevels > 0 && levels == nullptr)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "levels are null");
  return std::vector<long>(levels, levels + nlevels);
}

// transform_bounds with its std::invalid_argument mapped to the status code.
template <typename Visit>
std::vector<paliwa::PeriodicBounds>
plan_bounds(paliwa::PeriodicBounds outputs, long level, long maximum_level,
            std::vector<long> const &levels, FilterList const &filters,
            Visit visit) {
  try {
    return paliwa::transform_bounds(outputs, level, maximum_level, levels,
                                    filters, visit);
  } catch (std::invalid_argument const &e) {
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, e.what());
  }
}

} // namespace
} // namespace pgb

extern "C" {

int paliwa_gb_transform_bounds(int64_t outputs_min, int64_t outputs_max,
                               int64_t level, int64_t maximum_level,
                               const int64_t *levels, int nlevels,
                               const int32_t *offsets, int nfilters,
                               int64_t *bounds, int64_t *writes) {
  using namespace pgb;
  return guarded([&] {
    if (level < 0 || maximum_level < level || maximum_level > 62)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "requires 0 <= level <= maximum_level <= 62");
    if (bounds == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "bounds is null");
    auto const lv = level_list(nlevels, levels);
    if (nfilters < 0 || (nfilters > 0 && offsets == nullptr))
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "bad filters");
    FilterList f;
    for (int p = 0; p < nfilters; ++p) f.push_back({offsets[p], {0, 0, 0}});
    paliwa::PeriodicBounds out{static_cast<long>(outputs_min),
                               static_cast<long>(outputs_max)};
    auto const b = plan_bounds(
        out, static_cast<long>(level), static_cast<long>(maximum_level), lv, f,
        [&](size_t i, size_t p, paliwa::PeriodicBounds w) {
          if (writes == nullptr) return;
          writes[2 * (i * f.size() + p)] = w.min;
          writes[2 * (i * f.size() + p) + 1] = w.max;
        });
    for (size_t h = 0; h < b.size(); ++h) {
      bounds[2 * h] = b[h].min;
      bounds[2 * h + 1] = b[h].max;
    }
  });
}

int paliwa_gb_transform_outputs(
    void *grid, int dtype, int ndim, const int64_t *level,
    const int64_t *maximum_level, const int64_t *window_front,
    const int64_t *window_extents, int dim, const int64_t *levels,
    int nlevels, const int32_t *offsets, const double *coefficients,
    int nfilters, const int64_t *outputs_front,
    const int64_t *outputs_extents, const int64_t *outputs_strides,
    void *stream) {
  using namespace pgb;
  return guarded([&] {
    if (dtype != PALIWA_GB_F64 && dtype != PALIWA_GB_F32)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "restricted outputs support F64 and F32 grids");
    if (ndim < 1 || ndim > kOutMaxDims)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "ndim must be in [1, 12]");
    if (dim < 0 || dim >= ndim)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "bad dimension");
    if (level == nullptr || maximum_level == nullptr ||
        window_front == nullptr || window_extents == nullptr ||
        outputs_front == nullptr || outputs_extents == nullptr ||
        outputs_strides == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    for (int d = 0; d < ndim; ++d)
      if (outputs_extents[d] < 0)
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "negative output extent");
    auto const lv = level_list(nlevels, levels);
    auto const filters = filter_list(nfilters, offsets, coefficients);
    for (int d = 0; d < ndim; ++d)
      if (outputs_extents[d] == 0) return;  // paliwa_transform.hpp:270-271
    size_t const es = dtype_size(dtype);
    if (grid == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "grid is null");
    if (reinterpret_cast<uintptr_t>(grid) % es != 0)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "grid is misaligned");

    OutPass p{};
    p.base = reinterpret_cast<unsigned long long>(grid);
    p.ndim = ndim;
    p.dim = dim;
    long long elem = 1;
    for (int d = ndim - 1; d >= 0; --d) {
      if (level[d] < 0 || maximum_level[d] < level[d] || maximum_level[d] > 30)
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "requires 0 <= level <= maximum_level <= 30");
      long long const period = 1LL << maximum_level[d];
      long long const sp = 1LL << (maximum_level[d] - level[d]);
      long long const ext = window_extents[d];
      if (ext < 1 || ext > (1LL << level[d]))
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "window extent must be in [1, 2^level]");
      if (window_front[d] < 0 || window_front[d] >= period ||
          window_front[d] % sp != 0)
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "window front must be a point of the grid");
      if (outputs_front[d] < 0 || outputs_front[d] >= period)
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "output front outside the period");
      long long const oe = outputs_extents[d];
      long long const os = outputs_strides[d];
      if (oe > 1 && (os <= 0 || (oe - 1) * os >= period))
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "output stride must be positive and the outputs "
                          "within one period");
      p.elem[d] = elem;
      if (elem > (1LL << 40) / ext)
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "window too large");
      elem *= ext;
      if (d == dim) continue;
      // The outputs in the other dimensions: points of this grid, inside
      // the window (written through local_pole_domain, :305-306).
      long long const o0 = floor_mod(outputs_front[d] - window_front[d], period);
      if (o0 % sp != 0 || (oe > 1 && os % sp != 0) ||
          o0 + (oe - 1) * (oe > 1 ? os : 0) > (ext - 1) * sp)
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "outputs must be grid points inside the window");
      p.obase[d] = o0 / sp;
      p.ostep[d] = oe > 1 ? os / sp : 0;
      p.oext[d] = oe;
    }

    // Plan along dim (paliwa_transform.hpp:274-281).
    long long const L = maximum_level[dim];
    long long const period = 1LL << L;
    long long const sp = 1LL << (L - level[dim]);
    long long const ofirst = outputs_front[dim];
    long long const olast =
        ofirst + (outputs_extents[dim] - 1) *
                     (outputs_extents[dim] > 1 ? outputs_strides[dim] : 0);
    paliwa::PeriodicBounds const out{static_cast<long>(ofirst),
                                     static_cast<long>(olast % period)};
    std::vector<std::vector<paliwa::PeriodicBounds>> writes(
        lv.size(), std::vector<paliwa::PeriodicBounds>(filters.size()));
    auto const bounds = plan_bounds(
        out, static_cast<long>(level[dim]), static_cast<long>(L), lv, filters,
        [&](size_t i, size_t q, paliwa::PeriodicBounds w) { writes[i][q] = w; });
    // Every required input must be in the window (:282-289).
    long long const wf = window_front[dim], wext = window_extents[dim];
    for (size_t h = 0; h < bounds.size(); ++h) {
      auto const b = bounds[h];
      if (b.empty()) continue;
      long long const st = h == 0 ? period : 2LL << (L - h);
      long long const last = b.max + (b.min > b.max ? period : 0);
      for (long long x = b.min; x <= last; x += st) {
        long long const o = floor_mod(x - wf, period);
        if (o % sp != 0 || o / sp >= wext)
          throw StatusError(PALIWA_GB_RUNTIME_ERROR,
                            "Transform domain is missing required input "
                            "values");
      }
    }
    int log2_sp = 0;
    while ((1LL << log2_sp) < sp) ++log2_sp;
    p.log2_spacing = log2_sp;
    p.period = period;
    p.wfront = wf;
    long long others = 1;
    for (int d = 0; d < ndim; ++d)
      if (d != dim) others *= p.oext[d];

    bool const exact = exact_scalers([&] {
      std::vector<Filter> v;
      for (auto const &f : filters)
        v.push_back({f.first, {f.second[0], f.second[1], f.second[2]}});
      return v;
    }());
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    // Execute forwards (:310-329): per level and pass, the parity lattice
    // of that level restricted to the planned bounds, cut at the period.
    for (size_t i = 0; i < lv.size(); ++i) {
      long long const l = lv[i];
      long long const st = 1LL << (L - l);
      p.s = st;
      for (size_t q = 0; q < filters.size(); ++q) {
        auto const w = writes[i][q];
        if (w.empty()) continue;
        int const parity = filters[q].first;
        double const *c = filters[q].second.data();
        p.c = Coeffs{c[0], c[1], c[2], static_cast<float>(c[0]),
                     static_cast<float>(c[1]), static_cast<float>(c[2])};
        long long const first = parity * st;
        long long const lastp = first + ((1LL << (l - 1)) - 1) * 2 * st;
        auto run = [&](long long lower, long long upper) {
          lower = std::max(lower, first);
          upper = std::min(upper, lastp);
          long long const begin =
              first + ((lower - first + 2 * st - 1) / (2 * st)) * (2 * st);
          if (begin > upper) return;
          p.first = begin;
          p.step = 2 * st;
          p.count = (upper - begin) / (2 * st) + 1;
          p.oext[dim] = p.count;
          p.total = p.count * others;
          launch_out_pass(dtype, exact, p, s);
        };
        if (w.min <= w.max) {
          run(w.min, w.max);
        } else {
          run(w.min, period - 1);
          run(0, w.max);
        }
      }
    }
  });
}

} // extern "C"

extern "C" int paliwa_gb_transform_in_window(
    void *grid, int dtype, int ndim, const int64_t *level,
    const int64_t *maximum_level, const int64_t *window_front,
    const int64_t *window_extents, int dim, const int64_t *levels,
    int nlevels, const int32_t *offsets, const double *coefficients,
    int npasses, void *stream) {
  using namespace pgb;
  return guarded([&] {
    if (dtype != PALIWA_GB_F64 && dtype != PALIWA_GB_F32)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "windowed transforms support F64 and F32 grids");
    if (ndim < 1 || ndim > kOutMaxDims)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "ndim must be in [1, 12]");
    if (dim < 0 || dim >= ndim)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "bad dimension");
    if (level == nullptr || maximum_level == nullptr ||
        window_front == nullptr || window_extents == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    auto const lv = level_list(nlevels, levels);
    auto const filters = filter_list(npasses, offsets, coefficients);
    OutPass p{};
    p.base = reinterpret_cast<unsigned long long>(grid);
    p.ndim = ndim;
    p.dim = dim;
    long long elem = 1;
    bool empty = false;
    for (int d = ndim - 1; d >= 0; --d) {
      if (level[d] < 0 || maximum_level[d] < level[d] || maximum_level[d] > 30)
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "requires 0 <= level <= maximum_level <= 30");
      long long const period = 1LL << maximum_level[d];
      long long const sp = 1LL << (maximum_level[d] - level[d]);
      long long const ext = window_extents[d];
      // A chunk's domain: a box of the level lattice that does not wrap.
      if (ext < 0 || window_front[d] < 0 || window_front[d] % sp != 0 ||
          (ext > 0 && window_front[d] + (ext - 1) * sp >= period))
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "the window must be a box of the level's lattice "
                          "inside one period");
      if (ext == 0) empty = true;
      p.elem[d] = elem;
      if (ext > 0 && elem > (1LL << 40) / ext)
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "window too large");
      elem *= ext > 0 ? ext : 1;
      p.obase[d] = 0;
      p.ostep[d] = 1;
      p.oext[d] = ext;
    }
    long long const L = maximum_level[dim];
    for (long l : lv)
      if (l < 1 || l > level[dim])
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "requires 1 <= level <= the grid's level");
    for (auto const &f : filters)
      if (f.first != 0 && f.first != 1)
        throw StatusError(PALIWA_GB_RUNTIME_ERROR,
                          "Filter offset not supported");
    if (empty || lv.empty() || filters.empty()) return;
    size_t const es = dtype_size(dtype);
    if (grid == nullptr || reinterpret_cast<uintptr_t>(grid) % es != 0)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "grid is null or misaligned");
    long long const period = 1LL << L;
    long long const sp = 1LL << (L - level[dim]);
    long long const wf = window_front[dim];
    long long const wl = wf + (window_extents[dim] - 1) * sp;  // last uid
    int log2_sp = 0;
    while ((1LL << log2_sp) < sp) ++log2_sp;
    p.log2_spacing = log2_sp;
    p.period = period;
    p.wfront = wf;
    long long others = 1;
    for (int d = 0; d < ndim; ++d)
      if (d != dim) others *= p.oext[d];
    bool const exact = exact_scalers([&] {
      std::vector<Filter> v;
      for (auto const &f : filters)
        v.push_back({f.first, {f.second[0], f.second[1], f.second[2]}});
      return v;
    }());
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    // lifting_pass<CheckBounds = true> (paliwa_transform.hpp:24-51): a point
    // of the pass's lattice is written when it and both periodic
    // neighbours lie in the window. Along the axis those points are the
    // lattice points of [wf + d, wl - d] (neighbours at distance d), plus
    // uid 0 (lower neighbour period - d) and uid period - d (upper
    // neighbour 0) when the window holds their wrapped neighbours; both sit
    // at the ends of that range, so every pass writes one run.
    for (long l : lv) {
      long long const d = 1LL << (L - l);
      long long const step = 2 * d;
      p.s = d;
      for (auto const &f : filters) {
        long long const off = f.first * d;  // the lattice {off + k step}
        auto up_to = [&](long long x) {      // largest lattice point <= x
          return x - floor_mod(x - off, step);
        };
        auto from = [&](long long x) {       // smallest lattice point >= x
          return x + floor_mod(off - x, step);
        };
        long long lo = from(wf + d), hi = up_to(wl - d);
        auto inside = [&](long long x) { return x >= wf && x <= wl; };
        if (off == 0 && inside(0) && inside(period - d) && inside(d))
          lo = 0;  // uid 0 (only reached from the first point)
        if (off + (period / step - 1) * step == period - d &&
            inside(period - d) && inside(period - 2 * d) && inside(0))
          hi = period - d;
        if (hi < lo) continue;
        p.first = lo;
        p.step = step;
        p.count = (hi - lo) / step + 1;
        p.oext[dim] = p.count;
        p.total = p.count * others;
        double const *c = f.second.data();
        p.c = Coeffs{c[0], c[1], c[2], static_cast<float>(c[0]),
                     static_cast<float>(c[1]), static_cast<float>(c[2])};
        launch_out_pass(dtype, exact, p, s);
      }
    }
  });
}
