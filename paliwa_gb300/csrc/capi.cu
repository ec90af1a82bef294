// C ABI of paliwa_gb300: single-grid transforms (include/paliwa_gb300.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "paliwa_gb300.h"
#include "plan.hpp"

namespace pgb {

thread_local std::string g_last_error;

std::vector<Filter> wavelet_filters(int wavelet, bool forward) {
  // paliwa/paliwa_wavelets.hpp:17-20 (forward) and :24-27 (inverse).
  switch (wavelet) {
  case PALIWA_GB_HAT:
    if (forward) return {{1, {-0.5, 1.0, -0.5}}};
    return {{1, {0.5, 1.0, 0.5}}};
  case PALIWA_GB_BIORTHOGONAL:
    if (forward) return {{1, {-0.5, 1.0, -0.5}}, {0, {0.25, 1.0, 0.25}}};
    return {{0, {-0.25, 1.0, -0.25}}, {1, {0.5, 1.0, 0.5}}};
  case PALIWA_GB_FULLWEIGHTING:
    if (forward) return {{0, {0.25, 0.5, 0.25}}, {1, {-0.5, 1.0, -0.5}}};
    return {{1, {0.5, 1.0, 0.5}}, {0, {-0.5, 2.0, -0.5}}};
  }
  throw StatusError(PALIWA_GB_OUT_OF_RANGE, "unknown wavelet id");
}

// True when every coefficient is 0 or +-2^k with a product that stays exact
// in both float and double, so fused multiply-adds round like the
// reference's separate multiplies and adds.
bool exact_scalers(std::vector<Filter> const &filters) {
  for (auto const &f : filters)
    for (double c : f.c) {
      if (c == 0.0) continue;
      int e = 0;
      double const m = std::frexp(c, &e);
      if (std::fabs(m) != 0.5 || e < -60 || e > 60) return false;
    }
  return true;
}

int chunk_for(int log2_n) {
  if (log2_n <= 4) return 1 << log2_n;  // whole pencil in one thread
  if (log2_n <= 12) return 16;
  return 32;                              // 8192-point pencils
}

namespace {

long long ceil_div(long long a, long long b) { return (a + b - 1) / b; }

void fill_job(LiftJob &job, AxisView const &v, std::vector<int> const &sh,
              size_t first, size_t count) {
  job.offset = v.offset;
  job.columns = v.columns;
  job.tile_begin = 0;
  job.log2_inner = v.log2_inner;
  job.log2_kstride = v.log2_kstride;
  job.log2_astride = v.log2_astride;
  job.log2_n = v.log2_n;
  job.seg_len = 0;
  job.halo = 0;
  job.nlevels = static_cast<int>(count);
  for (size_t i = 0; i < count; ++i)
    job.shift[i] = static_cast<signed char>(sh[first + i]);
}

// Periodic whole-pencil launches; level lists longer than one job holds are
// split into consecutive launches (order preserved).
void plan_periodic(AxisView const &v, std::vector<int> const &shifts,
                   LaunchPlan const &proto, std::vector<LaunchPlan> &out) {
  int const R = chunk_for(v.log2_n);
  int const log2G = v.log2_n - (31 - __builtin_clz(R));
  long long const C = kThreads >> log2G;
  for (size_t first = 0; first < shifts.size(); first += kMaxLevels) {
    size_t const count =
        std::min(shifts.size() - first, static_cast<size_t>(kMaxLevels));
    LaunchPlan lp = proto;
    lp.R = R;
    lp.params.periodic = 1;
    lp.params.log2_window = v.log2_n;
    fill_job(lp.params.job, v, shifts, first, count);
    lp.params.job.col_tiles = ceil_div(v.columns, C);
    lp.tiles = lp.params.job.col_tiles;
    out.push_back(lp);
  }
}

// Fine levels of a long pencil on overlapping windows.
void plan_windows(AxisView const &v, std::vector<int> const &shifts,
                  std::vector<Filter> const &filters, LaunchPlan const &proto,
                  std::vector<LaunchPlan> &out) {
  long long const window = 1LL << kWindowLog2;
  int const R = 32;
  size_t first = 0;
  while (first < shifts.size()) {
    // Grow the run while the halo it needs fits the window.
    long long reach = 0;
    size_t count = 0;
    while (first + count < shifts.size() && count < kMaxLevels) {
      long long const add =
          static_cast<long long>(filters.size()) << shifts[first + count];
      long long const halo = ceil_div(reach + add, R) * R;
      if (2 * halo > window / 2 && count > 0) break;
      reach += add;
      ++count;
    }
    long long const halo = ceil_div(reach, R) * R;
    long long const seg_len = window - 2 * halo;
    if (seg_len <= 0)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "filter list too long for windowed long pencils");
    LaunchPlan lp = proto;
    lp.R = R;
    lp.params.periodic = 0;
    lp.params.log2_window = kWindowLog2;
    fill_job(lp.params.job, v, shifts, first, count);
    lp.params.job.seg_len = static_cast<int>(seg_len);
    lp.params.job.halo = static_cast<int>(halo);
    lp.params.job.col_tiles = v.columns;  // one column per CTA
    lp.tiles = ceil_div(1LL << v.log2_n, seg_len) * v.columns;
    out.push_back(lp);
    first += count;
  }
}

} // namespace

void plan_axis(AxisView const &view, std::vector<int> const &shifts,
               std::vector<Filter> const &filters, LaunchPlan const &proto,
               std::vector<LaunchPlan> &out) {
  if (shifts.empty() || filters.empty() || view.log2_n == 0) return;
  if (view.log2_n <= kWindowLog2) {
    plan_periodic(view, shifts, proto, out);
    return;
  }
  // Long pencil: levels closer than 2^m run on windows with a halo of at most
  // kHaloBudget points per side; the others run on the sub-lattice of every
  // 2^m-th point, which is a periodic pencil 2^m times shorter.
  int const P = static_cast<int>(filters.size());
  int m = 0;
  while (static_cast<long long>(P) * ((2LL << m) - 1) <= kHaloBudget) ++m;
  if (m < 1) m = 1;
  size_t i = 0;
  while (i < shifts.size()) {
    bool const fine = shifts[i] < m;
    size_t j = i;
    while (j < shifts.size() && (shifts[j] < m) == fine) ++j;
    std::vector<int> run(shifts.begin() + i, shifts.begin() + j);
    if (fine) {
      plan_windows(view, run, filters, proto, out);
    } else {
      AxisView sub = view;
      sub.log2_n = view.log2_n - m;
      sub.log2_kstride = view.log2_kstride + m;
      for (int &s : run) s -= m;
      plan_axis(sub, run, filters, proto, out);
    }
    i = j;
  }
}

} // namespace pgb

using namespace pgb;

namespace {

template <typename F> int guarded(F &&f) {
  try {
    f();
    return PALIWA_GB_OK;
  } catch (StatusError const &e) {
    g_last_error = e.what();
    return e.code;
  } catch (std::exception const &e) {
    g_last_error = e.what();
    return PALIWA_GB_RUNTIME_ERROR;
  }
}

void cuda_check(cudaError_t e, char const *what) {
  if (e != cudaSuccess)
    throw StatusError(PALIWA_GB_CUDA_ERROR,
                      std::string(what) + ": " + cudaGetErrorString(e));
}

template <class A>
void launch_one(LaunchPlan const &lp, cudaStream_t s) {
  dim3 const grid(static_cast<unsigned>(lp.tiles));
  switch (lp.R) {
  case 1: return;  // pencils of one point: nothing to do
  case 2: lift_kernel<A, 2, kThreads><<<grid, kThreads, 0, s>>>(lp.params); break;
  case 4: lift_kernel<A, 4, kThreads><<<grid, kThreads, 0, s>>>(lp.params); break;
  case 8: lift_kernel<A, 8, kThreads><<<grid, kThreads, 0, s>>>(lp.params); break;
  case 16: lift_kernel<A, 16, kThreads><<<grid, kThreads, 0, s>>>(lp.params); break;
  case 32: lift_kernel<A, 32, kThreads><<<grid, kThreads, 0, s>>>(lp.params); break;
  default: throw StatusError(PALIWA_GB_RUNTIME_ERROR, "bad chunk size");
  }
  cuda_check(cudaGetLastError(), "lift_kernel launch");
}

void launch(int dtype, bool exact, LaunchPlan const &lp, cudaStream_t s) {
  if (lp.tiles <= 0) return;
  if (lp.tiles > 0x7fffffffLL)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "grid too large");
  switch (dtype) {
  case PALIWA_GB_F64:
    if (exact) return launch_one<Plain<double, true>>(lp, s);
    return launch_one<Plain<double, false>>(lp, s);
  case PALIWA_GB_F32:
    if (exact) return launch_one<Plain<float, true>>(lp, s);
    return launch_one<Plain<float, false>>(lp, s);
  case PALIWA_GB_F32C:
    return launch_one<Compensated>(lp, s);
  }
  throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "unknown dtype");
}

size_t dtype_size(int dtype) {
  switch (dtype) {
  case PALIWA_GB_F64: return 8;
  case PALIWA_GB_F32:
  case PALIWA_GB_F32C: return 4;
  }
  throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "unknown dtype");
}

void check_shape(void *grid, int dtype, int ndim, int64_t const *level,
                 int64_t const *maximum_level) {
  dtype_size(dtype);
  if (grid == nullptr)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "grid is null");
  if (ndim < 1 || ndim > 32)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "ndim must be in [1, 32]");
  long long total = 0;
  for (int d = 0; d < ndim; ++d) {
    if (level[d] < 0 || level[d] > 40)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "level out of range");
    if (maximum_level != nullptr && maximum_level[d] < level[d])
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "level must not exceed maximum_level");
    total += level[d];
  }
  if (total > 40)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "grid too large");
}

AxisView axis_view(int ndim, int64_t const *level, int dim) {
  AxisView v;
  int log2_outer = 0, log2_inner = 0;
  for (int d = 0; d < dim; ++d) log2_outer += static_cast<int>(level[d]);
  for (int d = dim + 1; d < ndim; ++d) log2_inner += static_cast<int>(level[d]);
  v.offset = 0;
  v.columns = 1LL << (log2_outer + log2_inner);
  v.log2_inner = log2_inner;
  v.log2_kstride = log2_inner;
  v.log2_n = static_cast<int>(level[dim]);
  v.log2_astride = v.log2_n + log2_inner;
  return v;
}

LaunchPlan prototype(void *grid, std::vector<Filter> const &filters) {
  if (filters.size() > static_cast<size_t>(kMaxPasses))
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "at most 8 filter passes");
  LaunchPlan lp;
  std::memset(&lp.params, 0, sizeof(lp.params));
  lp.params.data = grid;
  lp.params.jobs = nullptr;
  lp.params.njobs = 1;
  lp.params.vec_ok = (reinterpret_cast<uintptr_t>(grid) % 16) == 0;
  lp.params.npasses = static_cast<int>(filters.size());
  lp.params.fp64_log2_points = 2;
  for (size_t p = 0; p < filters.size(); ++p) {
    if (filters[p].offset != 0 && filters[p].offset != 1)
      throw StatusError(PALIWA_GB_RUNTIME_ERROR, "Filter offset not supported");
    lp.params.offsets[p] = filters[p].offset;
    lp.params.coeffs[p] = {filters[p].c[0], filters[p].c[1], filters[p].c[2]};
    if (filters[p].c[1] == 1.0) lp.params.c1_one_mask |= 1u << p;
  }
  return lp;
}

void transform_axis(void *grid, int dtype, int ndim, int64_t const *level,
                    int dim, std::vector<int> const &shifts,
                    std::vector<Filter> const &filters, cudaStream_t s) {
  LaunchPlan const proto = prototype(grid, filters);
  std::vector<LaunchPlan> plans;
  plan_axis(axis_view(ndim, level, dim), shifts, filters, proto, plans);
  bool const exact = exact_scalers(filters);
  for (auto const &lp : plans) launch(dtype, exact, lp, s);
}

std::vector<int> level_shifts(int64_t lev, int64_t lmin, bool forward) {
  std::vector<int> sh;
  // hierarchize_in: levels lev .. lmin+1 (paliwa_transform.hpp:364-367);
  // dehierarchize_in: lmin+1 .. lev (:392-394). shift = lev - l.
  for (int64_t l = lmin + 1; l <= lev; ++l)
    sh.push_back(static_cast<int>(lev - l));
  // sh now follows increasing levels (the inverse order).
  if (forward) std::reverse(sh.begin(), sh.end());
  return sh;
}

void check_levels(int ndim, int64_t const *level, int64_t const *lmin,
                  int64_t const *lmax) {
  // paliwa/paliwa_transform.hpp:359-362 (asserted there).
  for (int d = 0; d < ndim; ++d)
    if (lmin[d] < 0 || lmin[d] > level[d] || level[d] > lmax[d])
      throw StatusError(
          PALIWA_GB_INVALID_ARGUMENT,
          "requires 0 <= minimum_level <= level <= maximum_level");
}

int hierarchize_dims(void *grid, int dtype, int ndim, int64_t const *level,
                     int64_t const *lmin, int64_t const *lmax, int dim_begin,
                     int dim_end, int wavelet, bool forward, void *stream) {
  return guarded([&] {
    check_shape(grid, dtype, ndim, level, lmax);
    check_levels(ndim, level, lmin, lmax);
    if (dim_begin < 0 || dim_end > ndim || dim_begin >= dim_end)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "bad dimension");
    auto const filters = wavelet_filters(wavelet, forward);
    for (int d = dim_begin; d < dim_end; ++d)
      transform_axis(grid, dtype, ndim, level, d,
                     level_shifts(level[d], lmin[d], forward), filters,
                     static_cast<cudaStream_t>(stream));
  });
}

} // namespace

extern "C" {

const char *paliwa_gb_last_error(void) { return g_last_error.c_str(); }

int paliwa_gb_version(void) { return 100; }

int paliwa_gb_wavelet_id(const char *name, int *id) {
  return guarded([&] {
    if (name == nullptr || id == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    std::string const n(name);
    if (n == "hat") *id = PALIWA_GB_HAT;
    else if (n == "biorthogonal") *id = PALIWA_GB_BIORTHOGONAL;
    else if (n == "fullweighting") *id = PALIWA_GB_FULLWEIGHTING;
    else throw StatusError(PALIWA_GB_OUT_OF_RANGE, "unknown wavelet: " + n);
  });
}

int paliwa_gb_wavelet_filters(int wavelet, int direction, int *npasses,
                              int32_t *offsets, double *coefficients) {
  return guarded([&] {
    auto const f = wavelet_filters(wavelet, direction > 0);
    *npasses = static_cast<int>(f.size());
    for (size_t p = 0; p < f.size(); ++p) {
      offsets[p] = f[p].offset;
      for (int k = 0; k < 3; ++k) coefficients[3 * p + k] = f[p].c[k];
    }
  });
}

int paliwa_gb_transform_in(void *grid, int dtype, int ndim,
                           const int64_t *level, const int64_t *maximum_level,
                           int dim, const int64_t *levels, int nlevels,
                           const int32_t *offsets, const double *coefficients,
                           int npasses, void *stream) {
  return guarded([&] {
    check_shape(grid, dtype, ndim, level, maximum_level);
    if (dim < 0 || dim >= ndim)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "bad dimension");
    if (npasses < 0 || nlevels < 0)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "negative count");
    std::vector<Filter> filters;
    for (int p = 0; p < npasses; ++p)
      filters.push_back({offsets[p],
                         {coefficients[3 * p], coefficients[3 * p + 1],
                          coefficients[3 * p + 2]}});
    for (auto const &f : filters)  // paliwa_transform.hpp:239-240
      if (f.offset != 0 && f.offset != 1)
        throw StatusError(PALIWA_GB_RUNTIME_ERROR,
                          "Filter offset not supported");
    std::vector<int> shifts;
    for (int i = 0; i < nlevels; ++i) {
      if (levels[i] < 1 || levels[i] > level[dim])  // :232 asserts l > 0
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "transform level out of range");
      shifts.push_back(static_cast<int>(level[dim] - levels[i]));
    }
    transform_axis(grid, dtype, ndim, level, dim, shifts, filters,
                   static_cast<cudaStream_t>(stream));
  });
}

int paliwa_gb_hierarchize_in(void *grid, int dtype, int ndim,
                             const int64_t *level, const int64_t *lmin,
                             const int64_t *lmax, int dim, int wavelet,
                             void *stream) {
  return hierarchize_dims(grid, dtype, ndim, level, lmin, lmax, dim, dim + 1,
                          wavelet, true, stream);
}

int paliwa_gb_dehierarchize_in(void *grid, int dtype, int ndim,
                               const int64_t *level, const int64_t *lmin,
                               const int64_t *lmax, int dim, int wavelet,
                               void *stream) {
  return hierarchize_dims(grid, dtype, ndim, level, lmin, lmax, dim, dim + 1,
                          wavelet, false, stream);
}

int paliwa_gb_hierarchize(void *grid, int dtype, int ndim,
                          const int64_t *level, const int64_t *lmin,
                          const int64_t *lmax, int wavelet, void *stream) {
  return hierarchize_dims(grid, dtype, ndim, level, lmin, lmax, 0, ndim,
                          wavelet, true, stream);
}

int paliwa_gb_dehierarchize(void *grid, int dtype, int ndim,
                            const int64_t *level, const int64_t *lmin,
                            const int64_t *lmax, int wavelet, void *stream) {
  return hierarchize_dims(grid, dtype, ndim, level, lmin, lmax, 0, ndim,
                          wavelet, false, stream);
}

} // extern "C"
