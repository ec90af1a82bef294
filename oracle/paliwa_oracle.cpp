// C entry points of the CPU oracle, loaded by tests/ and bench.py through
// ctypes. TEST INFRASTRUCTURE ONLY: see paliwa_oracle.hpp.
#include "paliwa_oracle.hpp"

#include <cstdio>
#include <string>

namespace {
thread_local std::string last_error;

template <typename F> int guarded(F &&f) {
  try {
    f();
    return 0;
  } catch (std::invalid_argument const &e) {
    last_error = e.what();
    return 1;
  } catch (std::out_of_range const &e) {
    last_error = e.what();
    return 3;
  } catch (std::exception const &e) {
    last_error = e.what();
    return 2;
  }
}

paliwa_oracle::Shape make_shape(int ndim, long const *level,
                                long const *maximum_level) {
  if (ndim < 1 || ndim > 16)
    throw std::invalid_argument("ndim must be in [1, 16]");
  paliwa_oracle::Shape s;
  s.ndim = ndim;
  for (int d = 0; d < ndim; ++d) {
    if (level[d] < 0 || level[d] > 40 || maximum_level[d] < level[d])
      throw std::invalid_argument("requires 0 <= level <= maximum_level");
    s.level[d] = level[d];
    s.maximum_level[d] = maximum_level[d];
  }
  return s;
}

paliwa_oracle::Filters make_filters(int const *offsets, double const *coeffs,
                                    int npasses) {
  paliwa_oracle::Filters f;
  for (int p = 0; p < npasses; ++p)
    f.push_back({offsets[p], {coeffs[3 * p], coeffs[3 * p + 1],
                              coeffs[3 * p + 2]}});
  return f;
}
} // namespace

extern "C" {

char const *oracle_last_error() { return last_error.c_str(); }

int oracle_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// transform_in over one dimension with explicit levels and filters
// (paliwa/paliwa_transform.hpp:215-251). dtype 0 = double, 1 = float.
int oracle_transform_in(void *grid, int dtype, int ndim, long const *level,
                        long const *maximum_level, int dim, long const *levels,
                        int nlevels, int const *offsets, double const *coeffs,
                        int npasses, int mode) {
  return guarded([&] {
    auto const shape = make_shape(ndim, level, maximum_level);
    if (dim < 0 || dim >= ndim) throw std::invalid_argument("bad dim");
    std::vector<long> lv(levels, levels + nlevels);
    auto const filters = make_filters(offsets, coeffs, npasses);
    auto const m = static_cast<paliwa_oracle::Mode>(mode);
    if (dtype == 0)
      paliwa_oracle::transform_in(static_cast<double *>(grid), shape, dim, lv,
                                  filters, m);
    else
      paliwa_oracle::transform_in(static_cast<float *>(grid), shape, dim, lv,
                                  filters, m);
  });
}

// transform_in over one dimension of a chunk holding a window of the level
// lattice (front uids, extents): the reference's checked lifting passes.
int oracle_transform_in_window(void *grid, int dtype, int ndim,
                               long const *level, long const *maximum_level,
                               long const *front, long const *extents, int dim,
                               long const *levels, int nlevels,
                               int const *offsets, double const *coeffs,
                               int npasses) {
  return guarded([&] {
    auto const shape = make_shape(ndim, level, maximum_level);
    if (dim < 0 || dim >= ndim) throw std::invalid_argument("bad dim");
    for (int d = 0; d < ndim; ++d)
      if (extents[d] < 0 || front[d] < 0 ||
          front[d] % (1L << (maximum_level[d] - level[d])) != 0)
        throw std::invalid_argument("window off the level lattice");
    std::vector<long> lv(levels, levels + nlevels);
    auto const filters = make_filters(offsets, coeffs, npasses);
    if (dtype == 0)
      paliwa_oracle::transform_in_window(static_cast<double *>(grid), shape,
                                         front, extents, dim, lv, filters);
    else
      paliwa_oracle::transform_in_window(static_cast<float *>(grid), shape,
                                         front, extents, dim, lv, filters);
  });
}

// hierarchize / dehierarchize over all dimensions
// (paliwa/paliwa_transform.hpp:401-431).
int oracle_hierarchize(void *grid, int dtype, int ndim, long const *level,
                       long const *minimum_level, long const *maximum_level,
                       int wavelet, int forward, int mode) {
  return guarded([&] {
    auto const shape = make_shape(ndim, level, maximum_level);
    auto const m = static_cast<paliwa_oracle::Mode>(mode);
    if (dtype == 0)
      paliwa_oracle::hierarchize(static_cast<double *>(grid), shape,
                                 minimum_level, wavelet, forward != 0, m);
    else
      paliwa_oracle::hierarchize(static_cast<float *>(grid), shape,
                                 minimum_level, wavelet, forward != 0, m);
  });
}

} // extern "C"
