// C entry points over the reference's own headers -- TEST INFRASTRUCTURE.
//
// Built by `make -C oracle ref` into oracle/_ref/libpaliwa_ref.so from the
// unmodified paliwa headers where they lie (include path = the reference
// checkout), against the serial DDC/Kokkos stand-ins in oracle/ref_shim/.
// The CPU tests load it through oracle/reference.py to hold the oracle's
// restatement (paliwa_oracle.hpp, oracle.py, restricted.py) equal to the
// reference itself. Nothing on the product path or on the GPU machine uses it
// (the reference sources are not there).
//
// Grids are dense row-major arrays over the given domain, as a ddc::Chunk
// over a StridedDiscreteDomain stores them. Dimensions use the reference's
// own tags (paliwa_dimensions.hpp), up to six.
#include <Kokkos_Core.hpp>
#include <ddc/ddc.hpp>

#include <paliwa/paliwa_dimensions.hpp>
#include <paliwa/paliwa_transform.hpp>
#include <paliwa/paliwa_utils.hpp>

#include <array>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

thread_local std::string g_error;

template <typename F> int guarded(F &&f) {
  try {
    f();
    return 0;
  } catch (std::invalid_argument const &e) {
    g_error = e.what();
    return 1;
  } catch (std::out_of_range const &e) {
    g_error = e.what();
    return 3;
  } catch (std::exception const &e) {
    g_error = e.what();
    return 2;
  }
}

template <class... D> struct Dims {};

template <class F> void with_dims(int ndim, F &&f) {
  using namespace paliwa;
  switch (ndim) {
  case 1: return f(Dims<DDimA>{});
  case 2: return f(Dims<DDimA, DDimB>{});
  case 3: return f(Dims<DDimA, DDimB, DDimC>{});
  case 4: return f(Dims<DDimA, DDimB, DDimC, DDimD>{});
  case 5: return f(Dims<DDimA, DDimB, DDimC, DDimD, DDimE>{});
  case 6: return f(Dims<DDimA, DDimB, DDimC, DDimD, DDimE, DDimF>{});
  }
  throw std::invalid_argument("ndim must be in [1, 6]");
}

// Calls f(Tag{}) for the dim-th tag of D...
template <class... D, class F> void with_dim(int dim, F &&f) {
  int i = 0;
  bool done = false;
  ((i++ == dim ? (f(D{}), done = true) : false), ...);
  if (!done) throw std::invalid_argument("bad dim");
}

template <std::size_t N> std::array<long, N> arr(long const *p) {
  std::array<long, N> a{};
  for (std::size_t i = 0; i < N; ++i) a[i] = p[i];
  return a;
}

using Filters = std::vector<std::pair<int, std::array<double, 3>>>;

Filters make_filters(int const *offsets, double const *coeffs, int n) {
  Filters f;
  for (int p = 0; p < n; ++p)
    f.push_back({offsets[p], {coeffs[3 * p], coeffs[3 * p + 1],
                              coeffs[3 * p + 2]}});
  return f;
}

// The grid's domain: the full level lattice, or a window of it (front uids,
// extents) when `front` is given.
template <class... D>
ddc::StridedDiscreteDomain<D...> grid_domain(long const *level,
                                             long const *maximum_level,
                                             long const *front,
                                             long const *extents) {
  constexpr std::size_t N = sizeof...(D);
  auto const full = paliwa::strided_domain_from_level<D...>(
      arr<N>(level), arr<N>(maximum_level));
  if (front == nullptr) return full;
  return ddc::StridedDiscreteDomain<D...>(ddc::DiscreteElement<D...>(arr<N>(front)),
                                          ddc::DiscreteVector<D...>(arr<N>(extents)),
                                          full.strides());
}

template <class T, class... D>
void hierarchize_impl(Dims<D...>, T *data, long const *level,
                      long const *minimum_level, long const *maximum_level,
                      char const *wavelet, bool forward) {
  constexpr std::size_t N = sizeof...(D);
  ddc::DiscreteVector<D...> const lv(arr<N>(level)), mn(arr<N>(minimum_level)),
      mx(arr<N>(maximum_level));
  for (std::size_t i = 0; i < N; ++i)
    if (!(minimum_level[i] >= 0 && minimum_level[i] <= level[i] &&
          level[i] <= maximum_level[i]))
      throw std::invalid_argument("requires 0 <= lmin <= level <= lmax");
  ddc::ChunkSpan<T, ddc::StridedDiscreteDomain<D...>> span(
      data, grid_domain<D...>(level, maximum_level, nullptr, nullptr));
  if (forward)
    paliwa::hierarchize(span, lv, mn, mx, std::string(wavelet),
                        Kokkos::Serial{});
  else
    paliwa::dehierarchize(span, lv, mn, mx, std::string(wavelet),
                          Kokkos::Serial{});
}

template <class T, class... D>
void transform_in_impl(Dims<D...>, T *data, long const *level,
                       long const *maximum_level, long const *front,
                       long const *extents, int dim,
                       std::vector<long> const &levels,
                       Filters const &filters) {
  constexpr std::size_t N = sizeof...(D);
  ddc::DiscreteVector<D...> const lv(arr<N>(level)), mx(arr<N>(maximum_level));
  ddc::ChunkSpan<T, ddc::StridedDiscreteDomain<D...>> span(
      data, grid_domain<D...>(level, maximum_level, front, extents));
  with_dim<D...>(dim, [&](auto tag) {
    using Dim = decltype(tag);
    paliwa::transform_in<Dim>(span, lv, mx, levels, filters, Kokkos::Serial{});
  });
}

template <class T, class... D>
void transform_outputs_impl(Dims<D...>, T *data, long const *level,
                            long const *maximum_level, long const *front,
                            long const *extents, int dim,
                            std::vector<long> const &levels,
                            Filters const &filters, long const *out_front,
                            long const *out_extents, long const *out_strides,
                            int pole_execution) {
  constexpr std::size_t N = sizeof...(D);
  ddc::DiscreteVector<D...> const lv(arr<N>(level)), mx(arr<N>(maximum_level));
  ddc::ChunkSpan<T, ddc::StridedDiscreteDomain<D...>> span(
      data, grid_domain<D...>(level, maximum_level, front, extents));
  ddc::StridedDiscreteDomain<D...> const outputs(
      ddc::DiscreteElement<D...>(arr<N>(out_front)),
      ddc::DiscreteVector<D...>(arr<N>(out_extents)),
      ddc::DiscreteVector<D...>(arr<N>(out_strides)));
  with_dim<D...>(dim, [&](auto tag) {
    using Dim = decltype(tag);
    paliwa::transform_in<Dim>(span, lv, mx, levels, filters, outputs,
                              Kokkos::Serial{},
                              static_cast<paliwa::PoleExecution>(pole_execution));
  });
}

} // namespace

extern "C" {

char const *ref_last_error() { return g_error.c_str(); }

// paliwa::hierarchize / dehierarchize (paliwa_transform.hpp:401-431).
// dtype 0 = double, 1 = float.
int ref_hierarchize(void *grid, int dtype, int ndim, long const *level,
                    long const *minimum_level, long const *maximum_level,
                    char const *wavelet, int forward) {
  return guarded([&] {
    with_dims(ndim, [&](auto dims) {
      if (dtype == 0)
        hierarchize_impl(dims, static_cast<double *>(grid), level,
                         minimum_level, maximum_level, wavelet, forward != 0);
      else
        hierarchize_impl(dims, static_cast<float *>(grid), level,
                         minimum_level, maximum_level, wavelet, forward != 0);
    });
  });
}

// paliwa::transform_in<Dim> full-grid overload (paliwa_transform.hpp:215-251)
// on the full lattice (front == NULL) or on a window of it (the CheckBounds
// path of lifting_pass).
int ref_transform_in(void *grid, int dtype, int ndim, long const *level,
                     long const *maximum_level, long const *front,
                     long const *extents, int dim, long const *levels,
                     int nlevels, int const *offsets, double const *coeffs,
                     int npasses) {
  return guarded([&] {
    std::vector<long> const lv(levels, levels + nlevels);
    auto const f = make_filters(offsets, coeffs, npasses);
    with_dims(ndim, [&](auto dims) {
      if (dtype == 0)
        transform_in_impl(dims, static_cast<double *>(grid), level,
                          maximum_level, front, extents, dim, lv, f);
      else
        transform_in_impl(dims, static_cast<float *>(grid), level,
                          maximum_level, front, extents, dim, lv, f);
    });
  });
}

// paliwa::transform_in<Dim> restricted-output overload
// (paliwa_transform.hpp:333-344) on a window buffer; pole_execution 0 Direct,
// 1 PackedPasses, 2 PackedPoles.
int ref_transform_outputs(void *grid, int dtype, int ndim, long const *level,
                          long const *maximum_level, long const *front,
                          long const *extents, int dim, long const *levels,
                          int nlevels, int const *offsets, double const *coeffs,
                          int npasses, long const *out_front,
                          long const *out_extents, long const *out_strides,
                          int pole_execution) {
  return guarded([&] {
    std::vector<long> const lv(levels, levels + nlevels);
    auto const f = make_filters(offsets, coeffs, npasses);
    with_dims(ndim, [&](auto dims) {
      if (dtype == 0)
        transform_outputs_impl(dims, static_cast<double *>(grid), level,
                               maximum_level, front, extents, dim, lv, f,
                               out_front, out_extents, out_strides,
                               pole_execution);
      else
        transform_outputs_impl(dims, static_cast<float *>(grid), level,
                               maximum_level, front, extents, dim, lv, f,
                               out_front, out_extents, out_strides,
                               pole_execution);
    });
  });
}

// paliwa::transform_bounds (paliwa_domains.hpp:365-434): bounds receives
// 2 * (level + 1) values, writes 2 * nlevels * nfilters (the visited write
// bounds per (level index, pass)).
int ref_transform_bounds(long outputs_min, long outputs_max, long level,
                         long maximum_level, long const *levels, int nlevels,
                         int const *offsets, int nfilters, long *bounds,
                         long *writes) {
  return guarded([&] {
    std::vector<long> const lv(levels, levels + nlevels);
    Filters f;
    for (int p = 0; p < nfilters; ++p) f.push_back({offsets[p], {0, 1, 0}});
    auto const b = paliwa::transform_bounds(
        paliwa::PeriodicBounds{outputs_min, outputs_max}, level, maximum_level,
        lv, f, [&](std::size_t i, std::size_t pass, paliwa::PeriodicBounds w) {
          if (writes) {
            writes[2 * (i * nfilters + pass)] = w.min;
            writes[2 * (i * nfilters + pass) + 1] = w.max;
          }
        });
    for (std::size_t l = 0; l < b.size(); ++l) {
      bounds[2 * l] = b[l].min;
      bounds[2 * l + 1] = b[l].max;
    }
  });
}

// paliwa::covering_periodic_bounds (paliwa_domains.hpp:471-485).
int ref_covering_periodic_bounds(long const *indices, int n, long period,
                                 long *out) {
  return guarded([&] {
    auto const b = paliwa::covering_periodic_bounds(
        std::vector<long>(indices, indices + n), period);
    out[0] = b.min;
    out[1] = b.max;
  });
}

// paliwa::pole_pass_segments (paliwa_domains.hpp:494-535): up to `capacity`
// segments of 5 ints (first, count, stride, lower, upper); *nsegments = all.
int ref_pole_pass_segments(long wmin, long wmax, long origin, int level,
                           int maximum_level, int pass_level, int capacity,
                           int *nsegments, int *out) {
  return guarded([&] {
    auto const s = paliwa::pole_pass_segments(
        paliwa::PeriodicBounds{wmin, wmax},
        static_cast<ddc::DiscreteElementType>(origin), level, maximum_level,
        pass_level);
    *nsegments = static_cast<int>(s.size());
    for (int i = 0; i < capacity && i < static_cast<int>(s.size()); ++i) {
      out[5 * i] = s[i].first;
      out[5 * i + 1] = s[i].count;
      out[5 * i + 2] = s[i].stride;
      out[5 * i + 3] = s[i].lower;
      out[5 * i + 4] = s[i].upper;
    }
  });
}

// Level index maps (paliwa_domains.hpp:33-83): kind 0 strided_domain_from_level,
// 1 strided_hierarchical_domain_from_level; each of front/extents/strides
// receives ndim values.
int ref_level_domain(int kind, int ndim, long const *level,
                     long const *finest_level, long const *lbound, long *front,
                     long *extents, long *strides) {
  return guarded([&] {
    with_dims(ndim, [&](auto dims) {
      [&]<class... D>(Dims<D...>) {
        constexpr std::size_t N = sizeof...(D);
        ddc::DiscreteElement<D...> const lb(arr<N>(lbound));
        auto const d =
            kind == 0
                ? paliwa::strided_domain_from_level<D...>(
                      arr<N>(level), arr<N>(finest_level), lb)
                : paliwa::strided_hierarchical_domain_from_level<D...>(
                      arr<N>(level), arr<N>(finest_level), lb);
        int i = 0;
        ((front[i] = static_cast<long>(d.front().template uid<D>()),
          extents[i] = d.extents().template get<D>(),
          strides[i] = d.strides().template get<D>(), ++i),
         ...);
      }(dims);
    });
  });
}

// paliwa::restrict_strided_with_discrete (paliwa_domains.hpp:195-214) of a
// strided domain with the box [box_front, box_front + box_extents).
int ref_restrict_strided_with_discrete(int ndim, long const *front,
                                       long const *extents,
                                       long const *strides,
                                       long const *box_front,
                                       long const *box_extents, long *out) {
  return guarded([&] {
    with_dims(ndim, [&](auto dims) {
      [&]<class... D>(Dims<D...>) {
        constexpr std::size_t N = sizeof...(D);
        ddc::StridedDiscreteDomain<D...> const s(
            ddc::DiscreteElement<D...>(arr<N>(front)),
            ddc::DiscreteVector<D...>(arr<N>(extents)),
            ddc::DiscreteVector<D...>(arr<N>(strides)));
        ddc::DiscreteDomain<D...> const box(
            ddc::DiscreteElement<D...>(arr<N>(box_front)),
            ddc::DiscreteVector<D...>(arr<N>(box_extents)));
        auto const r = paliwa::restrict_strided_with_discrete(s, box);
        int i = 0;
        ((out[i] = static_cast<long>(r.front().template uid<D>()),
          out[N + i] = r.extents().template get<D>(),
          out[2 * N + i] = r.strides().template get<D>(), ++i),
         ...);
      }(dims);
    });
  });
}

// paliwa::get_required_transform_domain<Dim> (paliwa_domains.hpp:590-640),
// one dimension: the full axis strided_domain_from_level(level, lmax), the
// local part as the uid box [local_front, local_front + local_extent).
// Writes up to `capacity` ghost uids; *count = all.
int ref_required_transform_domain(int forward, long level, long minimum_level,
                                  long maximum_level, long local_front,
                                  long local_extent, char const *wavelet,
                                  int capacity, long *count, long *out) {
  return guarded([&] {
    using Dim = paliwa::DDimA;
    auto const full = paliwa::strided_domain_from_level<Dim>(
        std::array<long, 1>{level}, std::array<long, 1>{maximum_level});
    ddc::DiscreteDomain<Dim> const local{ddc::DiscreteElement<Dim>(local_front),
                                         ddc::DiscreteVector<Dim>(local_extent)};
    auto const ghosts = paliwa::get_required_transform_domain<Dim>(
        forward != 0, full, local, ddc::DiscreteVector<Dim>(level),
        ddc::DiscreteVector<Dim>(minimum_level),
        ddc::DiscreteVector<Dim>(maximum_level), std::string(wavelet));
    long n = 0;
    for (auto it = ghosts.begin(); it != ghosts.end(); ++it, ++n)
      if (n < capacity) out[n] = static_cast<long>((*it).uid());
    *count = n;
  });
}

// paliwa::initialize_dim_periodic_unit_interval (paliwa_dimensions.hpp:71-79)
// for a resolution of n points: the coordinates of the returned domain.
int ref_periodic_unit_interval(long n, int capacity, long *count,
                               double *coordinates) {
  return guarded([&] {
    struct Tag {};
    using DDim = paliwa::D_Dim<Tag, 7>;
    auto const dom = paliwa::initialize_dim_periodic_unit_interval<DDim>(
        ddc::DiscreteVector<DDim>(n));
    long i = 0;
    ddc::host_for_each(dom, [&](ddc::DiscreteElement<DDim> e) {
      if (i < capacity) coordinates[i] = double(ddc::coordinate(e));
      ++i;
    });
    *count = i;
  });
}

// paliwa::iterate_hierarchical_subspaces (paliwa_utils.hpp:9-26): writes the
// visited level vectors (ndim values each) in visiting order.
int ref_hierarchical_subspaces(int ndim, long const *nodal_level, int capacity,
                               long *count, long *out) {
  return guarded([&] {
    std::vector<long> const nodal(nodal_level, nodal_level + ndim);
    std::vector<long> tmp(ndim, 0);
    long n = 0;
    paliwa::iterate_hierarchical_subspaces<std::vector<long>>(
        nodal, tmp, 0, [&](std::vector<long> const &s) {
          if (n < capacity)
            for (int d = 0; d < ndim; ++d) out[n * ndim + d] = s[d];
          ++n;
        });
    *count = n;
  });
}

// paliwa::restrict_periodic_bounds<DDimA> (paliwa_domains.hpp:539-568) of a
// 2D strided domain: up to 2 parts of 6 values (front, extents, strides).
int ref_restrict_periodic_bounds(long const *front, long const *extents,
                                 long const *strides, long bmin, long bmax,
                                 long period, int *nparts, long *out) {
  return guarded([&] {
    using namespace paliwa;
    ddc::StridedDiscreteDomain<DDimA, DDimB> const d{
        ddc::DiscreteElement<DDimA, DDimB>(front[0], front[1]),
        ddc::DiscreteVector<DDimA, DDimB>(extents[0], extents[1]),
        ddc::DiscreteVector<DDimA, DDimB>(strides[0], strides[1])};
    auto const parts = paliwa::restrict_periodic_bounds<DDimA>(
        d, paliwa::PeriodicBounds{bmin, bmax}, period);
    *nparts = static_cast<int>(parts.size());
    for (std::size_t i = 0; i < parts.size() && i < 2; ++i) {
      auto const &p = parts[i];
      long *o = out + 6 * i;
      o[0] = static_cast<long>(p.front().template uid<DDimA>());
      o[1] = static_cast<long>(p.front().template uid<DDimB>());
      o[2] = p.extents().template get<DDimA>();
      o[3] = p.extents().template get<DDimB>();
      o[4] = p.strides().template get<DDimA>();
      o[5] = p.strides().template get<DDimB>();
    }
  });
}

// paliwa::for_each_transform_index (paliwa_domains.hpp:437-450): the visited
// uids of per-level bounds (2 * nb values).
int ref_for_each_transform_index(long const *bounds, int nb,
                                 long maximum_level, int capacity, long *count,
                                 long *out) {
  return guarded([&] {
    std::vector<paliwa::PeriodicBounds> b(nb);
    for (int i = 0; i < nb; ++i) b[i] = {bounds[2 * i], bounds[2 * i + 1]};
    long n = 0;
    paliwa::for_each_transform_index<paliwa::DDimA>(
        b, maximum_level, [&](ddc::DiscreteElement<paliwa::DDimA> e) {
          if (n < capacity) out[n] = static_cast<long>(e.uid());
          ++n;
        });
    *count = n;
  });
}

} // extern "C"
