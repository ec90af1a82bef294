// Drop-in C++ API test: the reference's call shapes
//   paliwa::hierarchize(span, level, lmin, lmax, "biorthogonal", instance)
// over a ChunkSpan of device memory, checked bit for bit against the CPU
// oracle (test infrastructure). Without a GPU it only exercises the argument
// errors, which map to the reference's exception types.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <limits>
#include <random>
#include <stdexcept>
#include <vector>

#include <paliwa/paliwa_dimensions.hpp>
#include <paliwa/paliwa_domains.hpp>
#include <paliwa/paliwa_io.hpp>
#include <paliwa/paliwa_transform.hpp>
#include <paliwa/paliwa_utils.hpp>
#include <paliwa/paliwa_wavelets.hpp>

#include "paliwa_oracle.hpp"

struct X {};
struct Y {};
struct Z {};

#define EXPECT(cond)                                                         \
  do {                                                                       \
    if (!(cond)) {                                                           \
      std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
      return 1;                                                              \
    }                                                                        \
  } while (0)

template <class E, class F> bool throws(F &&f) {
  try {
    f();
  } catch (E const &) {
    return true;
  } catch (...) {
    return false;
  }
  return false;
}

int main() {
  using Vec = ddc::DiscreteVector<X, Y, Z>;
  using Dom = ddc::StridedDiscreteDomain<X, Y, Z>;
  Vec const level(5, 3, 4), lmin(1, 0, 2), lmax(6, 3, 5);
  Dom const dom = paliwa::strided_domain_from_level<X, Y, Z>(
      {5, 3, 4}, {6, 3, 5});
  EXPECT(dom.size() == 4096);
  EXPECT(dom.strides().get<X>() == 2 && dom.strides().get<Z>() == 2);

  // Errors that need no device: unknown wavelet (map::at), lmin > level,
  // incomplete grid.
  ddc::ChunkSpan<double, Dom> fake(reinterpret_cast<double *>(256), dom);
  EXPECT(throws<std::out_of_range>(
      [&] { paliwa::hierarchize(fake, level, lmin, lmax, "db4"); }));
  EXPECT(throws<std::invalid_argument>([&] {
    paliwa::hierarchize(fake, level, Vec(6, 0, 0), lmax, "hat");
  }));
  // A chunk that is not a box of the level's lattice (wrong strides).
  Dom const skew(dom.front(), Vec(16, 8, 16), Vec(1, 1, 1));
  ddc::ChunkSpan<double, Dom> skewed(reinterpret_cast<double *>(256), skew);
  EXPECT(throws<std::invalid_argument>(
      [&] { paliwa::hierarchize(skewed, level, lmin, lmax, "hat"); }));

  // Restricted-output planning (paliwa_domains.hpp), host only: the
  // reference's known answers (test/test_paliwa_plan.cpp:199-221, 403-429).
  {
    paliwa::LiftingPasses const one{{1, {0.0, 1.0, 0.0}}};
    auto ignore = [](size_t, size_t, paliwa::PeriodicBounds) {};
    for (auto const &ls : std::vector<std::vector<long>>{{4, 1}, {1, 4}, {1, 2, 1}})
      EXPECT(throws<std::invalid_argument>(
          [&] { paliwa::transform_bounds({0, 0}, 4, 4, ls, one, ignore); }));
    auto cover = [](std::vector<long> v, long lo, long hi) {
      auto b = paliwa::covering_periodic_bounds(v, 64);
      return b.min == lo && b.max == hi;
    };
    EXPECT(cover({}, -1, -1) && cover({12}, 12, 12) &&
           cover({8, 12, 16}, 8, 16) && cover({0, 4, 56, 60}, 56, 4) &&
           cover({0, 16, 32, 48}, 0, 48));
    constexpr int big = std::numeric_limits<std::ptrdiff_t>::digits;
    std::size_t const sp = std::size_t{1} << (big - 3);
    auto runs = paliwa::pole_pass_segments(
        {static_cast<long>(sp), static_cast<long>(5 * sp)}, 6 * sp, 3, big, 3);
    std::vector<std::array<int, 3>> got;
    for (auto const &r : runs)
      for (int k = 0; k < r.count; ++k)
        got.push_back({r.first + k * r.stride, r.lower + k * r.stride,
                       r.upper + k * r.stride});
    EXPECT((got == std::vector<std::array<int, 3>>{{3, 2, 4}, {5, 4, 6}, {7, 6, 0}}));
    EXPECT(throws<std::invalid_argument>([] {
      paliwa::pole_pass_segments({0, 0}, 0, std::numeric_limits<int>::digits,
                                 std::numeric_limits<int>::digits, 1);
    }));
    // pole_pass_segments against explicit slot arithmetic for every level,
    // pass, origin, parity, start and count on small pencils
    // (test/test_paliwa_plan.cpp:355-401).
    for (int level = 1; level <= 5; ++level) {
      int const period = 1 << level;
      long const spacing = 4;
      for (int pass = 1; pass <= level; ++pass) {
        int const dist = 1 << (level - pass);
        for (int origin = 0; origin < period; ++origin)
          for (int parity = 0; parity < 2; ++parity)
            for (int start = parity * dist; start < period; start += 2 * dist)
              for (int count = 1; count <= period / (2 * dist); ++count) {
                int const last = (start + (count - 1) * 2 * dist) % period;
                auto const parts = paliwa::pole_pass_segments(
                    {start * spacing, last * spacing},
                    static_cast<std::size_t>(origin * spacing), level,
                    level + 2, pass);
                std::vector<std::array<int, 3>> got, want;
                for (auto const &r : parts)
                  for (int k = 0; k < r.count; ++k)
                    got.push_back({r.first + k * r.stride,
                                   r.lower + k * r.stride,
                                   r.upper + k * r.stride});
                auto slot = [&](int x) {
                  return (x - origin + 2 * period) % period;
                };
                for (int i = 0; i < count; ++i) {
                  int const x = (start + i * 2 * dist) % period;
                  want.push_back({slot(x), slot(x - dist), slot(x + dist)});
                }
                EXPECT(got == want);
              }
      }
    }
    // restrict_periodic_bounds: the odd lattice of a 64-point axis (stride
    // 2 from uid 1) inside [60, 5] wrapped: {61, 63} and {1, 3, 5}.
    {
      using V2 = ddc::DiscreteVector<X, Y>;
      ddc::StridedDiscreteDomain<X, Y> const odd(
          ddc::DiscreteElement<X, Y>(std::array<long, 2>{1, 0}), V2(32, 4),
          V2(2, 1));
      auto const parts =
          paliwa::restrict_periodic_bounds<X>(odd, {60, 5}, 64);
      EXPECT(parts.size() == 2);
      EXPECT(parts[0].front().uid<X>() == 61 &&
             parts[0].extents().get<X>() == 2);
      EXPECT(parts[1].front().uid<X>() == 1 &&
             parts[1].extents().get<X>() == 3);
      EXPECT(parts[0].extents().get<Y>() == 4 &&
             parts[0].strides().get<X>() == 2);
      EXPECT(paliwa::restrict_periodic_bounds<X>(odd, {}, 64).empty());
    }
    // for_each_transform_index visits every uid of the planned bounds once
    // (paliwa_domains.hpp:454-469): outputs 4..7 of a 16-point hat
    // hierarchization need uids 0 and 4..8.
    {
      paliwa::LiftingPasses const hat{{1, {-0.5, 1.0, -0.5}}};
      auto const b = paliwa::transform_bounds(
          {4, 7}, 4, 4, std::vector<long>{4, 3, 2, 1}, hat, ignore);
      std::vector<int> seen(16, 0);
      paliwa::for_each_transform_index<X>(b, 4, [&](ddc::DiscreteElement<X> e) {
        ++seen[static_cast<size_t>(e.uid<X>())];
      });
      for (int u = 0; u < 16; ++u)
        EXPECT(seen[static_cast<size_t>(u)] == ((u == 0 || (u >= 4 && u <= 8)) ? 1 : 0));
    }
    // A window holding uids 0..7 of a 16-point axis cannot give outputs
    // 4..7 of the full hierarchization: their inputs wrap to 8..15.
    using V1 = ddc::DiscreteVector<X>;
    using D1 = ddc::StridedDiscreteDomain<X>;
    D1 const win(ddc::DiscreteElement<X>(std::array<long, 1>{0}), V1(8), V1(1));
    D1 const outs(ddc::DiscreteElement<X>(std::array<long, 1>{4}), V1(4), V1(1));
    ddc::ChunkSpan<double, D1> w(reinterpret_cast<double *>(256), win);
    EXPECT(throws<std::runtime_error>([&] {
      paliwa::transform_in<X>(w, V1(4), V1(4), std::vector<long>{4, 3, 2, 1},
                              paliwa::LiftingPasses{{1, {-0.5, 1.0, -0.5}}},
                              outs, paliwa::gb300::Stream{});
    }));
  }

  int devices = 0;
  if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) {
    std::printf("api_test: no GPU, argument checks passed\n");
    return 0;
  }

  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::vector<double> host(dom.size());
  for (auto &v : host) v = u(rng);
  double *dev = nullptr;
  EXPECT(cudaMalloc(&dev, host.size() * sizeof(double)) == cudaSuccess);
  EXPECT(cudaMemcpy(dev, host.data(), host.size() * sizeof(double),
                    cudaMemcpyHostToDevice) == cudaSuccess);
  ddc::ChunkSpan<double, Dom> grid(dev, dom);
  cudaStream_t s;
  EXPECT(cudaStreamCreate(&s) == cudaSuccess);
  paliwa::gb300::Stream instance{s};
  for (std::string w : {"hat", "biorthogonal", "fullweighting"}) {
    std::vector<double> want = host;
    paliwa_oracle::Shape shape;
    shape.ndim = 3;
    shape.level = {5, 3, 4};
    shape.maximum_level = {6, 3, 5};
    long const lm[3] = {1, 0, 2};
    int const wid = w == "hat" ? 0 : (w == "biorthogonal" ? 1 : 2);
    paliwa_oracle::hierarchize(want.data(), shape, lm, wid, true,
                               paliwa_oracle::Mode::Direct);
    EXPECT(cudaMemcpy(dev, host.data(), host.size() * sizeof(double),
                      cudaMemcpyHostToDevice) == cudaSuccess);
    paliwa::hierarchize(grid, level, lmin, lmax, w, instance);
    std::vector<double> got(host.size());
    EXPECT(cudaStreamSynchronize(s) == cudaSuccess);
    EXPECT(cudaMemcpy(got.data(), dev, got.size() * sizeof(double),
                      cudaMemcpyDeviceToHost) == cudaSuccess);
    EXPECT(got == want);
    // per-dimension calls in order, then the inverse
    EXPECT(cudaMemcpy(dev, host.data(), host.size() * sizeof(double),
                      cudaMemcpyHostToDevice) == cudaSuccess);
    paliwa::hierarchize_in<X>(grid, level, lmin, lmax, w, instance);
    paliwa::hierarchize_in<Y>(grid, level, lmin, lmax, w, instance);
    paliwa::hierarchize_in<Z>(grid, level, lmin, lmax, w, instance);
    paliwa::dehierarchize(grid, level, lmin, lmax, w, instance);
    EXPECT(cudaStreamSynchronize(s) == cudaSuccess);
    EXPECT(cudaMemcpy(got.data(), dev, got.size() * sizeof(double),
                      cudaMemcpyDeviceToHost) == cudaSuccess);
    double err = 0;
    for (size_t i = 0; i < got.size(); ++i)
      err = std::max(err, std::fabs(got[i] - host[i]));
    EXPECT(err <= 1e-13);
  }
  // transform_in with a filter offset the reference rejects
  EXPECT(throws<std::runtime_error>([&] {
    paliwa::transform_in<Y>(grid, level, lmax, std::vector<long>{3},
                            paliwa::LiftingPasses{{2, {0.0, 1.0, 0.0}}},
                            instance);
  }));
  // Restricted outputs covering the whole grid equal the full transform_in.
  {
    std::vector<double> full(host.size()), part(host.size());
    std::vector<long> ls{3, 2, 1};
    auto const &f = paliwa::lifting_wavelet_filter_offsets_and_coefficients
                        .at("biorthogonal");
    EXPECT(cudaMemcpy(dev, host.data(), host.size() * sizeof(double),
                      cudaMemcpyHostToDevice) == cudaSuccess);
    paliwa::transform_in<Y>(grid, level, lmax, ls, f, instance);
    EXPECT(cudaStreamSynchronize(s) == cudaSuccess);
    EXPECT(cudaMemcpy(full.data(), dev, full.size() * sizeof(double),
                      cudaMemcpyDeviceToHost) == cudaSuccess);
    EXPECT(cudaMemcpy(dev, host.data(), host.size() * sizeof(double),
                      cudaMemcpyHostToDevice) == cudaSuccess);
    paliwa::transform_in<Y>(grid, level, lmax, ls, f, dom, instance,
                            paliwa::PoleExecution::PackedPoles);
    EXPECT(cudaStreamSynchronize(s) == cudaSuccess);
    EXPECT(cudaMemcpy(part.data(), dev, part.size() * sizeof(double),
                      cudaMemcpyDeviceToHost) == cudaSuccess);
    EXPECT(part == full);
  }
  // A chunk holding a box of the lattice (a partial chunk): the reference's
  // bounds-checked passes, dimension by dimension, against the oracle.
  {
    Dom const box(Dom::discrete_element_type(std::array<long, 3>{8, 2, 6}),
                  Vec(9, 5, 7), dom.strides());
    std::vector<double> bhost(box.size());
    for (auto &v : bhost) v = u(rng);
    double *bdev = nullptr;
    EXPECT(cudaMalloc(&bdev, bhost.size() * sizeof(double)) == cudaSuccess);
    EXPECT(cudaMemcpy(bdev, bhost.data(), bhost.size() * sizeof(double),
                      cudaMemcpyHostToDevice) == cudaSuccess);
    ddc::ChunkSpan<double, Dom> part(bdev, box);
    paliwa::hierarchize(part, level, lmin, lmax, "biorthogonal", instance);
    instance.fence();
    std::vector<double> got(bhost.size()), want = bhost;
    EXPECT(cudaMemcpy(got.data(), bdev, got.size() * sizeof(double),
                      cudaMemcpyDeviceToHost) == cudaSuccess);
    paliwa_oracle::Shape shape;
    shape.ndim = 3;
    shape.level = {5, 3, 4};
    shape.maximum_level = {6, 3, 5};
    long const front[3] = {8, 2, 6}, ext[3] = {9, 5, 7};
    long const low[3] = {1, 0, 2}, high[3] = {5, 3, 4};
    auto const f = paliwa_oracle::forward_filters(1);
    for (int d = 0; d < 3; ++d) {
      std::vector<long> ls;
      for (long k = high[d]; k > low[d]; --k) ls.push_back(k);
      paliwa_oracle::transform_in_window(want.data(), shape, front, ext, d, ls,
                                         f);
    }
    EXPECT(got == want);
    cudaFree(bdev);
  }
  // Raw dump (paliwa_io.hpp): storage order, no header.
  {
    char const *path = "api_test_dump.raw";
    paliwa::dump_chunk_span_to_binary_file(grid, path, instance);
    std::vector<double> back(host.size()), now(host.size());
    std::FILE *f = std::fopen(path, "rb");
    EXPECT(f != nullptr);
    EXPECT(std::fread(back.data(), sizeof(double), back.size(), f) ==
           back.size());
    std::fclose(f);
    std::remove(path);
    EXPECT(cudaMemcpy(now.data(), dev, now.size() * sizeof(double),
                      cudaMemcpyDeviceToHost) == cudaSuccess);
    EXPECT(back == now);
  }
  cudaStreamDestroy(s);
  cudaFree(dev);
  std::printf("api_test: GPU transforms match the oracle\n");
  return 0;
}
