// Drop-in C++ API test: the reference's call shapes
//   paliwa::hierarchize(span, level, lmin, lmax, "biorthogonal", instance)
// over a ChunkSpan of device memory, checked bit for bit against the CPU
// oracle (test infrastructure). Without a GPU it only exercises the argument
// errors, which map to the reference's exception types.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <random>
#include <stdexcept>
#include <vector>

#include <paliwa/paliwa_transform.hpp>

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
  Dom const part(dom.front(), Vec(16, 8, 16), dom.strides());
  ddc::ChunkSpan<double, Dom> partial(reinterpret_cast<double *>(256), part);
  EXPECT(throws<std::invalid_argument>(
      [&] { paliwa::hierarchize(partial, level, lmin, lmax, "hat"); }));

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
  cudaStreamDestroy(s);
  cudaFree(dev);
  std::printf("api_test: GPU transforms match the oracle\n");
  return 0;
}
