// distributed_hierarchize / distributed_dehierarchize of the drop-in header,
// built with PALIWA_WITH_MPI against a fake <mpi.h> (tests/cpp/fake_mpi):
// more than one rank and a local grid that is not the full grid are
// rejected without a device; on a GPU one rank equals hierarchize (checked
// against the oracle) and the round trip holds.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <random>
#include <stdexcept>
#include <vector>

#include <paliwa/paliwa_distributed_transform.hpp>

#include "paliwa_oracle.hpp"

struct X {};
struct Y {};

#define EXPECT(c)                                                           \
  do {                                                                      \
    if (!(c)) {                                                             \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);            \
      return 1;                                                             \
    }                                                                       \
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
  using Vec = ddc::DiscreteVector<X, Y>;
  using Dom = ddc::StridedDiscreteDomain<X, Y>;
  Vec const level(5, 4), lmin(1, 0), lmax(6, 4);
  Dom const full = paliwa::strided_domain_from_level<X, Y>({5, 4}, {6, 4});
  ddc::ChunkSpan<double, Dom> fake(reinterpret_cast<double *>(256), full);
  EXPECT(throws<std::runtime_error>([&] {
    paliwa::distributed_hierarchize(fake, full, level, lmin, lmax, "hat", 2);
  }));
  Dom const half(full.front(), Vec(16, 16), full.strides());
  ddc::ChunkSpan<double, Dom> local(reinterpret_cast<double *>(256), half);
  EXPECT(throws<std::invalid_argument>([&] {
    paliwa::distributed_dehierarchize(local, full, level, lmin, lmax, "hat",
                                      MPI_COMM_SELF);
  }));
  int devices = 0;
  if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) {
    std::printf("distributed_test: no GPU, argument checks passed\n");
    return 0;
  }
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::vector<double> host(full.size());
  for (auto &v : host) v = u(rng);
  double *dev = nullptr;
  EXPECT(cudaMalloc(&dev, host.size() * sizeof(double)) == cudaSuccess);
  EXPECT(cudaMemcpy(dev, host.data(), host.size() * sizeof(double),
                    cudaMemcpyHostToDevice) == cudaSuccess);
  ddc::ChunkSpan<double, Dom> grid(dev, full);
  paliwa::distributed_hierarchize(grid, full, level, lmin, lmax,
                                  "biorthogonal", MPI_COMM_SELF);
  std::vector<double> got(host.size()), want = host;
  EXPECT(cudaDeviceSynchronize() == cudaSuccess);
  EXPECT(cudaMemcpy(got.data(), dev, got.size() * sizeof(double),
                    cudaMemcpyDeviceToHost) == cudaSuccess);
  paliwa_oracle::Shape shape;
  shape.ndim = 2;
  shape.level = {5, 4};
  shape.maximum_level = {6, 4};
  long const lm[2] = {1, 0};
  paliwa_oracle::hierarchize(want.data(), shape, lm, 1, true,
                             paliwa_oracle::Mode::Direct);
  EXPECT(got == want);
  paliwa::distributed_dehierarchize(grid, full, level, lmin, lmax,
                                    "biorthogonal", MPI_COMM_SELF);
  EXPECT(cudaDeviceSynchronize() == cudaSuccess);
  EXPECT(cudaMemcpy(got.data(), dev, got.size() * sizeof(double),
                    cudaMemcpyDeviceToHost) == cudaSuccess);
  double err = 0;
  for (size_t i = 0; i < got.size(); ++i)
    err = std::max(err, std::fabs(got[i] - host[i]));
  EXPECT(err <= 1e-13);
  cudaFree(dev);
  std::printf("distributed_test: one rank matches the oracle\n");
  return 0;
}
