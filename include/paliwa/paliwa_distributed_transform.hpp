// Drop-in for paliwa/paliwa_distributed_transform.hpp on one GB300:
// distributed_hierarchize / distributed_dehierarchize (:448-493) with the
// reference's signature, compiled, as there, only with PALIWA_WITH_MPI.
//
// One GPU per process and no sharding: the Cartesian communicator must have
// one rank. With one rank the reference exchanges no ghosts and transforms
// the local grid, which is then the whole grid, in place (its no-peer path
// transform(local, local), :327-330); here that is the GPU hierarchize /
// dehierarchize. A communicator of more ranks is rejected with
// std::runtime_error, as multi-rank decomposition is not part of this
// library; a single GPU holds the whole grid, and a slab with its periodic
// ghosts is transformed in one buffer by transform_in's restricted-output
// overload. PoleExecution and the axis permutation are accepted for source
// compatibility (one rank has nothing to permute or pack).
#pragma once

#include <array>
#include <cstddef>
#include <stdexcept>
#include <string>

#include "paliwa_domains.hpp"
#include "paliwa_transform.hpp"

#ifdef PALIWA_WITH_MPI
#include <mpi.h>
#endif // PALIWA_WITH_MPI

namespace paliwa {

#ifdef PALIWA_WITH_MPI

namespace detail {

template <std::size_t N>
constexpr std::array<int, N> identity_cartesian_axes() {
  std::array<int, N> axes{};
  for (std::size_t d = 0; d < N; ++d) axes[d] = static_cast<int>(d);
  return axes;
}

template <typename ChunkSpanType, typename... DDims>
void check_single_rank(ChunkSpanType const &local_grid,
                       ddc::StridedDiscreteDomain<DDims...> const &full,
                       MPI_Comm cart_comm) {
  int ranks = 0;
  if (MPI_Comm_size(cart_comm, &ranks) != MPI_SUCCESS)
    throw std::runtime_error("MPI_Comm_size failed");
  if (ranks != 1)
    throw std::runtime_error(
        "the GB300 transform runs one rank per GPU without decomposition: "
        "the Cartesian communicator must have one rank");
  if (!(local_grid.domain() == full))
    throw std::invalid_argument(
        "with one rank the local grid must be the full strided domain");
}

} // namespace detail

template <typename ChunkSpanType, typename ExecSpace = gb300::Stream,
          typename... DDims>
void distributed_hierarchize(
    ChunkSpanType const local_grid,
    ddc::StridedDiscreteDomain<DDims...> const &full_strided_domain,
    ddc::DiscreteVector<DDims...> const &level,
    ddc::DiscreteVector<DDims...> const &minimum_level,
    ddc::DiscreteVector<DDims...> const &maximum_level,
    std::string const &wavelet_name, MPI_Comm cart_comm,
    ExecSpace instance = ExecSpace(),
    [[maybe_unused]] std::array<int, sizeof...(DDims)> const &cartesian_axes =
        detail::identity_cartesian_axes<sizeof...(DDims)>(),
    [[maybe_unused]] PoleExecution pole_execution =
        PoleExecution::PackedPoles) {
  detail::check_single_rank(local_grid, full_strided_domain, cart_comm);
  hierarchize(local_grid, level, minimum_level, maximum_level, wavelet_name,
              instance);
}

template <typename ChunkSpanType, typename ExecSpace = gb300::Stream,
          typename... DDims>
void distributed_dehierarchize(
    ChunkSpanType const local_grid,
    ddc::StridedDiscreteDomain<DDims...> const &full_strided_domain,
    ddc::DiscreteVector<DDims...> const &level,
    ddc::DiscreteVector<DDims...> const &minimum_level,
    ddc::DiscreteVector<DDims...> const &maximum_level,
    std::string const &wavelet_name, MPI_Comm cart_comm,
    ExecSpace instance = ExecSpace(),
    [[maybe_unused]] std::array<int, sizeof...(DDims)> const &cartesian_axes =
        detail::identity_cartesian_axes<sizeof...(DDims)>(),
    [[maybe_unused]] PoleExecution pole_execution =
        PoleExecution::PackedPoles) {
  detail::check_single_rank(local_grid, full_strided_domain, cart_comm);
  dehierarchize(local_grid, level, minimum_level, maximum_level, wavelet_name,
                instance);
}

#endif // PALIWA_WITH_MPI

} // namespace paliwa
