// Stand-in for Kokkos_Random.hpp -- TEST INFRASTRUCTURE (see
// Kokkos_Core.hpp beside it). paliwa's transform header includes it but uses
// none of its generators.
#pragma once

#include <Kokkos_Core.hpp>
