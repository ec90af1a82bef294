// Stand-in for <ddc/ddc.hpp> -- TEST INFRASTRUCTURE. It lets the unmodified
// reference headers compile into oracle/_ref (oracle/Makefile, target `ref`)
// so that the CPU oracle can be checked against the reference itself. DDC is
// not in this image: the subset of its API that paliwa uses is the library's
// own include/paliwa/ddc_compat.hpp (written from DDC's documented
// semantics); Kokkos_Core.hpp beside this directory supplies the views that
// the reference builds sparse domains from.
#pragma once

#include <Kokkos_Core.hpp>

#include "../../../include/paliwa/ddc_compat.hpp"
