// Wavelet lifting tables of paliwa (paliwa/paliwa_wavelets.hpp:15-28): for
// each wavelet name, the ordered (parity offset, {c0, c1, c2}) lifting passes
// of the forward (hierarchize) and inverse (dehierarchize) transforms. The
// values are the reference's; they are also compiled into the CUDA library
// (paliwa_gb_wavelet_filters).
#pragma once

#include <array>
#include <map>
#include <string>
#include <utility>
#include <vector>

namespace paliwa {
using LiftingPasses = std::vector<std::pair<int, std::array<double, 3>>>;

inline const std::map<std::string, LiftingPasses>
    lifting_wavelet_filter_offsets_and_coefficients = {
        {"hat", {{1, {-0.5, 1.0, -0.5}}}},
        {"biorthogonal", {{1, {-0.5, 1.0, -0.5}}, {0, {0.25, 1.0, 0.25}}}},
        {"fullweighting", {{0, {0.25, 0.5, 0.25}}, {1, {-0.5, 1.0, -0.5}}}},
};
inline const std::map<std::string, LiftingPasses>
    lifting_wavelet_reconstruct_offsets_and_coefficients = {
        {"hat", {{1, {0.5, 1.0, 0.5}}}},
        {"biorthogonal", {{0, {-0.25, 1.0, -0.25}}, {1, {0.5, 1.0, 0.5}}}},
        {"fullweighting", {{1, {0.5, 1.0, 0.5}}, {0, {-0.5, 2.0, -0.5}}}},
};
} // namespace paliwa
