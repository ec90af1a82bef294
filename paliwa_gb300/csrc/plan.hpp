// Host-side planning of the per-axis lifting launches.
//
// Turns "apply these levels (in this order) with these filters along axis
// `dim` of a grid" into kernel launches (lift.cuh). This is where paliwa's
// level-strided index maps (paliwa/paliwa_domains.hpp:33-139:
// strided_domain_from_level, even/odd half domains) become arithmetic on a
// dense [outer][n][inner] view: level l of an axis at level `lev` has compact
// distance s = 2^(lev - l) between neighbours, writes the points k with
// k mod 2s == offset * s, and wraps periodically at n = 2^lev
// (paliwa/paliwa_transform.hpp:37-41, 236-241).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "lift.cuh"

namespace pgb {

struct StatusError : std::runtime_error {
  int code;
  StatusError(int c, std::string const &m) : std::runtime_error(m), code(c) {}
};

struct Filter {
  int offset;
  double c[3];
};

// Wavelet tables, paliwa/paliwa_wavelets.hpp:15-28.
std::vector<Filter> wavelet_filters(int wavelet, bool forward);

// A dense view of the pencils along one axis.
struct AxisView {
  long long offset = 0;  // element offset of the grid in the buffer
  long long columns = 1; // outer * inner
  int log2_inner = 0;
  int log2_kstride = 0;  // element stride between consecutive pencil points
  int log2_astride = 0;  // element stride between consecutive outer indices
  int log2_n = 0;        // pencil length
};

// A planned launch: kernel parameters with one inline job (single grid) or,
// for batches, a job index range; the tile count; the register chunk R.
struct LaunchPlan {
  LiftParams params{};
  int R = 0;
  long long tiles = 0;
  // Jobs of a batched launch (params.jobs is set when uploaded).
  std::vector<LiftJob> jobs;
};

constexpr int kWindowLog2 = 13;     // points per pencil per CTA (8192)
constexpr int kThreads = 256;
constexpr int kHaloBudget = 512;    // halo per side of a window, in points

int chunk_for(int log2_n);          // R for a periodic pencil of 2^log2_n
void plan_axis(AxisView const &view, std::vector<int> const &shifts,
               std::vector<Filter> const &filters, LaunchPlan const &proto,
               std::vector<LaunchPlan> &out);

bool exact_scalers(std::vector<Filter> const &filters);

} // namespace pgb
