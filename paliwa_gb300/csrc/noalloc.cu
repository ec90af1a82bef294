// Allocation-free single-grid transform (paliwa_gb_transform_noalloc).
//
// Some callers cannot let a library allocate device memory: programs whose
// own allocator already holds the GPU's memory (a framework's caching pool,
// a solver's arena), where a driver allocation can fail or fragment that
// memory, and time-step loops that cannot pay for allocator calls or for the
// device synchronization that cudaFree implies. paliwa_gb_hierarchize needs
// scratch only for grids with a pencil longer than 4096 points (the halo
// buffer of its windowed stages, the grid's size) and takes it from the
// stream-ordered allocator. This variant takes it from one file-scope device
// array instead and allocates nothing.
#include <array>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "launch.cuh"
#include "paliwa_gb300.h"

namespace {

// Scratch for the windowed stages: a grid whose transform needs it must fit.
constexpr size_t kStaticScratchBytes = size_t(64) << 20;  // 64 MiB

// Every GPU that loads the library holds this array until the process exits.
// All calls share it and it keeps the last call's contents; the transform
// writes every byte it later reads, so nothing needs clearing between calls.
static __device__ __align__(256) unsigned char g_scratch[kStaticScratchBytes];

std::mutex g_scratch_mutex;
std::array<void *, 256> g_scratch_address{};  // by device ordinal

// Host code may not use g_scratch's name as an address: the device address
// is looked up once per device, with that device current, by the first call
// on that device (so that call should come before any stream capture).
void *scratch_address() {
  int dev = 0;
  pgb::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= static_cast<int>(g_scratch_address.size()))
    throw pgb::StatusError(PALIWA_GB_RUNTIME_ERROR, "device ordinal too large");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_address[dev] == nullptr) {
    void *ptr = nullptr;
    pgb::cuda_check(cudaGetSymbolAddress(&ptr, g_scratch),
                    "cudaGetSymbolAddress(static scratch)");
    g_scratch_address[dev] = ptr;
  }
  return g_scratch_address[dev];
}

size_t grid_bytes(int dtype, int ndim, int64_t const *level) {
  size_t bytes = pgb::dtype_size(dtype);
  for (int d = 0; d < ndim; ++d) bytes <<= level[d];
  return bytes;
}

} // namespace

extern "C" int paliwa_gb_transform_noalloc(void *grid, int dtype, int ndim,
                                           const int64_t *level,
                                           const int64_t *minimum_level,
                                           const int64_t *maximum_level,
                                           int wavelet, int direction,
                                           void *stream) {
  using namespace pgb;
  return guarded([&] {
    size_t const es = dtype_size(dtype);
    if (grid == nullptr || reinterpret_cast<uintptr_t>(grid) % es != 0)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "grid is null or misaligned");
    if (ndim < 1 || ndim > 32 || level == nullptr ||
        minimum_level == nullptr || maximum_level == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "bad shape arguments");
    int64_t total = 0;
    for (int d = 0; d < ndim; ++d) {
      if (minimum_level[d] < 0 || minimum_level[d] > level[d] ||
          level[d] > maximum_level[d] || level[d] > 40)
        throw StatusError(
            PALIWA_GB_INVALID_ARGUMENT,
            "requires 0 <= minimum_level <= level <= maximum_level");
      total += level[d];
    }
    if (total > 40)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "grid too large");
    if (direction != 1 && direction != -1)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "direction must be 1 (hierarchize) or -1");
    bool const forward = direction > 0;
    auto const filters = wavelet_filters(wavelet, forward);
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    LiftParams const params = launch_params(filters);
    bool const exact = exact_scalers(filters);
    bool const sym = symmetric_filters(filters);
    int const ws = wavelet_schedule(filters);
    // Plan every axis first, so that a grid whose scratch does not fit is
    // rejected before any work is queued.
    std::vector<std::vector<Stage>> plans(ndim);
    for (int d = 0; d < ndim; ++d) {
      AxisView view = axis_view(reinterpret_cast<unsigned long long>(grid),
                                ndim, level, d, dtype);
      auto const shifts = level_shifts(level[d], minimum_level[d], forward);
      if (needs_shadow(view, shifts)) {
        if (grid_bytes(dtype, ndim, level) > kStaticScratchBytes)
          throw StatusError(
              PALIWA_GB_INVALID_ARGUMENT,
              "grid of " + std::to_string(grid_bytes(dtype, ndim, level)) +
                  " bytes has a pencil longer than 4096 points and needs that "
                  "much scratch; the allocation-free transform holds at most "
                  "67108864 bytes (64 MiB)");
        view.shadow = reinterpret_cast<unsigned long long>(scratch_address());
      }
      plan_axis(view, shifts, filters, plans[d]);
    }
    for (auto const &stages : plans)
      for (auto const &st : stages) {
        LiftParams p = params;
        p.job = st.job;
        int const sched =
            ws >= 0 && canonical_shifts(st.job, (ws & 1) != 0) ? ws : -1;
        launch_lift(dtype, exact, sym, sched, st.R, p, nullptr, 1, st.tiles,
                    s);
      }
  });
}
