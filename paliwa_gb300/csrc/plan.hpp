// Host-side planning of the per-axis lifting launches.
//
// Turns "apply these levels (in this order) with these filters along axis
// `dim` of a grid" into kernel jobs (lift.cuh). This is where paliwa's
// level-strided index maps (paliwa/paliwa_domains.hpp:33-139:
// strided_domain_from_level, even/odd half domains) become arithmetic on a
// dense [outer][n][inner] view: level l of an axis at level `lev` has compact
// distance s = 2^(lev - l) between neighbours, writes the points k with
// k mod 2s == offset * s, and wraps periodically at n = 2^lev
// (paliwa/paliwa_transform.hpp:37-41, 236-241).
#pragma once

#include <cstdint>
#include <map>
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
bool exact_scalers(std::vector<Filter> const &filters);
// Every pass has c0 == c2 (the symmetric lifting steps of all wavelets).
bool symmetric_filters(std::vector<Filter> const &filters);

// A dense view of the pencils along one axis.
struct AxisView {
  unsigned long long base = 0;  // byte address of the grid
  // Byte address of a buffer with the grid's size and layout that holds the
  // windowed stages' halos (pencils longer than one CTA holds; 0: none).
  unsigned long long shadow = 0;
  long long columns = 1;        // outer * inner
  int log2_inner = 0;
  int log2_kstride = 0;  // element stride between consecutive pencil points
  int log2_astride = 0;  // element stride between consecutive outer indices
  int log2_n = 0;        // pencil length
  // log2 of the adjacent columns one thread of the wide kernel holds for this
  // grid's storage type (0: the grid is not aligned to such a row).
  int log2_row = 0;
  // The wide kernel also takes the last axis (FP32 compensated only: plain
  // FP32 and FP64 run faster there on the direct kernel, which needs fewer
  // registers per pencil).
  bool wide_last = false;
  int log2_es = 0;  // log2 of the element size in bytes
};

AxisView axis_view(unsigned long long base, int ndim, int64_t const *level,
                   int dim, int dtype);

// Stage::R names the kernel and its chunk size: R > 0 the staged kernel with
// chunks of R points, -R the direct kernel, kWide + R the wide kernel on a
// strided axis, kWideContig + R the wide kernel on the last axis, kTile + R
// and kTileLong + R the tile kernel for pencils of up to 32 chunks and
// longer ones.
constexpr int kWide = 64;
constexpr int kWideContig = 128;
constexpr int kTile = 192;
constexpr int kTileLong = 256;
// Stage::R of a halo pass (halo_kernel) before a windowed stage.
constexpr int kHalo = 512;

// One stage of an axis transform: a job for one kernel. The stages of one
// axis must run in order; stages of different grids are independent.
struct Stage {
  int R = 0;
  long long tiles = 0;
  LiftJob job{};
  // Periodic stages: the tuning class and the kernels that apply (a bit per
  // KernelChoice); 0 for windowed and halo stages.
  int tclass = 0;
  unsigned kernels = 0;
  int dflt = 0;
  // A wide stage that a batch runs on the TMA wide kernel.
  bool tma = false;
};

constexpr int kWindowLog2 = 12;   // points per column per CTA round (4096)
constexpr int kThreads = 256;
constexpr int kRounds = kTileRounds;  // column rounds per tile
constexpr int kHaloBudget = 256;  // halo per side of a window, in points

int chunk_for(int log2_n);        // R for a periodic pencil of 2^log2_n

// Kernel choices for periodic stages, and a table that forces one per class
// of stage (tuning_class: last axis, sub-lattice, log2 n, inner extent in
// bytes). A forced kernel that does not apply to a stage is ignored.
enum KernelChoice {
  kChooseStaged = 0,    // staged, 16 points per thread (or n when shorter)
  kChooseDirect = 1,
  kChooseWide = 2,
  kChooseTile = 3,
  kChooseStaged32 = 4,  // staged, 32 points per thread
  // the wide kernel's transform with TMA copies (batches of FP32c grids;
  // elsewhere the wide kernel)
  kChooseTmaWide = 5,
  kChooseCount = 6
};
struct KernelSet {
  unsigned mask = 0;  // a bit per applicable KernelChoice
  int dflt = kChooseStaged;
  // The kernel that a stage choosing kChooseTmaWide is planned for (the
  // wide kernel, else the default without the TMA wide kernel): it runs the
  // stage outside batches and where the tensor map cannot be made.
  int fallback = kChooseStaged;
  bool has(int c) const { return (mask >> c) & 1u; }
};
struct Tuning {
  std::map<int, int> choice;  // tuning_class -> KernelChoice
};
KernelSet periodic_kernels(AxisView const &v, bool canonical);
int tuning_class(AxisView const &v);

void plan_axis(AxisView const &view, std::vector<int> const &shifts,
               std::vector<Filter> const &filters, std::vector<Stage> &out,
               Tuning const *tuning = nullptr);

// Points one stage reads and writes (the algorithmic bytes of its launch are
// twice this times the element size): every point of its pencils, or for a
// halo pass the points it copies.
long long stage_points(Stage const &st);

// True when planning `view` along `shifts` needs a halo buffer (the field
// `shadow`: the grid's size and layout).
inline bool needs_shadow(AxisView const &view, std::vector<int> const &shifts) {
  return !shifts.empty() && view.log2_n > kWindowLog2;
}

// Kernel-level parameters shared by every job of a launch.
LiftParams launch_params(std::vector<Filter> const &filters);

// Launch the lifting kernel for `dtype` over `njobs` jobs (device array
// `jobs`, or the inline job of `params` when jobs == nullptr).
// sched: 2 * wavelet + forward for the compile-time wavelet schedule (every
// job's shifts must be canonical), or -1 for the runtime schedule.
void launch_lift(int dtype, bool exact, bool symmetric, int sched, int R,
                 LiftParams params, LiftJob const *jobs, int njobs,
                 long long total_tiles, cudaStream_t stream);
// 2 * wavelet + forward when the filters are one of the wavelet tables.
int wavelet_schedule(std::vector<Filter> const &filters);
// Shifts 0 .. L-1 (forward) or L-1 .. 0: the level range of hierarchize_in.
bool canonical_shifts(LiftJob const &job, bool forward);

void cuda_check(cudaError_t e, char const *what);
size_t dtype_size(int dtype);

// Shifts (log2 distances) of hierarchize_in (forward: levels level..lmin+1)
// or dehierarchize_in (lmin+1..level).
std::vector<int> level_shifts(int64_t lev, int64_t lmin, bool forward);

extern thread_local std::string g_last_error;

template <typename F> int guarded(F &&f) {
  try {
    f();
    return 0;
  } catch (StatusError const &e) {
    g_last_error = e.what();
    return e.code;
  } catch (std::exception const &e) {
    g_last_error = e.what();
    return 2;
  }
}

} // namespace pgb
