// C ABI of paliwa_gb300: single-grid transforms (include/paliwa_gb300.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "paliwa_gb300.h"
#include "launch.cuh"

namespace pgb {

thread_local std::string g_last_error;

std::vector<Filter> wavelet_filters(int wavelet, bool forward) {
  // paliwa/paliwa_wavelets.hpp:17-20 (forward) and :24-27 (inverse).
  switch (wavelet) {
  case PALIWA_GB_HAT:
    if (forward) return {{1, {-0.5, 1.0, -0.5}}};
    return {{1, {0.5, 1.0, 0.5}}};
  case PALIWA_GB_BIORTHOGONAL:
    if (forward) return {{1, {-0.5, 1.0, -0.5}}, {0, {0.25, 1.0, 0.25}}};
    return {{0, {-0.25, 1.0, -0.25}}, {1, {0.5, 1.0, 0.5}}};
  case PALIWA_GB_FULLWEIGHTING:
    if (forward) return {{0, {0.25, 0.5, 0.25}}, {1, {-0.5, 1.0, -0.5}}};
    return {{1, {0.5, 1.0, 0.5}}, {0, {-0.5, 2.0, -0.5}}};
  }
  throw StatusError(PALIWA_GB_OUT_OF_RANGE, "unknown wavelet id");
}

// True when every coefficient is 0 or +-2^k with a product that stays exact
// in both float and double, so fused multiply-adds round like the
// reference's separate multiplies and adds.
bool exact_scalers(std::vector<Filter> const &filters) {
  for (auto const &f : filters)
    for (double c : f.c) {
      if (c == 0.0) continue;
      int e = 0;
      double const m = std::frexp(c, &e);
      if (std::fabs(m) != 0.5 || e < -60 || e > 60) return false;
    }
  return true;
}

bool symmetric_filters(std::vector<Filter> const &filters) {
  for (auto const &f : filters)
    if (f.c[0] != f.c[2]) return false;
  return true;
}

int chunk_for(int log2_n) {
  if (log2_n <= 4) return 1 << log2_n;  // whole pencil in one thread
  return 16;
}

// Points per thread and column of the wide kernel (0: pencil too long for
// it). Pencils of up to 16 points are held whole by one thread; pencils of
// 32 and 64 points by G = 4 lanes, so that a warp row is 8 column groups
// (32 or 64 contiguous bytes). With more lanes per pencil each warp load
// touches more distinct rows with fewer bytes each (16 lanes: 16-byte
// pieces; 32 lanes: 8): measured on a 2^26-point FP32 grid, the first axis
// at n = 256 fell from 2.2 TB/s (G = 16) to 0.47 TB/s (G = 32), so longer
// pencils go to the staged kernel.
// log2 of the bytes of one copied piece of the tile kernel (lift.cuh,
// tile_geo) for 256 threads: 8 when the chunk padding (one warp-row segment)
// or the tile row is not a multiple of 16 bytes, else 16.
int tile_piece_log2(int log2G, int log2_row_bytes) {
  static_assert(kThreads == 256, "tile geometry assumes 256 threads");
  int const log2seg = log2G >= 5 ? log2_row_bytes : 5 - log2G + log2_row_bytes;
  int const pad = (1 << log2seg) & 127;
  int const log2rb = 8 - log2G + log2_row_bytes;
  return (pad & 15) != 0 || log2rb < 4 ? 3 : 4;
}

// Points per thread of the staged kernel: 16, or 32 for FP32c pencils of
// 512 points and more (and their windows): half the chunks, so pencils of up
// to 1024 points exchange by shuffle only and longer ones through half as
// many shared-memory steps (measured on 2^26-point grids, first axis: 1024
// points 2.30 against 1.66 TB/s, 2048 points 1.68 against 1.12).
int staged_chunk(AxisView const &v) {
  return v.wide_last && v.log2_n >= 9 ? 32 : 16;
}

int wide_chunk(int log2_n) {
  if (log2_n <= 4) return 1 << log2_n;
  if (log2_n <= 6) return 1 << (log2_n - 2);
  return 0;
}

void cuda_check(cudaError_t e, char const *what) {
  if (e != cudaSuccess)
    throw StatusError(PALIWA_GB_CUDA_ERROR,
                      std::string(what) + ": " + cudaGetErrorString(e));
}

size_t dtype_size(int dtype) {
  switch (dtype) {
  case PALIWA_GB_F64: return 8;
  case PALIWA_GB_F32:
  case PALIWA_GB_F32C: return 4;
  }
  throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "unknown dtype");
}

AxisView axis_view(unsigned long long base, int ndim, int64_t const *level,
                   int dim, int dtype) {
  AxisView v;
  // Row vectors of the wide kernel: 4 floats (FP32), 2 floats (FP32
  // compensated: a row is one double-float pair of pairs), 2 doubles (FP64).
  int const log2_row = dtype == PALIWA_GB_F32 ? 2 : 1;
  v.log2_row = (base % 16) == 0 ? log2_row : 0;
  v.wide_last = dtype == PALIWA_GB_F32C;
  v.log2_es = dtype == PALIWA_GB_F64 ? 3 : 2;
  int log2_outer = 0, log2_inner = 0;
  for (int d = 0; d < dim; ++d) log2_outer += static_cast<int>(level[d]);
  for (int d = dim + 1; d < ndim; ++d) log2_inner += static_cast<int>(level[d]);
  v.base = base;
  v.columns = 1LL << (log2_outer + log2_inner);
  v.log2_inner = log2_inner;
  v.log2_kstride = log2_inner;
  v.log2_n = static_cast<int>(level[dim]);
  v.log2_astride = v.log2_n + log2_inner;
  return v;
}

std::vector<int> level_shifts(int64_t lev, int64_t lmin, bool forward) {
  std::vector<int> sh;
  // hierarchize_in: levels lev .. lmin+1 (paliwa_transform.hpp:364-367);
  // dehierarchize_in: lmin+1 .. lev (:392-394). shift = lev - l.
  for (int64_t l = lmin + 1; l <= lev; ++l)
    sh.push_back(static_cast<int>(lev - l));
  // sh now follows increasing levels (the inverse order).
  if (forward) std::reverse(sh.begin(), sh.end());
  return sh;
}

LiftParams launch_params(std::vector<Filter> const &filters) {
  if (filters.size() > static_cast<size_t>(kMaxPasses))
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "at most 8 filter passes");
  LiftParams p;
  std::memset(&p, 0, sizeof(p));
  p.npasses = static_cast<int>(filters.size());
  for (size_t i = 0; i < filters.size(); ++i) {
    if (filters[i].offset != 0 && filters[i].offset != 1)
      throw StatusError(PALIWA_GB_RUNTIME_ERROR, "Filter offset not supported");
    p.offsets[i] = filters[i].offset;
    p.coeffs[i] = {filters[i].c[0],        filters[i].c[1],
                   filters[i].c[2],        float(filters[i].c[0]),
                   float(filters[i].c[1]), float(filters[i].c[2])};
    if (filters[i].c[1] == 1.0) p.c1_one_mask |= 1u << i;
  }
  return p;
}

namespace {

long long ceil_div(long long a, long long b) { return (a + b - 1) / b; }

LiftJob make_job(AxisView const &v, std::vector<int> const &sh, size_t first,
                 size_t count) {
  LiftJob job;
  std::memset(&job, 0, sizeof(job));
  job.base = v.base;
  job.dst_base = v.base;
  job.columns = v.columns;
  job.tile_begin = 0;
  job.log2_inner = v.log2_inner;
  job.log2_kstride = v.log2_kstride;
  job.log2_astride = v.log2_astride;
  job.log2_n = v.log2_n;
  job.nlevels = static_cast<int>(count);
  for (size_t i = 0; i < count; ++i)
    job.shift[i] = static_cast<signed char>(sh[first + i]);
  return job;
}

} // namespace

// Kernels that can run the periodic stages of view `v` (a bit per
// KernelChoice), and the one chosen by default. Applicability: the wide and
// tile kernels need a wavelet schedule (canonical level range) and a grid
// aligned to 16 bytes; the wide kernel takes strided pencils of up to 64
// points whose inner extent holds a row vector, and last-axis pencils of up
// to 512 points when there is a row vector's worth of them; the tile kernel
// strided pencils of 128 to 4096 points whose inner extent holds whole copy
// pieces; the direct kernel pencils that one thread holds whole and
// last-axis pencils of up to 32 chunks; the staged kernel everything with
// chunks of 16 points.
KernelSet periodic_kernels(AxisView const &v, bool canon) {
  int const R = chunk_for(v.log2_n);
  int const log2G = v.log2_n - (31 - __builtin_clz(R));
  bool const aligned = canon && v.log2_row > 0;
  bool const last = v.log2_inner == 0 && v.log2_kstride == 0;
  KernelSet k;
  if (R == 16) k.mask |= 1 << kChooseStaged;
  if (v.log2_n >= 6) k.mask |= 1 << kChooseStaged32;
  if (R == (1 << v.log2_n) || (last && log2G <= 5))
    k.mask |= 1 << kChooseDirect;
  // The wide kernel counts column groups in 32 bits.
  if (aligned && v.columns < (1LL << 30) &&
      ((!last && wide_chunk(v.log2_n) > 0 && v.log2_inner >= v.log2_row) ||
       (last && log2G <= 5 && v.columns >= (1LL << v.log2_row))))
    k.mask |= 1 << kChooseWide;
  if (aligned && !last && R == 16 && log2G >= 3 && log2G <= 8 &&
      v.log2_inner + v.log2_es >=
          tile_piece_log2(log2G, v.log2_row + v.log2_es))
    k.mask |= 1 << kChooseTile;
  // The TMA wide kernel: FP32c strided stages, 16-byte aligned, inner
  // extents of 4 or more columns; wide stages of up to 4 chunks, and
  // pencils of 8 to 128 chunks of 16 points (128 to 2048 points).
  if (!last && v.wide_last && v.log2_inner >= 2 && v.base % 16 == 0 &&
      v.columns < (1LL << 30) &&
      ((k.has(kChooseWide) &&
        v.log2_n - (31 - __builtin_clz(static_cast<unsigned>(
                             wide_chunk(v.log2_n)))) <= 2) ||
       (R == 16 && log2G >= 3 && log2G <= 7)))
    k.mask |= 1 << kChooseTmaWide;
  // ... and the last axis' wide stages of chunks of 4 to 16 points and its
  // pencils of 64 to 256 chunks of 16 points (1024 to 4096 points), and the
  // wide stages of strided axes of inner extent 2 whose pencil pairs lie
  // one after another.
  if (last && v.wide_last && v.base % 16 == 0 &&
      ((k.has(kChooseWide) && R >= 4) ||
       (R == 16 && log2G >= 6 && log2G <= 8)))
    k.mask |= 1 << kChooseTmaWide;
  if (!last && v.wide_last && k.has(kChooseWide) && v.log2_inner == 1 &&
      v.log2_kstride == 1 && v.log2_astride == v.log2_n + 1 &&
      wide_chunk(v.log2_n) >= 4 && v.base % 16 == 0)
    k.mask |= 1 << kChooseTmaWide;
  // Default: the wide kernel for strided pencils (and FP32c last-axis
  // pencils: measured on 2^26-point grids, 3.0-4.5 TB/s against 2.8-4.1 on
  // the direct kernel), then the tile kernel up to the length where it was
  // measured faster than the staged kernel (first axis of 2^26-point grids,
  // and the 4D CT batch): 4096 points in FP32 (2.8 against 1.8 TB/s at
  // 1024), 512 in FP64, 256 in FP32c (at G = 32 its 8-byte row vectors need
  // 8-byte copy pieces, and beyond 32 chunks the batch ran slower than on
  // the staged kernel); then the direct kernel, then the staged one.
  int const tile_log2G_max = v.wide_last ? 4 : v.log2_es == 3 ? 5 : 8;
  if (k.has(kChooseWide) && (!last || v.wide_last))
    k.dflt = kChooseWide;
  else if (k.has(kChooseTile) && log2G <= tile_log2G_max)
    k.dflt = kChooseTile;
  else if (k.has(kChooseDirect))
    k.dflt = kChooseDirect;
  else
    k.dflt = staged_chunk(v) == 32 ? kChooseStaged32 : kChooseStaged;
  k.fallback = k.dflt;
  // (The TMA wide kernel is the default for strided wide chunks of 8 and
  // 16 points, for strided pencils of 8 to 128 chunks and for the last
  // axis' wide stages, measured on the 4D CT batch: per launch 4.73 against
  // 4.01 TB/s at 8 points, 4.73 against 3.16 at 16, about 3.7 against 2.29
  // on the tile kernel's pencils of 128 and 256 points, 0.46 against 0.71
  // ms on the staged kernel's pencils of 512; on pencils of 1024 and 2048
  // points, whose chunks exchange through shared memory, as fast as the
  // staged kernel per launch (0.92 ms each) and the step 21.59 against
  // 22.02 ms with it; on the last axis 4.86 against 3.60 TB/s at 16 points,
  // 4.97 against 4.42 at 8 and 4.96 against 4.79 at 4 (the step 20.37
  // against 21.20 ms), and on its pencils of 1024-4096 points 0.39 against
  // 0.41 ms on the staged kernel (19.71 against 19.81 ms); on strided axes
  // of inner extent 2, 3.3-3.5 against 1.4-2.0 TB/s (20.15 against 20.30
  // ms). On strided 4-point chunks of
  // wider inner extents the wide kernel is faster, 5.26 against 4.39-4.55
  // TB/s.)
  if (k.has(kChooseTmaWide) &&
      (last || v.log2_inner == 1 || wide_chunk(v.log2_n) >= 8 ||
       !k.has(kChooseWide)))
    k.dflt = kChooseTmaWide;
  return k;
}

int tuning_class(AxisView const &v) {
  bool const last = v.log2_inner == 0 && v.log2_kstride == 0;
  bool const sub = v.log2_kstride != v.log2_inner;
  int const inner_bytes = std::min(v.log2_inner + v.log2_es, 8);
  return (last ? 1 : 0) | (sub ? 2 : 0) | (v.log2_n << 2) |
         (inner_bytes << 8);
}

namespace {

// Periodic whole-pencil stages; level lists longer than one job holds are
// split into consecutive stages (order preserved). `ws` is the wavelet
// schedule of the filters (or -1); `tuning` may force a kernel per class.
void plan_periodic(AxisView const &v, std::vector<int> const &shifts, int ws,
                   Tuning const *tuning, std::vector<Stage> &out) {
  int const R = chunk_for(v.log2_n);
  int const log2G = v.log2_n - (31 - __builtin_clz(R));
  long long const C = static_cast<long long>(kRounds) * (kThreads >> log2G);
  int const wR = wide_chunk(v.log2_n);
  int const wlog2G = wR > 0 ? v.log2_n - (31 - __builtin_clz(wR)) : 0;
  long long const wC = static_cast<long long>(kRounds) * (kThreads >> wlog2G);
  bool const last = v.log2_inner == 0 && v.log2_kstride == 0;
  for (size_t first = 0; first < shifts.size(); first += kMaxLevels) {
    size_t const count =
        std::min(shifts.size() - first, static_cast<size_t>(kMaxLevels));
    Stage st;
    st.job = make_job(v, shifts, first, count);
    st.job.periodic = 1;
    st.job.log2_window = v.log2_n;
    bool const canon = ws >= 0 && canonical_shifts(st.job, (ws & 1) != 0);
    KernelSet const ks = periodic_kernels(v, canon);
    st.tclass = tuning_class(v);
    st.kernels = ks.mask;
    st.dflt = ks.dflt;
    int choice = ks.dflt;
    if (tuning != nullptr) {
      auto const it = tuning->choice.find(tuning_class(v));
      if (it != tuning->choice.end() && ks.has(it->second))
        choice = it->second;
    }
    auto tile_stage = [&] {
      st.R = (log2G <= 5 ? kTile : kTileLong) + 16;
      st.job.col_tiles =
          ceil_div(v.columns >> v.log2_row, kThreads >> log2G);
    };
    if (choice == kChooseTmaWide) {
      // Marked for the TMA wide kernel (batches); elsewhere, and for the
      // grids that do not qualify, planned for the kernel it stands in for.
      st.tma = true;
      choice = ks.fallback;
    }
    switch (choice) {
    case kChooseWide:
      if (last) {
        st.R = kWideContig + R;
        st.job.col_tiles = ceil_div(v.columns >> v.log2_row, C);
      } else {
        st.R = kWide + wR;
        st.job.col_tiles = ceil_div(v.columns >> v.log2_row, wC);
      }
      break;
    case kChooseTile:
      tile_stage();
      break;
    case kChooseDirect:
      st.R = -R;
      st.job.col_tiles = ceil_div(v.columns, C);
      break;
    default: {
      int const sR = choice == kChooseStaged32 ? 32 : R;
      int const slog2G = v.log2_n - (31 - __builtin_clz(sR));
      st.R = sR;
      st.job.col_tiles = ceil_div(
          v.columns, static_cast<long long>(kRounds) * (kThreads >> slog2G));
      break;
    }
    }
    st.tiles = st.job.col_tiles;
    out.push_back(st);
  }
}

// Fine levels of a long pencil on overlapping windows.
void plan_windows(AxisView const &v, std::vector<int> const &shifts,
                  std::vector<Filter> const &filters,
                  std::vector<Stage> &out) {
  long long const window = 1LL << kWindowLog2;
  AxisView wv = v;
  wv.log2_n = kWindowLog2;
  int const R = staged_chunk(wv);
  long long const C = static_cast<long long>(kRounds) *
                      (kThreads >> (kWindowLog2 - (31 - __builtin_clz(R))));
  size_t first = 0;
  while (first < shifts.size()) {
    // Grow the run while the halo it needs fits the window: each step of
    // distance s widens the dependency cone by s on both sides.
    long long reach = 0;
    size_t count = 0;
    while (first + count < shifts.size() && count < kMaxLevels) {
      long long const add =
          static_cast<long long>(filters.size()) << shifts[first + count];
      long long const halo = ceil_div(reach + add, R) * R;
      if (2 * halo > window / 2 && count > 0) break;
      reach += add;
      ++count;
    }
    long long const halo = ceil_div(reach, R) * R;
    long long const seg_len = window - 2 * halo;
    if (seg_len <= 0)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "filter list too long for windowed long pencils");
    if (v.shadow == 0)
      throw StatusError(PALIWA_GB_RUNTIME_ERROR,
                        "windowed stage planned without a halo buffer");
    // Windows read their halos from the neighbouring segments, which those
    // segments' windows overwrite in place: a halo pass first copies the
    // points around every segment boundary to the halo buffer, and the
    // windows read every point outside their own segment from there.
    Stage hs;
    hs.R = kHalo;
    hs.job = make_job(v, shifts, first, 0);
    hs.job.dst_base = v.shadow;
    hs.job.periodic = 0;
    hs.job.seg_len = static_cast<int>(seg_len);
    hs.job.halo = static_cast<int>(halo);
    // A tile: 32 positions around one boundary of up to 64 columns (2048
    // points, many tiles in flight for these small passes).
    int const log2cols = 63 - __builtin_clzll(static_cast<unsigned long long>(
                                   v.columns));
    int const lc = std::min(6, log2cols);
    hs.job.log2_window = lc;
    hs.job.col_tiles = ceil_div(v.columns, 1LL << lc);
    long long const nseg = ceil_div(1LL << v.log2_n, seg_len);
    hs.tiles = nseg * (halo / 16) * hs.job.col_tiles;
    out.push_back(hs);
    Stage st;
    st.R = R;
    st.job = make_job(v, shifts, first, count);
    st.job.halo_base = v.shadow;
    st.job.periodic = 0;
    st.job.log2_window = kWindowLog2;
    st.job.seg_len = static_cast<int>(seg_len);
    st.job.halo = static_cast<int>(halo);
    st.job.col_tiles = ceil_div(v.columns, C);
    st.tiles = nseg * st.job.col_tiles;
    out.push_back(st);
    first += count;
  }
}

} // namespace

void plan_axis(AxisView const &view, std::vector<int> const &shifts,
               std::vector<Filter> const &filters, std::vector<Stage> &out,
               Tuning const *tuning) {
  if (shifts.empty() || filters.empty() || view.log2_n == 0) return;
  if (view.log2_n <= kWindowLog2) {
    plan_periodic(view, shifts, wavelet_schedule(filters), tuning, out);
    return;
  }
  // Long pencil: levels closer than 2^m run on windows with a halo of at most
  // kHaloBudget points per side; the others run on the sub-lattice of every
  // 2^m-th point, which is a periodic pencil 2^m times shorter.
  int const P = static_cast<int>(filters.size());
  int m = 0;
  while (static_cast<long long>(P) * ((2LL << m) - 1) <= kHaloBudget) ++m;
  if (m < 1) m = 1;
  size_t i = 0;
  while (i < shifts.size()) {
    bool const fine = shifts[i] < m;
    size_t j = i;
    while (j < shifts.size() && (shifts[j] < m) == fine) ++j;
    std::vector<int> run(shifts.begin() + i, shifts.begin() + j);
    if (fine) {
      plan_windows(view, run, filters, out);
    } else {
      AxisView sub = view;
      sub.log2_n = view.log2_n - m;
      sub.log2_kstride = view.log2_kstride + m;
      for (int &s : run) s -= m;
      plan_axis(sub, run, filters, out, tuning);
    }
    i = j;
  }
}

int current_device() {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  return dev;
}

int device_sms() {
  int const dev = current_device();
  int sms = 0;
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
             "cudaDeviceGetAttribute");
  return sms;
}

int wavelet_schedule(std::vector<Filter> const &filters) {
  for (int w = 0; w < 3; ++w)
    for (int fwd = 0; fwd < 2; ++fwd) {
      auto const t = wavelet_filters(w, fwd != 0);
      if (t.size() != filters.size()) continue;
      bool same = true;
      for (size_t i = 0; i < t.size() && same; ++i)
        same = t[i].offset == filters[i].offset && t[i].c[0] == filters[i].c[0] &&
               t[i].c[1] == filters[i].c[1] && t[i].c[2] == filters[i].c[2];
      if (same) return 2 * w + fwd;
    }
  return -1;
}

bool canonical_shifts(LiftJob const &job, bool forward) {
  for (int i = 0; i < job.nlevels; ++i)
    if (job.shift[i] != (forward ? i : job.nlevels - 1 - i)) return false;
  return true;
}

void launch_lift(int dtype, bool exact, bool symmetric, int sched, int R,
                 LiftParams params, LiftJob const *jobs, int njobs,
                 long long total_tiles, cudaStream_t s) {
  if (total_tiles <= 0 || R == 0) return;
  params.jobs = jobs;
  params.njobs = njobs;
  params.total_tiles = total_tiles;
  params.rounds = kRounds;
  if (R == kHalo) return launch_halo(dtype, params, s);
  if (R > kWide) {  // the wide and tile kernels
    switch (dtype) {
    case PALIWA_GB_F64: return launch_wide_f64(sched, R, params, s);
    case PALIWA_GB_F32: return launch_wide_f32(sched, R, params, s);
    case PALIWA_GB_F32C: return launch_wide_f32c(sched, R, params, s);
    }
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "unknown dtype");
  }
  switch (dtype) {
  case PALIWA_GB_F64: return launch_lift_f64(exact, sched, R, params, s);
  case PALIWA_GB_F32: return launch_lift_f32(exact, sched, R, params, s);
  case PALIWA_GB_F32C:
    return launch_lift_f32c(exact && symmetric, sched, R, params, s);
  }
  throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "unknown dtype");
}

} // namespace pgb

using namespace pgb;

namespace {

void check_shape(void *grid, int dtype, int ndim, int64_t const *level,
                 int64_t const *maximum_level) {
  dtype_size(dtype);
  if (grid == nullptr)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "grid is null");
  if (reinterpret_cast<uintptr_t>(grid) % dtype_size(dtype) != 0)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "grid is misaligned");
  if (ndim < 1 || ndim > 32)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "ndim must be in [1, 32]");
  long long total = 0;
  for (int d = 0; d < ndim; ++d) {
    if (level[d] < 0 || level[d] > 40)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "level out of range");
    if (maximum_level != nullptr && maximum_level[d] < level[d])
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "level must not exceed maximum_level");
    total += level[d];
  }
  if (total > 40)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "grid too large");
}

void transform_axis(void *grid, int dtype, int ndim, int64_t const *level,
                    int dim, std::vector<int> const &shifts,
                    std::vector<Filter> const &filters, cudaStream_t s) {
  LiftParams const params = launch_params(filters);
  AxisView view = axis_view(reinterpret_cast<unsigned long long>(grid), ndim,
                            level, dim, dtype);
  void *shadow = nullptr;
  if (needs_shadow(view, shifts)) {
    // Stream-ordered scratch for the windowed stages of long pencils.
    size_t bytes = dtype_size(dtype);
    for (int d = 0; d < ndim; ++d) bytes <<= level[d];
    cuda_check(cudaMallocAsync(&shadow, bytes, s), "cudaMallocAsync(shadow)");
    view.shadow = reinterpret_cast<unsigned long long>(shadow);
  }
  try {
    std::vector<Stage> stages;
    plan_axis(view, shifts, filters, stages);
    bool const exact = exact_scalers(filters);
    bool const sym = symmetric_filters(filters);
    int const ws = wavelet_schedule(filters);
    for (auto const &st : stages) {
      LiftParams p = params;
      p.job = st.job;
      int const sched =
          ws >= 0 && canonical_shifts(st.job, (ws & 1) != 0) ? ws : -1;
      launch_lift(dtype, exact, sym, sched, st.R, p, nullptr, 1, st.tiles, s);
    }
  } catch (...) {
    if (shadow) cudaFreeAsync(shadow, s);
    throw;
  }
  if (shadow) cuda_check(cudaFreeAsync(shadow, s), "cudaFreeAsync(shadow)");
}

void check_levels(int ndim, int64_t const *level, int64_t const *lmin,
                  int64_t const *lmax) {
  // paliwa/paliwa_transform.hpp:359-362 (asserted there).
  for (int d = 0; d < ndim; ++d)
    if (lmin[d] < 0 || lmin[d] > level[d] || level[d] > lmax[d])
      throw StatusError(
          PALIWA_GB_INVALID_ARGUMENT,
          "requires 0 <= minimum_level <= level <= maximum_level");
}

int hierarchize_dims(void *grid, int dtype, int ndim, int64_t const *level,
                     int64_t const *lmin, int64_t const *lmax, int dim_begin,
                     int dim_end, int wavelet, bool forward, void *stream) {
  return guarded([&] {
    check_shape(grid, dtype, ndim, level, lmax);
    check_levels(ndim, level, lmin, lmax);
    if (dim_begin < 0 || dim_end > ndim || dim_begin >= dim_end)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "bad dimension");
    auto const filters = wavelet_filters(wavelet, forward);
    for (int d = dim_begin; d < dim_end; ++d)
      transform_axis(grid, dtype, ndim, level, d,
                     level_shifts(level[d], lmin[d], forward), filters,
                     static_cast<cudaStream_t>(stream));
  });
}

} // namespace

extern "C" {

const char *paliwa_gb_last_error(void) { return g_last_error.c_str(); }

int paliwa_gb_version(void) { return 100; }

int paliwa_gb_synchronize(void *stream) {
  return guarded([&] {
    cuda_check(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)),
               "cudaStreamSynchronize");
  });
}

int paliwa_gb_wavelet_id(const char *name, int *id) {
  return guarded([&] {
    if (name == nullptr || id == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    std::string const n(name);
    if (n == "hat") *id = PALIWA_GB_HAT;
    else if (n == "biorthogonal") *id = PALIWA_GB_BIORTHOGONAL;
    else if (n == "fullweighting") *id = PALIWA_GB_FULLWEIGHTING;
    else throw StatusError(PALIWA_GB_OUT_OF_RANGE, "unknown wavelet: " + n);
  });
}

int paliwa_gb_wavelet_filters(int wavelet, int direction, int *npasses,
                              int32_t *offsets, double *coefficients) {
  return guarded([&] {
    auto const f = wavelet_filters(wavelet, direction > 0);
    *npasses = static_cast<int>(f.size());
    for (size_t p = 0; p < f.size(); ++p) {
      offsets[p] = f[p].offset;
      for (int k = 0; k < 3; ++k) coefficients[3 * p + k] = f[p].c[k];
    }
  });
}

int paliwa_gb_transform_in(void *grid, int dtype, int ndim,
                           const int64_t *level, const int64_t *maximum_level,
                           int dim, const int64_t *levels, int nlevels,
                           const int32_t *offsets, const double *coefficients,
                           int npasses, void *stream) {
  return guarded([&] {
    check_shape(grid, dtype, ndim, level, maximum_level);
    if (dim < 0 || dim >= ndim)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "bad dimension");
    if (npasses < 0 || nlevels < 0)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "negative count");
    std::vector<Filter> filters;
    for (int p = 0; p < npasses; ++p)
      filters.push_back({offsets[p],
                         {coefficients[3 * p], coefficients[3 * p + 1],
                          coefficients[3 * p + 2]}});
    for (auto const &f : filters)  // paliwa_transform.hpp:239-240
      if (f.offset != 0 && f.offset != 1)
        throw StatusError(PALIWA_GB_RUNTIME_ERROR,
                          "Filter offset not supported");
    std::vector<int> shifts;
    for (int i = 0; i < nlevels; ++i) {
      if (levels[i] < 1 || levels[i] > level[dim])  // :232 asserts l > 0
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "transform level out of range");
      shifts.push_back(static_cast<int>(level[dim] - levels[i]));
    }
    transform_axis(grid, dtype, ndim, level, dim, shifts, filters,
                   static_cast<cudaStream_t>(stream));
  });
}

int paliwa_gb_hierarchize_in(void *grid, int dtype, int ndim,
                             const int64_t *level, const int64_t *lmin,
                             const int64_t *lmax, int dim, int wavelet,
                             void *stream) {
  return hierarchize_dims(grid, dtype, ndim, level, lmin, lmax, dim, dim + 1,
                          wavelet, true, stream);
}

int paliwa_gb_dehierarchize_in(void *grid, int dtype, int ndim,
                               const int64_t *level, const int64_t *lmin,
                               const int64_t *lmax, int dim, int wavelet,
                               void *stream) {
  return hierarchize_dims(grid, dtype, ndim, level, lmin, lmax, dim, dim + 1,
                          wavelet, false, stream);
}

int paliwa_gb_hierarchize(void *grid, int dtype, int ndim,
                          const int64_t *level, const int64_t *lmin,
                          const int64_t *lmax, int wavelet, void *stream) {
  return hierarchize_dims(grid, dtype, ndim, level, lmin, lmax, 0, ndim,
                          wavelet, true, stream);
}

int paliwa_gb_dehierarchize(void *grid, int dtype, int ndim,
                            const int64_t *level, const int64_t *lmin,
                            const int64_t *lmax, int wavelet, void *stream) {
  return hierarchize_dims(grid, dtype, ndim, level, lmin, lmax, 0, ndim,
                          wavelet, false, stream);
}

} // extern "C"

namespace pgb {

void launch_halo(int dtype, LiftParams const &p, cudaStream_t s) {
  if (dtype == PALIWA_GB_F64) {
    static thread_local Occupancy occ;
    launch_persistent(halo_kernel<double, kThreads>, 0, p, s, occ);
  } else {
    static thread_local Occupancy occ;
    launch_persistent(halo_kernel<float, kThreads>, 0, p, s, occ);
  }
}

long long stage_points(Stage const &st) {
  if (st.R != kHalo) return st.job.columns << st.job.log2_n;
  long long const nseg = ceil_div(1LL << st.job.log2_n, st.job.seg_len);
  return st.job.columns * nseg * 2 * st.job.halo;
}

} // namespace pgb
