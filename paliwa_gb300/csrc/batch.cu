// Batched transforms of many component grids and the combination-technique
// combine / restrict / scatter (include/paliwa_gb300.h).
//
// The reference transforms the component grids of a combination scheme one
// hierarchize() call each, spread over execution-space instances
// (test/test_paliwa_combination_technique.cpp:164-174). Here one plan covers
// every grid: for each axis, the per-grid stages of plan_axis() are merged
// into one launch per stage index and chunk size, whose device-side job list
// names every grid. The grids are dealt into up to kBatchGroups groups of
// about equal size, each planned on its own; a direction's launch sequences
// of the groups run on parallel branches (forked streams, joined at the
// end), so one group's launches fill the tails of another's and kernels of
// different kinds share the GPU. The whole direction is captured once into a
// CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include <cudaTypedefs.h>

#include "combine.cuh"
#include "paliwa_gb300.h"
#include "plan.hpp"
#include "slab.cuh"
#include "twide.cuh"

namespace pgb {
void launch_slab_f64(int sched, SlabParams const &p, cudaStream_t s);
void launch_slab_f32(int sched, SlabParams const &p, cudaStream_t s);
void launch_slab_f32c(int sched, SlabParams const &p, cudaStream_t s);
void launch_twide_f32c(int sched, int R, TWideParams const &p,
                       cudaStream_t s);
} // namespace pgb

using namespace pgb;

namespace {

// Groups of grids planned and run on parallel branches. Measured on the 4D
// CT workload (3,025 grids, FP32c, forward + inverse): 28.7 ms with one
// group, 26.1 with two, 25.7 with three, 25.6 with four.
constexpr int kBatchGroups = 4;

// Kernel code of a slab launch (slab.cuh) and, plus the chunk size, of a
// TMA wide launch (twide.cuh); the others are plan.hpp's.
constexpr int kSlab = 1024;
constexpr int kTWide = 2048;

struct Launch {
  int group = 0;
  int R = 0;
  int sched = -1;
  size_t job_first = 0;  // index into the device job array
  size_t tile_first = 0;  // slab launches: index into the tile-job table
  int njobs = 0;
  long long tiles = 0;
  long long points = 0;  // grid points stored by this launch
};

struct Direction {
  LiftParams params{};
  bool exact = true;
  bool symmetric = true;
  std::vector<Launch> launches;
  LiftJob *jobs_dev = nullptr;
  SlabJob *slab_dev = nullptr;  // jobs of the slab launches
  int *slab_tile_dev = nullptr;  // job of every tile of the slab launches
  // TMA wide launches: jobs, the job of every tile, the tensor maps.
  TWideJob *twide_dev = nullptr;
  int *twide_tile_dev = nullptr;
  CUtensorMap *maps_dev = nullptr;
  cudaGraphExec_t graph = nullptr;
  Tuning tuning;  // kernel forced per class (autotuner)
  // Slab launches where they apply (the batch's setting); the autotuner
  // clears it when the direction runs faster axis by axis.
  bool slabs = true;
  // TMA wide launches for the stages planned on them (the batch's setting).
  bool tma = true;
  // Classes of the plan's periodic stages: applicable kernels (bits), the
  // default choice of the first stage seen, and the points they store.
  struct ClassInfo {
    unsigned kernels = 0;
    int dflt = 0;
    long long points = 0;
  };
  std::map<int, ClassInfo> classes;
};

void free_direction(Direction &d) {
  if (d.graph) cudaGraphExecDestroy(d.graph);
  if (d.jobs_dev) cudaFree(d.jobs_dev);
  if (d.slab_dev) cudaFree(d.slab_dev);
  if (d.slab_tile_dev) cudaFree(d.slab_tile_dev);
  if (d.twide_dev) cudaFree(d.twide_dev);
  if (d.twide_tile_dev) cudaFree(d.twide_tile_dev);
  if (d.maps_dev) cudaFree(d.maps_dev);
  d.slab_tile_dev = nullptr;
  d.twide_dev = nullptr;
  d.twide_tile_dev = nullptr;
  d.maps_dev = nullptr;
  d.graph = nullptr;
  d.jobs_dev = nullptr;
  d.slab_dev = nullptr;
  d.launches.clear();
  d.classes.clear();
}

void check_grid_levels(int ndim, int ngrids, int64_t const *levels,
                       int64_t const *lmin, int64_t const *lmax) {
  if (ndim < 1 || ndim > kMaxDims)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "ndim must be in [1, 12]");
  if (ngrids < 1)
    throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "no grids");
  for (int g = 0; g < ngrids; ++g) {
    int64_t total = 0;
    for (int d = 0; d < ndim; ++d) {
      int64_t const l = levels[g * ndim + d];
      if (l < 0 || l > lmax[d] || lmax[d] > 30 ||
          (lmin != nullptr && (lmin[d] < 0 || lmin[d] > l)))
        throw StatusError(
            PALIWA_GB_INVALID_ARGUMENT,
            "requires 0 <= minimum_level <= level <= maximum_level <= 30");
      total += l;
    }
    if (total > 40)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "grid too large");
  }
}

} // namespace

struct paliwa_gb_batch {
  int ndim = 0;
  int ngrids = 0;
  int dtype = 0;
  int wavelet = 0;
  long long points = 0;
  bool use_graphs = true;
  Direction dir[2];  // 0 = forward, 1 = inverse
  // The grids as created (for re-planning).
  std::vector<int64_t> levels, lmin;
  std::vector<void *> grids;
  // Halo buffers of the windowed stages (grids with pencils longer than one
  // CTA holds; a region of the grid's size per grid and axis), reused by
  // every axis of a group (a group's axes run in order); the groups, which
  // run concurrently, have disjoint regions.
  void *shadow = nullptr;
  size_t shadow_bytes = 0;
  // group[g]: the group of grid g; group_shadow[k]: byte offset of group
  // k's shadow region. Group k > 0 runs on streams[k - 1] (non-blocking),
  // forked from and joined into the caller's stream with events.
  int ngroups = 1;
  std::vector<int> group;
  std::vector<size_t> group_shadow;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;  // [0] fork, [k] join of group k
  // Slab launches (slab.cuh): the tensor map over the grids' memory as
  // 128-byte rows from slab_base, and the error word of their bounded waits.
  bool use_slabs = true;
  // TMA wide launches for strided wide stages of FP32c grids.
  bool use_tma = true;
  bool slab_map_ok = false;
  unsigned long long slab_base = 0;
  CUtensorMap slab_map{};
  unsigned *slab_error = nullptr;
  // Cap on the CTAs per SM of every launch (0: as many as fit).
  int ctas_per_sm = 0;
};

namespace {

// The slab group of grid g: its trailing axes whose slab (the product of
// their extents) fits one tile, when that group holds at least two axes
// with levels to transform, the grid is a whole number of 1 KB boxes and
// starts on a row of the tensor map. Returns the group's first axis, or
// ndim for none.
int slab_start(paliwa_gb_batch const &b, int g, int64_t const *levels,
               int64_t const *lmin) {
  size_t const es = dtype_size(b.dtype);
  int const log2es = es == 8 ? 3 : 2;
  int64_t const *lv = levels + static_cast<size_t>(g) * b.ndim;
  int64_t total = 0;
  for (int d = 0; d < b.ndim; ++d) total += lv[d];
  if (total + log2es < 10) return b.ndim;  // under one 1 KB box
  unsigned long long const addr =
      reinterpret_cast<unsigned long long>(b.grids[g]);
  if (addr < b.slab_base || (addr - b.slab_base) % 128 != 0) return b.ndim;
  int m = b.ndim;
  int64_t vol = 0;
  while (m > 0 && vol + lv[m - 1] + log2es <= 15) vol += lv[--m];
  int work = 0;
  for (int d = m; d < b.ndim; ++d) work += lv[d] > lmin[d];
  return work >= 2 ? m : b.ndim;
}

// The slab job of grid g for its axes m..ndim-1: per axis with levels to
// transform, the pencil length, its element stride inside a tile (the
// product of the later extents) and the chunk size: 32 points (at most the
// pencil) for the contiguous last axis and for strides of 32 elements or
// more, 8 or fewer for smaller strides when the pencil's chunks then fit
// the CTA's 256 threads (distinct shared-memory banks under the swizzle).
SlabJob slab_job(paliwa_gb_batch const &b, int g, int m,
                 int64_t const *levels, int64_t const *lmin,
                 void *const *grid_ptrs) {
  size_t const es = dtype_size(b.dtype);
  int const log2es = es == 8 ? 3 : 2;
  int64_t const *lv = levels + static_cast<size_t>(g) * b.ndim;
  SlabJob job;
  std::memset(&job, 0, sizeof(job));
  int64_t total = 0;
  for (int d = 0; d < b.ndim; ++d) total += lv[d];
  job.log2_tile = static_cast<int>(std::min<int64_t>(total, 15 - log2es));
  job.row0 = static_cast<long long>(
      (reinterpret_cast<unsigned long long>(grid_ptrs[g]) - b.slab_base) / 128);
  int log2s = 0;
  std::vector<SlabAxis> axes;
  for (int d = b.ndim - 1; d >= m; --d) {
    int const log2n = static_cast<int>(lv[d]);
    int const nlev = static_cast<int>(lv[d] - lmin[d]);
    if (nlev > 0) {
      SlabAxis ax;
      ax.log2n = static_cast<signed char>(log2n);
      ax.log2s = static_cast<signed char>(log2s);
      ax.nlevels = static_cast<signed char>(nlev);
      int log2r = std::min(log2n, 5);
      if (log2s >= 1 && log2s <= 4 && log2n + log2s - 3 <= 8)
        log2r = std::min(log2n, 3);
      ax.log2r = static_cast<signed char>(log2r);
      axes.push_back(ax);
    }
    log2s += log2n;
  }
  std::reverse(axes.begin(), axes.end());
  job.naxes = static_cast<int>(axes.size());
  for (size_t i = 0; i < axes.size(); ++i) job.axis[i] = axes[i];
  return job;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda): a 2D view [rows][128 bytes] from `base`, 1 KB boxes
// (8 rows), 128-byte swizzle.
bool encode_slab_map(CUtensorMap *map, unsigned long long base,
                     unsigned long long rows, size_t es) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (encode == nullptr) {
    cudaDriverEntryPointQueryResult q{};
    void *fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                         cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || fn == nullptr)
      return false;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  if (rows == 0 || rows > (1ULL << 31)) return false;
  cuuint64_t dims[2] = {static_cast<cuuint64_t>(128 / es), rows};
  cuuint64_t strides[1] = {128};
  cuuint32_t box[2] = {static_cast<cuuint32_t>(128 / es), 8};
  cuuint32_t elem[2] = {1, 1};
  CUresult const r = encode(
      map, es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                   : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
      2, reinterpret_cast<void *>(base), dims, strides, box, elem,
      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (encode == nullptr) {
    cudaDriverEntryPointQueryResult q{};
    void *fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                         cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || fn == nullptr)
      return nullptr;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  return encode;
}

// Chunk size of the TMA wide launch that may take a stage (the stage's own
// kernel otherwise): strided wide stages (chunks of 2-16 points, up to 4 per
// pencil), and tile or staged stages of pencils of 128 to 2048 points (8 to
// 128 chunks of 16 points); 0 for the rest.
int twide_chunk(Stage const &st) {
  int const R = st.R;
  if (R == kWide + 2 || R == kWide + 4 || R == kWide + 8 || R == kWide + 16)
    return R - kWide;
  if (R == kWideContig + 4 || R == kWideContig + 8 || R == kWideContig + 16)
    return R - kWideContig;
  bool const last = st.job.log2_inner == 0 && st.job.log2_kstride == 0;
  if ((R == kTile + 16 || R == kTileLong + 16 || R == 16 || R == 32) &&
      st.job.log2_n >= 7 && st.job.log2_n <= (last ? 12 : 11))
    return 16;
  return 0;
}

// The TMA wide job and tensor map of a strided stage (FP32c, float storage)
// with chunks of r points, covering tiles of Ct = 2 NT / G columns. Up to 4
// chunks per pencil: the 3D view [outer][n][inner] of the stage's pencils
// with the axis' strides and boxes {Bx, n, Sx}. 8 to 128 chunks of 16
// points (the chunked layout): the 5D view [outer][inner / 4][row of
// chunk][chunk][4 columns] and one box per tile, so that shared memory holds
// the tile as [column quad][row of chunk][chunk][4 columns]. False when the
// stage does not qualify (alignment, inner extent under 4 columns, more than
// 128 chunks, 2^30 tiles or more, or the encoder refuses the map).
bool twide_job(Stage const &st, int r, TWideJob &job, CUtensorMap &map,
               long long &tiles) {
  auto encode = tensor_map_encoder();
  LiftJob const &lj = st.job;
  int const log2r = 31 - __builtin_clz(static_cast<unsigned>(r));
  int const log2G = lj.log2_n - log2r;
  if (encode == nullptr || lj.periodic != 1 || lj.base % 16 != 0)
    return false;
  bool const last = lj.log2_inner == 0 && lj.log2_kstride == 0;
  bool const pairs = lj.log2_inner == 1 && lj.log2_kstride == 1 &&
                     lj.log2_astride == lj.log2_n + 1;
  if (last || pairs) {
    // The last axis (contiguous layout), or a strided axis of inner extent
    // 2 whose pencil pairs lie one after another (pairs layout): the
    // stage's points as rows of 32 floats (128 bytes), boxes of the unit's
    // 16 r rows, 128-byte swizzle; units of 512 r floats (whole pencils).
    if (r < 4 || log2G < 0 || log2G > (pairs ? 2 : 5 + 3 * (r == 16)))
      return false;
    long long const points = lj.columns << lj.log2_n;
    int const log2unit = 9 + log2r;
    int const log2u = r >= 8 ? 0 : 3 - log2r;  // units per tile
    if (points % 32 != 0 || (points >> (log2unit + log2u)) >= (1LL << 30))
      return false;
    tiles = (points + (1LL << (log2unit + log2u)) - 1) >> (log2unit + log2u);
    std::memset(&job, 0, sizeof(job));
    job.log2_n = lj.log2_n;
    job.nlevels = lj.nlevels;
    job.chunked = pairs ? 3 : 2;
    job.nxb = 1;
    job.log2_bx = log2unit - lj.log2_n;  // box bytes = the unit
    job.log2_sx = 0;
    cuuint64_t dims[2] = {32, static_cast<cuuint64_t>(points / 32)};
    cuuint64_t strides[1] = {128};
    cuuint32_t box[2] = {32, static_cast<cuuint32_t>(16 * r)};
    cuuint32_t elem[2] = {1, 1};
    CUresult const res = encode(
        &map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
        reinterpret_cast<void *>(lj.base), dims, strides, box, elem,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return res == CUDA_SUCCESS;
  }
  if (lj.log2_inner < 2 || log2G < 0 || log2G > 7 || lj.log2_n > 11 ||
      (log2G > 2 && r != 16))
    return false;
  int const log2ct = Log2<kTWideThreads>::value + 1 - log2G;
  // Units per tile: TWideShape<R>::kUnits (16 KB tiles for chunks of up to
  // 8 points).
  int const log2u = r >= 8 ? 0 : 3 - log2r;
  std::memset(&job, 0, sizeof(job));
  job.log2_n = lj.log2_n;
  job.log2_inner = lj.log2_inner;
  job.nlevels = lj.nlevels;
  job.log2_bx = std::min(std::min(lj.log2_inner, log2ct), 8);
  job.log2_sx = std::max(0, log2ct - lj.log2_inner);
  job.nxb = 1 << (log2ct - job.log2_bx - job.log2_sx);
  job.log2_rs = job.log2_bx;
  tiles = (lj.columns + (1LL << (log2ct + log2u)) - 1) >> (log2ct + log2u);
  if (tiles >= (1LL << 30)) return false;
  long long const outer = lj.columns >> lj.log2_inner;
  if (log2G >= 3) {
    job.chunked = 1;
    job.nxb = 1;
    job.log2_bx = std::min(lj.log2_inner, log2ct);  // Bx >= 4: log2ct <= 6
    job.log2_sx = log2ct - job.log2_bx;
    // Groups of 8 columns (32-byte box rows) where the tile and the inner
    // extent hold them, else 4 (16 bytes, the least a box row may be):
    // wider rows halve the rows the tensor memory accelerator moves (the
    // chunked form: 3.91 against 3.5 TB/s on the 4D batch). Not for more
    // than 32 chunks, whose warps would read 8-way conflicting banks (the
    // long form measured slower with them).
    int const xlo = log2ct >= 3 && lj.log2_inner >= 3 && log2G <= 5 ? 3 : 2;
    job.log2_xlo = xlo;
    job.log2_rs = log2G + xlo;
    cuuint64_t dims[5] = {1u << xlo, static_cast<cuuint64_t>(1) << log2G,
                          static_cast<cuuint64_t>(r),
                          static_cast<cuuint64_t>(1) << (lj.log2_inner - xlo),
                          static_cast<cuuint64_t>(outer)};
    cuuint64_t strides[4] = {
        static_cast<cuuint64_t>(4 * r) << lj.log2_kstride,
        static_cast<cuuint64_t>(4) << lj.log2_kstride,
        static_cast<cuuint64_t>(4) << xlo,
        static_cast<cuuint64_t>(4) << lj.log2_astride};
    cuuint32_t box[5] = {1u << xlo, 1u << log2G, static_cast<cuuint32_t>(r),
                         1u << (job.log2_bx - xlo), 1u << job.log2_sx};
    cuuint32_t elem[5] = {1, 1, 1, 1, 1};
    CUresult const res = encode(
        &map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5,
        reinterpret_cast<void *>(lj.base), dims, strides, box, elem,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return res == CUDA_SUCCESS;
  }
  cuuint64_t dims[3] = {static_cast<cuuint64_t>(1) << lj.log2_inner,
                        static_cast<cuuint64_t>(1) << lj.log2_n,
                        static_cast<cuuint64_t>(outer)};
  cuuint64_t strides[2] = {static_cast<cuuint64_t>(4) << lj.log2_kstride,
                           static_cast<cuuint64_t>(4) << lj.log2_astride};
  cuuint32_t box[3] = {1u << job.log2_bx, 1u << lj.log2_n,
                       1u << job.log2_sx};
  // An outer index's n rows of `inner` columns are one contiguous block
  // when the pencil stride is the inner extent (no sub-lattice). When a
  // tile holds whole blocks (inner < Ct) and a block fits one box
  // dimension, the map takes the block as its rows: box rows of n inner
  // floats instead of inner (fewer, longer rows for the tensor memory
  // accelerator), the same bytes in the same shared-memory order, the same
  // box coordinates (x = y = 0).
  if (lj.log2_kstride == lj.log2_inner && lj.log2_inner < log2ct &&
      lj.log2_n + lj.log2_inner <= 8) {
    int const log2blk = lj.log2_n + lj.log2_inner;
    dims[0] = static_cast<cuuint64_t>(1) << log2blk;
    dims[1] = 1;
    strides[0] = static_cast<cuuint64_t>(4) << log2blk;
    box[0] = 1u << log2blk;
    box[1] = 1;
  }
  cuuint32_t elem[3] = {1, 1, 1};
  CUresult const res = encode(
      &map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
      reinterpret_cast<void *>(lj.base), dims, strides, box, elem,
      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return res == CUDA_SUCCESS;
}

// The tensor map over every grid of the batch (rows of 128 bytes from the
// lowest grid address, rounded down to 128 bytes).
void setup_slab_map(paliwa_gb_batch &b) {
  b.slab_map_ok = false;
  size_t const es = dtype_size(b.dtype);
  unsigned long long lo = ~0ULL, hi = 0;
  for (int g = 0; g < b.ngrids; ++g) {
    unsigned long long const a = reinterpret_cast<unsigned long long>(b.grids[g]);
    unsigned long long bytes = es;
    for (int d = 0; d < b.ndim; ++d) bytes <<= b.levels[g * b.ndim + d];
    lo = std::min(lo, a);
    hi = std::max(hi, a + bytes);
  }
  lo &= ~127ULL;
  b.slab_base = lo;
  b.slab_map_ok = encode_slab_map(&b.slab_map, lo, (hi - lo + 127) / 128, es);
}

void plan_direction(paliwa_gb_batch &b, Direction &dr, bool forward,
                    int64_t const *levels, int64_t const *lmin,
                    void *const *grid_ptrs) {
  auto const filters = wavelet_filters(b.wavelet, forward);
  dr.params = launch_params(filters);
  dr.exact = exact_scalers(filters);
  dr.symmetric = symmetric_filters(filters);
  std::vector<LiftJob> all_jobs;
  std::vector<SlabJob> all_slabs;
  std::vector<int> slab_tiles;  // per slab launch tile: its job in the launch
  std::vector<TWideJob> all_twide;
  std::vector<int> twide_tiles;  // per TMA wide launch tile: its job
  std::vector<CUtensorMap> maps;
  size_t const es = dtype_size(b.dtype);
  int const ws = wavelet_schedule(filters);
  bool const tma = b.use_tma && dr.tma && b.dtype == PALIWA_GB_F32C &&
                   ws >= 0 && tensor_map_encoder() != nullptr;
  // First axis of every grid's slab group (ndim: none).
  std::vector<int> slab_from(b.ngrids, b.ndim);
  if (b.use_slabs && dr.slabs && b.slab_map_ok && ws >= 0)
    for (int g = 0; g < b.ngrids; ++g)
      slab_from[g] = slab_start(b, g, levels, lmin);
  for (int grp = 0; grp < b.ngroups; ++grp) {
    std::vector<int> members;
    for (int g = 0; g < b.ngrids; ++g)
      if (b.group[g] == grp) members.push_back(g);
    for (int d = 0; d < b.ndim; ++d) {
      // stages[i] = the ordered stages of grid members[i] along axis d
      std::vector<std::vector<Stage>> stages(members.size());
      size_t depth = 0;
      size_t shadow_off = b.group_shadow[grp];
      for (size_t i = 0; i < members.size(); ++i) {
        int const g = members[i];
        if (d >= slab_from[g]) continue;  // in the grid's slab launch
        int64_t const *lv = levels + static_cast<size_t>(g) * b.ndim;
        AxisView view =
            axis_view(reinterpret_cast<unsigned long long>(grid_ptrs[g]),
                      b.ndim, lv, d, b.dtype);
        auto const shifts = level_shifts(lv[d], lmin[d], forward);
        if (needs_shadow(view, shifts)) {
          size_t bytes = es;
          for (int k = 0; k < b.ndim; ++k) bytes <<= lv[k];
          if (shadow_off + bytes > b.shadow_bytes)
            throw StatusError(PALIWA_GB_RUNTIME_ERROR,
                              "shadow plan overflow");
          view.shadow =
              reinterpret_cast<unsigned long long>(b.shadow) + shadow_off;
          shadow_off += (bytes + 255) / 256 * 256;
        }
        plan_axis(view, shifts, filters, stages[i], &dr.tuning);
        for (Stage const &st : stages[i]) {
          if (st.kernels == 0) continue;
          auto &ci = dr.classes[st.tclass];
          if (ci.kernels == 0) {
            ci.kernels = st.kernels;
            ci.dflt = st.dflt;
          }
          ci.points += st.job.columns << st.job.log2_n;
        }
        depth = std::max(depth, stages[i].size());
      }
      for (size_t k = 0; k < depth; ++k) {
        // One launch per chunk size among the k-th stages of the group;
        // strided wide stages that qualify go to the TMA wide kernel.
        std::map<int, std::vector<Stage const *>> by_r;
        for (size_t i = 0; i < members.size(); ++i)
          if (k < stages[i].size()) {
            Stage const &st = stages[i][k];
            int code = st.R;
            int const r = twide_chunk(st);
            if (tma && st.tma && r > 0 &&
                canonical_shifts(st.job, (ws & 1) != 0)) {
              int const log2G = st.job.log2_n - (31 - __builtin_clz(r));
              bool const last =
                  st.job.log2_inner == 0 && st.job.log2_kstride == 0;
              code = kTWide + r +
                     (last ? (log2G > 5 ? kTWideLongContig : kTWideContig)
                      : st.job.log2_inner == 1 ? kTWidePairs
                      : log2G > 5 ? kTWideLong
                      : log2G >= 3 ? kTWideChunked : 0);
            }
            by_r[code].push_back(&st);
          }
        for (auto const &[R, list] : by_r) {
          if (R > kTWide) {
            Launch L;
            L.group = grp;
            L.R = R;
            L.sched = ws;
            L.job_first = all_twide.size();
            L.tile_first = twide_tiles.size();
            // Stages that do not qualify, by their own kernel.
            std::map<int, std::vector<Stage const *>> rest;
            for (Stage const *st : list) {
              TWideJob job;
              CUtensorMap map;
              long long tiles = 0;
              if (!twide_job(*st, (R - kTWide) % kTWideChunked, job, map,
                             tiles)) {
                rest[st->R].push_back(st);
                continue;
              }
              job.tile_begin = L.tiles;
              job.map = static_cast<int>(maps.size());
              maps.push_back(map);
              all_twide.push_back(job);
              twide_tiles.insert(twide_tiles.end(), tiles, L.njobs);
              L.tiles += tiles;
              L.points += stage_points(*st);
              ++L.njobs;
            }
            if (L.njobs > 0) dr.launches.push_back(L);
            for (auto const &[rR, rlist] : rest) {
              Launch W;
              W.group = grp;
              W.R = rR;
              W.sched = ws;
              W.job_first = all_jobs.size();
              W.njobs = static_cast<int>(rlist.size());
              for (Stage const *st : rlist) {
                LiftJob job = st->job;
                job.tile_begin = W.tiles;
                W.tiles += st->tiles;
                W.points += stage_points(*st);
                all_jobs.push_back(job);
              }
              dr.launches.push_back(W);
            }
            continue;
          }
          Launch L;
          L.group = grp;
          L.R = R;
          L.sched = ws;
          for (Stage const *st : list)
            if (ws < 0 || !canonical_shifts(st->job, (ws & 1) != 0))
              L.sched = -1;
          L.job_first = all_jobs.size();
          L.njobs = static_cast<int>(list.size());
          for (Stage const *st : list) {
            LiftJob job = st->job;
            job.tile_begin = L.tiles;
            L.tiles += st->tiles;
            L.points += stage_points(*st);
            all_jobs.push_back(job);
          }
          if (L.R != 0 && L.tiles > 0) dr.launches.push_back(L);
        }
      }
    }
    // The group's slab launch, after every per-axis stage of its grids.
    Launch L;
    L.group = grp;
    L.R = kSlab;
    L.sched = ws;
    L.job_first = all_slabs.size();
    L.tile_first = slab_tiles.size();
    for (int g : members) {
      if (slab_from[g] >= b.ndim) continue;
      SlabJob job = slab_job(b, g, slab_from[g], levels, lmin, grid_ptrs);
      job.tile_begin = L.tiles;
      int64_t total = 0;
      for (int k = 0; k < b.ndim; ++k) total += levels[g * b.ndim + k];
      long long const tiles = 1LL << (total - job.log2_tile);
      slab_tiles.insert(slab_tiles.end(), tiles, L.njobs);
      L.tiles += tiles;
      L.points += 1LL << total;
      all_slabs.push_back(job);
      ++L.njobs;
    }
    if (L.njobs > 0) dr.launches.push_back(L);
  }
  if (!all_slabs.empty()) {
    size_t const bytes = all_slabs.size() * sizeof(SlabJob);
    cuda_check(cudaMalloc(&dr.slab_dev, bytes), "cudaMalloc(slab jobs)");
    cuda_check(cudaMemcpy(dr.slab_dev, all_slabs.data(), bytes,
                          cudaMemcpyHostToDevice),
               "cudaMemcpy(slab jobs)");
    size_t const tbytes = slab_tiles.size() * sizeof(int);
    cuda_check(cudaMalloc(&dr.slab_tile_dev, tbytes),
               "cudaMalloc(slab tiles)");
    cuda_check(cudaMemcpy(dr.slab_tile_dev, slab_tiles.data(), tbytes,
                          cudaMemcpyHostToDevice),
               "cudaMemcpy(slab tiles)");
  }
  if (!all_twide.empty()) {
    size_t const jb = all_twide.size() * sizeof(TWideJob);
    cuda_check(cudaMalloc(&dr.twide_dev, jb), "cudaMalloc(twide jobs)");
    cuda_check(cudaMemcpy(dr.twide_dev, all_twide.data(), jb,
                          cudaMemcpyHostToDevice),
               "cudaMemcpy(twide jobs)");
    size_t const tb = twide_tiles.size() * sizeof(int);
    cuda_check(cudaMalloc(&dr.twide_tile_dev, tb), "cudaMalloc(twide tiles)");
    cuda_check(cudaMemcpy(dr.twide_tile_dev, twide_tiles.data(), tb,
                          cudaMemcpyHostToDevice),
               "cudaMemcpy(twide tiles)");
    size_t const mb = maps.size() * sizeof(CUtensorMap);
    cuda_check(cudaMalloc(&dr.maps_dev, mb), "cudaMalloc(tensor maps)");
    cuda_check(cudaMemcpy(dr.maps_dev, maps.data(), mb,
                          cudaMemcpyHostToDevice),
               "cudaMemcpy(tensor maps)");
  }
  if (!all_jobs.empty()) {
    size_t const bytes = all_jobs.size() * sizeof(LiftJob);
    cuda_check(cudaMalloc(&dr.jobs_dev, bytes), "cudaMalloc(jobs)");
    cuda_check(cudaMemcpy(dr.jobs_dev, all_jobs.data(), bytes,
                          cudaMemcpyHostToDevice),
               "cudaMemcpy(jobs)");
  }
}

// One launch of a direction's plan: a lifting kernel or a slab kernel.
void launch_one(paliwa_gb_batch &b, Direction &dr, Launch const &L,
                cudaStream_t s) {
  if (L.R > kTWide) {
    TWideParams p;
    std::memset(&p, 0, sizeof(p));
    p.maps = dr.maps_dev;
    p.jobs = dr.twide_dev + L.job_first;
    p.tile_job = dr.twide_tile_dev + L.tile_first;
    p.total_tiles = L.tiles;
    p.error = b.slab_error;
    p.ctas_per_sm = b.ctas_per_sm;
    launch_twide_f32c(L.sched, L.R - kTWide, p, s);
    return;
  }
  if (L.R != kSlab) {
    LiftParams lp = dr.params;
    lp.ctas_per_sm = b.ctas_per_sm;
    launch_lift(b.dtype, dr.exact, dr.symmetric, L.sched, L.R, lp,
                dr.jobs_dev + L.job_first, L.njobs, L.tiles, s);
    return;
  }
  SlabParams p;
  std::memset(&p, 0, sizeof(p));
  p.ctas_per_sm = b.ctas_per_sm;
  p.map = b.slab_map;
  p.jobs = dr.slab_dev + L.job_first;
  p.tile_job = dr.slab_tile_dev + L.tile_first;
  p.njobs = L.njobs;
  p.total_tiles = L.tiles;
  p.error = b.slab_error;
  switch (b.dtype) {
  case PALIWA_GB_F64: return launch_slab_f64(L.sched, p, s);
  case PALIWA_GB_F32: return launch_slab_f32(L.sched, p, s);
  case PALIWA_GB_F32C: return launch_slab_f32c(L.sched, p, s);
  }
  throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "unknown dtype");
}

void run_direction(paliwa_gb_batch &b, Direction &dr, cudaStream_t s) {
  // Group 0 runs on the caller's stream, group k > 0 on streams[k - 1],
  // forked after the work already queued on `s` and joined back into it.
  auto launch_all = [&] {
    if (b.ngroups > 1)
      cuda_check(cudaEventRecord(b.events[0], s), "cudaEventRecord(fork)");
    for (int k = 1; k < b.ngroups; ++k)
      cuda_check(cudaStreamWaitEvent(b.streams[k - 1], b.events[0], 0),
                 "cudaStreamWaitEvent(fork)");
    for (auto const &L : dr.launches)
      launch_one(b, dr, L, L.group == 0 ? s : b.streams[L.group - 1]);
    for (int k = 1; k < b.ngroups; ++k) {
      cuda_check(cudaEventRecord(b.events[k], b.streams[k - 1]),
                 "cudaEventRecord(join)");
      cuda_check(cudaStreamWaitEvent(s, b.events[k], 0),
                 "cudaStreamWaitEvent(join)");
    }
  };
  cudaStreamCaptureStatus status = cudaStreamCaptureStatusNone;
  if (s != nullptr)
    cuda_check(cudaStreamIsCapturing(s, &status), "cudaStreamIsCapturing");
  // The legacy default stream cannot be captured; a stream that is already
  // capturing records our launches (and the fork) into the caller's graph.
  if (!b.use_graphs || s == nullptr || status != cudaStreamCaptureStatusNone) {
    launch_all();
    return;
  }
  if (dr.graph == nullptr) {
    cudaGraph_t graph = nullptr;
    cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
               "cudaStreamBeginCapture");
    try {
      launch_all();
    } catch (...) {
      cudaStreamEndCapture(s, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    cuda_check(cudaStreamEndCapture(s, &graph), "cudaStreamEndCapture");
    cudaError_t const e = cudaGraphInstantiate(&dr.graph, graph, 0);
    cudaGraphDestroy(graph);
    cuda_check(e, "cudaGraphInstantiate");
  }
  cuda_check(cudaGraphLaunch(dr.graph, s), "cudaGraphLaunch");
}

// Deals the grids, largest first, round-robin into groups, and sizes each
// group's shadow region (the largest per-axis total over the group's grids
// whose pencils along that axis need windowed stages).
void assign_groups(paliwa_gb_batch &b, int64_t const *levels,
                   int64_t const *lmin, int want) {
  size_t const es = dtype_size(b.dtype);
  std::vector<int> order(b.ngrids);
  std::vector<int> log2size(b.ngrids, 0);
  for (int g = 0; g < b.ngrids; ++g) {
    order[g] = g;
    for (int d = 0; d < b.ndim; ++d)
      log2size[g] += static_cast<int>(levels[g * b.ndim + d]);
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    return log2size[a] > log2size[c];
  });
  b.ngroups = std::max(1, std::min(want, b.ngrids));
  b.group.assign(b.ngrids, 0);
  for (int i = 0; i < b.ngrids; ++i) b.group[order[i]] = i % b.ngroups;
  b.group_shadow.assign(b.ngroups, 0);
  b.shadow_bytes = 0;
  for (int k = 0; k < b.ngroups; ++k) {
    size_t need = 0;
    for (int d = 0; d < b.ndim; ++d) {
      size_t total = 0;
      for (int g = 0; g < b.ngrids; ++g) {
        if (b.group[g] != k) continue;
        int64_t const *lv = levels + static_cast<size_t>(g) * b.ndim;
        if (lv[d] <= kWindowLog2 || lv[d] == lmin[d]) continue;
        size_t bytes = es;
        for (int j = 0; j < b.ndim; ++j) bytes <<= lv[j];
        total += (bytes + 255) / 256 * 256;
      }
      need = std::max(need, total);
    }
    b.group_shadow[k] = b.shadow_bytes;
    b.shadow_bytes += need;
  }
}

void free_batch_streams(paliwa_gb_batch &b) {
  for (cudaStream_t st : b.streams)
    if (st != nullptr) cudaStreamDestroy(st);
  for (cudaEvent_t ev : b.events)
    if (ev != nullptr) cudaEventDestroy(ev);
  b.streams.clear();
  b.events.clear();
}

// (Re)groups the batch into `want` groups and plans both directions (keeping
// the autotuner's choices): shadow regions, branch streams and events.
void setup_groups(paliwa_gb_batch &b, int want) {
  free_direction(b.dir[0]);
  free_direction(b.dir[1]);
  free_batch_streams(b);
  if (b.shadow) cudaFree(b.shadow);
  b.shadow = nullptr;
  assign_groups(b, b.levels.data(), b.lmin.data(), want);
  setup_slab_map(b);
  if (b.shadow_bytes)
    cuda_check(cudaMalloc(&b.shadow, b.shadow_bytes), "cudaMalloc(shadow)");
  b.events.assign(b.ngroups, nullptr);
  for (auto &ev : b.events)
    cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming),
               "cudaEventCreate");
  b.streams.assign(b.ngroups - 1, nullptr);
  for (auto &st : b.streams)
    cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking),
               "cudaStreamCreate");
  plan_direction(b, b.dir[0], true, b.levels.data(), b.lmin.data(),
                 b.grids.data());
  plan_direction(b, b.dir[1], false, b.levels.data(), b.lmin.data(),
                 b.grids.data());
}

} // namespace

// ---------------------------------------------------------------------------
// Combination technique.

struct paliwa_gb_ct {
  int ndim = 0;
  int ngrids = 0;
  int dtype = 0;
  long long npoints = 0;
  std::vector<std::vector<int>> subspace_levels;  // lexicographic order
  std::vector<long long> offsets;
  CtSubspace *subspaces_dev = nullptr;
  int *lists_dev = nullptr;
  CtGrid *grids_dev = nullptr;
  int *heavy_dev = nullptr;
  long long *heavy_first_dev = nullptr;
  int *block_sub_dev = nullptr;
  CtParams params{};
};

namespace {

// Key of a level vector (<= 12 dims, levels <= 30: 5 bits each).
uint64_t level_key(int const *s, int ndim) {
  uint64_t k = 0;
  for (int d = 0; d < ndim; ++d) k = (k << 5) | static_cast<uint64_t>(s[d]);
  return k;
}

void build_ct(paliwa_gb_ct &ct, int64_t const *levels,
              double const *coefficients, int64_t const *lmax,
              void *const *grid_ptrs, int keep_all) {
  int const nd = ct.ndim;
  // Count every hierarchical subspace 0 <= s <= l of every grid
  // (paliwa_utils.hpp:9-26; test_paliwa_combination_technique.cpp:177-192).
  std::unordered_map<uint64_t, int> count;
  std::vector<int> s(nd);
  for (int g = 0; g < ct.ngrids; ++g) {
    int64_t const *lv = levels + static_cast<size_t>(g) * nd;
    std::fill(s.begin(), s.end(), 0);
    while (true) {
      ++count[level_key(s.data(), nd)];
      int d = nd - 1;
      while (d >= 0 && s[d] == lv[d]) s[d--] = 0;
      if (d < 0) break;
      ++s[d];
    }
  }
  // Keep subspaces present in more than one grid (:212-225), ordered like
  // the reference's std::map (lexicographic on the level vector).
  std::vector<std::vector<int>> kept;
  for (auto const &[key, c] : count) {
    if (c <= 1 && !keep_all) continue;
    std::vector<int> v(nd);
    uint64_t k = key;
    for (int d = nd - 1; d >= 0; --d) {
      v[d] = static_cast<int>(k & 31);
      k >>= 5;
    }
    kept.push_back(v);
  }
  std::sort(kept.begin(), kept.end());
  std::vector<CtSubspace> subs(kept.size());
  std::vector<int> lists;
  long long off = 0;
  for (size_t i = 0; i < kept.size(); ++i) {
    CtSubspace &ss = subs[i];
    std::memset(&ss, 0, sizeof(ss));
    ss.offset = off;
    long long size = 1;
    for (int d = 0; d < nd; ++d) {
      ss.level[d] = static_cast<signed char>(kept[i][d]);
      if (kept[i][d] > 0) size <<= (kept[i][d] - 1);
    }
    off += size;
    ss.grid_begin = static_cast<int>(lists.size());
    for (int g = 0; g < ct.ngrids; ++g) {
      bool contains = true;  // :270-276
      for (int d = 0; d < nd; ++d)
        if (kept[i][d] > levels[static_cast<size_t>(g) * nd + d]) {
          contains = false;
          break;
        }
      if (contains) lists.push_back(g);
    }
    ss.grid_end = static_cast<int>(lists.size());
  }
  ct.npoints = off;
  ct.subspace_levels = kept;
  ct.offsets.resize(kept.size());
  for (size_t i = 0; i < kept.size(); ++i) ct.offsets[i] = subs[i].offset;
  std::vector<CtGrid> grids(ct.ngrids);
  for (int g = 0; g < ct.ngrids; ++g) {
    std::memset(&grids[g], 0, sizeof(CtGrid));
    grids[g].base = reinterpret_cast<unsigned long long>(grid_ptrs[g]);
    grids[g].coefficient = coefficients[g];
    for (int d = 0; d < nd; ++d)
      grids[g].level[d] =
          static_cast<signed char>(levels[static_cast<size_t>(g) * nd + d]);
  }
  auto upload = [](auto **dst, auto const &v, char const *what) {
    if (v.empty()) return;
    size_t const bytes = v.size() * sizeof(v[0]);
    cuda_check(cudaMalloc(reinterpret_cast<void **>(dst), bytes), what);
    cuda_check(cudaMemcpy(*dst, v.data(), bytes, cudaMemcpyHostToDevice),
               what);
  };
  std::vector<int> heavy;
  std::vector<long long> heavy_first;
  long long nheavy_points = 0;
  for (size_t i = 0; i < subs.size(); ++i) {
    if (subs[i].grid_end - subs[i].grid_begin <= kCtHeavy) continue;
    heavy.push_back(static_cast<int>(i));
    heavy_first.push_back(nheavy_points);
    long long const next =
        i + 1 < subs.size() ? subs[i + 1].offset : off;
    nheavy_points += next - subs[i].offset;
  }
  upload(&ct.subspaces_dev, subs, "upload subspaces");
  upload(&ct.lists_dev, lists, "upload grid lists");
  upload(&ct.grids_dev, grids, "upload grids");
  upload(&ct.heavy_dev, heavy, "upload heavy subspaces");
  upload(&ct.heavy_first_dev, heavy_first, "upload heavy offsets");
  // First subspace of every CTA's 256 points (the subspace holding point
  // 256 b), so that no CTA searches the whole subspace list.
  std::vector<int> block_sub((off + kCtBlock - 1) / kCtBlock);
  {
    size_t si = 0;
    for (size_t b = 0; b < block_sub.size(); ++b) {
      long long const first = static_cast<long long>(b) * kCtBlock;
      while (si + 1 < subs.size() && subs[si + 1].offset <= first) ++si;
      block_sub[b] = static_cast<int>(si);
    }
  }
  upload(&ct.block_sub_dev, block_sub, "upload block subspaces");
  std::memset(&ct.params, 0, sizeof(ct.params));
  ct.params.subspaces = ct.subspaces_dev;
  ct.params.nsubspaces = static_cast<int>(subs.size());
  ct.params.grid_lists = ct.lists_dev;
  ct.params.grids = ct.grids_dev;
  ct.params.ndim = nd;
  ct.params.npoints = ct.npoints;
  for (int d = 0; d < nd && d < kMaxDims; ++d)
    ct.params.max_level[d] = static_cast<signed char>(lmax[d]);
  ct.params.heavy = ct.heavy_dev;
  ct.params.heavy_first = ct.heavy_first_dev;
  ct.params.block_sub = ct.block_sub_dev;
  ct.params.nheavy = static_cast<int>(heavy.size());
  ct.params.nheavy_points = nheavy_points;
  // Products c * v are exact in FP64 when c has at most 53 - 24 = 29
  // significant bits and v is a float (whose magnitude lies in
  // [2^-149, 2^128]), provided |c| stays within [2^-500, 2^500] so that the
  // product neither underflows nor overflows. For FP64 grids only |c| = 1
  // is exact for every value.
  bool exact = true;
  for (int g = 0; g < ct.ngrids && exact; ++g) {
    double const c = coefficients[g];
    if (c == 0.0) continue;
    if (!std::isfinite(c)) {
      exact = false;
      break;
    }
    if (ct.dtype == PALIWA_GB_F64) {
      exact = std::fabs(c) == 1.0;
      continue;
    }
    int e = 0;
    double m = std::frexp(std::fabs(c), &e);  // m in [0.5, 1)
    long long bits = static_cast<long long>(std::ldexp(m, 53));
    int sig = 53;
    while ((bits & 1) == 0) {
      bits >>= 1;
      --sig;
    }
    if (sig > 29 || e < -500 || e > 500) exact = false;
  }
  ct.params.exact_products = exact ? 1 : 0;
}

template <int OP>
void ct_launch(paliwa_gb_ct const &ct, double *sparse, double *full,
               cudaStream_t s) {
  if (ct.npoints == 0) return;
  CtParams p = ct.params;
  p.sparse = sparse;
  p.full = full;
  unsigned const blocks =
      static_cast<unsigned>((ct.npoints + kCtBlock - 1) / kCtBlock);
  switch (ct.dtype) {
  case PALIWA_GB_F64:
    ct_kernel<double, OP><<<blocks, kCtBlock, 0, s>>>(p);
    break;
  case PALIWA_GB_F32:
  case PALIWA_GB_F32C:
    ct_kernel<float, OP><<<blocks, kCtBlock, 0, s>>>(p);
    break;
  default: throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "unknown dtype");
  }
  cuda_check(cudaGetLastError(), "ct_kernel launch");
  if (OP == kRestrict && p.nheavy_points > 0) {
    unsigned const hblocks =
        static_cast<unsigned>((p.nheavy_points * 32 + 255) / 256);
    if (ct.dtype == PALIWA_GB_F64)
      ct_heavy_restrict_kernel<double><<<hblocks, 256, 0, s>>>(p);
    else
      ct_heavy_restrict_kernel<float><<<hblocks, 256, 0, s>>>(p);
    cuda_check(cudaGetLastError(), "ct_heavy_restrict_kernel launch");
  }
}

} // namespace

extern "C" {

int paliwa_gb_batch_create(int ndim, int ngrids, const int64_t *levels,
                           const int64_t *minimum_level,
                           const int64_t *maximum_level, int dtype,
                           int wavelet, void *const *grid_ptrs,
                           paliwa_gb_batch **out) {
  return guarded([&] {
    if (out == nullptr || levels == nullptr || minimum_level == nullptr ||
        maximum_level == nullptr || grid_ptrs == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    check_grid_levels(ndim, ngrids, levels, minimum_level, maximum_level);
    size_t const es = dtype_size(dtype);
    wavelet_filters(wavelet, true);  // validates the id
    auto b = std::make_unique<paliwa_gb_batch>();
    b->ndim = ndim;
    b->ngrids = ngrids;
    b->dtype = dtype;
    b->wavelet = wavelet;
    b->levels.assign(levels, levels + static_cast<size_t>(ngrids) * ndim);
    b->lmin.assign(minimum_level, minimum_level + ndim);
    b->grids.assign(grid_ptrs, grid_ptrs + ngrids);
    for (int g = 0; g < ngrids; ++g) {
      if (grid_ptrs[g] == nullptr ||
          reinterpret_cast<uintptr_t>(grid_ptrs[g]) % es != 0)
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "grid pointer is null or misaligned");
      int64_t total = 0;
      for (int d = 0; d < ndim; ++d) total += levels[g * ndim + d];
      b->points += 1LL << total;
    }
    try {
      cuda_check(cudaMalloc(&b->slab_error, sizeof(unsigned)),
                 "cudaMalloc(error word)");
      cuda_check(cudaMemset(b->slab_error, 0, sizeof(unsigned)),
                 "cudaMemset(error word)");
      setup_groups(*b, kBatchGroups);
    } catch (...) {
      free_direction(b->dir[0]);
      free_direction(b->dir[1]);
      free_batch_streams(*b);
      if (b->shadow) cudaFree(b->shadow);
      if (b->slab_error) cudaFree(b->slab_error);
      throw;
    }
    *out = b.release();
  });
}

int paliwa_gb_batch_hierarchize(paliwa_gb_batch *batch, void *stream) {
  return guarded([&] {
    if (batch == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null batch");
    run_direction(*batch, batch->dir[0], static_cast<cudaStream_t>(stream));
  });
}

int paliwa_gb_batch_dehierarchize(paliwa_gb_batch *batch, void *stream) {
  return guarded([&] {
    if (batch == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null batch");
    run_direction(*batch, batch->dir[1], static_cast<cudaStream_t>(stream));
  });
}

int paliwa_gb_batch_use_graphs(paliwa_gb_batch *batch, int enable) {
  return guarded([&] {
    if (batch == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null batch");
    batch->use_graphs = enable != 0;
  });
}

int paliwa_gb_batch_set_groups(paliwa_gb_batch *batch, int ngroups) {
  return guarded([&] {
    if (batch == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null batch");
    if (ngroups < 1)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "ngroups must be >= 1");
    cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    setup_groups(*batch, ngroups);
  });
}

int paliwa_gb_batch_use_slabs(paliwa_gb_batch *batch, int enable) {
  return guarded([&] {
    if (batch == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null batch");
    cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    batch->use_slabs = enable != 0;
    setup_groups(*batch, batch->ngroups);
  });
}

int paliwa_gb_batch_use_tma(paliwa_gb_batch *batch, int enable) {
  return guarded([&] {
    if (batch == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null batch");
    cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    batch->use_tma = enable != 0;
    setup_groups(*batch, batch->ngroups);
  });
}

int paliwa_gb_batch_set_ctas_per_sm(paliwa_gb_batch *batch, int ctas) {
  return guarded([&] {
    if (batch == nullptr || ctas < 0)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                        "null batch or negative CTA count");
    cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    batch->ctas_per_sm = ctas;
    setup_groups(*batch, batch->ngroups);
  });
}

int paliwa_gb_batch_status(paliwa_gb_batch *batch) {
  return guarded([&] {
    if (batch == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null batch");
    unsigned err = 0;
    cuda_check(cudaMemcpy(&err, batch->slab_error, sizeof(err),
                          cudaMemcpyDeviceToHost),
               "cudaMemcpy(error word)");
    if (err != 0) {
      cuda_check(cudaMemset(batch->slab_error, 0, sizeof(err)),
                 "cudaMemset(error word)");
      throw StatusError(PALIWA_GB_TIMEOUT,
                        "a slab kernel's bounded wait for its tile copy "
                        "gave up");
    }
  });
}

int paliwa_gb_batch_info(const paliwa_gb_batch *batch, int64_t *points,
                         int64_t *launches_forward,
                         int64_t *launches_inverse) {
  return guarded([&] {
    if (batch == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null batch");
    if (points) *points = batch->points;
    if (launches_forward)
      *launches_forward = static_cast<int64_t>(batch->dir[0].launches.size());
    if (launches_inverse)
      *launches_inverse = static_cast<int64_t>(batch->dir[1].launches.size());
  });
}

namespace {

// Milliseconds of direction `which` (0 forward, 1 inverse), best of `reps`
// event-timed runs as the batch runs them (its groups on parallel branches,
// from a graph when graphs are on: a plan's speed depends on how its
// launches overlap); every run is followed (forward) or preceded (inverse)
// by the other direction, so that the grids return to their contents up to
// rounding.
float time_direction(paliwa_gb_batch &b, int which, int reps,
                     cudaStream_t s) {
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
  cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
  auto run = [&](Direction &dr) { run_direction(b, dr, s); };
  float best = 1e30f;
  for (int r = 0; r < reps; ++r) {
    if (which == 1) run(b.dir[0]);
    cuda_check(cudaEventRecord(e0, s), "cudaEventRecord");
    run(b.dir[which]);
    cuda_check(cudaEventRecord(e1, s), "cudaEventRecord");
    if (which == 0) run(b.dir[1]);
    cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
    float ms = 0;
    cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
    best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

void replan(paliwa_gb_batch &b, int which) {
  Direction &dr = b.dir[which];
  free_direction(dr);
  plan_direction(b, dr, which == 0, b.levels.data(), b.lmin.data(),
                 b.grids.data());
}

} // namespace

int paliwa_gb_batch_autotune(paliwa_gb_batch *batch, void *stream, int reps,
                             int *changed) {
  return guarded([&] {
    if (batch == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null batch");
    if (reps < 1) reps = 1;
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    int nchanged = 0;
    for (int which = 0; which < 2; ++which) {
      Direction &dr = batch->dir[which];
      float best = time_direction(*batch, which, reps, s);
      // Slab launches against the same axes planned one by one (either way
      // round, so that a second call can bring the slabs back).
      bool has_slab = false;
      for (auto const &L : dr.launches) has_slab |= L.R == kSlab;
      if (batch->use_slabs && batch->slab_map_ok && (has_slab || !dr.slabs)) {
        dr.slabs = !dr.slabs;
        replan(*batch, which);
        float const t = time_direction(*batch, which, reps, s);
        if (t < best * 0.99f) {
          best = t;
          ++nchanged;
        } else {
          dr.slabs = !dr.slabs;
          replan(*batch, which);
        }
      }
      // Coordinate descent over the classes of periodic stages: try every
      // kernel that applies to a class, keep the fastest whole direction.
      auto const classes = dr.classes;
      long long total = 0;
      for (auto const &kv : classes) total += kv.second.points;
      for (auto const &[tclass, info] : classes) {
        unsigned const mask = info.kernels;
        int const dflt = info.dflt;
        if ((mask & (mask - 1)) == 0) continue;  // one kernel applies
        // A class with under 2 % of the points cannot move the direction's
        // time by the 1 % a change must gain.
        if (info.points * 50 < total) continue;
        auto const it = dr.tuning.choice.find(tclass);
        int const current = it != dr.tuning.choice.end() ? it->second : dflt;
        int keep = current;
        for (int c = 0; c < kChooseCount; ++c) {
          if (c == current || !((mask >> c) & 1u)) continue;
          dr.tuning.choice[tclass] = c;
          replan(*batch, which);
          float const t = time_direction(*batch, which, reps, s);
          if (t < best * 0.99f) {
            best = t;
            keep = c;
          }
        }
        if (keep == dflt && it == dr.tuning.choice.end())
          dr.tuning.choice.erase(tclass);
        else
          dr.tuning.choice[tclass] = keep;
        if (keep != current) ++nchanged;
        replan(*batch, which);
      }
    }
    if (changed != nullptr) *changed = nchanged;
  });
}

int paliwa_gb_batch_tuning(const paliwa_gb_batch *batch, int forward,
                           int capacity, int *nclasses, int32_t *classes,
                           int32_t *kernels, int32_t *choices) {
  return guarded([&] {
    if (batch == nullptr || nclasses == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    Direction const &dr = batch->dir[forward ? 0 : 1];
    *nclasses = static_cast<int>(dr.classes.size());
    if (capacity < *nclasses || classes == nullptr || kernels == nullptr ||
        choices == nullptr)
      return;
    int i = 0;
    for (auto const &[tclass, info] : dr.classes) {
      auto const it = dr.tuning.choice.find(tclass);
      classes[i] = tclass;
      kernels[i] = static_cast<int32_t>(info.kernels);
      choices[i] = it != dr.tuning.choice.end() ? it->second : info.dflt;
      ++i;
    }
  });
}

int paliwa_gb_batch_set_tuning(paliwa_gb_batch *batch, int forward,
                               int nclasses, const int32_t *classes,
                               const int32_t *choices) {
  return guarded([&] {
    if (batch == nullptr || nclasses < 0 ||
        (nclasses > 0 && (classes == nullptr || choices == nullptr)))
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    int const which = forward ? 0 : 1;
    Direction &dr = batch->dir[which];
    // Check every entry before changing anything.
    for (int i = 0; i < nclasses; ++i) {
      auto const it = dr.classes.find(classes[i]);
      if (it == dr.classes.end())
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "no stage of the batch is in tuning class " +
                              std::to_string(classes[i]));
      if (choices[i] < 0 || choices[i] >= kChooseCount ||
          !((it->second.kernels >> choices[i]) & 1u))
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "kernel " + std::to_string(choices[i]) +
                              " does not apply to tuning class " +
                              std::to_string(classes[i]));
    }
    for (int i = 0; i < nclasses; ++i) {
      if (choices[i] == dr.classes.at(classes[i]).dflt)
        dr.tuning.choice.erase(classes[i]);
      else
        dr.tuning.choice[classes[i]] = choices[i];
    }
    replan(*batch, which);
  });
}

int paliwa_gb_batch_profile(paliwa_gb_batch *batch, int forward, void *stream,
                            int capacity, int *nlaunches, float *ms,
                            int64_t *bytes, int32_t *kernels) {
  return guarded([&] {
    if (batch == nullptr || nlaunches == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    Direction &dr = batch->dir[forward ? 0 : 1];
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    int const n = static_cast<int>(dr.launches.size());
    *nlaunches = n;
    if (capacity < n || ms == nullptr || bytes == nullptr) return;
    std::vector<cudaEvent_t> ev(n + 1);
    for (auto &e : ev) cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    size_t const es = dtype_size(batch->dtype);
    cuda_check(cudaEventRecord(ev[0], s), "cudaEventRecord");
    for (int i = 0; i < n; ++i) {
      Launch const &L = dr.launches[i];
      launch_one(*batch, dr, L, s);
      cuda_check(cudaEventRecord(ev[i + 1], s), "cudaEventRecord");
      bytes[i] = static_cast<int64_t>(2 * es) * L.points;
      if (kernels != nullptr) kernels[i] = L.R;
    }
    cuda_check(cudaEventSynchronize(ev[n]), "cudaEventSynchronize");
    for (int i = 0; i < n; ++i)
      cuda_check(cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]),
                 "cudaEventElapsedTime");
    for (auto &e : ev) cudaEventDestroy(e);
  });
}

void paliwa_gb_batch_destroy(paliwa_gb_batch *batch) {
  if (batch == nullptr) return;
  free_direction(batch->dir[0]);
  free_direction(batch->dir[1]);
  free_batch_streams(*batch);
  if (batch->shadow) cudaFree(batch->shadow);
  if (batch->slab_error) cudaFree(batch->slab_error);
  delete batch;
}

int paliwa_gb_ct_create(int ndim, int ngrids, const int64_t *levels,
                        const double *coefficients,
                        const int64_t *maximum_level, int dtype,
                        void *const *grid_ptrs, int keep_all,
                        paliwa_gb_ct **out) {
  return guarded([&] {
    if (out == nullptr || levels == nullptr || coefficients == nullptr ||
        maximum_level == nullptr || grid_ptrs == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    check_grid_levels(ndim, ngrids, levels, nullptr, maximum_level);
    size_t const es = dtype_size(dtype);
    for (int g = 0; g < ngrids; ++g)
      if (grid_ptrs[g] == nullptr ||
          reinterpret_cast<uintptr_t>(grid_ptrs[g]) % es != 0)
        throw StatusError(PALIWA_GB_INVALID_ARGUMENT,
                          "grid pointer is null or misaligned");
    auto ct = std::make_unique<paliwa_gb_ct>();
    ct->ndim = ndim;
    ct->ngrids = ngrids;
    ct->dtype = dtype;
    try {
      build_ct(*ct, levels, coefficients, maximum_level, grid_ptrs, keep_all);
    } catch (...) {
      cudaFree(ct->subspaces_dev);
      cudaFree(ct->lists_dev);
      cudaFree(ct->grids_dev);
      cudaFree(ct->heavy_dev);
      cudaFree(ct->heavy_first_dev);
      cudaFree(ct->block_sub_dev);
      throw;
    }
    *out = ct.release();
  });
}

int paliwa_gb_ct_info(const paliwa_gb_ct *ct, int64_t *npoints,
                      int64_t *nsubspaces) {
  return guarded([&] {
    if (ct == nullptr) throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null ct");
    if (npoints) *npoints = ct->npoints;
    if (nsubspaces)
      *nsubspaces = static_cast<int64_t>(ct->subspace_levels.size());
  });
}

int paliwa_gb_ct_subspaces(const paliwa_gb_ct *ct, int64_t *levels,
                           int64_t *offsets) {
  return guarded([&] {
    if (ct == nullptr) throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null ct");
    for (size_t i = 0; i < ct->subspace_levels.size(); ++i) {
      if (levels)
        for (int d = 0; d < ct->ndim; ++d)
          levels[i * ct->ndim + d] = ct->subspace_levels[i][d];
      if (offsets) offsets[i] = ct->offsets[i];
    }
  });
}

int paliwa_gb_ct_combine(paliwa_gb_ct *ct, double *sparse, void *stream) {
  return guarded([&] {
    if (ct == nullptr || sparse == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    ct_launch<kCombine>(*ct, sparse, nullptr,
                        static_cast<cudaStream_t>(stream));
  });
}

int paliwa_gb_ct_restrict(paliwa_gb_ct *ct, const double *sparse,
                          void *stream) {
  return guarded([&] {
    if (ct == nullptr || sparse == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    ct_launch<kRestrict>(*ct, const_cast<double *>(sparse), nullptr,
                         static_cast<cudaStream_t>(stream));
  });
}

int paliwa_gb_ct_scatter(paliwa_gb_ct *ct, const double *sparse, double *full,
                         void *stream) {
  return guarded([&] {
    if (ct == nullptr || sparse == nullptr || full == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "null argument");
    // The full grid starts from zero (test_paliwa_combination_technique.cpp
    // :295-298); every kept subspace point is then added once.
    long long total = 0;
    for (int d = 0; d < ct->ndim; ++d) total += ct->params.max_level[d];
    if (total > 36)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "full grid too large");
    cuda_check(cudaMemsetAsync(full, 0, sizeof(double) << total,
                               static_cast<cudaStream_t>(stream)),
               "cudaMemsetAsync");
    ct_launch<kScatter>(*ct, const_cast<double *>(sparse), full,
                        static_cast<cudaStream_t>(stream));
  });
}

void paliwa_gb_ct_destroy(paliwa_gb_ct *ct) {
  if (ct == nullptr) return;
  cudaFree(ct->subspaces_dev);
  cudaFree(ct->lists_dev);
  cudaFree(ct->grids_dev);
  cudaFree(ct->heavy_dev);
  cudaFree(ct->heavy_first_dev);
  cudaFree(ct->block_sub_dev);
  delete ct;
}

} // extern "C"
