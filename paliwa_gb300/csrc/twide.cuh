// TMA wide kernel: the wide kernel's register transform (rows of two
// adjacent columns as double-float f32x2 pairs, chunks of one pencil in
// lanes 32 / G apart, shuffles only) for strided axes with pencils of up to
// 64 points, with the data moved by the tensor memory accelerator instead
// of per-thread copies.
//
// A tile is one unit of the wide kernel: NT threads x R rows x 2 columns =
// Ct = 2 NT / G consecutive columns (column = (outer index, inner index)) of
// all n rows of their pencils. Each grid and axis has a 3D tensor map over
// its [outer][n][inner] view (strides of the axis: sub-lattices included);
// a tile is 1 or 2 boxes {Bx columns of one outer index, n rows, Sx outer
// indices} (Bx = min(inner, Ct, 256), Sx = Ct / inner when inner < Ct),
// loaded into shared memory as [box][outer][row][column], completion on an
// mbarrier with a bounded wait. After the transform the threads write their
// rows back into the same place and one thread stores the boxes with bulk
// tensor stores. Columns past the end of the grid are read as zeros and not
// stored (the tensor map's bounds). Each CTA keeps S tiles in flight: the
// copies are asynchronous and issued by one thread, which removes the
// per-thread copy instructions that throttled the wide kernel's memory
// pipeline (measured on a copy-only build: MIO throttle of 10 per issue).
//
// The maps live in global memory, written by the host before the launch;
// they cover only this GPU's grid memory (no multicast).
#pragma once

#include <cstdint>
#include <cuda.h>

#include "lift.cuh"
#include "slab.cuh"

namespace pgb {

constexpr int kTWideThreads = 256;

struct TWideJob {
  long long tile_begin;  // first tile of this job in the launch
  int map;               // index of the job's tensor map
  int log2_n;            // pencil length
  int log2_inner;        // columns per outer index
  int nlevels;
  int log2_bx;           // box: 2^log2_bx columns of one outer index
  int log2_sx;           // box: 2^log2_sx outer indices
  int nxb;               // boxes per tile
  int pad_;
};

struct TWideParams {
  CUtensorMap const *maps;  // 64-byte aligned, in global memory
  TWideJob const *jobs;     // sorted by tile_begin
  int const *tile_job;      // the job of every tile of the launch
  long long total_tiles;
  unsigned *error;          // set to 1 when a bounded wait gives up
  int ctas_per_sm;          // cap on the launch's CTAs per SM (0: none)
};

__device__ __forceinline__ void tma_load_3d(void *dst, void const *map, int x,
                                            int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx"
      "::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z),
      "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_3d(void const *map, int x, int y,
                                             int z, void const *src) {
  asm volatile(
      "cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, "
      "%3}], [%4];\n" ::"l"(reinterpret_cast<unsigned long long>(map)),
      "r"(x), "r"(y), "r"(z), "r"(smem_u32(src))
      : "memory");
}
// Orders the host's writes of a tensor map in global memory before its use
// by the tensor memory accelerator.
__device__ __forceinline__ void fence_tensormap(void const *map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(
                   reinterpret_cast<unsigned long long>(map))
               : "memory");
}

// A tile is kUnits units of Ct * n * 4 = (2 NT / G) * (G R) * 4 bytes
// (16 KB tiles for chunks of up to 8 points: per-tile synchronisation
// dominated 8 KB ones). kStages tiles per CTA: one transformed, kLook
// loading ahead, and kDefer whose stores may still be reading shared memory
// when a buffer is reloaded (so the reload does not wait for the store just
// issued).
template <int R> struct TWideShape {
  static constexpr int kUnits = R >= 8 ? 1 : 8 / R;
  static constexpr int kUnitBytes = 8 * kTWideThreads * R;
  static constexpr int kTileBytes = kUnits * kUnitBytes;
  static constexpr int kStages = R >= 16 ? 3 : 4;
  static constexpr int kDefer = R >= 16 ? 0 : 1;
  static constexpr int kLook = kStages - 1 - kDefer;
  static constexpr size_t kSmemBytes =
      size_t(kStages) * kTileBytes + 128;  // + 128-byte alignment slack
};

__device__ __forceinline__ void bulk_wait_read_1() {
  asm volatile("cp.async.bulk.wait_group.read 1;\n" ::: "memory");
}
template <int R> constexpr size_t twide_smem_bytes() {
  return TWideShape<R>::kSmemBytes;
}

template <class A, int R, class Sched>
__global__ void __launch_bounds__(kTWideThreads, R >= 16 ? 2 : R == 8 ? 3 : 4)
    twide_kernel(__grid_constant__ const TWideParams p) {
  using V = typename A::V;
  using W = typename A::Store;
  static_assert(sizeof(W) == 8, "rows of two float columns");
  constexpr int NT = kTWideThreads;
  constexpr int S = TWideShape<R>::kStages;
  constexpr int TILE = TWideShape<R>::kTileBytes;
  constexpr int U = TWideShape<R>::kUnits;
  constexpr int UNIT = TWideShape<R>::kUnitBytes;
  constexpr int LOOK = TWideShape<R>::kLook;
  constexpr int DEFER = TWideShape<R>::kDefer;
  constexpr int LOG2R = Log2<R>::value;
  constexpr int LOG2NT = Log2<NT>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned const base_addr = smem_u32(smem_raw);
  unsigned char *const tiles =
      smem_raw + ((128 - (base_addr & 127)) & 127);  // 128-byte aligned
  __shared__ uint64_t full[S];
  __shared__ TWideJob sjob[S];

  int const t = threadIdx.x;
  int const lane = t & 31;
  long long const first = blockIdx.x;
  long long const step = gridDim.x;
  if (first >= p.total_tiles) return;
  long long const ntiles = (p.total_tiles - first + step - 1) / step;

  if (t == 0) {
    for (int b = 0; b < S; ++b) mbar_init(&full[b], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // Unit u of tile `tile` of `job`: its first column's (inner, outer)
  // coordinates.
  auto origin = [](TWideJob const &job, long long tile, int u, int &x0,
                   int &z0) {
    int const log2ct = LOG2NT + 1 - (job.log2_n - LOG2R);
    long long const col0 = ((tile - job.tile_begin) * U + u) << log2ct;
    z0 = static_cast<int>(col0 >> job.log2_inner);
    x0 = static_cast<int>(col0 & ((1LL << job.log2_inner) - 1));
  };
  // The tile's boxes: along the inner index when one outer index holds the
  // tile (Sx == 1), else along the outer index.
  auto box_at = [](TWideJob const &job, int xb, int x0, int z0, int &x,
                   int &z) {
    x = x0;
    z = z0;
    if (job.log2_sx == 0)
      x += xb << job.log2_bx;
    else
      z += xb << job.log2_sx;
  };
  auto box_bytes = [](TWideJob const &job) {
    return 4 << (job.log2_bx + job.log2_n + job.log2_sx);
  };

  // Thread 0 issues every copy; it keeps the last map it fenced.
  int fenced = -1;
  auto issue_load = [&](long long k) {
    int const b = static_cast<int>(k % S);
    long long const tile = first + k * step;
    sjob[b] = p.jobs[p.tile_job[tile]];
    TWideJob const &job = sjob[b];
    void const *const map = p.maps + job.map;
    if (job.map != fenced) {
      fence_tensormap(map);
      fenced = job.map;
    }
    int const bb = box_bytes(job);
    mbar_expect_tx(&full[b], static_cast<unsigned>(U * bb * job.nxb));
    for (int u = 0; u < U; ++u) {
      int x0, z0;
      origin(job, tile, u, x0, z0);
      unsigned char *const dst = tiles + b * TILE + u * UNIT;
      for (int xb = 0; xb < job.nxb; ++xb) {
        int x, z;
        box_at(job, xb, x0, z0, x, z);
        tma_load_3d(dst + xb * bb, map, x, 0, z, &full[b]);
      }
    }
  };
  auto issue_store = [&](long long k) {
    int const b = static_cast<int>(k % S);
    long long const tile = first + k * step;
    TWideJob const &job = sjob[b];
    void const *const map = p.maps + job.map;
    int const bb = box_bytes(job);
    for (int u = 0; u < U; ++u) {
      int x0, z0;
      origin(job, tile, u, x0, z0);
      unsigned char const *const src = tiles + b * TILE + u * UNIT;
      for (int xb = 0; xb < job.nxb; ++xb) {
        int x, z;
        box_at(job, xb, x0, z0, x, z);
        tma_store_3d(map, x, 0, z, src + xb * bb);
      }
    }
    bulk_commit();
  };

  long long issued = 0;
  if (t == 0)
    for (; issued < LOOK && issued < ntiles; ++issued) issue_load(issued);

  long long k = 0;
  bool failed = false;
  for (; k < ntiles; ++k) {
    int const b = static_cast<int>(k % S);
    if (t == 0 && issued < ntiles) {
      // The buffer of tile k + LOOK held tile k + LOOK - S = k - 1 - DEFER:
      // its stores (all but the DEFER most recent store groups) must have
      // read it.
      if constexpr (DEFER == 0)
        bulk_wait_read_all();
      else
        bulk_wait_read_1();
      issue_load(issued);
      ++issued;
    }
    // Bounded wait for tile k (about a second of clock), then a vote so
    // that every thread leaves together if it gave up.
    unsigned const parity = static_cast<unsigned>((k / S) & 1);
    bool done = false;
    long long const t0 = clock64();
    while (!(done = mbar_try_wait(&full[b], parity)))
      if (clock64() - t0 > (1LL << 31)) break;
    if (!__syncthreads_and(done)) {
      failed = true;
      break;
    }
    TWideJob const &job = sjob[b];
    // Thread = (chunk c, column pair g): the chunks of a column pair are
    // lanes W = 32 / G apart, the W column pairs of one chunk consecutive.
    int const log2G = job.log2_n - LOG2R;
    int const log2W = 5 - log2G;
    int const c = lane >> log2W;
    int const g = ((t >> 5) << log2W) | (lane & ((1 << log2W) - 1));
    int const col = 2 * g;
    int const log2bs = job.log2_bx + job.log2_sx;
    int const xb = col >> log2bs;
    int const rem = col & ((1 << log2bs) - 1);
    int const s = rem >> job.log2_bx;
    int const bcol = rem & ((1 << job.log2_bx) - 1);
    // float index of row c R of the thread's columns; rows are Bx apart
    int const idx0 = (xb << (log2bs + job.log2_n)) +
                     ((((s << job.log2_n) + (c << LOG2R)) << job.log2_bx) +
                      bcol);
    for (int u = 0; u < U; ++u) {
      float *const tf =
          reinterpret_cast<float *>(tiles + b * TILE + u * UNIT);
      V v[R];
#pragma unroll
      for (int j = 0; j < R; ++j)
        v[j] = A::load(
            *reinterpret_cast<W const *>(tf + idx0 + (j << job.log2_bx)));
      RoundCtx<A, NT> ctx(t, c, 1 << log2G, log2G, lane, 1, nullptr, nullptr,
                          log2W);
      Sched::template run_levels<A, R, NT>(v, ctx, job.nlevels);
#pragma unroll
      for (int j = 0; j < R; ++j)
        *reinterpret_cast<W *>(tf + idx0 + (j << job.log2_bx)) =
            A::store(v[j]);
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (t == 0) issue_store(k);
  }
  if (t == 0) {
    if (failed) {
      atomicExch(p.error, 1u);
      // Wait (bounded) for the loads still in flight before the CTA's
      // shared memory goes away.
      for (long long q = k; q < issued; ++q) {
        unsigned const par = static_cast<unsigned>((q / S) & 1);
        long long const t0 = clock64();
        while (!mbar_try_wait(&full[q % S], par))
          if (clock64() - t0 > (1LL << 31)) break;
      }
    }
    bulk_wait_all();
  }
}

} // namespace pgb
