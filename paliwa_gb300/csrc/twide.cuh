// TMA wide kernel: the wide kernel's register transform (rows of two
// adjacent columns as double-float f32x2 pairs, chunks of one pencil in
// lanes, shuffles) for strided pencils of up to 2048 points (G <= 128
// chunks) and the last axis' pencils of up to 4096 points, with the data
// moved by the tensor memory accelerator instead of per-thread copies.
//
// A tile is one unit of the wide kernel (several for chunks of up to 8
// points): NT threads x R rows x 2 columns = Ct = 2 NT / G consecutive
// columns (column = (outer index, inner index)) of all n rows of their
// pencils. Each grid and axis has a tensor map, in one of four layouts:
//  * dense (up to 4 chunks): a 3D map over the [outer][n][inner] view
//    (strides of the axis: sub-lattices included); a tile is 1 or 2 boxes
//    {Bx columns of one outer index, n rows, Sx outer indices} (Bx =
//    min(inner, Ct, 256), Sx = Ct / inner when inner < Ct), in shared
//    memory as [box][outer][row][column];
//  * chunk-interleaved (8 to 128 chunks of 16 points): a 5D map {X columns,
//    G chunks, R rows of a chunk, column groups, outer index} (X = 4 or 8)
//    and one box per tile, in shared memory as [column group][row of
//    chunk][chunk][X columns], so that the chunks a warp reads together lie
//    in consecutive X-column groups (with the dense layout they would read
//    rows R apart, on the same banks; a pad after a box per chunk is not
//    possible, since bulk tensor copies need 128-byte aligned shared-memory
//    destinations);
//  * contiguous (the last axis) and pairs (strided, inner extent 2): the
//    stage's points as 128-byte rows of a 2D map with the 128-byte swizzle,
//    see FORMs 3 and 4 of twide_kernel.
// Completion is on an mbarrier with a bounded wait. After the transform the
// threads write their rows back into the same place and one thread stores
// the boxes with bulk tensor stores. Columns past the end of the grid are
// read as zeros and not stored (the tensor map's bounds). The copies are
// asynchronous and issued by one thread, which removes the per-thread copy
// instructions that throttled the wide kernel's memory pipeline (measured
// on a copy-only build: MIO throttle of 10 per issue).
//
// twide_kernel's CTA is warp-specialised: NT transform threads (eight
// warps) and one producer warp, of which one lane issues every copy. S tile
// buffers cycle through two mbarriers each: `full` (the tile's loads have
// landed; the producer arrives with the byte count) and `empty` (all NT
// transform threads have written the tile back). The producer stores a
// tile once it is empty, waits until that store has read the buffer, and
// loads the tile S later into it; the transform warps never meet at a CTA
// barrier and never wait for a store (a version with one CTA barrier per
// tile and the copies issued by thread 0 between tiles stalled on the
// barrier more than on anything else). twide_long_kernel (pencils of more
// than 32 chunks) has no producer warp; see there.
//
// The maps live in global memory, written by the host before the launch;
// they cover only this GPU's grid memory (no multicast).
#pragma once

#include <cstdint>
#include <cuda.h>

#include "lift.cuh"
#include "slab.cuh"

namespace pgb {

constexpr int kTWideThreads = 256;               // transform threads
constexpr int kTWideBlock = kTWideThreads + 32;  // + the producer warp
// Added to the chunk size of a launch whose pencils have 8 to 32 chunks
// (chunked form), more than 32 chunks (long form), lie along the last axis
// (contiguous form; more than 32 chunks: long contiguous form) or along a
// strided axis of inner extent 2 (pairs form).
constexpr int kTWideChunked = 32;
constexpr int kTWideLong = 64;
constexpr int kTWideContig = 96;
constexpr int kTWidePairs = 128;
constexpr int kTWideLongContig = 160;

struct TWideJob {
  long long tile_begin;  // first tile of this job in the launch
  int map;               // index of the job's tensor map
  int log2_n;            // pencil length
  int log2_inner;        // columns per outer index
  int nlevels;
  int log2_bx;           // box: 2^log2_bx columns of one outer index
  int log2_sx;           // box: 2^log2_sx outer indices
  int nxb;               // boxes per tile
  int chunked;           // 0: the dense layout, 1: the chunk-interleaved
                         // layout (G >= 8), 2: the contiguous layout (the
                         // last axis), 3: the pairs layout (strided,
                         // inner extent 2)
  int log2_rs;           // floats between a thread's rows in shared memory
  int log2_xlo;          // chunk-interleaved layout: columns per group
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
// Chunk-interleaved layout, [column group][row of chunk][chunk][X columns]
// (X = 2^log2_xlo, 4 or 8): the float index of row 0 of chunk c of column
// pair g (rows follow X G floats apart).
template <int LOG2R>
__device__ __forceinline__ int chunk_index(TWideJob const &job, int g, int c,
                                           int log2G) {
  int const x = job.log2_xlo;
  return (((((g >> (x - 1)) << LOG2R) << log2G) + c) << x) +
         2 * (g & ((1 << (x - 1)) - 1));
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
// dominated 8 KB ones); kStages tile buffers per CTA.
template <int R> struct TWideShape {
  static constexpr int kUnits = R >= 8 ? 1 : 8 / R;
  static constexpr int kUnitBytes = 8 * kTWideThreads * R;
  static constexpr int kTileBytes = kUnits * kUnitBytes;
  static constexpr int kStages = R >= 16 ? 3 : 4;
  static constexpr size_t kSmemBytes =
      size_t(kStages) * kTileBytes + 1024;  // + 1024-byte alignment slack
};

// The long form also holds the exchange buffers of its chunk heads (NT rows)
// and fine steps (2 NT rows).
template <int R, bool LONG> constexpr size_t twide_smem_bytes() {
  return TWideShape<R>::kSmemBytes + (LONG ? 3 * kTWideThreads * 16 : 0);
}

__device__ __forceinline__ void tma_load_5d(void *dst, void const *map,
                                            int q, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx"
      "::bytes [%0], [%1, {%2, %2, %2, %3, %4}], [%5];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(0), "r"(q), "r"(z),
      "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_5d(void const *map, int q, int z,
                                             void const *src) {
  asm volatile(
      "cp.async.bulk.tensor.5d.global.shared::cta.bulk_group [%0, {%1, %1, "
      "%1, %2, %3}], [%4];\n" ::"l"(reinterpret_cast<unsigned long long>(map)),
      "r"(0), "r"(q), "r"(z), "r"(smem_u32(src))
      : "memory");
}

// Waits until all but this thread's most recent bulk store group have read
// their shared memory.
__device__ __forceinline__ void bulk_wait_read_1() {
  asm volatile("cp.async.bulk.wait_group.read 1;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// Waits for phase `parity` of `bar` for about a second of clock, or until
// *abort is set; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar,
                                                  unsigned parity,
                                                  int const volatile *abort) {
  long long const t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if ((abort != nullptr && *abort) || clock64() - t0 > (1LL << 31))
      return false;
  return true;
}

// FORM (the same for every job of a launch):
//  0, pencils of up to 4 chunks in the dense layout;
//  1, pencils of 8 to 32 chunks of 16 points in the chunk-interleaved
//     layout;
//  3, last-axis pencils of up to 32 chunks of 4, 8 or 16 points in the
//     contiguous layout: a unit is 2 NT R consecutive floats (whole
//     pencils), moved as 128-byte rows of a 2D tensor map with the 128-byte
//     swizzle (16-byte piece q of row r stored at q ^ (r mod 8)), so that
//     the lanes of a warp, each reading 16-byte pieces of its own pencils'
//     rows, fall on different banks (at most two lanes per bank group);
//  4, pencils of up to 4 chunks along a strided axis whose inner extent is
//     2 columns (kstride 2, outer stride 2 n): a pencil pair's rows are
//     consecutive 8-byte pairs, so a unit is again 2 NT R consecutive floats
//     moved as swizzled 128-byte rows, and a thread's chunk is R / 2
//     consecutive 16-byte pieces of two rows each.
// All forms exchange by shuffles and have no barrier after the start. (One
// kernel for several forms kept more registers live and spilled.) Longer
// pencils (form 2 and 5 of the launch codes): twide_long_kernel below.
template <class A, int R, class Sched, int FORM>
__global__ void __launch_bounds__(kTWideBlock, R >= 16 ? 2 : 3)
    twide_kernel(__grid_constant__ const TWideParams p) {
  constexpr bool CHUNKED = FORM == 1;
  constexpr bool PAIRS = FORM == 4;
  constexpr bool CONTIG = FORM == 3 || PAIRS;
  using V = typename A::V;
  using W = typename A::Store;
  static_assert(sizeof(W) == 8, "rows of two float columns");
  constexpr int NT = kTWideThreads;
  constexpr int S = TWideShape<R>::kStages;
  constexpr int TILE = TWideShape<R>::kTileBytes;
  constexpr int U = TWideShape<R>::kUnits;
  constexpr int UNIT = TWideShape<R>::kUnitBytes;
  constexpr int LOG2R = Log2<R>::value;
  constexpr int LOG2NT = Log2<NT>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned const base_addr = smem_u32(smem_raw);
  unsigned char *const tiles =
      smem_raw + ((1024 - (base_addr & 1023)) & 1023);  // swizzle atoms
  __shared__ uint64_t full[S], empty[S];
  __shared__ TWideJob sjob[S];
  __shared__ int abort_flag;  // set when a bounded wait gave up
  int volatile *const abort = &abort_flag;

  int const t = threadIdx.x;
  int const lane = t & 31;
  long long const first = blockIdx.x;
  long long const step = gridDim.x;
  if (first >= p.total_tiles) return;
  long long const ntiles = (p.total_tiles - first + step - 1) / step;

  if (t == 0) {
    for (int b = 0; b < S; ++b) {
      mbar_init(&full[b], 1);
      mbar_init(&empty[b], NT);
    }
    *abort = 0;
    fence_mbar_init();
  }
  __syncthreads();  // the CTA's only barrier

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
  // Contiguous layout: the first 128-byte row of unit u of `tile` (a unit
  // is 16 R rows).
  auto contig_row = [](TWideJob const &job, long long tile, int u) {
    return static_cast<int>(((tile - job.tile_begin) * U + u) << (LOG2R + 4));
  };

  // The producer lane issues every copy; it keeps the last map it fenced.
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
      if constexpr (CONTIG) {  // one box of 16 R rows of 128 bytes
        tma_load_2d(dst, reinterpret_cast<CUtensorMap const *>(map), 0,
                    contig_row(job, tile, u), &full[b]);
        continue;
      }
      if (job.chunked) {  // one box: the unit (nxb = 1)
        tma_load_5d(dst, map, x0 >> job.log2_xlo, z0, &full[b]);
        continue;
      }
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
      if constexpr (CONTIG) {
        tma_store_2d(reinterpret_cast<CUtensorMap const *>(map), 0,
                     contig_row(job, tile, u), src);
        continue;
      }
      if (job.chunked) {
        tma_store_5d(map, x0 >> job.log2_xlo, z0, src);
        continue;
      }
      for (int xb = 0; xb < job.nxb; ++xb) {
        int x, z;
        box_at(job, xb, x0, z0, x, z);
        tma_store_3d(map, x, 0, z, src + xb * bb);
      }
    }
    bulk_commit();
  };

  if (t >= NT) {
    // Producer warp: lane 0 alone.
    if (t != NT) return;
    long long issued = 0;
    for (; issued < S && issued < ntiles; ++issued) issue_load(issued);
    bool failed = false;
    for (long long k = 0; k < ntiles; ++k) {
      int const b = static_cast<int>(k % S);
      if (!mbar_wait_bounded(&empty[b], static_cast<unsigned>((k / S) & 1),
                             abort)) {
        failed = true;
        break;
      }
      issue_store(k);
      if (issued < ntiles) {  // issued == k + S: the next tile for buffer b
        bulk_wait_read_all();  // the store just issued has read buffer b
        issue_load(issued);
        ++issued;
      }
    }
    if (failed) {
      atomicExch(p.error, 1u);
      *abort = 1;
      // Wait (bounded) for the last load issued into each buffer, so that
      // no copy is in flight when the CTA's shared memory goes away.
      for (long long q = issued > S ? issued - S : 0; q < issued; ++q)
        mbar_wait_bounded(&full[q % S], static_cast<unsigned>((q / S) & 1),
                          nullptr);
    }
    bulk_wait_all();
    return;
  }

  // Transform threads.
  for (long long k = 0; k < ntiles; ++k) {
    int const b = static_cast<int>(k % S);
    bool const ok = mbar_wait_bounded(
        &full[b], static_cast<unsigned>((k / S) & 1), abort);
    // A warp leaves as a whole (its lanes exchange by shuffles).
    if (!__all_sync(0xffffffffu, ok)) {
      if (lane == 0) {
        atomicExch(p.error, 1u);
        *abort = 1;
      }
      break;
    }
    TWideJob const &job = sjob[b];
    int const log2G = job.log2_n - LOG2R;
    // Jobs as the planner makes them for the launch's form (pencils of
    // more than 32 chunks would take exchange paths that need a barrier).
    bool const valid =
        CONTIG ? R >= 4 && job.chunked == (PAIRS ? 3 : 2) &&
                     static_cast<unsigned>(log2G) <= (PAIRS ? 2u : 5u)
               : (CHUNKED ? R == 16 && job.chunked == 1 && log2G >= 3 &&
                                log2G <= 5
                          : !job.chunked &&
                                static_cast<unsigned>(log2G) <= 2u) &&
                     job.log2_rs ==
                         (CHUNKED ? log2G + job.log2_xlo : job.log2_bx) &&
                     (!CHUNKED || (job.log2_xlo >= 2 && job.log2_xlo <= 3));
    if constexpr (CONTIG) {
      if (valid) {
        // Thread = (chunk c, column pair g): the G chunks of a pencil pair
        // are consecutive lanes; column e of the pair is pencil 2 g + e,
        // whose chunk starts at float (2 g + e) n + c R of the unit.
        int const c = lane & ((1 << log2G) - 1);
        int const g = t >> log2G;
        if constexpr (PAIRS) {
          // Piece i of the chunk: rows 2 i and 2 i + 1 of both columns, at
          // float 2 g n + 2 c R + 4 i of the unit.
          auto piece = [&](int i) {
            int const o =
                (g << (job.log2_n + 1)) + (c << (LOG2R + 1)) + 4 * i;
            int const row = o >> 5;
            return (row << 7) + ((((o & 31) >> 2) ^ (row & 7)) << 4);
          };
          for (int u = 0; u < U; ++u) {
            unsigned char *const ub = tiles + b * TILE + u * UNIT;
            V v[R];
#pragma unroll
            for (int i = 0; i < R / 2; ++i) {
              uint4 const f = *reinterpret_cast<uint4 const *>(ub + piece(i));
              v[2 * i] = A::load(W{f.x, f.y});
              v[2 * i + 1] = A::load(W{f.z, f.w});
            }
            RoundCtx<A, NT, true> ctx(t, c, 1 << log2G, log2G, lane, 1,
                                      nullptr, nullptr);
            Sched::template run_levels<A, R, NT>(v, ctx, job.nlevels);
#pragma unroll
            for (int i = 0; i < R / 2; ++i) {
              W const r0 = A::store(v[2 * i]);
              W const r1 = A::store(v[2 * i + 1]);
              *reinterpret_cast<uint4 *>(ub + piece(i)) =
                  uint4{r0.x, r0.y, r1.x, r1.y};
            }
          }
        } else {
        // The byte offset of piece i of column e: rows of 128 bytes, pieces
        // of 16 bytes swizzled within their row.
        auto piece = [&](int e, int i) {
          int const o = ((2 * g + e) << job.log2_n) + (c << LOG2R);
          int const row = o >> 5;
          return (row << 7) + (((((o & 31) >> 2) + i) ^ (row & 7)) << 4);
        };
        for (int u = 0; u < U; ++u) {
          unsigned char *const ub = tiles + b * TILE + u * UNIT;
          V v[R];
#pragma unroll
          for (int i = 0; i < R / 4; ++i) {
            uint4 const f0 = *reinterpret_cast<uint4 const *>(ub + piece(0, i));
            uint4 const f1 = *reinterpret_cast<uint4 const *>(ub + piece(1, i));
            v[4 * i] = A::load(W{f0.x, f1.x});
            v[4 * i + 1] = A::load(W{f0.y, f1.y});
            v[4 * i + 2] = A::load(W{f0.z, f1.z});
            v[4 * i + 3] = A::load(W{f0.w, f1.w});
          }
          RoundCtx<A, NT, true> ctx(t, c, 1 << log2G, log2G, lane, 1,
                                    nullptr, nullptr);
          Sched::template run_levels<A, R, NT>(v, ctx, job.nlevels);
#pragma unroll
          for (int i = 0; i < R / 4; ++i) {
            W const r0 = A::store(v[4 * i]);
            W const r1 = A::store(v[4 * i + 1]);
            W const r2 = A::store(v[4 * i + 2]);
            W const r3 = A::store(v[4 * i + 3]);
            *reinterpret_cast<uint4 *>(ub + piece(0, i)) =
                uint4{r0.x, r1.x, r2.x, r3.x};
            *reinterpret_cast<uint4 *>(ub + piece(1, i)) =
                uint4{r0.y, r1.y, r2.y, r3.y};
          }
        }
        }
      } else if (lane == 0) {
        atomicExch(p.error, 1u);
      }
    } else if (valid) {
      int const G = 1 << log2G;
      // Thread = (chunk c, column pair g): the chunks of a column pair are
      // lanes W = 32 / G apart, the W column pairs of one chunk consecutive.
      int const log2ls = 5 - log2G;
      int const c = lane >> log2ls;
      int const g = ((t >> 5) << log2ls) | (lane & ((1 << log2ls) - 1));
      // Float index of the thread's row j: idx0 + (j << job.log2_rs) (the
      // row stride read from the job in shared memory where needed: a
      // register holding it through the transform made the kernel spill).
      int idx0;
      if constexpr (CHUNKED) {
        // [column quad][row of chunk][chunk][4 columns]
        idx0 = chunk_index<LOG2R>(job, g, c, log2G);
      } else {
        int const col = 2 * g;
        int const log2bs = job.log2_bx + job.log2_sx;
        int const xb = col >> log2bs;
        int const rem = col & ((1 << log2bs) - 1);
        int const s = rem >> job.log2_bx;
        int const bcol = rem & ((1 << job.log2_bx) - 1);
        // [box][outer][row][column]: row c R of the thread's columns; rows
        // are Bx apart
        idx0 = (xb << (log2bs + job.log2_n)) +
               ((((s << job.log2_n) + (c << LOG2R)) << job.log2_bx) + bcol);
      }
      for (int u = 0; u < U; ++u) {
        float *const tf =
            reinterpret_cast<float *>(tiles + b * TILE + u * UNIT);
        V v[R];
#pragma unroll
        for (int j = 0; j < R; ++j)
          v[j] = A::load(
              *reinterpret_cast<W const *>(tf + idx0 + (j << job.log2_rs)));
        RoundCtx<A, NT, true> ctx(t, c, G, log2G, lane, 1, nullptr, nullptr,
                                  log2ls);
        Sched::template run_levels<A, R, NT>(v, ctx, job.nlevels);
#pragma unroll
        for (int j = 0; j < R; ++j)
          *reinterpret_cast<W *>(tf + idx0 + (j << job.log2_rs)) =
              A::store(v[j]);
      }
    } else if (lane == 0) {
      atomicExch(p.error, 1u);
    }
    fence_proxy_async_smem();  // the writes above, before the tile's store
    mbar_arrive(&empty[b]);
  }
}


// Long form: periodic pencils of 64 or 128 chunks of 16 points (1024 and
// 2048 points) in the chunk-interleaved layout, or (CONTIG) the last axis'
// pencils of 64 to 256 chunks (1024 to 4096 points) in the contiguous
// layout (a tile is whole pencils: 2 NT R consecutive floats, as swizzled
// 128-byte rows, see FORM 3 of twide_kernel). Their chunks are
// consecutive threads and exchange through shared memory with a CTA barrier
// per step, so every thread meets at barriers anyway: there is no producer
// warp. Thread 0 issues the copies right after each tile's vote barrier
// (every thread has then written the previous tile back): the store of tile
// k - 1, and the load of tile k + 1 into the buffer of tile k - 2 once that
// tile's store has read it. 256 threads per CTA leave 128 registers per
// thread for two CTAs per SM (a producer warp would leave 96, and the form
// spilled there).
template <class A, class Sched, bool CONTIG>
__global__ void __launch_bounds__(kTWideThreads, 2)
    twide_long_kernel(__grid_constant__ const TWideParams p) {
  using V = typename A::V;
  using W = typename A::Store;
  static_assert(sizeof(W) == 8, "rows of two float columns");
  constexpr int R = 16;
  constexpr int NT = kTWideThreads;
  constexpr int S = TWideShape<R>::kStages;
  static_assert(S == 3, "the copy order below assumes three tile buffers");
  constexpr int TILE = TWideShape<R>::kTileBytes;
  constexpr int LOG2R = Log2<R>::value;
  constexpr int LOG2NT = Log2<NT>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned const base_addr = smem_u32(smem_raw);
  unsigned char *const tiles =
      smem_raw + ((1024 - (base_addr & 1023)) & 1023);  // swizzle atoms
  V *const heads = reinterpret_cast<V *>(tiles + S * TILE);
  V *const xch = heads + NT;
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

  // Thread 0's copies (one box per tile: 5D, or 2D of 16 R rows of 128
  // bytes); it keeps the last map it fenced.
  int fenced = -1;
  auto origin = [](TWideJob const &job, long long tile, int &q0, int &z0) {
    int const log2ct = LOG2NT + 1 - (job.log2_n - LOG2R);
    long long const col0 = (tile - job.tile_begin) << log2ct;
    z0 = static_cast<int>(col0 >> job.log2_inner);
    q0 = static_cast<int>((col0 & ((1LL << job.log2_inner) - 1)) >>
                          job.log2_xlo);
  };
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
    mbar_expect_tx(&full[b], static_cast<unsigned>(TILE));
    if constexpr (CONTIG) {
      tma_load_2d(tiles + b * TILE, reinterpret_cast<CUtensorMap const *>(map),
                  0, static_cast<int>((tile - job.tile_begin) << (LOG2R + 4)),
                  &full[b]);
    } else {
      int q0, z0;
      origin(job, tile, q0, z0);
      tma_load_5d(tiles + b * TILE, map, q0, z0, &full[b]);
    }
  };
  auto issue_store = [&](long long k) {
    int const b = static_cast<int>(k % S);
    long long const tile = first + k * step;
    TWideJob const &job = sjob[b];
    if constexpr (CONTIG) {
      tma_store_2d(reinterpret_cast<CUtensorMap const *>(p.maps + job.map), 0,
                   static_cast<int>((tile - job.tile_begin) << (LOG2R + 4)),
                   tiles + b * TILE);
    } else {
      int q0, z0;
      origin(job, tile, q0, z0);
      tma_store_5d(p.maps + job.map, q0, z0, tiles + b * TILE);
    }
    bulk_commit();
  };

  if (t == 0) issue_load(0);
  long long k = 0;
  for (; k < ntiles; ++k) {
    int const b = static_cast<int>(k % S);
    // Bounded wait for tile k, then a vote so that every thread leaves
    // together if one gave up (no barrier is left waiting).
    bool done = false;
    long long const t0 = clock64();
    while (!(done = mbar_try_wait(&full[b],
                                  static_cast<unsigned>((k / S) & 1))))
      if (clock64() - t0 > (1LL << 31)) break;
    if (!__syncthreads_and(done)) break;
    if (t == 0) {
      if (k >= 1) issue_store(k - 1);  // its writes are in (the barrier)
      if (k + 1 < ntiles) {
        bulk_wait_read_1();  // the store of tile k - 2 has read its buffer
        issue_load(k + 1);
      }
    }
    TWideJob const &job = sjob[b];
    int const log2G = job.log2_n - LOG2R;
    // Jobs as the planner makes them (uniform over the tile, so every
    // thread takes the same barriers).
    if constexpr (CONTIG) {
      if (job.chunked == 2 && log2G >= 6 && log2G <= 8) {
        int const G = 1 << log2G;
        // Thread = (chunk c, pencil pair g): chunks in consecutive threads;
        // column e of the pair is pencil 2 g + e, whose chunk starts at
        // float (2 g + e) n + c R of the tile.
        int const c = t & (G - 1);
        int const g = t >> log2G;
        auto piece = [&](int e, int i) {
          int const o = ((2 * g + e) << job.log2_n) + (c << LOG2R);
          int const row = o >> 5;
          return (row << 7) + (((((o & 31) >> 2) + i) ^ (row & 7)) << 4);
        };
        unsigned char *const ub = tiles + b * TILE;
        V v[R];
#pragma unroll
        for (int i = 0; i < R / 4; ++i) {
          uint4 const f0 = *reinterpret_cast<uint4 const *>(ub + piece(0, i));
          uint4 const f1 = *reinterpret_cast<uint4 const *>(ub + piece(1, i));
          v[4 * i] = A::load(W{f0.x, f1.x});
          v[4 * i + 1] = A::load(W{f0.y, f1.y});
          v[4 * i + 2] = A::load(W{f0.z, f1.z});
          v[4 * i + 3] = A::load(W{f0.w, f1.w});
        }
        RoundCtx<A, NT, false, 256> ctx(t, c, G, log2G, lane, 1, heads, xch);
        Sched::template run_levels<A, R, NT>(v, ctx, job.nlevels);
#pragma unroll
        for (int i = 0; i < R / 4; ++i) {
          W const r0 = A::store(v[4 * i]);
          W const r1 = A::store(v[4 * i + 1]);
          W const r2 = A::store(v[4 * i + 2]);
          W const r3 = A::store(v[4 * i + 3]);
          *reinterpret_cast<uint4 *>(ub + piece(0, i)) =
              uint4{r0.x, r1.x, r2.x, r3.x};
          *reinterpret_cast<uint4 *>(ub + piece(1, i)) =
              uint4{r0.y, r1.y, r2.y, r3.y};
        }
      } else if (t == 0) {
        atomicExch(p.error, 1u);
      }
    } else if (job.chunked == 1 && log2G >= 6 && log2G <= 7 &&
               job.log2_xlo >= 2 && job.log2_xlo <= 3 &&
               job.log2_rs == log2G + job.log2_xlo) {
      int const G = 1 << log2G;
      // Thread = (chunk c, column pair g): chunks in consecutive threads.
      int const c = t & (G - 1);
      int const g = t >> log2G;
      // [column group][row of chunk][chunk][X columns]
      int const idx0 = chunk_index<LOG2R>(job, g, c, log2G);
      float *const tf = reinterpret_cast<float *>(tiles + b * TILE);
      V v[R];
#pragma unroll
      for (int j = 0; j < R; ++j)
        v[j] = A::load(
            *reinterpret_cast<W const *>(tf + idx0 + (j << job.log2_rs)));
      RoundCtx<A, NT, false, 128> ctx(t, c, G, log2G, lane, 1, heads, xch);
      Sched::template run_levels<A, R, NT>(v, ctx, job.nlevels);
#pragma unroll
      for (int j = 0; j < R; ++j)
        *reinterpret_cast<W *>(tf + idx0 + (j << job.log2_rs)) =
            A::store(v[j]);
    } else if (t == 0) {
      atomicExch(p.error, 1u);
    }
    fence_proxy_async_smem();  // the writes above, before the tile's store
  }
  if (k == ntiles) {
    __syncthreads();  // every thread has written the last tile back
    if (t == 0) issue_store(k - 1);
  } else if (t == 0) {
    atomicExch(p.error, 1u);
    // Tile k's load (the only one in flight) must end before the CTA's
    // shared memory goes away.
    long long const t0 = clock64();
    while (!mbar_try_wait(&full[k % S], static_cast<unsigned>((k / S) & 1)))
      if (clock64() - t0 > (1LL << 31)) break;
  }
  if (t == 0) bulk_wait_all();
}

} // namespace pgb
