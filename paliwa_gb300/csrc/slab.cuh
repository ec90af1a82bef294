// Slab kernel: every level of a grid's trailing axes in one HBM pass.
//
// For a grid viewed as [lead][n_m]...[n_{d-1}], the trailing axes m..d-1
// span contiguous blocks ("slabs") of V = n_m * ... * n_{d-1} points. When a
// slab fits in shared memory, one launch transforms all of those axes, in
// order, for every slab: one HBM read and one write per point for the whole
// group, where the per-axis kernels (lift.cuh) read and write once per axis.
// The reference runs one parallel region per (axis, level, pass)
// (paliwa/paliwa_transform.hpp:231-249, folded over the dimensions at
// :401-431); the order of axes, levels and passes is the same here, so the
// results are the same bits as the per-axis path.
//
// Tiles. A tile is kSlabTileBytes (or the whole grid, if smaller) of
// consecutive slabs of one grid: a contiguous block, moved between HBM and
// shared memory by the tensor memory accelerator as 1 KB boxes of a 2D view
// of the batch's memory ([rows][128 bytes]) with the 128-byte swizzle (the
// 16-byte pieces of row r permuted by r mod 8), completion on an mbarrier.
// Each CTA keeps kSlabStages tiles in flight: while it transforms one, the
// next ones load and the previous one stores.
//
// Compute. Along an axis of extent n and element stride s inside the tile,
// a thread holds R consecutive points of one pencil (a chunk) in registers
// and runs the wavelet schedule of lift.cuh on it. Items (pencil, chunk)
// are numbered i = (o G + c) s + w (o outer index, c chunk, w inner index,
// G = n / R), so that consecutive threads take consecutive inner indices:
// for s >= 32 a warp reads rows of 32 consecutive elements; for small s the
// planner picks R (8 or less) so that the swizzle keeps the reads on
// distinct banks; the contiguous last axis is read as 16-byte pieces. The G
// chunks of a pencil exchange neighbours by warp shuffle when G s <= 32
// (lanes s apart), else through shared memory with one barrier per pass.
#pragma once

#include <cstdint>
#include <cuda.h>

#include "lift.cuh"

namespace pgb {

constexpr int kSlabThreads = 256;
constexpr int kSlabStages = 3;
constexpr int kSlabTileBytes = 32768;
constexpr int kSlabBoxBytes = 1024;  // 8 rows of 128 bytes: one swizzle atom
constexpr int kSlabMaxAxes = 12;

struct SlabAxis {
  signed char log2n;    // pencil length
  signed char log2s;    // element stride of the pencil in the tile
  signed char nlevels;  // levels to run (shifts 0 .. nlevels - 1)
  signed char log2r;    // chunk size R = 2^log2r
};

struct SlabJob {
  long long row0;        // the grid's first 128-byte row in the tensor map
  long long tile_begin;  // first tile of this job in the launch
  int log2_tile;         // log2 of the elements per tile
  int naxes;
  SlabAxis axis[kSlabMaxAxes];
};

struct SlabParams {
  CUtensorMap map;          // [rows][128 bytes] over the batch's grids
  SlabJob const *jobs;      // sorted by tile_begin
  int const *tile_job;      // the job of every tile of the launch
  int njobs;
  long long total_tiles;
  unsigned *error;          // set to 1 when a bounded wait gives up
  int ctas_per_sm;          // cap on the launch's CTAs per SM (0: none)
};

// ---- PTX wrappers (sm_90+ bulk tensor copies and mbarriers)

__device__ __forceinline__ unsigned smem_u32(void const *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void tma_load_2d(void *dst, CUtensorMap const *map,
                                            int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx"
      "::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y),
      "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_2d(CUtensorMap const *map, int x,
                                             int y, void const *src) {
  asm volatile(
      "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], "
      "[%3];\n" ::"l"(reinterpret_cast<unsigned long long>(map)),
      "r"(x), "r"(y), "r"(smem_u32(src))
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}
// Waits until this thread's bulk stores have read their shared memory.
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
}
// Waits until this thread's bulk stores are complete.
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
}
// Orders this thread's shared-memory writes before later bulk copies.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// Byte offset of logical byte b of a tile under the 128-byte swizzle.
__device__ __forceinline__ int swz128(int b) {
  return b ^ (((b >> 7) & 7) << 4);
}

// Exchanges of the chunks of one pencil inside a slab axis (the interface
// the wavelet schedules use, see RoundCtx): chunk c of a pencil is item
// i = (o G + c) s + w, so its neighbours are s items away. With G s <= 32
// they are lanes of one warp (shuffles); otherwise they go through shared
// memory, one barrier per exchange (the same for every thread: G and s are
// uniform per axis).
template <class A, int NT> struct SlabCtx {
  using V = typename A::V;
  static constexpr bool kHeadPencil = false;
  static constexpr bool kShflOnly = false;
  static constexpr int kMaxG = 256;
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  int t, c, G, log2G, log2ls, gbase_lane, cbase;
  bool in_warp;
  int periodic = 1;
  V *heads, *xch;
  int buf = 0;
  bool heads_valid = false;

  __device__ __forceinline__ SlabCtx(int t_, int c_, int log2G_, int lane,
                                     int log2s, bool in_warp_, V *heads_,
                                     V *xch_)
      : t(t_), c(c_), G(1 << log2G_), log2G(log2G_), log2ls(log2s),
        gbase_lane(lane & ~(((1 << log2G_) - 1) << log2s)),
        cbase(t_ - (c_ << log2s)), in_warp(in_warp_), heads(heads_),
        xch(xch_) {}

  __device__ __forceinline__ int lane_of(int cc) const {
    return gbase_lane | ((cc & (G - 1)) << log2ls);
  }
  __device__ __forceinline__ int slot_of(int cc) const {
    return cbase + ((cc & (G - 1)) << log2ls);
  }
  __device__ __forceinline__ V fine_neighbor(int o, V pub) {
    if (G == 1) return pub;
    int const nc = (o == 1) ? c + 1 : c - 1;
    if (in_warp) return shfl(pub, lane_of(nc));
    xch[buf * NT + t] = pub;
    __syncthreads();
    V const r = xch[buf * NT + slot_of(nc)];
    buf ^= 1;
    return r;
  }
  __device__ __forceinline__ void fine_wrote_heads(int o) {
    if (o == 0) heads_valid = false;
  }
  template <class Upd>
  __device__ __forceinline__ void coarse(V &v0, int o, int d, Upd upd) {
    bool const mine = (c & (2 * d - 1)) == o * d;
    if (in_warp) {
      V const lo = shfl(v0, lane_of(c - d));
      V const up = shfl(v0, lane_of(c + d));
      if (mine) v0 = upd(lo, v0, up);
      return;
    }
    if (!heads_valid) {
      heads[t] = v0;
      __syncthreads();
      heads_valid = true;
    }
    if (mine) {
      v0 = upd(heads[slot_of(c - d)], v0, heads[slot_of(c + d)]);
      heads[t] = v0;
    }
    __syncthreads();
  }
};

// U items per thread and iteration of one axis of a tile (U > 1 only for
// axes whose chunks exchange by shuffle or not at all): the U chunks are
// independent, so their level steps interleave and hide each other's
// latencies (short pencils have few updates per chunk).
template <class A, int R, int NT, class Sched, int U>
__device__ __forceinline__ void slab_items(unsigned char *tile, SlabAxis ax,
                                           int log2T, int t, int lane,
                                           typename A::V *heads,
                                           typename A::V *xch, bool in_warp) {
  using V = typename A::V;
  using S = typename A::Store;
  constexpr int ES = sizeof(S);
  constexpr int LOG2R = Log2<R>::value;
  int const log2n = ax.log2n, log2s = ax.log2s;
  int const log2G = log2n - LOG2R;
  int const items = 1 << (log2T - LOG2R);
  bool const vec = log2s == 0 && R * ES >= 16;  // contiguous 16-byte pieces
  for (int base = 0; base < items; base += U * NT) {
    int e0[U], c[U];
    bool active[U];
    V v[U][R];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      int const i = base + u * NT + t;
      active[u] = i < items;
      int const w = i & ((1 << log2s) - 1);
      c[u] = (i >> log2s) & ((1 << log2G) - 1);
      int const o = i >> (log2s + log2G);
      // element index of the chunk's first point
      e0[u] = (o << (log2n + log2s)) + (c[u] << (LOG2R + log2s)) + w;
      if (active[u]) {
        if (vec) {
          constexpr int PER = 16 / ES;
#pragma unroll
          for (int q = 0; q < R / PER; ++q) {
            uint4 const x = *reinterpret_cast<uint4 const *>(
                tile + swz128(e0[u] * ES + q * 16));
            S tmp[PER];
            memcpy(tmp, &x, 16);
#pragma unroll
            for (int e = 0; e < PER; ++e) v[u][q * PER + e] = A::load(tmp[e]);
          }
        } else {
#pragma unroll
          for (int j = 0; j < R; ++j)
            v[u][j] = A::load(*reinterpret_cast<S const *>(
                tile + swz128((e0[u] + (j << log2s)) * ES)));
        }
      } else {
#pragma unroll
        for (int j = 0; j < R; ++j) v[u][j] = A::load(S(0));
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      SlabCtx<A, NT> ctx(t, c[u], log2G, lane, log2s, in_warp, heads, xch);
      Sched::template run_levels<A, R, NT>(v[u], ctx, ax.nlevels);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (!active[u]) continue;
      if (vec) {
        constexpr int PER = 16 / ES;
#pragma unroll
        for (int q = 0; q < R / PER; ++q) {
          S tmp[PER];
#pragma unroll
          for (int e = 0; e < PER; ++e) tmp[e] = A::store(v[u][q * PER + e]);
          uint4 x;
          memcpy(&x, tmp, 16);
          *reinterpret_cast<uint4 *>(tile + swz128(e0[u] * ES + q * 16)) = x;
        }
      } else {
#pragma unroll
        for (int j = 0; j < R; ++j)
          *reinterpret_cast<S *>(tile + swz128((e0[u] + (j << log2s)) * ES)) =
              A::store(v[u][j]);
      }
    }
    if (!in_warp) __syncthreads();  // heads / xch are reused
  }
}

// One axis of a tile held in shared memory: every pencil, every level.
// Chunks of up to 8 points run 2 or 4 per thread at once where the axis has
// enough of them.
template <class A, int R, int NT, class Sched>
__device__ __forceinline__ void slab_axis(unsigned char *tile, SlabAxis ax,
                                          int log2T, int t, int lane,
                                          typename A::V *heads,
                                          typename A::V *xch) {
  constexpr int LOG2R = Log2<R>::value;
  constexpr int UMAX = R <= 4 ? 4 : (R <= 8 ? 2 : 1);
  int const log2G = ax.log2n - LOG2R;
  int const items = 1 << (log2T - LOG2R);
  // A pencil held by one thread (G == 1) exchanges nothing; otherwise its
  // chunks are lanes of one warp when G s <= 32.
  bool const in_warp = log2G == 0 || log2G + ax.log2s <= 5;
  if constexpr (UMAX > 1) {
    if (in_warp && items >= UMAX * NT) {
      slab_items<A, R, NT, Sched, UMAX>(tile, ax, log2T, t, lane, heads, xch,
                                        true);
      return;
    }
  }
  slab_items<A, R, NT, Sched, 1>(tile, ax, log2T, t, lane, heads, xch,
                                 in_warp);
}

// Dynamic shared memory: the tile buffers (1 KB aligned for the swizzle,
// plus 1 KB of alignment slack) and the chunk heads and exchange buffers.
template <class A> constexpr size_t slab_smem_bytes() {
  return size_t(kSlabStages) * kSlabTileBytes + kSlabBoxBytes +
         3 * kSlabThreads * sizeof(typename A::V);
}

template <class A, class Sched>
__global__ void __launch_bounds__(kSlabThreads, 2)
    slab_kernel(__grid_constant__ const SlabParams p) {
  using V = typename A::V;
  using S = typename A::Store;
  constexpr int NT = kSlabThreads;
  constexpr int ES = sizeof(S);
  constexpr int LOG2ES = Log2<ES>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned const base_addr = smem_u32(smem_raw);
  unsigned char *const tiles =
      smem_raw + ((kSlabBoxBytes - (base_addr & (kSlabBoxBytes - 1))) &
                  (kSlabBoxBytes - 1));
  V *const heads =
      reinterpret_cast<V *>(tiles + kSlabStages * kSlabTileBytes);
  V *const xch = heads + NT;
  __shared__ uint64_t full[kSlabStages];
  __shared__ SlabJob sjob[kSlabStages];

  int const t = threadIdx.x;
  int const lane = t & 31;
  long long const first = blockIdx.x;
  long long const step = gridDim.x;
  if (first >= p.total_tiles) return;
  long long const ntiles = (p.total_tiles - first + step - 1) / step;

  if (t == 0) {
    for (int b = 0; b < kSlabStages; ++b) mbar_init(&full[b], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // Warp 0 issues the copies: the job of the tile (one table lookup, its
  // words copied by the lanes in parallel), lane 0 the transaction count,
  // every lane some of the tile's 1 KB boxes.
  constexpr int kJobWords = sizeof(SlabJob) / 4;
  static_assert(sizeof(SlabJob) % 4 == 0 && kJobWords <= 32,
                "a slab job is copied one word per lane");
  auto issue_load = [&](long long k) {
    int const b = static_cast<int>(k % kSlabStages);
    long long const tile = first + k * step;
    int const j = p.tile_job[tile];
    if (lane < kJobWords)
      reinterpret_cast<unsigned *>(&sjob[b])[lane] =
          reinterpret_cast<unsigned const *>(p.jobs + j)[lane];
    __syncwarp();
    SlabJob const &job = sjob[b];
    int const bytes = 1 << (job.log2_tile + LOG2ES);
    long long const row =
        job.row0 + ((tile - job.tile_begin) << (job.log2_tile + LOG2ES - 7));
    if (lane == 0) mbar_expect_tx(&full[b], static_cast<unsigned>(bytes));
    __syncwarp();
    unsigned char *const dst = tiles + b * kSlabTileBytes;
    for (int box = lane; box * kSlabBoxBytes < bytes; box += 32)
      tma_load_2d(dst + box * kSlabBoxBytes, &p.map, 0,
                  static_cast<int>(row + box * 8), &full[b]);
  };
  auto issue_store = [&](long long k) {
    int const b = static_cast<int>(k % kSlabStages);
    long long const tile = first + k * step;
    SlabJob const &job = sjob[b];
    int const bytes = 1 << (job.log2_tile + LOG2ES);
    long long const row =
        job.row0 + ((tile - job.tile_begin) << (job.log2_tile + LOG2ES - 7));
    unsigned char const *const src = tiles + b * kSlabTileBytes;
    for (int box = lane; box * kSlabBoxBytes < bytes; box += 32)
      tma_store_2d(&p.map, 0, static_cast<int>(row + box * 8),
                   src + box * kSlabBoxBytes);
    bulk_commit();
  };

  if (t < 32)
    for (long long k = 0; k < kSlabStages - 1 && k < ntiles; ++k) issue_load(k);

  for (long long k = 0; k < ntiles; ++k) {
    int const b = static_cast<int>(k % kSlabStages);
    if (t < 32 && k + kSlabStages - 1 < ntiles) {
      // The buffer of tile k - 1: its stores must have read it.
      bulk_wait_read_all();
      issue_load(k + kSlabStages - 1);
    }
    // Bounded wait for tile k (about a second of clock), then a vote so
    // that every thread leaves together if it gave up.
    unsigned const parity = static_cast<unsigned>((k / kSlabStages) & 1);
    bool done = false;
    long long const t0 = clock64();
    while (!(done = mbar_try_wait(&full[b], parity)))
      if (clock64() - t0 > (1LL << 31)) break;
    if (!__syncthreads_and(done)) {
      if (t == 0) atomicExch(p.error, 1u);
      break;
    }
    SlabJob const &job = sjob[b];
    unsigned char *const tile = tiles + b * kSlabTileBytes;
    for (int a = 0; a < job.naxes; ++a) {
      SlabAxis const ax = job.axis[a];
      switch (ax.log2r) {
      case 1: slab_axis<A, 2, NT, Sched>(tile, ax, job.log2_tile, t, lane, heads, xch); break;
      case 2: slab_axis<A, 4, NT, Sched>(tile, ax, job.log2_tile, t, lane, heads, xch); break;
      case 3: slab_axis<A, 8, NT, Sched>(tile, ax, job.log2_tile, t, lane, heads, xch); break;
      case 4: slab_axis<A, 16, NT, Sched>(tile, ax, job.log2_tile, t, lane, heads, xch); break;
      case 5: slab_axis<A, 32, NT, Sched>(tile, ax, job.log2_tile, t, lane, heads, xch); break;
      default: break;
      }
      __syncthreads();  // the next axis reads what this one wrote
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (t < 32) issue_store(k);
  }
  if (t < 32) bulk_wait_all();
}

} // namespace pgb
