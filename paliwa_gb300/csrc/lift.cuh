// Multi-level lifting along one axis of dense row-major grids.
//
// Replaces the per-(level, pass) parallel regions of paliwa's
// detail::lifting_pass (paliwa/paliwa_transform.hpp:24-51, driven by
// transform_in :215-251) with one kernel per axis that runs every level and
// pass of that axis on data held on chip: one HBM read and one write per
// element per axis instead of one per level.
//
// Geometry. A grid is viewed around the transformed axis as [outer][n][inner]
// (n = 2^level along the axis). A column is one (outer, inner) pair, i.e. one
// pencil of n points at element stride `inner`. A CTA takes C columns; each
// pencil is cut into G = n / R chunks of R consecutive points and each thread
// keeps one chunk of one column in registers (NT = C * G threads).
//
// Levels. A level with compact distance s < R only couples points inside a
// chunk, except for one boundary neighbour that is exchanged through shared
// memory (a value of chunk c +- 1). A level with s >= R only touches chunk
// heads (slot 0); those steps run on a shared-memory copy of the heads.
//
// Windows. Pencils longer than one CTA can hold are processed in two kinds of
// phases, planned on the host: the fine levels on overlapping windows
// (segment plus halo, non-periodic; only the segment is stored), and the
// coarse levels on the strided sub-lattice of the remaining points, which is
// itself a short periodic pencil. A window's halo lies in the neighbouring
// segments, which their own windows overwrite in place, so a halo pass
// (halo_kernel) first copies the points within a halo of every segment
// boundary to a side buffer of the grid's layout, and the windows read their
// halos from there.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "arith.cuh"

namespace pgb {

constexpr int kMaxPasses = 8;
constexpr int kMaxLevels = 48;

// One unit of work for a launch: one grid (or one sub-lattice of a grid)
// along one axis. Jobs of a launch are sorted by tile_begin.
struct LiftJob {
  unsigned long long base;  // byte address of the grid's first element
  // Byte address the results are stored to (same layout; `base` for every
  // stage the planner makes).
  unsigned long long dst_base;
  // Windows: byte address of a buffer in the grid's layout holding the
  // points around the segment boundaries, from which the window reads every
  // point outside its own segment (0: read them from `base`).
  unsigned long long halo_base;
  long long columns;        // outer * inner
  long long tile_begin;     // index of the first tile of this job
  long long col_tiles;      // tiles per window row (ceil(columns / C))
  int log2_inner;           // inner extent: splits a column index into (a, b)
  int log2_kstride;         // element stride between consecutive pencil points
  int log2_astride;         // element stride between consecutive outer indices
  int log2_n;               // pencil length of the whole (sub-lattice) axis
  int log2_window;          // points per pencil held by one CTA
  int periodic;             // 1: whole periodic pencils; 0: windows
  // Window mode: the window covers points
  // [seg * seg_len - halo, seg * seg_len + seg_len + halo) of the pencil.
  int seg_len;
  int halo;
  int nlevels;
  signed char shift[kMaxLevels];  // log2 of each level's distance, in order
};

struct LiftParams {
  LiftJob const *jobs;  // device array, or nullptr to use `job`
  int njobs;
  long long total_tiles;
  int npasses;
  int rounds;           // column rounds per tile (tile = rounds * NT * R)
  int ctas_per_sm;      // cap on a persistent launch's CTAs per SM (0: none)
  unsigned c1_one_mask;
  int offsets[kMaxPasses];
  Coeffs coeffs[kMaxPasses];
  LiftJob job;
};

// Column rounds per staged tile: a tile holds kTileRounds * NT * R points.
constexpr int kTileRounds = 2;

template <int X> struct Log2 {
  static constexpr int value = 1 + Log2<X / 2>::value;
};
template <> struct Log2<1> {
  static constexpr int value = 0;
};

// v[R - 2^sh] with a compile-time register index.
template <int R, typename V>
__device__ __forceinline__ V tail_value(V const (&v)[R], int sh) {
  V r = v[R - 1];
#pragma unroll
  for (int k = 0; (1 << k) < R; ++k)
    if (sh == k) r = v[R - (1 << k)];
  return r;
}

// One fine step (distance S < R) on the chunk held in registers. `nb` is the
// neighbour from the adjacent chunk: for odd passes (offset 1) the next
// chunk's slot 0, for even passes (offset 0) the previous chunk's slot R - S.
template <class A, int R, int S, bool C1, typename V>
__device__ __forceinline__ void fine_step(V (&v)[R], int o, V nb,
                                          Coeffs const &cf) {
  if (o == 1) {
#pragma unroll
    for (int j = S; j < R; j += 2 * S) {
      V up = (j + S < R) ? v[(j + S) % R] : nb;
      v[j] = A::template update<C1>(cf, v[j - S], v[j], up);
    }
  } else {
#pragma unroll
    for (int j = 0; j < R; j += 2 * S) {
      V lo = (j >= S) ? v[(j + R - S) % R] : nb;
      v[j] = A::template update<C1>(cf, lo, v[j], v[j + S]);
    }
  }
}

// Selects the compile-time distance 2^K == 2^sh (sh < log2 R).
template <class A, int R, bool C1, int K = 0, typename V>
__device__ __forceinline__ void fine_distance(V (&v)[R], int sh, int o, V nb,
                                              Coeffs const &cf) {
  if constexpr ((1 << K) < R) {
    if (sh == K) {
      fine_step<A, R, (1 << K), C1>(v, o, nb, cf);
      return;
    }
    fine_distance<A, R, C1, K + 1>(v, sh, o, nb, cf);
  }
}

template <class A, int R, typename V>
__device__ __forceinline__ void fine_dispatch(V (&v)[R], int sh, int o, V nb,
                                              Coeffs const &cf, bool c1one) {
  if (c1one)
    fine_distance<A, R, true>(v, sh, o, nb, cf);
  else
    fine_distance<A, R, false>(v, sh, o, nb, cf);
}

template <class A, typename V>
__device__ __forceinline__ V coarse_update(Coeffs const &cf, bool c1one, V lo,
                                           V me, V up) {
  if (c1one) return A::template update<true>(cf, lo, me, up);
  return A::template update<false>(cf, lo, me, up);
}

// Warp shuffles of one value (double, float or a double-float pair).
__device__ __forceinline__ double shfl(double x, int src) {
  return __shfl_sync(0xffffffffu, x, src);
}
__device__ __forceinline__ float shfl(float x, int src) {
  return __shfl_sync(0xffffffffu, x, src);
}
__device__ __forceinline__ DF shfl(DF x, int src) {
  return {__shfl_sync(0xffffffffu, x.h, src),
          __shfl_sync(0xffffffffu, x.l, src)};
}
// Rows of adjacent columns (the wide kernel's values).
__device__ __forceinline__ f2 shfl(f2 x, int src) {
  return __shfl_sync(0xffffffffu, x, src);
}
__device__ __forceinline__ DF2 shfl(DF2 x, int src) {
  return {shfl(x.h, src), shfl(x.l, src)};
}
__device__ __forceinline__ F32Row4 shfl(F32Row4 x, int src) {
  return {shfl(x.a, src), shfl(x.b, src)};
}
__device__ __forceinline__ F64Row2 shfl(F64Row2 x, int src) {
  return {shfl(x.x, src), shfl(x.y, src)};
}

// Shared-memory staging layout of one tile: column w, chunk c, slot j at
//   w * pitch + c * (R + 1) + j,   pitch = G * (R + 1) rounded up to odd.
// The per-chunk pad makes the chunk reads of a warp (lanes = consecutive
// chunks) conflict free; the odd column pitch makes the coalesced copy
// (lanes = consecutive columns of one row) conflict free.
template <int R>
__device__ __forceinline__ int stage_pitch(int G) {
  return (G * (R + 1)) | 1;
}

// Column pitch of a staged tile of 2^log2cols columns of G chunks. Narrow
// rows of RL = min(inner extent, columns) <= 2^kNarrowRowLog2 elements are
// loaded with consecutive lanes along a row (TileCopy::rows_load), so a warp
// covers RL columns of 32 / RL consecutive rows. With G >= 32 a warp's chunk
// reads lie in one column and the pitch does not matter to them; then
// pitch = 32 / RL (mod 32) puts the warp's copies at banks q * 32 / RL + r,
// all distinct (an odd pitch would give conflicts). Otherwise the pitch is
// odd (stage_pitch). The tile still fits lift_smem_bytes: the pitch grows by
// at most 31 and cols <= rounds * NT / 32.
constexpr int kNarrowRowLog2 = 3;  // rows of up to 8 elements: rows_load

template <int R, typename S>
__device__ __forceinline__ int tile_pitch(int G, int log2_inner,
                                          int log2cols, bool contiguous) {
  int const base = G * (R + 1);
  int const log2RL = log2_inner < log2cols ? log2_inner : log2cols;
  if (G < 32 || contiguous || log2RL > kNarrowRowLog2) return base | 1;
  int const want = 32 >> log2RL;
  return base + ((want - base) & 31);
}

// Exchanges between the chunks of one column during the level steps of a
// round. When G <= 32 the chunks of a column are lanes of one warp and
// exchange by shuffle: chunk c is lane (lane & ~mask) | (c << log2ls) with
// mask = (G - 1) << log2ls, i.e. consecutive lanes (log2ls = 0) or lanes
// 2^log2ls apart (the wide kernel, whose neighbouring lanes hold
// neighbouring columns). Longer columns exchange through shared memory with
// one barrier per step (the same for every thread of the CTA: G is uniform
// per tile). SHFL: the caller guarantees G <= 32 (the shared-memory paths
// compile out); MAXG: the most chunks a pencil of the caller has (longer
// head pencils compile out).
template <class A, int NT, bool SHFL = false, int MAXG = 256>
struct RoundCtx {
  using V = typename A::V;
  static constexpr bool kShflOnly = SHFL;
  static constexpr int kMaxG = MAXG;
  // Chunk heads of one column are consecutive threads (coarse_heads may
  // run a column's coarse levels as a pencil of heads in one warp).
  static constexpr bool kHeadPencil = true;
  int t, c, G, log2G, log2ls, gbase_lane, periodic;
  V *heads, *xch;
  int buf = 0;
  bool heads_valid = false;

  __device__ __forceinline__ RoundCtx(int t_, int c_, int G_, int log2G_,
                                      int lane, int periodic_, V *heads_,
                                      V *xch_, int log2ls_ = 0)
      : t(t_), c(c_), G(G_), log2G(log2G_), log2ls(log2ls_),
        gbase_lane(lane & ~((G_ - 1) << log2ls_)), periodic(periodic_),
        heads(heads_), xch(xch_) {}

  __device__ __forceinline__ int chunk_lane(int cc) const {
    return gbase_lane | ((cc & (G - 1)) << log2ls);
  }
  __device__ __forceinline__ void sync() const { __syncthreads(); }

  // The neighbour of a fine step: slot 0 of the next chunk (o = 1) or slot
  // R - s of the previous chunk (o = 0); `pub` is this chunk's value of it.
  __device__ __forceinline__ V fine_neighbor(int o, V pub) {
    if (G == 1) return pub;
    int nc = (o == 1) ? c + 1 : c - 1;
    if (SHFL || G <= 32) return shfl(pub, chunk_lane(nc));
    xch[buf * NT + t] = pub;
    sync();
    if (periodic)
      nc &= G - 1;
    else
      nc = nc < 0 ? 0 : (nc >= G ? G - 1 : nc);
    V const r = xch[buf * NT + ((t >> log2G) << log2G) + nc];
    buf ^= 1;
    return r;
  }
  __device__ __forceinline__ void fine_wrote_heads(int o) {
    if (o == 0) heads_valid = false;  // slot 0 changed
  }

  // One coarse step (distance d chunks) on the chunk heads.
  template <class Upd>
  __device__ __forceinline__ void coarse(V &v0, int o, int d, Upd upd) {
    bool const mine = (c & (2 * d - 1)) == o * d;
    if (SHFL || G <= 32) {
      V const lo = shfl(v0, chunk_lane(c - d));
      V const up = shfl(v0, chunk_lane(c + d));
      if (mine) v0 = upd(lo, v0, up);
      return;
    }
    if (!heads_valid) {
      heads[t] = v0;
      sync();
      heads_valid = true;
    }
    if (mine) {
      int cl = c - d, cu = c + d;
      if (periodic) {
        cl &= G - 1;
        cu &= G - 1;
      } else {
        cl = cl < 0 ? c : cl;
        cu = cu >= G ? c : cu;
      }
      int const colbase = (t >> log2G) << log2G;
      v0 = upd(heads[colbase + cl], v0, heads[colbase + cu]);
      heads[t] = v0;
    }
    sync();
  }
};

// Schedule for arbitrary level lists and filters (transform_in): levels,
// parities and coefficients are read per step.
struct RuntimeSched {
  static constexpr bool kSplit = false;  // no fine_only / coarse_only
  template <class A, int R, int NT, class Ctx>
  static __device__ __forceinline__ void run(typename A::V (&v)[R],
                                             Ctx &ctx,
                                             LiftJob const &job,
                                             LiftParams const &p) {
    using V = typename A::V;
    constexpr int LOG2R = Log2<R>::value;
    int const nlev = job.nlevels;
    for (int li = 0; li < nlev; ++li) {
      int const sh = job.shift[li];
      for (int ps = 0; ps < p.npasses; ++ps) {
        int const o = p.offsets[ps];
        Coeffs const cf = p.coeffs[ps];
        bool const c1one = (p.c1_one_mask >> ps) & 1u;
        if (sh < LOG2R) {
          V const pub = (o == 1) ? v[0] : tail_value<R>(v, sh);
          V const nb = ctx.fine_neighbor(o, pub);
          fine_dispatch<A, R>(v, sh, o, nb, cf, c1one);
          ctx.fine_wrote_heads(o);
        } else {
          ctx.coarse(v[0], o, 1 << (sh - LOG2R), [&](V lo, V me, V up) {
            return coarse_update<A>(cf, c1one, lo, me, up);
          });
        }
      }
    }
  }
};

// Wavelet tables at compile time (paliwa/paliwa_wavelets.hpp:15-28).
template <int O, int C0N, int C1N, int C2N, int DEN> struct Pass {
  static constexpr int offset = O;
  static constexpr bool c1one = C1N == DEN;
  static __device__ __forceinline__ constexpr Coeffs coeffs() {
    return {double(C0N) / DEN, double(C1N) / DEN, double(C2N) / DEN,
            float(C0N) / DEN,  float(C1N) / DEN,  float(C2N) / DEN};
  }
};
template <class... P> struct PassList {
  static constexpr int size = sizeof...(P);
};
template <int W, bool FWD> struct WaveletPasses;
// hat: forward {(1, {-1/2, 1, -1/2})}, inverse {(1, {1/2, 1, 1/2})}
template <> struct WaveletPasses<0, true> {
  using type = PassList<Pass<1, -2, 4, -2, 4>>;
};
template <> struct WaveletPasses<0, false> {
  using type = PassList<Pass<1, 2, 4, 2, 4>>;
};
// biorthogonal: forward {(1, {-1/2, 1, -1/2}), (0, {1/4, 1, 1/4})},
// inverse {(0, {-1/4, 1, -1/4}), (1, {1/2, 1, 1/2})}
template <> struct WaveletPasses<1, true> {
  using type = PassList<Pass<1, -2, 4, -2, 4>, Pass<0, 1, 4, 1, 4>>;
};
template <> struct WaveletPasses<1, false> {
  using type = PassList<Pass<0, -1, 4, -1, 4>, Pass<1, 2, 4, 2, 4>>;
};
// fullweighting: forward {(0, {1/4, 1/2, 1/4}), (1, {-1/2, 1, -1/2})},
// inverse {(1, {1/2, 1, 1/2}), (0, {-1/2, 2, -1/2})}
template <> struct WaveletPasses<2, true> {
  using type = PassList<Pass<0, 1, 2, 1, 4>, Pass<1, -2, 4, -2, 4>>;
};
template <> struct WaveletPasses<2, false> {
  using type = PassList<Pass<1, 2, 4, 2, 4>, Pass<0, -2, 8, -2, 4>>;
};

// Schedule of hierarchize (FWD: levels fine to coarse, distances 1, 2, 4, ...)
// and dehierarchize (coarse to fine) with a compile-time wavelet: the fine
// levels are unrolled with compile-time distance, parity and coefficients.
// The job's shifts are 0 .. L-1 (FWD) or L-1 .. 0.
template <int W, bool FWD> struct WaveletSched {
  using Passes = typename WaveletPasses<W, FWD>::type;
  static constexpr bool kForward = FWD;
  static constexpr bool kSplit = true;  // fine_only / coarse_only below

  template <class A, int R, int NT, int K, class P, class Ctx>
  static __device__ __forceinline__ void fine_pass(typename A::V (&v)[R],
                                                   Ctx &ctx) {
    using V = typename A::V;
    constexpr int S = 1 << K;
    constexpr Coeffs cf = P::coeffs();
    V const pub = P::offset == 1 ? v[0] : v[R - S];
    V const nb = ctx.fine_neighbor(P::offset, pub);
    if constexpr (P::offset == 1) {
#pragma unroll
      for (int j = S; j < R; j += 2 * S) {
        V const up = (j + S < R) ? v[(j + S) % R] : nb;
        v[j] = A::template update<P::c1one>(cf, v[j - S], v[j], up);
      }
    } else {
#pragma unroll
      for (int j = 0; j < R; j += 2 * S) {
        V const lo = (j >= S) ? v[(j + R - S) % R] : nb;
        v[j] = A::template update<P::c1one>(cf, lo, v[j], v[j + S]);
      }
    }
    ctx.fine_wrote_heads(P::offset);
  }

  template <class A, int R, int NT, int K, class... P, class Ctx>
  static __device__ __forceinline__ void fine_level(typename A::V (&v)[R],
                                                    Ctx &ctx,
                                                    PassList<P...>) {
    (fine_pass<A, R, NT, K, P>(v, ctx), ...);
  }

  template <class A, int R, int NT, class... P, class Ctx>
  static __device__ __forceinline__ void coarse_level(typename A::V (&v)[R],
                                                      Ctx &ctx,
                                                      int d, PassList<P...>) {
    using V = typename A::V;
    (ctx.coarse(v[0], P::offset, d,
                [](V lo, V me, V up) {
                  constexpr Coeffs cf = P::coeffs();
                  return A::template update<P::c1one>(cf, lo, me, up);
                }),
     ...);
  }

  template <class A, int R, int NT, int K, class Ctx>
  static __device__ __forceinline__ void fine_up(typename A::V (&v)[R],
                                                 Ctx &ctx, int L) {
    if constexpr ((1 << K) < R) {
      if (K < L) {
        fine_level<A, R, NT, K>(v, ctx, Passes{});
        fine_up<A, R, NT, K + 1>(v, ctx, L);
      }
    }
  }
  template <class A, int R, int NT, int K, class Ctx>
  static __device__ __forceinline__ void fine_down(typename A::V (&v)[R],
                                                   Ctx &ctx,
                                                   int L) {
    if constexpr (K >= 0) {
      if (K < L) fine_level<A, R, NT, K>(v, ctx, Passes{});
      fine_down<A, R, NT, K - 1>(v, ctx, L);
    }
  }

  // ---- packed variant (A::kPacked): registers hold pairs (slot x,
  // slot x + R/2) so that fine steps of distance <= R/4 update two points
  // per f32x2 instruction.
  template <class A, int R, int NT, int K, class P, class Ctx>
  static __device__ __forceinline__ void fine_pass_packed(DF2 (&q)[R / 2],
                                                          Ctx &ctx) {
    using V = typename A::V;
    constexpr int H = R / 2;
    constexpr int S = 1 << K;
    constexpr Coeffs cf = P::coeffs();
    if constexpr (2 * S <= H) {
      if constexpr (P::offset == 1) {
        V const pub = {f2_x(q[0].h), f2_x(q[0].l)};  // slot 0
        V const nb = ctx.fine_neighbor(1, pub);       // next chunk's slot 0
#pragma unroll
        for (int x = S; x < H; x += 2 * S) {
          DF2 up;
          if (x + S < H)
            up = q[(x + S) % H];
          else  // slots (H, R): this chunk's slot H, next chunk's slot 0
            up = {f2_pack(f2_y(q[0].h), nb.h), f2_pack(f2_y(q[0].l), nb.l)};
          q[x] = sym_update2<P::c1one>(cf, q[x - S], q[x], up);
        }
      } else {
        V const pub = {f2_y(q[H - S].h), f2_y(q[H - S].l)};  // slot R - S
        V const nb = ctx.fine_neighbor(0, pub);  // previous chunk's R - S
#pragma unroll
        for (int x = 0; x < H; x += 2 * S) {
          DF2 lo;
          if (x >= S)
            lo = q[(x + H - S) % H];
          else  // slots (-S, H - S)
            lo = {f2_pack(nb.h, f2_x(q[H - S].h)),
                  f2_pack(nb.l, f2_x(q[H - S].l))};
          q[x] = sym_update2<P::c1one>(cf, lo, q[x], q[x + S]);
        }
        ctx.fine_wrote_heads(0);
      }
    } else {  // S == H: the two halves' first slots, one scalar update
      V s0 = {f2_x(q[0].h), f2_x(q[0].l)};  // slot 0
      V sH = {f2_y(q[0].h), f2_y(q[0].l)};  // slot H
      if constexpr (P::offset == 1) {
        V const nb = ctx.fine_neighbor(1, s0);
        sH = A::template update<P::c1one>(cf, s0, sH, nb);
      } else {
        V const nb = ctx.fine_neighbor(0, sH);  // previous chunk's slot H
        s0 = A::template update<P::c1one>(cf, nb, s0, sH);
        ctx.fine_wrote_heads(0);
      }
      q[0].h = f2_pack(s0.h, sH.h);
      q[0].l = f2_pack(s0.l, sH.l);
    }
  }

  template <class A, int R, int NT, int K, class... P, class Ctx>
  static __device__ __forceinline__ void fine_level_packed(
      DF2 (&q)[R / 2], Ctx &ctx, PassList<P...>) {
    (fine_pass_packed<A, R, NT, K, P>(q, ctx), ...);
  }
  template <class A, int R, int NT, int K, class Ctx>
  static __device__ __forceinline__ void fine_up_packed(DF2 (&q)[R / 2],
                                                        Ctx &ctx,
                                                        int L) {
    if constexpr ((1 << K) < R) {
      if (K < L) {
        fine_level_packed<A, R, NT, K>(q, ctx, Passes{});
        fine_up_packed<A, R, NT, K + 1>(q, ctx, L);
      }
    }
  }
  template <class A, int R, int NT, int K, class Ctx>
  static __device__ __forceinline__ void fine_down_packed(
      DF2 (&q)[R / 2], Ctx &ctx, int L) {
    if constexpr (K >= 0) {
      if (K < L) fine_level_packed<A, R, NT, K>(q, ctx, Passes{});
      fine_down_packed<A, R, NT, K - 1>(q, ctx, L);
    }
  }
  // Coarse levels act on slot 0 only: unpack it, run them, pack it back.
  template <class A, int R, int NT, class Ctx>
  static __device__ __forceinline__ void coarse_packed(DF2 (&q)[R / 2],
                                                       Ctx &ctx,
                                                       int sh_first,
                                                       int sh_last, int step) {
    using V = typename A::V;
    constexpr int LOG2R = Log2<R>::value;
    if ((step > 0 && sh_first > sh_last) || (step < 0 && sh_first < sh_last))
      return;
    V s0[1] = {{f2_x(q[0].h), f2_x(q[0].l)}};
    if (!coarse_heads<A, R, NT>(s0[0], ctx, (step > 0 ? sh_last : sh_first) -
                                               LOG2R + 1)) {
      for (int sh = sh_first;; sh += step) {
        coarse_level<A, 1, NT>(s0, ctx, 1 << (sh - LOG2R), Passes{});
        if (sh == sh_last) break;
      }
    }
    q[0].h = f2_pack(s0[0].h, f2_y(q[0].h));
    q[0].l = f2_pack(s0[0].l, f2_y(q[0].l));
  }

  // The coarse levels of pencils of more than 32 chunks (staged kernel,
  // chunks in consecutive threads): instead of one shared-memory exchange
  // and barrier per level pass, the chunk heads go to shared memory once,
  // one warp per column runs all Lc coarse levels on its column's G heads as
  // a pencil of 32 chunks of G / 32 heads (shuffles only: the same updates
  // in the same order), and the heads come back. Returns false (nothing
  // done) when the pencil has at most 32 chunks. Called by every thread.
  template <int K, class A, int NT>
  static __device__ __forceinline__ void head_pencil(typename A::V *col,
                                                     int lane, int periodic,
                                                     int Lc) {
    using V = typename A::V;
    V hv[K];
#pragma unroll
    for (int k = 0; k < K; ++k) hv[k] = col[lane * K + k];
    RoundCtx<A, NT> hctx(lane, lane, 32, 5, lane, periodic, nullptr, nullptr);
    run_levels<A, K, NT>(hv, hctx, Lc);
#pragma unroll
    for (int k = 0; k < K; ++k) col[lane * K + k] = hv[k];
  }
  template <class A, int R, int NT, class Ctx>
  static __device__ __forceinline__ bool coarse_heads(typename A::V &head,
                                                      Ctx &ctx,
                                                      int Lc) {
    if constexpr (R < 16 || !Ctx::kHeadPencil || Ctx::kShflOnly) {
      return false;
    } else {
      if (ctx.G <= 32 || ctx.G > 256) return false;
      using V = typename A::V;
      ctx.heads[ctx.t] = head;
      ctx.sync();
      int const w = ctx.t >> 5;
      int const lane = ctx.t & 31;
      if (w < (NT >> ctx.log2G)) {  // one warp per column of the round
        V *const col = ctx.heads + (w << ctx.log2G);
        switch (ctx.G) {
        case 64: head_pencil<2, A, NT>(col, lane, ctx.periodic, Lc); break;
        case 128:
          if constexpr (Ctx::kMaxG >= 128)
            head_pencil<4, A, NT>(col, lane, ctx.periodic, Lc);
          break;
        case 256:
          if constexpr (Ctx::kMaxG >= 256)
            head_pencil<8, A, NT>(col, lane, ctx.periodic, Lc);
          break;
        }
      }
      ctx.sync();
      head = ctx.heads[ctx.t];
      ctx.heads_valid = false;
      return true;
    }
  }

  template <class A, int R, int NT, class Ctx>
  static __device__ __forceinline__ void run(typename A::V (&v)[R],
                                             Ctx &ctx,
                                             LiftJob const &job,
                                             LiftParams const &) {
    run_levels<A, R, NT>(v, ctx, job.nlevels);
  }

  // The fine levels (shifts below log2 R) of run_levels alone, the same
  // operations in the same order; with coarse_only on the chunk heads after
  // (forward) or before (inverse) them, they make up run_levels.
  template <class A, int R, int NT, class Ctx>
  static __device__ __forceinline__ void fine_only(typename A::V (&v)[R],
                                                   Ctx &ctx, int L) {
    constexpr int LOG2R = Log2<R>::value;
    if constexpr (A::kPacked && R >= 4) {
      constexpr int H = R / 2;
      DF2 q[H];
#pragma unroll
      for (int x = 0; x < H; ++x) {
        q[x].h = f2_pack(v[x].h, v[x + H].h);
        q[x].l = f2_pack(v[x].l, v[x + H].l);
      }
      if constexpr (FWD)
        fine_up_packed<A, R, NT, 0>(q, ctx, L);
      else
        fine_down_packed<A, R, NT, LOG2R - 1>(q, ctx, L);
#pragma unroll
      for (int x = 0; x < H; ++x) {
        v[x] = {f2_x(q[x].h), f2_x(q[x].l)};
        v[x + H] = {f2_y(q[x].h), f2_y(q[x].l)};
      }
    } else {
      if constexpr (FWD)
        fine_up<A, R, NT, 0>(v, ctx, L);
      else
        fine_down<A, R, NT, LOG2R - 1>(v, ctx, L);
    }
  }
  // The coarse levels (shifts log2 R .. L-1) of run_levels alone, on the
  // chunk head `head` of chunks of R points (A may hold the heads of several
  // columns, e.g. a row policy with one column per lane of a pair).
  template <class A, int R, int NT, class Ctx>
  static __device__ __forceinline__ void coarse_only(typename A::V &head,
                                                     Ctx &ctx, int L) {
    constexpr int LOG2R = Log2<R>::value;
    if (L <= LOG2R) return;
    typename A::V h1[1] = {head};
    if (!coarse_heads<A, R, NT>(h1[0], ctx, L - LOG2R)) {
      if constexpr (FWD) {
        for (int sh = LOG2R; sh < L; ++sh)
          coarse_level<A, 1, NT>(h1, ctx, 1 << (sh - LOG2R), Passes{});
      } else {
        for (int sh = L - 1; sh >= LOG2R; --sh)
          coarse_level<A, 1, NT>(h1, ctx, 1 << (sh - LOG2R), Passes{});
      }
    }
    head = h1[0];
  }

  // The L levels of a job (shifts 0 .. L-1 forward, L-1 .. 0 inverse).
  template <class A, int R, int NT, class Ctx>
  static __device__ __forceinline__ void run_levels(typename A::V (&v)[R],
                                                    Ctx &ctx,
                                                    int L) {
    constexpr int LOG2R = Log2<R>::value;
    if constexpr (A::kPacked && R >= 4) {
      constexpr int H = R / 2;
      DF2 q[H];
#pragma unroll
      for (int x = 0; x < H; ++x) {
        q[x].h = f2_pack(v[x].h, v[x + H].h);
        q[x].l = f2_pack(v[x].l, v[x + H].l);
      }
      if constexpr (FWD) {
        fine_up_packed<A, R, NT, 0>(q, ctx, L);
        coarse_packed<A, R, NT>(q, ctx, LOG2R, L - 1, 1);
      } else {
        coarse_packed<A, R, NT>(q, ctx, L - 1, LOG2R, -1);
        fine_down_packed<A, R, NT, LOG2R - 1>(q, ctx, L);
      }
#pragma unroll
      for (int x = 0; x < H; ++x) {
        v[x] = {f2_x(q[x].h), f2_x(q[x].l)};
        v[x + H] = {f2_y(q[x].h), f2_y(q[x].l)};
      }
      return;
    }
    if constexpr (FWD) {
      fine_up<A, R, NT, 0>(v, ctx, L);
      if (L <= LOG2R || !coarse_heads<A, R, NT>(v[0], ctx, L - LOG2R))
        for (int sh = LOG2R; sh < L; ++sh)
          coarse_level<A, R, NT>(v, ctx, 1 << (sh - LOG2R), Passes{});
    } else {
      if (L <= LOG2R || !coarse_heads<A, R, NT>(v[0], ctx, L - LOG2R))
        for (int sh = L - 1; sh >= LOG2R; --sh)
          coarse_level<A, R, NT>(v, ctx, 1 << (sh - LOG2R), Passes{});
      fine_down<A, R, NT, LOG2R - 1>(v, ctx, L);
    }
  }
};

// Asynchronous 4-, 8- or 16-byte copy from global to shared memory (sm_80+):
// loads stay in flight without occupying registers. The copies go through
// L1 (.ca): a warp's copies often cover only part of each 32-byte sector,
// and the rest of the sector is read by the next copy instructions.
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, void const *gmem) {
  unsigned const dst = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst),
               "l"(gmem), "n"(BYTES)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// Waits until at most N of this thread's most recent groups are in flight.
template <int N> __device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// R values of one pencil: 16-byte vectors when contiguous and aligned,
// otherwise element by element at stride kstride.
template <typename S, int R>
__device__ __forceinline__ void load_chunk(S const *p, long long kstride,
                                           bool vec, S (&out)[R]) {
  constexpr int PER = 16 / sizeof(S);
  if constexpr (R % PER == 0) {
    if (vec) {
#pragma unroll
      for (int q = 0; q < R / PER; ++q) {
        uint4 u = *reinterpret_cast<uint4 const *>(p + q * PER);
        S tmp[PER];
        memcpy(tmp, &u, 16);
#pragma unroll
        for (int e = 0; e < PER; ++e) out[q * PER + e] = tmp[e];
      }
      return;
    }
  }
#pragma unroll
  for (int j = 0; j < R; ++j) out[j] = p[j * kstride];
}

template <typename S, int R>
__device__ __forceinline__ void store_chunk(S *p, long long kstride, bool vec,
                                            S const (&in)[R]) {
  constexpr int PER = 16 / sizeof(S);
  if constexpr (R % PER == 0) {
    if (vec) {
#pragma unroll
      for (int q = 0; q < R / PER; ++q) {
        S tmp[PER];
#pragma unroll
        for (int e = 0; e < PER; ++e) tmp[e] = in[q * PER + e];
        uint4 u;
        memcpy(&u, tmp, 16);
        *reinterpret_cast<uint4 *>(p + q * PER) = u;
      }
      return;
    }
  }
#pragma unroll
  for (int j = 0; j < R; ++j) p[j * kstride] = in[j];
}

// Copies one tile between global memory and the staging layout.
//
// The tile is `cols` consecutive columns (global column index gc0 + w) by
// 2^log2W pencil points. A column index splits into (a, b) with b < inner; the
// point k of column (a, b) lives at element
//   a * astride + b + pos(k) * kstride,  pos(k) = (wstart + k) mod n.
// Three paths, chosen per tile (uniform over the CTA):
//  * rows: memory rows of RL = min(inner, cols) >= VEC contiguous elements,
//    copied as 16-byte vectors (strided axes);
//  * pencils: inner == 1 and kstride == 1, each column contiguous along k,
//    copied as 16-byte vectors (the last axis);
//  * scalar: anything else (narrow inner extents, sub-lattices).
// Stores (Store == true) keep only in-range columns and, for windows, the
// points k in [halo, halo + seg_len) that fall inside the pencil. Loads of a
// window take those points from the grid and every other point from the
// halo buffer (same offsets).
template <typename S, int R, int NT> struct TileCopy {
  static constexpr int VEC = 16 / sizeof(S);
  static constexpr int LOG2R = Log2<R>::value;
  LiftJob const &job;
  int periodic, log2W, cols, pitch;
  long long gc0, wstart, n;
  unsigned char *gbase, *hbase;

  __device__ TileCopy(LiftJob const &j, int per, int lw, int c, long long g0,
                      long long ws, long long nn, int pt, unsigned char *gb)
      : job(j), periodic(per), log2W(lw), cols(c), pitch(pt), gc0(g0),
        wstart(ws), n(nn), gbase(gb),
        hbase(j.halo_base ? reinterpret_cast<unsigned char *>(j.halo_base)
                          : gb) {}

  // Point k of the tile belongs to the window's own segment (always, for a
  // periodic pencil): it is loaded from the grid, else from the halo buffer.
  // Segment bounds are multiples of 16 points, so a vector of up to 16
  // consecutive points along k is either all inside or all outside.
  __device__ __forceinline__ bool own(int k) const {
    return periodic || (static_cast<unsigned>(k - job.halo) <
                            static_cast<unsigned>(job.seg_len) &&
                        wstart + k < n);
  }
  __device__ __forceinline__ S const *source(int k) const {
    return reinterpret_cast<S const *>(own(k) ? gbase : hbase);
  }

  __device__ __forceinline__ int sidx(int w, int k) const {
    return w * pitch + (k >> LOG2R) * (R + 1) + (k & (R - 1));
  }
  __device__ __forceinline__ long long pos(int k) const {
    long long p = wstart + k;
    if (!periodic) {
      p %= n;
      if (p < 0) p += n;
    }
    return p;
  }
  __device__ __forceinline__ bool keep(long long seg, int k, int halo,
                                       int seg_len) const {
    if (periodic) return true;
    return k >= halo && k < halo + seg_len &&
           seg * seg_len + (k - halo) < n;
  }

  // True when the tile is copied along k as 16-byte vectors (each column a
  // contiguous pencil: the last axis); otherwise row by row.
  static __device__ __forceinline__ bool contiguous(LiftJob const &j) {
    bool const aligned = ((j.base | j.dst_base) & 15ull) == 0;
    return aligned && VEC > 1 && j.log2_inner == 0 && j.log2_kstride == 0 &&
           R >= VEC;
  }

  // Row-wise load of narrow rows (RL = 2^log2RL <= 2^kNarrowRowLog2
  // elements; row rho = (a_off, k)): one element per lane and step with
  // consecutive lanes along a row, so a warp's 32 asynchronous copies read
  // 32 / RL rows and, with tile_pitch, write 32 distinct banks. Copying a
  // whole vector per lane (rows) would touch 32 rows per instruction, as the
  // elements of a vector land `pitch` apart and each is one copy. When the
  // tile lies in one outer slab (inner >= cols, so a_off = 0), consecutive
  // steps are a constant number of rows apart, a multiple of R: addresses
  // advance by constants (for windows, modulo the pencil length).
  __device__ __forceinline__ void rows_load(S *stage, int t,
                                            int log2RL) const {
    constexpr int PER = kTileRounds * R;  // elements per thread
    S const *const g = reinterpret_cast<S const *>(gbase);
    int const log2B = job.log2_inner;
    long long const base = ((gc0 >> log2B) << job.log2_astride) +
                           (gc0 & ((1LL << log2B) - 1));
    long long const room = job.columns - gc0;  // columns left in the job
    int const rmask = (1 << log2RL) - 1;
    int const q = t & rmask;  // the same in every step: NT is a multiple
    if (log2B >= 31 - __clz(cols)) {
      if (q >= room) return;
      int const drho = NT >> log2RL;  // rows per step, a multiple of R
      int k = t >> log2RL;
      long long pk = pos(k);  // pencil position of row k
      int sb = sidx(q, k);
      int const dsb = (drho >> LOG2R) * (R + 1);
      S const *const gq = g + base + q;
      S const *const hq = reinterpret_cast<S const *>(hbase) + base + q;
#pragma unroll 8
      for (int i = 0; i < PER; ++i) {
        cp_async<sizeof(S)>(stage + sb,
                            (own(k) ? gq : hq) + (pk << job.log2_kstride));
        k += drho;
        pk += drho;
        if (pk >= n) pk -= n;  // a window wrapping around the period
        sb += dsb;
      }
      return;
    }
    int const kmask = (1 << log2W) - 1;
#pragma unroll 4
    for (int i = 0; i < PER; ++i) {
      int const rho = (t + i * NT) >> log2RL;
      int const k = rho & kmask;
      int const a_off = rho >> log2W;
      int const w = (a_off << log2RL) + q;
      if (w >= room) continue;
      long long const off =
          base + (static_cast<long long>(a_off) << job.log2_astride) +
          (pos(k) << job.log2_kstride) + q;
      cp_async<sizeof(S)>(stage + sidx(w, k), source(k) + off);
    }
  }

  // Rows of RL = min(inner, cols) contiguous elements; row rho = (a_off, k);
  // VW elements per memory access (VW * sizeof(S) <= 16 bytes). A tile holds
  // exactly NT * PER vectors, and every thread issues all of its loads before
  // it writes any of them to shared memory, to keep PER loads in flight.
  template <bool Store, int VW>
  __device__ __forceinline__ void rows(S *stage, int t, long long seg,
                                       int halo, int seg_len, int log2RL) const {
    using U = typename std::conditional<
        VW * sizeof(S) == 16, uint4,
        typename std::conditional<VW * sizeof(S) == 8, uint2,
                                  unsigned>::type>::type;
    static_assert(VW * sizeof(S) == sizeof(U), "vector width");
    constexpr int PER = kTileRounds * R / VW;  // vectors per thread
    S *const g = reinterpret_cast<S *>(
        Store ? reinterpret_cast<unsigned char *>(job.dst_base) : gbase);
    int const log2B = job.log2_inner;
    int const log2vpr = log2RL - Log2<VW>::value;
    long long const a0 = gc0 >> log2B;
    long long const b0 = gc0 & ((1LL << log2B) - 1);
    long long const columns = job.columns;
    if ((1 << log2RL) == cols) {
      // The rows span the tile's columns (one outer slab): every vector of
      // this thread has the same column q * VW, and its row advances by
      // dk = NT / (vectors per row) per step, so offsets advance by
      // constants (modulo the pencil for windows).
      int const q = t & ((1 << log2vpr) - 1);
      int const w0 = q * VW;
      if (gc0 + w0 >= columns) return;
      int const dk = NT >> log2vpr;
      int k = t >> log2vpr;
      long long pk = pos(k);
      long long const obase = (a0 << job.log2_astride) + b0 + w0;
      int const sbase = w0 * pitch;
#pragma unroll 4
      for (int i = 0; i < PER; ++i) {
        int const sb = sbase + (k >> LOG2R) * (R + 1) + (k & (R - 1));
        long long const off = obase + (pk << job.log2_kstride);
        if constexpr (Store) {
          if (keep(seg, k, halo, seg_len)) {
            S tmp[VW];
#pragma unroll
            for (int e = 0; e < VW; ++e) tmp[e] = stage[sb + e * pitch];
            U u;
            memcpy(&u, tmp, sizeof(U));
            *reinterpret_cast<U *>(g + off) = u;
          }
        } else {
          S const *const src = source(k) + off;
#pragma unroll
          for (int e = 0; e < VW; ++e)
            cp_async<sizeof(S)>(stage + sb + e * pitch, src + e);
        }
        k += dk;
        pk += dk;
        if (pk >= n) pk -= n;  // a window wrapping around the period
      }
      return;
    }
    auto locate = [&](int v, long long &off, int &sb, int &k) -> bool {
      int const rho = v >> log2vpr;
      int const q = v & ((1 << log2vpr) - 1);
      k = rho & ((1 << log2W) - 1);
      int const a_off = rho >> log2W;
      int const w0 = (a_off << log2RL) + q * VW;
      off = ((a0 + a_off) << job.log2_astride) + b0 +
            (pos(k) << job.log2_kstride) + q * VW;
      sb = sidx(w0, k);
      return gc0 + w0 < columns && (!Store || keep(seg, k, halo, seg_len));
    };
#pragma unroll 4
    for (int i = 0; i < PER; ++i) {
      long long off;
      int sb, k;
      bool const ok = locate(t + i * NT, off, sb, k);
      if (!ok) continue;
      if constexpr (Store) {
        S tmp[VW];
#pragma unroll
        for (int e = 0; e < VW; ++e) tmp[e] = stage[sb + e * pitch];
        U u;
        memcpy(&u, tmp, sizeof(U));
        *reinterpret_cast<U *>(g + off) = u;
      } else {
        // element-wise asynchronous copies into the padded layout (the
        // elements of one vector land `pitch` apart)
        S const *const src = source(k) + off;
#pragma unroll
        for (int e = 0; e < VW; ++e)
          cp_async<sizeof(S)>(stage + sb + e * pitch, src + e);
      }
    }
  }

  template <bool Store>
  __device__ __forceinline__ void run(S *stage, int t, long long seg,
                                      int halo, int seg_len) const {
    int const log2B = job.log2_inner;
    int const log2cols = 31 - __clz(cols);
    S *const g = reinterpret_cast<S *>(
        Store ? reinterpret_cast<unsigned char *>(job.dst_base) : gbase);
    long long const columns = job.columns;
    bool const aligned = ((job.base | job.dst_base) & 15ull) == 0;
    if (aligned && VEC > 1 && log2B == 0 && job.log2_kstride == 0 &&
        R >= VEC) {
      // each column contiguous along k
      constexpr int PER = kTileRounds * R / VEC;
      int const log2vpc = log2W - Log2<VEC>::value;
#pragma unroll 4
      for (int i = 0; i < PER; ++i) {
        int const v = t + i * NT;
        int const w = v >> log2vpc;
        int const k = (v & ((1 << log2vpc) - 1)) * VEC;
        if (gc0 + w >= columns) continue;
        if (Store && !keep(seg, k, halo, seg_len)) continue;
        long long const off = ((gc0 + w) << job.log2_astride) + pos(k);
        int const sb = sidx(w, k);
        if constexpr (Store) {
          S tmp[VEC];
#pragma unroll
          for (int e = 0; e < VEC; ++e) tmp[e] = stage[sb + e];
          uint4 u;
          memcpy(&u, tmp, 16);
          *reinterpret_cast<uint4 *>(g + off) = u;
        } else {
          S const *const src = source(k) + off;
#pragma unroll
          for (int e = 0; e < VEC; ++e)
            cp_async<sizeof(S)>(stage + sb + e, src + e);
        }
      }
      return;
    }
    int const log2RL = log2B < log2cols ? log2B : log2cols;
    if constexpr (!Store) {
      if (log2RL <= kNarrowRowLog2) return rows_load(stage, t, log2RL);
    }
    // Vector width: as wide as the rows and the alignment allow.
    if constexpr (VEC >= 4) {
      if (aligned && log2RL >= 2)
        return rows<Store, 4>(stage, t, seg, halo, seg_len, log2RL);
    }
    if constexpr (VEC >= 2) {
      if ((((job.base | job.dst_base) & (2 * sizeof(S) - 1)) == 0) &&
          log2RL >= 1)
        return rows<Store, 2>(stage, t, seg, halo, seg_len, log2RL);
    }
    rows<Store, 1>(stage, t, seg, halo, seg_len, log2RL);
  }
};

// Moves a job cursor forward to the last job that starts at or before
// `tile`. The jobs after ji are examined 32 at a time, one per lane, with
// independent loads (tile_begin increases along the list, so the jobs that
// start at or before `tile` form a prefix). CTAs that take every
// gridDim.x-th tile step over many small jobs per tile; one job per step
// would be a chain of dependent loads per tile. Called by all lanes of the
// warp with the same tile.
__device__ __forceinline__ int advance_job(LiftParams const &p, int ji,
                                           long long tile, int lane) {
  for (;;) {
    int const j = ji + 1 + lane;
    bool const ok = j < p.njobs && p.jobs[j].tile_begin <= tile;
    unsigned const m = __ballot_sync(0xffffffffu, ok);
    ji += __popc(m);
    if (m != 0xffffffffu) return ji;
  }
}

// Moves the job cursor `ji` forward to the job of `tile` and copies that job
// into shared memory when it changed. Called by every thread of the CTA.
// The current job lives in shared memory: its fields are read in the inner
// loops, and a generic pointer into parameter or global space would turn
// every read into a memory instruction.
template <int NT>
__device__ __forceinline__ void fetch_job(LiftParams const &p, long long tile,
                                          int t, int &ji, LiftJob &sjob,
                                          int &sjob_index) {
  if (p.jobs != nullptr) ji = advance_job(p, ji, tile, t & 31);
  if (sjob_index != ji) {
    __syncthreads();  // every thread has read sjob_index
    constexpr int WORDS = sizeof(LiftJob) / 4;
    static_assert(sizeof(LiftJob) % 4 == 0, "LiftJob is copied in words");
    unsigned const *src = reinterpret_cast<unsigned const *>(
        p.jobs != nullptr ? p.jobs + ji : &p.job);
    for (int i = t; i < WORDS; i += NT)
      reinterpret_cast<unsigned *>(&sjob)[i] = src[i];
    if (t == 0) sjob_index = ji;
    __syncthreads();
  }
}

// The two column rounds of a staged tile with their coarse levels run
// together: FP32-compensated chunks under a wavelet schedule whose pencils
// have coarse levels (more than R points). The fine levels run round by
// round as before; the two rounds' chunk heads (columns w and w + NT / G,
// both held by this thread) then form one pair of a row policy of two
// columns, so each coarse step updates both heads with one set of f32x2
// operations (the same operations per column: the results are the same
// bits) and the coarse steps' latency chains are shared by two columns.
// Forward runs fine levels, then the coarse levels on the heads; inverse
// the reverse. During the coarse levels the exchange buffer holds the
// pairs. Returns false (nothing done) when the tile does not qualify.
template <class A, int R, int NT, class Sched>
__device__ __forceinline__ bool staged_split_rounds(
    typename A::Store *stage, int pitch, int G, int log2G, int log2CR, int t,
    int lane, int periodic, typename A::V *heads, typename A::V *xch,
    LiftJob const &job) {
  constexpr int LOG2R = Log2<R>::value;
  if constexpr (!Sched::kSplit || !std::is_same<A, CompensatedT<true>>::value ||
                kTileRounds != 2) {
    return false;
  } else {
    using V = typename A::V;
    using S = typename A::Store;
    using AR = RowF32C;
    int const L = job.nlevels;
    if (L <= LOG2R) return false;
    int const c = t & (G - 1);
    S *chunk[2];
#pragma unroll
    for (int r = 0; r < 2; ++r)
      chunk[r] = stage + ((r << log2CR) + (t >> log2G)) * pitch + c * (R + 1);
    V head[2];
    AR::V *const pairs = reinterpret_cast<AR::V *>(xch);  // NT pairs
    auto coarse = [&] {
      AR::V hp = {f2_pack(head[0].h, head[1].h), f2_pack(head[0].l, head[1].l)};
      RoundCtx<AR, NT> ctx2(t, c, G, log2G, lane, periodic,
                            reinterpret_cast<AR::V *>(pairs), nullptr);
      Sched::template coarse_only<AR, R, NT>(hp, ctx2, L);
      head[0] = {f2_x(hp.h), f2_x(hp.l)};
      head[1] = {f2_y(hp.h), f2_y(hp.l)};
    };
    if constexpr (!Sched::kForward) {
#pragma unroll
      for (int r = 0; r < 2; ++r) head[r] = A::load(chunk[r][0]);
      coarse();
      if (G > 32) __syncthreads();  // the pairs are out of xch
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      V v[R];
#pragma unroll
      for (int j = 0; j < R; ++j) v[j] = A::load(chunk[r][j]);
      if constexpr (!Sched::kForward) v[0] = head[r];
      RoundCtx<A, NT> ctx(t, c, G, log2G, lane, periodic, heads, xch);
      Sched::template fine_only<A, R, NT>(v, ctx, L);
      if constexpr (Sched::kForward) head[r] = v[0];
#pragma unroll
      for (int j = 0; j < R; ++j) chunk[r][j] = A::store(v[j]);
      if (G > 32) __syncthreads();  // heads / xch reused next
    }
    if constexpr (Sched::kForward) {
      coarse();
#pragma unroll
      for (int r = 0; r < 2; ++r) chunk[r][0] = A::store(head[r]);
    }
    return true;
  }
}

// Direct: every job of the launch is a periodic pencil of n == R points held
// by one thread (no staging); otherwise tiles are staged through shared
// memory. The two paths are separate instantiations so that neither's
// register budget constrains the other.
template <class A, int R, int NT, class Sched, bool Direct>
__device__ __forceinline__ void lift_body(LiftParams const &p) {
  using V = typename A::V;
  using S = typename A::Store;
  constexpr int LOG2R = Log2<R>::value;
  constexpr int LOG2NT = Log2<NT>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *heads = reinterpret_cast<V *>(smem_raw);
  V *xch = heads + NT;  // two buffers of NT
  S *stage = reinterpret_cast<S *>(xch + 2 * NT);

  int const t = threadIdx.x;
  int const lane = t & 31;
  __shared__ LiftJob sjob;
  __shared__ int sjob_index;
  LiftJob const *const job = &sjob;
  int ji = 0;
  if (t == 0) sjob_index = -1;
  // Persistent CTAs: tiles are visited in increasing order, so the job
  // cursor only moves forward.
  for (long long tile = blockIdx.x; tile < p.total_tiles; tile += gridDim.x) {
    __syncthreads();  // the previous tile is out of shared memory
    fetch_job<NT>(p, tile, t, ji, sjob, sjob_index);
    int const log2W = job->log2_window;       // points per column held
    int const log2G = log2W - LOG2R;          // chunks per column
    int const G = 1 << log2G;
    int const log2CR = LOG2NT - log2G;        // columns per round
    constexpr int rounds = kTileRounds;
    int const cols = rounds << log2CR;        // columns per tile
    int const pitch = tile_pitch<R, typename A::Store>(
        G, job->log2_inner, LOG2NT - log2G + 1,
        TileCopy<typename A::Store, R, NT>::contiguous(*job));
    static_assert(kTileRounds == 2, "tile_pitch takes log2(cols) = log2CR + 1");
    int const periodic = job->periodic;
    long long const n = 1LL << job->log2_n;

    long long const local = tile - job->tile_begin;
    // A periodic job has one segment (no 64-bit division per tile).
    long long const seg = periodic ? 0 : local / job->col_tiles;
    long long const gc0 = (local - seg * job->col_tiles) * cols;
    long long const wstart =
        periodic ? 0 : seg * job->seg_len - job->halo;  // window origin

    unsigned char *const gbase = reinterpret_cast<unsigned char *>(job->base);

    if constexpr (Direct) {
      // Pencils straight between HBM and registers, no staging and no
      // barrier: either one whole pencil per thread (n == R, lanes along
      // columns), or a contiguous pencil (last axis) of G <= 32 chunks held
      // by G consecutive lanes that exchange by shuffle.
      bool const vec = job->log2_kstride == 0 &&
                       ((job->base | job->dst_base) & 15ull) == 0;
      long long const kstride = 1LL << job->log2_kstride;
      int const log2B = job->log2_inner;
      int const c = t & (G - 1);
      for (int r = 0; r < rounds; ++r) {
        long long gc = gc0 + (r << log2CR) + (t >> log2G);
        // A warp skips only as a whole (its lanes shuffle with each other);
        // lanes past the last column of a partly filled warp recompute the
        // last column and do not store it.
        if (gc0 + (r << log2CR) + ((t & ~31) >> log2G) >= job->columns)
          continue;
        bool const keep = gc < job->columns;
        if (!keep) gc = job->columns - 1;
        long long const off = ((gc >> log2B) << job->log2_astride) +
                              (gc & ((1LL << log2B) - 1)) +
                              static_cast<long long>(c) * R * kstride;
        V v[R];
        {
          S raw[R];
          load_chunk<S, R>(reinterpret_cast<S const *>(gbase) + off, kstride,
                           vec, raw);
#pragma unroll
          for (int j = 0; j < R; ++j) v[j] = A::load(raw[j]);
        }
        RoundCtx<A, NT> ctx(t, c, G, log2G, lane, periodic, heads, xch);
        Sched::template run<A, R, NT>(v, ctx, *job, p);
        {
          S raw[R];
#pragma unroll
          for (int j = 0; j < R; ++j) raw[j] = A::store(v[j]);
          if (keep)
            store_chunk<S, R>(reinterpret_cast<S *>(job->dst_base) + off,
                              kstride, vec, raw);
        }
      }
      continue;
    } else {
    (void)G;

    // ---- load: global -> stage
    TileCopy<S, R, NT> cp(*job, periodic, log2W, cols, gc0, wstart, n, pitch,
                          gbase);
    cp.template run<false>(stage, t, seg, 0, 0);
    cp_async_wait_all();
    __syncthreads();

    // ---- compute: one round = NT / G columns, thread = (column, chunk)
    if (!staged_split_rounds<A, R, NT, Sched>(stage, pitch, G, log2G, log2CR,
                                              t, lane, periodic, heads, xch,
                                              *job)) {
      for (int r = 0; r < rounds; ++r) {
        int const c = t & (G - 1);
        int const wl = (r << log2CR) + (t >> log2G);
        S *chunk = stage + wl * pitch + c * (R + 1);
        V v[R];
#pragma unroll
        for (int j = 0; j < R; ++j) v[j] = A::load(chunk[j]);
        RoundCtx<A, NT> ctx(t, c, G, log2G, lane, periodic, heads, xch);
        Sched::template run<A, R, NT>(v, ctx, *job, p);
#pragma unroll
        for (int j = 0; j < R; ++j) chunk[j] = A::store(v[j]);
        if (G > 32) __syncthreads();  // heads / xch reused by the next round
      }
    }
    __syncthreads();

    // ---- store: stage -> global (only this tile's segment of a window)
    cp.template run<true>(stage, t, seg, job->halo, job->seg_len);
    }
  }
}

// The kernel entry points: the register budget is the compiler's for
// 256-thread CTAs, except for the staged kernel with 16-point chunks of float
// grids, which is held to three CTAs per SM (80 registers; launch code picks
// lift_kernel3 for it).
template <class A, int R, int NT, class Sched, bool Direct>
__global__ void __launch_bounds__(NT)
    lift_kernel(__grid_constant__ const LiftParams p) {
  lift_body<A, R, NT, Sched, Direct>(p);
}
template <class A, int R, int NT, class Sched, bool Direct>
__global__ void __launch_bounds__(NT, 3)
    lift_kernel3(__grid_constant__ const LiftParams p) {
  lift_body<A, R, NT, Sched, Direct>(p);
}
template <class A, int R, bool Direct>
constexpr bool lift_three_ctas() {
  return !Direct && R == 16 && sizeof(typename A::Store) == 4;
}

// Wide kernel: each thread holds the same chunk of R points of kCols
// adjacent pencils in registers (A::V is one row of them: the kCols points at
// the same pencil position), for two layouts:
//
//  * strided axes (Contig = false) whose inner extent is at least kCols,
//    pencils of up to 64 points: the G = n / R <= 4 chunks of a pencil are
//    lanes 32 / G apart, so the lanes of one warp that hold the same chunk
//    hold consecutive column groups and every row a warp reads is
//    32 / G * kCols contiguous elements;
//  * the last axis (Contig = true), pencils of up to 512 points: a thread's
//    chunk of each of its kCols pencils is R contiguous points, and the
//    G = n / R <= 32 chunks of a pencil group are consecutive lanes, so a
//    warp reads whole runs of consecutive pencils.
//
// Chunks exchange by shuffle; there is no barrier. A CTA takes a contiguous
// range of tiles (a tile is kTileRounds units; a unit is NT / G column groups
// of kCols columns). Loads are software pipelined: each thread copies the
// data of the unit WideStages - 1 ahead with cp.async into its own
// shared-memory slots while it transforms the current unit, whose data it
// then reads from those slots; results are stored straight to global memory.
template <class A> struct WideStages {
  static constexpr int value = sizeof(typename A::Store) == 16 ? 2 : 3;
};

// Geometry of one unit for one thread. Units, tiles and column groups are
// 32-bit (the planner gives the wide kernel only jobs of under 2^30 columns
// and launches of under 2^30 tiles); element offsets are 64-bit.
struct WideUnit {
  long long off;  // element offset of the thread's chunk of its first column
  int wfirst;     // first column group of the warp
  int groups;     // column groups of the job
  int c;          // chunk index
  int log2ls;     // log2 of the lane distance between chunks of a column
  bool active;    // the warp has at least one column group in range
  bool keep;      // the thread's column group is in range (else recomputed)
};

// Strided wide units whose inner extent is one or two row vectors (kCols or
// 2 kCols columns) while a warp holds more column groups than that: each
// lane's rows then lie in slabs of other outer indices than its neighbours',
// so copying row by row touches 16 to 32 lines per instruction. The warp's
// columns cover whole slabs, which lie contiguously in memory: such warps
// copy their block (32 * R row vectors) as consecutive 16-byte pieces
// instead, into their shared-memory region with an XOR swizzle of the piece
// index (piece b at b ^ ((b >> 3) & 7): the 8 pieces of a 128-byte line
// rotate with the line), and each thread reads its rows from there. With
// wider inner extents the row-by-row copy touches 8 lines or fewer and its
// fewer instructions win (measured: block copies for inner extents up to
// 32 kCols made the 4D CT step 2 % slower). Only the 16-point units use it:
// for R = 4 and 8 its address work cost more than the copies it saved.
struct WideBlock {
  static __device__ __forceinline__ bool use(LiftJob const &job,
                                             WideUnit const &w, int log2gw,
                                             int log2cw) {
    return job.log2_inner <= log2cw + 1 && log2cw + 1 < log2gw + log2cw &&
           job.log2_kstride == job.log2_inner &&
           job.log2_astride == job.log2_n + job.log2_inner &&
           w.wfirst + (1 << log2gw) <= w.groups &&
           ((job.base | job.dst_base) & 15ull) == 0;
  }
  static __device__ __forceinline__ int swz(int b) {
    return b ^ ((b >> 3) & 7);
  }
};

template <int LOG2R, int LOG2NT, int LOG2CW, bool Contig>
__device__ __forceinline__ WideUnit wide_unit(LiftJob const &job, int unit,
                                              int t) {
  static_assert(kTileRounds == 2, "a tile is two units");
  int const lane = t & 31;
  int const log2G = job.log2_n - LOG2R;
  int const log2gw = 5 - log2G;  // column groups per warp
  int const log2CR = LOG2NT - log2G;
  int const local = (unit >> 1) - static_cast<int>(job.tile_begin);
  int const r = unit & 1;
  int const groups = static_cast<int>(job.columns >> LOG2CW);
  int const wfirst = (local << (log2CR + 1)) + (r << log2CR) +
                     ((t >> 5) << log2gw);
  WideUnit w;
  w.wfirst = wfirst;
  w.groups = groups;
  w.active = wfirst < groups;
  int gl;  // column group within the warp
  if (Contig) {
    w.c = lane & ((1 << log2G) - 1);
    gl = lane >> log2G;
    w.log2ls = 0;
  } else {
    w.c = lane >> log2gw;
    gl = lane & ((1 << log2gw) - 1);
    w.log2ls = log2gw;
  }
  int gg = wfirst + gl;
  w.keep = gg < groups;
  if (!w.keep) gg = groups - 1;
  int const gc = gg << LOG2CW;  // first column of the group
  int const log2B = job.log2_inner;
  w.off = (static_cast<long long>(gc >> log2B) << job.log2_astride) +
          (gc & ((1 << log2B) - 1)) +
          (static_cast<long long>(w.c) << (LOG2R + job.log2_kstride));
  return w;
}

// Last job whose first tile is <= tile (jobs sorted by tile_begin).
__device__ __forceinline__ int find_job(LiftParams const &p, long long tile) {
  int lo = 0, hi = p.njobs - 1;
  while (lo < hi) {
    int const mid = (lo + hi + 1) >> 1;
    if (p.jobs[mid].tile_begin <= tile)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// A forward-only cursor over a launch's job list, used by all lanes of a
// warp with the same tile. The cursor lives in a warp-private shared-memory
// slot: the current job (the inner loops read its fields from shared
// memory, not from the global job list), its index and the next job's first
// tile, so that a tile of the same job costs one shared-memory load and a
// comparison, and no registers are held between uses.
struct JobSlot {
  LiftJob job;
  long long next_begin;
  int ji;
  int pad_;
};

struct JobCursor {
  JobSlot *slot;

  __device__ __forceinline__ void load(LiftParams const &p, int ji,
                                       int lane) {
    constexpr int WORDS = sizeof(LiftJob) / 4;
    static_assert(sizeof(LiftJob) % 4 == 0, "LiftJob is copied in words");
    unsigned const *src = reinterpret_cast<unsigned const *>(
        p.jobs != nullptr ? p.jobs + ji : &p.job);
    __syncwarp();  // every lane is done with the previous job
    for (int i = lane; i < WORDS; i += 32)
      reinterpret_cast<unsigned *>(&slot->job)[i] = src[i];
    if (lane == 0) {
      slot->ji = ji;
      slot->next_begin = p.jobs != nullptr && ji + 1 < p.njobs
                             ? p.jobs[ji + 1].tile_begin
                             : 0x7fffffffffffffffLL;
    }
    __syncwarp();
  }
  __device__ __forceinline__ void init(LiftParams const &p, JobSlot *s,
                                       long long tile, int lane) {
    slot = s;
    load(p, p.jobs != nullptr ? find_job(p, tile) : 0, lane);
  }
  __device__ __forceinline__ LiftJob const &at(LiftParams const &p,
                                               long long tile, int lane) {
    if (tile >= slot->next_begin)
      load(p, advance_job(p, slot->ji, tile, lane), lane);
    return slot->job;
  }
};

// The same interface over the global job list, holding only the job index:
// for kernels whose registers are too tight for the shared-memory slot's
// pointer and generic loads (measured on the strided wide kernel at R = 16:
// 3.26 against 2.96 TB/s with JobCursor; at R = 4 and 8, and on the last
// axis, JobCursor is faster).
struct GlobalCursor {
  int ji;
  __device__ __forceinline__ void init(LiftParams const &p, JobSlot *,
                                       long long tile, int) {
    ji = p.jobs != nullptr ? find_job(p, tile) : 0;
  }
  __device__ __forceinline__ LiftJob const &at(LiftParams const &p,
                                               long long tile, int) {
    if (p.jobs == nullptr) return p.job;
    while (ji + 1 < p.njobs && p.jobs[ji + 1].tile_begin <= tile) ++ji;
    return p.jobs[ji];
  }
};

// Contiguous layout: the thread's elements e = k * R + j (column k, point j)
// in 16-byte pieces; piece i starts at element i * PER, which lies at
// k * n + j from the thread's offset (a piece never crosses a column: R is a
// multiple of PER, or the kCols chunks are whole adjacent pencils, n == R).
template <class A, int R> struct ContigPieces {
  using E = typename A::Elem;
  static constexpr int PER = 16 / sizeof(E);
  static constexpr int LOG2PER = Log2<PER>::value;
  static constexpr int N = A::kCols * R / PER;
  static constexpr int LOG2N = Log2<N>::value;
  static_assert(A::kCols * R % PER == 0, "whole 16-byte pieces");
  static __device__ __forceinline__ long long at(int i, int log2_n) {
    int const e = i * PER;
    return (static_cast<long long>(e / R) << log2_n) + e % R;
  }
  // The pencils of one warp are one contiguous block of 32 * N pieces that
  // the lanes copy in order (coalesced). Piece b of the block belongs to
  // lane `owner` as its piece p.
  static __device__ __forceinline__ void owner_of(int b, int log2_n,
                                                  int &owner, int &p) {
    constexpr int LOG2CW = Log2<A::kCols>::value;
    constexpr int LOG2R = Log2<R>::value;
    // One chunk per pencil (always so when a chunk is shorter than a
    // piece): each lane's N pieces are consecutive.
    if (R < PER || log2_n == LOG2R) {
      owner = b >> LOG2N;
      p = b & (N - 1);
      return;
    }
    if constexpr (R >= PER) {
      int const o = b << LOG2PER;
      int const pk = o >> log2_n;  // pencil in the block
      int const point = o & ((1 << log2_n) - 1);
      int const log2G = log2_n - LOG2R;
      owner = ((pk >> LOG2CW) << log2G) | (point >> LOG2R);
      p = ((pk & (A::kCols - 1)) << (LOG2R - LOG2PER)) |
          ((point & (R - 1)) >> LOG2PER);
    }
  }
  // Slot of lane's piece p among the warp's 32 * N slots: lane-major with a
  // rotation that puts the same piece of 8 consecutive lanes in 8 distinct
  // 16-byte bank groups (conflict-free reads).
  static __device__ __forceinline__ int slot(int lane, int p) {
    constexpr int SH = LOG2N >= 3 ? 0 : 3 - LOG2N;
    return (lane << LOG2N) + ((p + (lane >> SH)) & (N - 1));
  }
};

// Register budgets: 2, 3 and 4 CTAs of 256 threads per SM for R = 16, 8
// and <= 4 (128, 80 and 64 registers); one register above a budget costs a
// whole CTA per SM, measured as 10% of the R = 8 kernel's throughput.
template <class A, int R, int NT, class Sched, bool Contig>
__global__ void __launch_bounds__(NT, R >= 16 ? 2 : R == 8 ? 3 : 4)
    wide_kernel(__grid_constant__ const LiftParams p) {
  using V = typename A::V;
  using W = typename A::Store;
  using E = typename A::Elem;
  using CP = ContigPieces<A, R>;
  constexpr int CW = A::kCols;
  constexpr int LOG2CW = Log2<CW>::value;
  constexpr int LOG2R = Log2<R>::value;
  constexpr int LOG2NT = Log2<NT>::value;
  constexpr int S = WideStages<A>::value;
  static_assert(sizeof(W) == CW * sizeof(E), "row vector size");
  static_assert(R * sizeof(W) % 16 == 0, "slots of whole 16-byte pieces");
  // Per stage R * NT rows of W (strided) or CP::N * NT pieces (contiguous):
  // the same bytes, slot-major so that a warp's slots are consecutive.
  constexpr int SLOT_BYTES = R * sizeof(W);
  extern __shared__ __align__(16) unsigned char smem_raw[];

  int const t = threadIdx.x;
  int const lane = t & 31;
  long long const T = p.total_tiles;
  int const u0 = static_cast<int>(T * blockIdx.x / gridDim.x * kTileRounds);
  int const u1 =
      static_cast<int>(T * (blockIdx.x + 1) / gridDim.x * kTileRounds);
  if (u0 >= u1) return;
  // Job cursors of the copy stream and of the compute stream: both only
  // move forward through the CTA's contiguous range.
  constexpr bool kGlobal = R >= 16 && !Contig;
  using Cursor =
      typename std::conditional<kGlobal, GlobalCursor, JobCursor>::type;
  __shared__ JobSlot wjobs[kGlobal ? 1 : NT / 32][2];
  Cursor jl, jc;
  jl.init(p, &wjobs[kGlobal ? 0 : t >> 5][0], u0 >> 1, lane);
  jc.init(p, &wjobs[kGlobal ? 0 : t >> 5][1], u0 >> 1, lane);
  auto job_of = [&](Cursor &cur, int unit) -> LiftJob const & {
    return cur.at(p, unit >> 1, lane);
  };
  // Unit u uses stage (u - u0) mod S, tracked by counters.
  auto stage_base = [&](int stage) {
    return smem_raw + stage * (SLOT_BYTES * NT);
  };
  auto prefetch = [&](int unit, int stage) {
    LiftJob const &job = job_of(jl, unit);
    WideUnit const w =
        wide_unit<LOG2R, LOG2NT, LOG2CW, Contig>(job, unit, t);
    if (w.active) {
      unsigned char *const st = stage_base(stage);
      if constexpr (Contig) {
        // Lanes copy consecutive pieces of the warp's block; pieces of
        // lanes past the last column group come from the last group.
        int const log2blk = LOG2CW + job.log2_n;  // elements per group
        E const *const wsrc = reinterpret_cast<E const *>(job.base) +
                              (static_cast<long long>(w.wfirst) << log2blk);
        uint4 *const wslots =
            reinterpret_cast<uint4 *>(st) + (t & ~31) * CP::N;
#pragma unroll
        for (int i = 0; i < CP::N; ++i) {
          int const b = i * 32 + lane;
          int owner, pc;
          CP::owner_of(b, job.log2_n, owner, pc);
          long long o = static_cast<long long>(b) << CP::LOG2PER;
          long long const over =
              static_cast<long long>(w.wfirst) + (o >> log2blk) -
              (w.groups - 1);
          if (over > 0) o -= over << log2blk;
          cp_async<16>(wslots + CP::slot(owner, pc), wsrc + o);
        }
      } else if constexpr (R < 16) {
        // Pencils of up to 8 points: row by row (the block copy's extra
        // address work measured slower for these issue-bound units).
        E const *const src = reinterpret_cast<E const *>(job.base) + w.off;
        W *const dst = reinterpret_cast<W *>(st) + t;
        long long const kstride = 1LL << job.log2_kstride;
#pragma unroll
        for (int j = 0; j < R; ++j)
          cp_async<sizeof(W)>(dst + j * NT, src + j * kstride);
      } else {
        // The warp's region of the stage: 32 * R row vectors.
        unsigned char *const wreg = st + (t >> 5) * (32 * SLOT_BYTES);
        int const log2gw = 5 - (job.log2_n - LOG2R);
        if (WideBlock::use(job, w, log2gw, LOG2CW)) {
          constexpr int PL = SLOT_BYTES / 16;  // pieces per lane
          constexpr int LOG2E16 = Log2<16 / sizeof(E)>::value;
          long long const slab0 =
              (static_cast<long long>(w.wfirst) << LOG2CW) >> job.log2_inner;
          E const *const bsrc = reinterpret_cast<E const *>(job.base) +
                                (slab0 << job.log2_astride);
#pragma unroll
          for (int i = 0; i < PL; ++i) {
            int const b = i * 32 + lane;
            cp_async<16>(wreg + (WideBlock::swz(b) << 4),
                         bsrc + (static_cast<long long>(b) << LOG2E16));
          }
        } else {
          E const *const src = reinterpret_cast<E const *>(job.base) + w.off;
          W *const dst = reinterpret_cast<W *>(wreg) + lane;
          long long const kstride = 1LL << job.log2_kstride;
#pragma unroll
          for (int j = 0; j < R; ++j)
            cp_async<sizeof(W)>(dst + j * 32, src + j * kstride);
        }
      }
    }
    cp_async_commit();
  };

#pragma unroll
  for (int k = 0; k < S - 1; ++k)
    if (u0 + k < u1) prefetch(u0 + k, k); else cp_async_commit();
  int cs = 0;          // stage of unit u
  int ps = S - 1;      // stage of unit u + S - 1
  for (int u = u0; u < u1; ++u) {
    // Contiguous layout: lanes copy into each other's slots, so every lane
    // must be done reading the stage that the next prefetch overwrites, and
    // must see the other lanes' copies of unit u.
    if constexpr (Contig) __syncwarp();
    if (u + S - 1 < u1) prefetch(u + S - 1, ps); else cp_async_commit();
    ps = ps + 1 == S ? 0 : ps + 1;
    cp_async_wait_group<S - 1>();  // this thread's copies of unit u are in
    if constexpr (Contig) __syncwarp();
    int const stage = cs;
    cs = cs + 1 == S ? 0 : cs + 1;
    LiftJob const &job = job_of(jc, u);
    WideUnit const w = wide_unit<LOG2R, LOG2NT, LOG2CW, Contig>(job, u, t);
    if (!w.active) continue;  // the whole warp
    unsigned char const *const st = stage_base(stage);
    V v[R];
    if constexpr (Contig) {
      E el[CW * R];
      uint4 const *const wslots =
          reinterpret_cast<uint4 const *>(st) + (t & ~31) * CP::N;
#pragma unroll
      for (int i = 0; i < CP::N; ++i) {
        uint4 const q = wslots[CP::slot(lane, i)];
        memcpy(el + i * CP::PER, &q, 16);
      }
#pragma unroll
      for (int j = 0; j < R; ++j) {
        E row[CW];
#pragma unroll
        for (int k = 0; k < CW; ++k) row[k] = el[k * R + j];
        W x;
        memcpy(&x, row, sizeof(W));
        v[j] = A::load(x);
      }
    } else if constexpr (R < 16) {
#pragma unroll
      for (int j = 0; j < R; ++j)
        v[j] = A::load(reinterpret_cast<W const *>(st)[j * NT + t]);
    } else {
      unsigned char const *const wreg = st + (t >> 5) * (32 * SLOT_BYTES);
      int const log2gw = 5 - (job.log2_n - LOG2R);
      if (WideBlock::use(job, w, log2gw, LOG2CW)) {
        // Element offset of the thread's chunk of its column group in the
        // block: slab gl * kCols / inner, column gl * kCols mod inner.
        int const gl = lane & ((1 << log2gw) - 1);
        int const log2B = job.log2_inner;
        int const e0 = (((gl << LOG2CW) >> log2B) << (job.log2_n + log2B)) +
                       ((w.c << LOG2R) << log2B) +
                       ((gl << LOG2CW) & ((1 << log2B) - 1));
#pragma unroll
        for (int j = 0; j < R; ++j) {
          int const byte = (e0 + (j << log2B)) * static_cast<int>(sizeof(E));
          W x;
          memcpy(&x, wreg + (WideBlock::swz(byte >> 4) << 4) + (byte & 15),
                 sizeof(W));
          v[j] = A::load(x);
        }
      } else {
#pragma unroll
        for (int j = 0; j < R; ++j)
          v[j] = A::load(reinterpret_cast<W const *>(wreg)[j * 32 + lane]);
      }
    }
    int const log2G = job.log2_n - LOG2R;
    RoundCtx<A, NT> ctx(t, w.c, 1 << log2G, log2G, lane, 1, nullptr, nullptr,
                        w.log2ls);
    Sched::template run_levels<A, R, NT>(v, ctx, job.nlevels);
    if (w.keep) {
      E *const dst = reinterpret_cast<E *>(job.dst_base) + w.off;
      if constexpr (Contig) {
        E el[CW * R];
#pragma unroll
        for (int j = 0; j < R; ++j) {
          W const x = A::store(v[j]);
          E row[CW];
          memcpy(row, &x, sizeof(W));
#pragma unroll
          for (int k = 0; k < CW; ++k) el[k * R + j] = row[k];
        }
#pragma unroll
        for (int i = 0; i < CP::N; ++i) {
          uint4 q;
          memcpy(&q, el + i * CP::PER, 16);
          *reinterpret_cast<uint4 *>(dst + CP::at(i, job.log2_n)) = q;
        }
      } else {
        long long const kstride = 1LL << job.log2_kstride;
#pragma unroll
        for (int j = 0; j < R; ++j)
          *reinterpret_cast<W *>(dst + j * kstride) = A::store(v[j]);
      }
    }
  }
  cp_async_wait_all();
}

template <class A, int R, int NT> constexpr size_t wide_smem_bytes() {
  return size_t(WideStages<A>::value) * R * NT * sizeof(typename A::Store);
}

// Tile kernel: periodic pencils of 128 to 4096 points along a strided axis.
// A tile is NT / G column groups of kCols columns (G = n / R chunks per
// pencil) times the n pencil rows; it is copied between HBM and shared
// memory in row order with 16- or 8-byte cp.async and stores (lanes along
// the row, coalesced), in a row-major layout where each chunk's R rows are
// followed by PAD bytes. Each thread then holds the same chunk of kCols
// adjacent pencils as rows of A::V in registers, as in the wide kernel, and
// writes its rows back before the tile is stored.
//
// Lanes: for G <= 32 the G chunks of a column group are lanes 32 / G apart
// (a warp holds 32 / G column groups) and exchange by shuffle; for G > 32 a
// warp holds 32 consecutive chunks of one column group and the exchanges go
// through shared memory (one barrier per level pass). PAD is one warp-row
// segment (the bytes of the column groups a warp holds, at least one row
// vector): it steps the chunk blocks' bank offsets so that the rows a warp
// reads at once fall on distinct banks. Pieces are 8 bytes when PAD is not
// a multiple of 16 (8-byte row vectors with 32 or more chunks).
//
// Two forms (Long): pencils of up to 32 chunks (shuffles only) and longer
// ones (G > 32). The short form gives each CTA a contiguous range of tiles
// and keeps three tile buffers in flight for 8-byte row vectors (two for
// 16-byte ones); measured on the 4D CT batch this is faster for short
// pencils. The long form double buffers and has the CTAs take every
// gridDim.x-th tile, so that the CTAs running at one time work on
// neighbouring tiles: its tile rows are 8 to 64 bytes, and neighbouring
// tiles share DRAM sectors and pages (FP32, 4096-point pencils: 1.6 against
// 1.1 TB/s with contiguous ranges).
template <class A, bool Long> struct TileStages {
  static constexpr int value =
      Long || sizeof(typename A::Store) == 16 ? 2 : 3;
};
// Bytes of one tile buffer: n * row bytes = R * NT row vectors, plus the
// padding of G chunks (at most max(32, G) row vectors).
template <class A, int R, int NT, bool Long> struct TileStageBytes {
  static constexpr int value = (R * NT + (Long ? 256 : 32)) *
                               static_cast<int>(sizeof(typename A::Store));
};
// Chunk heads and the two exchange buffers of RoundCtx (G > 32).
template <class A, int NT, bool Long> struct TileXchBytes {
  static constexpr int value =
      Long ? 3 * NT * static_cast<int>(sizeof(typename A::V)) : 0;
};
template <class A, int R, int NT, bool Long>
constexpr size_t tile_smem_bytes() {
  return size_t(TileStages<A, Long>::value) *
             TileStageBytes<A, R, NT, Long>::value +
         TileXchBytes<A, NT, Long>::value;
}

// Geometry of one tile of a job.
struct TileGeo {
  long long gc0;     // first column of the tile
  long long columns;
  int log2G;         // chunks per pencil
  int log2rb;        // bytes per tile row
  int log2pb;        // bytes per copied piece (3 or 4)
  int pad;           // bytes after each chunk's rows
  int cpitch;        // bytes per chunk block: R rows + pad
};

template <class A, int LOG2R, int LOG2NT>
__device__ __forceinline__ TileGeo tile_geo(LiftJob const &job,
                                            long long tile) {
  constexpr int LOG2CW = Log2<A::kCols>::value;
  constexpr int LOG2W = Log2<sizeof(typename A::Store)>::value;
  TileGeo g;
  g.log2G = job.log2_n - LOG2R;
  int const log2tcg = LOG2NT - g.log2G;  // column groups per tile
  g.gc0 = (tile - job.tile_begin) << (log2tcg + LOG2CW);
  g.columns = job.columns;
  g.log2rb = log2tcg + LOG2W;
  int const log2seg = g.log2G >= 5 ? LOG2W : 5 - g.log2G + LOG2W;
  g.pad = (1 << log2seg) & 127;  // one warp-row segment
  g.cpitch = (1 << (LOG2R + g.log2rb)) + g.pad;
  g.log2pb = (g.pad & 15) != 0 || g.log2rb < 4 ? 3 : 4;
  return g;
}

template <class A, int R, int NT, class Sched, bool Long>
__global__ void __launch_bounds__(NT, 2)
    tile_kernel(__grid_constant__ const LiftParams p) {
  using V = typename A::V;
  using W = typename A::Store;
  using E = typename A::Elem;
  constexpr int CW = A::kCols;
  constexpr int LOG2R = Log2<R>::value;
  constexpr int LOG2NT = Log2<NT>::value;
  constexpr int S = TileStages<A, Long>::value;
  constexpr int LOG2ES = Log2<sizeof(E)>::value;
  constexpr int STAGE = TileStageBytes<A, R, NT, Long>::value;
  static_assert(sizeof(W) == CW * sizeof(E), "row vector size");
  static_assert(sizeof(W) >= 8, "pieces of at least 8 bytes");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *const heads =
      Long ? reinterpret_cast<V *>(smem_raw + S * STAGE) : nullptr;
  V *const xch = Long ? heads + NT : nullptr;

  int const t = threadIdx.x;
  int const lane = t & 31;
  long long const T = p.total_tiles;
  // Tiles of this CTA: u0, u0 + step, ... below u1.
  long long const step = Long ? gridDim.x : 1;
  long long const u0 = Long ? blockIdx.x : T * blockIdx.x / gridDim.x;
  long long const u1 = Long ? T : T * (blockIdx.x + 1) / gridDim.x;
  if (u0 >= u1) return;
  // Job cursors of the copy stream and of the compute stream (tiles only
  // increase along each).
  __shared__ JobSlot wjobs[NT / 32][2];
  JobCursor jl, jc;
  jl.init(p, &wjobs[t >> 5][0], u0, lane);
  jc.init(p, &wjobs[t >> 5][1], u0, lane);
  auto job_of = [&](JobCursor &cur, long long tile) -> LiftJob const & {
    return cur.at(p, tile, lane);
  };
  // Element offset of tile column `tc` (a multiple of the piece's columns)
  // in row k; pieces past the job's last column read its last piece.
  auto elem = [](LiftJob const &job, TileGeo const &g, long long tc, int k) {
    long long const last = g.columns - (1 << (g.log2pb - LOG2ES));
    long long gc = g.gc0 + tc;
    if (gc > last) gc = last;
    int const log2B = job.log2_inner;
    return ((gc >> log2B) << job.log2_astride) +
           (gc & ((1LL << log2B) - 1)) +
           (static_cast<long long>(k) << job.log2_kstride);
  };
  auto smem_off = [](TileGeo const &g, int k, int q) {
    return (k >> LOG2R) * g.cpitch + ((k & (R - 1)) << g.log2rb) +
           (q << g.log2pb);
  };
  auto prefetch = [&](long long tile, int buf) {
    LiftJob const &job = job_of(jl, tile);
    TileGeo const g = tile_geo<A, LOG2R, LOG2NT>(job, tile);
    unsigned char *const st = smem_raw + buf * STAGE;
    E const *const src = reinterpret_cast<E const *>(job.base);
    int const log2q = g.log2rb - g.log2pb;  // pieces per row
    int const cols_q = g.log2pb - LOG2ES;   // log2 columns per piece
    // Piece i = t + j NT is row k = i >> log2q, piece q = i mod 2^log2q of
    // the row; a row has at most NT pieces, so q is the same for all of a
    // thread's pieces and k advances by NT >> log2q.
    int const q = t & ((1 << log2q) - 1);
    int const dk = NT >> log2q;
    E const *const from0 =
        src + elem(job, g, static_cast<long long>(q) << cols_q, 0);
    int const n = 1 << job.log2_n;
    for (int k = t >> log2q; k < n; k += dk) {
      E const *const from = from0 + (static_cast<long long>(k)
                                     << job.log2_kstride);
      if (g.log2pb == 4)
        cp_async<16>(st + smem_off(g, k, q), from);
      else
        cp_async<8>(st + smem_off(g, k, q), from);
    }
    cp_async_commit();
  };

  // The CTA's k-th tile (u0 + k * step) uses buffer k % S.
#pragma unroll
  for (int k = 0; k < S - 1; ++k)
    if (u0 + k * step < u1) prefetch(u0 + k * step, k); else cp_async_commit();
  int slot = 0;  // buffer of tile u
  for (long long u = u0; u < u1;
       u += step, slot = slot + 1 == S ? 0 : slot + 1) {
    __syncthreads();  // the buffer the next prefetch fills is free
    long long const ahead = u + (S - 1) * step;
    int const ahead_slot = (slot + S - 1) % S;
    if (ahead < u1) prefetch(ahead, ahead_slot); else cp_async_commit();
    cp_async_wait_group<S - 1>();
    __syncthreads();  // every thread's copies of tile u are visible
    LiftJob const &job = job_of(jc, u);
    TileGeo const g = tile_geo<A, LOG2R, LOG2NT>(job, u);
    unsigned char *const st = smem_raw + slot * STAGE;
    int c, grp, log2ls;
    if (!Long || g.log2G <= 5) {  // chunks of a column group 32 / G lanes apart
      log2ls = 5 - g.log2G;
      c = lane >> log2ls;
      grp = ((t >> 5) << log2ls) | (lane & ((1 << log2ls) - 1));
    } else {             // 32 consecutive chunks per warp
      log2ls = 0;
      c = t & ((1 << g.log2G) - 1);
      grp = t >> g.log2G;
    }
    unsigned char *const mine =
        st + c * g.cpitch + grp * static_cast<int>(sizeof(W));
    V v[R];
#pragma unroll
    for (int j = 0; j < R; ++j)
      v[j] = A::load(*reinterpret_cast<W const *>(mine + (j << g.log2rb)));
    RoundCtx<A, NT> ctx(t, c, 1 << g.log2G, g.log2G, lane, 1, heads, xch,
                        log2ls);
    Sched::template run_levels<A, R, NT>(v, ctx, job.nlevels);
#pragma unroll
    for (int j = 0; j < R; ++j)
      *reinterpret_cast<W *>(mine + (j << g.log2rb)) = A::store(v[j]);
    __syncthreads();  // the transformed tile is in shared memory
    E *const dst = reinterpret_cast<E *>(job.dst_base);
    int const log2q = g.log2rb - g.log2pb;
    int const cols_q = g.log2pb - LOG2ES;
    int const q = t & ((1 << log2q) - 1);  // as in the copy in
    long long const tc = static_cast<long long>(q) << cols_q;
    if (g.gc0 + tc < g.columns) {
      int const dk = NT >> log2q;
      E *const to0 = dst + elem(job, g, tc, 0);
      int const n = 1 << job.log2_n;
      for (int k = t >> log2q; k < n; k += dk) {
        unsigned char const *const from = st + smem_off(g, k, q);
        E *const to = to0 + (static_cast<long long>(k) << job.log2_kstride);
        if (g.log2pb == 4)
          *reinterpret_cast<uint4 *>(to) =
              *reinterpret_cast<uint4 const *>(from);
        else
          *reinterpret_cast<uint2 *>(to) =
              *reinterpret_cast<uint2 const *>(from);
      }
    }
  }
  cp_async_wait_all();
}

// Halo kernel: runs before a windowed stage and copies, from the grid
// (`base`) to the halo buffer (`dst_base`, same offsets), the points within
// `halo` of every segment boundary b * seg_len, b = 0 .. ceil(n / seg_len)
// - 1 (positions [b seg_len - halo, b seg_len + halo) modulo n): every point
// a window reads outside its own segment, taken before the windows overwrite
// their segments in place. Boundaries closer than 2 halo (a short last
// segment) copy some points twice, with the same values. A tile is 32
// consecutive positions around one boundary (halo is a multiple of 16) of
// 2^log2_window columns; its points are visited with the grid's contiguous
// direction fastest: along the pencil for the last axis, along the columns
// otherwise.
template <typename S, int NT>
__global__ void __launch_bounds__(NT)
    halo_kernel(__grid_constant__ const LiftParams p) {
  constexpr int UNROLL = 4;
  int const t = threadIdx.x;
  int const lane = t & 31;
  __shared__ JobSlot wjobs[NT / 32];
  JobCursor cur;
  long long const first = blockIdx.x;
  if (first >= p.total_tiles) return;
  cur.init(p, &wjobs[t >> 5], first, lane);
  for (long long tile = first; tile < p.total_tiles; tile += gridDim.x) {
    LiftJob const &job = cur.at(p, tile, lane);
    long long const local = tile - job.tile_begin;
    long long const rest = local / job.col_tiles;
    int const log2C = job.log2_window;
    long long const gc0 = (local - rest * job.col_tiles) << log2C;
    int const blocks = job.halo >> 4;  // 32-position blocks per boundary
    long long const bnd = rest / blocks;
    int const pb = static_cast<int>(rest - bnd * blocks);
    int const total = 32 << log2C;
    long long const n = 1LL << job.log2_n;
    long long const p0 = bnd * job.seg_len - job.halo + 32 * pb;
    bool const along = job.log2_kstride == 0;
    long long const imask = (1LL << job.log2_inner) - 1;
    S const *const src = reinterpret_cast<S const *>(job.base);
    S *const dst = reinterpret_cast<S *>(job.dst_base);
    for (int i0 = t; i0 < total; i0 += UNROLL * NT) {
      long long off[UNROLL];
      bool ok[UNROLL];
      S v[UNROLL];
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        int const i = i0 + u * NT;
        int w, j;
        if (along) {
          w = i >> 5;
          j = i & 31;
        } else {
          w = i & ((1 << log2C) - 1);
          j = i >> log2C;
        }
        long long pp = p0 + j;
        if (pp < 0) pp += n;
        if (pp >= n) pp -= n;
        long long const gc = gc0 + w;
        ok[u] = i < total && gc < job.columns;
        off[u] = ((gc >> job.log2_inner) << job.log2_astride) + (gc & imask) +
                 (pp << job.log2_kstride);
        if (ok[u]) v[u] = src[off[u]];
      }
#pragma unroll
      for (int u = 0; u < UNROLL; ++u)
        if (ok[u]) dst[off[u]] = v[u];
    }
  }
}

// Dynamic shared memory of one CTA (an upper bound over every column shape:
// cols * pitch <= rounds * NT * (R + 1) + cols and cols <= rounds * NT).
template <class A, int R, int NT>
constexpr size_t lift_smem_bytes(int rounds) {
  using V = typename A::V;
  using S = typename A::Store;
  return 3 * NT * sizeof(V) + size_t(rounds) * NT * (R + 2) * sizeof(S);
}

} // namespace pgb
