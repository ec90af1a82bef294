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
// itself a short periodic pencil.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "arith.cuh"

namespace pgb {

constexpr int kMaxPasses = 8;
constexpr int kMaxLevels = 48;

// One unit of work for a launch: one grid (or one sub-lattice of a grid)
// along one axis.
struct LiftJob {
  long long offset;      // element offset of the grid in the data buffer
  long long columns;     // outer * inner
  long long tile_begin;  // index of the first CTA of this job in the launch
  long long col_tiles;   // CTAs per window row (ceil(columns / C))
  int log2_inner;        // inner extent: splits a column index into (a, b)
  int log2_kstride;      // element stride between consecutive pencil points
  int log2_astride;      // element stride between consecutive outer indices
  int log2_n;            // pencil length of the whole (sub-lattice) axis
  // Window mode (periodic == 0): the window covers points
  // [seg * seg_len - halo, seg * seg_len + seg_len + halo) of the pencil.
  int seg_len;
  int halo;
  int nlevels;
  signed char shift[kMaxLevels];  // log2 of each level's distance, in order
};

struct LiftParams {
  void *data;
  LiftJob const *jobs;  // device array, or nullptr to use `job`
  int njobs;
  int log2_window;      // log2 of the points per pencil held by one CTA
  int periodic;         // 1: whole periodic pencils; 0: windows
  int vec_ok;           // 16-byte aligned contiguous chunks may be vectorized
  int npasses;
  int fp64_log2_points; // steps updating <= 2^this points per pencil in FP64
  unsigned c1_one_mask;
  int offsets[kMaxPasses];
  Coeffs coeffs[kMaxPasses];
  LiftJob job;
};

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
template <class A, int R, int S, bool C1, bool F64, typename V>
__device__ __forceinline__ void fine_step(V (&v)[R], int o, V nb,
                                          Coeffs const &cf) {
  if (o == 1) {
#pragma unroll
    for (int j = S; j < R; j += 2 * S) {
      V up = (j + S < R) ? v[(j + S) % R] : nb;
      v[j] = A::template update<C1, F64>(cf, v[j - S], v[j], up);
    }
  } else {
#pragma unroll
    for (int j = 0; j < R; j += 2 * S) {
      V lo = (j >= S) ? v[(j + R - S) % R] : nb;
      v[j] = A::template update<C1, F64>(cf, lo, v[j], v[j + S]);
    }
  }
}

// Selects the compile-time distance 2^K == 2^sh (sh < log2 R).
template <class A, int R, bool C1, bool F64, int K = 0, typename V>
__device__ __forceinline__ void fine_distance(V (&v)[R], int sh, int o, V nb,
                                              Coeffs const &cf) {
  if constexpr ((1 << K) < R) {
    if (sh == K) {
      fine_step<A, R, (1 << K), C1, F64>(v, o, nb, cf);
      return;
    }
    fine_distance<A, R, C1, F64, K + 1>(v, sh, o, nb, cf);
  }
}

template <class A, int R, typename V>
__device__ __forceinline__ void fine_dispatch(V (&v)[R], int sh, int o, V nb,
                                              Coeffs const &cf, bool c1one,
                                              bool f64) {
  if (A::kHasFp64Mode && f64) {
    if (c1one)
      fine_distance<A, R, true, A::kHasFp64Mode>(v, sh, o, nb, cf);
    else
      fine_distance<A, R, false, A::kHasFp64Mode>(v, sh, o, nb, cf);
  } else {
    if (c1one)
      fine_distance<A, R, true, false>(v, sh, o, nb, cf);
    else
      fine_distance<A, R, false, false>(v, sh, o, nb, cf);
  }
}

template <class A, typename V>
__device__ __forceinline__ V coarse_update(Coeffs const &cf, bool c1one,
                                           bool f64, V lo, V me, V up) {
  if (A::kHasFp64Mode && f64) {
    if (c1one) return A::template update<true, A::kHasFp64Mode>(cf, lo, me, up);
    return A::template update<false, A::kHasFp64Mode>(cf, lo, me, up);
  }
  if (c1one) return A::template update<true, false>(cf, lo, me, up);
  return A::template update<false, false>(cf, lo, me, up);
}

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

template <class A, int R, int NT>
__global__ void __launch_bounds__(NT)
    lift_kernel(__grid_constant__ const LiftParams p) {
  using V = typename A::V;
  using S = typename A::Store;
  constexpr int LOG2R = Log2<R>::value;
  constexpr int LOG2NT = Log2<NT>::value;
  __shared__ V heads[NT];
  __shared__ V xch[2][NT];

  long long const tile = blockIdx.x;
  LiftJob const *job = &p.job;
  if (p.jobs != nullptr) {
    int lo = 0, hi = p.njobs - 1;
    while (lo < hi) {
      int const mid = (lo + hi + 1) >> 1;
      if (p.jobs[mid].tile_begin <= tile)
        lo = mid;
      else
        hi = mid - 1;
    }
    job = p.jobs + lo;
  }
  int const log2G = p.log2_window - LOG2R;
  int const G = 1 << log2G;
  int const log2C = LOG2NT - log2G;
  int const t = threadIdx.x;
  int const col = t & ((1 << log2C) - 1);
  int const c = t >> log2C;

  long long const local = tile - job->tile_begin;
  long long const seg = local / job->col_tiles;
  long long const gc = (local - seg * job->col_tiles) * (1LL << log2C) + col;
  bool const active = gc < job->columns;
  int const log2B = job->log2_inner;
  long long const a = gc >> log2B;
  long long const b = gc & ((1LL << log2B) - 1);
  long long const n = 1LL << job->log2_n;
  long long const kstride = 1LL << job->log2_kstride;

  // Position of this thread's chunk along the pencil.
  long long pos = (long long)c * R;
  bool store_me = active;
  if (!p.periodic) {
    long long const start = seg * job->seg_len - job->halo;
    bool const in_segment =
        pos >= job->halo && pos < job->halo + job->seg_len &&
        seg * job->seg_len + (pos - job->halo) < n;
    store_me = active && in_segment;
    pos = (start + pos) % n;
    if (pos < 0) pos += n;
  }
  S *g = static_cast<S *>(p.data) + job->offset + (a << job->log2_astride) +
         b + pos * kstride;
  bool const vec = p.vec_ok && job->log2_kstride == 0;

  V v[R];
  {
    S raw[R];
    if (active) {
      load_chunk<S, R>(g, kstride, vec, raw);
    } else {
#pragma unroll
      for (int j = 0; j < R; ++j) raw[j] = S(0);
    }
#pragma unroll
    for (int j = 0; j < R; ++j) v[j] = A::load(raw[j]);
  }

  bool heads_valid = false;
  int buf = 0;
  int const nlev = job->nlevels;
  for (int li = 0; li < nlev; ++li) {
    int const sh = job->shift[li];
    // Points updated per pencil by one pass of this level: n / (2 s).
    bool const f64 = (job->log2_n - sh - 1) <= p.fp64_log2_points;
    for (int ps = 0; ps < p.npasses; ++ps) {
      int const o = p.offsets[ps];
      Coeffs const cf = p.coeffs[ps];
      bool const c1one = (p.c1_one_mask >> ps) & 1u;
      if (sh < LOG2R) {
        V nb;
        if (G > 1) {
          xch[buf][t] = (o == 1) ? v[0] : tail_value<R>(v, sh);
          __syncthreads();
          int nc = (o == 1) ? c + 1 : c - 1;
          if (p.periodic)
            nc &= G - 1;
          else
            nc = nc < 0 ? 0 : (nc >= G ? G - 1 : nc);
          nb = xch[buf][(nc << log2C) | col];
          buf ^= 1;
        } else {
          nb = (o == 1) ? v[0] : tail_value<R>(v, sh);
        }
        fine_dispatch<A, R>(v, sh, o, nb, cf, c1one, f64);
        if (o == 0) heads_valid = false;
      } else {
        if (!heads_valid) {
          heads[t] = v[0];
          __syncthreads();
          heads_valid = true;
        }
        int const d = 1 << (sh - LOG2R);
        if ((c & (2 * d - 1)) == o * d) {
          int cl = c - d, cu = c + d;
          if (p.periodic) {
            cl &= G - 1;
            cu &= G - 1;
          } else {
            cl = cl < 0 ? c : cl;
            cu = cu >= G ? c : cu;
          }
          V const lo = heads[(cl << log2C) | col];
          V const up = heads[(cu << log2C) | col];
          v[0] = coarse_update<A>(cf, c1one, f64, lo, v[0], up);
          heads[t] = v[0];
        }
        __syncthreads();
      }
    }
  }

  if (store_me) {
    S raw[R];
#pragma unroll
    for (int j = 0; j < R; ++j) raw[j] = A::store(v[j]);
    store_chunk<S, R>(g, kstride, vec, raw);
  }
}

} // namespace pgb
