// Combination-technique kernels: FP64 combine of component-grid surpluses
// into sparse-grid subspaces, restriction of the combined subspaces back to
// the component grids, and scatter of the subspaces into a full grid.
//
// Restates the reference's test driver
// (test/test_paliwa_combination_technique.cpp): combine :256-290
// (subspace += coefficient * grid, FP64, grids in order), scatter :293-318
// (full grid += subspace). The subspace of level vector s is
// strided_hierarchical_domain_from_level(s, lmax) (paliwa_domains.hpp:51-83):
// per dimension 2^(s-1) points at uids 2^(L-s) + j * 2^(L-s+1), or the single
// point 0 at s = 0. Inside a grid at level l the same point has the compact
// index (2 j + 1) * 2^(l - s) (0 at s = 0).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pgb {

constexpr int kMaxDims = 12;

struct CtSubspace {
  long long offset;      // first sparse point of this subspace
  int grid_begin;        // range in the containing-grid list
  int grid_end;
  signed char level[kMaxDims];
};

struct CtGrid {
  unsigned long long base;  // byte address of the grid
  double coefficient;
  signed char level[kMaxDims];
};

struct CtParams {
  CtSubspace const *subspaces;
  int nsubspaces;
  int const *grid_lists;  // containing grids of each subspace, in grid order
  CtGrid const *grids;
  int ndim;
  long long npoints;       // sparse points in total
  double *sparse;          // combined values (FP64)
  double *full;            // full grid at the maximum level (scatter)
  signed char max_level[kMaxDims];
  // Every coefficient times every grid value is exact in FP64 (coefficients
  // of at most 29 significant bits and moderate magnitude on FP32 grids,
  // +-1 on FP64 grids): the combine then fuses multiply and add.
  int exact_products;
  // Subspaces contained in more than kCtHeavy grids are restricted one warp
  // per point (ct_heavy_restrict_kernel): heavy[i] is the subspace index,
  // heavy_first[i] the first of its points in the heavy numbering (prefix
  // sums of the sizes).
  int const *heavy;
  long long const *heavy_first;
  int nheavy;
  long long nheavy_points;
  // block_sub[b]: the subspace holding point kCtBlock * b (the first point
  // of CTA b), planned on the host.
  int const *block_sub;
};

// Points (threads) per CTA of ct_kernel.
constexpr int kCtBlock = 256;

// Grid count above which restrict writes a subspace's points one warp per
// point (lanes over grids) instead of one thread per point: a thread would
// walk thousands of grids (the coarsest subspaces are in every grid) while
// the rest of the launch has finished. Measured on GB300 (FP32 grids):
// 6D scheme |l|_1 = 16 - q, restrict 5.3 -> 2.8 ms; 4D |l|_1 = 20 - q
// unchanged (8.1 -> 8.3 ms). Combine keeps one thread per point for every
// subspace: the warp form made the 4D combine slower (9.0 -> 11.3 ms).
constexpr int kCtHeavy = 1024;

// float -> double without the conversion instruction, which on GB300 runs
// on the FP64 pipe: for normal numbers the double is the float's sign,
// exponent rebiased by 1023 - 127 and fraction shifted by 29 bits (the
// exact value); zeros, subnormals, infinities and NaNs take the conversion.
__device__ __forceinline__ double widen(float x) {
  unsigned const u = __float_as_uint(x);
  unsigned const e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return static_cast<double>(x);
  unsigned long long const bits =
      (static_cast<unsigned long long>(u >> 31) << 63) |
      (static_cast<unsigned long long>(e + (1023 - 127)) << 52) |
      (static_cast<unsigned long long>(u & 0x7fffffu) << 29);
  return __longlong_as_double(static_cast<long long>(bits));
}
__device__ __forceinline__ double widen(double x) { return x; }

// Multi-index of point `p` of subspace `sub` -> compact index inside a grid
// at level `lv` (element offset, row-major, last dimension fastest).
__device__ __forceinline__ long long ct_offset(long long p,
                                              signed char const *s,
                                              signed char const *lv,
                                              int ndim) {
  long long off = 0;
  int shift = 0;  // log2 of the element stride of the current dimension
  for (int d = ndim - 1; d >= 0; --d) {
    int const sd = s[d];
    int const ld = lv[d];
    int const ext_log2 = sd == 0 ? 0 : sd - 1;  // 2^(s-1) points, 1 at s=0
    long long const j = p & ((1LL << ext_log2) - 1);
    p >>= ext_log2;
    long long const k = sd == 0 ? 0 : ((2 * j + 1) << (ld - sd));
    off += k << shift;
    shift += ld;
  }
  return off;
}

// Combined value of one sparse point: sum over the containing grids, in
// grid order, of coefficient * value. One grid per iteration: loading
// several grids ahead (8 per batch: 64 registers) measured slower on the 4D
// scheme (10.6 against 9.0 ms), as the loop is limited by the scattered
// loads, not by their latency.
template <typename S, bool Fused>
__device__ __forceinline__ double ct_combine_point(CtParams const &p,
                                                   CtSubspace const &ss,
                                                   long long local) {
  double acc = 0.0;
  for (int gi = ss.grid_begin; gi < ss.grid_end; ++gi) {
    CtGrid const &g = p.grids[p.grid_lists[gi]];
    long long const off = ct_offset(local, ss.level, g.level, p.ndim);
    double const v = widen(reinterpret_cast<S const *>(g.base)[off]);
    if constexpr (Fused)
      acc = __fma_rn(g.coefficient, v, acc);
    else
      acc = __dadd_rn(acc, __dmul_rn(g.coefficient, v));
  }
  return acc;
}

// Which of the three operations a launch performs.
enum CtOp { kCombine = 0, kRestrict = 1, kScatter = 2 };

template <typename S, int OP>
__global__ void __launch_bounds__(kCtBlock) ct_kernel(CtParams const p) {
  long long const first = static_cast<long long>(blockIdx.x) * kCtBlock;
  long long const point = first + threadIdx.x;
  if (point >= p.npoints) return;
  // The CTA's first subspace comes from the host's table (a search of the
  // whole list per CTA, behind a barrier, measured as the combine's second
  // stall reason).
  int const sub0 = p.block_sub[blockIdx.x];
  // Most CTAs lie inside one subspace: one load settles that. Otherwise
  // the CTA's 256 points span at most 256 subspaces (each has at least one
  // point): a binary search over those, instead of a walk that is as long
  // as the number of small subspaces before the point.
  int sub = sub0;
  if (sub0 + 1 < p.nsubspaces && p.subspaces[sub0 + 1].offset <= point) {
    int lo = sub0 + 1;
    int hi = min(sub0 + kCtBlock - 1, p.nsubspaces - 1);
    while (lo < hi) {
      int const mid = (lo + hi + 1) >> 1;
      if (p.subspaces[mid].offset <= point)
        lo = mid;
      else
        hi = mid - 1;
    }
    sub = lo;
  }
  CtSubspace const &ss = p.subspaces[sub];
  long long const local = point - ss.offset;
  if (OP == kRestrict && ss.grid_end - ss.grid_begin > kCtHeavy) return;
  if constexpr (OP == kScatter) {
    long long const off = ct_offset(local, ss.level, p.max_level, p.ndim);
    p.full[off] = __dadd_rn(p.full[off], p.sparse[point]);
    return;
  } else if constexpr (OP == kCombine) {
    // acc = acc + c * v in grid order, rounded like the reference driver.
    // With exact products fma(c, v, acc) rounds identically and issues one
    // FP64 instruction instead of two; the choice is made once per thread,
    // outside the loop, so that no thread evaluates both forms.
    p.sparse[point] = p.exact_products != 0
                          ? ct_combine_point<S, true>(p, ss, local)
                          : ct_combine_point<S, false>(p, ss, local);
  } else {
    S const v = static_cast<S>(p.sparse[point]);
    for (int gi = ss.grid_begin; gi < ss.grid_end; ++gi) {
      CtGrid const &g = p.grids[p.grid_lists[gi]];
      long long const off = ct_offset(local, ss.level, g.level, p.ndim);
      reinterpret_cast<S *>(g.base)[off] = v;
    }
  }
}

// Restrict of the points of heavy subspaces, one warp per point: the lanes
// write the point's value into 32 of its grids at a time.
template <typename S>
__global__ void __launch_bounds__(256) ct_heavy_restrict_kernel(
    CtParams const p) {
  long long const w =
      (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  int const lane = threadIdx.x & 31;
  if (w >= p.nheavy_points) return;
  int lo = 0, hi = p.nheavy - 1;
  while (lo < hi) {
    int const mid = (lo + hi + 1) >> 1;
    if (p.heavy_first[mid] <= w)
      lo = mid;
    else
      hi = mid - 1;
  }
  CtSubspace const &ss = p.subspaces[p.heavy[lo]];
  long long const local = w - p.heavy_first[lo];
  S const v = static_cast<S>(p.sparse[ss.offset + local]);
  for (int gi = ss.grid_begin + lane; gi < ss.grid_end; gi += 32) {
    CtGrid const &g = p.grids[p.grid_lists[gi]];
    long long const off = ct_offset(local, ss.level, g.level, p.ndim);
    reinterpret_cast<S *>(g.base)[off] = v;
  }
}

} // namespace pgb
