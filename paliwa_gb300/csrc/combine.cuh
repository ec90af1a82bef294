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
};

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

__device__ __forceinline__ int ct_find_subspace(CtParams const &p,
                                                long long point) {
  int lo = 0, hi = p.nsubspaces - 1;
  while (lo < hi) {
    int const mid = (lo + hi + 1) >> 1;
    if (p.subspaces[mid].offset <= point)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Which of the three operations a launch performs.
enum CtOp { kCombine = 0, kRestrict = 1, kScatter = 2 };

template <typename S, int OP>
__global__ void __launch_bounds__(256) ct_kernel(CtParams const p) {
  long long const first = static_cast<long long>(blockIdx.x) * blockDim.x;
  if (first >= p.npoints) return;
  // One search per CTA; threads walk forward from the CTA's first subspace.
  __shared__ int sub0;
  if (threadIdx.x == 0) sub0 = ct_find_subspace(p, first);
  __syncthreads();
  long long const point = first + threadIdx.x;
  if (point >= p.npoints) return;
  int sub = sub0;
  while (sub + 1 < p.nsubspaces && p.subspaces[sub + 1].offset <= point) ++sub;
  CtSubspace const &ss = p.subspaces[sub];
  long long const local = point - ss.offset;
  if constexpr (OP == kScatter) {
    long long const off = ct_offset(local, ss.level, p.max_level, p.ndim);
    p.full[off] = __dadd_rn(p.full[off], p.sparse[point]);
    return;
  } else if constexpr (OP == kCombine) {
    double acc = 0.0;
    for (int gi = ss.grid_begin; gi < ss.grid_end; ++gi) {
      CtGrid const &g = p.grids[p.grid_lists[gi]];
      long long const off = ct_offset(local, ss.level, g.level, p.ndim);
      double const v = static_cast<double>(
          reinterpret_cast<S const *>(g.base)[off]);
      acc = __dadd_rn(acc, __dmul_rn(g.coefficient, v));
    }
    p.sparse[point] = acc;
  } else {
    double const v = p.sparse[point];
    for (int gi = ss.grid_begin; gi < ss.grid_end; ++gi) {
      CtGrid const &g = p.grids[p.grid_lists[gi]];
      long long const off = ct_offset(local, ss.level, g.level, p.ndim);
      reinterpret_cast<S *>(g.base)[off] = static_cast<S>(v);
    }
  }
}

} // namespace pgb
