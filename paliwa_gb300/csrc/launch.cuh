// Kernel instantiation and launch helpers shared by the per-dtype
// translation units (lift_f64.cu, lift_f32.cu, lift_f32c.cu), which are
// compiled in parallel.
#pragma once

#include <algorithm>
#include <string>

#include "lift.cuh"
#include "plan.hpp"

namespace pgb {

int device_sms();
int current_device();

// Occupancy of one kernel instantiation, per device: the dynamic shared
// memory opt-in (cudaFuncSetAttribute) and the occupancy query apply to the
// device that is current when they are made, so a host thread that drives
// several GPUs needs one entry per device ordinal.
struct Occupancy {
  static constexpr int kMaxDevices = 64;
  int per_sm[kMaxDevices] = {};
  int sms[kMaxDevices] = {};
};

// CTAs per SM of a persistent launch: as many as fit, capped by `cap` when
// cap > 0 (fewer CTAs per SM leave room for the launches of other streams
// to run on the same SMs).
inline int capped_per_sm(int fit, int cap) {
  return cap > 0 && cap < fit ? cap : fit;
}

// One persistent launch on the current device: as many CTAs as fit on it at
// once (capped by p.ctas_per_sm), or one per tile when there are fewer
// tiles.
template <typename Kernel>
void launch_persistent(Kernel kernel, size_t smem, LiftParams const &p,
                       cudaStream_t s, Occupancy &occ) {
  int const dev = current_device();
  if (dev < 0 || dev >= Occupancy::kMaxDevices)
    throw StatusError(2, "device ordinal beyond the launch cache");
  int &per_sm = occ.per_sm[dev];
  int &sms = occ.sms[dev];
  if (per_sm == 0) {
    if (smem > 0)
      cuda_check(cudaFuncSetAttribute(
                     kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                     static_cast<int>(smem)),
                 "cudaFuncSetAttribute");
    int n = 0;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel,
                                                             kThreads, smem),
               "occupancy query");
    sms = device_sms();
    per_sm = n < 1 ? 1 : n;
  }
  long long const resident =
      static_cast<long long>(capped_per_sm(per_sm, p.ctas_per_sm)) * sms;
  long long const blocks = std::min(p.total_tiles, resident);
  kernel<<<static_cast<unsigned>(blocks), kThreads, smem, s>>>(p);
  cuda_check(cudaGetLastError(), "lifting kernel launch");
}

template <class A, int R, class Sched, bool Direct>
void launch_r(LiftParams const &p, cudaStream_t s) {
  // Direct kernels keep pencils in registers and need no staging memory.
  size_t const smem = Direct ? 0 : lift_smem_bytes<A, R, kThreads>(kRounds);
  static thread_local Occupancy occ;
  if constexpr (lift_three_ctas<A, R, Direct>())
    launch_persistent(lift_kernel3<A, R, kThreads, Sched, Direct>, smem, p, s,
                      occ);
  else
    launch_persistent(lift_kernel<A, R, kThreads, Sched, Direct>, smem, p, s,
                      occ);
}

template <class A, int R, class Sched, bool Contig>
void launch_wide_r(LiftParams const &p, cudaStream_t s) {
  // The wide kernel counts units (two per tile) in 32 bits.
  if (p.total_tiles >= (1LL << 30))
    throw StatusError(2, "wide launch of 2^30 tiles or more");
  static thread_local Occupancy occ;
  launch_persistent(wide_kernel<A, R, kThreads, Sched, Contig>,
                    wide_smem_bytes<A, R, kThreads>(), p, s, occ);
}

template <class A, int R, class Sched, bool Long>
void launch_tile_r(LiftParams const &p, cudaStream_t s) {
  static thread_local Occupancy occ;
  launch_persistent(tile_kernel<A, R, kThreads, Sched, Long>,
                    tile_smem_bytes<A, R, kThreads, Long>(), p, s, occ);
}

// Row policy A (arith.cuh), code kWide + R (strided axis) or kWideContig + R
// (last axis) with R in {2, 4, 8, 16}; the wide kernel exists for the
// wavelet schedules only.
template <class A>
void launch_wide(int sched, int code, LiftParams const &p, cudaStream_t s) {
  auto by_r = [&](auto sch) {
    using Sched = decltype(sch);
    switch (code) {
    case kWide + 2: return launch_wide_r<A, 2, Sched, false>(p, s);
    case kWide + 4: return launch_wide_r<A, 4, Sched, false>(p, s);
    case kWide + 8: return launch_wide_r<A, 8, Sched, false>(p, s);
    case kWide + 16: return launch_wide_r<A, 16, Sched, false>(p, s);
    case kWideContig + 2: return launch_wide_r<A, 2, Sched, true>(p, s);
    case kWideContig + 4: return launch_wide_r<A, 4, Sched, true>(p, s);
    case kWideContig + 8: return launch_wide_r<A, 8, Sched, true>(p, s);
    case kWideContig + 16: return launch_wide_r<A, 16, Sched, true>(p, s);
    case kTile + 16: return launch_tile_r<A, 16, Sched, false>(p, s);
    case kTileLong + 16: return launch_tile_r<A, 16, Sched, true>(p, s);
    }
    throw StatusError(2, "bad chunk size");
  };
  switch (sched) {
  case 0: return by_r(WaveletSched<0, false>{});
  case 1: return by_r(WaveletSched<0, true>{});
  case 2: return by_r(WaveletSched<1, false>{});
  case 3: return by_r(WaveletSched<1, true>{});
  case 4: return by_r(WaveletSched<2, false>{});
  case 5: return by_r(WaveletSched<2, true>{});
  }
  throw StatusError(2, "wide kernel planned without a wavelet schedule");
}

// R > 0: staged tiles with chunks of R points; R < 0: direct pencils of
// -R points (one per thread).
template <class A, class Sched>
void launch_sched(int R, LiftParams const &p, cudaStream_t s) {
  switch (R) {
  case -2: return launch_r<A, 2, Sched, true>(p, s);
  case -4: return launch_r<A, 4, Sched, true>(p, s);
  case -8: return launch_r<A, 8, Sched, true>(p, s);
  case -16: return launch_r<A, 16, Sched, true>(p, s);
  case 16: return launch_r<A, 16, Sched, false>(p, s);
  case 32: return launch_r<A, 32, Sched, false>(p, s);
  }
  throw StatusError(2, "bad chunk size");
}

// sched < 0: runtime schedule; otherwise 2 * wavelet + (forward ? 1 : 0).
template <class A, bool WithWavelets>
void launch_any(int sched, int R, LiftParams const &p, cudaStream_t s) {
  if constexpr (WithWavelets) {
    switch (sched) {
    case 0: return launch_sched<A, WaveletSched<0, false>>(R, p, s);
    case 1: return launch_sched<A, WaveletSched<0, true>>(R, p, s);
    case 2: return launch_sched<A, WaveletSched<1, false>>(R, p, s);
    case 3: return launch_sched<A, WaveletSched<1, true>>(R, p, s);
    case 4: return launch_sched<A, WaveletSched<2, false>>(R, p, s);
    case 5: return launch_sched<A, WaveletSched<2, true>>(R, p, s);
    default: break;
    }
  }
  return launch_sched<A, RuntimeSched>(R, p, s);
}

void launch_lift_f64(bool exact, int sched, int R, LiftParams const &p,
                     cudaStream_t s);
void launch_lift_f32(bool exact, int sched, int R, LiftParams const &p,
                     cudaStream_t s);
void launch_lift_f32c(bool exact_sym, int sched, int R, LiftParams const &p,
                      cudaStream_t s);
void launch_halo(int dtype, LiftParams const &p, cudaStream_t s);
void launch_wide_f64(int sched, int code, LiftParams const &p, cudaStream_t s);
void launch_wide_f32(int sched, int code, LiftParams const &p, cudaStream_t s);
void launch_wide_f32c(int sched, int code, LiftParams const &p,
                      cudaStream_t s);

} // namespace pgb
