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

template <class A, int R, class Sched, bool Direct>
void launch_r(LiftParams const &p, cudaStream_t s) {
  auto kernel = lift_kernel<A, R, kThreads, Sched, Direct>;
  // Direct kernels keep pencils in registers and need no staging memory.
  size_t const smem = Direct ? 0 : lift_smem_bytes<A, R, kThreads>(kRounds);
  static thread_local int per_sm = 0;
  static thread_local int sms = 0;
  if (per_sm == 0) {
    if (smem > 0)
      cuda_check(cudaFuncSetAttribute(
                     kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                     static_cast<int>(smem)),
                 "cudaFuncSetAttribute");
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &per_sm, kernel, kThreads, smem),
               "occupancy query");
    sms = device_sms();
    if (per_sm < 1) per_sm = 1;
  }
  long long const resident = static_cast<long long>(per_sm) * sms;
  long long const blocks = std::min(p.total_tiles, resident);
  kernel<<<static_cast<unsigned>(blocks), kThreads, smem, s>>>(p);
  cuda_check(cudaGetLastError(), "lift_kernel launch");
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

} // namespace pgb
