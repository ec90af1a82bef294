// Launch of the slab kernel (slab.cuh) for one arithmetic policy; included
// by the per-dtype translation units slab_f64.cu, slab_f32.cu, slab_f32c.cu.
#pragma once

#include "launch.cuh"
#include "slab.cuh"

namespace pgb {

template <class A, class Sched>
void launch_slab_r(SlabParams const &p, cudaStream_t s) {
  static thread_local Occupancy occ;
  auto kernel = slab_kernel<A, Sched>;
  size_t const smem = slab_smem_bytes<A>();
  int const dev = current_device();
  if (dev < 0 || dev >= Occupancy::kMaxDevices)
    throw StatusError(2, "device ordinal beyond the launch cache");
  int &per_sm = occ.per_sm[dev];
  int &sms = occ.sms[dev];
  if (per_sm == 0) {
    cuda_check(cudaFuncSetAttribute(
                   kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                   static_cast<int>(smem)),
               "cudaFuncSetAttribute(slab)");
    int n = 0;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &n, kernel, kSlabThreads, smem),
               "occupancy query (slab)");
    sms = device_sms();
    per_sm = n < 1 ? 1 : n;
  }
  long long const resident =
      static_cast<long long>(capped_per_sm(per_sm, p.ctas_per_sm)) * sms;
  long long const blocks = std::min(p.total_tiles, resident);
  kernel<<<static_cast<unsigned>(blocks), kSlabThreads, smem, s>>>(p);
  cuda_check(cudaGetLastError(), "slab kernel launch");
}

// sched = 2 * wavelet + (forward ? 1 : 0).
template <class A>
void launch_slab_any(int sched, SlabParams const &p, cudaStream_t s) {
  switch (sched) {
  case 0: return launch_slab_r<A, WaveletSched<0, false>>(p, s);
  case 1: return launch_slab_r<A, WaveletSched<0, true>>(p, s);
  case 2: return launch_slab_r<A, WaveletSched<1, false>>(p, s);
  case 3: return launch_slab_r<A, WaveletSched<1, true>>(p, s);
  case 4: return launch_slab_r<A, WaveletSched<2, false>>(p, s);
  case 5: return launch_slab_r<A, WaveletSched<2, true>>(p, s);
  }
  throw StatusError(2, "slab kernel planned without a wavelet schedule");
}

} // namespace pgb
