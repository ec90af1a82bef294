// Launches of the TMA wide kernel (twide.cuh) for FP32-compensated grids
// (rows of two columns as double-float f32x2 pairs).
#include "launch.cuh"
#include "twide.cuh"

namespace pgb {

namespace {

template <int R, class Sched, int FORM>
void launch_twide_r(TWideParams const &p, cudaStream_t s) {
  static thread_local Occupancy occ;
  constexpr bool kLong = FORM == 2 || FORM == 5;
  constexpr int kBlock = kLong ? kTWideThreads : kTWideBlock;
  auto kernel = [] {
    if constexpr (kLong)
      return twide_long_kernel<RowF32C, Sched, FORM == 5>;
    else
      return twide_kernel<RowF32C, R, Sched, FORM>;
  }();
  size_t const smem = twide_smem_bytes<R, kLong>();
  int const dev = current_device();
  if (dev < 0 || dev >= Occupancy::kMaxDevices)
    throw StatusError(2, "device ordinal beyond the launch cache");
  int &per_sm = occ.per_sm[dev];
  int &sms = occ.sms[dev];
  if (per_sm == 0) {
    cuda_check(cudaFuncSetAttribute(
                   kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                   static_cast<int>(smem)),
               "cudaFuncSetAttribute(twide)");
    int n = 0;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &n, kernel, kBlock, smem),
               "occupancy query (twide)");
    sms = device_sms();
    per_sm = n < 1 ? 1 : n;
  }
  long long const resident =
      static_cast<long long>(capped_per_sm(per_sm, p.ctas_per_sm)) * sms;
  long long const blocks = std::min(p.total_tiles, resident);
  kernel<<<static_cast<unsigned>(blocks), kBlock, smem, s>>>(p);
  cuda_check(cudaGetLastError(), "twide kernel launch");
}

template <class Sched>
void by_r(int R, TWideParams const &p, cudaStream_t s) {
  switch (R) {
  case 2: return launch_twide_r<2, Sched, 0>(p, s);
  case 4: return launch_twide_r<4, Sched, 0>(p, s);
  case 8: return launch_twide_r<8, Sched, 0>(p, s);
  case 16: return launch_twide_r<16, Sched, 0>(p, s);
  case kTWideChunked + 16: return launch_twide_r<16, Sched, 1>(p, s);
  case kTWideContig + 4: return launch_twide_r<4, Sched, 3>(p, s);
  case kTWideContig + 8: return launch_twide_r<8, Sched, 3>(p, s);
  case kTWideContig + 16: return launch_twide_r<16, Sched, 3>(p, s);
  case kTWidePairs + 4: return launch_twide_r<4, Sched, 4>(p, s);
  case kTWidePairs + 8: return launch_twide_r<8, Sched, 4>(p, s);
  case kTWidePairs + 16: return launch_twide_r<16, Sched, 4>(p, s);
  case kTWideLong + 16: return launch_twide_r<16, Sched, 2>(p, s);
  case kTWideLongContig + 16: return launch_twide_r<16, Sched, 5>(p, s);
  }
  throw StatusError(2, "twide launch with an unsupported chunk size");
}

} // namespace

// sched = 2 * wavelet + (forward ? 1 : 0); R = rows per chunk, plus
// kTWideChunked for pencils of 8 to 32 chunks, kTWideLong for more,
// kTWideContig for the last axis (kTWideLongContig for its pencils of more
// than 32 chunks) and kTWidePairs for strided axes of inner extent 2.
void launch_twide_f32c(int sched, int R, TWideParams const &p,
                       cudaStream_t s) {
  switch (sched) {
  case 0: return by_r<WaveletSched<0, false>>(R, p, s);
  case 1: return by_r<WaveletSched<0, true>>(R, p, s);
  case 2: return by_r<WaveletSched<1, false>>(R, p, s);
  case 3: return by_r<WaveletSched<1, true>>(R, p, s);
  case 4: return by_r<WaveletSched<2, false>>(R, p, s);
  case 5: return by_r<WaveletSched<2, true>>(R, p, s);
  }
  throw StatusError(2, "twide kernel planned without a wavelet schedule");
}

} // namespace pgb
