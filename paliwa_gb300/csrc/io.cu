// Raw dump of a device grid: paliwa::dump_chunk_span_to_binary_file
// (paliwa/paliwa_io.hpp:13-23) writes a chunk's values in storage order
// (row-major, native byte order, no header) after mirroring it to pinned host
// memory; paliwa/postprocess.py:30-35 reads such files back with
// numpy.fromfile. Here the copy and the file write overlap: the grid moves to
// the host in pieces through two pinned buffers, and the next piece's copy
// runs while the previous one is written.
#include <cstdint>
#include <cstdio>
#include <string>

#include "paliwa_gb300.h"
#include "plan.hpp"

namespace pgb {
namespace {

constexpr size_t kDumpPiece = size_t{32} << 20;

struct PinnedPair {
  void *buf[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  ~PinnedPair() {
    for (int k = 0; k < 2; ++k) {
      if (done[k] != nullptr) cudaEventDestroy(done[k]);
      if (buf[k] != nullptr) cudaFreeHost(buf[k]);
    }
  }
};

struct File {
  std::FILE *f = nullptr;
  ~File() {
    if (f != nullptr) std::fclose(f);
  }
};

} // namespace
} // namespace pgb

extern "C" {

int paliwa_gb_dump_to_binary_file(const void *data, int64_t bytes,
                                  const char *filename, void *stream) {
  using namespace pgb;
  return guarded([&] {
    if (filename == nullptr)
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "filename is null");
    if (bytes < 0 || (bytes > 0 && data == nullptr))
      throw StatusError(PALIWA_GB_INVALID_ARGUMENT, "bad buffer");
    File out;
    out.f = std::fopen(filename, "wb");  // truncates, like the reference
    if (out.f == nullptr)
      throw StatusError(PALIWA_GB_RUNTIME_ERROR,
                        std::string("cannot open ") + filename);
    if (bytes == 0) return;
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    size_t const total = static_cast<size_t>(bytes);
    size_t const piece = total < kDumpPiece ? total : kDumpPiece;
    PinnedPair pp;
    for (int k = 0; k < 2; ++k) {
      cuda_check(cudaMallocHost(&pp.buf[k], piece), "cudaMallocHost");
      cuda_check(cudaEventCreateWithFlags(&pp.done[k],
                                          cudaEventDisableTiming),
                 "cudaEventCreate");
    }
    char const *src = static_cast<char const *>(data);
    size_t const npieces = (total + piece - 1) / piece;
    auto issue = [&](size_t i) {
      size_t const off = i * piece;
      size_t const n = total - off < piece ? total - off : piece;
      // Stream-ordered: the copy waits for the work queued before it.
      cuda_check(cudaMemcpyAsync(pp.buf[i & 1], src + off, n,
                                 cudaMemcpyDeviceToHost, s),
                 "cudaMemcpyAsync");
      cuda_check(cudaEventRecord(pp.done[i & 1], s), "cudaEventRecord");
    };
    issue(0);
    for (size_t i = 0; i < npieces; ++i) {
      if (i + 1 < npieces) issue(i + 1);  // buffer (i+1)&1 was written out
      cuda_check(cudaEventSynchronize(pp.done[i & 1]), "cudaEventSynchronize");
      size_t const off = i * piece;
      size_t const n = total - off < piece ? total - off : piece;
      if (std::fwrite(pp.buf[i & 1], 1, n, out.f) != n)
        throw StatusError(PALIWA_GB_RUNTIME_ERROR,
                          std::string("short write to ") + filename);
    }
    if (std::fflush(out.f) != 0)
      throw StatusError(PALIWA_GB_RUNTIME_ERROR,
                        std::string("cannot flush ") + filename);
  });
}

} // extern "C"
