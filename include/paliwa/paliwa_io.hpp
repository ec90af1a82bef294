// Drop-in replacement of paliwa/paliwa_io.hpp: dump a chunk span of device
// memory to a raw binary file (storage order, native byte order, no header),
// the format paliwa/postprocess.py reads. Runs through the C ABI in
// paliwa_gb300.h; the copy is ordered after the work on `instance` (default:
// the legacy default stream), and the call returns once the file is written.
#pragma once

#include <cstdint>
#include <string>

#include "../paliwa_gb300.h"
#include "paliwa_transform.hpp"

namespace paliwa {

// paliwa_io.hpp:13-23
template <typename ChunkType, class ExecSpace = gb300::Stream>
constexpr void dump_chunk_span_to_binary_file(ChunkType const span,
                                              std::string const &filename,
                                              ExecSpace instance = ExecSpace()) {
  using T = typename ChunkType::element_type;
  gb300::check(paliwa_gb_dump_to_binary_file(
      static_cast<void const *>(span.data_handle()),
      static_cast<int64_t>(span.domain().size() * sizeof(T)),
      filename.c_str(), gb300::stream_of(instance)));
}

} // namespace paliwa
