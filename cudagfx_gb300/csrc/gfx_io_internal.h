// gfx_io_internal.h -- helpers shared by the file code (gfx_io.cpp) and the
// context code that writes checkpoints (gfx_api.cu).
#pragma once
#include <cstddef>
#include <string>

namespace gfx {
// the message gfx_last_error(NULL) returns
void set_global_error(const std::string& msg);
// n 8-byte / 4-byte words between host order and big-endian (in and out may alias)
void to_be64(const void* in, size_t n, void* out);
void from_be64(const void* in, size_t n, void* out);
void to_be32(const void* in, size_t n, void* out);
void from_be32(const void* in, size_t n, void* out);
}  // namespace gfx
