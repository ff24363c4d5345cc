// On-disk brick store of the reference (BricksManager.cpp:81-227,
// BrickKey.cpp:38-44, MetaData.cpp:36-101): internal interface shared by the
// C entry points (brickfiles.cpp) and the cache's file-backed loader.
#pragma once

#include <cstdint>
#include <string>

namespace gc {

// "<dir>bricks_B_B_B/L<l>/L<l>_<x>_<y>_<z>.raw" (dir ends with '/' or is empty)
std::string brick_file_path(const std::string &dir, uint32_t B, uint32_t level, uint32_t x, uint32_t y, uint32_t z);

// liblz4 is loaded on first use; false (with the reason) when it is missing.
bool lz4_available(std::string *why);

// Reads and decompresses one big-brick file into dst (exactly `bytes` bytes).
// Returns 0 on success, 1 when the file does not exist, 2 when it is corrupt
// (short, unreadable, or not an LZ4 block of `bytes` bytes).
int read_brick_file(const std::string &path, void *dst, uint64_t bytes);

}  // namespace gc
