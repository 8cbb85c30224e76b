// brm_hostpool.h -- cache of page-locked host blocks for host drop-in results.
#pragma once

#include <cstddef>

namespace brm {

// A host block of at least `bytes` bytes, page-locked when possible (malloc
// otherwise).  nullptr only when both fail.
void *host_alloc(size_t bytes);

// Returns a block from host_alloc to the cache (true), or false when `p` did
// not come from host_alloc's page-locked path (the caller frees it).
bool host_release(void *p);

// Releases every cached, unused block.
void host_trim();

}  // namespace brm
