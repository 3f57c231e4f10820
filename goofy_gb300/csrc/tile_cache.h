// tile_cache.h -- tuned image-kernel tiles kept in a text file per GPU model
// (tile_cache.cpp).
#pragma once
#include <cstdint>
#include <string>

#include "host_util.h"
#include "kernels.h"

namespace goofy_gpu {

// The cache file in use: the path given to set_tile_cache_path, else
// $GOOFY_TILE_CACHE, else $XDG_CACHE_HOME/goofy_gb300/tiles.txt, else
// $HOME/.cache/goofy_gb300/tiles.txt.  "" means no cache.
std::string tile_cache_path();

// Overrides the path (nullptr: back to the environment / default).
void set_tile_cache_path(const char* path);

// The recorded tile of `codec` (0 BC1, 1 ETC1s, 2 the two-codec pass) for a
// GPU named `gpu` with `sms` SMs; false when there is none.
bool tile_cache_lookup(const std::string& path, const std::string& gpu, uint32_t sms, int codec, Tile* out);

// Records (replaces) that entry with its measured launch time.  GOOFY_OK or
// GOOFY_ERR_INVALID with the reason in the last error.
int tile_cache_store(const std::string& path, const std::string& gpu, uint32_t sms, int codec, const Tile& t,
                     float us);

}  // namespace goofy_gpu
