// kernels.h -- host-side launchers of the encoder kernels (internal C++ API
// between the C-ABI layer and the CUDA translation unit).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace goofy_gpu {

struct Tile {
    uint32_t threads;     // threads per CTA: 128, 256 or 512
    uint32_t bpt;         // 4x4 blocks per thread and segment: 1, 2 or 4 (1 or 2 when persistent)
    uint32_t persistent;  // 0: one segment per warp; 1: resident grid looping over segments with prefetch;
                          // 2: resident grid fed by bulk copies into a shared-memory ring (+1 producer warp)
};

inline bool tile_valid(const Tile& t)
{
    if (t.threads != 128 && t.threads != 256 && t.threads != 512) return false;
    if (t.persistent > 2) return false;
    return t.bpt == 1 || t.bpt == 2 || (t.bpt == 4 && !t.persistent);
}

// How the image kernel reads its source rows.
enum class SrcAccess : int {
    kVec16 = 0,  // 16-byte aligned base and stride: one 128-bit load per block row
    kWord4 = 1,  // 4-byte aligned: four 32-bit loads per block row
};

// Encode a whole image (width, height multiples of 4) into row-major 8-byte
// blocks at `dst`.  Only enqueues; returns the launch error, if any.  With
// codec kBoth (block_codec.cuh) one pass writes the BC1 blocks to `dst` and
// the ETC1s blocks to `dst2` (shapes: 1 or 2 blocks a thread; a resident
// grid with prefetch runs as the plain grid).
cudaError_t launch_image(int codec, const uint8_t* src, size_t stride, uint8_t* dst, uint32_t width,
                         uint32_t height, Tile tile, SrcAccess access, cudaStream_t stream, uint8_t* dst2 = nullptr);

// The bulk-copy pipeline kernel (tile.persistent == 2); needs a 16-byte
// aligned source base and stride.
cudaError_t launch_image_tma(int codec, const uint8_t* src, size_t stride, uint8_t* dst, uint32_t width,
                             uint32_t height, Tile tile, cudaStream_t stream, uint8_t* dst2 = nullptr);

// Pipeline waits that gave up on the current device since the last reset.
cudaError_t pipeline_timeouts(unsigned int* count, bool reset);

// One bounded wait on a barrier that nothing completes (async_copy.cuh):
// returns the wait's result (false: it gave up), whether it raised the abort
// flag and how many time-outs it counted.  Synchronous.
cudaError_t bounded_wait_selftest(bool* completed, bool* aborted, unsigned int* counted);

}  // namespace goofy_gpu
