// batch.h -- device descriptor of a batch image and the batch launcher
// (shared by batch_kernels.cu and the host code in batch.cpp).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

struct goofy_gpu_image;  // include/goofy_gpu.h

namespace goofy_gpu {

// One image of a batch, as the persistent kernel reads it.  Filled and
// validated on the host (dimensions multiples of 4, alignment, sizes).
struct BatchImage {
    const uint8_t* src;   // device RGBA8, `stride` bytes per row
    uint8_t* dst;         // device output, bw * bh blocks of 8 bytes
    uint32_t stride;      // bytes per source row
    uint32_t bw, bh;      // blocks per row, block rows
    uint32_t bw_magic;    // floor((2^32 - 1) / bw), for block index -> (row, column)
    uint32_t first_unit;  // first work unit of this image
    uint32_t codec;       // kBC1 or kETC1S
    uint32_t vec16;       // 1: 16-byte aligned rows (vector loads), 0: 4-byte aligned
    uint32_t reserved;
};
static_assert(sizeof(BatchImage) == 48, "BatchImage layout");

struct BatchTile {
    uint32_t threads;      // threads per CTA: 128, 256, 512 (compute threads with pipeline = 1)
    uint32_t bpt;          // blocks per lane per step: 1 or 2
    uint32_t unit_blocks;  // blocks per work unit (multiple of 32 * bpt; threads * bpt with pipeline = 1)
    uint32_t pipeline;     // 0: warps pull units and load rows themselves; 1: a producer warp per CTA
                           // bulk-copies each unit's rows into a shared-memory ring (encode_tma.cu)
};

inline bool batch_tile_valid(const BatchTile& t)
{
    if (t.threads != 128 && t.threads != 256 && t.threads != 512) return false;
    if (t.bpt != 1 && t.bpt != 2) return false;
    if (t.pipeline > 1) return false;
    if (t.pipeline) return t.unit_blocks == t.threads * t.bpt;
    return t.unit_blocks >= 32 * t.bpt && t.unit_blocks <= 65536 && t.unit_blocks % (32 * t.bpt) == 0;
}

// CTAs of the batch kernel that fit on the current device at once.
int batch_resident_ctas(uint32_t threads, uint32_t bpt, uint32_t pipeline = 0);

// The same for the pipelined batch kernel (encode_tma.cu), and its launcher:
// one unit of threads * bpt blocks per stage.
int batch_tma_resident_ctas(uint32_t threads, uint32_t bpt);
cudaError_t launch_batch_tma(const BatchImage* images, uint32_t n_images, const uint32_t* first_unit,
                             uint32_t total_units, uint32_t* work_counter, const BatchTile& tile, uint32_t ctas,
                             cudaStream_t stream);

// A pipelined batch of at most kInlineImages images, passed by value as the
// kernel's parameter (3.3 KB): the launch needs no descriptor upload.
constexpr uint32_t kInlineImages = 64;
struct InlineBatch {
    BatchImage images[kInlineImages];
    uint32_t first_unit[kInlineImages];
};
cudaError_t launch_batch_tma_inline(const InlineBatch& batch, uint32_t n_images, uint32_t total_units,
                                    const BatchTile& tile, uint32_t ctas, cudaStream_t stream);

// Checks `count` caller images (codec, sizes multiples of 4, non-null and
// aligned buffers, stride) and fills their device descriptors, the first-unit
// table (`first[i]` = desc[i].first_unit) and the total of work units of
// `unit_blocks` blocks.  Empty images get no units.  Returns GOOFY_OK or the
// status of the first bad image (with its message in the last error).
int validate_and_fill(const goofy_gpu_image* images, uint32_t count, uint32_t unit_blocks, BatchImage* desc,
                      uint32_t* first, uint32_t* total_units);

// Enqueue the persistent batch kernel.  `work_counter` must read 0 when the
// kernel starts; `first_unit[i]` is images[i].first_unit (ascending, [0] = 0).
cudaError_t launch_batch(const BatchImage* images, uint32_t n_images, const uint32_t* first_unit,
                         uint32_t total_units, uint32_t* work_counter, const BatchTile& tile, uint32_t ctas,
                         cudaStream_t stream);

}  // namespace goofy_gpu
