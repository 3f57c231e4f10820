// decode.h -- launchers of the block decoder and the squared-error reduction.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace goofy_gpu {

// Decode (width/4)*(height/4) blocks into RGBA8 rows (`rgba`, `stride`: both
// 16-byte aligned).  Adds the count of unsupported ETC1 blocks to *unsupported.
cudaError_t launch_decode(int codec, const uint8_t* blocks, uint32_t width, uint32_t height, uint8_t* rgba,
                          size_t stride, unsigned long long* unsupported, cudaStream_t stream);

// Adds the per-channel sums of squared differences between `src` and the
// decoded blocks to sums[0..3], the unsupported-block count to sums[4] and the
// sum of squared luminosity differences (hundredths) to sums[5].
cudaError_t launch_block_error(int codec, const uint8_t* blocks, const uint8_t* src, uint32_t width, uint32_t height,
                               size_t stride, bool vec16, unsigned long long* sums, cudaStream_t stream);

struct BatchImage;

// Adds the six error sums of every image of a batch (blocks at `dst`, source
// at `src`) to sums[6 * i + c]; work units as for the batch encoder
// (`first_unit`, `unit_blocks`), `work_counter` reading 0 at the start.
cudaError_t launch_quality_batch(const BatchImage* images, uint32_t n_images, const uint32_t* first_unit,
                                 uint32_t total_units, uint32_t unit_blocks, uint32_t* work_counter,
                                 unsigned long long* sums, cudaStream_t stream);

}  // namespace goofy_gpu
