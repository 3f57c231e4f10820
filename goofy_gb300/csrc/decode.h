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

}  // namespace goofy_gpu
