// batch_kernels.cu -- many images of uneven sizes (textures, mip levels) in
// one persistent launch.
//
// The reference encodes one image per call (goofy::compressDXT1/ETC1,
// GoofyTC/goofy_tc.h:1497-1557); here a batch of images is flattened into
// work units of `unit_blocks` consecutive 4x4 blocks of one image (the last
// unit of an image may be short).  A resident grid of warps pulls units from
// a device work counter (one atomicAdd per unit, by lane 0), finds the unit's
// image by binary search over the per-image first-unit table, and encodes the
// unit's blocks with the same per-block codec as the image kernel.  Codec and
// load mode are uniform per unit, so warps never diverge on them.  There is no
// waiting: a warp that draws a unit number past the end exits.
#include <cuda_runtime.h>

#include "batch.h"
#include "block_codec.cuh"
#include "device_io.cuh"

namespace goofy_gpu {

template <int BPT>
__global__ void __launch_bounds__(512) encode_batch_kernel(const BatchImage* __restrict__ images, uint32_t n_images,
                                                           const uint32_t* __restrict__ first_unit,
                                                           uint32_t total_units, uint32_t unit_blocks,
                                                           uint32_t* __restrict__ work_counter)
{
    __shared__ uint8_t ctrl_lut[128];
    fill_ctrl_lut(ctrl_lut);
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(work_counter, 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= total_units) return;
        const uint32_t ii = find_image(first_unit, n_images, u);
        const BatchImage im = images[ii];
        const uint32_t nblk = im.bw * im.bh;
        const uint32_t first = (u - im.first_unit) * unit_blocks;
        const uint32_t last = min(first + unit_blocks, nblk);
        const bool vec16 = im.vec16 != 0;
        for (uint32_t b0 = first; b0 < last; b0 += 32u * BPT) {
            uint32_t w[BPT][16];
            uint32_t blk[BPT];
#pragma unroll
            for (int j = 0; j < BPT; ++j) {
                blk[j] = b0 + lane + 32u * j;
                if (blk[j] < last) {
                    uint32_t bx;
                    const uint32_t by = div_magic(blk[j], im.bw, im.bw_magic, bx);
                    load_block_rows(im.src + (size_t)by * 4u * im.stride + 16u * (size_t)bx, im.stride, vec16, w[j]);
                }
            }
#pragma unroll
            for (int j = 0; j < BPT; ++j) {
                if (blk[j] < last) {
                    const uint2 e = im.codec == kBC1 ? encode_bc1(w[j]) : encode_etc1s(w[j], ctrl_lut);
                    st_stream8(im.dst + 8u * (size_t)blk[j], e);
                }
            }
        }
    }
}

int batch_resident_ctas(uint32_t threads, uint32_t bpt, uint32_t pipeline)
{
    if (pipeline) return batch_tma_resident_ctas(threads, bpt);
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (bpt == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, encode_batch_kernel<1>, threads, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, encode_batch_kernel<2>, threads, 0);
    return sms * (per_sm > 0 ? per_sm : 1);
}

cudaError_t launch_batch(const BatchImage* images, uint32_t n_images, const uint32_t* first_unit,
                         uint32_t total_units, uint32_t* work_counter, const BatchTile& tile, uint32_t ctas,
                         cudaStream_t stream)
{
    if (total_units == 0) return cudaSuccess;
    if (tile.pipeline) return launch_batch_tma(images, n_images, first_unit, total_units, work_counter, tile, ctas, stream);
    if (tile.bpt == 1)
        encode_batch_kernel<1><<<ctas, tile.threads, 0, stream>>>(images, n_images, first_unit, total_units,
                                                                   tile.unit_blocks, work_counter);
    else
        encode_batch_kernel<2><<<ctas, tile.threads, 0, stream>>>(images, n_images, first_unit, total_units,
                                                                   tile.unit_blocks, work_counter);
    return cudaGetLastError();
}

}  // namespace goofy_gpu
