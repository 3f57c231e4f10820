// quality.cpp -- C ABI of the GPU decoder and the encode-quality measurement
// (the reference harness's check: decode with Src/decoder.cpp, compare with
// getMsePsnr, Src/main.cpp:403-469).
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <mutex>

#include "../../include/goofy_gpu.h"
#include "decode.h"
#include "host_util.h"

namespace {

int check(int codec, const void* a, const void* b, uint32_t width, uint32_t height)
{
    if (codec != GOOFY_CODEC_BC1 && codec != GOOFY_CODEC_ETC1S) return GOOFY_ERR_INVALID;
    if (width % 4) return GOOFY_ERR_WIDTH;
    if (height % 4) return GOOFY_ERR_HEIGHT;
    if (width == 0 || height == 0) return GOOFY_OK;
    if (!a || !b) return GOOFY_ERR_INVALID;
    if ((uint64_t)(width / 4) * (height / 4) > 0x7fffffffull) return GOOFY_ERR_TOO_LARGE;
    return 1;
}

std::mutex g_mu;
unsigned long long* g_sums[64] = {};  // per device: 5 accumulators of goofy_gpu_psnr_rgb

}  // namespace

extern "C" {

GOOFY_EXPORT int goofy_gpu_decode_device(int codec, void* rgba, uint32_t rgba_stride, const void* blocks,
                                         uint32_t width, uint32_t height, uint64_t* d_unsupported, void* stream)
{
    int rc = check(codec, rgba, blocks, width, height);
    if (rc <= 0) return rc;
    if (!d_unsupported || reinterpret_cast<uintptr_t>(d_unsupported) % 8) return GOOFY_ERR_INVALID;
    if ((uint64_t)rgba_stride < 4ull * width) return GOOFY_ERR_INVALID;
    if (reinterpret_cast<uintptr_t>(rgba) % 16 || rgba_stride % 16 || reinterpret_cast<uintptr_t>(blocks) % 8)
        return GOOFY_ERR_ALIGNMENT;
    GOOFY_CUDA_TRY(goofy_gpu::launch_decode(codec, static_cast<const uint8_t*>(blocks), width, height,
                                            static_cast<uint8_t*>(rgba), rgba_stride,
                                            reinterpret_cast<unsigned long long*>(d_unsupported),
                                            static_cast<cudaStream_t>(stream)));
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_block_error_device(int codec, const void* blocks, const void* src, uint32_t width,
                                              uint32_t height, uint32_t stride, uint64_t* d_sums, void* stream)
{
    int rc = check(codec, blocks, src, width, height);
    if (rc <= 0) return rc;
    if (!d_sums || reinterpret_cast<uintptr_t>(d_sums) % 8) return GOOFY_ERR_INVALID;
    if ((uint64_t)stride < 4ull * width) return GOOFY_ERR_INVALID;
    const uintptr_t s = reinterpret_cast<uintptr_t>(src);
    if (s % 4 || stride % 4 || reinterpret_cast<uintptr_t>(blocks) % 8) return GOOFY_ERR_ALIGNMENT;
    GOOFY_CUDA_TRY(goofy_gpu::launch_block_error(codec, static_cast<const uint8_t*>(blocks),
                                                 static_cast<const uint8_t*>(src), width, height, stride,
                                                 s % 16 == 0 && stride % 16 == 0,
                                                 reinterpret_cast<unsigned long long*>(d_sums),
                                                 static_cast<cudaStream_t>(stream)));
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_psnr_rgb(int codec, const void* blocks, const void* src, uint32_t width, uint32_t height,
                                    uint32_t stride, double* psnr_rgb, uint64_t* sums_out)
{
    int rc = check(codec, blocks, src, width, height);
    if (rc <= 0) return rc == GOOFY_OK ? GOOFY_ERR_INVALID : rc;
    int dev = 0;
    GOOFY_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return GOOFY_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_sums[dev]) GOOFY_CUDA_TRY(cudaMalloc(&g_sums[dev], 5 * sizeof(unsigned long long)));
    cudaStream_t st = nullptr;
    GOOFY_CUDA_TRY(cudaMemsetAsync(g_sums[dev], 0, 5 * sizeof(unsigned long long), st));
    rc = goofy_gpu_block_error_device(codec, blocks, src, width, height, stride,
                                      reinterpret_cast<uint64_t*>(g_sums[dev]), st);
    if (rc != GOOFY_OK) return rc;
    unsigned long long h[5];
    GOOFY_CUDA_TRY(cudaMemcpy(h, g_sums[dev], sizeof h, cudaMemcpyDeviceToHost));
    if (sums_out)
        for (int i = 0; i < 5; ++i) sums_out[i] = h[i];
    // getPSNR(mseRGB, 768), Src/main.cpp:386-395 and :455, :466
    const double mse = (double)(h[0] + h[1] + h[2]) / ((double)width * (double)height);
    if (psnr_rgb) *psnr_rgb = mse < 0.0000001 ? DBL_MAX : 10.0 * std::log10((768.0 * 768.0) / mse);
    return GOOFY_OK;
}

}  // extern "C"
