// quality.cpp -- C ABI of the GPU decoder and the encode-quality measurement
// (the reference harness's check: decode with Src/decoder.cpp, compare with
// getMsePsnr, Src/main.cpp:403-469).
#include <cuda_runtime.h>

#include <cfloat>
#include <algorithm>
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
unsigned long long* g_sums[64] = {};  // per device: the 6 accumulators of the synchronous quality calls

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

}  // extern "C"

namespace {

// getPSNR, Src/main.cpp:386-395
double psnr_of(double mse, double peak) { return mse < 0.0000001 ? DBL_MAX : 10.0 * std::log10((peak * peak) / mse); }

// Runs the error kernel on the current device into a library-owned
// accumulator and reads the six sums back.
int error_sums(int codec, const void* blocks, const void* src, uint32_t width, uint32_t height, uint32_t stride,
               unsigned long long h[6])
{
    int rc = check(codec, blocks, src, width, height);
    if (rc <= 0) return rc == GOOFY_OK ? GOOFY_ERR_INVALID : rc;
    int dev = 0;
    GOOFY_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return GOOFY_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_sums[dev]) GOOFY_CUDA_TRY(cudaMalloc(&g_sums[dev], 6 * sizeof(unsigned long long)));
    cudaStream_t st = nullptr;
    GOOFY_CUDA_TRY(cudaMemsetAsync(g_sums[dev], 0, 6 * sizeof(unsigned long long), st));
    rc = goofy_gpu_block_error_device(codec, blocks, src, width, height, stride,
                                      reinterpret_cast<uint64_t*>(g_sums[dev]), st);
    if (rc != GOOFY_OK) return rc;
    GOOFY_CUDA_TRY(cudaMemcpy(h, g_sums[dev], 6 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    return GOOFY_OK;
}

}  // namespace

extern "C" {

GOOFY_EXPORT int goofy_gpu_psnr_rgb(int codec, const void* blocks, const void* src, uint32_t width, uint32_t height,
                                    uint32_t stride, double* psnr_rgb, uint64_t* sums_out)
{
    unsigned long long h[6];
    const int rc = error_sums(codec, blocks, src, width, height, stride, h);
    if (rc != GOOFY_OK) return rc;
    if (sums_out)
        for (int i = 0; i < 5; ++i) sums_out[i] = h[i];
    // getPSNR(mseRGB, 768), Src/main.cpp:455, :466
    const double mse = (double)(h[0] + h[1] + h[2]) / ((double)width * (double)height);
    if (psnr_rgb) *psnr_rgb = psnr_of(mse, 768.0);
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_mse_psnr(int codec, const void* blocks, const void* src, uint32_t width, uint32_t height,
                                    uint32_t stride, goofy_gpu_quality* out)
{
    if (!out) return GOOFY_ERR_INVALID;
    unsigned long long h[6];
    const int rc = error_sums(codec, blocks, src, width, height, stride, h);
    if (rc != GOOFY_OK) return rc;
    // Src/main.cpp:456-468; the harness's r is byte 2 and its b byte 0
    const double n = (double)(uint32_t)(width * height);
    goofy_gpu_quality& r = *out;
    r.mse_r = (double)h[2] / n;
    r.mse_g = (double)h[1] / n;
    r.mse_b = (double)h[0] / n;
    r.mse_a = (double)h[3] / n;
    r.mse_rgb = (double)(h[0] + h[1] + h[2]) / n;
    r.mse_y = (double)h[5] / 10000.0 / n;
    r.mse_max = std::max(std::max(r.mse_r, r.mse_g), std::max(r.mse_b, r.mse_a));
    r.psnr_r = psnr_of(r.mse_r, 255.0);
    r.psnr_g = psnr_of(r.mse_g, 255.0);
    r.psnr_b = psnr_of(r.mse_b, 255.0);
    r.psnr_a = psnr_of(r.mse_a, 255.0);
    r.psnr_min = std::min(std::min(r.psnr_r, r.psnr_g), std::min(r.psnr_b, r.psnr_a));
    r.psnr_rgb = psnr_of(r.mse_rgb, 768.0);
    r.psnr_y = psnr_of(r.mse_y, 255.0);
    r.unsupported_blocks = h[4];
    return GOOFY_OK;
}

}  // extern "C"
