// batch_noalloc.cu -- batch encoding that allocates nothing.
//
// Some callers may not allocate on the path that encodes: a texture-streaming
// thread working inside a renderer's frame budget, where cudaMalloc / cudaFree
// can stall or synchronise the whole device, or a host engine that owns every
// byte of GPU memory through its own allocator and does not let libraries call
// the CUDA allocator.  goofy_gpu_batch_create allocates descriptor tables and
// a work counter, so those callers cannot use it.  This entry point keeps that
// scratch in one fixed-size file-scope device array instead; the array is part
// of the library's module and is held on every GPU that loads the library
// until the process exits.  Inputs and outputs are still the caller's device
// buffers.  The kernel is the ordinary batch kernel, given pointers into the
// array.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/goofy_gpu.h"
#include "batch.h"
#include "host_util.h"

namespace {

constexpr uint32_t kMaxImages = GOOFY_NOALLOC_MAX_IMAGES;

struct Scratch {
    uint32_t work_counter;                     // must read 0 when a launch starts
    uint32_t pad[63];                          // tables start 256 bytes in
    uint32_t first_unit[kMaxImages];           // first work unit of each image
    goofy_gpu::BatchImage images[kMaxImages];  // descriptors
};

// The whole scratch: 256 + 4 * 256 + 48 * 256 = 13,568 bytes per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(Scratch)];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
Scratch* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  The first call
// per device asks the runtime for it (cudaGetSymbolAddress) and caches it.
int scratch_address(Scratch** out)
{
    int dev = 0;
    GOOFY_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return goofy_gpu::fail(GOOFY_ERR_NO_DEVICE, "noalloc: device index too large");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return goofy_gpu::cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
        g_scratch_addr[dev] = static_cast<Scratch*>(p);
    }
    *out = g_scratch_addr[dev];
    return GOOFY_OK;
}

// Descriptor of one image (same rules as goofy_gpu_batch_encode).
int describe(const goofy_gpu_image& im, uint32_t unit_blocks, uint64_t* units, goofy_gpu::BatchImage* d)
{
    std::memset(d, 0, sizeof *d);
    if (im.codec != GOOFY_CODEC_BC1 && im.codec != GOOFY_CODEC_ETC1S)
        return goofy_gpu::fail(GOOFY_ERR_INVALID, "noalloc: bad codec");
    if (im.width % 4) return goofy_gpu::fail(GOOFY_ERR_WIDTH, "noalloc: width % 4 != 0");
    if (im.height % 4) return goofy_gpu::fail(GOOFY_ERR_HEIGHT, "noalloc: height % 4 != 0");
    const uint64_t bw = im.width / 4, bh = im.height / 4;
    if (bw * bh > 0x7fffffffull) return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "noalloc: image too large");
    d->first_unit = (uint32_t)*units;
    if (bw == 0 || bh == 0) return GOOFY_OK;
    if (!im.src || !im.dst) return goofy_gpu::fail(GOOFY_ERR_INVALID, "noalloc: null pointer");
    if ((uint64_t)im.stride < 4ull * im.width) return goofy_gpu::fail(GOOFY_ERR_INVALID, "noalloc: stride");
    const uintptr_t s = reinterpret_cast<uintptr_t>(im.src);
    if (reinterpret_cast<uintptr_t>(im.dst) % 8 || s % 4 || im.stride % 4)
        return goofy_gpu::fail(GOOFY_ERR_ALIGNMENT, "noalloc: alignment");
    d->src = static_cast<const uint8_t*>(im.src);
    d->dst = static_cast<uint8_t*>(im.dst);
    d->stride = im.stride;
    d->bw = (uint32_t)bw;
    d->bh = (uint32_t)bh;
    d->bw_magic = 0xffffffffu / (uint32_t)bw;
    d->codec = (uint32_t)im.codec;
    d->vec16 = (s % 16 == 0 && im.stride % 16 == 0) ? 1u : 0u;
    *units += (bw * bh + unit_blocks - 1) / unit_blocks;
    if (*units > 0x7fffffffull) return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "noalloc: too many work units");
    return GOOFY_OK;
}

}  // namespace

extern "C" GOOFY_EXPORT int goofy_gpu_batch_encode_noalloc(const goofy_gpu_image* images, uint32_t count,
                                                           void* stream)
{
    if (count > kMaxImages) {
        char msg[128];
        std::snprintf(msg, sizeof msg, "goofy_gpu_batch_encode_noalloc: at most %u images per call, got %u",
                      kMaxImages, count);
        return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, msg);
    }
    if (count == 0) return GOOFY_OK;
    if (!images) return GOOFY_ERR_INVALID;
    const goofy_gpu::BatchTile tile{128, 1, 256};
    // Host copies of the tables live on this thread's stack (13 KB).
    goofy_gpu::BatchImage desc[kMaxImages];
    uint32_t first[kMaxImages];
    uint64_t units = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const int rc = describe(images[i], tile.unit_blocks, &units, &desc[i]);
        if (rc != GOOFY_OK) return rc;
        first[i] = desc[i].first_unit;
    }
    if (units == 0) return GOOFY_OK;
    Scratch* s = nullptr;
    const int rc = scratch_address(&s);
    if (rc != GOOFY_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // Pageable source: each copy returns once the bytes are staged, so the
    // stack tables may go out of scope right after.
    GOOFY_CUDA_TRY(cudaMemcpyAsync(s->images, desc, sizeof(goofy_gpu::BatchImage) * count, cudaMemcpyHostToDevice, st));
    GOOFY_CUDA_TRY(cudaMemcpyAsync(s->first_unit, first, sizeof(uint32_t) * count, cudaMemcpyHostToDevice, st));
    // The previous call left its final count in the work counter: clear it.
    GOOFY_CUDA_TRY(cudaMemsetAsync(&s->work_counter, 0, sizeof(uint32_t), st));
    const uint64_t needed = (units * 32 + tile.threads - 1) / tile.threads;
    const uint64_t resident = (uint64_t)goofy_gpu::batch_resident_ctas(tile.threads, tile.bpt);
    const uint32_t ctas = (uint32_t)(needed < resident ? needed : resident);
    GOOFY_CUDA_TRY(goofy_gpu::launch_batch(s->images, count, s->first_unit, (uint32_t)units, &s->work_counter, tile,
                                           ctas, st));
    return GOOFY_OK;
}
