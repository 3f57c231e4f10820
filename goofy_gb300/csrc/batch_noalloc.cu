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
// buffers.
//
// A call is two launches on the caller's stream: a one-CTA kernel that takes
// the call's descriptor and first-unit tables as its by-value parameter,
// writes them into the array and zeroes the work counter; then the ordinary
// batch kernel, given pointers into the array.  No host-to-device copy is
// made, so nothing is read from the calling thread's memory after the call
// returns.
#include <cuda.h>  // driver types for the context queries (entry points fetched at run time)
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

// A call's tables as a kernel parameter: N descriptors and first units
// (13,312 bytes for N = 256, within the 32,764-byte parameter limit).  Small
// calls use the 32-image form, whose launch carries 1.7 KB.
template <uint32_t N>
struct Tables {
    goofy_gpu::BatchImage images[N];
    uint32_t first_unit[N];
};

template <uint32_t N>
__global__ void __launch_bounds__(256) noalloc_stage_kernel(const __grid_constant__ Tables<N> t, uint32_t count)
{
    Scratch* s = reinterpret_cast<Scratch*>(g_noalloc_scratch);
    for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
        s->images[i] = t.images[i];
        s->first_unit[i] = t.first_unit[i];
    }
    if (threadIdx.x == 0) s->work_counter = 0u;  // the previous call left its final count here
}

// Unique id of the calling thread's current context (0 when none is current
// or the driver lacks the queries).  Context ids are never reused within a
// process, unlike context handles.
unsigned long long current_context_id()
{
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(p);
        cudaGetLastError();
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

constexpr int kMaxDevices = 64;
struct Resolved {
    unsigned long long context_id = 0;
    Scratch* addr = nullptr;
};
std::mutex g_setup_mu;
Resolved g_resolved[kMaxDevices];

// Device address of the scratch array in the current device's context.  The
// first call in a context asks the runtime for it (cudaGetSymbolAddress) and
// keeps it with that context's id; a later call in the same context reuses
// it.  A reset device (cudaDeviceReset) or another context made current gets
// a new id, so the address is looked up again instead of reusing one that
// belongs to a destroyed or different context.
int scratch_address(Scratch** out)
{
    int dev = 0;
    GOOFY_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return goofy_gpu::fail(GOOFY_ERR_NO_DEVICE, "noalloc: device index too large");
    unsigned long long id = current_context_id();
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (id != 0 && g_resolved[dev].context_id == id) {
            *out = g_resolved[dev].addr;
            return GOOFY_OK;
        }
    }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // makes the primary context current if none is
    if (e != cudaSuccess || !p) return goofy_gpu::cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
    id = current_context_id();
    std::lock_guard<std::mutex> lk(g_setup_mu);
    g_resolved[dev].context_id = id;  // 0 (no context queries): looked up again on every call
    g_resolved[dev].addr = static_cast<Scratch*>(p);
    *out = g_resolved[dev].addr;
    return GOOFY_OK;
}

// Validates the images into tables of N entries, then (if there is work)
// launches the staging kernel and the batch kernel on `st`.
template <uint32_t N>
int encode_with(const goofy_gpu_image* images, uint32_t count, cudaStream_t st)
{
    const goofy_gpu::BatchTile tile{128, 1, 256, 0};
    Tables<N> t;  // on this thread's stack; the launch copies it
    std::memset(&t, 0, sizeof t);
    uint32_t units = 0;
    int rc = goofy_gpu::validate_and_fill(images, count, tile.unit_blocks, t.images, t.first_unit, &units);
    if (rc != GOOFY_OK || units == 0) return rc;  // nothing launched for an invalid or empty batch
    Scratch* s = nullptr;
    if ((rc = scratch_address(&s)) != GOOFY_OK) return rc;
    noalloc_stage_kernel<N><<<1, 256, 0, st>>>(t, count);
    GOOFY_CUDA_TRY(cudaGetLastError());
    const uint64_t needed = ((uint64_t)units * 32 + tile.threads - 1) / tile.threads;
    const uint64_t resident = (uint64_t)goofy_gpu::batch_resident_ctas(tile.threads, tile.bpt);
    const uint32_t ctas = (uint32_t)(needed < resident ? needed : resident);
    GOOFY_CUDA_TRY(goofy_gpu::launch_batch(s->images, count, s->first_unit, units, &s->work_counter, tile, ctas, st));
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
    if (!images) return goofy_gpu::fail(GOOFY_ERR_INVALID, "goofy_gpu_batch_encode_noalloc: images is NULL");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return count <= 32 ? encode_with<32>(images, count, st) : encode_with<kMaxImages>(images, count, st);
}
