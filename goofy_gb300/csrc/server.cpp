// server.cpp -- continuous-batching request server for host-memory encode
// requests (no reference counterpart: the reference is a synchronous
// function, GoofyTC/goofy_tc.h:1497-1557).
//
// Clients submit requests (host src / dst, size, codec) from any thread and get
// a ticket.  One scheduler thread
//   * admits waiting requests in arrival order while they fit the device
//     budget (staged mode: a ring arena of device memory allocated once;
//     direct mode: bytes of requests in flight),
//   * folds every admitted request that is not yet running into the next
//     launch of the persistent batch kernel, as soon as a launch slot is free
//     -- requests that arrive while others run join the following launch, so
//     copies of one batch overlap the kernel and read-back of the previous,
//   * staged mode: per request one host->device copy into the arena (copy
//     stream), the batch kernel over the arena (compute stream), one
//     device->host copy per request (read-back stream);
//     direct mode: the batch kernel reads the request's pinned source and
//     writes its pinned destination itself over NVLink-C2C (one launch, no
//     copy calls),
//   * with config.quality, decodes each launch's fresh blocks on the GPU and
//     sums the harness's squared errors per request (same work units, one
//     more launch), so every request also gets its RGB PSNR,
//   * releases arena space and launch slots when a launch's completion
//     callback fires (cudaLaunchHostFunc), which also timestamps the requests
//     -- or, with config.completion = EVENT, when a thread of the server that
//     waits on each launch's last event in turn sees it complete.
// A batch of size 1 with one launch slot is the plain one-request-per-launch
// loop, used as the baseline.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/goofy_gpu.h"
#include "batch.h"
#include "decode.h"
#include "host_util.h"

using goofy_gpu::BatchImage;
using goofy_gpu::BatchTile;
using goofy_gpu::cuda_fail;
using goofy_gpu::DeviceGuard;

namespace {

using Clock = std::chrono::steady_clock;

inline int64_t now_ns() { return std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now().time_since_epoch()).count(); }

constexpr size_t kAlign = 256;
inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

enum ReqState : int { kFree = 0, kQueued = 1, kAdmitted = 2, kRunning = 3, kDone = 4 };

struct Request {
    uint64_t ticket = 0;
    goofy_gpu_request req{};
    size_t in_bytes = 0, out_bytes = 0, dpitch = 0;  // staged layout
    size_t arena_off = 0;
    size_t charge = 0;  // bytes counted against the budget
    int status = GOOFY_OK;
    int state = kFree;
    int64_t t_submit = 0, t_admit = 0, t_launch = 0, t_done = 0;
    double psnr_rgb = 0.0;
};

// Device memory handed out in arrival order and returned roughly in order.
class RingArena {
  public:
    void init(size_t cap) { cap_ = cap; }
    size_t capacity() const { return cap_; }
    bool alloc(size_t n, size_t* off)
    {
        if (n == 0 || n > cap_) return false;
        if (live_.empty()) head_ = tail_ = 0;
        if (!live_.empty() && head_ == tail_) return false;  // full
        if (live_.empty() || head_ > tail_) {
            if (cap_ - head_ >= n) {
                *off = head_;
            } else if (tail_ >= n) {
                *off = 0;  // wrap; the end of the buffer stays unused this lap
            } else {
                return false;
            }
        } else {  // head_ < tail_: free space is [head_, tail_)
            if (tail_ - head_ < n) return false;
            *off = head_;
        }
        head_ = *off + n;
        live_.push_back({*off, n, false});
        if (live_.size() == 1) tail_ = *off;
        return true;
    }
    void release(size_t off)
    {
        for (auto& a : live_)
            if (a.off == off && !a.freed) {
                a.freed = true;
                break;
            }
        while (!live_.empty() && live_.front().freed) live_.pop_front();
        if (live_.empty()) head_ = tail_ = 0;
        else tail_ = live_.front().off;
    }

  private:
    struct A {
        size_t off, size;
        bool freed;
    };
    std::deque<A> live_;
    size_t cap_ = 0, head_ = 0, tail_ = 0;
};

struct CallbackArg {
    goofy_gpu_server* s;
    int slot;
};

struct LaunchSlot {
    BatchImage* h_desc = nullptr;
    uint32_t* h_first = nullptr;
    BatchImage* d_desc = nullptr;
    uint32_t* d_first = nullptr;
    uint32_t* d_counter = nullptr;
    unsigned long long* d_qsums = nullptr;  // quality: 6 error sums per request
    unsigned long long* h_qsums = nullptr;
    cudaEvent_t ev_in = nullptr, ev_kernel = nullptr;
    cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;        // timing events around the batch kernel
    cudaEvent_t ev_first = nullptr, ev_last = nullptr;  // before its first and after its last GPU operation
    int64_t t_enqueue = 0;                              // start of this launch's enqueue (host clock)
    int64_t t_callback = 0;                             // its completion callback (host clock)
    uint64_t enqueue_ns = 0;                            // the scheduler's time enqueueing it
    std::vector<uint64_t> tickets;
    bool busy = false;
};

}  // namespace

struct goofy_gpu_server {
    goofy_gpu_server_config cfg{};
    BatchTile tile{128, 1, 256};
    std::mutex mu;
    std::condition_variable cv_sched, cv_done, cv_poll;
    std::thread sched, poller;
    bool stop = false;
    bool stop_poller = false;
    std::deque<int> polling;  // COMPLETION_EVENT: launch slots in flight, in launch order

    std::vector<Request> pool;  // ring of request records, indexed by ticket % size
    uint64_t next_ticket = 1;
    std::deque<uint64_t> waiting;    // submitted, not admitted (arrival order)
    std::vector<uint64_t> admitted;  // admitted, not launched
    std::vector<int> finished_slots; // launch slots whose completion callback fired

    uint8_t* arena_mem = nullptr;
    RingArena arena;
    size_t inflight_bytes = 0;

    cudaStream_t s_copy = nullptr, s_compute = nullptr, s_back = nullptr;
    std::vector<LaunchSlot> slots;
    std::vector<CallbackArg> cbs;  // completion-callback arguments, one per slot
    int resident_ctas = 0;
    bool pageable_ok = false;      // the GPU reads pageable host memory (direct mode)

    // stats
    uint64_t n_launches = 0, n_requests_done = 0, max_batch = 0, pixels_done = 0;
    uint64_t max_enqueue_ns = 0, max_kernel_ns = 0, max_launch_ns = 0;  // since the last stats read
    uint64_t slowest_enqueue_ns = 0, slowest_gpu_span_ns = 0, slowest_kernel_ns = 0;  // of the max_launch_ns one
    int error = GOOFY_OK;

    Request& rec(uint64_t t) { return pool[t % pool.size()]; }
};

namespace {

// A launch finished at host time t: stamp its requests and hand the slot to
// the scheduler (lock held).
void finish_launch_locked(goofy_gpu_server* s, int slot, int64_t t)
{
    LaunchSlot& sl = s->slots[slot];
    for (uint64_t tk : sl.tickets) s->rec(tk).t_done = t;
    sl.t_callback = t;
    s->finished_slots.push_back(slot);
}

void CUDART_CB on_launch_done(void* p)
{
    CallbackArg* a = static_cast<CallbackArg*>(p);
    goofy_gpu_server* s = a->s;
    const int64_t t = now_ns();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        finish_launch_locked(s, a->slot, t);
    }
    s->cv_sched.notify_one();
}

// Scheduler-thread work with the lock held: retire finished launches.
void retire_locked(goofy_gpu_server* s)
{
    for (int si : s->finished_slots) {
        LaunchSlot& sl = s->slots[si];
        // timing of the finished launch (CUDA calls are not allowed in the callback, so here)
        float k_ms = 0.f, span_ms = 0.f;
        if (cudaEventElapsedTime(&k_ms, sl.ev_k0, sl.ev_k1) != cudaSuccess ||
            cudaEventElapsedTime(&span_ms, sl.ev_first, sl.ev_last) != cudaSuccess)
            cudaGetLastError();
        const uint64_t kernel_ns = (uint64_t)(k_ms * 1e6f), total_ns = (uint64_t)(sl.t_callback - sl.t_enqueue);
        s->max_kernel_ns = std::max(s->max_kernel_ns, kernel_ns);
        if (total_ns > s->max_launch_ns) {
            s->max_launch_ns = total_ns;
            s->slowest_enqueue_ns = sl.enqueue_ns;
            s->slowest_gpu_span_ns = (uint64_t)(span_ms * 1e6f);
            s->slowest_kernel_ns = kernel_ns;
        }
        for (size_t i = 0; i < sl.tickets.size(); ++i) {
            Request& r = s->rec(sl.tickets[i]);
            if (s->cfg.quality) {
                // getPSNR(mseRGB, 768), Src/main.cpp:386-395, :455, :466
                const unsigned long long* q = sl.h_qsums + 6 * i;
                const double mse = (double)(q[0] + q[1] + q[2]) / ((double)r.req.width * (double)r.req.height);
                r.psnr_rgb = mse < 0.0000001 ? DBL_MAX : 10.0 * std::log10((768.0 * 768.0) / mse);
            }
            if (s->cfg.mode == GOOFY_SERVER_STAGED) s->arena.release(r.arena_off);
            s->inflight_bytes -= r.charge;
            r.state = kDone;
            r.status = GOOFY_OK;
            ++s->n_requests_done;
            s->pixels_done += (uint64_t)r.req.width * r.req.height;
        }
        sl.tickets.clear();
        sl.busy = false;
    }
    if (!s->finished_slots.empty()) s->cv_done.notify_all();
    s->finished_slots.clear();
}

// Admit waiting requests in arrival order while they fit.
void admit_locked(goofy_gpu_server* s)
{
    while (!s->waiting.empty() && s->admitted.size() < s->cfg.max_batch_images) {
        Request& r = s->rec(s->waiting.front());
        if (s->cfg.mode == GOOFY_SERVER_STAGED) {
            size_t off = 0;
            if (!s->arena.alloc(r.charge, &off)) break;
            r.arena_off = off;
        } else {
            if (s->inflight_bytes + r.charge > s->cfg.device_budget_bytes) break;
        }
        s->inflight_bytes += r.charge;
        r.state = kAdmitted;
        r.t_admit = now_ns();
        s->admitted.push_back(r.ticket);
        s->waiting.pop_front();
    }
}

int free_slot_locked(goofy_gpu_server* s)
{
    for (size_t i = 0; i < s->slots.size(); ++i)
        if (!s->slots[i].busy) return (int)i;
    return -1;
}

// Build and enqueue one launch for `tickets` on slot `si` (lock NOT held;
// the tickets' records are owned by the scheduler until completion).
int launch(goofy_gpu_server* s, int si, const std::vector<uint64_t>& tickets, CallbackArg* cb)
{
    LaunchSlot& sl = s->slots[si];
    const bool staged = s->cfg.mode == GOOFY_SERVER_STAGED;
    uint64_t units = 0;
    const uint32_t n = (uint32_t)tickets.size();
    const int64_t t = now_ns();
    sl.t_enqueue = t;
    for (uint32_t i = 0; i < n; ++i) {
        Request& r = s->rec(tickets[i]);
        r.t_launch = t;
        const goofy_gpu_request& q = r.req;
        BatchImage& d = sl.h_desc[i];
        std::memset(&d, 0, sizeof d);
        const uint32_t bw = q.width / 4, bh = q.height / 4;
        d.bw = bw;
        d.bh = bh;
        d.bw_magic = 0xffffffffu / (bw ? bw : 1);
        d.codec = (uint32_t)q.codec;
        d.first_unit = (uint32_t)units;
        sl.h_first[i] = (uint32_t)units;
        if (staged) {
            d.src = s->arena_mem + r.arena_off;
            d.dst = s->arena_mem + r.arena_off + r.in_bytes;
            d.stride = (uint32_t)r.dpitch;
            d.vec16 = 1;
        } else {
            d.src = q.src;
            d.dst = q.dst;
            d.stride = q.stride;
            d.vec16 = (reinterpret_cast<uintptr_t>(q.src) % 16 == 0 && q.stride % 16 == 0) ? 1u : 0u;
        }
        units += ((uint64_t)bw * bh + s->tile.unit_blocks - 1) / s->tile.unit_blocks;
    }
    GOOFY_CUDA_TRY(cudaEventRecord(sl.ev_first, staged ? s->s_copy : s->s_compute));
    if (staged) {
        for (uint64_t tk : tickets) {
            Request& r = s->rec(tk);
            const goofy_gpu_request& q = r.req;
            GOOFY_CUDA_TRY(cudaMemcpy2DAsync(s->arena_mem + r.arena_off, r.dpitch, q.src, q.stride, 4ull * q.width,
                                             q.height, cudaMemcpyHostToDevice, s->s_copy));
        }
        GOOFY_CUDA_TRY(cudaEventRecord(sl.ev_in, s->s_copy));
        GOOFY_CUDA_TRY(cudaStreamWaitEvent(s->s_compute, sl.ev_in, 0));
    }
    GOOFY_CUDA_TRY(cudaMemcpyAsync(sl.d_desc, sl.h_desc, sizeof(BatchImage) * n, cudaMemcpyHostToDevice, s->s_compute));
    GOOFY_CUDA_TRY(cudaMemcpyAsync(sl.d_first, sl.h_first, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s->s_compute));
    GOOFY_CUDA_TRY(cudaMemsetAsync(sl.d_counter, 0, sizeof(uint32_t), s->s_compute));
    const uint32_t ctas = (uint32_t)std::min<uint64_t>((uint64_t)s->resident_ctas,
                                                       (units * 32 + s->tile.threads - 1) / s->tile.threads);
    GOOFY_CUDA_TRY(cudaEventRecord(sl.ev_k0, s->s_compute));
    GOOFY_CUDA_TRY(goofy_gpu::launch_batch(sl.d_desc, n, sl.d_first, (uint32_t)units, sl.d_counter, s->tile,
                                           ctas ? ctas : 1, s->s_compute));
    GOOFY_CUDA_TRY(cudaEventRecord(sl.ev_k1, s->s_compute));
    if (s->cfg.quality) {  // decode the fresh blocks and compare with each request's source, same units
        GOOFY_CUDA_TRY(cudaMemsetAsync(sl.d_qsums, 0, 6 * sizeof(unsigned long long) * n, s->s_compute));
        GOOFY_CUDA_TRY(cudaMemsetAsync(sl.d_counter, 0, sizeof(uint32_t), s->s_compute));
        GOOFY_CUDA_TRY(goofy_gpu::launch_quality_batch(sl.d_desc, n, sl.d_first, (uint32_t)units, s->tile.unit_blocks,
                                                       sl.d_counter, sl.d_qsums, s->s_compute));
        GOOFY_CUDA_TRY(cudaMemcpyAsync(sl.h_qsums, sl.d_qsums, 6 * sizeof(unsigned long long) * n,
                                       cudaMemcpyDeviceToHost, s->s_compute));
    }
    cudaStream_t last = s->s_compute;
    if (staged) {
        GOOFY_CUDA_TRY(cudaEventRecord(sl.ev_kernel, s->s_compute));
        GOOFY_CUDA_TRY(cudaStreamWaitEvent(s->s_back, sl.ev_kernel, 0));
        for (uint64_t tk : tickets) {
            Request& r = s->rec(tk);
            GOOFY_CUDA_TRY(cudaMemcpyAsync(r.req.dst, s->arena_mem + r.arena_off + r.in_bytes,
                                           (size_t)(r.req.width / 4) * (r.req.height / 4) * 8,
                                           cudaMemcpyDeviceToHost, s->s_back));
        }
        last = s->s_back;
    }
    GOOFY_CUDA_TRY(cudaEventRecord(sl.ev_last, last));
    const bool poll = s->cfg.completion == GOOFY_SERVER_COMPLETION_EVENT;  // a server thread waits on ev_last
    if (!poll) GOOFY_CUDA_TRY(cudaLaunchHostFunc(last, on_launch_done, cb));
    const uint64_t enq = (uint64_t)(now_ns() - t);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        sl.enqueue_ns = enq;  // the scheduler retires this launch only after launch() returns
        s->max_enqueue_ns = std::max(s->max_enqueue_ns, enq);
        if (poll) s->polling.push_back(cb->slot);
    }
    if (poll) s->cv_poll.notify_one();
    return GOOFY_OK;
}

// COMPLETION_EVENT: waits for the launches in flight in launch order (they
// finish in that order: each stream runs its part of the launches in turn)
// on each one's last event, a blocking-sync event: the thread sleeps until
// the GPU has passed it.
void poller_main(goofy_gpu_server* s)
{
    cudaSetDevice(s->cfg.device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        if (s->polling.empty()) {
            if (s->stop_poller) break;
            s->cv_poll.wait_for(lk, std::chrono::milliseconds(2));
            continue;
        }
        const int si = s->polling.front();
        const cudaEvent_t ev = s->slots[si].ev_last;
        lk.unlock();
        if (cudaEventSynchronize(ev) != cudaSuccess) cudaGetLastError();  // a failed launch still releases its slot
        const int64_t t = now_ns();
        lk.lock();
        s->polling.pop_front();
        finish_launch_locked(s, si, t);
        s->cv_sched.notify_one();
    }
}

void scheduler_main(goofy_gpu_server* s)
{
    cudaSetDevice(s->cfg.device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        retire_locked(s);
        admit_locked(s);
        if (s->stop && s->waiting.empty() && s->admitted.empty()) {
            bool idle = true;
            for (auto& sl : s->slots) idle = idle && !sl.busy;
            if (idle) break;
        }
        const int si = s->admitted.empty() ? -1 : free_slot_locked(s);
        if (si >= 0) {
            std::vector<uint64_t> batch;
            batch.swap(s->admitted);
            for (uint64_t tk : batch) s->rec(tk).state = kRunning;
            LaunchSlot& sl = s->slots[si];
            sl.busy = true;
            sl.tickets = batch;
            s->max_batch = std::max<uint64_t>(s->max_batch, batch.size());
            ++s->n_launches;
            lk.unlock();
            const int rc = launch(s, si, batch, &s->cbs[si]);
            lk.lock();
            if (rc != GOOFY_OK) {  // the launch did not go out: fail its requests
                for (uint64_t tk : batch) {
                    Request& r = s->rec(tk);
                    if (s->cfg.mode == GOOFY_SERVER_STAGED) s->arena.release(r.arena_off);
                    s->inflight_bytes -= r.charge;
                    r.state = kDone;
                    r.status = rc;
                    r.t_done = now_ns();
                }
                sl.tickets.clear();
                sl.busy = false;
                s->error = rc;
                s->cv_done.notify_all();
            }
            continue;
        }
        s->cv_sched.wait_for(lk, std::chrono::milliseconds(2));
    }
}

int init_server(goofy_gpu_server* s)
{
    const goofy_gpu_server_config& c = s->cfg;
    DeviceGuard g(c.device);
    GOOFY_CUDA_TRY(g.err);
    GOOFY_CUDA_TRY(cudaStreamCreateWithFlags(&s->s_compute, cudaStreamNonBlocking));
    if (c.mode == GOOFY_SERVER_STAGED) {
        GOOFY_CUDA_TRY(cudaStreamCreateWithFlags(&s->s_copy, cudaStreamNonBlocking));
        GOOFY_CUDA_TRY(cudaStreamCreateWithFlags(&s->s_back, cudaStreamNonBlocking));
        GOOFY_CUDA_TRY(cudaMalloc(&s->arena_mem, c.device_budget_bytes));
        // Write the whole arena once before serving.  Without this, right after a fresh allocation
        // of this size the copies of the first requests stalled for 25-90 ms in about one server
        // in four (staged mode only, whose requests go through the copy engines); with it, none
        // in eight.
        GOOFY_CUDA_TRY(cudaMemsetAsync(s->arena_mem, 0, c.device_budget_bytes, s->s_copy));
        GOOFY_CUDA_TRY(cudaStreamSynchronize(s->s_copy));
        s->arena.init(c.device_budget_bytes);
    }
    int pageable = 0;
    GOOFY_CUDA_TRY(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c.device));
    s->pageable_ok = pageable != 0;
    s->slots.resize(c.max_inflight_batches);
    s->cbs.resize(c.max_inflight_batches);
    for (uint32_t i = 0; i < c.max_inflight_batches; ++i) {
        LaunchSlot& sl = s->slots[i];
        s->cbs[i] = CallbackArg{s, (int)i};
        GOOFY_CUDA_TRY(cudaHostAlloc(&sl.h_desc, sizeof(BatchImage) * c.max_batch_images, cudaHostAllocDefault));
        GOOFY_CUDA_TRY(cudaHostAlloc(&sl.h_first, sizeof(uint32_t) * c.max_batch_images, cudaHostAllocDefault));
        GOOFY_CUDA_TRY(cudaMalloc(&sl.d_desc, sizeof(BatchImage) * c.max_batch_images));
        GOOFY_CUDA_TRY(cudaMalloc(&sl.d_first, sizeof(uint32_t) * c.max_batch_images));
        GOOFY_CUDA_TRY(cudaMalloc(&sl.d_counter, sizeof(uint32_t)));
        if (c.quality) {
            GOOFY_CUDA_TRY(cudaMalloc(&sl.d_qsums, 6 * sizeof(unsigned long long) * c.max_batch_images));
            GOOFY_CUDA_TRY(cudaHostAlloc(&sl.h_qsums, 6 * sizeof(unsigned long long) * c.max_batch_images,
                                         cudaHostAllocDefault));
        }
        GOOFY_CUDA_TRY(cudaEventCreateWithFlags(&sl.ev_in, cudaEventDisableTiming));
        GOOFY_CUDA_TRY(cudaEventCreateWithFlags(&sl.ev_kernel, cudaEventDisableTiming));
        GOOFY_CUDA_TRY(cudaEventCreate(&sl.ev_k0));
        GOOFY_CUDA_TRY(cudaEventCreate(&sl.ev_k1));
        GOOFY_CUDA_TRY(cudaEventCreate(&sl.ev_first));
        GOOFY_CUDA_TRY(cudaEventCreateWithFlags(&sl.ev_last, cudaEventBlockingSync));
    }
    s->resident_ctas = goofy_gpu::batch_resident_ctas(s->tile.threads, s->tile.bpt);
    s->pool.resize(c.max_requests);
    return GOOFY_OK;
}

void teardown(goofy_gpu_server* s)
{
    DeviceGuard g(s->cfg.device);
    for (cudaStream_t st : {s->s_copy, s->s_compute, s->s_back})
        if (st) cudaStreamSynchronize(st);
    for (auto& sl : s->slots) {
        if (sl.h_desc) cudaFreeHost(sl.h_desc);
        if (sl.h_first) cudaFreeHost(sl.h_first);
        if (sl.d_desc) cudaFree(sl.d_desc);
        if (sl.d_first) cudaFree(sl.d_first);
        if (sl.d_counter) cudaFree(sl.d_counter);
        if (sl.d_qsums) cudaFree(sl.d_qsums);
        if (sl.h_qsums) cudaFreeHost(sl.h_qsums);
        if (sl.ev_in) cudaEventDestroy(sl.ev_in);
        if (sl.ev_kernel) cudaEventDestroy(sl.ev_kernel);
        if (sl.ev_k0) cudaEventDestroy(sl.ev_k0);
        if (sl.ev_k1) cudaEventDestroy(sl.ev_k1);
        if (sl.ev_first) cudaEventDestroy(sl.ev_first);
        if (sl.ev_last) cudaEventDestroy(sl.ev_last);
    }
    if (s->arena_mem) cudaFree(s->arena_mem);
    for (cudaStream_t st : {s->s_copy, s->s_compute, s->s_back})
        if (st) cudaStreamDestroy(st);
}

}  // namespace

extern "C" {

GOOFY_EXPORT void goofy_gpu_server_default_config(goofy_gpu_server_config* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->device = 0;
    c->mode = GOOFY_SERVER_STAGED;
    c->device_budget_bytes = 16ull << 30;
    c->max_batch_images = 1024;
    c->max_inflight_batches = 4;
    c->max_requests = 1u << 20;
}

GOOFY_EXPORT int goofy_gpu_server_create(goofy_gpu_server** out, const goofy_gpu_server_config* cfg)
{
    if (!out || !cfg) return GOOFY_ERR_INVALID;
    *out = nullptr;
    if (cfg->mode != GOOFY_SERVER_STAGED && cfg->mode != GOOFY_SERVER_DIRECT) return GOOFY_ERR_INVALID;
    if (cfg->quality > 1 || cfg->completion > GOOFY_SERVER_COMPLETION_EVENT) return GOOFY_ERR_INVALID;
    if (cfg->device_budget_bytes < (1u << 20) || cfg->max_batch_images == 0 || cfg->max_batch_images > 65536 ||
        cfg->max_inflight_batches == 0 || cfg->max_inflight_batches > 64 || cfg->max_requests < 16)
        return GOOFY_ERR_INVALID;
    int n = 0;
    GOOFY_CUDA_TRY(cudaGetDeviceCount(&n));
    if (cfg->device < 0 || cfg->device >= n) return GOOFY_ERR_NO_DEVICE;
    goofy_gpu_server* s = new (std::nothrow) goofy_gpu_server();
    if (!s) return GOOFY_ERR_NOMEM;
    s->cfg = *cfg;
    s->cfg.device_budget_bytes = round_up(cfg->device_budget_bytes, kAlign);
    const int rc = init_server(s);
    if (rc != GOOFY_OK) {
        teardown(s);
        delete s;
        return rc;
    }
    if (s->cfg.completion == GOOFY_SERVER_COMPLETION_EVENT) s->poller = std::thread(poller_main, s);
    s->sched = std::thread(scheduler_main, s);
    *out = s;
    return GOOFY_OK;
}

GOOFY_EXPORT void goofy_gpu_server_destroy(goofy_gpu_server* s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_sched.notify_all();
    if (s->sched.joinable()) s->sched.join();  // returns once every launch has completed
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop_poller = true;
    }
    s->cv_poll.notify_all();
    if (s->poller.joinable()) s->poller.join();
    teardown(s);
    delete s;
}

GOOFY_EXPORT int goofy_gpu_server_submit(goofy_gpu_server* s, const goofy_gpu_request* q, uint64_t* ticket)
{
    if (!s || !q || !ticket) return GOOFY_ERR_INVALID;
    if (q->codec != GOOFY_CODEC_BC1 && q->codec != GOOFY_CODEC_ETC1S) return GOOFY_ERR_INVALID;
    if (q->width % 4) return GOOFY_ERR_WIDTH;
    if (q->height % 4) return GOOFY_ERR_HEIGHT;
    if (q->width == 0 || q->height == 0 || !q->src || !q->dst) return GOOFY_ERR_INVALID;
    if ((uint64_t)q->stride < 4ull * q->width) return GOOFY_ERR_INVALID;
    if ((uint64_t)(q->width / 4) * (q->height / 4) > 0x7fffffffull) return GOOFY_ERR_TOO_LARGE;
    const bool staged = s->cfg.mode == GOOFY_SERVER_STAGED;
    if (!staged) {
        if (reinterpret_cast<uintptr_t>(q->dst) % 8 || reinterpret_cast<uintptr_t>(q->src) % 4 || q->stride % 4)
            return GOOFY_ERR_ALIGNMENT;
        if (!s->pageable_ok) {  // the kernel touches the buffers itself: they must be GPU-accessible
            for (const void* p : {(const void*)q->src, (const void*)q->dst}) {
                cudaPointerAttributes a;
                if (cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type == cudaMemoryTypeUnregistered) {
                    cudaGetLastError();
                    return goofy_gpu::fail(GOOFY_ERR_INVALID, "server: direct mode needs pinned buffers on this GPU");
                }
            }
        }
    }
    const size_t dpitch = round_up(4ull * q->width, 16);
    const size_t in_bytes = round_up(dpitch * q->height, kAlign);
    const size_t out_bytes = round_up((size_t)(q->width / 4) * (q->height / 4) * 8, kAlign);
    const size_t charge = staged ? in_bytes + out_bytes : (size_t)q->stride * q->height + out_bytes;
    if (charge > s->cfg.device_budget_bytes) return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "server: request exceeds the budget");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->error != GOOFY_OK) return s->error;
    Request& r = s->rec(s->next_ticket);
    if (r.state != kFree) return goofy_gpu::fail(GOOFY_ERR_BUSY, "server: too many unreleased tickets");
    r = Request{};
    r.ticket = s->next_ticket++;
    r.req = *q;
    r.dpitch = dpitch;
    r.in_bytes = in_bytes;
    r.out_bytes = out_bytes;
    r.charge = charge;
    r.state = kQueued;
    r.t_submit = now_ns();
    s->waiting.push_back(r.ticket);
    *ticket = r.ticket;
    s->cv_sched.notify_one();
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_server_wait(goofy_gpu_server* s, uint64_t ticket, uint32_t timeout_ms,
                                       goofy_gpu_request_times* times)
{
    if (!s || ticket == 0) return GOOFY_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    Request& r = s->rec(ticket);
    if (r.ticket != ticket || r.state == kFree) return GOOFY_ERR_INVALID;
    const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r.state == kDone; });
    if (!ok) return GOOFY_ERR_TIMEOUT;
    if (times) {
        times->submit_ns = r.t_submit;
        times->admit_ns = r.t_admit;
        times->launch_ns = r.t_launch;
        times->done_ns = r.t_done;
        times->psnr_rgb = r.psnr_rgb;
    }
    const int status = r.status;
    r.state = kFree;  // the ticket is released
    return status;
}

GOOFY_EXPORT int goofy_gpu_server_get_stats(goofy_gpu_server* s, goofy_gpu_server_stats* st)
{
    if (!s || !st) return GOOFY_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    st->launches = s->n_launches;
    st->requests_done = s->n_requests_done;
    st->pixels_done = s->pixels_done;
    st->max_batch = s->max_batch;
    st->waiting = s->waiting.size();
    st->inflight_bytes = s->inflight_bytes;
    st->max_enqueue_ns = s->max_enqueue_ns;
    st->max_kernel_ns = s->max_kernel_ns;
    st->max_launch_ns = s->max_launch_ns;
    st->slowest_enqueue_ns = s->slowest_enqueue_ns;
    st->slowest_gpu_span_ns = s->slowest_gpu_span_ns;
    st->slowest_kernel_ns = s->slowest_kernel_ns;
    s->max_enqueue_ns = s->max_kernel_ns = s->max_launch_ns = 0;
    s->slowest_enqueue_ns = s->slowest_gpu_span_ns = s->slowest_kernel_ns = 0;
    return GOOFY_OK;
}

GOOFY_EXPORT int64_t goofy_gpu_now_ns(void) { return now_ns(); }

}  // extern "C"
