// backend.cu -- gpis_backend_*: the asynchronous batch backend
// (GpRayBatchBackend::submitBatch, GpRayBatchBackend.hpp:43-55, as
// SeBatchBackend implements it in PathTracerSeBatchBackend.cpp:358-397).
//
// One dispatcher thread per backend takes submitted batches in order.  Each
// batch is copied at submission into host memory the backend owns; the
// dispatcher stages it in pinned memory, copies it to the device, enqueues the
// flight kernels (gpis_flights_submit) and the copy of the results back on the
// backend's stream, then a host function on that stream copies the records to
// the caller's buffer and calls its done callback.  Two staging slots let the
// dispatcher stage the next batch while the previous one runs; a slot is reused
// only after its event has completed.
#include <cuda_runtime.h>

#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gpis.h"

extern "C" int gpis_internal_set_error(int code, const char *msg);

namespace {

struct Batch {
    uint32_t n = 0;
    std::vector<float> origin_near, dir_far, prev;
    std::vector<uint32_t> seeds, medium;
    bool has_prev = false, has_medium = false;
    float *out = nullptr;
    gpis_batch_done_fn done = nullptr;
    void *user = nullptr;
};

struct Slot {
    size_t cap = 0;
    char *host = nullptr;       // pinned: in streams, then result records
    char *dev = nullptr;
    cudaEvent_t ev = nullptr;
    bool busy = false;
};

struct Completion {
    gpis_backend *backend = nullptr;
    Batch batch;
    float *host_rec = nullptr;  // pinned result records of the slot
};

}  // namespace

struct gpis_backend {
    gpis_ctx *ctx = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    Slot slots[2];
    int next_slot = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Batch> queue;
    size_t in_flight = 0;       // batches submitted and not yet completed
    bool stop = false;
    std::thread worker;
};

namespace {

void finish_one(gpis_backend *b)
{
    std::lock_guard<std::mutex> lk(b->mu);
    b->in_flight--;
    b->cv.notify_all();
}

// host function on the backend's stream: publish the records, notify, retire
void CUDART_CB complete(void *arg)
{
    Completion *c = static_cast<Completion *>(arg);
    std::memcpy(c->batch.out, c->host_rec, (size_t)c->batch.n * 32);
    if (c->batch.done) c->batch.done(c->batch.user, GPIS_OK);
    gpis_backend *b = c->backend;
    delete c;
    finish_one(b);
}

int stage_and_launch(gpis_backend *b, Batch &bt)
{
    Slot &s = b->slots[b->next_slot];
    b->next_slot ^= 1;
    if (s.busy) {
        if (cudaEventSynchronize(s.ev) != cudaSuccess) return GPIS_EIO;
        s.busy = false;
    }
    const size_t n = bt.n, r16 = n * 16;
    const size_t need = 4 * r16 + ((n * 4 + 255) & ~(size_t)255) + 2 * r16;
    if (need > s.cap) {
        cudaFreeHost(s.host);
        cudaFree(s.dev);
        s.host = nullptr;
        s.dev = nullptr;
        s.cap = 0;
        if (cudaHostAlloc(&s.host, need, cudaHostAllocDefault) != cudaSuccess) return GPIS_ENOMEM;
        if (cudaMalloc(&s.dev, need) != cudaSuccess) return GPIS_ENOMEM;
        s.cap = need;
    }
    char *h = s.host;
    std::memcpy(h, bt.origin_near.data(), r16);
    std::memcpy(h + r16, bt.dir_far.data(), r16);
    std::memcpy(h + 2 * r16, bt.seeds.data(), r16);
    if (bt.has_prev) std::memcpy(h + 3 * r16, bt.prev.data(), r16);
    else std::memset(h + 3 * r16, 0, r16);
    if (bt.has_medium) std::memcpy(h + 4 * r16, bt.medium.data(), n * 4);
    const size_t in_bytes = 4 * r16 + (bt.has_medium ? n * 4 : 0);
    const size_t rec_off = 4 * r16 + ((n * 4 + 255) & ~(size_t)255);
    if (cudaMemcpyAsync(s.dev, h, in_bytes, cudaMemcpyHostToDevice, b->stream) != cudaSuccess) return GPIS_EIO;
    gpis_flight_soa din;
    din.origin_near = reinterpret_cast<float *>(s.dev);
    din.dir_far = reinterpret_cast<float *>(s.dev + r16);
    din.seeds = reinterpret_cast<uint32_t *>(s.dev + 2 * r16);
    din.prev = reinterpret_cast<float *>(s.dev + 3 * r16);
    din.medium = bt.has_medium ? reinterpret_cast<uint32_t *>(s.dev + 4 * r16) : nullptr;
    gpis_result_soa dout;
    dout.rec = reinterpret_cast<float *>(s.dev + rec_off);
    int rc = gpis_flights_submit(b->ctx, &din, &dout, bt.n, b->stream);
    if (rc) return rc;
    if (cudaMemcpyAsync(h + rec_off, s.dev + rec_off, 2 * r16, cudaMemcpyDeviceToHost, b->stream) != cudaSuccess)
        return GPIS_EIO;
    Completion *c = new Completion;
    c->backend = b;
    c->batch = std::move(bt);
    c->host_rec = reinterpret_cast<float *>(h + rec_off);
    if (cudaLaunchHostFunc(b->stream, complete, c) != cudaSuccess) {
        bt = std::move(c->batch);
        delete c;
        return GPIS_EIO;
    }
    cudaEventRecord(s.ev, b->stream);
    s.busy = true;
    return GPIS_OK;
}

void dispatcher(gpis_backend *b)
{
    cudaSetDevice(b->device);
    for (;;) {
        Batch bt;
        {
            std::unique_lock<std::mutex> lk(b->mu);
            b->cv.wait(lk, [&] { return b->stop || !b->queue.empty(); });
            if (b->queue.empty()) return;
            bt = std::move(b->queue.front());
            b->queue.pop_front();
        }
        gpis_batch_done_fn done = bt.done;
        void *user = bt.user;
        const int rc = stage_and_launch(b, bt);
        if (rc) {
            // the batch failed before its completion was enqueued: report it here
            if (done) done(user, rc);
            finish_one(b);
        }
    }
}

}  // namespace

extern "C" int gpis_backend_create(const gpis_medium_desc *media, int n_media, gpis_backend **out)
{
    if (!out) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    *out = nullptr;
    gpis_backend *b = new gpis_backend;
    int rc = gpis_ctx_create(media, n_media, &b->ctx);
    if (rc) {
        delete b;
        return rc;
    }
    cudaGetDevice(&b->device);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->slots[0].ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->slots[1].ev, cudaEventDisableTiming) != cudaSuccess) {
        gpis_ctx_destroy(b->ctx);
        delete b;
        return gpis_internal_set_error(GPIS_EIO, "backend stream or event creation failed");
    }
    b->worker = std::thread(dispatcher, b);
    *out = b;
    return GPIS_OK;
}

extern "C" void gpis_backend_destroy(gpis_backend *b)
{
    if (!b) return;
    {
        std::unique_lock<std::mutex> lk(b->mu);
        b->cv.wait(lk, [&] { return b->in_flight == 0; });
        b->stop = true;
        b->cv.notify_all();
    }
    b->worker.join();
    cudaStreamSynchronize(b->stream);
    for (Slot &s : b->slots) {
        cudaFreeHost(s.host);
        cudaFree(s.dev);
        cudaEventDestroy(s.ev);
    }
    cudaStreamDestroy(b->stream);
    gpis_ctx_destroy(b->ctx);
    delete b;
}

extern "C" int gpis_backend_submit(gpis_backend *b, const gpis_flight_soa *in, float *out_rec, uint32_t n,
                                   gpis_batch_done_fn done, void *user)
{
    if (!b || !in || (n && !out_rec)) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    if (n && (!in->origin_near || !in->dir_far || !in->seeds))
        return gpis_internal_set_error(GPIS_EINVAL, "streams origin_near, dir_far and seeds are required");
    if (n == 0) {
        if (done) done(user, GPIS_OK);
        return GPIS_OK;
    }
    Batch bt;
    bt.n = n;
    bt.origin_near.assign(in->origin_near, in->origin_near + 4 * (size_t)n);
    bt.dir_far.assign(in->dir_far, in->dir_far + 4 * (size_t)n);
    bt.seeds.assign(in->seeds, in->seeds + 4 * (size_t)n);
    if (in->prev) {
        bt.prev.assign(in->prev, in->prev + 4 * (size_t)n);
        bt.has_prev = true;
    }
    if (in->medium) {
        bt.medium.assign(in->medium, in->medium + (size_t)n);
        bt.has_medium = true;
    }
    bt.out = out_rec;
    bt.done = done;
    bt.user = user;
    std::lock_guard<std::mutex> lk(b->mu);
    b->queue.push_back(std::move(bt));
    b->in_flight++;
    b->cv.notify_all();
    return GPIS_OK;
}
