/*
 * gpis_backend.hpp -- a C++ batch backend over the gpis C ABI with the shape of
 * the reference's GpRayBatchBackend (GpRayBatchBackend.hpp:15-55): requests,
 * replies, a blocking trace() and submitBatch() returning a future of the
 * replies in request order.  Header-only; it needs only gpis.h and the
 * library, no CUDA headers.
 *
 * Differences in form, not in contract: a request names its medium by its
 * index in the backend's medium list (the reference holds a medium pointer),
 * and a reply also carries the hit gradient and the flight status, so a caller
 * need not re-evaluate the gradient on the CPU.
 */
#ifndef GPIS_BACKEND_HPP_
#define GPIS_BACKEND_HPP_

#include <cstdint>
#include <cstring>
#include <functional>
#include <future>
#include <memory>
#include <vector>

#include "gpis.h"

namespace gpis {

/* GpRaySegmentRequest (GpRayBatchBackend.hpp:15-29) */
struct SegmentRequest {
    enum class Purpose { Path, Shadow };
    Purpose purpose = Purpose::Path;
    uint32_t medium = 0;
    float origin[3] = {0.0f, 0.0f, 0.0f};
    float direction[3] = {0.0f, 0.0f, 1.0f};
    float near_t = 0.0f;
    float far_t = 0.0f;
    float jitter = 0.0f;
    uint32_t noise_seed = 0;
    uint32_t normal_seed = 0;
    bool first_scatter = true;
    float previous_value = 0.0f;
    float previous_gradient[3] = {0.0f, 0.0f, 0.0f};
};

/* GpRaySegmentResult (:31-35) plus the gradient, steps and flight status */
struct SegmentResult {
    float t = 0.0f;
    float value = 0.0f;
    bool hit = false;
    float gradient[3] = {0.0f, 0.0f, 0.0f};
    uint32_t steps = 0;
    uint32_t status = 0;
};

/* GpRaySegmentReply (:37-40): valid = false leaves the caller free to trace
 * the segment on the CPU */
struct SegmentReply {
    bool valid = false;
    SegmentResult result;
};

class BatchBackend {
public:
    /* One context over the media; returns nullptr and sets *error on failure. */
    static std::unique_ptr<BatchBackend> create(const gpis_medium_desc *media, int n_media, int *error = nullptr)
    {
        gpis_backend *b = nullptr;
        const int rc = gpis_backend_create(media, n_media, &b);
        if (error) *error = rc;
        if (rc) return nullptr;
        return std::unique_ptr<BatchBackend>(new BatchBackend(b));
    }

    ~BatchBackend() { gpis_backend_destroy(b_); }
    BatchBackend(const BatchBackend &) = delete;
    BatchBackend &operator=(const BatchBackend &) = delete;

    /* Blocking single segment (GpRayBatchBackend::trace). */
    bool trace(const SegmentRequest &request, SegmentResult &result)
    {
        std::vector<SegmentReply> r = submitBatch({request}).get();
        result = r[0].result;
        return r[0].valid;
    }

    /* Requests are copied before the call returns; replies come in request order;
     * onComplete runs once after the replies are published, possibly on a CUDA
     * callback thread: notify a scheduler there, make no CUDA calls. */
    std::future<std::vector<SegmentReply>> submitBatch(const std::vector<SegmentRequest> &requests,
                                                       std::function<void()> onComplete = {})
    {
        Job *job = new Job;
        job->on_complete = std::move(onComplete);
        const size_t n = requests.size();
        job->rec.assign(8 * n, 0.0f);
        std::vector<float> on(4 * n), df(4 * n), pv(4 * n);
        std::vector<uint32_t> sd(4 * n), md(n);
        for (size_t i = 0; i < n; ++i) {
            const SegmentRequest &q = requests[i];
            for (int k = 0; k < 3; ++k) {
                on[4 * i + k] = q.origin[k];
                df[4 * i + k] = q.direction[k];
                pv[4 * i + 1 + k] = q.previous_gradient[k];
            }
            on[4 * i + 3] = q.near_t;
            df[4 * i + 3] = q.far_t;
            pv[4 * i] = q.previous_value;
            uint32_t jb;
            std::memcpy(&jb, &q.jitter, 4);
            sd[4 * i] = q.noise_seed;
            sd[4 * i + 1] = q.normal_seed;
            sd[4 * i + 2] = (q.first_scatter ? GPIS_FLAG_FIRST_SCATTER : 0u) |
                            (q.purpose == SegmentRequest::Purpose::Shadow ? GPIS_FLAG_SHADOW : 0u);
            sd[4 * i + 3] = jb;
            md[i] = q.medium;
        }
        std::future<std::vector<SegmentReply>> f = job->promise.get_future();
        gpis_flight_soa in{on.data(), df.data(), sd.data(), pv.data(), md.data()};
        const int rc = gpis_backend_submit(b_, &in, job->rec.data(), (uint32_t)n, &BatchBackend::done, job);
        if (rc) done(job, rc);
        return f;
    }

private:
    struct Job {
        std::vector<float> rec;
        std::promise<std::vector<SegmentReply>> promise;
        std::function<void()> on_complete;
    };

    explicit BatchBackend(gpis_backend *b) : b_(b) {}

    static void done(void *user, int status)
    {
        Job *job = static_cast<Job *>(user);
        const size_t n = job->rec.size() / 8;
        std::vector<SegmentReply> replies(n);
        for (size_t i = 0; i < n && status == GPIS_OK; ++i) {
            const float *r = &job->rec[8 * i];
            uint32_t st, steps;
            std::memcpy(&steps, &r[6], 4);
            std::memcpy(&st, &r[7], 4);
            SegmentReply &y = replies[i];
            y.result.t = r[0];
            y.result.value = r[1];
            y.result.gradient[0] = r[2];
            y.result.gradient[1] = r[3];
            y.result.gradient[2] = r[4];
            y.result.hit = r[5] == 0.0f;
            y.result.steps = steps;
            y.result.status = st;
            y.valid = (st & 0xFFu) == GPIS_FLIGHT_OK;
        }
        job->promise.set_value(std::move(replies));
        if (job->on_complete) job->on_complete();
        delete job;
    }

    gpis_backend *b_;
};

}  // namespace gpis

#endif
