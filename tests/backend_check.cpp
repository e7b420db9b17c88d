// Check program of the C++ batch backend (include/gpis_backend.hpp) built by
// tests/test_backend.py: replies of submitBatch against gpis_flights_trace_host
// on the same flights, two batches in flight at once, request order, one
// onComplete per batch, an invalid medium index reported per request.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gpis_backend.hpp"

static float frand(uint32_t &s)
{
    s = s * 1664525u + 1013904223u;
    return (float)(s >> 8) * (1.0f / 16777216.0f);
}

int main()
{
    gpis_medium_desc d;
    gpis_medium_desc_init(&d);
    d.sigma = 0.05f; d.length_scale = 0.1f; d.kernel_scale = 3.0f; d.impulse_density = 8.0f; d.seed = 1;
    d.one_d_sampling = 1; d.correlation_context = GPIS_CTX_RENEWAL_PLUS; d.step_size = 0.01f; d.min_step = 8;
    d.mean_kind = GPIS_MEAN_SPHERE; d.mean_params[3] = 1.0f;
    int err = 0;
    auto backend = gpis::BatchBackend::create(&d, 1, &err);
    if (!backend) { std::printf("FAIL create %d %s\n", err, gpis_last_error()); return 1; }
    const int n = 3000;
    std::vector<gpis::SegmentRequest> req(n);
    uint32_t s = 12345u;
    for (int i = 0; i < n; ++i) {
        gpis::SegmentRequest &q = req[i];
        float o[3] = {2.0f * frand(s) - 1.0f, 2.0f * frand(s) - 1.0f, -1.5f};
        float t[3] = {0.6f * frand(s) - 0.3f, 0.6f * frand(s) - 0.3f, 0.0f};
        float dv[3] = {t[0] - o[0], t[1] - o[1], t[2] - o[2]};
        const float len = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
        for (int k = 0; k < 3; ++k) { q.origin[k] = o[k]; q.direction[k] = dv[k] / len; }
        q.near_t = 0.0f; q.far_t = 3.0f; q.jitter = frand(s);
        q.noise_seed = 1000u + (uint32_t)i; q.normal_seed = 7u * (uint32_t)i + 3u;
        q.first_scatter = true;
        q.purpose = (i % 5 == 0) ? gpis::SegmentRequest::Purpose::Shadow : gpis::SegmentRequest::Purpose::Path;
    }
    req[17].medium = 5;  // not in the backend
    std::atomic<int> completions{0};
    auto f1 = backend->submitBatch(req, [&] { completions++; });
    std::vector<gpis::SegmentRequest> half(req.begin(), req.begin() + n / 2);
    auto f2 = backend->submitBatch(half, [&] { completions++; });
    std::vector<gpis::SegmentReply> r1 = f1.get(), r2 = f2.get();
    // the same flights through the blocking host entry point
    gpis_ctx *ctx = nullptr;
    if (gpis_ctx_create(&d, 1, &ctx)) { std::printf("FAIL ctx\n"); return 1; }
    std::vector<float> on(4 * n), df(4 * n), pv(4 * n, 0.0f), rec(8 * n);
    std::vector<uint32_t> sd(4 * n), md(n);
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) { on[4 * i + k] = req[i].origin[k]; df[4 * i + k] = req[i].direction[k]; }
        on[4 * i + 3] = req[i].near_t; df[4 * i + 3] = req[i].far_t;
        std::memcpy(&sd[4 * i + 3], &req[i].jitter, 4);
        sd[4 * i] = req[i].noise_seed; sd[4 * i + 1] = req[i].normal_seed;
        sd[4 * i + 2] = GPIS_FLAG_FIRST_SCATTER | (req[i].purpose == gpis::SegmentRequest::Purpose::Shadow ? GPIS_FLAG_SHADOW : 0u);
        md[i] = req[i].medium;
    }
    gpis_flight_soa in{on.data(), df.data(), sd.data(), pv.data(), md.data()};
    gpis_result_soa out{rec.data()};
    if (gpis_flights_trace_host(ctx, &in, &out, n)) { std::printf("FAIL trace\n"); return 1; }
    int mismatch = 0, hits = 0, invalid = 0;
    for (int i = 0; i < n; ++i) {
        const float *r = &rec[8 * i];
        uint32_t st;
        std::memcpy(&st, &r[7], 4);
        const bool ok = (st & 0xFFu) == GPIS_FLIGHT_OK;
        const gpis::SegmentReply &y = r1[i];
        if (y.valid != ok || (ok && (y.result.t != r[0] || y.result.hit != (r[5] == 0.0f) || y.result.value != r[1] ||
                                     y.result.gradient[0] != r[2])))
            mismatch++;
        if (i < n / 2 && (r2[i].valid != y.valid || r2[i].result.t != y.result.t)) mismatch++;
        hits += y.valid && y.result.hit;
        invalid += !y.valid;
    }
    gpis_ctx_destroy(ctx);
    gpis::SegmentResult one;
    const bool v = backend->trace(req[3], one);
    if (!v || one.t != r1[3].result.t) mismatch++;
    backend.reset();
    std::printf("%s n=%d mismatch=%d hits=%d invalid=%d completions=%d\n",
                (mismatch == 0 && invalid == 1 && !r1[17].valid && completions == 2) ? "OK" : "FAIL", n, mismatch,
                hits, invalid, completions.load());
    return (mismatch == 0 && invalid == 1 && completions == 2) ? 0 : 1;
}
