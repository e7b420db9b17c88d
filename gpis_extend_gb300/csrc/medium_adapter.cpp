// medium_adapter.cpp -- the GaussianProcessMedium distance and transmittance
// state machines over the flight kernels (gpis_medium_sample_distance,
// gpis_medium_transmittance).
//
// Follows GaussianProcessMedium::sampleDistance / beginDistance /
// resumeDistance / finishDistance (GaussianProcessMedium.cpp:222-381),
// transmittance / beginTransmittance / resumeTransmittance (:383-440), the
// state updates of SparseConvolutionNoiseMedium::finishGpisSegment
// (SparseConvolutionNoiseMedium.cpp:265-347) and MediumState::advance
// (Medium.hpp:100-106).  The segment queries themselves (intersectGP and the
// gradient sample) run as one batch of flights on the GPU.
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "../../include/gpis.h"

extern "C" int gpis_internal_set_error(int code, const char *msg);
extern "C" const gpis_medium_desc *gpis_internal_ctx_medium(gpis_ctx *ctx, uint32_t index);

namespace {

struct Sigmas {
    float sa, ss, st;
    bool absorption_only;
};

// GaussianProcessMedium::prepareForRender (GaussianProcessMedium.cpp:153-159)
Sigmas sigmas(const gpis_medium_desc &d)
{
    Sigmas s;
    s.sa = d.sigma_a * d.density;
    s.ss = d.sigma_s * d.density;
    s.st = s.sa + s.ss;
    s.absorption_only = s.ss == 0.0f;
    return s;
}

struct Flights {
    std::vector<float> on, df, pv, rec;
    std::vector<uint32_t> sd;
    std::vector<uint32_t> ray;     // ray index of each flight
    void add(const gpis_medium_desc &d, const gpis_ray &r, float far_t, const gpis_medium_state &st,
             float jitter, bool shadow, uint32_t index)
    {
        on.insert(on.end(), {r.pos[0], r.pos[1], r.pos[2], r.near_t});
        df.insert(df.end(), {r.dir[0], r.dir[1], r.dir[2], far_t});
        uint32_t ns = 0, nm = 0;
        gpis_flight_seeds(&d, st.pixel_sample_segment, st.scene_seed, &ns, &nm);
        uint32_t jb;
        std::memcpy(&jb, &jitter, 4);
        const bool first = st.first_scatter != 0;
        sd.insert(sd.end(), {ns, nm, (first ? GPIS_FLAG_FIRST_SCATTER : 0u) | (shadow ? GPIS_FLAG_SHADOW : 0u), jb});
        pv.insert(pv.end(), {first ? 0.0f : st.last_val, first ? 0.0f : st.last_aniso[0],
                             first ? 0.0f : st.last_aniso[1], first ? 0.0f : st.last_aniso[2]});
        ray.push_back(index);
    }
    uint32_t size() const { return (uint32_t)ray.size(); }
    int run(gpis_ctx *ctx, uint32_t medium)
    {
        const uint32_t n = size();
        rec.assign((size_t)n * 8, 0.0f);
        if (n == 0) return GPIS_OK;
        std::vector<uint32_t> med(n, medium);
        gpis_flight_soa in{on.data(), df.data(), sd.data(), pv.data(), med.data()};
        gpis_result_soa out{rec.data()};
        return gpis_flights_trace_host(ctx, &in, &out, n);
    }
    float t(uint32_t i) const { return rec[8 * (size_t)i]; }
    float value(uint32_t i) const { return rec[8 * (size_t)i + 1]; }
    bool hit(uint32_t i) const { return rec[8 * (size_t)i + 5] == 0.0f; }
    const float *grad(uint32_t i) const { return &rec[8 * (size_t)i + 2]; }
    uint32_t status(uint32_t i) const
    {
        uint32_t s;
        std::memcpy(&s, &rec[8 * (size_t)i + 7], 4);
        return s;
    }
};

// samplingScheme at the end point (SparseConvolutionNoise.cpp:68-76); the
// observed-origin case needs the stationary SE covariance.
uint32_t scheme_at(const gpis_medium_desc &d, bool conditioned_rp, float t)
{
    if (d.single_realization || !d.one_d_sampling) return GPIS_SCHEME_UNI;
    if (d.sigma < 1e-6f) return GPIS_SCHEME_UNI;
    if (d.correlation_xy && conditioned_rp && t == 0.0f && d.ls_kind == GPIS_LS_CONSTANT)
        return GPIS_SCHEME_UNI;  // p == ray origin
    return d.sampling_scheme;
}

bool conditioned_rp(const gpis_medium_desc &d, const gpis_medium_state &st)
{
    return !d.single_realization && d.correlation_context == GPIS_CTX_RENEWAL_PLUS && st.first_scatter == 0;
}

// finishGpisSegment's state update (SparseConvolutionNoiseMedium.cpp:272-285, 331-345).
void finish_segment(const gpis_medium_desc &d, const Flights &f, uint32_t i, gpis_medium_state &st)
{
    const bool rp = conditioned_rp(d, st);
    if (f.hit(i)) {
        st.last_gp_id = (int32_t)((f.status(i) >> 8) & 0xFFu);
        st.sampling_scheme = scheme_at(d, rp, f.t(i));
        st.last_val = 0.0f;
    } else {
        st.sampling_scheme = GPIS_SCHEME_UNI;
        st.last_val = f.value(i);
    }
}

void set3(float *a, float x, float y, float z) { a[0] = x; a[1] = y; a[2] = z; }

}  // namespace

extern "C" int gpis_medium_sample_distance(gpis_ctx *ctx, uint32_t medium, const gpis_ray *rays,
                                           gpis_medium_state *states, const float *jitter,
                                           gpis_medium_sample *samples, uint32_t n)
{
    const gpis_medium_desc *dp = ctx ? gpis_internal_ctx_medium(ctx, medium) : nullptr;
    if (!dp) return gpis_internal_set_error(GPIS_EINVAL, "unknown context or medium index");
    if (n && (!rays || !states || !jitter || !samples)) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    const gpis_medium_desc &d = *dp;
    const Sigmas sg = sigmas(d);
    Flights dist, trans;
    std::vector<float> far_of(n);
    for (uint32_t i = 0; i < n; ++i) {
        const gpis_ray &r = rays[i];
        gpis_medium_sample &s = samples[i];
        std::memset(&s, 0, sizeof(s));
        gpis_medium_state &st = states[i];
        // beginDistance (GaussianProcessMedium.cpp:236-287)
        float far_t = r.far_t;
        if (!std::isfinite(far_t)) far_t = (float)((double)r.near_t + 2000);
        far_of[i] = far_t;
        const float maxT = far_t;
        if (st.bounce >= d.max_bounces) {
            s.status = 0;
            continue;
        }
        if (maxT <= r.near_t) {
            s.t = maxT;
            set3(s.weight, 1.0f, 1.0f, 1.0f);
            s.pdf = 1.0f;
            s.exited = 1;
            for (int k = 0; k < 3; ++k) s.p[k] = r.pos[k] + s.t * r.dir[k];
            s.gp_id = 0;
            s.sampling_scheme = GPIS_SCHEME_UNI;
            s.status = 1;
            continue;
        }
        if (sg.absorption_only) {
            trans.add(d, r, far_t, st, jitter[i], true, i);
            continue;
        }
        dist.add(d, r, far_t, st, jitter[i], false, i);
    }
    int rc = dist.run(ctx, medium);
    if (rc) return rc;
    rc = trans.run(ctx, medium);
    if (rc) return rc;
    // absorption-only media: sample.t = maxT with the transmittance as the weight
    for (uint32_t j = 0; j < trans.size(); ++j) {
        const uint32_t i = trans.ray[j];
        const gpis_ray &r = rays[i];
        gpis_medium_sample &s = samples[i];
        gpis_medium_state &st = states[i];
        finish_segment(d, trans, j, st);
        const float tr = trans.hit(j) ? 0.0f : 1.0f;
        if (trans.t(j) < far_of[i]) {
            const float *g = trans.grad(j);
            set3(st.last_aniso, g[0], g[1], g[2]);
            st.first_scatter = 0;
        }
        s.t = far_of[i];
        set3(s.weight, tr, tr, tr);
        s.pdf = 1.0f;
        s.exited = 1;
        s.sampling_scheme = GPIS_SCHEME_UNI;
        for (int k = 0; k < 3; ++k) s.p[k] = r.pos[k] + s.t * r.dir[k];
        s.gp_id = st.last_gp_id;
        st.info_t += s.t;
        s.status = 1;
    }
    // resumeDistance (GaussianProcessMedium.cpp:289-369) and finishDistance (:371-381)
    for (uint32_t j = 0; j < dist.size(); ++j) {
        const uint32_t i = dist.ray[j];
        const gpis_ray &r = rays[i];
        gpis_medium_sample &s = samples[i];
        gpis_medium_state &st = states[i];
        if ((dist.status(j) & 0xFFu) != GPIS_FLIGHT_OK) {
            s.status = 0;
            continue;
        }
        finish_segment(d, dist, j, st);
        const float maxT = far_of[i];
        const double t = dist.t(j);
        const bool hit = dist.hit(j);
        s.exited = hit ? 0 : 1;
        const float *g = dist.grad(j);
        if (t < maxT) {
            set3(s.aniso, g[0], g[1], g[2]);
            set3(st.last_aniso, g[0], g[1], g[2]);
            st.first_scatter = 0;
            if (!std::isfinite((g[0] + g[1] + g[2]) / 3.0f)) {
                set3(s.aniso, 1.0f, 0.0f, 0.0f);
                s.status = 0;
                continue;
            }
        }
        if (hit) {
            const double dot = (double)s.aniso[0] * r.dir[0] + (double)s.aniso[1] * r.dir[1] + (double)s.aniso[2] * r.dir[2];
            if (dot > 0) {
                s.status = 0;  // outward crossing rejected
                continue;
            }
            const double l2 = (double)s.aniso[0] * s.aniso[0] + (double)s.aniso[1] * s.aniso[1] + (double)s.aniso[2] * s.aniso[2];
            if (l2 < 0.0000001f) {
                set3(s.aniso, 1.0f, 0.0f, 0.0f);
                s.status = 0;
                continue;
            }
        } else {
            // the gradient of the end point of a miss is sampled too (GaussianProcessMedium.cpp:353)
            set3(s.aniso, g[0], g[1], g[2]);
        }
        set3(s.weight, 1.0f, 1.0f, 1.0f);
        set3(s.continued_weight, 1.0f, 1.0f, 1.0f);
        s.t = std::fmin((float)t, maxT);
        s.continued_t = (float)t;
        const float ratio = sg.ss / sg.st;
        for (int k = 0; k < 3; ++k) {
            s.weight[k] *= ratio;
            s.continued_weight[k] *= ratio;
        }
        s.pdf = 1.0f;
        set3(st.last_aniso, s.aniso[0], s.aniso[1], s.aniso[2]);
        s.sampling_scheme = st.sampling_scheme;
        // MediumState::advance
        st.first_scatter = 0;
        st.bounce += 1;
        st.sampling_scheme = GPIS_SCHEME_UNI;
        // finishDistance
        for (int k = 0; k < 3; ++k) s.p[k] = r.pos[k] + s.t * r.dir[k];
        s.gp_id = st.last_gp_id;
        st.info_t += s.t;
        s.status = 1;
    }
    return GPIS_OK;
}

extern "C" int gpis_medium_transmittance(gpis_ctx *ctx, uint32_t medium, const gpis_ray *rays,
                                         gpis_medium_state *states, const float *jitter,
                                         float *transmittance, uint32_t n)
{
    const gpis_medium_desc *dp = ctx ? gpis_internal_ctx_medium(ctx, medium) : nullptr;
    if (!dp) return gpis_internal_set_error(GPIS_EINVAL, "unknown context or medium index");
    if (n && (!rays || !states || !jitter || !transmittance)) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    const gpis_medium_desc &d = *dp;
    Flights f;
    std::vector<float> far_of(n);
    for (uint32_t i = 0; i < n; ++i) {
        const gpis_ray &r = rays[i];
        transmittance[i] = 1.0f;
        if (r.far_t <= r.near_t) continue;   // GaussianProcessMedium.cpp:428-429
        float far_t = r.far_t;
        if (!std::isfinite(far_t)) far_t = (float)((double)r.near_t + 2000);
        far_of[i] = far_t;
        f.add(d, r, far_t, states[i], jitter[i], true, i);
    }
    int rc = f.run(ctx, medium);
    if (rc) return rc;
    for (uint32_t j = 0; j < f.size(); ++j) {
        const uint32_t i = f.ray[j];
        gpis_medium_state &st = states[i];
        if ((f.status(j) & 0xFFu) != GPIS_FLIGHT_OK) {
            transmittance[i] = 0.0f;
            continue;
        }
        finish_segment(d, f, j, st);
        if (f.t(j) < far_of[i]) {
            const float *g = f.grad(j);
            set3(st.last_aniso, g[0], g[1], g[2]);
            st.first_scatter = 0;
            if (!std::isfinite((g[0] + g[1] + g[2]) / 3.0f)) {
                transmittance[i] = 0.0f;
                continue;
            }
        }
        transmittance[i] = f.hit(j) ? 0.0f : 1.0f;
    }
    return GPIS_OK;
}
