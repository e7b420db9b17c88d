/*
 * pt_oracle.c -- CPU restatement of the wavefront path tracer around the GPIS
 * medium (gpis_render).  TEST INFRASTRUCTURE ONLY: the image parity tests and
 * the CPU baseline call it as the checker.
 *
 * It follows PathTracer::traceSample (PathTracer.cpp:49-292) for the scene
 * class of gpis_scene_desc: pinhole camera, the medium's bounding cube as a
 * forward boundary (no bounce counted when crossing it), one one-sided quad
 * light outside the cube, GP surface events from
 * GaussianProcessMedium::sampleDistance (gor_medium_sample_distance) shaded by
 * BRDFPhaseFunction over LambertBsdf, MirrorBsdf or ConductorBsdf
 * (BRDFPhaseFunction.cpp:29-119, MirrorBsdf.cpp:31-109, ConductorBsdf.cpp:58-137),
 * and handleVolume's direct lighting (TraceBase.cpp:993-1014): volumeLightSample
 * (:798-839) plus volumePhaseSample (:841-874), each with a transmittance query
 * (gor_medium_transmittance), on the medium state of the next bounce
 * (pixelSampleSegment.w + 1).  The specular phases follow the event's 1D
 * sampling scheme: the light sample under NEE and MIS (neePDF / neeGrad, gor_nee),
 * the phase sample under UNI and MIS, the power heuristic under MIS only.
 *
 * Every float expression is written as the CUDA side writes it and the file is
 * built with -ffp-contract=off, so both make the same decisions: no
 * trigonometry (directions come from rejection in the unit disk), correctly
 * rounded sqrtf and divisions only.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "gpis_oracle.h"

#define INV_PI_F 0.31830988618379067f

/* counter RNG: splitmix64 finaliser over (seed, path, bounce, dimension) */
static inline uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline float rng(uint32_t seed, uint64_t path, uint32_t bounce, uint32_t dim)
{
    uint64_t k = mix64(((uint64_t)seed << 32) ^ path);
    k = mix64(k ^ (((uint64_t)bounce << 32) | dim));
    return (float)(k >> 40) * (1.0f / 16777216.0f);
}

/* dimensions of one bounce */
enum { D_JIT = 0, D_LU = 1, D_LV = 2, D_JS1 = 3, D_PHASE = 4, D_JS2 = 20, D_CONT = 21, D_PIX = 40 };
#define CAMERA_BOUNCE 0xFFFFu

static inline float dot3(const float a[3], const float b[3])
{
    float s = a[0] * b[0];
    s = s + a[1] * b[1];
    s = s + a[2] * b[2];
    return s;
}

static inline void normalize3(float v[3])
{
    const float inv = 1.0f / sqrtf(dot3(v, v));
    v[0] = v[0] * inv; v[1] = v[1] * inv; v[2] = v[2] * inv;
}

static inline void cross3(const float a[3], const float b[3], float o[3])
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* TangentFrame(n) (TangentFrame.hpp:74-83) */
typedef struct { float t[3], b[3], n[3]; } pframe_t;
static void pframe(const float n_in[3], pframe_t *f)
{
    memcpy(f->n, n_in, sizeof(f->n));
    normalize3(f->n);
    const float *n = f->n;
    const float sign = copysignf(1.0f, n[2]);
    const float a = -1.0f / (sign + n[2]);
    const float b = n[0] * n[1] * a;
    f->t[0] = 1.0f + sign * n[0] * n[0] * a; f->t[1] = sign * b; f->t[2] = -sign * n[0];
    f->b[0] = b; f->b[1] = sign + n[1] * n[1] * a; f->b[2] = -n[1];
    normalize3(f->t);
    normalize3(f->b);
}

static inline void to_local(const pframe_t *f, const float v[3], float o[3])
{
    o[0] = dot3(f->t, v); o[1] = dot3(f->b, v); o[2] = dot3(f->n, v);
}

static inline void to_global(const pframe_t *f, const float l[3], float o[3])
{
    for (int i = 0; i < 3; ++i) {
        float s = f->t[i] * l[0];
        s = s + f->b[i] * l[1];
        s = s + f->n[i] * l[2];
        o[i] = s;
    }
}

/* Cosine-weighted hemisphere direction in local coordinates from rejection in
 * the unit disk (dimensions dim0, dim0 + 1, ... of this bounce, at most 8 tries;
 * the centre after that).  Returns the local direction. */
static void cosine_dir(uint32_t seed, uint64_t path, uint32_t bounce, uint32_t dim0, float w[3])
{
    float x = 0.0f, y = 0.0f;
    for (int k = 0; k < 8; ++k) {
        const float u = 2.0f * rng(seed, path, bounce, dim0 + 2 * k) - 1.0f;
        const float v = 2.0f * rng(seed, path, bounce, dim0 + 2 * k + 1) - 1.0f;
        if (u * u + v * v < 1.0f) { x = u; y = v; break; }
    }
    w[0] = x; w[1] = y;
    const float r2 = x * x + y * y;
    w[2] = sqrtf(fmaxf(0.0f, 1.0f - r2));
}

/* slab test of the cube [-h, h]^3: entry and exit parameters */
static int box_hit(const float o[3], const float d[3], float h, float *t0, float *t1)
{
    float tmin = -INFINITY, tmax = INFINITY;
    for (int i = 0; i < 3; ++i) {
        if (d[i] == 0.0f) {
            if (o[i] < -h || o[i] > h) return 0;
            continue;
        }
        const float inv = 1.0f / d[i];
        float ta = (-h - o[i]) * inv, tb = (h - o[i]) * inv;
        if (ta > tb) { const float s = ta; ta = tb; tb = s; }
        tmin = fmaxf(tmin, ta);
        tmax = fminf(tmax, tb);
    }
    if (tmax < fmaxf(tmin, 0.0f)) return 0;
    *t0 = tmin; *t1 = tmax;
    return 1;
}

/* one-sided quad light: parameter of the front-side hit, or -1 */
static float light_hit(const gpis_scene_desc *sc, const float ln[3], const float o[3], const float d[3])
{
    const float den = dot3(d, ln);
    if (!(den < 0.0f)) return -1.0f;
    float co[3];
    for (int i = 0; i < 3; ++i) co[i] = sc->light_center[i] - o[i];
    const float t = dot3(co, ln) / den;
    if (!(t > 0.0f)) return -1.0f;
    float x[3];
    for (int i = 0; i < 3; ++i) x[i] = (o[i] + t * d[i]) - sc->light_center[i];
    const float s = dot3(x, sc->light_u) / dot3(sc->light_u, sc->light_u);
    const float r = dot3(x, sc->light_v) / dot3(sc->light_v, sc->light_v);
    if (fabsf(s) > 0.5f || fabsf(r) > 0.5f) return -1.0f;
    return t;
}

/* SampleWarp::powerHeuristic (SampleWarp.hpp:189-199): the bounded ratio in double */
static inline float power_heuristic(double pdf0, double pdf1)
{
    if (pdf0 >= pdf1) {
        const double ratio = pdf1 / pdf0;
        return (float)(1.0 / (1.0 + ratio * ratio));
    }
    const double ratio = pdf0 / pdf1;
    return (float)(ratio * ratio / (1.0 + ratio * ratio));
}

/* Fresnel::conductorReflectance (Fresnel.hpp:102-123) of one channel; the
 * mirror phase reflects everything */
static float conductor_reflectance(const gpis_scene_desc *sc, int c, float cos_i)
{
    if (sc->phase != GPIS_PHASE_CONDUCTOR) return 1.0f;
    const float eta = sc->eta[c], k = sc->k[c];
    if (eta == 0.0f && k == 0.0f) return 1.0f;
    const float c2 = cos_i * cos_i;
    const float s2 = fmaxf(1.0f - c2, 0.0f);
    const float s4 = s2 * s2;
    const float inner = eta * eta - k * k - s2;
    const float ab = sqrtf(fmaxf(inner * inner + 4.0f * eta * eta * k * k, 0.0f));
    const float a = sqrtf(fmaxf((ab + inner) * 0.5f, 0.0f));
    const float rs = ((ab + c2) - (2.0f * a * cos_i)) / ((ab + c2) + (2.0f * a * cos_i));
    const float rp = ((c2 * ab + s4) - (2.0f * a * cos_i * s2)) / ((c2 * ab + s4) + (2.0f * a * cos_i * s2));
    return 0.5f * (rs + rs * rp);
}

/* transmittance (0/1) through the medium from p along d to the cube's exit */
static float shadow(const gpis_medium_desc *md, const gpis_scene_desc *sc, const float p[3], const float d[3],
                    const gpis_medium_state *st, float jitter, uint64_t *nflights)
{
    float t0, t1;
    if (!box_hit(p, d, sc->box_half, &t0, &t1) || !(t1 > 0.0f)) return 1.0f;
    gpis_ray r;
    memcpy(r.pos, p, sizeof(r.pos));
    memcpy(r.dir, d, sizeof(r.dir));
    r.near_t = 0.0f;
    r.far_t = t1;
    gpis_medium_state s2 = *st;
    float tr = 1.0f;
    gor_medium_transmittance(md, &r, &s2, &jitter, &tr, 1);
    (*nflights)++;
    return tr;
}

typedef struct { uint64_t distance, shadow, events, failed; } pt_counts_t;

static void trace_path(const gpis_medium_desc *md, const gpis_scene_desc *sc, uint32_t px, uint32_t py, uint32_t s,
                       float out[3], pt_counts_t *cnt)
{
    const uint64_t path = ((uint64_t)py * sc->width + px) * sc->spp + s;
    const uint32_t seed = sc->sampler_seed;
    /* camera */
    float fwd[3], right[3], up[3];
    for (int i = 0; i < 3; ++i) fwd[i] = sc->cam_target[i] - sc->cam_pos[i];
    normalize3(fwd);
    cross3(fwd, sc->cam_up, right);
    normalize3(right);
    cross3(right, fwd, up);
    const float aspect = (float)sc->width / (float)sc->height;
    const float u0 = rng(seed, path, CAMERA_BOUNCE, D_PIX), u1 = rng(seed, path, CAMERA_BOUNCE, D_PIX + 1);
    const float sx = (2.0f * ((float)px + u0) / (float)sc->width - 1.0f) * sc->tan_half_fov * aspect;
    const float sy = (1.0f - 2.0f * ((float)py + u1) / (float)sc->height) * sc->tan_half_fov;
    float pos[3], dir[3];
    for (int i = 0; i < 3; ++i) {
        pos[i] = sc->cam_pos[i];
        dir[i] = fwd[i] + sx * right[i] + sy * up[i];
    }
    normalize3(dir);
    float ln[3];
    cross3(sc->light_u, sc->light_v, ln);
    const float area = sqrtf(dot3(ln, ln));
    normalize3(ln);

    gpis_medium_state st;
    memset(&st, 0, sizeof(st));
    st.pixel_sample_segment[0] = px; st.pixel_sample_segment[1] = py; st.pixel_sample_segment[2] = s;
    st.scene_seed = sc->scene_seed;
    st.first_scatter = 1;
    float T[3] = {1.0f, 1.0f, 1.0f}, L[3] = {0.0f, 0.0f, 0.0f};
    int inside = 0, was_specular = 1;
    uint32_t bounce = 0;
    for (int guard = 0; guard < 4 * (int)sc->max_bounces + 8 && bounce < sc->max_bounces; ++guard) {
        if (!inside) {
            float t0, t1;
            const int hb = box_hit(pos, dir, sc->box_half, &t0, &t1) && t0 > 0.0f;
            const float tl = light_hit(sc, ln, pos, dir);
            if (tl > 0.0f && (!hb || tl < t0)) {
                if (was_specular)
                    for (int c = 0; c < 3; ++c) L[c] = L[c] + T[c] * sc->light_emission[c];
                break;
            }
            if (!hb) break;
            for (int i = 0; i < 3; ++i) {
                const float e = pos[i] + t0 * dir[i];
                pos[i] = fminf(fmaxf(e, -sc->box_half), sc->box_half);
            }
            inside = 1;
            continue;
        }
        /* inside: one sampleDistance query to the cube's exit */
        float t0, t1;
        if (!box_hit(pos, dir, sc->box_half, &t0, &t1)) { inside = 0; continue; }
        gpis_ray r;
        memcpy(r.pos, pos, sizeof(r.pos));
        memcpy(r.dir, dir, sizeof(r.dir));
        r.near_t = 0.0f;
        r.far_t = fmaxf(t1, 0.0f);
        st.pixel_sample_segment[3] = bounce;
        const float jit = rng(seed, path, bounce, D_JIT);
        /* the distance flight's inputs (gm_flight), for NEE queries on its realization */
        float fo[3], fd[3], fpv[4];
        uint32_t fsd[4];
        {
            const int first = st.first_scatter != 0;
            gor_flight_seeds(md, st.pixel_sample_segment, st.scene_seed, &fsd[0], &fsd[1]);
            fsd[2] = first ? GPIS_FLAG_FIRST_SCATTER : 0u;
            memcpy(&fsd[3], &jit, 4);
            memcpy(fo, pos, sizeof(fo));
            memcpy(fd, dir, sizeof(fd));
            fpv[0] = first ? 0.0f : st.last_val;
            for (int i = 0; i < 3; ++i) fpv[1 + i] = first ? 0.0f : st.last_aniso[i];
        }
        gpis_medium_sample ms;
        gor_medium_sample_distance(md, &r, &st, &jit, &ms, 1);
        cnt->distance++;
        if (ms.status != 1) { cnt->failed++; break; }
        for (int c = 0; c < 3; ++c) T[c] = T[c] * ms.weight[c];
        if (ms.exited) {
            /* forward boundary: continue from the exit point outside the cube */
            /* (a ray leaving the cube from its surface never re-enters it) */
            for (int i = 0; i < 3; ++i) pos[i] = ms.p[i];
            inside = 0;
            continue;
        }
        cnt->events++;
        pframe_t f;
        pframe(ms.aniso, &f);
        float wi[3], nd[3] = {-dir[0], -dir[1], -dir[2]};
        to_local(&f, nd, wi);
        if (sc->phase != GPIS_PHASE_LAMBERT) {
            /* BRDFPhaseFunction over MirrorBsdf / ConductorBsdf: se.wi = frame.toLocal(-w).normalized(),
               the reflection (-wi.x, -wi.y, wi.z) with weight albedo * F(wi.z) */
            normalize3(wi);
            float fr[3], wr[3] = {-wi[0], -wi[1], wi[2]}, wrg[3];
            for (int c = 0; c < 3; ++c) fr[c] = sc->albedo[c] * conductor_reflectance(sc, c, wi[2]);
            to_global(&f, wr, wrg);
            normalize3(wrg);
            const uint32_t scheme = ms.sampling_scheme;
            const float *p = ms.p;
            if (bounce + 1 < sc->max_bounces) {
                gpis_medium_state s2 = st;
                s2.pixel_sample_segment[3] = bounce + 1;
                if (scheme != GPIS_SCHEME_UNI) {
                    /* volumeLightSample: f = albedo * F * neePDF at the half-vector normal
                       (MirrorBsdf::eval), the shadow flight conditioned on neeGrad (evalGrad) */
                    const float lu = rng(seed, path, bounce, D_LU) - 0.5f, lv = rng(seed, path, bounce, D_LV) - 0.5f;
                    float ld[3];
                    for (int i = 0; i < 3; ++i)
                        ld[i] = ((sc->light_center[i] + lu * sc->light_u[i]) + lv * sc->light_v[i]) - p[i];
                    const float dist2 = dot3(ld, ld), dist = sqrtf(dist2);
                    for (int i = 0; i < 3; ++i) ld[i] = ld[i] / dist;
                    const float cos_l = -dot3(ld, ln);
                    if (cos_l > 0.0f) {
                        const float pdf_l = dist2 / (area * cos_l);
                        float wo[3], hl[3], hw[3], grad[3] = {0.0f, 0.0f, 0.0f}, pdf = 0.0f;
                        to_local(&f, ld, wo);
                        normalize3(wo);
                        for (int i = 0; i < 3; ++i) hl[i] = (wi[i] + wo[i]) * 0.5f;
                        to_global(&f, hl, hw);
                        normalize3(hw);
                        gor_nee(md, fo, fd, p, hw, ms.t, fsd, fpv, &pdf, grad);
                        float fl[3];
                        for (int c = 0; c < 3; ++c) fl[c] = fr[c] * pdf;
                        if (fl[0] != 0.0f || fl[1] != 0.0f || fl[2] != 0.0f) {
                            gpis_medium_state s3 = s2;
                            memcpy(s3.last_aniso, grad, sizeof(grad));
                            const float tr = shadow(md, sc, p, ld, &s3, rng(seed, path, bounce, D_JS1), &cnt->shadow);
                            if (tr > 0.0f) {
                                const float w = scheme == GPIS_SCHEME_MIS ? power_heuristic(pdf_l, pdf) : 1.0f;
                                for (int c = 0; c < 3; ++c)
                                    L[c] = L[c] + T[c] * (fl[c] * sc->light_emission[c] / pdf_l * w);
                            }
                        }
                    }
                }
                if (scheme != GPIS_SCHEME_NEE) {
                    /* volumePhaseSample: the reflection, when it reaches the light; MIS weight 1
                       under UNI (volumeScatterMisWeight), else against neePDF at the event's normal */
                    const float tlh = light_hit(sc, ln, p, wrg);
                    if (tlh > 0.0f) {
                        float w = 1.0f;
                        if (scheme == GPIS_SCHEME_MIS) {
                            float pdf_s = 0.0f, g[3];
                            gor_nee(md, fo, fd, p, f.n, ms.t, fsd, fpv, &pdf_s, g);
                            const float cl = -dot3(wrg, ln);
                            const float pdf_l = (tlh * tlh) / (area * cl);
                            w = power_heuristic(pdf_s, pdf_l);
                        }
                        const float tr = shadow(md, sc, p, wrg, &s2, rng(seed, path, bounce, D_JS2), &cnt->shadow);
                        if (tr > 0.0f)
                            for (int c = 0; c < 3; ++c) L[c] = L[c] + T[c] * (fr[c] * sc->light_emission[c] * w);
                    }
                }
            }
            for (int c = 0; c < 3; ++c) T[c] = T[c] * fr[c];
            memcpy(pos, p, sizeof(pos));
            memcpy(dir, wrg, sizeof(dir));
            was_specular = 0;
            bounce++;
            continue;
        }
        if (!(wi[2] > 0.0f)) { cnt->failed++; break; }      /* LambertBsdf::sample fails */
        const float *p = ms.p;
        if (bounce + 1 < sc->max_bounces) {
            gpis_medium_state s2 = st;
            s2.pixel_sample_segment[3] = bounce + 1;
            /* volumeLightSample: a point on the quad */
            const float lu = rng(seed, path, bounce, D_LU) - 0.5f, lv = rng(seed, path, bounce, D_LV) - 0.5f;
            float ld[3];
            for (int i = 0; i < 3; ++i) ld[i] = ((sc->light_center[i] + lu * sc->light_u[i]) + lv * sc->light_v[i]) - p[i];
            const float dist2 = dot3(ld, ld), dist = sqrtf(dist2);
            for (int i = 0; i < 3; ++i) ld[i] = ld[i] / dist;
            const float cos_l = -dot3(ld, ln);
            if (cos_l > 0.0f) {
                const float pdf_l = dist2 / (area * cos_l);
                float wo[3];
                to_local(&f, ld, wo);
                if (wo[2] > 0.0f) {
                    const float pdf_p = wo[2] * INV_PI_F;
                    const float tr = shadow(md, sc, p, ld, &s2, rng(seed, path, bounce, D_JS1), &cnt->shadow);
                    if (tr > 0.0f) {
                        const float w = power_heuristic(pdf_l, pdf_p);
                        for (int c = 0; c < 3; ++c) {
                            const float fc = sc->albedo[c] * INV_PI_F * wo[2];
                            L[c] = L[c] + T[c] * (fc * sc->light_emission[c] / pdf_l * w);
                        }
                    }
                }
            }
            /* volumePhaseSample: a phase direction that reaches the light */
            float wl[3], wg[3];
            cosine_dir(seed, path, bounce, D_PHASE, wl);
            to_global(&f, wl, wg);
            normalize3(wg);
            const float tlh = light_hit(sc, ln, p, wg);
            if (tlh > 0.0f && wl[2] > 0.0f) {
                const float tr = shadow(md, sc, p, wg, &s2, rng(seed, path, bounce, D_JS2), &cnt->shadow);
                if (tr > 0.0f) {
                    const float pdf_p = wl[2] * INV_PI_F;
                    const float cos_l = -dot3(wg, ln);
                    const float pdf_l = (tlh * tlh) / (area * cos_l);
                    const float w = power_heuristic(pdf_p, pdf_l);
                    for (int c = 0; c < 3; ++c) L[c] = L[c] + T[c] * (sc->albedo[c] * sc->light_emission[c] * w);
                }
            }
        }
        /* phase sample: the continuation */
        float wl[3], wg[3];
        cosine_dir(seed, path, bounce, D_CONT, wl);
        to_global(&f, wl, wg);
        normalize3(wg);
        for (int c = 0; c < 3; ++c) T[c] = T[c] * sc->albedo[c];
        memcpy(pos, p, sizeof(pos));
        memcpy(dir, wg, sizeof(dir));
        was_specular = 0;
        bounce++;
    }
    memcpy(out, L, sizeof(L));
}

int gor_render(const gpis_medium_desc *md, const gpis_scene_desc *sc, float *image, uint64_t counts[4],
               uint32_t row0, uint32_t rows)
{
    if (!md || !sc || !image || sc->width == 0 || sc->height == 0 || sc->spp == 0) return GPIS_EINVAL;
    if (sc->phase > GPIS_PHASE_CONDUCTOR) return GPIS_EINVAL;
    pt_counts_t cnt = {0, 0, 0, 0};
    for (uint32_t y = row0; y < row0 + rows && y < sc->height; ++y)
        for (uint32_t x = 0; x < sc->width; ++x) {
            float acc[3] = {0.0f, 0.0f, 0.0f};
            for (uint32_t s = 0; s < sc->spp; ++s) {
                float l[3];
                trace_path(md, sc, x, y, s, l, &cnt);
                for (int c = 0; c < 3; ++c) acc[c] = acc[c] + l[c];
            }
            float *px = image + 3 * ((size_t)y * sc->width + x);
            for (int c = 0; c < 3; ++c) px[c] = acc[c] / (float)sc->spp;
        }
    if (counts) {
        counts[0] += cnt.distance; counts[1] += cnt.shadow; counts[2] += cnt.events; counts[3] += cnt.failed;
    }
    return GPIS_OK;
}

/* Columns [col0, col0 + cols) of one row (a band of the image rendered over many
 * threads); the same paths as gor_render. */
int gor_render_span(const gpis_medium_desc *md, const gpis_scene_desc *sc, float *image, uint64_t counts[4],
                    uint32_t row, uint32_t col0, uint32_t cols)
{
    if (!md || !sc || !image || sc->width == 0 || sc->height == 0 || sc->spp == 0) return GPIS_EINVAL;
    if (sc->phase > GPIS_PHASE_CONDUCTOR || row >= sc->height) return GPIS_EINVAL;
    pt_counts_t cnt = {0, 0, 0, 0};
    for (uint32_t x = col0; x < col0 + cols && x < sc->width; ++x) {
        float acc[3] = {0.0f, 0.0f, 0.0f};
        for (uint32_t s = 0; s < sc->spp; ++s) {
            float l[3];
            trace_path(md, sc, x, row, s, l, &cnt);
            for (int c = 0; c < 3; ++c) acc[c] = acc[c] + l[c];
        }
        float *px = image + 3 * ((size_t)row * sc->width + x);
        for (int c = 0; c < 3; ++c) px[c] = acc[c] / (float)sc->spp;
    }
    if (counts) {
        counts[0] += cnt.distance; counts[1] += cnt.shadow; counts[2] += cnt.events; counts[3] += cnt.failed;
    }
    return GPIS_OK;
}
