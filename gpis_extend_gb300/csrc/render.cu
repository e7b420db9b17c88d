// render.cu -- gpis_render: a wavefront path tracer around the GPIS medium.
//
// The subset of PathTracer::traceSample (PathTracer.cpp:49-292) described in
// gpis.h: pinhole camera, the medium's bounding cube as a forward boundary, one
// one-sided quad light outside the cube, GP surface events shaded by
// BRDFPhaseFunction over LambertBsdf, MirrorBsdf or ConductorBsdf
// (BRDFPhaseFunction.cpp:29-119, MirrorBsdf.cpp:31-109, ConductorBsdf.cpp:58-137)
// with handleVolume's direct lighting (TraceBase.cpp:993-1014, 798-874).
//
// Wavefront form: the paths of a chunk (all pixels x a run of samples) live in a
// device array.  Each round, k_rt_advance moves every path that is outside the
// cube to the cube or the light and queues one sampleDistance flight per path
// inside; the flight kernels trace the queue; k_rt_event applies
// GaussianProcessMedium::sampleDistance's decisions (GaussianProcessMedium.cpp:
// 289-381), queues the two direct-lighting transmittance flights of each GP
// event and samples the continuation; a second flight batch traces those
// shadow flights and k_rt_shadow adds the light that got through.  Specular
// events under the NEE or MIS scheme first queue their neePDF / neeGrad
// queries (one batch of gpis_nee per round); k_rt_nee turns the answers into
// shadow flights.  Every queue length stays in device memory, so a pass runs a
// fixed 2 * bounces + 4 rounds (enough for every path to end: at most a forward
// crossing and an event per bounce, plus entry and exit) replayed from one
// captured CUDA graph, with no host synchronization between rounds.
//
// This file is compiled with -fmad=false: every float expression rounds as the
// CPU restatement's (built with -ffp-contract=off), and path decisions use no
// trigonometry, so both make the same decisions from the same counter RNG.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/gpis.h"

extern "C" int gpis_internal_set_error(int code, const char *msg);
extern "C" const gpis_medium_desc *gpis_internal_ctx_medium(gpis_ctx *ctx, uint32_t index);

namespace {

constexpr float kInvPi = 0.31830988618379067f;
enum : uint32_t { D_JIT = 0, D_LU = 1, D_LV = 2, D_JS1 = 3, D_PHASE = 4, D_JS2 = 20, D_CONT = 21, D_PIX = 40 };
constexpr uint32_t kCameraBounce = 0xFFFFu;

enum : uint32_t { PF_ALIVE = 1u, PF_INSIDE = 2u, PF_SPECULAR = 4u, PF_FIRST = 8u };

// one path of the chunk (MediumState fields the medium reads and writes inline)
struct PathRec {
    float pos[3], dir[3], T[3], L[3];
    float last_val, last_aniso[3];
    uint32_t flags, bounce, pixel, sample;
    int32_t st_bounce, gp_id;
    uint32_t pad[2];
};

// what the medium state machine needs of the medium
struct RtMedium {
    float ratio;                // sigma_s / sigma_t
    int32_t max_bounces;
    uint32_t seed;
    uint32_t single_realization;
    uint32_t global_ctx;
    uint32_t scene_seed;
    // samplingScheme (SparseConvolutionNoise.cpp:68-76) of an event
    uint32_t scheme;            // the medium's 1D sampling scheme
    uint32_t scheme_uni;        // UNI whatever the event: single realization, 3D noise or sigma < 1e-6
    uint32_t xy_renewal_plus;   // correlationXY under Renewal+ (SE covariance): UNI at t = 0 after a conditioned flight
};

struct RtScene {
    gpis_scene_desc sc;
    float fwd[3], right[3], up[3];
    float ln[3];
    float area;
    float aspect;
    RtMedium M;                 // the scene's medium
    uint32_t medium;            // its index in the context
    uint32_t acc_off;           // first pixel of the scene in the image accumulator
    uint32_t n_pixels;
    uint32_t pad_;
};

// a run of samples of one scene inside a pass: paths [start, start + n_pixels * ns)
// hold samples s0 .. s0 + ns - 1 of every pixel (pixel-major); pixels
// [pix_start, pix_start + n_pixels) of the pass's pixel range
struct Seg {
    uint32_t start, scene, s0, ns, pix_start, pad_[3];
};

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ float rng(uint32_t seed, uint64_t path, uint32_t bounce, uint32_t dim)
{
    uint64_t k = mix64(((uint64_t)seed << 32) ^ path);
    k = mix64(k ^ (((uint64_t)bounce << 32) | dim));
    return (float)(k >> 40) * (1.0f / 16777216.0f);
}

__device__ __forceinline__ uint32_t rotl17(uint32_t h) { return (h << 17) | (h >> 15); }
__device__ __forceinline__ uint32_t xx_fin(uint32_t h)
{
    h = 2246822519u * (h ^ (h >> 15));
    h = 3266489917u * (h ^ (h >> 13));
    return h ^ (h >> 16);
}
// MathUtil::xxhash32(uint) and (Vec4u) (MathUtil.hpp:179-224)
__device__ __forceinline__ uint32_t xx1(uint32_t p) { return xx_fin(668265263u * rotl17(p + 374761393u)); }
__device__ __forceinline__ uint32_t xx4(uint32_t x, uint32_t y, uint32_t z, uint32_t w)
{
    uint32_t h = w + 374761393u + x * 3266489917u;
    h = 668265263u * rotl17(h);
    h += y * 3266489917u;
    h = 668265263u * rotl17(h);
    h += z * 3266489917u;
    h = 668265263u * rotl17(h);
    return xx_fin(h);
}

__device__ __forceinline__ float dot3(const float a[3], const float b[3])
{
    float s = a[0] * b[0];
    s = s + a[1] * b[1];
    s = s + a[2] * b[2];
    return s;
}

__device__ __forceinline__ void normalize3(float v[3])
{
    const float inv = 1.0f / sqrtf(dot3(v, v));
    v[0] = v[0] * inv; v[1] = v[1] * inv; v[2] = v[2] * inv;
}

struct PFrame { float t[3], b[3], n[3]; };

// TangentFrame(n) (TangentFrame.hpp:74-83)
__device__ void pframe(const float n_in[3], PFrame &f)
{
    f.n[0] = n_in[0]; f.n[1] = n_in[1]; f.n[2] = n_in[2];
    normalize3(f.n);
    const float *n = f.n;
    const float sign = copysignf(1.0f, n[2]);
    const float a = -1.0f / (sign + n[2]);
    const float b = n[0] * n[1] * a;
    f.t[0] = 1.0f + sign * n[0] * n[0] * a; f.t[1] = sign * b; f.t[2] = -sign * n[0];
    f.b[0] = b; f.b[1] = sign + n[1] * n[1] * a; f.b[2] = -n[1];
    normalize3(f.t);
    normalize3(f.b);
}

__device__ __forceinline__ void to_local(const PFrame &f, const float v[3], float o[3])
{
    o[0] = dot3(f.t, v); o[1] = dot3(f.b, v); o[2] = dot3(f.n, v);
}

__device__ __forceinline__ void to_global(const PFrame &f, const float l[3], float o[3])
{
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float s = f.t[i] * l[0];
        s = s + f.b[i] * l[1];
        s = s + f.n[i] * l[2];
        o[i] = s;
    }
}

__device__ void cosine_dir(uint32_t seed, uint64_t path, uint32_t bounce, uint32_t dim0, float w[3])
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

__device__ bool box_hit(const float o[3], const float d[3], float h, float &t0, float &t1)
{
    float tmin = -INFINITY, tmax = INFINITY;
    for (int i = 0; i < 3; ++i) {
        if (d[i] == 0.0f) {
            if (o[i] < -h || o[i] > h) return false;
            continue;
        }
        const float inv = 1.0f / d[i];
        float ta = (-h - o[i]) * inv, tb = (h - o[i]) * inv;
        if (ta > tb) { const float s = ta; ta = tb; tb = s; }
        tmin = fmaxf(tmin, ta);
        tmax = fminf(tmax, tb);
    }
    if (tmax < fmaxf(tmin, 0.0f)) return false;
    t0 = tmin;
    t1 = tmax;
    return true;
}

__device__ float light_hit(const RtScene &S, const float o[3], const float d[3])
{
    const gpis_scene_desc &sc = S.sc;
    const float den = dot3(d, S.ln);
    if (!(den < 0.0f)) return -1.0f;
    float co[3];
    for (int i = 0; i < 3; ++i) co[i] = sc.light_center[i] - o[i];
    const float t = dot3(co, S.ln) / den;
    if (!(t > 0.0f)) return -1.0f;
    float x[3];
    for (int i = 0; i < 3; ++i) x[i] = (o[i] + t * d[i]) - sc.light_center[i];
    const float s = dot3(x, sc.light_u) / dot3(sc.light_u, sc.light_u);
    const float r = dot3(x, sc.light_v) / dot3(sc.light_v, sc.light_v);
    if (fabsf(s) > 0.5f || fabsf(r) > 0.5f) return -1.0f;
    return t;
}

// SampleWarp::powerHeuristic (SampleWarp.hpp:189-199): the bounded ratio in double
__device__ __forceinline__ float power_heuristic(double pdf0, double pdf1)
{
    if (pdf0 >= pdf1) {
        const double ratio = pdf1 / pdf0;
        return (float)(1.0 / (1.0 + ratio * ratio));
    }
    const double ratio = pdf0 / pdf1;
    return (float)(ratio * ratio / (1.0 + ratio * ratio));
}

// Fresnel::conductorReflectance (Fresnel.hpp:102-123) of one channel; the
// mirror phase reflects everything
__device__ float conductor_reflectance(const gpis_scene_desc &sc, int c, float cos_i)
{
    if (sc.phase != GPIS_PHASE_CONDUCTOR) return 1.0f;
    const float eta = sc.eta[c], k = sc.k[c];
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

__device__ __forceinline__ uint32_t event_scheme(const RtMedium &M, bool conditioned, float t)
{
    if (M.scheme_uni) return GPIS_SCHEME_UNI;
    if (M.xy_renewal_plus && conditioned && t == 0.0f) return GPIS_SCHEME_UNI;
    return M.scheme;
}

// flight streams of one queue
struct Queue {
    float4 *origin_near, *dir_far, *prev;
    uint4 *seeds;
    float4 *rec;                // 2 per flight
    uint32_t *path;             // path index of each flight
    float4 *payload;            // shadow queues: contribution (rgb) and slot
    uint32_t *medium;           // medium index of each flight
    uint32_t *count;
};

// NEE queries of specular events (gpis_nee streams) and what shading needs
// after them: a = (T, light pdf), b = (albedo * F, unused), c = (direction,
// bounce | kind << 31); kind 0 = the light sample at the half-vector normal,
// kind 1 = the MIS phase sample at the event's normal
struct NeeQueue {
    float4 *origin_near, *dir_far, *prev;
    uint4 *seeds;
    float4 *point_t, *normal, *out;
    float4 *a, *b, *c;
    uint32_t *path;
    uint32_t *medium;
    uint32_t *count;
};

__device__ void push_flight(const Queue &q, uint32_t slot, const float o[3], const float d[3], float far_t,
                            uint32_t noise_seed, uint32_t normal_seed, uint32_t flags, float jitter, float pv,
                            const float pg[3], uint32_t medium)
{
    q.medium[slot] = medium;
    q.origin_near[slot] = make_float4(o[0], o[1], o[2], 0.0f);
    q.dir_far[slot] = make_float4(d[0], d[1], d[2], far_t);
    q.seeds[slot] = make_uint4(noise_seed, normal_seed, flags, __float_as_uint(jitter));
    q.prev[slot] = make_float4(pv, pg[0], pg[1], pg[2]);
}

// computeSeed and the request's normal seed (SparseConvolutionNoise.cpp:57-66,
// SparseConvolutionNoiseMedium.cpp:235-238)
__device__ void flight_seeds(const RtMedium &M, uint32_t px, uint32_t py, uint32_t s, uint32_t w, uint32_t &ns,
                             uint32_t &nm)
{
    const uint32_t sc = xx1(M.scene_seed);
    ns = M.seed + (M.single_realization ? 0u : xx4(px, py, s, M.global_ctx ? 0u : w) + sc);
    nm = xx4(px, py, s, w) + sc + 1u;
}

// the segment holding path i: the last one starting at or before i
__device__ __forceinline__ int find_seg(const Seg *segs, int n_segs, uint32_t i, bool by_pixel)
{
    int lo = 0, hi = n_segs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const uint32_t st = by_pixel ? segs[mid].pix_start : segs[mid].start;
        if (st <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_rt_camera(const RtScene *scenes, const Seg *segs, int n_segs, PathRec *paths, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Seg &g = segs[find_seg(segs, n_segs, i, false)];
    const RtScene &S = scenes[g.scene];
    const gpis_scene_desc &sc = S.sc;
    const uint32_t j = i - g.start;
    const uint32_t pixel = j / g.ns, s = g.s0 + j % g.ns;
    const uint32_t px = pixel % sc.width, py = pixel / sc.width;
    const uint64_t path = ((uint64_t)py * sc.width + px) * sc.spp + s;
    const float u0 = rng(sc.sampler_seed, path, kCameraBounce, D_PIX);
    const float u1 = rng(sc.sampler_seed, path, kCameraBounce, D_PIX + 1);
    const float sx = (2.0f * ((float)px + u0) / (float)sc.width - 1.0f) * sc.tan_half_fov * S.aspect;
    const float sy = (1.0f - 2.0f * ((float)py + u1) / (float)sc.height) * sc.tan_half_fov;
    PathRec r;
    for (int k = 0; k < 3; ++k) {
        r.pos[k] = sc.cam_pos[k];
        r.dir[k] = S.fwd[k] + sx * S.right[k] + sy * S.up[k];
        r.T[k] = 1.0f;
        r.L[k] = 0.0f;
        r.last_aniso[k] = 0.0f;
    }
    normalize3(r.dir);
    r.last_val = 0.0f;
    r.flags = PF_ALIVE | PF_SPECULAR | PF_FIRST;
    r.bounce = 0;
    r.pixel = pixel;
    r.sample = s;
    r.st_bounce = 0;
    r.gp_id = 0;
    r.pad[0] = g.scene;
    r.pad[1] = 0u;
    paths[i] = r;
}

// Outside the cube: reach the light, the cube or nothing.  Inside: queue the
// sampleDistance flight to the cube's exit.
__device__ void advance_one(const RtScene *scenes, PathRec *paths, uint32_t i, Queue q, unsigned long long *counters)
{
    PathRec r = paths[i];
    if (!(r.flags & PF_ALIVE)) return;
    const RtScene &S = scenes[r.pad[0]];
    const RtMedium &M = S.M;
    const gpis_scene_desc &sc = S.sc;
    if (r.bounce >= sc.max_bounces) {
        r.flags &= ~PF_ALIVE;
        paths[i] = r;
        return;
    }
    if (!(r.flags & PF_INSIDE)) {
        float t0, t1;
        const bool hb = box_hit(r.pos, r.dir, sc.box_half, t0, t1) && t0 > 0.0f;
        const float tl = light_hit(S, r.pos, r.dir);
        if (tl > 0.0f && (!hb || tl < t0)) {
            if (r.flags & PF_SPECULAR)
                for (int c = 0; c < 3; ++c) r.L[c] = r.L[c] + r.T[c] * sc.light_emission[c];
            r.flags &= ~PF_ALIVE;
            paths[i] = r;
            return;
        }
        if (!hb) {
            r.flags &= ~PF_ALIVE;
            paths[i] = r;
            return;
        }
        for (int k = 0; k < 3; ++k) {
            const float e = r.pos[k] + t0 * r.dir[k];
            r.pos[k] = fminf(fmaxf(e, -sc.box_half), sc.box_half);
        }
        r.flags |= PF_INSIDE;
    }
    float t0, t1;
    if (!box_hit(r.pos, r.dir, sc.box_half, t0, t1)) {
        // numerically outside after all: leaves the cube at once
        r.flags &= ~PF_INSIDE;
        paths[i] = r;
        return;
    }
    if (r.st_bounce >= M.max_bounces) {
        // sampleDistance fails at the medium's bounce limit (GaussianProcessMedium.cpp:222-232)
        r.flags &= ~PF_ALIVE;
        atomicAdd(counters + 1, 1ull);
        paths[i] = r;
        return;
    }
    if (!(t1 > 0.0f)) {
        // maxT <= nearT: the segment exits at once with weight 1 and no flight
        r.flags &= ~PF_INSIDE;
        paths[i] = r;
        return;
    }
    const uint32_t px = r.pixel % sc.width, py = r.pixel / sc.width;
    const uint64_t path = ((uint64_t)py * sc.width + px) * sc.spp + r.sample;
    uint32_t ns, nm;
    flight_seeds(M, px, py, r.sample, r.bounce, ns, nm);
    const bool first = (r.flags & PF_FIRST) != 0;
    const float zero[3] = {0.0f, 0.0f, 0.0f};
    const uint32_t slot = atomicAdd(q.count, 1u);
    push_flight(q, slot, r.pos, r.dir, t1, ns, nm, first ? GPIS_FLAG_FIRST_SCATTER : 0u,
                rng(sc.sampler_seed, path, r.bounce, D_JIT), first ? 0.0f : r.last_val, first ? zero : r.last_aniso,
                S.medium);
    q.path[slot] = i;
    paths[i] = r;
}

__global__ void k_rt_advance(const RtScene *scenes, PathRec *paths, const uint32_t *n_paths, Queue q,
                             unsigned long long *counters)
{
    const uint32_t n = *n_paths;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        advance_one(scenes, paths, i, q, counters);
}

// queue a direct-lighting transmittance flight from p along d on the medium
// state of segment `seg` conditioned on (pv, pg) (the light lies outside the
// cube, so the flight ends at the cube's exit)
__device__ void push_shadow(const RtScene &S, const RtMedium &M, const Queue &q, const PathRec &r, uint32_t seg,
                            uint32_t pi, const float p[3], const float d[3], float jitter, const float contrib[3],
                            uint32_t slot_kind, float *direct, float pv, const float pg[3])
{
    float t0, t1;
    if (!box_hit(p, d, S.sc.box_half, t0, t1) || !(t1 > 0.0f)) {
        // no medium in the way: the light arrives (the restatement's shadow() returns 1)
        for (int c = 0; c < 3; ++c) direct[3 * slot_kind + c] = contrib[c];
        return;
    }
    const uint32_t px = r.pixel % S.sc.width, py = r.pixel / S.sc.width;
    uint32_t ns, nm;
    flight_seeds(M, px, py, r.sample, seg, ns, nm);
    const uint32_t slot = atomicAdd(q.count, 1u);
    push_flight(q, slot, p, d, t1, ns, nm, GPIS_FLAG_SHADOW, jitter, pv, pg, S.medium);
    q.path[slot] = pi;
    q.payload[slot] = make_float4(contrib[0], contrib[1], contrib[2], __uint_as_float(slot_kind));
}

__device__ void push_nee(const NeeQueue &nq, const Queue &q, uint32_t k, uint32_t pi, const float p[3], float t,
                         const float nrm[3], const float T[3], float pdf_l, const float fr[3], const float d[3],
                         uint32_t b, uint32_t kind)
{
    const uint32_t slot = atomicAdd(nq.count, 1u);
    nq.origin_near[slot] = q.origin_near[k];
    nq.dir_far[slot] = q.dir_far[k];
    nq.seeds[slot] = q.seeds[k];
    nq.prev[slot] = q.prev[k];
    nq.medium[slot] = q.medium[k];
    nq.point_t[slot] = make_float4(p[0], p[1], p[2], t);
    nq.normal[slot] = make_float4(nrm[0], nrm[1], nrm[2], 0.0f);
    nq.a[slot] = make_float4(T[0], T[1], T[2], pdf_l);
    nq.b[slot] = make_float4(fr[0], fr[1], fr[2], 0.0f);
    nq.c[slot] = make_float4(d[0], d[1], d[2], __uint_as_float(b | (kind << 31)));
    nq.path[slot] = pi;
}

// GaussianProcessMedium::sampleDistance after the flight (GaussianProcessMedium.cpp:
// 289-381), then handleVolume (TraceBase.cpp:993-1048) for GP events.
__device__ void event_one(const RtScene *scenes, PathRec *paths, Queue q, uint32_t k, Queue sq, NeeQueue eq,
                          float *direct, unsigned long long *counters)
{
    const uint32_t pi = q.path[k];
    PathRec r = paths[pi];
    const RtScene &S = scenes[r.pad[0]];
    const RtMedium &M = S.M;
    const gpis_scene_desc &sc = S.sc;
    const float4 r0 = q.rec[2 * k], r1 = q.rec[2 * k + 1];
    const uint32_t status = __float_as_uint(r1.w);
    const float far_t = q.dir_far[k].w;
    float *dslot = direct + 6 * (size_t)pi;
#pragma unroll
    for (int c = 0; c < 6; ++c) dslot[c] = 0.0f;
    if ((status & 0xFFu) != GPIS_FLIGHT_OK) {
        r.flags &= ~PF_ALIVE;
        atomicAdd(counters + 1, 1ull);
        paths[pi] = r;
        return;
    }
    const bool hit = r1.y == 0.0f;
    const float t = r0.x;
    float aniso[3] = {r0.z, r0.w, r1.x};
    const bool first_before = (r.flags & PF_FIRST) != 0;
    if (hit) {
        r.gp_id = (int32_t)((status >> 8) & 0xFFu);
        r.last_val = 0.0f;
    } else {
        r.last_val = r0.y;
    }
    if (t < far_t) {
        r.last_aniso[0] = aniso[0]; r.last_aniso[1] = aniso[1]; r.last_aniso[2] = aniso[2];
        r.flags &= ~PF_FIRST;
        if (!isfinite((aniso[0] + aniso[1] + aniso[2]) / 3.0f)) {
            r.flags &= ~PF_ALIVE;
            atomicAdd(counters + 1, 1ull);
            paths[pi] = r;
            return;
        }
    }
    if (hit) {
        const double dd = (double)aniso[0] * r.dir[0] + (double)aniso[1] * r.dir[1] + (double)aniso[2] * r.dir[2];
        const double l2 = (double)aniso[0] * aniso[0] + (double)aniso[1] * aniso[1] + (double)aniso[2] * aniso[2];
        if (dd > 0 || l2 < 0.0000001f) {
            r.flags &= ~PF_ALIVE;
            atomicAdd(counters + 1, 1ull);
            paths[pi] = r;
            return;
        }
    }
    const float ts = fminf(t, far_t);
    float p[3];
    for (int i = 0; i < 3; ++i) p[i] = r.pos[i] + ts * r.dir[i];
    r.last_aniso[0] = aniso[0]; r.last_aniso[1] = aniso[1]; r.last_aniso[2] = aniso[2];
    r.flags &= ~PF_FIRST;
    r.st_bounce += 1;
    for (int c = 0; c < 3; ++c) r.T[c] = r.T[c] * M.ratio;
    if (!hit) {
        // forward boundary: the path continues outside the cube
        r.pos[0] = p[0]; r.pos[1] = p[1]; r.pos[2] = p[2];
        r.flags &= ~PF_INSIDE;
        paths[pi] = r;
        return;
    }
    atomicAdd(counters + 0, 1ull);
    PFrame f;
    pframe(aniso, f);
    float wi[3];
    const float nd[3] = {-r.dir[0], -r.dir[1], -r.dir[2]};
    to_local(f, nd, wi);
    if (sc.phase != GPIS_PHASE_LAMBERT) {
        // BRDFPhaseFunction over MirrorBsdf / ConductorBsdf: se.wi = frame.toLocal(-w).normalized(),
        // the reflection (-wi.x, -wi.y, wi.z) with weight albedo * F(wi.z)
        normalize3(wi);
        float fr[3], wrg[3];
        const float wr[3] = {-wi[0], -wi[1], wi[2]};
        for (int c = 0; c < 3; ++c) fr[c] = sc.albedo[c] * conductor_reflectance(sc, c, wi[2]);
        to_global(f, wr, wrg);
        normalize3(wrg);
        const uint32_t scheme = event_scheme(M, !first_before, t);
        const uint32_t px = r.pixel % sc.width, py = r.pixel / sc.width;
        const uint64_t path = ((uint64_t)py * sc.width + px) * sc.spp + r.sample;
        const uint32_t seed = sc.sampler_seed, b = r.bounce;
        if (b + 1 < sc.max_bounces) {
            if (scheme != GPIS_SCHEME_UNI) {
                // volumeLightSample: neePDF / neeGrad at the half-vector normal, shaded by k_rt_nee
                const float lu = rng(seed, path, b, D_LU) - 0.5f, lv = rng(seed, path, b, D_LV) - 0.5f;
                float ld[3];
                for (int i = 0; i < 3; ++i)
                    ld[i] = ((sc.light_center[i] + lu * sc.light_u[i]) + lv * sc.light_v[i]) - p[i];
                const float dist2 = dot3(ld, ld), dist = sqrtf(dist2);
                for (int i = 0; i < 3; ++i) ld[i] = ld[i] / dist;
                const float cos_l = -dot3(ld, S.ln);
                if (cos_l > 0.0f) {
                    const float pdf_l = dist2 / (S.area * cos_l);
                    float wo[3], hl[3], hw[3];
                    to_local(f, ld, wo);
                    normalize3(wo);
                    for (int i = 0; i < 3; ++i) hl[i] = (wi[i] + wo[i]) * 0.5f;
                    to_global(f, hl, hw);
                    normalize3(hw);
                    push_nee(eq, q, k, pi, p, ts, hw, r.T, pdf_l, fr, ld, b, 0u);
                }
            }
            if (scheme != GPIS_SCHEME_NEE) {
                // volumePhaseSample: the reflection, when it reaches the light
                const float tlh = light_hit(S, p, wrg);
                if (tlh > 0.0f) {
                    if (scheme == GPIS_SCHEME_MIS) {
                        // weighed against neePDF at the event's normal in k_rt_nee
                        const float cl = -dot3(wrg, S.ln);
                        const float pdf_l = (tlh * tlh) / (S.area * cl);
                        push_nee(eq, q, k, pi, p, ts, f.n, r.T, pdf_l, fr, wrg, b, 1u);
                    } else {
                        const float w = 1.0f;
                        float contrib[3];
                        for (int c = 0; c < 3; ++c) contrib[c] = r.T[c] * (fr[c] * sc.light_emission[c] * w);
                        push_shadow(S, M, sq, r, b + 1, pi, p, wrg, rng(seed, path, b, D_JS2), contrib, 1u, dslot,
                                    r.last_val, r.last_aniso);
                    }
                }
            }
        }
        for (int c = 0; c < 3; ++c) r.T[c] = r.T[c] * fr[c];
        for (int i = 0; i < 3; ++i) { r.pos[i] = p[i]; r.dir[i] = wrg[i]; }
        r.flags &= ~PF_SPECULAR;
        r.bounce += 1;
        paths[pi] = r;
        return;
    }
    if (!(wi[2] > 0.0f)) {
        r.flags &= ~PF_ALIVE;
        atomicAdd(counters + 1, 1ull);
        paths[pi] = r;
        return;
    }
    const uint32_t px = r.pixel % sc.width, py = r.pixel / sc.width;
    const uint64_t path = ((uint64_t)py * sc.width + px) * sc.spp + r.sample;
    const uint32_t seed = sc.sampler_seed, b = r.bounce;
    if (b + 1 < sc.max_bounces) {
        // volumeLightSample
        const float lu = rng(seed, path, b, D_LU) - 0.5f, lv = rng(seed, path, b, D_LV) - 0.5f;
        float ld[3];
        for (int i = 0; i < 3; ++i)
            ld[i] = ((sc.light_center[i] + lu * sc.light_u[i]) + lv * sc.light_v[i]) - p[i];
        const float dist2 = dot3(ld, ld), dist = sqrtf(dist2);
        for (int i = 0; i < 3; ++i) ld[i] = ld[i] / dist;
        const float cos_l = -dot3(ld, S.ln);
        if (cos_l > 0.0f) {
            const float pdf_l = dist2 / (S.area * cos_l);
            float wo[3];
            to_local(f, ld, wo);
            if (wo[2] > 0.0f) {
                const float pdf_p = wo[2] * kInvPi;
                const float w = power_heuristic(pdf_l, pdf_p);
                float contrib[3];
                for (int c = 0; c < 3; ++c) {
                    const float fc = sc.albedo[c] * kInvPi * wo[2];
                    contrib[c] = r.T[c] * (fc * sc.light_emission[c] / pdf_l * w);
                }
                push_shadow(S, M, sq, r, b + 1, pi, p, ld, rng(seed, path, b, D_JS1), contrib, 0u, dslot, r.last_val,
                            r.last_aniso);
            }
        }
        // volumePhaseSample
        float wl[3], wg[3];
        cosine_dir(seed, path, b, D_PHASE, wl);
        to_global(f, wl, wg);
        normalize3(wg);
        const float tlh = light_hit(S, p, wg);
        if (tlh > 0.0f && wl[2] > 0.0f) {
            const float pdf_p = wl[2] * kInvPi;
            const float cl = -dot3(wg, S.ln);
            const float pdf_l = (tlh * tlh) / (S.area * cl);
            const float w = power_heuristic(pdf_p, pdf_l);
            float contrib[3];
            for (int c = 0; c < 3; ++c) contrib[c] = r.T[c] * (sc.albedo[c] * sc.light_emission[c] * w);
            push_shadow(S, M, sq, r, b + 1, pi, p, wg, rng(seed, path, b, D_JS2), contrib, 1u, dslot, r.last_val,
                        r.last_aniso);
        }
    }
    // the continuation (BRDFPhaseFunction::sample over LambertBsdf)
    float wl[3], wg[3];
    cosine_dir(seed, path, b, D_CONT, wl);
    to_global(f, wl, wg);
    normalize3(wg);
    for (int c = 0; c < 3; ++c) r.T[c] = r.T[c] * sc.albedo[c];
    for (int i = 0; i < 3; ++i) { r.pos[i] = p[i]; r.dir[i] = wg[i]; }
    r.flags &= ~PF_SPECULAR;
    r.bounce += 1;
    paths[pi] = r;
}

__global__ void k_rt_event(const RtScene *scenes, PathRec *paths, Queue q, const uint32_t *counts, Queue sq,
                           NeeQueue eq, float *direct, unsigned long long *counters)
{
    const uint32_t n = counts[0];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        event_one(scenes, paths, q, k, sq, eq, direct, counters);
}

// after the NEE queries of specular events: the light sample's BSDF value
// albedo * F * neePDF and its transmittance flight conditioned on neeGrad
// (volumeLightSample with MirrorBsdf::eval / evalGrad), or the MIS weight of the
// phase sample against neePDF (MirrorBsdf::sample's pdf)
__device__ void nee_shade_one(const RtScene *scenes, const PathRec *paths, NeeQueue eq, uint32_t k, Queue sq,
                              float *direct)
{
    const uint32_t pi = eq.path[k];
    const PathRec &r = paths[pi];
    const RtScene &S = scenes[r.pad[0]];
    const RtMedium &M = S.M;
    const gpis_scene_desc &sc = S.sc;
    const float4 o = eq.out[k], pa = eq.a[k], pb = eq.b[k], pc = eq.c[k], pt = eq.point_t[k];
    const uint32_t bk = __float_as_uint(pc.w), b = bk & 0x7FFFFFFFu, kind = bk >> 31;
    const float T[3] = {pa.x, pa.y, pa.z}, fr[3] = {pb.x, pb.y, pb.z};
    const float p[3] = {pt.x, pt.y, pt.z}, d[3] = {pc.x, pc.y, pc.z};
    const float pdf_l = pa.w, pdf = o.x;
    const uint32_t px = r.pixel % sc.width, py = r.pixel / sc.width;
    const uint64_t path = ((uint64_t)py * sc.width + px) * sc.spp + r.sample;
    float *dslot = direct + 6 * (size_t)pi;
    const uint32_t scheme = M.scheme;
    float contrib[3];
    if (kind == 0u) {
        float fl[3];
        for (int c = 0; c < 3; ++c) fl[c] = fr[c] * pdf;
        if (!(fl[0] != 0.0f || fl[1] != 0.0f || fl[2] != 0.0f)) return;
        const float w = scheme == GPIS_SCHEME_MIS ? power_heuristic(pdf_l, pdf) : 1.0f;
        for (int c = 0; c < 3; ++c) contrib[c] = T[c] * (fl[c] * sc.light_emission[c] / pdf_l * w);
        const float g[3] = {o.y, o.z, o.w};
        push_shadow(S, M, sq, r, b + 1, pi, p, d, rng(sc.sampler_seed, path, b, D_JS1), contrib, 0u, dslot,
                    r.last_val, g);
    } else {
        const float w = power_heuristic(pdf, pdf_l);
        for (int c = 0; c < 3; ++c) contrib[c] = T[c] * (fr[c] * sc.light_emission[c] * w);
        push_shadow(S, M, sq, r, b + 1, pi, p, d, rng(sc.sampler_seed, path, b, D_JS2), contrib, 1u, dslot,
                    r.last_val, r.last_aniso);
    }
}

__global__ void k_rt_nee(const RtScene *scenes, const PathRec *paths, NeeQueue eq, const uint32_t *counts, Queue sq,
                         float *direct)
{
    const uint32_t n = counts[2];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        nee_shade_one(scenes, paths, eq, k, sq, direct);
}

// a transmittance of 1 lets the queued contribution through
__device__ void shadow_one(Queue sq, uint32_t k, float *direct)
{
    const float4 pl = sq.payload[k];
    const uint32_t kind = __float_as_uint(pl.w);
    const float4 r1 = sq.rec[2 * k + 1];
    // transmittance 1 only for a finished flight that misses (resumeTransmittance)
    if ((__float_as_uint(r1.w) & 0xFFu) == GPIS_FLIGHT_OK && r1.y > 0.0f) {
        float *d = direct + 6 * (size_t)sq.path[k] + 3 * kind;
        d[0] = pl.x; d[1] = pl.y; d[2] = pl.z;
    }
}

__global__ void k_rt_shadow(Queue sq, const uint32_t *counts, float *direct)
{
    const uint32_t n = counts[1];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        shadow_one(sq, k, direct);
}

// L += light sample, then L += phase sample, in the restatement's order
__global__ void k_rt_collect(PathRec *paths, const uint32_t *qpath, const uint32_t *counts, float *direct)
{
    const uint32_t n = counts[0];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t pi = qpath[k];
        float *d = direct + 6 * (size_t)pi;
        PathRec &r = paths[pi];
        for (int c = 0; c < 3; ++c) r.L[c] = r.L[c] + d[c];
        for (int c = 0; c < 3; ++c) r.L[c] = r.L[c] + d[3 + c];
    }
}

// the round's queue lengths into the render's flight counters
__global__ void k_rt_tally(const uint32_t *counts, unsigned long long *counters)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        counters[2] += counts[0];
        counters[3] += counts[1];
        counters[4] += counts[2];
    }
}

// pixel t of the pass: add its ns samples (in sample order) to the scene's accumulator
__global__ void k_rt_accumulate(const RtScene *scenes, const Seg *segs, int n_segs, const PathRec *paths,
                                uint32_t n_pix, float *acc)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_pix) return;
    const Seg &g = segs[find_seg(segs, n_segs, t, true)];
    const uint32_t px = t - g.pix_start;
    float *a = acc + 3 * ((size_t)scenes[g.scene].acc_off + px);
    float v[3] = {a[0], a[1], a[2]};
    for (uint32_t s = 0; s < g.ns; ++s) {
        const PathRec &r = paths[g.start + (size_t)px * g.ns + s];
        for (int c = 0; c < 3; ++c) v[c] = v[c] + r.L[c];
    }
    a[0] = v[0]; a[1] = v[1]; a[2] = v[2];
}

// the mean over each scene's spp
__global__ void k_rt_finish(const RtScene *scenes, int n_scenes, float *acc, uint32_t total_pixels)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total_pixels) return;
    int lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (scenes[mid].acc_off <= t) lo = mid;
        else hi = mid - 1;
    }
    const float spp = (float)scenes[lo].sc.spp;
    for (int c = 0; c < 3; ++c) acc[3 * (size_t)t + c] = acc[3 * (size_t)t + c] / spp;
}

inline void hnorm(float v[3])
{
    float s = v[0] * v[0];
    s = s + v[1] * v[1];
    s = s + v[2] * v[2];
    const float inv = 1.0f / std::sqrt(s);
    v[0] = v[0] * inv; v[1] = v[1] * inv; v[2] = v[2] * inv;
}

inline void hcross(const float a[3], const float b[3], float o[3])
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

struct DevBuf {
    std::vector<void *> ptrs;
    ~DevBuf() { for (void *p : ptrs) cudaFree(p); }
    template <class T>
    cudaError_t alloc(T *&p, size_t n)
    {
        void *v = nullptr;
        cudaError_t e = cudaMalloc(&v, std::max<size_t>(n, 1) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back(v);
        p = static_cast<T *>(v);
        return e;
    }
};

int cuda_fail(cudaError_t e, const char *what)
{
    static thread_local char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return gpis_internal_set_error(GPIS_EIO, buf);
}

}  // namespace

#define RT_TRY(expr, what)                              \
    do {                                                \
        cudaError_t e_ = (expr);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

extern "C" int gpis_internal_submit_live(gpis_ctx *ctx, const gpis_flight_soa *in, const gpis_result_soa *out,
                                         uint32_t cap, const uint32_t *n_dev, void *cuda_stream,
                                         const float *intervals);
extern "C" int gpis_internal_features_live(gpis_ctx *ctx, const gpis_flight_soa *in, float *features, uint32_t cap,
                                           const uint32_t *n_dev, void *cuda_stream);
extern "C" int gpis_internal_infer_live(gpis_proposal *p, const gpis_flight_soa *in, const float *features,
                                        float *intervals, uint32_t cap, const uint32_t *n_dev, void *cuda_stream);
extern "C" int gpis_internal_proposal_quiesce(gpis_proposal *p);
extern "C" int gpis_internal_nee_live(gpis_ctx *ctx, const gpis_nee_soa *in, float *out, uint32_t cap,
                                      const uint32_t *n_dev, void *cuda_stream);
extern "C" int gpis_internal_ctx_info(gpis_ctx *ctx, int *num_sms, int *profiling, int *prepare_runs);
extern "C" uint32_t gpis_internal_render_pass(gpis_ctx *ctx);

namespace {

// scene and medium constants of one scene (host)
int make_scene(gpis_ctx *ctx, const gpis_scene_desc &sc, RtScene &S, bool &specular_nee)
{
    if (sc.width == 0 || sc.height == 0 || sc.spp == 0 || sc.max_bounces == 0)
        return gpis_internal_set_error(GPIS_EINVAL, "width, height, spp and max_bounces must be > 0");
    if (sc.phase > GPIS_PHASE_CONDUCTOR) return gpis_internal_set_error(GPIS_EINVAL, "unknown phase");
    if (!(sc.box_half > 0.0f) || !(sc.tan_half_fov > 0.0f))
        return gpis_internal_set_error(GPIS_EINVAL, "box_half and tan_half_fov must be > 0");
    if ((uint64_t)sc.width * sc.height > (1ull << 28))
        return gpis_internal_set_error(GPIS_ERANGE, "image too large");
    const gpis_medium_desc *md = gpis_internal_ctx_medium(ctx, sc.medium);
    if (!md) return gpis_internal_set_error(GPIS_EINVAL, "unknown medium index");
    const float sa = md->sigma_a * md->density, ss = md->sigma_s * md->density;
    if (!(ss > 0.0f)) return gpis_internal_set_error(GPIS_ENOTSUP, "the renderer needs a scattering medium (sigma_s > 0)");
    RtMedium &M = S.M;
    M.ratio = ss / (sa + ss);
    M.max_bounces = md->max_bounces;
    M.seed = md->seed;
    M.single_realization = md->single_realization;
    M.global_ctx = md->correlation_context == GPIS_CTX_GLOBAL;
    M.scene_seed = sc.scene_seed;
    M.scheme = md->sampling_scheme;
    M.scheme_uni = md->single_realization || !md->one_d_sampling || md->sigma < 1e-6f;
    M.xy_renewal_plus = md->correlation_xy && !md->single_realization &&
                        md->correlation_context == GPIS_CTX_RENEWAL_PLUS && md->ls_kind == GPIS_LS_CONSTANT;
    specular_nee = sc.phase != GPIS_PHASE_LAMBERT && !M.scheme_uni && M.scheme != GPIS_SCHEME_UNI;
    S.sc = sc;
    for (int i = 0; i < 3; ++i) S.fwd[i] = sc.cam_target[i] - sc.cam_pos[i];
    hnorm(S.fwd);
    hcross(S.fwd, sc.cam_up, S.right);
    hnorm(S.right);
    hcross(S.right, S.fwd, S.up);
    hcross(sc.light_u, sc.light_v, S.ln);
    {
        float v = S.ln[0] * S.ln[0];
        v = v + S.ln[1] * S.ln[1];
        v = v + S.ln[2] * S.ln[2];
        S.area = std::sqrt(v);
    }
    hnorm(S.ln);
    S.aspect = (float)sc.width / (float)sc.height;
    S.medium = sc.medium;
    S.n_pixels = sc.width * sc.height;
    S.pad_ = 0;
    return GPIS_OK;
}

}  // namespace

// Render a batch of scenes in one wavefront: the paths of all scenes share the
// flight batches of every round (the flight kernels take each flight's medium),
// so many small images fill the GPU together.  A pass holds up to 2^22 paths
// (GPIS_TUNE_RENDER_PASS_PATHS)
// (runs of samples of one or several scenes); each pass runs rounds of the
// bounce loop until every path has ended, with the queue lengths in device
// memory, so a round needs no host synchronization and is replayed from one
// captured CUDA graph (launched directly while the context profiles its kernels).
extern "C" int gpis_render_batch_proposed(gpis_ctx *ctx, gpis_proposal *prop, const gpis_scene_desc *scenes,
                                          uint32_t n_scenes, float *const *images, gpis_render_stats *stats)
{
    if (!ctx || !scenes || !images || n_scenes == 0) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    if (prop) {
        const int qrc = gpis_internal_proposal_quiesce(prop);
        if (qrc) return qrc;
    }
    std::vector<RtScene> hs(n_scenes);
    bool any_nee = false;
    uint32_t max_bounces = 0;
    uint64_t total_pixels = 0, total_paths = 0;
    for (uint32_t k = 0; k < n_scenes; ++k) {
        if (!images[k]) return gpis_internal_set_error(GPIS_EINVAL, "null image");
        bool nee = false;
        int rc = make_scene(ctx, scenes[k], hs[k], nee);
        if (rc) return rc;
        any_nee = any_nee || nee;
        max_bounces = std::max(max_bounces, scenes[k].max_bounces);
        hs[k].acc_off = (uint32_t)total_pixels;
        total_pixels += hs[k].n_pixels;
        total_paths += (uint64_t)hs[k].n_pixels * scenes[k].spp;
        if (total_pixels > 0xFFFFFFFFull) return gpis_internal_set_error(GPIS_ERANGE, "images too large");
    }
    // passes: runs of samples, up to `target` paths each (one sample of an image
    // larger than that makes a pass of its own)
    const uint32_t target = gpis_internal_render_pass(ctx);
    std::vector<std::vector<Seg>> passes(1);
    std::vector<uint32_t> pass_n(1, 0), pass_pix(1, 0);
    for (uint32_t k = 0; k < n_scenes; ++k) {
        const uint32_t np = hs[k].n_pixels;
        uint32_t left = scenes[k].spp, s0 = 0;
        while (left > 0) {
            uint32_t room = target > pass_n.back() ? target - pass_n.back() : 0;
            if (room < np && pass_n.back() > 0) {
                passes.emplace_back();
                pass_n.push_back(0);
                pass_pix.push_back(0);
                room = target;
            }
            const uint32_t ns = std::max(1u, std::min(left, room / std::max(1u, np)));
            Seg g;
            g.start = pass_n.back();
            g.scene = k;
            g.s0 = s0;
            g.ns = ns;
            g.pix_start = pass_pix.back();
            g.pad_[0] = g.pad_[1] = g.pad_[2] = 0;
            passes.back().push_back(g);
            pass_n.back() += np * ns;
            pass_pix.back() += np;
            s0 += ns;
            left -= ns;
        }
    }
    uint32_t cap = 0, max_segs = 0;
    for (size_t p = 0; p < passes.size(); ++p) {
        cap = std::max(cap, pass_n[p]);
        max_segs = std::max<uint32_t>(max_segs, (uint32_t)passes[p].size());
    }
    int num_sms = 1, profiling = 0, prepare_runs = 1;
    gpis_internal_ctx_info(ctx, &num_sms, &profiling, &prepare_runs);

    DevBuf mem;
    RtScene *d_scenes;
    Seg *d_segs;
    PathRec *paths;
    float *direct, *acc;
    Queue q{}, sq{};
    NeeQueue eq{};
    uint32_t *counts, *n_paths;
    unsigned long long *dcnt;
    RT_TRY(mem.alloc(d_scenes, n_scenes), "allocate scenes");
    RT_TRY(mem.alloc(d_segs, max_segs), "allocate segments");
    RT_TRY(mem.alloc(paths, cap), "allocate paths");
    RT_TRY(mem.alloc(direct, (size_t)cap * 6), "allocate direct light");
    RT_TRY(mem.alloc(acc, (size_t)total_pixels * 3), "allocate images");
    RT_TRY(mem.alloc(counts, 3), "allocate queue counters");
    RT_TRY(mem.alloc(n_paths, 1), "allocate path count");
    RT_TRY(mem.alloc(dcnt, 5), "allocate counters");
    // the learned arm: features and proposed intervals of the distance queue
    float *feats = nullptr, *ivals = nullptr;
    if (prop) {
        RT_TRY(mem.alloc(feats, (size_t)cap * 24), "allocate proposal features");
        RT_TRY(mem.alloc(ivals, (size_t)cap * 4), "allocate proposal intervals");
    }
    for (Queue *qq : {&q, &sq}) {
        const size_t m = qq == &q ? cap : 2 * (size_t)cap;
        RT_TRY(mem.alloc(qq->origin_near, m), "allocate queue");
        RT_TRY(mem.alloc(qq->dir_far, m), "allocate queue");
        RT_TRY(mem.alloc(qq->prev, m), "allocate queue");
        RT_TRY(mem.alloc(qq->seeds, m), "allocate queue");
        RT_TRY(mem.alloc(qq->rec, 2 * m), "allocate queue");
        RT_TRY(mem.alloc(qq->path, m), "allocate queue");
        RT_TRY(mem.alloc(qq->payload, m), "allocate queue");
        RT_TRY(mem.alloc(qq->medium, m), "allocate queue");
    }
    q.count = counts;
    sq.count = counts + 1;
    eq.count = counts + 2;
    if (any_nee) {
        // at most two queries per event: the light sample and the MIS phase sample
        const size_t m = 2 * (size_t)cap;
        RT_TRY(mem.alloc(eq.origin_near, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.dir_far, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.prev, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.seeds, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.point_t, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.normal, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.out, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.a, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.b, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.c, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.path, m), "allocate NEE queue");
        RT_TRY(mem.alloc(eq.medium, m), "allocate NEE queue");
    }
    cudaStream_t st;
    RT_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "create stream");
    struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{st};
    cudaEvent_t e0, e1;
    RT_TRY(cudaEventCreate(&e0), "create event");
    RT_TRY(cudaEventCreate(&e1), "create event");
    struct EventGuard { cudaEvent_t a, b; ~EventGuard() { cudaEventDestroy(a); cudaEventDestroy(b); } } eg{e0, e1};
    RT_TRY(cudaMemcpyAsync(d_scenes, hs.data(), hs.size() * sizeof(RtScene), cudaMemcpyHostToDevice, st),
           "upload scenes");
    RT_TRY(cudaMemsetAsync(acc, 0, (size_t)total_pixels * 3 * sizeof(float), st), "clear images");
    RT_TRY(cudaMemsetAsync(dcnt, 0, 5 * sizeof(unsigned long long), st), "clear counters");
    RT_TRY(cudaMemsetAsync(counts, 0, 3 * sizeof(uint32_t), st), "clear queue counters");

    gpis_flight_soa fin{reinterpret_cast<float *>(q.origin_near), reinterpret_cast<float *>(q.dir_far),
                        reinterpret_cast<uint32_t *>(q.seeds), reinterpret_cast<float *>(q.prev), q.medium};
    gpis_result_soa fout{reinterpret_cast<float *>(q.rec)};
    gpis_flight_soa sin{reinterpret_cast<float *>(sq.origin_near), reinterpret_cast<float *>(sq.dir_far),
                        reinterpret_cast<uint32_t *>(sq.seeds), reinterpret_cast<float *>(sq.prev), sq.medium};
    gpis_result_soa sout{reinterpret_cast<float *>(sq.rec)};
    gpis_nee_soa nin{};
    if (any_nee) {
        nin.flight = gpis_flight_soa{reinterpret_cast<float *>(eq.origin_near), reinterpret_cast<float *>(eq.dir_far),
                                     reinterpret_cast<uint32_t *>(eq.seeds), reinterpret_cast<float *>(eq.prev),
                                     eq.medium};
        nin.point_t = reinterpret_cast<const float *>(eq.point_t);
        nin.normal = reinterpret_cast<const float *>(eq.normal);
    }
    // the flight scratch for the largest batch, allocated before any capture (the
    // queue counters are zero here, so these launches trace nothing)
    int rc = gpis_internal_submit_live(ctx, &sin, &sout, 2 * cap, counts + 1, st, nullptr);
    if (rc) return rc;
    if (any_nee) {
        rc = gpis_internal_nee_live(ctx, &nin, reinterpret_cast<float *>(eq.out), 2 * cap, counts + 2, st);
        if (rc) return rc;
    }
    const unsigned tb = 128;
    const unsigned gs = (unsigned)std::max(1, num_sms * 8);   // grid of the grid-stride kernels
    // one round of the bounce loop; every length it needs is in device memory
    auto round = [&]() -> int {
        cudaError_t e = cudaMemsetAsync(counts, 0, 3 * sizeof(uint32_t), st);
        if (e != cudaSuccess) return cuda_fail(e, "clear queue counters");
        k_rt_advance<<<gs, tb, 0, st>>>(d_scenes, paths, n_paths, q, dcnt);
        int r;
        if (prop) {
            r = gpis_internal_features_live(ctx, &fin, feats, cap, counts, st);
            if (r) return r;
            r = gpis_internal_infer_live(prop, &fin, feats, ivals, cap, counts, st);
            if (r) return r;
        }
        r = gpis_internal_submit_live(ctx, &fin, &fout, cap, counts, st, ivals);
        if (r) return r;
        k_rt_event<<<gs, tb, 0, st>>>(d_scenes, paths, q, counts, sq, eq, direct, dcnt);
        if (any_nee) {
            r = gpis_internal_nee_live(ctx, &nin, reinterpret_cast<float *>(eq.out), 2 * cap, counts + 2, st);
            if (r) return r;
            k_rt_nee<<<gs, tb, 0, st>>>(d_scenes, paths, eq, counts, sq, direct);
        }
        r = gpis_internal_submit_live(ctx, &sin, &sout, 2 * cap, counts + 1, st, nullptr);
        if (r) return r;
        k_rt_shadow<<<gs, tb, 0, st>>>(sq, counts, direct);
        k_rt_collect<<<gs, tb, 0, st>>>(paths, q.path, counts, direct);
        k_rt_tally<<<1, 32, 0, st>>>(counts, dcnt);
        return GPIS_OK;
    };
    // kernels of one round: advance, event, shadow, collect, tally, and per flight batch
    // prepare (when it runs), march, resume and finish; NEE adds its kernel and the shading
    const uint64_t per_batch = 3 + (prepare_runs ? 1 : 0);
    const uint64_t per_round = 5 + 2 * per_batch + (any_nee ? 2 : 0) + (prop ? 2 : 0);
    const uint32_t rounds = 2 * max_bounces + 4;
    cudaGraphExec_t gexec = nullptr;
    struct GraphGuard { cudaGraphExec_t g; ~GraphGuard() { if (g) cudaGraphExecDestroy(g); } } gg{nullptr};
    bool graphed = false;
    if (!profiling) {
        // a capture that fails leaves the rounds to direct launches
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            rc = round();
            const cudaError_t ce = cudaStreamEndCapture(st, &graph);
            if (rc == GPIS_OK && ce == cudaSuccess && graph &&
                cudaGraphInstantiate(&gexec, graph, 0) == cudaSuccess) {
                gg.g = gexec;
                graphed = true;
            } else {
                gexec = nullptr;
            }
            if (graph) cudaGraphDestroy(graph);
        }
        (void)cudaGetLastError();
    }
    if (stats) stats->graphed = graphed ? 1u : 0u;
    RT_TRY(cudaEventRecord(e0, st), "record event");
    uint64_t n_launch = 0;
    for (size_t p = 0; p < passes.size(); ++p) {
        const std::vector<Seg> &segs = passes[p];
        RT_TRY(cudaMemcpyAsync(d_segs, segs.data(), segs.size() * sizeof(Seg), cudaMemcpyHostToDevice, st),
               "upload segments");
        RT_TRY(cudaMemcpyAsync(n_paths, &pass_n[p], sizeof(uint32_t), cudaMemcpyHostToDevice, st), "upload pass size");
        k_rt_camera<<<(pass_n[p] + tb - 1) / tb, tb, 0, st>>>(d_scenes, d_segs, (int)segs.size(), paths, pass_n[p]);
        n_launch += 1;
        for (uint32_t k = 0; k < rounds; ++k) {
            if (gexec) {
                RT_TRY(cudaGraphLaunch(gexec, st), "launch the round graph");
            } else {
                rc = round();
                if (rc) return rc;
            }
            n_launch += per_round;
        }
        k_rt_accumulate<<<(pass_pix[p] + tb - 1) / tb, tb, 0, st>>>(d_scenes, d_segs, (int)segs.size(), paths,
                                                                    pass_pix[p], acc);
        n_launch += 1;
        // the host's segment table and pass size must outlive their asynchronous copies
        RT_TRY(cudaStreamSynchronize(st), "synchronize pass");
    }
    k_rt_finish<<<(unsigned)((total_pixels + tb - 1) / tb), tb, 0, st>>>(d_scenes, (int)n_scenes, acc,
                                                                         (uint32_t)total_pixels);
    n_launch += 1;
    RT_TRY(cudaEventRecord(e1, st), "record event");
    for (uint32_t k = 0; k < n_scenes; ++k)
        RT_TRY(cudaMemcpyAsync(images[k], acc + 3 * (size_t)hs[k].acc_off, (size_t)hs[k].n_pixels * 3 * sizeof(float),
                               cudaMemcpyDeviceToHost, st),
               "read image");
    unsigned long long hc[5] = {0, 0, 0, 0, 0};
    RT_TRY(cudaMemcpyAsync(hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost, st), "read counters");
    RT_TRY(cudaStreamSynchronize(st), "synchronize render");
    RT_TRY(cudaGetLastError(), "render kernels");
    if (stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        stats->paths = total_paths;
        stats->distance_flights = hc[2];
        stats->shadow_flights = hc[3];
        stats->medium_events = hc[0];
        stats->failed = hc[1];
        stats->ms = ms;
        stats->launches = n_launch;
        stats->nee_queries = hc[4];
        stats->passes = (uint32_t)passes.size();
    }
    return GPIS_OK;
}

extern "C" int gpis_render_batch(gpis_ctx *ctx, const gpis_scene_desc *scenes, uint32_t n_scenes, float *const *images,
                                 gpis_render_stats *stats)
{
    return gpis_render_batch_proposed(ctx, nullptr, scenes, n_scenes, images, stats);
}

extern "C" int gpis_render(gpis_ctx *ctx, const gpis_scene_desc *scene, float *image_rgb, gpis_render_stats *stats)
{
    if (!ctx || !scene || !image_rgb) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    float *const images[1] = {image_rgb};
    return gpis_render_batch(ctx, scene, 1, images, stats);
}
