/*
 * gpis_oracle.c -- CPU restatement of the reference sparse-convolution-noise
 * GPIS ray-flight path.  TEST INFRASTRUCTURE ONLY (the checker of the parity
 * tests, the smoke check and the benchmark's CPU baseline); the product
 * library never links it.
 *
 * Precision: "float mode" keeps every float/double choice of the reference
 * C++ (Vec3f vs Vec3d, double march parameter t, float field values).  The
 * reference was built with MSVC, whose <cmath> resolves exp/sqrt of a float
 * argument to the float overloads.  sqrtf is correctly rounded everywhere; the
 * float exp is not specified by IEEE 754 and differs between C libraries in the
 * last bit (glibc's expf differs from the correctly rounded value on about 1e-4
 * of the splat arguments), so this file evaluates the reference's float exp as
 * the correctly rounded float of e^x, rexpf(x) = (float)exp((double)x): a value
 * that any implementation can reproduce, which the GPU's precise evaluator
 * does.  Build
 * with -ffp-contract=off so that no multiply-add is fused (SSE2 x86-64 and the
 * reference CPU build have no FMA contraction).
 *
 * Scope: stationary squared-exponential covariance with diagonal anisotropy,
 * 1D (isotropic ray space) and 3D (world space) sparse convolution noise,
 * Global / None / Renewal / Renewal+ memory models (with correlationXY),
 * sphere / homogeneous / plane / torus / torus-union-plane / dense-grid means,
 * and the nonstationary sin-cos length-scale field with octaves.
 */
#define _GNU_SOURCE
#include "gpis_oracle.h"

/* multi-resolution grid: _base (SparseConvolutionNoise.cpp:49), read at run time so
 * that logf / powf of it are the float library's, and the range of levels a
 * medium may use */
static volatile float mr_base_v = 2.5f;
#define MR_BASE ((float)mr_base_v)
#define MR_LEVEL_MAX 16

#include <math.h>

/* the reference's float exp, correctly rounded (see the header) */
static inline float rexpf(float x) { return (float)exp((double)x); }
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* Hash and sampler                                                          */
/* ------------------------------------------------------------------------ */
#define P2 2246822519u
#define P3 3266489917u
#define P4 668265263u
#define P5 374761393u

static inline uint32_t rotl17(uint32_t h) { return (h << 17) | (h >> 15); }

/* MathUtil.hpp:179-187 */
uint32_t gor_xxhash32_1(uint32_t p)
{
    uint32_t h = p + P5;
    h = P4 * rotl17(h);
    h = P2 * (h ^ (h >> 15));
    h = P3 * (h ^ (h >> 13));
    return h ^ (h >> 16);
}

/* MathUtil.hpp:190-198 */
uint32_t gor_xxhash32_2(uint32_t x, uint32_t y)
{
    uint32_t h = y + P5 + x * P3;
    h = P4 * rotl17(h);
    h = P2 * (h ^ (h >> 15));
    h = P3 * (h ^ (h >> 13));
    return h ^ (h >> 16);
}

/* MathUtil.hpp:212-224 */
uint32_t gor_xxhash32_4(uint32_t x, uint32_t y, uint32_t z, uint32_t w)
{
    uint32_t h = w + P5 + x * P3;
    h = P4 * rotl17(h);
    h += y * P3;
    h = P4 * rotl17(h);
    h += z * P3;
    h = P4 * rotl17(h);
    h = P2 * (h ^ (h >> 15));
    h = P3 * (h ^ (h >> 13));
    return h ^ (h >> 16);
}

/* UniformSampler.hpp:41-75 with sequence 0 (increment 1) */
typedef struct { uint64_t s; } pcg_t;

static inline uint32_t pcg_next(pcg_t *g)
{
    uint64_t old = g->s;
    g->s = old * 6364136223846793005ULL + 1ULL;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((uint32_t)(-(int32_t)rot) & 31u));
}

/* BitManip.hpp:47-50 */
static inline float norm_uint(uint32_t i)
{
    union { uint32_t u; float f; } v;
    v.u = (i >> 9u) | 0x3F800000u;
    return v.f - 1.0f;
}

static inline float pcg_1d(pcg_t *g) { return norm_uint(pcg_next(g)); }

static inline void pcg_set_state(pcg_t *g, uint64_t s)
{
    g->s = s;
    (void)pcg_1d(g);
    (void)pcg_1d(g);
}

void gor_pcg_stream(uint64_t state, uint32_t n, float *out_float, uint32_t *out_raw)
{
    pcg_t g;
    pcg_set_state(&g, state);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t r = pcg_next(&g);
        if (out_raw) out_raw[i] = r;
        if (out_float) out_float[i] = norm_uint(r);
    }
}

/* Box-Muller, Gaussian.cpp:23-35.  PI is the float constant of Angle.hpp:8, so
 * 2*PI is formed in float before it meets the double u2. */
static void rand_normal_2(pcg_t *g, double out[2])
{
    const float PIf = 3.1415926536f;
    double u1 = pcg_1d(g);
    double u2 = pcg_1d(g);
    double r = sqrt(-2 * log(1. - u1));
    float two_pi = 2 * PIf;
    double x = cos(two_pi * u2);
    double y = sin(two_pi * u2);
    out[0] = r * x;
    out[1] = r * y;
}

void gor_normal_pair(uint64_t state, uint32_t pairs, double *out)
{
    pcg_t g;
    pcg_set_state(&g, state);
    for (uint32_t i = 0; i < pairs; ++i) rand_normal_2(&g, out + 2 * i);
}

/* ------------------------------------------------------------------------ */
/* Small float/double vector helpers with the reference's operation order   */
/* ------------------------------------------------------------------------ */
static inline float dot3f(const float a[3], const float b[3])
{
    float s = a[0] * b[0];
    s += a[1] * b[1];
    s += a[2] * b[2];
    return s;
}

static inline void normalize3f(const float v[3], float o[3])
{
    float inv = 1.0f / sqrtf(dot3f(v, v));
    o[0] = v[0] * inv; o[1] = v[1] * inv; o[2] = v[2] * inv;
}

static inline double dot3d(const double a[3], const double b[3])
{
    double s = a[0] * b[0];
    s += a[1] * b[1];
    s += a[2] * b[2];
    return s;
}

/* TangentFrame(const Vec3f &n), TangentFrame.hpp:74-98 */
typedef struct { float n[3], t[3], b[3]; } frame_t;

static void frame_make(const float n_in[3], frame_t *f)
{
    normalize3f(n_in, f->n);
    const float *n = f->n;
    float sign = copysignf(1.0f, n[2]);
    const float a = -1.0f / (sign + n[2]);
    const float b = n[0] * n[1] * a;
    float t[3] = {1.0f + sign * n[0] * n[0] * a, sign * b, -sign * n[0]};
    float bt[3] = {b, sign + n[1] * n[1] * a, -n[1]};
    normalize3f(t, f->t);
    normalize3f(bt, f->b);
}

static inline void frame_to_local(const frame_t *f, const float p[3], float o[3])
{
    o[0] = dot3f(f->t, p);
    o[1] = dot3f(f->b, p);
    o[2] = dot3f(f->n, p);
}

static inline void frame_to_global(const frame_t *f, const float p[3], float o[3])
{
    for (int i = 0; i < 3; ++i)
        o[i] = f->t[i] * p[0] + f->b[i] * p[1] + f->n[i] * p[2];
}

/* ------------------------------------------------------------------------ */
/* Medium constants                                                          */
/* ------------------------------------------------------------------------ */
typedef struct {
    gpis_medium_desc d;
    uint32_t n_imp;          /* uint(impulseDensity), SparseConvolutionNoise.cpp:470 */
    int activate_cond;       /* SparseConvolutionNoise.cpp:38 */
    int scheme;              /* SparseConvolutionNoise.cpp:40-43 */
    int nonstationary;       /* ls field present */
    float lc;                /* _l_conv = l*sqrt(2)/2, GPFunctions.cpp:661 */
    float l_aniso[3];        /* _l_aniso = l_conv*aniso, GPFunctions.cpp:665 */
    float l_inv[3];          /* _l_aniso_inv (world_to_local diagonal) */
    float kr_iso;            /* splattingKernelRadius(true, 1), GPFunctions.cpp:706-709 */
    float kr_world;          /* splattingKernelRadius(false, 1), GPFunctions.cpp:711-718 */
    float ls_max;            /* sparseConvNoiseMaxLateralScale */
    int multires;            /* 2-level multi-resolution blend (SparseConvolutionNoise.cpp:47-49) */
    int iso3d;               /* 3D noise in isotropic ray space (isotropic_3D_sampling) */
    /* grid mean copy */
    const float *grid_vox;
} om_t;

static int om_init(om_t *m, const gpis_medium_desc *d)
{
    memset(m, 0, sizeof(*m));
    m->d = *d;
    if (!(d->length_scale > 0.0f) || !(d->kernel_scale > 0.0f) || !(d->impulse_density > 0.0f))
        return GPIS_EINVAL;
    if (d->n_octaves < 1 || d->n_octaves > 4) return GPIS_EINVAL;
    if (d->mean_kind == GPIS_MEAN_GRID && (!d->grid || !d->grid->voxels)) return GPIS_EINVAL;
    /* octaves are this restatement's composition of 1D realizations */
    if (d->n_octaves != 1 && !d->one_d_sampling) return GPIS_ENOTSUP;
    if (d->ls_kind != GPIS_LS_CONSTANT && !(d->ls_max > 0.0f)) return GPIS_EINVAL;
    /* _multiResolutionGrid = !isStationaryKernel() && useMultiResolutionGrid() */
    m->multires = d->multires && d->ls_kind != GPIS_LS_CONSTANT;
    if (m->multires) {
        if (d->n_octaves != 1) return GPIS_ENOTSUP;
        /* the levels need ls(p) > 0 everywhere: a - |b| > 0 for the sin-cos field, and
           levels inside [-MR_LEVEL_MAX, MR_LEVEL_MAX) */
        const float lo = d->ls_params[0] - fabsf(d->ls_params[1]), hi = d->ls_params[0] + fabsf(d->ls_params[1]);
        if (!(lo > 0.0f) || !isfinite(hi)) return GPIS_EINVAL;
        if (floorf(logf(lo) / logf(MR_BASE)) < -MR_LEVEL_MAX || floorf(logf(hi) / logf(MR_BASE)) >= MR_LEVEL_MAX - 1)
            return GPIS_ERANGE;
    }
    m->n_imp = (uint32_t)d->impulse_density;
    m->iso3d = d->isotropic_3d_sampling && !d->one_d_sampling;
    m->activate_cond = !d->single_realization &&
        (d->correlation_context == GPIS_CTX_RENEWAL || d->correlation_context == GPIS_CTX_RENEWAL_PLUS);
    m->scheme = GPIS_SCHEME_UNI;
    if (!d->single_realization && d->one_d_sampling) m->scheme = (int)d->sampling_scheme;
    /* sqrt(2.f) resolves to the float overload (MSVC <cmath>). */
    m->lc = d->length_scale * sqrtf(2.f) / 2;
    for (int i = 0; i < 3; ++i) {
        m->l_aniso[i] = m->lc * d->aniso[i];
        float inv = 1.0f / m->l_aniso[i];
        if (isinf(inv) || isnan(inv)) inv = 0;   /* filterWithZero, GPFunctions.hpp:153-162 */
        m->l_inv[i] = inv;
    }
    m->nonstationary = d->ls_kind != GPIS_LS_CONSTANT;
    /* the maximum lateral scale enters the brute-force transforms only */
    m->ls_max = m->nonstationary && !m->multires ? d->ls_max : 1.0f;
    float mtx = fmaxf(fmaxf(m->l_aniso[0], m->l_aniso[1]), m->l_aniso[2]);
    /* NonstationaryCovariance::splattingKernelRadius (GPFunctions.cpp:1250-1254) scales
       localScale by the maximum lateral scale in brute-force mode. */
    m->kr_iso = d->kernel_scale;
    m->kr_world = d->kernel_scale * (1.0f * m->ls_max) * mtx;
    m->grid_vox = d->mean_kind == GPIS_MEAN_GRID ? d->grid->voxels : NULL;
    return GPIS_OK;
}

/* Length-scale field ls(p) (ProceduralNonstationaryCovariance::getKernelScale,
 * GPFunctions.cpp:1738-1744) for the sin-cos field. */
static inline float ls_field(const om_t *m, const float p[3])
{
    if (!m->nonstationary) return 1.0f;
    const float *q = m->d.ls_params;
    /* a code-defined procedural vector evaluated on Vec3d(p), returned as float
       (getKernelScale, GPFunctions.cpp:1738-1744) */
    return (float)((double)q[0] + (double)q[1] * sin((double)q[2] * p[0]) * cos((double)q[3] * p[2]));
}

/* nonStationarySplattingKernelScale, GPFunctions.cpp:1229-1235: ls(p) / ls_max by
 * brute force, 1 on the multi-resolution grid */
static inline float ns_scale(const om_t *m, const float p[3])
{
    if (!m->nonstationary || m->multires) return 1.0f;
    return ls_field(m, p) / m->ls_max;
}

/* transformPosDirWorldtoLocal (GPFunctions.cpp:634-636; nonstationary 1270-1273:
 * the maximum lateral scale by brute force, the level scale on the
 * multi-resolution grid) */
static inline float ns_transform_scale(const om_t *m, float scale)
{
    return m->nonstationary && !m->multires ? m->ls_max : scale;
}

static inline void w2l_pos(const om_t *m, const float v[3], float scale, float o[3])
{
    float s = ns_transform_scale(m, scale);
    for (int i = 0; i < 3; ++i) o[i] = (m->l_inv[i] * v[i]) / s;
}

/* transformGradLocaltoWorld (GPFunctions.cpp:644; nonstationary 1285-1288) */
static inline void l2w_grad(const om_t *m, const float v[3], float scale, float o[3])
{
    float s = ns_transform_scale(m, scale);
    for (int i = 0; i < 3; ++i) o[i] = (m->l_inv[i] * v[i]) / s;
}

/* transformGradWorldtoLocal (GPFunctions.cpp:642; nonstationary 1280-1283) */
static inline void w2l_grad(const om_t *m, const float v[3], float scale, float o[3])
{
    float s = ns_transform_scale(m, scale);
    for (int i = 0; i < 3; ++i) o[i] = (m->l_aniso[i] * v[i]) * s;
}

/* kernelScaleLevelRatio (SparseConvolutionNoise.cpp:101-111), float overloads of
 * log / floor / pow: (scale of the low level, of the high level, weight of the
 * low level, weight of the high level), the weights of unit total variance. */
static void level_ratio(const om_t *m, const float p[3], float info[4])
{
    const float ls = ls_field(m, p);
    const float level_low = floorf(logf(ls) / logf(MR_BASE));
    const float level_high = level_low + 1;
    const float sl = powf(MR_BASE, level_low), sh = powf(MR_BASE, level_high);
    const float frac = (ls - sl) / (sh - sl);
    const double den = sqrt(1.0 - 2.0 * frac + 2.0 * frac * frac);
    info[0] = sl;
    info[1] = sh;
    info[2] = (float)((1.0 - frac) / den);
    info[3] = (float)(frac / den);
}

/* the per-level seed offset floor(log(scale) / log(base)) of evaluateNoise1DNormalized
 * (SparseConvolutionNoise.cpp:385) */
static inline uint32_t level_seed(float scale)
{
    return (uint32_t)(int)floorf(logf(scale) / logf(MR_BASE));
}

/* ------------------------------------------------------------------------ */
/* Means (double, as MeanFunction::mean / dmean_da)                         */
/* ------------------------------------------------------------------------ */
static float grid_voxel(const gpis_mean_grid *g, int x, int y, int z)
{
    x = x - g->origin[0]; y = y - g->origin[1]; z = z - g->origin[2];
    x = x < 0 ? 0 : (x > g->dims[0] - 1 ? g->dims[0] - 1 : x);
    y = y < 0 ? 0 : (y > g->dims[1] - 1 ? g->dims[1] - 1 : y);
    z = z < 0 ? 0 : (z > g->dims[2] - 1 ? g->dims[2] - 1 : z);
    size_t idx = ((size_t)z * (size_t)g->dims[1] + (size_t)y) * (size_t)g->dims[0] + (size_t)x;
    return g->voxels[idx];
}

/* Dense trilinear grid: RaySegmentBatch.cu:73-95 (the tabulated mean baked to a grid). */
static float grid_mean(const gpis_mean_grid *g, const float p[3])
{
    const float *M = g->world_to_index;
    float q[3];
    for (int r = 0; r < 3; ++r) {
        float v = M[4 * r + 0] * p[0];
        v += M[4 * r + 1] * p[1];
        v += M[4 * r + 2] * p[2];
        v += M[4 * r + 3];
        q[r] = fminf(fmaxf(v, g->clamp_min[r]), g->clamp_max[r]);
    }
    int x = (int)floorf(q[0]), y = (int)floorf(q[1]), z = (int)floorf(q[2]);
    float fx = q[0] - (float)x, fy = q[1] - (float)y, fz = q[2] - (float)z;
    float layer[2];
    for (int dz = 0; dz < 2; ++dz) {
        float row[2];
        for (int dy = 0; dy < 2; ++dy) {
            float a = grid_voxel(g, x, y + dy, z + dz);
            float b = grid_voxel(g, x + 1, y + dy, z + dz);
            row[dy] = a + fx * (b - a);
        }
        layer[dz] = row[0] + fy * (row[1] - row[0]);
    }
    return (layer[0] + fz * (layer[1] - layer[0]) + g->offset) * g->scale;
}

static double torus_sdf(const float *q, const double a[3])
{
    double x = a[0] - q[0], y = a[1] - q[1], z = a[2] - q[2];
    double rxz = sqrt(x * x + z * z) - q[3];
    return sqrt(rxz * rxz + y * y) - q[4];
}

/* mean_weight_space (GaussianProcess.cpp:382-396): value and GP id. */
static double mean_value(const om_t *m, const double a[3], int *id)
{
    const float *q = m->d.mean_params;
    *id = 0;
    switch (m->d.mean_kind) {
    case GPIS_MEAN_SPHERE: {   /* SphericalMean, GPFunctions.hpp:986-988 */
        double v[3] = {a[0] - q[0], a[1] - q[1], a[2] - q[2]};
        return sqrt(dot3d(v, v)) - q[3];
    }
    case GPIS_MEAN_HOMOGENEOUS:
        return q[0];
    case GPIS_MEAN_PLANE:
        return (double)q[0] * a[0] + (double)q[1] * a[1] + (double)q[2] * a[2] - q[3];
    case GPIS_MEAN_TORUS:
        return torus_sdf(q, a);
    case GPIS_MEAN_TORUS_PLANE: {
        double t = torus_sdf(q, a);
        double pl = a[1] - q[5];
        if (pl < t) { *id = 1; return pl; }
        return t;
    }
    case GPIS_MEAN_GRID: {     /* TabulatedMean::mean, GPFunctions.cpp:165-172 */
        float p[3] = {(float)a[0], (float)a[1], (float)a[2]};
        return grid_mean(m->d.grid, p);
    }
    default:
        return 0.0;
    }
}

static void mean_grad(const om_t *m, const double a[3], double g[3])
{
    const float *q = m->d.mean_params;
    int id;
    switch (m->d.mean_kind) {
    case GPIS_MEAN_SPHERE: {   /* (a-c).normalized(), GPFunctions.hpp:990-992 */
        double v[3] = {a[0] - q[0], a[1] - q[1], a[2] - q[2]};
        double inv = 1.0 / sqrt(dot3d(v, v));
        for (int i = 0; i < 3; ++i) g[i] = v[i] * inv;
        return;
    }
    case GPIS_MEAN_HOMOGENEOUS:
        g[0] = g[1] = g[2] = 0.0;
        return;
    case GPIS_MEAN_PLANE:
        g[0] = q[0]; g[1] = q[1]; g[2] = q[2];
        return;
    case GPIS_MEAN_TORUS:
    case GPIS_MEAN_TORUS_PLANE: {
        (void)mean_value(m, a, &id);
        if (m->d.mean_kind == GPIS_MEAN_TORUS_PLANE && id == 1) {
            g[0] = 0.0; g[1] = 1.0; g[2] = 0.0;
            return;
        }
        double x = a[0] - q[0], y = a[1] - q[1], z = a[2] - q[2];
        double rxz = sqrt(x * x + z * z);
        double s = rxz - q[3];
        double len = sqrt(s * s + y * y);
        double dr = s / len, dy = y / len;
        g[0] = rxz > 0 ? dr * x / rxz : 0.0;
        g[1] = dy;
        g[2] = rxz > 0 ? dr * z / rxz : 0.0;
        return;
    }
    case GPIS_MEAN_GRID: {     /* TabulatedMean::dmean_da, GPFunctions.cpp:179-190 */
        double eps = 0.001;
        double v0, vx, vy, vz, b[3];
        b[0] = a[0] + eps; b[1] = a[1]; b[2] = a[2]; vx = mean_value(m, b, &id);
        b[0] = a[0]; b[1] = a[1] + eps; vy = mean_value(m, b, &id);
        b[1] = a[1]; b[2] = a[2] + eps; vz = mean_value(m, b, &id);
        v0 = mean_value(m, a, &id);
        g[0] = (vx - v0) / eps; g[1] = (vy - v0) / eps; g[2] = (vz - v0) / eps;
        return;
    }
    default:
        g[0] = g[1] = g[2] = 0.0;
    }
}

/* ------------------------------------------------------------------------ */
/* Realization (SparseConvolutionNoiseRealization)                          */
/* ------------------------------------------------------------------------ */
typedef struct {
    float value_scale;
    float gs[3];
    float origin[3];
    float tgn[3];            /* target_gradient_noise (1D) */
    int has_grad_obs;
} coef_t;

typedef struct {
    const om_t *m;
    uint32_t noise_seed, normal_seed;
    int octave;              /* octave index of the realization */
    coef_t c1, c3;
} real_t;

/* Octave k: amplitude, length-scale multiplier and seed offset.  For one
 * octave this is the reference realization with amplitude sigma. */
static inline float oct_sigma(const om_t *m, int k)
{
    return m->d.n_octaves == 1 ? m->d.sigma : m->d.octave_sigma[k];
}

static inline float oct_scale(const om_t *m, int k)
{
    return m->d.n_octaves == 1 ? 1.0f : m->d.octave_scale[k];
}

static inline uint32_t oct_seed(const om_t *m, int k)
{
    return m->d.n_octaves == 1 ? 0u : m->d.octave_seed[k];
}

/* amplitude sparseConvNoiseAmplitude(p) */
static inline float amplitude(const real_t *r)
{
    return oct_sigma(r->m, r->octave);
}

/* --- 1D noise ----------------------------------------------------------- */

/* 1D query coordinate p_iso_ray.z (evaluateNoise1DNormalized, SparseConvolutionNoise.cpp:381-384),
 * with the octave's length-scale multiplier folded into the iso transform. */
static float coord_1d(const real_t *r, const float p[3], const float dir[3], float ks, frame_t *f)
{
    const om_t *m = r->m;
    float sc = oct_scale(m, r->octave);
    float diso[3], diso_n[3], piso[3];
    w2l_pos(m, dir, 1.0f, diso);
    normalize3f(diso, diso_n);
    frame_make(diso_n, f);
    w2l_pos(m, p, ks, piso);
    if (sc != 1.0f)
        for (int i = 0; i < 3; ++i) piso[i] = piso[i] / sc;
    return dot3f(f->n, piso);
}

/* noise1D + cell1D (SparseConvolutionNoise.cpp:454-485) in float mode;
 * returns (value, d/dz) of the raw sum.  ls = nonstationary kernel scale at the
 * query (splattingKernel1D takes the scale at the query, GPFunctions.cpp:582-588). */
static void noise1d_f(const om_t *m, float z, uint32_t seed, float ls, float out[2])
{
    const float kr = m->kr_iso;
    float tg = z / kr;
    float fl = floorf(tg);
    float frac = tg - fl;
    int i = (int)fl;
    float sv = 0.0f, sg = 0.0f;
    for (int dx = -1; dx <= 1; ++dx) {
        float tl = frac - (float)dx;
        pcg_t g;
        pcg_set_state(&g, (uint64_t)(uint32_t)(gor_xxhash32_2((uint32_t)(i + dx), seed) + 1u));
        float cv = 0.0f, cg = 0.0f;
        for (uint32_t k = 0; k < m->n_imp; ++k) {
            float ti = pcg_1d(&g);
            float wi = pcg_1d(&g) < 0.5f ? -1.0f : 1.0f;
            float tp = tl - ti;
            if (tp * tp < 1.0f) {
                float ab = kr * tl - kr * ti;
                float den = 2.0f * (ls * ls);   /* splattingKernel1DVal, GPFunctions.cpp:845-848 */
                float f = rexpf(-(ab * ab / den));
                float gr = (float)(-2.0 * (double)ab / (double)den * (double)f);
                cv += wi * f;
                cg += wi * gr;
            }
        }
        sv += cv;
        sg += cg;
    }
    out[0] = sv;
    out[1] = sg;
}

/* Same impulse set (float inside test), every value in FP64. */
static void noise1d_d(const om_t *m, float z, uint32_t seed, double ls, double out[2])
{
    const float kr = m->kr_iso;
    float tg = z / kr;
    float fl = floorf(tg);
    float frac = tg - fl;
    int i = (int)fl;
    double sv = 0.0, sg = 0.0;
    double fracd = (double)z / (double)kr - (double)fl;
    for (int dx = -1; dx <= 1; ++dx) {
        float tl = frac - (float)dx;
        pcg_t g;
        pcg_set_state(&g, (uint64_t)(uint32_t)(gor_xxhash32_2((uint32_t)(i + dx), seed) + 1u));
        for (uint32_t k = 0; k < m->n_imp; ++k) {
            float ti = pcg_1d(&g);
            double wi = pcg_1d(&g) < 0.5f ? -1.0 : 1.0;
            float tp = tl - ti;
            if (tp * tp < 1.0f) {
                double ab = (double)kr * (fracd - dx - (double)ti);
                double f = exp(-(ab * ab) / (2.0 * ls * ls));
                sv += wi * f;
                sg += wi * (-ab / (ls * ls) * f);
            }
        }
    }
    out[0] = sv;
    out[1] = sg;
}

/* covarianceKernel1DVal / 1stGrad / 2D2ndGrad / 2D2ndGradFor3DNormal
 * (GPFunctions.cpp:850-875) with localScale a (1 when stationary). */
static void cov1d_f(float d, float a, float out[4])
{
    /* covarianceKernel1DVal(ab, a) = splattingKernel1DVal(ab, a*sqrt(2)); sqrt(2) is the
       double overload (integer argument), the product is passed as float. */
    float s2 = (float)((double)a * sqrt(2));
    float den2 = (float)(2.0 * (double)(s2 * s2));
    float f = rexpf(-(d * d / den2));
    float g1 = (float)(-2.0 * (double)d / (double)den2 * (double)f);
    float den4 = (float)(4.0 * (double)(a * a));
    float gr = (float)(-2.0 * (double)d / (double)den4);
    float g2 = (float)(((double)(gr * gr) - 2.0 / (double)den4) * (double)f);
    float g2n = (float)(-2.0 / (double)den4 * (double)f);
    out[0] = f; out[1] = g1; out[2] = g2; out[3] = g2n;
}

static void cov1d_d(double d, double a, double out[4])
{
    double f = exp(-d * d / (4.0 * a * a));
    double g1 = -d / (2.0 * a * a) * f;
    double gr = -d / (2.0 * a * a);
    out[0] = f; out[1] = g1; out[2] = (gr * gr - 1.0 / (2.0 * a * a)) * f;
    out[3] = -1.0 / (2.0 * a * a) * f;
}

/* getNonstationaryCovSplatCov1D for the isotropic ls field (GPFunctions.cpp:1723-1734) */
static inline float splat_cov_1d(const om_t *m, const float pq[3], const float pc[3])
{
    if (!m->nonstationary) return 1.0f;
    float a = ns_scale(m, pq), b = ns_scale(m, pc);
    float s = (float)(0.5 * (double)(a * a + b * b));
    return sqrtf(s);
}

/* evaluateNoise1DNormalized (SparseConvolutionNoise.cpp:379-417) at kernel spatial
 * scale ks (1, or a level scale of the multi-resolution grid; low selects the
 * origin's level weight of the conditioning splats).
 * out = (value, cond x splat, cond y splat, dvalue/dz); float mode or FP64. */
static void noise1d_level(const real_t *r, const float p[3], const float dir[3], int cond,
                          int dbl, float ks, int low, double out[4])
{
    const om_t *m = r->m;
    frame_t f;
    float z = coord_1d(r, p, dir, ks, &f);
    uint32_t seed = r->noise_seed + oct_seed(m, r->octave) + (m->multires ? level_seed(ks) : 0u);
    float ls = ns_scale(m, p);
    /* sparseConvNoiseVariance1D: impulseDensity/kernelRadius (float) * sqrt(pi) * localScale */
    float var = (float)((double)(m->d.impulse_density / m->kr_iso) * (sqrt(M_PI) * (double)ls));
    float normf = sqrtf(var);
    double v[2];
    if (!dbl) {
        float s[2];
        noise1d_f(m, z, seed, ls, s);
        s[0] /= normf;
        s[1] /= normf;
        v[0] = s[0]; v[1] = s[1];
    } else {
        noise1d_d(m, z, seed, (double)ls, v);
        double nd = sqrt((double)m->d.impulse_density / (double)m->kr_iso * sqrt(M_PI) * (double)ls);
        v[0] /= nd;
        v[1] /= nd;
    }
    double gx = 0.0, gy = 0.0;
    if (m->activate_cond && cond) {
        const coef_t *c = &r->c1;
        float oiso[3], oray[3];
        float sc = oct_scale(m, r->octave);
        /* kernelSpatialScale: the level scale, or the octave's length multiplier */
        const float kss = m->multires ? ks : sc;
        /* origin_scale_factor: the origin's weight of this level (multi-resolution) */
        float osf = 1.0f;
        if (m->multires) {
            float oinfo[4];
            level_ratio(m, c->origin, oinfo);
            osf = low ? oinfo[2] : oinfo[3];
        }
        w2l_pos(m, c->origin, ks, oiso);
        if (sc != 1.0f)
            for (int i = 0; i < 3; ++i) oiso[i] = oiso[i] / sc;
        frame_to_local(&f, oiso, oray);
        float a = splat_cov_1d(m, p, c->origin);
        if (!dbl) {
            float d = z - oray[2];
            float k[4];
            cov1d_f(d, a, k);
            float vs0 = c->value_scale * k[0], vs1 = c->value_scale * k[1];
            float gz0 = kss * c->gs[2] * k[1], gz1 = kss * c->gs[2] * k[2];
            float nv = (float)v[0] + osf * (vs0 + gz0);
            float ng = (float)v[1] + osf * (vs1 + gz1);
            v[0] = nv; v[1] = ng;
            if (m->d.correlation_xy) {
                float kt[4], kb[4];
                cov1d_f(d, a, kt);   /* the tangent/bitangent directions only enter through a */
                cov1d_f(d, a, kb);
                gx = osf * kss * c->gs[0] * kt[3];
                gy = osf * kss * c->gs[1] * kb[3];
            }
        } else {
            double d = (double)z - (double)oray[2];
            double k[4];
            cov1d_d(d, (double)a, k);
            v[0] += (double)osf * (c->value_scale * k[0] + (double)kss * c->gs[2] * k[1]);
            v[1] += (double)osf * (c->value_scale * k[1] + (double)kss * c->gs[2] * k[2]);
            if (m->d.correlation_xy) {
                gx = (double)osf * kss * c->gs[0] * k[3];
                gy = (double)osf * kss * c->gs[1] * k[3];
            }
        }
    }
    out[0] = v[0]; out[1] = gx; out[2] = gy; out[3] = v[1];
}

/* evaluateValueNoise1D (SparseConvolutionNoise.cpp:156-165): one level, or the
 * blend w_low * noise_low + w_high * noise_high of the two levels around ls(p)
 * on the multi-resolution grid (every component blended the same way). */
static void noise1d_norm(const real_t *r, const float p[3], const float dir[3], int cond,
                         int dbl, double out[4])
{
    const om_t *m = r->m;
    if (!m->multires) {
        noise1d_level(r, p, dir, cond, dbl, 1.0f, 1, out);
        return;
    }
    float info[4];
    level_ratio(m, p, info);
    double lo[4], hi[4];
    noise1d_level(r, p, dir, cond, dbl, info[0], 1, lo);
    noise1d_level(r, p, dir, cond, dbl, info[1], 0, hi);
    for (int k = 0; k < 4; ++k)
        out[k] = dbl ? (double)info[2] * lo[k] + (double)info[3] * hi[k]
                     : (double)(info[2] * (float)lo[k] + info[3] * (float)hi[k]);
}

/* --- 3D noise ---------------------------------------------------------- */

static inline void draw3(pcg_t *g, uint32_t order, float p[3])
{
    if (order == 0) {          /* Vec3f(next1D(), next1D(), next1D()) evaluated right to left */
        p[2] = pcg_1d(g);
        p[1] = pcg_1d(g);
        p[0] = pcg_1d(g);
    } else {
        p[0] = pcg_1d(g);
        p[1] = pcg_1d(g);
        p[2] = pcg_1d(g);
    }
}

/* getInvCovMtx diagonal (GPFunctions.cpp:784-812): world space (the inverse
 * squared length scales over sqr(globalScale)) or isotropic space (identity),
 * isCov, then over sqr(localScale) a, times 0.5. */
static inline void inv_cov3(const om_t *m, int iso, int is_cov, float a, float gs, float M[3])
{
    for (int i = 0; i < 3; ++i) {
        float v = iso ? 1.0f : m->l_inv[i] * m->l_inv[i];
        if (!iso && gs != 1.0f) v /= gs * gs;
        if (is_cov) v *= 0.5f;
        v /= a * a;
        v *= 0.5f;
        M[i] = v;
    }
}

/* One level of evaluateNoise3D (SparseConvolutionNoise.cpp:142-165): the cell size
 * kernelRadius, the kernelSpatialScale and its seed offset floor(log(s)/log(2.5)). */
typedef struct { float kr, ks; uint32_t seed_add; } lv3_t;

/* The levels of a 3D evaluation at p: one (stationary: world kernelRadius and
 * worldSamplingSpatialScale 1; brute-force nonstationary: both at the largest
 * lateral scale, GPFunctions.cpp:1241-1258; isotropic: kernelRadius = localScale
 * and kernelSpatialScale 1) or the two of the multi-resolution grid around ls(p)
 * with their weights (kernelScaleLevelRatio). */
static int levels3(const om_t *m, const float p[3], lv3_t lv[2], float w[2])
{
    const float mtx = fmaxf(fmaxf(m->l_aniso[0], m->l_aniso[1]), m->l_aniso[2]);
    if (m->multires) {
        float info[4];
        level_ratio(m, p, info);
        for (int j = 0; j < 2; ++j) {
            lv[j].ks = info[j];
            lv[j].seed_add = level_seed(info[j]);
            lv[j].kr = m->iso3d ? m->d.kernel_scale : m->d.kernel_scale * info[j] * mtx;
        }
        w[0] = info[2];
        w[1] = info[3];
        return 2;
    }
    lv[0].kr = m->iso3d ? m->kr_iso : m->kr_world;
    lv[0].ks = m->iso3d ? 1.0f : m->ls_max;
    lv[0].seed_add = level_seed(lv[0].ks);
    w[0] = 1.0f;
    w[1] = 0.0f;
    return 1;
}

/* The isotropic ray-space frame of a direction and a point's coordinates in it
 * (evaluateNoise3DIsotropicRayNormalized, SparseConvolutionNoise.cpp:348-360). */
static void iso_ray_point(const om_t *m, const float p[3], const float dir[3], float ks, frame_t *f, float q[3])
{
    float diso[3], dn[3], piso[3];
    w2l_pos(m, dir, 1.0f, diso);
    normalize3f(diso, dn);
    frame_make(dn, f);
    w2l_pos(m, p, ks, piso);
    frame_to_local(f, piso, q);
}

/* noise3D + cell3D (SparseConvolutionNoise.cpp:419-452) at the point q of the
 * level's space: raw sum and gradient.  dbl: the same impulse set (float inside
 * test), every value in FP64. */
static void lattice3(const om_t *m, const float q[3], float kr, const float M[3], uint32_t seed, int dbl,
                     double out[4])
{
    float pg[3], fr[3];
    int ijk[3];
    for (int i = 0; i < 3; ++i) {
        pg[i] = q[i] / kr;
        float fl = floorf(pg[i]);
        fr[i] = pg[i] - fl;
        ijk[i] = (int)fl;
    }
    float sf[4] = {0, 0, 0, 0};
    double sd[4] = {0, 0, 0, 0};
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                uint32_t cx = (uint32_t)(ijk[0] + dx), cy = (uint32_t)(ijk[1] + dy), cz = (uint32_t)(ijk[2] + dz);
                float tl[3] = {fr[0] - (float)dx, fr[1] - (float)dy, fr[2] - (float)dz};
                pcg_t g;
                pcg_set_state(&g, (uint64_t)(uint32_t)(gor_xxhash32_4(cz, cy, cx, seed) + 1u));
                float cf[4] = {0, 0, 0, 0};
                for (uint32_t k = 0; k < m->n_imp; ++k) {
                    float pi[3];
                    draw3(&g, m->d.impulse_xyz_order, pi);
                    float wi = pcg_1d(&g) < 0.5f ? -1.0f : 1.0f;
                    float tp[3] = {tl[0] - pi[0], tl[1] - pi[1], tl[2] - pi[2]};
                    if (dot3f(tp, tp) < 1.0f) {
                        if (!dbl) {
                            float ab[3];
                            for (int c = 0; c < 3; ++c) ab[c] = kr * tl[c] - kr * pi[c];
                            float absq = ab[0] * M[0] * ab[0];
                            absq += ab[1] * M[1] * ab[1];
                            absq += ab[2] * M[2] * ab[2];
                            float f = rexpf(-absq);
                            cf[0] += wi * f;
                            for (int c = 0; c < 3; ++c) cf[1 + c] += wi * (-2.f * (ab[c] * M[c]) * f);
                        } else {
                            double ab[3], absq = 0.0;
                            for (int c = 0; c < 3; ++c) {
                                ab[c] = (double)kr * ((double)q[c] / (double)kr - (double)(ijk[c] + (c == 0 ? dx : c == 1 ? dy : dz)) - (double)pi[c]);
                                absq += ab[c] * (double)M[c] * ab[c];
                            }
                            double f = exp(-absq);
                            sd[0] += wi * f;
                            for (int c = 0; c < 3; ++c) sd[1 + c] += wi * (-2.0 * ab[c] * (double)M[c] * f);
                        }
                    }
                }
                for (int c = 0; c < 4; ++c) sf[c] += cf[c];
            }
    for (int c = 0; c < 4; ++c) out[c] = dbl ? sd[c] : (double)sf[c];
}

/* sqrt(sparseConvNoiseVariance3D) (GPFunctions.cpp:751-764; nonstationary
 * 1260-1263): float as the reference rounds it, and FP64. */
static void norm3(const om_t *m, int iso, float kr, float gs, float a, float *nf, double *nd)
{
    float ud = m->d.impulse_density / (kr * kr * kr);
    double det = 1.0, detd = 1.0;
    if (!iso) {
        float detf = m->l_aniso[0] * m->l_aniso[1] * m->l_aniso[2];
        det = (double)detf * pow((double)gs, 3);
        detd = (double)m->l_aniso[0] * m->l_aniso[1] * m->l_aniso[2] * pow((double)gs, 3);
    }
    det *= pow((double)a, 3);
    detd *= pow((double)a, 3);
    float var = (float)((double)ud * (pow(M_PI, 1.5) * det));
    *nf = sqrtf(var);
    *nd = sqrt((double)m->d.impulse_density / ((double)kr * kr * kr) * pow(M_PI, 1.5) * detd);
}

/* One level: evaluateNoise3DNormalized (world, :308-317) or
 * evaluateNoise3DIsotropicRayNormalized (:348-377) with its conditioning splats
 * (splattingKernel3D / 3DGrad, GPFunctions.cpp:555-580, 814-843).  out = (value,
 * world gradient) of the normalized noise. */
static void noise3d_level(const real_t *r, const float p[3], const float dir[3], int cond, int dbl,
                          const lv3_t *L, double out[4])
{
    const om_t *m = r->m;
    const int iso = m->iso3d;
    const float a = ns_scale(m, p);
    const uint32_t seed = r->noise_seed + oct_seed(m, r->octave) + L->seed_add;
    const float gs = iso ? 1.0f : L->ks;
    float q[3];
    frame_t f;
    if (iso) iso_ray_point(m, p, dir, L->ks, &f, q);
    else { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
    float M[3];
    inv_cov3(m, iso, 0, a, gs, M);
    double s4[4];
    lattice3(m, q, L->kr, M, seed, dbl, s4);
    float nf;
    double nd;
    norm3(m, iso, L->kr, gs, a, &nf, &nd);
    if (!dbl) {
        float g[3] = {(float)s4[1], (float)s4[2], (float)s4[3]};
        if (iso) {
            float gi[3];
            frame_to_global(&f, g, gi);
            l2w_grad(m, gi, L->ks, g);
        }
        out[0] = (float)s4[0] / nf;
        for (int c = 0; c < 3; ++c) out[1 + c] = g[c] / nf;
    } else {
        double g[3] = {s4[1], s4[2], s4[3]};
        if (iso) {
            double gi[3];
            for (int i = 0; i < 3; ++i) gi[i] = (double)f.t[i] * g[0] + (double)f.b[i] * g[1] + (double)f.n[i] * g[2];
            const double sdiv = (double)ns_transform_scale(m, L->ks);
            for (int i = 0; i < 3; ++i) g[i] = (double)m->l_inv[i] * gi[i] / sdiv;
        }
        out[0] = s4[0] / nd;
        for (int c = 0; c < 3; ++c) out[1 + c] = g[c] / nd;
    }
    if (!(m->activate_cond && cond)) return;
    const coef_t *c = &r->c3;
    float Mc[3];
    inv_cov3(m, iso, 1, a, gs, Mc);
    float ab[3];
    if (iso) {
        float oiso[3], oq[3];
        w2l_pos(m, c->origin, L->ks, oiso);
        frame_to_local(&f, oiso, oq);
        for (int i = 0; i < 3; ++i) ab[i] = q[i] - oq[i];
    } else {
        for (int i = 0; i < 3; ++i) ab[i] = p[i] - c->origin[i];
    }
    if (!dbl) {
        float absq = ab[0] * Mc[0] * ab[0];
        absq += ab[1] * Mc[1] * ab[1];
        absq += ab[2] * Mc[2] * ab[2];
        float fk = rexpf(-absq);
        float dp[3], g1[3];
        for (int i = 0; i < 3; ++i) {
            dp[i] = -2.f * (ab[i] * Mc[i]);
            g1[i] = dp[i] * fk;
        }
        float add[4];
        add[0] = fk * c->value_scale;
        for (int i = 0; i < 3; ++i) add[1 + i] = g1[i] * c->value_scale;
        /* sum_c gs_c * (grad1st_c, grad2nd(c, .)) */
        float gv = 0.0f, gg[3] = {0, 0, 0};
        for (int cc = 0; cc < 3; ++cc) {
            gv += g1[cc] * c->gs[cc];
            for (int j = 0; j < 3; ++j) {
                float h = dp[cc] * dp[j] - (cc == j ? 2.f * Mc[cc] : 0.0f);
                gg[j] += (h * fk) * c->gs[cc];
            }
        }
        float dg[3] = {add[1] + gg[0], add[2] + gg[1], add[3] + gg[2]};
        if (iso) {
            float gi[3];
            frame_to_global(&f, dg, gi);
            l2w_grad(m, gi, L->ks, dg);
        }
        out[0] = (float)out[0] + (add[0] + gv);
        for (int j = 0; j < 3; ++j) out[1 + j] = (float)out[1 + j] + dg[j];
    } else {
        double absq = 0.0;
        for (int i = 0; i < 3; ++i) absq += (double)ab[i] * ab[i] * Mc[i];
        double fk = exp(-absq), dp[3], dg[3] = {0, 0, 0};
        for (int i = 0; i < 3; ++i) dp[i] = -2.0 * ab[i] * Mc[i];
        out[0] += fk * c->value_scale;
        for (int j = 0; j < 3; ++j) dg[j] += dp[j] * fk * c->value_scale;
        for (int cc = 0; cc < 3; ++cc) {
            out[0] += dp[cc] * fk * c->gs[cc];
            for (int j = 0; j < 3; ++j)
                dg[j] += (dp[cc] * dp[j] - (cc == j ? 2.0 * Mc[cc] : 0.0)) * fk * c->gs[cc];
        }
        if (iso) {
            double gi[3];
            for (int i = 0; i < 3; ++i) gi[i] = (double)f.t[i] * dg[0] + (double)f.b[i] * dg[1] + (double)f.n[i] * dg[2];
            const double sdiv = (double)ns_transform_scale(m, L->ks);
            for (int i = 0; i < 3; ++i) dg[i] = (double)m->l_inv[i] * gi[i] / sdiv;
        }
        for (int j = 0; j < 3; ++j) out[1 + j] += dg[j];
    }
}

/* evaluateNoise3D (SparseConvolutionNoise.cpp:142-165): one level, or the blend
 * w_low * noise_low + w_high * noise_high of the multi-resolution grid. */
static void noise3d_norm(const real_t *r, const float p[3], const float dir[3], int cond, int dbl, double out[4])
{
    lv3_t lv[2];
    float w[2];
    const int n = levels3(r->m, p, lv, w);
    if (n == 1) {
        noise3d_level(r, p, dir, cond, dbl, &lv[0], out);
        return;
    }
    double lo[4], hi[4];
    noise3d_level(r, p, dir, cond, dbl, &lv[0], lo);
    noise3d_level(r, p, dir, cond, dbl, &lv[1], hi);
    for (int k = 0; k < 4; ++k)
        out[k] = dbl ? (double)w[0] * lo[k] + (double)w[1] * hi[k]
                     : (double)(w[0] * (float)lo[k] + w[1] * (float)hi[k]);
}

/* --- gradient sampling, conditioning ------------------------------------ */

/* correlatedGradientMoments (SparseConvolutionNoise.cpp:13-22) */
static void corr_moments(float distance, double *factor, double *variance)
{
    const double x = 0.5 * (double)distance * (double)distance;
    *factor = 0.5 * exp(-0.5 * x) * (1.0 - x);
    *variance = x < 1.0 ? 0.5 * (-expm1(-x) + exp(-x) * x * (2.0 - x))
                        : 0.5 - 2.0 * (*factor) * (*factor);
}

static inline int transverse_law(const om_t *m)
{
    /* seTransverseGradientMoments needs a SquaredExponentialCovariance (a
       nonstationary wrapper fails the dynamic_cast) and one realization */
    return m->d.one_d_sampling && m->d.correlation_xy &&
           m->d.correlation_context == GPIS_CTX_RENEWAL_PLUS && !m->multires &&
           !m->nonstationary && m->d.n_octaves == 1;
}

/* seTransverseGradientMoments (SparseConvolutionNoise.cpp:78-99) */
static int transverse_moments(const real_t *r, const float p[3], const float dir[3], int cond,
                              double mean[2], double *var)
{
    const om_t *m = r->m;
    if (!transverse_law(m)) return 0;
    mean[0] = mean[1] = 0.0;
    *var = 0.5;
    if (cond && r->c1.has_grad_obs) {
        float dl[3], delta[3];
        for (int i = 0; i < 3; ++i) dl[i] = p[i] - r->c1.origin[i];
        w2l_pos(m, dl, 1.f, delta);
        double dd[3] = {delta[0], delta[1], delta[2]};
        const double q2 = 0.5 * dot3d(dd, dd);
        const double rho = exp(-0.5 * q2);
        *var = -0.5 * expm1(-q2);
        float diso[3], dn[3], og[3], obs[3];
        w2l_pos(m, dir, 1.f, diso);
        normalize3f(diso, dn);
        frame_t f;
        frame_make(dn, &f);
        w2l_grad(m, r->c1.tgn, 1.f, og);
        frame_to_local(&f, og, obs);
        mean[0] = rho * obs[0];
        mean[1] = rho * obs[1];
    }
    return 1;
}

/* evaluateGradientNoise1D on the multi-resolution grid (SparseConvolutionNoise.cpp:
 * 244-295): the two levels' base gradients, two normal pairs (low, high) at the
 * start of the ray and two more at its end, each level's gradient taken to world
 * space through its own frame and scale, blended by the level weights. */
static void grad_noise_1d_levels(const real_t *r, const float p[3], float t_segment, const float dir[3],
                                 int cond, double xs0, double xs1, float out[3])
{
    const om_t *m = r->m;
    float info[4];
    level_ratio(m, p, info);
    double lo4[4], hi4[4];
    noise1d_level(r, p, dir, cond, 0, info[0], 1, lo4);
    noise1d_level(r, p, dir, cond, 0, info[1], 0, hi4);
    const float blo[3] = {(float)lo4[1], (float)lo4[2], (float)lo4[3]};
    const float bhi[3] = {(float)hi4[1], (float)hi4[2], (float)hi4[3]};
    pcg_t g;
    pcg_set_state(&g, (uint64_t)r->normal_seed);
    double x1l[2], x1h[2];
    rand_normal_2(&g, x1l);
    rand_normal_2(&g, x1h);
    const double s2 = (double)sqrtf(2.f);
    for (int i = 0; i < 2; ++i) {
        x1l[i] /= s2;
        x1h[i] /= s2;
    }
    float gl[3], gh[3];
    if (t_segment == 0) {
        x1l[0] *= xs0; x1l[1] *= xs1;
        x1h[0] *= xs0; x1h[1] *= xs1;
        gl[0] = (float)x1l[0] + blo[0]; gl[1] = (float)x1l[1] + blo[1];
        gh[0] = (float)x1h[0] + bhi[0]; gh[1] = (float)x1h[1] + bhi[1];
    } else if (!(m->d.correlation_context == GPIS_CTX_RENEWAL_PLUS && m->d.correlation_xy)) {
        double x2l[2], x2h[2];
        rand_normal_2(&g, x2l);
        rand_normal_2(&g, x2h);
        x2l[0] = x2l[0] / s2 * xs0; x2l[1] = x2l[1] / s2 * xs1;
        x2h[0] = x2h[0] / s2 * xs0; x2h[1] = x2h[1] / s2 * xs1;
        gl[0] = (float)x2l[0] + blo[0]; gl[1] = (float)x2l[1] + blo[1];
        gh[0] = (float)x2h[0] + bhi[0]; gh[1] = (float)x2h[1] + bhi[1];
    } else {
        double fac, cov;
        corr_moments(t_segment, &fac, &cov);
        double x2l[2], x2h[2];
        rand_normal_2(&g, x2l);
        rand_normal_2(&g, x2h);
        const double sc = sqrt(cov);
        gl[0] = (float)(x2l[0] * sc + fac * 2.0 * x1l[0]) + blo[0];
        gl[1] = (float)(x2l[1] * sc + fac * 2.0 * x1l[1]) + blo[1];
        gh[0] = (float)(x2h[0] * sc + fac * 2.0 * x1h[0]) + bhi[0];
        gh[1] = (float)(x2h[1] * sc + fac * 2.0 * x1h[1]) + bhi[1];
    }
    gl[2] = 0.f + blo[2];
    gh[2] = 0.f + bhi[2];
    float dl[3], dh[3], dln[3], dhn[3], gil[3], gih[3], gwl[3], gwh[3];
    frame_t fl, fh;
    w2l_pos(m, dir, info[0], dl);
    normalize3f(dl, dln);
    frame_make(dln, &fl);
    w2l_pos(m, dir, info[1], dh);
    normalize3f(dh, dhn);
    frame_make(dhn, &fh);
    frame_to_global(&fl, gl, gil);
    frame_to_global(&fh, gh, gih);
    l2w_grad(m, gil, info[0], gwl);
    l2w_grad(m, gih, info[1], gwh);
    for (int i = 0; i < 3; ++i) out[i] = info[2] * gwl[i] + info[3] * gwh[i];
}

/* evaluateGradientNoise1D (SparseConvolutionNoise.cpp:178-243), stationary branch. */
static void grad_noise_1d(const real_t *r, const float p[3], float t_segment, const float dir[3],
                          int cond, float out[3])
{
    const om_t *m = r->m;
    float diso[3], dn[3];
    w2l_pos(m, dir, 1.0f, diso);
    normalize3f(diso, dn);
    frame_t f;
    frame_make(dn, &f);
    double tm[2], tv;
    pcg_t g;
    if (transverse_moments(r, p, dir, cond, tm, &tv)) {
        double base[4];
        noise1d_norm(r, p, dir, cond, 0, base);
        pcg_set_state(&g, (uint64_t)r->normal_seed);
        double z[2];
        rand_normal_2(&g, z);
        const double s = sqrt(tv);
        float gl[3] = {(float)(tm[0] + s * z[0]), (float)(tm[1] + s * z[1]), (float)base[3]};
        float gi[3];
        frame_to_global(&f, gl, gi);
        l2w_grad(m, gi, 1.f, out);
        return;
    }
    float scx = splat_cov_1d(m, p, p), scy = scx;
    double xs0 = 1.0 / scx, xs1 = 1.0 / scy;
    if (m->multires) {
        grad_noise_1d_levels(r, p, t_segment, dir, cond, xs0, xs1, out);
        return;
    }
    double b4[4];
    noise1d_norm(r, p, dir, cond, 0, b4);
    float base[3] = {(float)b4[1], (float)b4[2], (float)b4[3]};
    pcg_set_state(&g, (uint64_t)r->normal_seed);
    double xy1[2];
    rand_normal_2(&g, xy1);
    const double s2 = (double)sqrtf(2.f);
    xy1[0] /= s2;
    xy1[1] /= s2;
    float gr[3];
    if (t_segment == 0) {
        xy1[0] *= xs0;
        xy1[1] *= xs1;
        gr[0] = (float)xy1[0] + base[0];
        gr[1] = (float)xy1[1] + base[1];
        gr[2] = 0.f + base[2];
    } else if (!(m->d.correlation_context == GPIS_CTX_RENEWAL_PLUS && m->d.correlation_xy)) {
        double xy2[2];
        rand_normal_2(&g, xy2);
        xy2[0] = xy2[0] / s2 * xs0;
        xy2[1] = xy2[1] / s2 * xs1;
        gr[0] = (float)xy2[0] + base[0];
        gr[1] = (float)xy2[1] + base[1];
        gr[2] = 0.f + base[2];
    } else {
        double fac, cov;
        corr_moments(t_segment, &fac, &cov);
        double mu0 = fac * 2.0 * xy1[0], mu1 = fac * 2.0 * xy1[1];
        double xy2[2];
        rand_normal_2(&g, xy2);
        double sc = sqrt(cov);
        gr[0] = (float)(xy2[0] * sc + mu0) + base[0];
        gr[1] = (float)(xy2[1] * sc + mu1) + base[1];
        gr[2] = 0.f + base[2];
    }
    float gi[3];
    frame_to_global(&f, gr, gi);
    l2w_grad(m, gi, 1.0f, out);
    const float sc = oct_scale(m, r->octave);
    if (sc != 1.0f)
        for (int i = 0; i < 3; ++i) out[i] = out[i] / sc;
}

static void mean_grad_f(const om_t *m, const float p[3], float g[3])
{
    double a[3] = {p[0], p[1], p[2]}, gd[3];
    mean_grad(m, a, gd);
    g[0] = (float)gd[0]; g[1] = (float)gd[1]; g[2] = (float)gd[2];
}

static float mean_f(const om_t *m, const float p[3], int *id)
{
    double a[3] = {p[0], p[1], p[2]};
    return (float)mean_value(m, a, id);
}

/* One octave's conditioning (conditioning1D / conditioning3D,
 * SparseConvolutionNoise.cpp:498-656).  target_* are the octave's share. */
static void conditioning_1d(real_t *r, const float p[3], const float dir[3], float target_val,
                            const float target_grad[3], float mean, const float mgrad[3])
{
    const om_t *m = r->m;
    coef_t *c = &r->c1;
    memset(c, 0, sizeof(*c));
    memcpy(c->origin, p, sizeof(float) * 3);
    float amp = amplitude(r);
    if (amp == 0) return;
    double v4[4];
    noise1d_norm(r, p, dir, 0, 0, v4);
    float cur = (float)v4[0];
    c->value_scale = (target_val - mean) / amp - cur;
    /* the multi-resolution splats carry both levels' weights (conditioning1D,
       SparseConvolutionNoise.cpp:602-604, 631-633) */
    float mr_norm = 1.0f;
    if (m->multires) {
        float info[4];
        level_ratio(m, p, info);
        mr_norm = info[2] * info[2] + info[3] * info[3];
        c->value_scale /= mr_norm;
    }
    if (m->d.correlation_context == GPIS_CTX_RENEWAL_PLUS) {
        float cg[3];
        grad_noise_1d(r, p, 0.0f, dir, 0, cg);
        float delta[3];
        for (int i = 0; i < 3; ++i) delta[i] = (target_grad[i] - mgrad[i]) / amp - cg[i];
        float diso[3], dn[3];
        w2l_pos(m, dir, 1.0f, diso);
        normalize3f(diso, dn);
        frame_t f;
        frame_make(dn, &f);
        float gi[3], gl[3];
        /* the octave's length multiplier enters once, where the splats are
           evaluated (noise1d_norm scales gs by it) */
        w2l_grad(m, delta, 1.0f, gi);
        frame_to_local(&f, gi, gl);
        float s = splat_cov_1d(m, p, p);
        float s2 = s * s;
        for (int i = 0; i < 3; ++i) c->gs[i] = -2.f * gl[i] * s2;
        if (m->multires)
            for (int i = 0; i < 3; ++i) c->gs[i] /= mr_norm;
        if (!m->d.correlation_xy) c->gs[0] = c->gs[1] = 0;
        for (int i = 0; i < 3; ++i) c->tgn[i] = (target_grad[i] - mgrad[i]) / amp;
        c->has_grad_obs = 1;
    }
}

static void conditioning_3d(real_t *r, const float p[3], const float dir[3], float target_val,
                            const float target_grad[3], float mean, const float mgrad[3])
{
    const om_t *m = r->m;
    coef_t *c = &r->c3;
    memset(c, 0, sizeof(*c));
    memcpy(c->origin, p, sizeof(float) * 3);
    float amp = amplitude(r);
    if (amp == 0) return;
    float info[4] = {1.0f, 1.0f, 1.0f, 0.0f};
    if (m->multires) level_ratio(m, p, info);
    double n4[4];
    noise3d_norm(r, p, dir, 0, 0, n4);
    c->value_scale = (target_val - mean) / amp - (float)n4[0];
    if (m->multires) c->value_scale /= info[2] + info[3];
    if (m->d.correlation_context != GPIS_CTX_RENEWAL_PLUS) return;
    float delta[3];
    for (int i = 0; i < 3; ++i) delta[i] = (target_grad[i] - mgrad[i]) / amp - (float)n4[1 + i];
    if (m->iso3d) {
        /* the world residual to isotropic (ray) space, times the inverse of the
           isotropic second derivative -2 * 0.25 I, which is -2 I exactly */
        float gi[3], diso[3], dn[3], gl[3];
        w2l_grad(m, delta, 1.0f, gi);
        w2l_pos(m, dir, 1.0f, diso);
        normalize3f(diso, dn);
        frame_t f;
        frame_make(dn, &f);
        frame_to_local(&f, gi, gl);
        for (int i = 0; i < 3; ++i) c->gs[i] = -2.f * gl[i];
        if (m->multires) {
            const float dv = info[2] / info[0] + info[3] / info[1];
            for (int i = 0; i < 3; ++i) c->gs[i] /= dv;
        } else {
            const float a = ns_scale(m, p);
            for (int i = 0; i < 3; ++i) c->gs[i] *= a * a;
        }
        return;
    }
    for (int i = 0; i < 3; ++i) {
        /* sparseConvNoiseOneOverSecondDerivative (GPFunctions.cpp:723-749): the inverse
           of -2*(0.25*l_inv^2) for a diagonal covariance, restated as the division */
        float inv2 = m->l_inv[i] * m->l_inv[i];
        float d2 = -2.f * (inv2 * 0.25f);
        c->gs[i] = delta[i] / d2;
    }
    if (m->multires) {
        const float dv = info[2] / (info[0] * info[0]) + info[3] / (info[1] * info[1]);
        for (int i = 0; i < 3; ++i) c->gs[i] /= dv;
    } else {
        /* sqr(sparseConvNoiseLateralScale(p)): ls(p) itself by brute force, 1 stationary */
        const float ls = ls_field(m, p);
        for (int i = 0; i < 3; ++i) c->gs[i] *= ls * ls;
    }
}

/* ------------------------------------------------------------------------ */
/* Field (all octaves) and flights                                          */
/* ------------------------------------------------------------------------ */
typedef struct {
    const om_t *m;
    int n;                       /* octaves */
    real_t oct[4];
    float dir[3];
} field_t;

static void field_init(field_t *F, const om_t *m, uint32_t noise_seed, uint32_t normal_seed,
                       const float dir[3])
{
    memset(F, 0, sizeof(*F));
    F->m = m;
    F->n = (int)m->d.n_octaves;
    for (int k = 0; k < F->n; ++k) {
        F->oct[k].m = m;
        F->oct[k].octave = k;
        F->oct[k].noise_seed = noise_seed;
        F->oct[k].normal_seed = normal_seed + (uint32_t)k * 0x9E3779B9u * (F->n > 1);
    }
    memcpy(F->dir, dir, sizeof(float) * 3);
}

/* Noise of octave k at p (value, gradient or 1D parts). */
static void oct_noise(const field_t *F, int k, const float p[3], int cond, int dbl, double out[4])
{
    if (F->m->d.one_d_sampling)
        noise1d_norm(&F->oct[k], p, F->dir, cond, dbl, out);
    else
        noise3d_norm(&F->oct[k], p, F->dir, cond, dbl, out);
}

/* evaluateValue (SparseConvolutionNoise.cpp:114-130): amplitude*noise + mean. */
static float field_value(const field_t *F, const float p[3], int *id, double *mean_out)
{
    double a[3] = {p[0], p[1], p[2]};
    double mean = mean_value(F->m, a, id);
    if (mean_out) *mean_out = mean;
    if (F->n == 1) {
        double n4[4];
        oct_noise(F, 0, p, 1, 0, n4);
        float amp = amplitude(&F->oct[0]);
        return (float)((double)(amp * (float)n4[0]) + mean);
    }
    float s = 0.0f;
    for (int k = 0; k < F->n; ++k) {
        double n4[4];
        oct_noise(F, k, p, 1, 0, n4);
        s += amplitude(&F->oct[k]) * (float)n4[0];
    }
    return (float)((double)s + mean);
}

/* evaluateGradient (SparseConvolutionNoise.cpp:133-140) */
static void field_grad(const field_t *F, const float p[3], float t_segment, float out[3])
{
    float mg[3];
    mean_grad_f(F->m, p, mg);
    float g[3] = {0, 0, 0};
    for (int k = 0; k < F->n; ++k) {
        float ng[3];
        if (F->m->d.one_d_sampling) {
            grad_noise_1d(&F->oct[k], p, t_segment, F->dir, 1, ng);
        } else {
            double n4[4];
            noise3d_norm(&F->oct[k], p, F->dir, 1, 0, n4);
            ng[0] = (float)n4[1]; ng[1] = (float)n4[2]; ng[2] = (float)n4[3];
        }
        float amp = amplitude(&F->oct[k]);
        for (int i = 0; i < 3; ++i) g[i] += amp * ng[i];
    }
    for (int i = 0; i < 3; ++i) out[i] = g[i] + mg[i];
}

/* conditioning (SparseConvolutionNoise.cpp:488-496).  With several octaves the
 * residual of the value (and gradient) is shared in proportion to each
 * octave's variance sigma_k^2. */
static void field_condition(field_t *F, const float p[3], float target_val, const float target_grad[3])
{
    const om_t *m = F->m;
    if (!m->activate_cond) return;
    int id;
    float mean = mean_f(m, p, &id);
    float mg[3];
    if (m->d.correlation_context == GPIS_CTX_RENEWAL_PLUS) mean_grad_f(m, p, mg);
    else mg[0] = mg[1] = mg[2] = 0.0f;
    if (F->n == 1) {
        if (m->d.one_d_sampling) conditioning_1d(&F->oct[0], p, F->dir, target_val, target_grad, mean, mg);
        else conditioning_3d(&F->oct[0], p, F->dir, target_val, target_grad, mean, mg);
        return;
    }
    /* Octaves (1D): the residual of the value, and of the gradient under
       Renewal+, is shared between the octaves in proportion to their variance
       sigma_k^2, so that the summed field meets the birth value and gradient. */
    float total = 0.0f;
    for (int k = 0; k < F->n; ++k) total += oct_sigma(m, k) * oct_sigma(m, k);
    double cur[4][4];
    float curg[4][3];
    for (int k = 0; k < F->n; ++k) {
        oct_noise(F, k, p, 0, 0, cur[k]);
        grad_noise_1d(&F->oct[k], p, 0.0f, F->dir, 0, curg[k]);
    }
    float sum_v = 0.0f, sum_g[3] = {0.0f, 0.0f, 0.0f};
    for (int k = 0; k < F->n; ++k) {
        sum_v += oct_sigma(m, k) * (float)cur[k][0];
        for (int i = 0; i < 3; ++i) sum_g[i] += oct_sigma(m, k) * curg[k][i];
    }
    const float resid = (target_val - mean) - sum_v;
    float resid_g[3];
    for (int i = 0; i < 3; ++i) resid_g[i] = (target_grad[i] - mg[i]) - sum_g[i];
    for (int k = 0; k < F->n; ++k) {
        const float sk = oct_sigma(m, k);
        const float share = sk * sk / total;
        const float tv = mean + sk * (float)cur[k][0] + share * resid;
        float tg[3];
        for (int i = 0; i < 3; ++i) tg[i] = mg[i] + sk * curg[k][i] + share * resid_g[i];
        conditioning_1d(&F->oct[k], p, F->dir, tv, tg, mean, mg);
    }
}

void gor_flight_seeds(const gpis_medium_desc *desc, const uint32_t pss[4], uint32_t scene_seed,
                      uint32_t *noise_seed, uint32_t *normal_seed)
{
    uint32_t w = desc->correlation_context == GPIS_CTX_GLOBAL ? 0u : pss[3];
    uint32_t seed = desc->seed;
    if (!desc->single_realization)
        seed += gor_xxhash32_4(pss[0], pss[1], pss[2], w) + gor_xxhash32_1(scene_seed);
    *noise_seed = seed;
    *normal_seed = gor_xxhash32_4(pss[0], pss[1], pss[2], pss[3]) + gor_xxhash32_1(scene_seed) + 1u;
}

typedef struct {
    float o[3], d[3], near_t, far_t, jitter, prev_v, prev_g[3];
    uint32_t noise_seed, normal_seed, flags;
} fin_t;

static inline void point_at(const fin_t *in, double t, float p[3])
{
    for (int i = 0; i < 3; ++i) p[i] = (float)((double)in->o[i] + t * (double)in->d[i]);
}

static inline void point_at_unit(const fin_t *in, double t, float p[3])
{
    double d[3] = {in->d[0], in->d[1], in->d[2]};
    double inv = 1.0 / sqrt(dot3d(d, d));
    for (int i = 0; i < 3; ++i) p[i] = (float)((double)in->o[i] + d[i] * inv * t);
}

static int flight_valid(const fin_t *in)
{
    int first = (in->flags & GPIS_FLAG_FIRST_SCATTER) != 0;
    if (!isfinite(in->near_t) || !isfinite(in->far_t) || in->far_t <= in->near_t) return 0;
    if (!isfinite(in->jitter) || in->jitter < 0.0f || in->jitter >= 1.0f) return 0;
    for (int i = 0; i < 3; ++i)
        if (!isfinite(in->o[i]) || !isfinite(in->d[i])) return 0;
    if (!first && (!isfinite(in->prev_v) || !isfinite(in->prev_g[0]) || !isfinite(in->prev_g[1]) ||
                   !isfinite(in->prev_g[2])))
        return 0;
    if (fabsf(dot3f(in->d, in->d) - 1.0f) > 0.001f) return 0;
    return 1;
}

/* One flight: prepareGpisSegment (SparseConvolutionNoiseMedium.cpp:199-263),
 * finishGpisSegment (:265-347) and the gradient sample of resumeDistance /
 * resumeTransmittance (GaussianProcessMedium.cpp:305-316, 353, 400-409). */
static void oracle_flight(const om_t *m, const fin_t *in, float rec[8])
{
    uint32_t *ru = (uint32_t *)rec;
    memset(rec, 0, sizeof(float) * 8);
    rec[5] = 1.0f;
    if (!flight_valid(in)) {
        ru[7] = GPIS_FLIGHT_INVALID_INPUT;
        return;
    }
    int first = (in->flags & GPIS_FLAG_FIRST_SCATTER) != 0;
    int shadow = (in->flags & GPIS_FLAG_SHADOW) != 0;
    field_t F;
    field_init(&F, m, in->noise_seed, in->normal_seed, in->d);
    if (!first) field_condition(&F, in->o, in->prev_v, in->prev_g);

    uint32_t max_steps = m->d.max_steps ? m->d.max_steps : 16384u;
    float step = (in->far_t - in->near_t) / (float)m->d.min_step;
    if (m->d.step_size < step) step = m->d.step_size;
    int id = 0;
    float p[3];
    double t = in->near_t;
    point_at(in, t, p);
    double f0 = field_value(&F, p, &id, NULL);
    int sign0 = f0 < 0 ? -1 : 1;
    double pf = f0;
    t = (double)(float)(in->near_t + step * in->jitter);
    uint32_t steps = 0;
    while (t < (double)in->far_t) {
        if (steps >= max_steps) {
            rec[0] = in->far_t;
            ru[6] = steps;
            ru[7] = GPIS_FLIGHT_STEP_LIMIT;
            rec[2] = in->prev_g[0]; rec[3] = in->prev_g[1]; rec[4] = in->prev_g[2];
            return;
        }
        steps++;
        point_at(in, t, p);
        double fc = field_value(&F, p, &id, NULL);
        int signc = fc < 0 ? -1 : 1;
        if (!first && steps == 1) {
            sign0 = signc;
        } else if (signc != sign0) {
            double factor = pf / (pf - fc);
            double a = t - step, b = t;
            double t_test, t_prev = a * (1.0 - factor) + b * factor;
            for (;;) {
                t_test = a * (1.0 - factor) + b * factor;
                point_at(in, t_test, p);
                double ft = field_value(&F, p, &id, NULL);
                int st = ft < 0 ? -1 : 1;
                if (st == sign0) break;
                factor *= 0.9;
                if (factor <= 0.01) {
                    t_prev = t_test = 0;
                    break;
                }
                t_prev = t_test;
            }
            t = t_prev;
            float ph[3], g[3];
            point_at_unit(in, t, ph);
            field_grad(&F, ph, (float)t, g);
            rec[0] = (float)t;
            rec[1] = 0.0f;
            rec[2] = g[0]; rec[3] = g[1]; rec[4] = g[2];
            rec[5] = 0.0f;
            ru[6] = steps;
            ru[7] = GPIS_FLIGHT_OK | ((uint32_t)id << 8);
            return;
        }
        pf = fc;
        t += step;
    }
    t = in->far_t;
    point_at(in, t, p);
    rec[0] = in->far_t;
    rec[1] = field_value(&F, p, &id, NULL);
    if (!shadow) {
        float ph[3], g[3];
        point_at_unit(in, t, ph);
        field_grad(&F, ph, (float)t, g);
        rec[2] = g[0]; rec[3] = g[1]; rec[4] = g[2];
    } else {
        rec[2] = in->prev_g[0]; rec[3] = in->prev_g[1]; rec[4] = in->prev_g[2];
    }
    rec[5] = 1.0f;
    ru[6] = steps;
    ru[7] = GPIS_FLIGHT_OK | ((uint32_t)id << 8);
}

static void load_flight(const gpis_flight_soa *in, uint32_t i, fin_t *f)
{
    const float *on = in->origin_near + 4 * (size_t)i;
    const float *df = in->dir_far + 4 * (size_t)i;
    const uint32_t *sd = in->seeds + 4 * (size_t)i;
    f->o[0] = on[0]; f->o[1] = on[1]; f->o[2] = on[2]; f->near_t = on[3];
    f->d[0] = df[0]; f->d[1] = df[1]; f->d[2] = df[2]; f->far_t = df[3];
    f->noise_seed = sd[0]; f->normal_seed = sd[1]; f->flags = sd[2];
    memcpy(&f->jitter, &sd[3], sizeof(float));
    if (in->prev) {
        const float *pv = in->prev + 4 * (size_t)i;
        f->prev_v = pv[0]; f->prev_g[0] = pv[1]; f->prev_g[1] = pv[2]; f->prev_g[2] = pv[3];
    } else {
        f->prev_v = 0; f->prev_g[0] = f->prev_g[1] = f->prev_g[2] = 0;
    }
}

typedef struct {
    const om_t *media;
    int n_media;
    const gpis_flight_soa *in;
    const gpis_result_soa *out;
    uint32_t n;
    atomic_uint next;
} job_t;

static void *worker(void *arg)
{
    job_t *J = (job_t *)arg;
    const uint32_t chunk = 64;
    for (;;) {
        uint32_t b = atomic_fetch_add(&J->next, chunk);
        if (b >= J->n) break;
        uint32_t e = b + chunk < J->n ? b + chunk : J->n;
        for (uint32_t i = b; i < e; ++i) {
            fin_t f;
            load_flight(J->in, i, &f);
            uint32_t mi = J->in->medium ? J->in->medium[i] : 0u;
            float *rec = J->out->rec + 8 * (size_t)i;
            if ((int)mi >= J->n_media) {
                memset(rec, 0, 32);
                ((uint32_t *)rec)[7] = GPIS_FLIGHT_INVALID_INPUT;
                continue;
            }
            oracle_flight(&J->media[mi], &f, rec);
        }
    }
    return NULL;
}

int gor_trace_flights(const gpis_medium_desc *media, int n_media, const gpis_flight_soa *in,
                      const gpis_result_soa *out, uint32_t n, int n_threads)
{
    if (n_media <= 0 || !media || !in || !out) return GPIS_EINVAL;
    om_t *M = (om_t *)calloc((size_t)n_media, sizeof(om_t));
    if (!M) return GPIS_ENOMEM;
    for (int i = 0; i < n_media; ++i) {
        int rc = om_init(&M[i], &media[i]);
        if (rc) { free(M); return rc; }
    }
    if (n_threads <= 0) n_threads = (int)sysconf(_SC_NPROCESSORS_ONLN);
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 256) n_threads = 256;
    job_t J;
    J.media = M; J.n_media = n_media; J.in = in; J.out = out; J.n = n;
    atomic_init(&J.next, 0u);
    if (n_threads == 1) {
        worker(&J);
    } else {
        pthread_t th[256];
        int started = 0;
        for (int i = 0; i < n_threads; ++i)
            if (pthread_create(&th[i], NULL, worker, &J) == 0) started++;
            else break;
        if (started == 0) worker(&J);
        for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
    }
    free(M);
    return GPIS_OK;
}

/* ------------------------------------------------------------------------ */
/* Unit entry points                                                         */
/* ------------------------------------------------------------------------ */
void gor_cell_1d(uint32_t cell, uint32_t seed, uint32_t impulses, float *pos, float *weight)
{
    pcg_t g;
    pcg_set_state(&g, (uint64_t)(uint32_t)(gor_xxhash32_2(cell, seed) + 1u));
    for (uint32_t k = 0; k < impulses; ++k) {
        pos[k] = pcg_1d(&g);
        weight[k] = pcg_1d(&g) < 0.5f ? -1.0f : 1.0f;
    }
}

void gor_cell_3d(int32_t i, int32_t j, int32_t k, uint32_t seed, uint32_t impulses,
                 uint32_t xyz_order, float *pos, float *weight)
{
    pcg_t g;
    pcg_set_state(&g, (uint64_t)(uint32_t)(gor_xxhash32_4((uint32_t)k, (uint32_t)j, (uint32_t)i, seed) + 1u));
    for (uint32_t n = 0; n < impulses; ++n) {
        draw3(&g, xyz_order, pos + 3 * n);
        weight[n] = pcg_1d(&g) < 0.5f ? -1.0f : 1.0f;
    }
}

static int field_setup(const gpis_medium_desc *desc, om_t *m, field_t *F, const float origin[3],
                       const float dir[3], const uint32_t seeds[4], const float prev[4])
{
    int rc = om_init(m, desc);
    if (rc) return rc;
    field_init(F, m, seeds[0], seeds[1], dir);
    if (!(seeds[2] & GPIS_FLAG_FIRST_SCATTER)) {
        float tg[3] = {prev[1], prev[2], prev[3]};
        field_condition(F, origin, prev[0], tg);
    }
    return GPIS_OK;
}

int gor_field(const gpis_medium_desc *desc, const float origin[3], const float dir[3],
              const float p[3], const uint32_t seeds[4], const float prev[4],
              int double_mode, double out[6])
{
    om_t m;
    field_t F;
    int rc = field_setup(desc, &m, &F, origin, dir, seeds, prev);
    if (rc) return rc;
    double n4[4] = {0, 0, 0, 0};
    int id;
    double mean;
    if (F.n == 1) {
        oct_noise(&F, 0, p, 1, double_mode, n4);
    } else {
        for (int k = 0; k < F.n; ++k) {
            double o4[4];
            oct_noise(&F, k, p, 1, double_mode, o4);
            for (int c = 0; c < 4; ++c) n4[c] += (double)oct_sigma(&m, k) * o4[c];
        }
    }
    float fv = field_value(&F, p, &id, &mean);
    for (int c = 0; c < 4; ++c) out[c] = n4[c];
    out[4] = fv;
    out[5] = mean;
    return GPIS_OK;
}

int gor_level_ratio(const gpis_medium_desc *desc, const float p[3], float info[4], uint32_t level_seeds[2])
{
    om_t m;
    int rc = om_init(&m, desc);
    if (rc) return rc;
    if (!m.multires) return GPIS_EINVAL;
    level_ratio(&m, p, info);
    level_seeds[0] = level_seed(info[0]);
    level_seeds[1] = level_seed(info[1]);
    return GPIS_OK;
}

int gor_gradient(const gpis_medium_desc *desc, const float origin[3], const float dir[3],
                 const float p[3], float t_segment, const uint32_t seeds[4],
                 const float prev[4], float out[3])
{
    om_t m;
    field_t F;
    int rc = field_setup(desc, &m, &F, origin, dir, seeds, prev);
    if (rc) return rc;
    field_grad(&F, p, t_segment, out);
    return GPIS_OK;
}

int gor_transverse_moments(const gpis_medium_desc *desc, const float origin[3],
                           const float dir[3], const float p[3], const uint32_t seeds[4],
                           const float prev[4], int conditioning, double mean[2], double *var)
{
    om_t m;
    field_t F;
    int rc = field_setup(desc, &m, &F, origin, dir, seeds, prev);
    if (rc) return rc;
    return transverse_moments(&F.oct[0], p, dir, conditioning, mean, var);
}

int gor_sampling_scheme(const gpis_medium_desc *desc, const float origin[3], const float p[3],
                        const uint32_t seeds[4])
{
    om_t m;
    int rc = om_init(&m, desc);
    if (rc) return -rc;
    (void)seeds;
    float amp = oct_sigma(&m, 0);
    int has_obs = m.activate_cond && m.d.correlation_context == GPIS_CTX_RENEWAL_PLUS &&
                  m.d.one_d_sampling && !(seeds[2] & GPIS_FLAG_FIRST_SCATTER);
    int at_origin = p[0] == origin[0] && p[1] == origin[1] && p[2] == origin[2];
    if (amp < 1e-6f || (m.d.correlation_xy && has_obs && at_origin))
        return GPIS_SCHEME_UNI;
    return m.scheme;
}

/* 3x3 inverse by cofactors (float). */
static void inv3(const float A[9], float R[9])
{
    float c00 = A[4] * A[8] - A[5] * A[7];
    float c01 = A[5] * A[6] - A[3] * A[8];
    float c02 = A[3] * A[7] - A[4] * A[6];
    float det = A[0] * c00 + A[1] * c01 + A[2] * c02;
    float id = 1.0f / det;
    R[0] = c00 * id;
    R[1] = (A[2] * A[7] - A[1] * A[8]) * id;
    R[2] = (A[1] * A[5] - A[2] * A[4]) * id;
    R[3] = c01 * id;
    R[4] = (A[0] * A[8] - A[2] * A[6]) * id;
    R[5] = (A[2] * A[3] - A[0] * A[5]) * id;
    R[6] = c02 * id;
    R[7] = (A[1] * A[6] - A[0] * A[7]) * id;
    R[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

/* neeShared / neeGrad / neePDF (SparseConvolutionNoise.cpp:662-821), single-resolution
 * branch, one octave (stationary or nonstationary length scale). */
/* neeShared / neePDF for a field of several octaves (no reference form: the
 * reference NEE is defined for one realization).  Octave k contributes
 * c_k (x_k, y_k, dv_k) in the common iso-ray frame, c_k = amplitude / length
 * multiplier, with independent transverse draws of the law its gradient sample
 * uses (grad_noise_1d): N(base_k, 1 / (2 scx^2)) per component, or under
 * Renewal+ with correlationXY away from the origin N(base_k + 2 fac x1_k, cov).
 * So the summed transverse gradient (X, Y) is Gaussian with mean sum c_k m_k and
 * variance v sum c_k^2, the along-ray component is Z = sum c_k dv_k, and the
 * gradient plane, its intersection with the normal and the solid-angle Jacobian
 * are those of the one-realization case with the matrix l2w * [t b n]. */
static int nee_octaves(const om_t *m, const field_t *F, const float dir[3], const float p[3],
                       const float normal[3], float t_segment, float *pdf, float grad[3])
{
    float mg[3];
    mean_grad_f(m, p, mg);
    float diso[3], dn[3];
    w2l_pos(m, dir, 1.0f, diso);
    normalize3f(diso, dn);
    frame_t f;
    frame_make(dn, &f);
    double A[9];
    for (int i = 0; i < 3; ++i) {
        const double li = m->nonstationary ? (double)m->l_inv[i] / m->ls_max : (double)m->l_inv[i];
        A[3 * i + 0] = li * f.t[i];
        A[3 * i + 1] = li * f.b[i];
        A[3 * i + 2] = li * f.n[i];
    }
    const int corr = m->d.correlation_context == GPIS_CTX_RENEWAL_PLUS && m->d.correlation_xy && t_segment != 0.0f;
    double fac = 0.0, cov = 0.0;
    if (corr) corr_moments(t_segment, &fac, &cov);
    const double scx = splat_cov_1d(m, p, p);
    const double v1 = corr ? cov : 1.0 / (2.0 * scx * scx);
    double Z = 0.0, MX = 0.0, MY = 0.0, S2 = 0.0;
    for (int k = 0; k < F->n; ++k) {
        const real_t *r = &F->oct[k];
        const double c = (double)amplitude(r) / oct_scale(m, k);
        double o4[4];
        noise1d_norm(r, p, dir, 1, 0, o4);
        Z += c * o4[3];
        double bx = o4[1], by = o4[2];
        if (corr) {
            pcg_t g;
            pcg_set_state(&g, (uint64_t)r->normal_seed);
            double xy1[2];
            rand_normal_2(&g, xy1);
            const double s2 = (double)sqrtf(2.f);
            bx += fac * 2.0 * (xy1[0] / s2);
            by += fac * 2.0 * (xy1[1] / s2);
        }
        MX += c * bx;
        MY += c * by;
        S2 += c * c;
    }
    const double V = v1 * S2;
    /* the gradient plane {A (X, Y, Z) + mg}, its normal and the stretch of its axes */
    double ppt[3], cr[3], ax[3] = {A[0], A[3], A[6]}, ay[3] = {A[1], A[4], A[7]};
    for (int i = 0; i < 3; ++i) ppt[i] = A[3 * i + 2] * Z + mg[i];
    cr[0] = ax[1] * ay[2] - ax[2] * ay[1];
    cr[1] = ax[2] * ay[0] - ax[0] * ay[2];
    cr[2] = ax[0] * ay[1] - ax[1] * ay[0];
    const double jac = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    double pn[3] = {cr[0] / jac, cr[1] / jac, cr[2] / jac};
    const double npn = normal[0] * pn[0] + normal[1] * pn[1] + normal[2] * pn[2];
    const double isect = (ppt[0] * pn[0] + ppt[1] * pn[1] + ppt[2] * pn[2]) / npn;
    for (int i = 0; i < 3; ++i) grad[i] = (float)(isect * normal[i]);
    if (!(isect >= 0.0) || !(V > 0.0)) {
        *pdf = 0.0f;
        return GPIS_OK;
    }
    /* (X, Y) of the gradient isect * normal: solve A (X, Y, Z') = g - mg */
    double Af[9], Ai[9];
    for (int i = 0; i < 9; ++i) Af[i] = A[i];
    const double c00 = Af[4] * Af[8] - Af[5] * Af[7], c01 = Af[5] * Af[6] - Af[3] * Af[8], c02 = Af[3] * Af[7] - Af[4] * Af[6];
    const double id = 1.0 / (Af[0] * c00 + Af[1] * c01 + Af[2] * c02);
    Ai[0] = c00 * id; Ai[1] = (Af[2] * Af[7] - Af[1] * Af[8]) * id; Ai[2] = (Af[1] * Af[5] - Af[2] * Af[4]) * id;
    Ai[3] = c01 * id; Ai[4] = (Af[0] * Af[8] - Af[2] * Af[6]) * id; Ai[5] = (Af[2] * Af[3] - Af[0] * Af[5]) * id;
    double gw[3];
    for (int i = 0; i < 3; ++i) gw[i] = isect * normal[i] - mg[i];
    const double X = Ai[0] * gw[0] + Ai[1] * gw[1] + Ai[2] * gw[2];
    const double Y = Ai[3] * gw[0] + Ai[4] * gw[1] + Ai[5] * gw[2];
    const double dx = X - MX, dy = Y - MY;
    const double pdf_area = exp(-0.5 * (dx * dx + dy * dy) / V) / (2.0 * M_PI * V);
    const double pdf_n = pdf_area * isect * isect / fabs(npn) / jac;
    const double ndr = -(normal[0] * dir[0] + normal[1] * dir[1] + normal[2] * dir[2]);
    *pdf = (float)(pdf_n / (4.0 * ndr));
    return GPIS_OK;
}

int gor_nee(const gpis_medium_desc *desc, const float origin[3], const float dir[3],
            const float p[3], const float normal[3], float t_segment, const uint32_t seeds[4],
            const float prev[4], float *pdf, float grad[3])
{
    om_t m;
    field_t F;
    int rc = field_setup(desc, &m, &F, origin, dir, seeds, prev);
    if (rc) return rc;
    if (!m.d.one_d_sampling) return GPIS_ENOTSUP;
    if (F.n > 1) return nee_octaves(&m, &F, dir, p, normal, t_segment, pdf, grad);
    const real_t *r = &F.oct[0];
    float amp = amplitude(r);
    float mg[3];
    mean_grad_f(&m, p, mg);
    float diso[3], dn[3];
    w2l_pos(&m, dir, 1.0f, diso);
    normalize3f(diso, dn);
    frame_t f;
    frame_make(dn, &f);
    /* mtx_pt = amplitude * localToWorldInvTransposeMatrix(p) * [t b n] (row-major
       here); the nonstationary matrix divides diag(l_inv) by the maximum lateral
       scale (NonstationaryCovariance::localToWorldInvTransposeMatrix, GPFunctions.cpp:1291-1294) */
    float A[9];
    for (int i = 0; i < 3; ++i) {
        const float li = m.nonstationary ? m.l_inv[i] / m.ls_max : m.l_inv[i];
        A[3 * i + 0] = amp * li * f.t[i];
        A[3 * i + 1] = amp * li * f.b[i];
        A[3 * i + 2] = amp * li * f.n[i];
    }
    float Ai[9];
    inv3(A, Ai);
    float gc[3], info[4] = {1.0f, 1.0f, 1.0f, 0.0f};
    if (m.multires) {
        /* grad_constraint_3d on the multi-resolution grid (SparseConvolutionNoise.cpp:687-692) */
        level_ratio(&m, p, info);
        double lo[4], hi[4];
        noise1d_level(r, p, dir, 1, 0, info[0], 1, lo);
        noise1d_level(r, p, dir, 1, 0, info[1], 0, hi);
        for (int i = 0; i < 3; ++i) gc[i] = (float)lo[1 + i] * info[2] / info[0] + (float)hi[1 + i] * info[3] / info[1];
    } else {
        double gc4[4];
        noise1d_norm(r, p, dir, 1, 0, gc4);
        gc[0] = (float)gc4[1]; gc[1] = (float)gc4[2]; gc[2] = (float)gc4[3];
    }
    float ppt[3], px[3], py[3], cr[3];
    for (int i = 0; i < 3; ++i) {
        ppt[i] = A[3 * i + 2] * gc[2] + mg[i];
        px[i] = A[3 * i + 0];
        py[i] = A[3 * i + 1];
    }
    cr[0] = px[1] * py[2] - px[2] * py[1];
    cr[1] = px[2] * py[0] - px[0] * py[2];
    cr[2] = px[0] * py[1] - px[1] * py[0];
    float jac = sqrtf(dot3f(cr, cr));
    float pn[3];
    normalize3f(cr, pn);
    float isect = dot3f(ppt, pn) / dot3f(normal, pn);
    float g3w[3], g3[3];
    for (int i = 0; i < 3; ++i) grad[i] = isect * normal[i];
    for (int i = 0; i < 3; ++i) g3w[i] = grad[i] - mg[i];
    for (int i = 0; i < 3; ++i) g3[i] = Ai[3 * i + 0] * g3w[0] + Ai[3 * i + 1] * g3w[1] + Ai[3 * i + 2] * g3w[2];
    if (isect < 0.0f) { *pdf = 0.0f; return GPIS_OK; }
    float pdf_area;
    double tm[2], tv;
    if (transverse_moments(r, p, dir, 1, tm, &tv)) {
        if (!(tv > 0.)) { *pdf = 0.0f; return GPIS_OK; }
        const double dx = g3[0] - tm[0], dy = g3[1] - tm[1];
        pdf_area = (float)(exp(-0.5 * (dx * dx + dy * dy) / tv) / (2.0 * M_PI * tv));
    } else if (m.multires) {
        /* the multi-resolution law (SparseConvolutionNoise.cpp:776-808): the transverse
           scales shrink by 1 / sqrt((w_low / s_low)^2 + (w_high / s_high)^2) */
        const float a = info[2] / info[0], b = info[3] / info[1];
        const float nss = (float)(1.0 / (double)sqrtf(a * a + b * b));
        const float scx = splat_cov_1d(&m, p, p) * nss, scy = scx;
        if (!(m.d.correlation_context == GPIS_CTX_RENEWAL_PLUS && m.d.correlation_xy) || t_segment == 0.0f) {
            float sx = (float)((double)(g3[0] - gc[0]) * sqrt(2.0) * scx);
            float sy = (float)((double)(g3[1] - gc[1]) * sqrt(2.0) * scy);
            pdf_area = (float)(exp(-sx * sx / 2.0) * exp(-sy * sy / 2.0) / (2.0 * M_PI) * 2.0 * scx * scy);
        } else {
            pcg_t g;
            pcg_set_state(&g, (uint64_t)r->normal_seed);
            double xy1[2], xy2[2];
            rand_normal_2(&g, xy1);
            rand_normal_2(&g, xy2);
            const double s2 = (double)sqrtf(2.f);
            double fac, cov, mu[2];
            corr_moments(t_segment, &fac, &cov);
            for (int i = 0; i < 2; ++i) {
                xy1[i] /= s2;
                xy2[i] /= s2;
                mu[i] = fac * 2.0 * (xy1[i] * info[2] / info[0] + xy2[i] * info[3] / info[1]);
            }
            float sx = (float)((g3[0] - gc[0] - mu[0]) / sqrt(cov) * nss);
            float sy = (float)((g3[1] - gc[1] - mu[1]) / sqrt(cov) * nss);
            pdf_area = (float)(exp(-sx * sx / 2.0) * exp(-sy * sy / 2.0) / (2.0 * M_PI * cov) * (nss * nss));
        }
    } else if (!(m.d.correlation_context == GPIS_CTX_RENEWAL_PLUS && m.d.correlation_xy) || t_segment == 0.0f) {
        float scx = splat_cov_1d(&m, p, p), scy = scx;
        float sx = (float)((double)(g3[0] - gc[0]) * sqrt(2.0) * scx);
        float sy = (float)((double)(g3[1] - gc[1]) * sqrt(2.0) * scy);
        pdf_area = (float)(exp(-sx * sx / 2.0) * exp(-sy * sy / 2.0) / (2.0 * M_PI) * 2.0 * scx * scy);
    } else {
        pcg_t g;
        pcg_set_state(&g, (uint64_t)r->normal_seed);
        double xy1[2];
        rand_normal_2(&g, xy1);
        double s2 = (double)sqrtf(2.f);
        xy1[0] /= s2; xy1[1] /= s2;
        double fac, cov;
        corr_moments(t_segment, &fac, &cov);
        float sx = (float)((g3[0] - gc[0] - fac * 2.0 * xy1[0]) / sqrt(cov));
        float sy = (float)((g3[1] - gc[1] - fac * 2.0 * xy1[1]) / sqrt(cov));
        pdf_area = (float)(exp(-sx * sx / 2.0) * exp(-sy * sy / 2.0) / (2.0 * M_PI) / cov);
    }
    float cos_l = fabsf(dot3f(normal, pn));
    float pdf_n = pdf_area * (isect * isect) / cos_l / jac;
    float nd[3] = {-dir[0], -dir[1], -dir[2]};
    *pdf = (float)(pdf_n / (4.0 * dot3f(normal, nd)));
    return GPIS_OK;
}

void gor_se_splat_1d(const float *q, const float *c, uint32_t n, float scale,
                     double *values, double *derivatives)
{
    for (uint32_t i = 0; i < n; ++i) {
        const double delta = (double)q[i] - c[i];
        values[i] = exp(-delta * delta / (2.0 * scale * scale));
        derivatives[i] = -delta / ((double)scale * scale) * values[i];
    }
}

/* ------------------------------------------------------------------------ */
/* Medium queries: GaussianProcessMedium state machines                      */
/* ------------------------------------------------------------------------ */
/* sampleDistance / beginDistance / resumeDistance / finishDistance
 * (GaussianProcessMedium.cpp:222-381) and transmittance (:383-440), with the
 * state updates of finishGpisSegment (SparseConvolutionNoiseMedium.cpp:265-347). */

static void gm_flight(const gpis_medium_desc *d, const gpis_ray *r, float far_t, const gpis_medium_state *st,
                      float jitter, int shadow, float rec[8])
{
    float on[4] = {r->pos[0], r->pos[1], r->pos[2], r->near_t};
    float df[4] = {r->dir[0], r->dir[1], r->dir[2], far_t};
    uint32_t sd[4], ns, nm, jb;
    gor_flight_seeds(d, st->pixel_sample_segment, st->scene_seed, &ns, &nm);
    memcpy(&jb, &jitter, 4);
    int first = st->first_scatter != 0;
    sd[0] = ns; sd[1] = nm; sd[2] = (first ? GPIS_FLAG_FIRST_SCATTER : 0u) | (shadow ? GPIS_FLAG_SHADOW : 0u); sd[3] = jb;
    float pv[4] = {first ? 0.0f : st->last_val, first ? 0.0f : st->last_aniso[0], first ? 0.0f : st->last_aniso[1],
                   first ? 0.0f : st->last_aniso[2]};
    gpis_flight_soa in = {on, df, sd, pv, NULL};
    gpis_result_soa out = {rec};
    gor_trace_flights(d, 1, &in, &out, 1, 1);
}

/* samplingScheme (SparseConvolutionNoise.cpp:68-76) at a hit t along the flight: UNI
 * for a vanishing amplitude, and at the observed origin (t = 0 after a Renewal+
 * conditioning) under correlationXY for the stationary SE covariance */
static uint32_t gm_scheme(const gpis_medium_desc *d, int conditioned_rp, float t)
{
    if (d->single_realization || !d->one_d_sampling) return GPIS_SCHEME_UNI;
    if (d->sigma < 1e-6f) return GPIS_SCHEME_UNI;
    if (d->correlation_xy && conditioned_rp && t == 0.0f && d->ls_kind == GPIS_LS_CONSTANT) return GPIS_SCHEME_UNI;
    return d->sampling_scheme;
}

static void gm_finish_segment(const gpis_medium_desc *d, const float rec[8], gpis_medium_state *st)
{
    int rp = !d->single_realization && d->correlation_context == GPIS_CTX_RENEWAL_PLUS && st->first_scatter == 0;
    uint32_t status;
    memcpy(&status, &rec[7], 4);
    if (rec[5] == 0.0f) {
        st->last_gp_id = (int32_t)((status >> 8) & 0xFFu);
        st->sampling_scheme = gm_scheme(d, rp, rec[0]);
        st->last_val = 0.0f;
    } else {
        st->sampling_scheme = GPIS_SCHEME_UNI;
        st->last_val = rec[1];
    }
}

int gor_medium_sample_distance(const gpis_medium_desc *d, const gpis_ray *rays, gpis_medium_state *states,
                               const float *jitter, gpis_medium_sample *samples, uint32_t n)
{
    float sa = d->sigma_a * d->density, ss = d->sigma_s * d->density, stt = sa + ss;
    int absorption_only = ss == 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        const gpis_ray *r = &rays[i];
        gpis_medium_sample *s = &samples[i];
        gpis_medium_state *st = &states[i];
        memset(s, 0, sizeof(*s));
        float far_t = r->far_t;
        if (!isfinite(far_t)) far_t = (float)((double)r->near_t + 2000);
        float maxT = far_t;
        if (st->bounce >= d->max_bounces) { s->status = 0; continue; }
        if (maxT <= r->near_t) {
            s->t = maxT;
            s->weight[0] = s->weight[1] = s->weight[2] = 1.0f;
            s->pdf = 1.0f; s->exited = 1;
            for (int k = 0; k < 3; ++k) s->p[k] = r->pos[k] + s->t * r->dir[k];
            s->sampling_scheme = GPIS_SCHEME_UNI; s->status = 1;
            continue;
        }
        float rec[8];
        if (absorption_only) {
            gm_flight(d, r, far_t, st, jitter[i], 1, rec);
            gm_finish_segment(d, rec, st);
            float tr = rec[5] == 0.0f ? 0.0f : 1.0f;
            if (rec[0] < far_t) {
                st->last_aniso[0] = rec[2]; st->last_aniso[1] = rec[3]; st->last_aniso[2] = rec[4];
                st->first_scatter = 0;
            }
            s->t = far_t;
            s->weight[0] = s->weight[1] = s->weight[2] = tr;
            s->pdf = 1.0f; s->exited = 1; s->sampling_scheme = GPIS_SCHEME_UNI;
            for (int k = 0; k < 3; ++k) s->p[k] = r->pos[k] + s->t * r->dir[k];
            s->gp_id = st->last_gp_id;
            st->info_t += s->t;
            s->status = 1;
            continue;
        }
        gm_flight(d, r, far_t, st, jitter[i], 0, rec);
        uint32_t fst;
        memcpy(&fst, &rec[7], 4);
        if ((fst & 0xFFu) != GPIS_FLIGHT_OK) { s->status = 0; continue; }
        gm_finish_segment(d, rec, st);
        double t = rec[0];
        int hit = rec[5] == 0.0f;
        s->exited = !hit;
        if (t < maxT) {
            s->aniso[0] = rec[2]; s->aniso[1] = rec[3]; s->aniso[2] = rec[4];
            st->last_aniso[0] = rec[2]; st->last_aniso[1] = rec[3]; st->last_aniso[2] = rec[4];
            st->first_scatter = 0;
            if (!isfinite((rec[2] + rec[3] + rec[4]) / 3.0f)) {
                s->aniso[0] = 1.0f; s->aniso[1] = s->aniso[2] = 0.0f;
                s->status = 0;
                continue;
            }
        }
        if (hit) {
            double dot = (double)s->aniso[0] * r->dir[0] + (double)s->aniso[1] * r->dir[1] + (double)s->aniso[2] * r->dir[2];
            if (dot > 0) { s->status = 0; continue; }
            double l2 = (double)s->aniso[0] * s->aniso[0] + (double)s->aniso[1] * s->aniso[1] + (double)s->aniso[2] * s->aniso[2];
            if (l2 < 0.0000001f) {
                s->aniso[0] = 1.0f; s->aniso[1] = s->aniso[2] = 0.0f;
                s->status = 0;
                continue;
            }
        } else {
            s->aniso[0] = rec[2]; s->aniso[1] = rec[3]; s->aniso[2] = rec[4];
        }
        float ratio = ss / stt;
        s->t = fminf((float)t, maxT);
        s->continued_t = (float)t;
        for (int k = 0; k < 3; ++k) { s->weight[k] = ratio; s->continued_weight[k] = ratio; }
        s->pdf = 1.0f;
        st->last_aniso[0] = s->aniso[0]; st->last_aniso[1] = s->aniso[1]; st->last_aniso[2] = s->aniso[2];
        s->sampling_scheme = st->sampling_scheme;
        st->first_scatter = 0;
        st->bounce += 1;
        st->sampling_scheme = GPIS_SCHEME_UNI;
        for (int k = 0; k < 3; ++k) s->p[k] = r->pos[k] + s->t * r->dir[k];
        s->gp_id = st->last_gp_id;
        st->info_t += s->t;
        s->status = 1;
    }
    return GPIS_OK;
}

int gor_medium_transmittance(const gpis_medium_desc *d, const gpis_ray *rays, gpis_medium_state *states,
                             const float *jitter, float *transmittance, uint32_t n)
{
    for (uint32_t i = 0; i < n; ++i) {
        const gpis_ray *r = &rays[i];
        gpis_medium_state *st = &states[i];
        transmittance[i] = 1.0f;
        if (r->far_t <= r->near_t) continue;
        float far_t = r->far_t;
        if (!isfinite(far_t)) far_t = (float)((double)r->near_t + 2000);
        float rec[8];
        gm_flight(d, r, far_t, st, jitter[i], 1, rec);
        uint32_t fst;
        memcpy(&fst, &rec[7], 4);
        if ((fst & 0xFFu) != GPIS_FLIGHT_OK) { transmittance[i] = 0.0f; continue; }
        gm_finish_segment(d, rec, st);
        if (rec[0] < far_t) {
            st->last_aniso[0] = rec[2]; st->last_aniso[1] = rec[3]; st->last_aniso[2] = rec[4];
            st->first_scatter = 0;
            if (!isfinite((rec[2] + rec[3] + rec[4]) / 3.0f)) { transmittance[i] = 0.0f; continue; }
        }
        transmittance[i] = rec[5] == 0.0f ? 0.0f : 1.0f;
    }
    return GPIS_OK;
}
