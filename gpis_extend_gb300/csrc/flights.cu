// flights.cu -- sm_103a kernels of the GPIS ray-flight path.
//
// One batch of flights runs as three kernels on one stream:
//   k_prepare  Renewal / Renewal+ conditioning at the origin of every
//              secondary flight (SparseConvolutionNoise.cpp:488-656), one thread
//              per flight, coefficients to a scratch record;
//   k_march    the first-sign-change march and regula-falsi back-off
//              (SparseConvolutionNoiseMedium.cpp:287-346): persistent warps pull
//              flights from a device work counter and refill finished lanes, so
//              flights of very uneven length keep every lane busy; value-only
//              field evaluations; the 1D variant keeps the impulses of the three
//              cells around the query in registers and regenerates a cell only
//              when the query crosses a cell boundary;
//   k_finish   the gradient sample at the end point (evaluateGradient,
//              SparseConvolutionNoise.cpp:133-296), one thread per flight.
//
// Bit-exactness: cell hashes and PCG draws are integer-exact; the march
// parameter t is a float-float pair equal to the reference's double t; the point,
// the isotropic transform, the ray-space coordinate and the cell decomposition
// are evaluated op-for-op in IEEE float without contraction, so the set of
// impulses inside the truncated kernel is the reference's.  The splat values
// use ex2.approx and agree with an FP64 evaluation to ~1e-6 relative.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <type_traits>

#include <cooperative_groups.h>

#include "flights.cuh"
#include "ffmath.cuh"

namespace gpis {

__constant__ PcgJump c_jump[kMaxDraws];

cudaError_t upload_pcg_table()
{
    PcgJump h[kMaxDraws];
    uint64_t a = 1, c = 0;
    const uint64_t M = 6364136223846793005ULL;
    for (int k = 0; k < kMaxDraws; ++k) {
        h[k].alo = (uint32_t)a; h[k].ahi = (uint32_t)(a >> 32);
        h[k].clo = (uint32_t)c; h[k].chi = (uint32_t)(c >> 32);
        a = a * M;
        c = c * M + 1ULL;
    }
    return cudaMemcpyToSymbol(c_jump, h, sizeof(h));
}

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr float LOG2E = 1.4426950408889634f;

// Conditioning kernels of the 1D Renewal(+) update (GPFunctions.cpp:850-875) for the
// local scale a (1 when stationary; sqrt of the mean squared kernel scale of the
// two points otherwise, getNonstationaryCovSplatCov1D, GPFunctions.cpp:1723-1734):
// exp(-d^2/(4a^2)), its first and second derivative and the transverse factor.
struct Cov1D { float k0, k1, k2, k3; };

__device__ __forceinline__ Cov1D cov1d(float d, float a = 1.0f)
{
    Cov1D c;
    const float ia2 = a == 1.0f ? 1.0f : 1.0f / (a * a);
    c.k0 = ex2_approx((-0.25f * LOG2E) * ia2 * d * d);
    c.k1 = -0.5f * ia2 * d * c.k0;
    c.k2 = (0.25f * ia2 * ia2 * d * d - 0.5f * ia2) * c.k0;
    c.k3 = -0.5f * ia2 * c.k0;
    return c;
}

// ---- octaves and the nonstationary length scale --------------------------------
__device__ __forceinline__ float oct_sigma(const DevMedium &m, int k) { return m.n_oct == 1 ? m.sigma : m.oct_sigma[k]; }
__device__ __forceinline__ float oct_scale(const DevMedium &m, int k) { return m.n_oct == 1 ? 1.0f : m.oct_scale[k]; }
__device__ __forceinline__ uint32_t oct_seed(const DevMedium &m, int k) { return m.n_oct == 1 ? 0u : m.oct_seed[k]; }
__device__ __forceinline__ uint32_t oct_normal_seed(const DevMedium &m, uint32_t s, int k)
{
    return m.n_oct == 1 ? s : s + (uint32_t)k * 0x9E3779B9u;
}

// nonStationarySplattingKernelScale = ls(p) / ls_max (GPFunctions.cpp:1229-1235); 1 when stationary.
__device__ __forceinline__ float ns_scale(const DevMedium &m, float x, float z)
{
    if (m.ls_kind == 0u) return 1.0f;
    const float *q = m.ls_params;
    return __fdiv_rn(q[0] + q[1] * sinf(q[2] * x) * cosf(q[3] * z), m.ls_max);
}

// The same with the procedural vector evaluated in double, as on Vec3d(p).
__device__ __forceinline__ float ns_scale_precise(const DevMedium &m, float x, float z)
{
    if (m.ls_kind == 0u) return 1.0f;
    const float *q = m.ls_params;
    const double v = __dmul_rn(__dmul_rn((double)q[1], sin(__dmul_rn((double)q[2], (double)x))),
                               cos(__dmul_rn((double)q[3], (double)z)));
    const float ls = (float)__dadd_rn((double)q[0], v);
    return __fdiv_rn(ls, m.ls_max);
}

// ---- multi-resolution grid ---------------------------------------------------------
// ls(p) of the procedural length scale (the grid's lateral scale): float, and the
// double evaluation on Vec3d(p) as ns_scale_precise takes it.
__device__ __forceinline__ float ls_value(const DevMedium &m, float x, float z)
{
    const float *q = m.ls_params;
    return q[0] + q[1] * sinf(q[2] * x) * cosf(q[3] * z);
}

__device__ __forceinline__ float ls_value_precise(const DevMedium &m, float x, float z)
{
    const float *q = m.ls_params;
    const double v = __dmul_rn(__dmul_rn((double)q[1], sin(__dmul_rn((double)q[2], (double)x))),
                               cos(__dmul_rn((double)q[3], (double)z)));
    return (float)__dadd_rn((double)q[0], v);
}

// The two levels around ls: scales, weights and noise-seed offsets
// (kernelScaleLevelRatio, SparseConvolutionNoise.cpp:101-111, and the seed
// offset of evaluateNoise1DNormalized, :385).
struct MrLevels {
    float s[2], w[2];
    uint32_t seed[2];
};

__device__ __forceinline__ MrLevels mr_levels(const DevMedium &m, float ls)
{
    const float lv = floorf(__fdiv_rn(logf(ls), m.mr_log_base));
    int li = (int)lv;
    li = li < -kMrLevels ? -kMrLevels : (li > kMrLevels - 2 ? kMrLevels - 2 : li);
    MrLevels r;
    r.s[0] = m.mr_pow[li + kMrLevels];
    r.s[1] = m.mr_pow[li + kMrLevels + 1];
    r.seed[0] = (uint32_t)m.mr_seed[li + kMrLevels];
    r.seed[1] = (uint32_t)m.mr_seed[li + kMrLevels + 1];
    const float frac = __fdiv_rn(__fsub_rn(ls, r.s[0]), __fsub_rn(r.s[1], r.s[0]));
    const double f = (double)frac;
    const double den = __dsqrt_rn(__dadd_rn(__dsub_rn(1.0, __dmul_rn(2.0, f)), __dmul_rn(__dmul_rn(2.0, f), f)));
    r.w[0] = (float)__ddiv_rn(__dsub_rn(1.0, f), den);
    r.w[1] = (float)__ddiv_rn(f, den);
    return r;
}

// sqr(w_low) + sqr(w_high): the conditioning coefficients' divisor (conditioning1D, :602-633)
__device__ __forceinline__ float mr_norm(const MrLevels &l)
{
    return __fadd_rn(__fmul_rn(l.w[0], l.w[0]), __fmul_rn(l.w[1], l.w[1]));
}

// getNonstationaryCovSplatCov1D(pq, pc) for the isotropic field.
__device__ __forceinline__ float splat_cov_1d(float sq, float sc)
{
    if (sq == 1.0f && sc == 1.0f) return 1.0f;
    // (float)(0.5 * (double)x) is exactly 0.5f * x for normal x
    return __fsqrt_rn(__fmul_rn(0.5f, __fadd_rn(__fmul_rn(sq, sq), __fmul_rn(sc, sc))));
}

// World -> isotropic ray-space direction frame of a flight (the nonstationary
// transform divides by the maximum lateral scale before normalising).
__device__ __forceinline__ void ray_frame(const DevMedium &m, float dx, float dy, float dz, Frame &f)
{
    float ix = __fmul_rn(m.l_inv[0], dx), iy = __fmul_rn(m.l_inv[1], dy), iz = __fmul_rn(m.l_inv[2], dz);
    if (m.ls_kind) {
        ix = __fdiv_rn(ix, m.ls_max);
        iy = __fdiv_rn(iy, m.ls_max);
        iz = __fdiv_rn(iz, m.ls_max);
    }
    normalize3_rn(ix, iy, iz);
    make_frame(ix, iy, iz, f);
}

// The frame of transformPosDirWorldtoLocal(dir, s).normalized() at a level scale s.
__device__ __forceinline__ void ray_frame_level(const DevMedium &m, const float d[3], float s, Frame &f)
{
    float ix = __fdiv_rn(__fmul_rn(m.l_inv[0], d[0]), s);
    float iy = __fdiv_rn(__fmul_rn(m.l_inv[1], d[1]), s);
    float iz = __fdiv_rn(__fmul_rn(m.l_inv[2], d[2]), s);
    normalize3_rn(ix, iy, iz);
    make_frame(ix, iy, iz, f);
}

// Isotropic ray-space coordinate p_iso_ray.z (SparseConvolutionNoise.cpp:381-384).
__device__ __forceinline__ float ray_coord(const float *li, const float *n, float px, float py, float pz)
{
    return dot3_rn(n[0], n[1], n[2], __fmul_rn(li[0], px), __fmul_rn(li[1], py), __fmul_rn(li[2], pz));
}

// The coordinate of octave k (length scale x sc) of a nonstationary or octave medium.
__device__ __forceinline__ float ray_coord_oct(const DevMedium &m, const float *n, float px, float py, float pz, float sc)
{
    float x = __fmul_rn(m.l_inv[0], px), y = __fmul_rn(m.l_inv[1], py), z = __fmul_rn(m.l_inv[2], pz);
    if (m.ls_kind) {
        x = __fdiv_rn(x, m.ls_max);
        y = __fdiv_rn(y, m.ls_max);
        z = __fdiv_rn(z, m.ls_max);
    }
    if (sc != 1.0f) {
        x = __fdiv_rn(x, sc);
        y = __fdiv_rn(y, sc);
        z = __fdiv_rn(z, sc);
    }
    return dot3_rn(n[0], n[1], n[2], x, y, z);
}

// 1 / sqrt(sparseConvNoiseVariance1D) at kernel scale ls.
__device__ __forceinline__ float inv_norm_1d(const DevMedium &m, float ls)
{
    return ls == 1.0f ? m.inv_norm1d : m.inv_norm1d * rsqrtf(ls);
}

// ---- 1D noise, generic impulse count (no cache) --------------------------------
// Returns the raw (unnormalized) sum and its derivative w.r.t. the iso coordinate;
// ls is the local kernel scale (splattingKernel1D takes it at the query point).
template <bool DERIV, bool MARGIN = false>
__device__ void noise1d_generic(const DevMedium &m, float z, uint32_t seed, float &v, float &dv, float ls = 1.0f,
                                float *margin = nullptr)
{
    const float tg = __fdiv_rn(z, m.kr_iso);
    const float fl = floorf(tg);
    const float frac = __fsub_rn(tg, fl);
    const int ci = (int)fl;
    const float il2 = 1.0f / (ls * ls);
    const float kexp = m.kexp1d * il2;
    float sv = 0.0f, sd = 0.0f;
    // MARGIN: the distance in cells from the query to the nearest support edge of
    // an impulse of the three cells or to its cell's faces
    float mg = fminf(frac, 1.0f - frac);
    for (int dx = -1; dx <= 1; ++dx) {
        const float tl = __fsub_rn(frac, (float)dx);
        const uint32_t s = xxhash2((uint32_t)(ci + dx), seed) + 1u;
        for (uint32_t k = 0; k < m.n_imp; ++k) {
            const float ti = unit_float(pcg_draw(c_jump[2 + 2 * k], s));
            const uint32_t wr = pcg_draw(c_jump[3 + 2 * k], s);
            const float tp = __fsub_rn(tl, ti);
            if (MARGIN) mg = fminf(mg, fabsf(fabsf(tp) - 1.0f));
            if (fabsf(tp) < 1.0f) {
                const float e = ex2_approx(kexp * (tp * tp));
                const float w = (wr >> 31) ? 1.0f : -1.0f;
                sv += w * e;
                if (DERIV) sd += w * (-(m.kr_iso * tp) * il2 * e);
            }
        }
    }
    v = sv;
    dv = sd;
    // less 16 ulps of the cell coordinate for the rounding of the points and of z
    if (MARGIN) *margin = mg - 0x1p-19f * (fabsf(tg) + 1.0f);
}

// ---- 3D world-space noise, generic (no cache) ----------------------------------
// Raw sum and gradient (world units), noise3D + cell3D (SparseConvolutionNoise.cpp:419-452).
//
// With BOUND, also the range of the raw sum over the segment [p, p + E] (E in cell
// units, the segment inside p's cell, so that the 27 cells hold every impulse whose
// support meets it): per impulse the kernel's largest value on the segment (at the
// nearest point, with the least negative exponent coefficient kmax2 per squared cell
// distance; 0 when the segment misses the support) and its smallest (at the farther
// end, coefficient kmin2; 0 when the segment leaves the support).  A positive weight
// adds [smallest, largest] to [lo, hi], a negative one [-largest, -smallest].  The
// support tests are widened by kSupportEps against the float rounding of the points,
// and the kernel values moved outward by 1e-5 against ex2.approx.
constexpr float kSupportEps = 1e-4f;

template <bool GRAD, bool BOUND>
__device__ void noise3d_core(const DevMedium &m, float px, float py, float pz, uint32_t seed, float &v, float g[3],
                             const float E[3], float ee, float kmax2, float kmin2, float &lo, float &hi)
{
    const float kr = m.kr_world;
    const float p[3] = {px, py, pz};
    float fr[3];
    int ijk[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float q = __fdiv_rn(p[i], kr);
        const float fl = floorf(q);
        fr[i] = __fsub_rn(q, fl);
        ijk[i] = (int)fl;
    }
    const bool xfirst = (m.flags & MF_XYZ_ORDER) != 0;
    float sv = 0.0f, s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
    float blo = 0.0f, bhi = 0.0f;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                const float t0 = __fsub_rn(fr[0], (float)dx), t1 = __fsub_rn(fr[1], (float)dy),
                            t2 = __fsub_rn(fr[2], (float)dz);
                const uint32_t s = xxhash4((uint32_t)(ijk[2] + dz), (uint32_t)(ijk[1] + dy),
                                           (uint32_t)(ijk[0] + dx), seed) + 1u;
                for (uint32_t k = 0; k < m.n_imp; ++k) {
                    // all four draws unconditionally: early exits per coordinate make the
                    // lanes diverge and measured slower than the straight-line form
                    const int b = 2 + 4 * (int)k;
                    const float r0 = unit_float(pcg_draw(c_jump[b], s));
                    const float r1 = unit_float(pcg_draw(c_jump[b + 1], s));
                    const float r2 = unit_float(pcg_draw(c_jump[b + 2], s));
                    const uint32_t wr = pcg_draw(c_jump[b + 3], s);
                    const float ix = xfirst ? r0 : r2, iy = r1, iz = xfirst ? r2 : r0;
                    const float a0 = __fsub_rn(t0, ix), a1 = __fsub_rn(t1, iy), a2 = __fsub_rn(t2, iz);
                    const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(a0, a0), __fmul_rn(a1, a1)), __fmul_rn(a2, a2));
                    if (l2 < 1.0f) {
                        const float ab0 = kr * a0, ab1 = kr * a1, ab2 = kr * a2;
                        const float e = ex2_approx(m.kexp3d[0] * ab0 * ab0 + m.kexp3d[1] * ab1 * ab1 +
                                                   m.kexp3d[2] * ab2 * ab2);
                        const float w = (wr >> 31) ? 1.0f : -1.0f;
                        sv += w * e;
                        if (GRAD) {
                            s0 += w * (-2.0f * (ab0 * m.m3[0]) * e);
                            s1 += w * (-2.0f * (ab1 * m.m3[1]) * e);
                            s2 += w * (-2.0f * (ab2 * m.m3[2]) * e);
                        }
                    }
                    if (BOUND) {
                        const float ae = a0 * E[0] + a1 * E[1] + a2 * E[2];
                        const float sn = fminf(fmaxf(-ae / ee, 0.0f), 1.0f);
                        const float b2 = fmaxf(l2 + sn * (2.0f * ae + sn * ee), 0.0f);
                        if (b2 < 1.0f + kSupportEps) {
                            const float big = ex2_approx(kmax2 * b2) * 1.00001f;
                            const float far2 = fmaxf(l2, l2 + 2.0f * ae + ee);
                            const float small = far2 < 1.0f - kSupportEps ? ex2_approx(kmin2 * far2) * 0.99999f : 0.0f;
                            if (wr >> 31) {
                                blo += small;
                                bhi += big;
                            } else {
                                blo -= big;
                                bhi -= small;
                            }
                        }
                    }
                }
            }
    v = sv;
    if (GRAD) { g[0] = s0; g[1] = s1; g[2] = s2; }
    if (BOUND) { lo = blo; hi = bhi; }
}

template <bool GRAD>
__device__ void noise3d_generic(const DevMedium &m, float px, float py, float pz, uint32_t seed,
                                float &v, float g[3])
{
    const float E[3] = {0.0f, 0.0f, 0.0f};
    float lo, hi;
    noise3d_core<GRAD, false>(m, px, py, pz, seed, v, g, E, 1.0f, 0.0f, 0.0f, lo, hi);
}

// 3D conditioning splat (value and gradient) of the coefficients c at p.
__device__ __forceinline__ void cond3d(const DevMedium &m, const CondRec &c, const float o[3],
                                       const float p[3], float &v, float g[3])
{
    float ab[3], dp[3];
    float absq = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        ab[i] = p[i] - o[i];
        absq += ab[i] * m.m3c[i] * ab[i];
    }
    const float f = ex2_approx(-LOG2E * absq);
#pragma unroll
    for (int i = 0; i < 3; ++i) dp[i] = -2.0f * (ab[i] * m.m3c[i]);
    const CondOct &co = c.oct[0];
    v = f * co.vs;
#pragma unroll
    for (int j = 0; j < 3; ++j) g[j] = dp[j] * f * co.vs;
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
        v += dp[cc] * f * co.gs[cc];
#pragma unroll
        for (int j = 0; j < 3; ++j) g[j] += (dp[cc] * dp[j] - (cc == j ? 2.0f * m.m3c[cc] : 0.0f)) * f * co.gs[cc];
    }
}

// Box-Muller pair (Gaussian.cpp:23-35) from two PCG outputs, in float.
__device__ __forceinline__ void normal_pair(uint32_t r1, uint32_t r2, float &z0, float &z1)
{
    const float u1 = unit_float(r1), u2 = unit_float(r2);
    const float rad = sqrtf(-2.0f * logf(1.0f - u1));
    float sn, cs;
    sincosf(6.28318548f * u2, &sn, &cs);
    z0 = rad * cs;
    z1 = rad * sn;
}

// The normal-seed stream: set_state(normalSeed) then draws 2.. (after the 2 warm-ups).
__device__ __forceinline__ void normal_draws(uint32_t seed, int pair, float &z0, float &z1)
{
    normal_pair(pcg_draw(c_jump[2 + 2 * pair], seed), pcg_draw(c_jump[3 + 2 * pair], seed), z0, z1);
}

// Box-Muller as the reference evaluates it, in double (Gaussian.cpp:23-35; PI is
// the float constant of Angle.hpp:8, so 2*PI is formed in float before it meets
// the double u2), of the uniform draws u1f, u2f.  Out of line: normal_pair_scaled
// takes it only when its float-float evaluation cannot decide the rounding.
__device__ __noinline__ void normal_draws_double(float u1f, float u2f, double &z0, double &z1)
{
    const double u1 = (double)u1f;
    const double u2 = (double)u2f;
    const double r = sqrt(-2.0 * log(1.0 - u1));
    const float two_pi = 2.0f * 3.1415926536f;
    double sn, cs;
    sincos((double)two_pi * u2, &sn, &cs);
    z0 = r * cs;
    z1 = r * sn;
}

// The pair of draws `pair` of the normal-seed stream as the reference's double
// Box-Muller gives it, divided by sqrt(2)_f and by sc in double and rounded to
// float (the conditioning gradient of a conditioned flight, where the transverse
// draws enter the along-ray coefficient through the rounding of the frame
// transforms): float-float with a test of the rounding (ffm_normal_pair), the
// double evaluation for the draws it cannot decide (about 2e-4 of the pairs).
__device__ __forceinline__ void normal_pair_scaled(uint32_t seed, int pair, float sc, float &g0, float &g1)
{
    const float u1 = unit_float(pcg_draw(c_jump[2 + 2 * pair], seed));
    const float u2 = unit_float(pcg_draw(c_jump[3 + 2 * pair], seed));
    if (ffm_normal_pair(u1, u2, sc, g0, g1)) return;
    double z0, z1;
    normal_draws_double(u1, u2, z0, z1);
    const double s2 = 1.4142135381698608;   // (double)sqrtf(2.f)
    const double xs = 1.0 / (double)sc;
    g0 = (float)(z0 / s2 * xs);
    g1 = (float)(z1 / s2 * xs);
}

// correlatedGradientMoments (SparseConvolutionNoise.cpp:13-22)
__device__ __forceinline__ void corr_moments(float dist, float &factor, float &variance)
{
    const float x = 0.5f * dist * dist;
    factor = 0.5f * expf(-0.5f * x) * (1.0f - x);
    variance = x < 1.0f ? 0.5f * (-expm1f(-x) + expf(-x) * x * (2.0f - x)) : 0.5f - 2.0f * factor * factor;
}

struct FlightIn {
    float o[3], d[3], near_t, far_t, jitter;
    uint32_t noise_seed, normal_seed, flags;
    float prev_v, prev_g[3];
};

__device__ __forceinline__ FlightIn load_flight(const FlightArgs &a, uint32_t i)
{
    FlightIn f;
    const float4 on = a.origin_near[i];
    const float4 df = a.dir_far[i];
    const uint4 sd = a.seeds[i];
    f.o[0] = on.x; f.o[1] = on.y; f.o[2] = on.z; f.near_t = on.w;
    f.d[0] = df.x; f.d[1] = df.y; f.d[2] = df.z; f.far_t = df.w;
    f.noise_seed = sd.x; f.normal_seed = sd.y; f.flags = sd.z; f.jitter = __uint_as_float(sd.w);
    if (a.prev) {
        const float4 pv = a.prev[i];
        f.prev_v = pv.x; f.prev_g[0] = pv.y; f.prev_g[1] = pv.z; f.prev_g[2] = pv.w;
    } else {
        f.prev_v = 0.0f; f.prev_g[0] = f.prev_g[1] = f.prev_g[2] = 0.0f;
    }
    return f;
}

// Input validation of RaySegmentBatch.cu:198-206.
__device__ __forceinline__ bool flight_valid(const FlightIn &f)
{
    const bool first = (f.flags & GPIS_FLAG_FIRST_SCATTER) != 0;
    bool ok = isfinite(f.near_t) && isfinite(f.far_t) && f.far_t > f.near_t && isfinite(f.jitter) &&
              f.jitter >= 0.0f && f.jitter < 1.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) ok = ok && isfinite(f.o[i]) && isfinite(f.d[i]);
    if (!first)
        ok = ok && isfinite(f.prev_v) && isfinite(f.prev_g[0]) && isfinite(f.prev_g[1]) && isfinite(f.prev_g[2]);
    const float dd = f.d[0] * f.d[0] + f.d[1] * f.d[1] + f.d[2] * f.d[2];
    return ok && fabsf(dd - 1.0f) <= 0.001f;
}

__device__ __forceinline__ const DevMedium *medium_of(const FlightArgs &a, uint32_t i, bool &ok)
{
    const uint32_t mi = a.medium ? a.medium[i] : 0u;
    ok = mi < (uint32_t)a.n_media;
    return a.media + (ok ? mi : 0u);
}

// flights of the launch: the capacity n, or the live count in device memory
__device__ __forceinline__ uint32_t live_n(const FlightArgs &a)
{
    return a.n_dev ? min(*a.n_dev, a.n) : a.n;
}

__device__ __forceinline__ bool conditioned(const DevMedium &m, const FlightIn &f)
{
    return (m.flags & MF_COND) && !(f.flags & GPIS_FLAG_FIRST_SCATTER);
}

// Transverse moments of the exact SE law (seTransverseGradientMoments, :78-99).
__device__ void transverse_moments(const DevMedium &m, const CondRec &c, const float o[3],
                                   const float p[3], const Frame &f, bool cond, float &m0, float &m1, float &var)
{
    m0 = m1 = 0.0f;
    var = 0.5f;
    if (cond && c.has_obs) {
        float dl[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) dl[i] = __fmul_rn(m.l_inv[i], __fsub_rn(p[i], o[i]));
        const double q2 = 0.5 * ((double)dl[0] * dl[0] + (double)dl[1] * dl[1] + (double)dl[2] * dl[2]);
        const float rho = (float)exp(-0.5 * q2);
        var = (float)(-0.5 * expm1(-q2));
        float og[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) og[i] = m.l_aniso[i] * c.tgn[i];
        const float ox = dot3_rn(f.t[0], f.t[1], f.t[2], og[0], og[1], og[2]);
        const float oy = dot3_rn(f.b[0], f.b[1], f.b[2], og[0], og[1], og[2]);
        m0 = rho * ox;
        m1 = rho * oy;
    }
}

// One level of the multi-resolution 1D noise at p (evaluateNoise1DNormalized at
// kernelSpatialScale s): value, derivative along the ray and the transverse
// conditioning splats; ow is the origin's weight of the level.
__device__ __forceinline__ void noise1d_level(const DevMedium &m, const FlightIn &fl, const CondOct &co, bool cond,
                                              const Frame &f, const float p[3], float s, uint32_t seed_off, float ow,
                                              float &v, float &dv, float &gcx, float &gcy)
{
    const float z = ray_coord_oct(m, f.n, p[0], p[1], p[2], s);
    noise1d_generic<true>(m, z, fl.noise_seed + seed_off, v, dv, 1.0f);
    v *= m.inv_norm1d;
    dv *= m.inv_norm1d;
    gcx = gcy = 0.0f;
    if (cond) {
        const float oz = ray_coord_oct(m, f.n, fl.o[0], fl.o[1], fl.o[2], s);
        const Cov1D k = cov1d(z - oz);
        const float gzs = s * co.gs[2];
        v += ow * (co.vs * k.k0 + gzs * k.k1);
        dv += ow * (co.vs * k.k1 + gzs * k.k2);
        if (m.flags & MF_CORR_XY) {
            gcx = ow * s * co.gs[0] * k.k3;
            gcy = ow * s * co.gs[1] * k.k3;
        }
    }
}

// evaluateGradientNoise1D on the multi-resolution grid (SparseConvolutionNoise.cpp:
// 244-295): both levels' base gradients, a normal pair per level at the start of
// the ray (pairs 0, 1) and at its end (pairs 2, 3), each level's gradient taken
// to world space through its own frame and scale, blended by the level weights.
__device__ void noise1d_precise_vd(const DevMedium &m, float z, uint32_t seed, float ls, float &value, float &deriv);

__device__ void noise_gradient_mr(const DevMedium &m, const FlightIn &fl, const CondRec &c, bool cond,
                                  const float p[3], float t_segment, float &value, float g[3],
                                  bool precise = false)
{
    const MrLevels lv = mr_levels(m, ls_value_precise(m, p[0], p[2]));
    if (precise && !cond && t_segment == 0.0f) {
        // the conditioning's value and birth gradient at the origin, operation for
        // operation: each level's precise value and derivative, the double normal
        // pairs (low level first), the level frames and scales, the blend unfused
        Frame f;
        ray_frame(m, fl.d[0], fl.d[1], fl.d[2], f);
        float v[2], dv[2];
#pragma unroll 1
        for (int j = 0; j < 2; ++j) {
            const float z = ray_coord_oct(m, f.n, p[0], p[1], p[2], lv.s[j]);
            noise1d_precise_vd(m, z, fl.noise_seed + lv.seed[j], 1.0f, v[j], dv[j]);
        }
        value = __fadd_rn(__fmul_rn(lv.w[0], v[0]), __fmul_rn(lv.w[1], v[1]));
        float gw[2][3];
#pragma unroll 1
        for (int j = 0; j < 2; ++j) {
            float g0, g1;
            normal_pair_scaled(fl.normal_seed, j, 1.0f, g0, g1);
            const float gq[3] = {__fadd_rn(g0, 0.0f), __fadd_rn(g1, 0.0f), __fadd_rn(0.0f, dv[j])};
            Frame fj;
            ray_frame_level(m, fl.d, lv.s[j], fj);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float gi = __fadd_rn(__fadd_rn(__fmul_rn(fj.t[i], gq[0]), __fmul_rn(fj.b[i], gq[1])),
                                           __fmul_rn(fj.n[i], gq[2]));
                gw[j][i] = __fdiv_rn(__fmul_rn(m.l_inv[i], gi), lv.s[j]);
            }
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) g[i] = __fadd_rn(__fmul_rn(lv.w[0], gw[0][i]), __fmul_rn(lv.w[1], gw[1][i]));
        return;
    }
    float ow[2] = {1.0f, 1.0f};
    if (cond) {
        const MrLevels lo = mr_levels(m, ls_value_precise(m, fl.o[0], fl.o[2]));
        ow[0] = lo.w[0];
        ow[1] = lo.w[1];
    }
    Frame f;
    ray_frame(m, fl.d[0], fl.d[1], fl.d[2], f);
    const float inv_s2 = 1.0f / 1.41421354f;
    value = 0.0f;
    g[0] = g[1] = g[2] = 0.0f;
#pragma unroll 1
    for (int j = 0; j < 2; ++j) {
        float v, dv, gcx, gcy;
        noise1d_level(m, fl, c.oct[0], cond, f, p, lv.s[j], lv.seed[j], ow[j], v, dv, gcx, gcy);
        value += lv.w[j] * v;
        float z0, z1;
        normal_draws(fl.normal_seed, j, z0, z1);
        const float x1 = z0 * inv_s2, y1 = z1 * inv_s2;
        float gl[3];
        if (t_segment == 0.0f) {
            gl[0] = x1 + gcx;
            gl[1] = y1 + gcy;
        } else if (!((m.flags & MF_RENEWAL_PLUS) && (m.flags & MF_CORR_XY))) {
            float z2, z3;
            normal_draws(fl.normal_seed, 2 + j, z2, z3);
            gl[0] = z2 * inv_s2 + gcx;
            gl[1] = z3 * inv_s2 + gcy;
        } else {
            float fac, cv, z2, z3;
            corr_moments(t_segment, fac, cv);
            normal_draws(fl.normal_seed, 2 + j, z2, z3);
            const float sq = sqrtf(cv);
            gl[0] = (z2 * sq + fac * 2.0f * x1) + gcx;
            gl[1] = (z3 * sq + fac * 2.0f * y1) + gcy;
        }
        gl[2] = dv;
        Frame fj;
        ray_frame_level(m, fl.d, lv.s[j], fj);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float gi = fj.t[i] * gl[0] + fj.b[i] * gl[1] + fj.n[i] * gl[2];
            g[i] += lv.w[j] * (m.l_inv[i] * gi / lv.s[j]);
        }
    }
}

// Noise of octave k at p with its world gradient (evaluateGradientNoise1D /
// evaluateNoise3D gradient).  cond: the octave's conditioning splats are active.
__device__ void noise1d_precise_vd(const DevMedium &m, float z, uint32_t seed, float ls, float &value, float &deriv);
__device__ float mean_plus_precise(const DevMedium &m, float an, float x, float y, float z, int &id);
template <bool GRAD, bool PRECISE>
__device__ int noise3d_gen(const DevMedium &m, const float p[3], const float d[3], const CondRec *c, const float o[3],
                           uint32_t seed, float &v, float g[3]);
__device__ void noise3d_precise_grad(const DevMedium &m, float px, float py, float pz, uint32_t seed, float &value,
                                     float g[3]);

// precise: the noise value and its derivative along the ray (1D) or gradient (3D)
// come from the precise evaluator (the conditioning at a flight's origin), else
// from the generic one
__device__ __forceinline__ void noise_gradient_oct(const DevMedium &m, const FlightIn &fl, const CondRec &c, bool cond,
                                   const float p[3], float t_segment, int oc, float &value, float g[3],
                                   bool precise = false)
{
    if (general_3d(m)) {
        // isotropic, nonstationary or multi-resolution 3D noise: the precise
        // evaluation (the conditioning and the end-point gradient take it)
        noise3d_gen<true, true>(m, p, fl.d, cond ? &c : nullptr, fl.o, fl.noise_seed, value, g);
        return;
    }
    if (!(m.flags & MF_ONE_D)) {
        if (precise) {
            noise3d_precise_grad(m, p[0], p[1], p[2], fl.noise_seed, value, g);
        } else {
            float v, gg[3];
            noise3d_generic<true>(m, p[0], p[1], p[2], fl.noise_seed, v, gg);
            value = v * m.inv_norm3d;
#pragma unroll
            for (int i = 0; i < 3; ++i) g[i] = gg[i] * m.inv_norm3d;
        }
        if (cond) {
            float cv, cg[3];
            cond3d(m, c, fl.o, p, cv, cg);
            value += cv;
#pragma unroll
            for (int i = 0; i < 3; ++i) g[i] += cg[i];
        }
        return;
    }
    if (m.flags & MF_MULTIRES) {
        noise_gradient_mr(m, fl, c, cond, p, t_segment, value, g, precise);
        return;
    }
    const CondOct &co = c.oct[oc];
    const float sc = oct_scale(m, oc);
    Frame f;
    ray_frame(m, fl.d[0], fl.d[1], fl.d[2], f);
    const float z = ray_coord_oct(m, f.n, p[0], p[1], p[2], sc);
    const float ls = precise ? ns_scale_precise(m, p[0], p[2]) : ns_scale(m, p[0], p[2]);
    float v, dv;
    if (precise) {
        noise1d_precise_vd(m, z, fl.noise_seed + oct_seed(m, oc), ls, v, dv);
    } else {
        noise1d_generic<true>(m, z, fl.noise_seed + oct_seed(m, oc), v, dv, ls);
        const float inrm = inv_norm_1d(m, ls);
        v *= inrm;
        dv *= inrm;
    }
    float gcx = 0.0f, gcy = 0.0f;
    if (cond) {
        const float oz = ray_coord_oct(m, f.n, fl.o[0], fl.o[1], fl.o[2], sc);
        const float a = splat_cov_1d(ls, ns_scale(m, fl.o[0], fl.o[2]));
        const Cov1D k = cov1d(z - oz, a);
        v += co.vs * k.k0 + (sc * co.gs[2]) * k.k1;
        dv += co.vs * k.k1 + (sc * co.gs[2]) * k.k2;
        if (m.flags & MF_CORR_XY) {
            gcx = (sc * co.gs[0]) * k.k3;
            gcy = (sc * co.gs[1]) * k.k3;
        }
    }
    value = v;
    const uint32_t nseed = oct_normal_seed(m, fl.normal_seed, oc);
    float gl[3];
    if ((m.flags & MF_TRANSVERSE) && m.ls_kind == 0u && m.n_oct == 1) {
        float m0, m1, var, z0, z1;
        transverse_moments(m, c, fl.o, p, f, cond, m0, m1, var);
        normal_draws(nseed, 0, z0, z1);
        const float s = sqrtf(var);
        gl[0] = m0 + s * z0;
        gl[1] = m1 + s * z1;
        gl[2] = dv;
    } else if (precise && t_segment == 0.0f) {
        // the birth gradient of the conditioning (grad_noise at the origin), operation
        // for operation: the double draws scaled by 1/sqrt(2) and 1/splat scale in
        // double, rounded to float, taken to world space through the frame and the
        // inverse length scales (evaluateGradientNoise1D, SparseConvolutionNoise.cpp:
        // 178-296; TangentFrame::toGlobal; transformGradLocaltoWorld)
        const float scx = splat_cov_1d(ls, ls);
        float gx0, gy0;
        normal_pair_scaled(nseed, 0, scx, gx0, gy0);
        const float gq[3] = {__fadd_rn(gx0, gcx), __fadd_rn(gy0, gcy), __fadd_rn(0.0f, dv)};
        const float sdiv = m.ls_kind ? m.ls_max : 1.0f;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float gi = __fadd_rn(__fadd_rn(__fmul_rn(f.t[i], gq[0]), __fmul_rn(f.b[i], gq[1])),
                                       __fmul_rn(f.n[i], gq[2]));
            float gw = __fdiv_rn(__fmul_rn(m.l_inv[i], gi), sdiv);
            if (sc != 1.0f) gw = __fdiv_rn(gw, sc);
            g[i] = gw;
        }
        return;
    } else {
        const float scx = splat_cov_1d(ls, ls);
        const float xs = 1.0f / scx;
        float z0, z1;
        normal_draws(nseed, 0, z0, z1);
        const float inv_s2 = 1.0f / 1.41421354f;
        const float x1 = z0 * inv_s2, y1 = z1 * inv_s2;
        if (t_segment == 0.0f) {
            gl[0] = x1 * xs + gcx;
            gl[1] = y1 * xs + gcy;
        } else if (!((m.flags & MF_RENEWAL_PLUS) && (m.flags & MF_CORR_XY))) {
            float z2, z3;
            normal_draws(nseed, 1, z2, z3);
            gl[0] = z2 * inv_s2 * xs + gcx;
            gl[1] = z3 * inv_s2 * xs + gcy;
        } else {
            float fac, cv, z2, z3;
            corr_moments(t_segment, fac, cv);
            normal_draws(nseed, 1, z2, z3);
            const float sq = sqrtf(cv);
            gl[0] = (z2 * sq + fac * 2.0f * x1) + gcx;
            gl[1] = (z3 * sq + fac * 2.0f * y1) + gcy;
        }
        gl[2] = dv;
    }
    const float div = (m.ls_kind ? m.ls_max : 1.0f) * sc;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float gi = f.t[i] * gl[0] + f.b[i] * gl[1] + f.n[i] * gl[2];
        g[i] = m.l_inv[i] * gi / div;
    }
}

__device__ __forceinline__ void noise_gradient(const DevMedium &m, const FlightIn &fl, const CondRec &c, bool cond,
                                               const float p[3], float t_segment, float &value, float g[3])
{
    noise_gradient_oct(m, fl, c, cond, p, t_segment, 0, value, g);
}

__device__ __forceinline__ void write_status(const FlightArgs &a, uint32_t i, float t, float value,
                                             float trans, uint32_t steps, uint32_t status)
{
    a.out[2 * i] = make_float4(t, value, 0.0f, 0.0f);
    a.out[2 * i + 1] = make_float4(0.0f, trans, __uint_as_float(steps), __uint_as_float(status));
}

// conditioning3D (SparseConvolutionNoise.cpp:498-574) for isotropic, nonstationary
// or multi-resolution 3D media; co.vs holds (target - mean) / amplitude - noise.
// The multi-resolution value scale is divided by w_low + w_high.  Renewal+: the
// world residual of the gradient; in isotropic ray space it is taken to the
// isotropic frame and times -2 (the inverse of -2 * 0.25 I), then divided by
// w_low / s_low + w_high / s_high or times sqr(ls(o) / ls_max); in world space it is
// divided by -2 * (l_inv^2 * 0.25) (the diagonal inverse written as the division),
// then divided by w_low / s_low^2 + w_high / s_high^2 or times sqr(ls(o)).
__device__ __forceinline__ void condition_3d_general(const DevMedium &m, const FlightIn &fl, const float g[3],
                                                     const float tg[3], const float mg[3], float amp, CondOct &co)
{
    const bool mr = (m.flags & MF_MULTIRES) != 0;
    MrLevels lv = {};
    if (mr) {
        lv = mr_levels(m, ls_value_precise(m, fl.o[0], fl.o[2]));
        co.vs = __fdiv_rn(co.vs, __fadd_rn(lv.w[0], lv.w[1]));
    }
    if (!(m.flags & MF_RENEWAL_PLUS)) return;
    float delta[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) delta[i] = __fsub_rn(__fdiv_rn(__fsub_rn(tg[i], mg[i]), amp), g[i]);
    if (m.flags & MF_ISO3D) {
        Frame f;
        ray_frame(m, fl.d[0], fl.d[1], fl.d[2], f);
        const float sw = m.ls_kind ? m.ls_max : 1.0f;
        float gi[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) gi[i] = __fmul_rn(__fmul_rn(m.l_aniso[i], delta[i]), sw);
        co.gs[0] = __fmul_rn(-2.0f, dot3_rn(f.t[0], f.t[1], f.t[2], gi[0], gi[1], gi[2]));
        co.gs[1] = __fmul_rn(-2.0f, dot3_rn(f.b[0], f.b[1], f.b[2], gi[0], gi[1], gi[2]));
        co.gs[2] = __fmul_rn(-2.0f, dot3_rn(f.n[0], f.n[1], f.n[2], gi[0], gi[1], gi[2]));
        if (mr) {
            const float dv = __fadd_rn(__fdiv_rn(lv.w[0], lv.s[0]), __fdiv_rn(lv.w[1], lv.s[1]));
#pragma unroll
            for (int i = 0; i < 3; ++i) co.gs[i] = __fdiv_rn(co.gs[i], dv);
        } else {
            const float a = ns_scale_precise(m, fl.o[0], fl.o[2]);
#pragma unroll
            for (int i = 0; i < 3; ++i) co.gs[i] = __fmul_rn(co.gs[i], __fmul_rn(a, a));
        }
        return;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float inv2 = __fmul_rn(m.l_inv[i], m.l_inv[i]);
        co.gs[i] = __fdiv_rn(delta[i], __fmul_rn(-2.0f, __fmul_rn(inv2, 0.25f)));
    }
    if (mr) {
        const float dv = __fadd_rn(__fdiv_rn(lv.w[0], __fmul_rn(lv.s[0], lv.s[0])),
                                   __fdiv_rn(lv.w[1], __fmul_rn(lv.s[1], lv.s[1])));
#pragma unroll
        for (int i = 0; i < 3; ++i) co.gs[i] = __fdiv_rn(co.gs[i], dv);
    } else {
        const float ls = m.ls_kind ? ls_value_precise(m, fl.o[0], fl.o[2]) : 1.0f;
#pragma unroll
        for (int i = 0; i < 3; ++i) co.gs[i] = __fmul_rn(co.gs[i], __fmul_rn(ls, ls));
    }
}

// One octave's coefficients from its target value and gradient at the origin
// (conditioning1D / conditioning3D, SparseConvolutionNoise.cpp:498-656).
__device__ __forceinline__ void condition_octave(const DevMedium &m, const FlightIn &fl, int k, float v,
                                                 const float g[3], float tv, const float tg[3], float mean,
                                                 const float mg[3], CondRec &c)
{
    const float amp = oct_sigma(m, k);
    if (amp == 0.0f) return;
    CondOct &co = c.oct[k];
    co.vs = (tv - mean) / amp - v;
    if (general_3d(m)) {
        condition_3d_general(m, fl, g, tg, mg, amp, co);
        return;
    }
    // the multi-resolution splats carry both levels' weights (conditioning1D, :602-633)
    const float mrn = (m.flags & MF_MULTIRES) ? mr_norm(mr_levels(m, ls_value_precise(m, fl.o[0], fl.o[2]))) : 1.0f;
    if (m.flags & MF_MULTIRES) co.vs = __fdiv_rn(co.vs, mrn);
    if (!(m.flags & MF_RENEWAL_PLUS)) return;
    float delta[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) delta[i] = (tg[i] - mg[i]) / amp - g[i];
    if (m.flags & MF_ONE_D) {
        Frame f;
        ray_frame(m, fl.d[0], fl.d[1], fl.d[2], f);
        // the octave's length multiplier enters where the splats are evaluated
        const float mul = m.ls_kind ? m.ls_max : 1.0f;
        float gi[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) gi[i] = (m.l_aniso[i] * delta[i]) * mul;
        const float ls = ns_scale_precise(m, fl.o[0], fl.o[2]);
        const float sc = splat_cov_1d(ls, ls);
        const float s2 = sc * sc;
        const float gx = dot3_rn(f.t[0], f.t[1], f.t[2], gi[0], gi[1], gi[2]);
        const float gy = dot3_rn(f.b[0], f.b[1], f.b[2], gi[0], gi[1], gi[2]);
        const float gz = dot3_rn(f.n[0], f.n[1], f.n[2], gi[0], gi[1], gi[2]);
        const bool xy = (m.flags & MF_CORR_XY) != 0;
        co.gs[0] = xy ? -2.0f * gx * s2 : 0.0f;
        co.gs[1] = xy ? -2.0f * gy * s2 : 0.0f;
        co.gs[2] = -2.0f * gz * s2;
        if (m.flags & MF_MULTIRES) {
#pragma unroll
            for (int i = 0; i < 3; ++i) co.gs[i] = __fdiv_rn(co.gs[i], mrn);
        }
        if (k == 0) {
#pragma unroll
            for (int i = 0; i < 3; ++i) c.tgn[i] = (tg[i] - mg[i]) / amp;
            c.has_obs = 1u;
        }
    } else {
        // delta / (-2 * (l_inv^2 * 0.25)), the inverse of sparseConvNoiseOneOverSecondDerivative's
        // diagonal applied as the division it is (GPFunctions.cpp:723-749)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float inv2 = __fmul_rn(m.l_inv[i], m.l_inv[i]);
            const float d2 = __fmul_rn(-2.0f, __fmul_rn(inv2, 0.25f));
            co.gs[i] = inv2 > 0.0f ? __fdiv_rn(delta[i], d2) : 0.0f;
        }
    }
}

// The mean gradient as the reference evaluates it in double and rounds to float
// (dmean_da): the torus (and its union with the plane) in FP64 with the
// operations unfused (once per conditioned flight); the other means as mean_grad.
__device__ __forceinline__ void mean_grad_precise(const DevMedium &m, float px, float py, float pz, float g[3])
{
    if (m.mean_kind != 4 && m.mean_kind != 5) {
        mean_grad(m, px, py, pz, g);
        return;
    }
    const float *q = m.mean_params;
    const double x = __dsub_rn((double)px, (double)q[0]), y = __dsub_rn((double)py, (double)q[1]),
                 z = __dsub_rn((double)pz, (double)q[2]);
    const double rxz = __dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(z, z)));
    const double s = __dsub_rn(rxz, (double)q[3]);
    const double len = __dsqrt_rn(__dadd_rn(__dmul_rn(s, s), __dmul_rn(y, y)));
    if (m.mean_kind == 5) {
        const double t = __dsub_rn(len, (double)q[4]);
        const double pl = __dsub_rn((double)py, (double)q[5]);
        if (pl < t) {
            g[0] = 0.0f; g[1] = 1.0f; g[2] = 0.0f;
            return;
        }
    }
    const double dr = __ddiv_rn(s, len), dy = __ddiv_rn(y, len);
    g[0] = rxz > 0.0 ? (float)__ddiv_rn(__dmul_rn(dr, x), rxz) : 0.0f;
    g[1] = (float)dy;
    g[2] = rxz > 0.0 ? (float)__ddiv_rn(__dmul_rn(dr, z), rxz) : 0.0f;
}

// Conditioning coefficients of a flight at its origin (conditioning,
// SparseConvolutionNoise.cpp:488-496).  With several octaves the residual of
// the value (and of the gradient under Renewal+) is shared in proportion to
// each octave's variance.
__device__ __forceinline__ CondRec make_condition(const DevMedium &m, const FlightIn &fl)
{
    CondRec c = {};
    const float *p = fl.o;
    int id;
    // the mean as the reference rounds it (float of the double mean) and the noise
    // from the precise evaluator, so that the conditioned field at the origin
    // leaves the residual the reference leaves
    const float mean = mean_plus_precise(m, 0.0f, p[0], p[1], p[2], id);
    float mg[3] = {0.0f, 0.0f, 0.0f};
    if (m.flags & MF_RENEWAL_PLUS) mean_grad_precise(m, p[0], p[1], p[2], mg);
    const CondRec none = {};
    const int n = (m.flags & MF_ONE_D) ? (int)m.n_oct : 1;
    if (n == 1) {
        float v, g[3];
        noise_gradient_oct(m, fl, none, false, p, 0.0f, 0, v, g, true);
        condition_octave(m, fl, 0, v, g, fl.prev_v, fl.prev_g, mean, mg, c);
        return c;
    }
    float v[4], g[4][3];
    for (int k = 0; k < n; ++k) noise_gradient_oct(m, fl, none, false, p, 0.0f, k, v[k], g[k], true);
    // the shares in the restatement's float operations, unfused
    float total = 0.0f;
    for (int k = 0; k < n; ++k) total = __fadd_rn(total, __fmul_rn(oct_sigma(m, k), oct_sigma(m, k)));
    float sum_v = 0.0f, sum_g[3] = {0.0f, 0.0f, 0.0f};
    for (int k = 0; k < n; ++k) {
        const float sk = oct_sigma(m, k);
        sum_v = __fadd_rn(sum_v, __fmul_rn(sk, v[k]));
#pragma unroll
        for (int i = 0; i < 3; ++i) sum_g[i] = __fadd_rn(sum_g[i], __fmul_rn(sk, g[k][i]));
    }
    const float resid = __fsub_rn(__fsub_rn(fl.prev_v, mean), sum_v);
    float resid_g[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) resid_g[i] = __fsub_rn(__fsub_rn(fl.prev_g[i], mg[i]), sum_g[i]);
    for (int k = 0; k < n; ++k) {
        const float sk = oct_sigma(m, k);
        const float share = __fdiv_rn(__fmul_rn(sk, sk), total);
        const float tv = __fadd_rn(__fadd_rn(mean, __fmul_rn(sk, v[k])), __fmul_rn(share, resid));
        float tg[3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
            tg[i] = __fadd_rn(__fadd_rn(mg[i], __fmul_rn(sk, g[k][i])), __fmul_rn(share, resid_g[i]));
        condition_octave(m, fl, k, v[k], g[k], tv, tg, mean, mg, c);
    }
    return c;
}

// ---------------------------------------------------------------------------
// k_prepare: conditioning coefficients at the origin of secondary flights.
// ---------------------------------------------------------------------------
// Per-flight set-up of the stationary cooperative fast pass, computed here with
// every lane busy instead of inside the march, where it runs for the few lanes
// that start a flight while the rest of the warp waits.  Four float4 per flight:
// {frame normal, origin coordinate}, {value scale, gradient scale, step, t0},
// {skip slope, skip jump, skip jump per step, -}, {seed, flags (1 valid, 2
// conditioned, 4 first scatter), -, -}.
enum : uint32_t { SF_VALID = 1u, SF_COND = 2u, SF_FIRST = 4u };

__device__ __forceinline__ void skip_params(const DevMedium &m, const float d[3], float sigma, bool cond, float vs,
                                            float gsz, float step, float &lip, float &j0, float &j1)
{
    // |df/dt| <= mean slope + sigma (noise + conditioning slopes) dz/dt with
    // dz/dt = |l_inv o d| (iso units per world unit); a truncated splat jumps by at
    // most skip_jump where the query crosses its support, and an iso interval of
    // D cells holds at most 2 N (D + 1) such crossings
    lip = -1.0f;
    j0 = j1 = 0.0f;
    if (m.skip_mean_lip < 0.0f) return;
    const float lx = m.l_inv[0] * d[0], ly = m.l_inv[1] * d[1], lz = m.l_inv[2] * d[2];
    const float dz = sqrtf(lx * lx + ly * ly + lz * lz) * 1.0001f;
    const float sg = fabsf(sigma);
    const float cslope = cond ? 0.42888194f * fabsf(vs) + 0.5f * fabsf(gsz) : 0.0f;
    lip = (m.skip_mean_lip + sg * (m.skip_noise_lip + cslope) * dz) * 1.01f;
    const float jn = sg * m.skip_jump * 2.0f * (float)m.n_imp * 1.01f;
    j0 = jn * 3.0f;
    j1 = jn * (step * dz / m.kr_iso);
}

__device__ __forceinline__ void prepare_one(const FlightArgs &a, uint32_t i)
{
    bool mok;
    const DevMedium &m = *medium_of(a, i, mok);
    const FlightIn fl = load_flight(a, i);
    const bool valid = mok && flight_valid(fl);
    const bool cond = valid && conditioned(m, fl);
    CondRec c = {};
    if (cond) {
        c = make_condition(m, fl);
        // only conditioned flights' records are read; a 1D single-octave medium's
        // readers take the first octave's coefficients and the transverse observation
        float4 *cr = reinterpret_cast<float4 *>(a.cond + i);
        const float4 *cs = reinterpret_cast<const float4 *>(&c);
        if ((m.flags & MF_ONE_D) && m.n_oct == 1 && !(m.flags & MF_MULTIRES)) {
            cr[0] = cs[0];
            cr[4] = cs[4];
        } else {
            a.cond[i] = c;
        }
    }
    if (!a.setup) return;
    float4 *s = a.setup + 4 * (size_t)i;
    if (!valid || !(m.flags & MF_ONE_D)) {
        s[3] = make_float4(0.0f, __uint_as_float(0u), 0.0f, 0.0f);
        return;
    }
    Frame f;
    ray_frame(m, fl.d[0], fl.d[1], fl.d[2], f);
    const float ozc = cond ? ray_coord_oct(m, f.n, fl.o[0], fl.o[1], fl.o[2], 1.0f) : 0.0f;
    const float vs = cond ? c.oct[0].vs : 0.0f, gsz = cond ? c.oct[0].gs[2] : 0.0f;
    float step = __fdiv_rn(__fsub_rn(fl.far_t, fl.near_t), (float)m.min_step);
    if (m.step_size < step) step = m.step_size;
    const float t0 = __fadd_rn(fl.near_t, __fmul_rn(step, fl.jitter));
    float lip, j0, j1;
    skip_params(m, fl.d, m.sigma, cond, vs, gsz, step, lip, j0, j1);
    const uint32_t flags = SF_VALID | (cond ? SF_COND : 0u) | ((fl.flags & GPIS_FLAG_FIRST_SCATTER) ? SF_FIRST : 0u);
    s[0] = make_float4(f.n[0], f.n[1], f.n[2], ozc);
    s[1] = make_float4(vs, gsz, step, t0);
    s[2] = make_float4(lip, j0, j1, 0.0f);
    s[3] = make_float4(__uint_as_float(fl.noise_seed), __uint_as_float(flags), 0.0f, 0.0f);
}

// MINB blocks of 128 per SM: 8 (at most 64 registers) for batches of 1D media, 1.14
// against 1.38 ms per bench step at 4 blocks and 128 registers (the precise
// conditioning's FP64 work needs the warps); 4 when 3D media are present, whose 27-cell
// evaluations spill heavily at 64 registers
template <int MINB>
__global__ void __launch_bounds__(128, MINB) k_prepare(FlightArgs a)
{
    const uint32_t n = live_n(a);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) prepare_one(a, i);
}

// ---------------------------------------------------------------------------
// Field evaluators used by the march.
// ---------------------------------------------------------------------------
// Registers of one lane's flight that the evaluators read.
struct LaneField {
    const DevMedium *m;
    float n[3];             // ray-space frame normal (1D)
    float li[3];
    float kr, kexp, inv_norm, sigma;
    uint32_t seed;
    float vs, gsz, ozc;     // 1D conditioning
    bool cond;
    CondRec c3;             // 3D conditioning
    float o[3];
    uint32_t mean_kind;     // mean function in registers (all kinds but the grid)
    float mq[6];
    uint32_t n_imp;         // impulses per cell
    bool ns;                // nonstationary length scale
    float ls_o;             // kernel scale at the origin (conditioning)
    float mr_ow[2];         // multi-resolution: the origin's weights of the low and high level
    float d[3];             // the flight's direction (isotropic-space 3D noise)
};

// Safe contents for a lane without a flight (collective evaluators run every lane).
__device__ __forceinline__ void lane_field_idle(LaneField &L, const DevMedium *m0)
{
    L.m = m0;
    L.n[0] = 0.0f; L.n[1] = 0.0f; L.n[2] = 1.0f;
    L.li[0] = L.li[1] = L.li[2] = 1.0f;
    L.kr = 1.0f; L.kexp = -1.0f; L.inv_norm = 1.0f; L.sigma = 0.0f;
    L.seed = 0u;
    L.vs = L.gsz = L.ozc = 0.0f;
    L.cond = false;
    L.c3 = CondRec{};
    L.o[0] = L.o[1] = L.o[2] = 0.0f;
    L.mean_kind = 1u;
#pragma unroll
    for (int k = 0; k < 6; ++k) L.mq[k] = 0.0f;
    L.n_imp = 0u;
    L.ns = false;
    L.ls_o = 1.0f;
    L.mr_ow[0] = L.mr_ow[1] = 1.0f;
    L.d[0] = 0.0f; L.d[1] = 0.0f; L.d[2] = 1.0f;
}

// A lane's registers for flight fl of medium m; cond points at its conditioning record.
// GENERAL = false: a stationary single-octave flight (the fast evaluator's case).
template <bool GENERAL = true>
__device__ __forceinline__ void lane_field_setup(LaneField &L, const DevMedium &m, const FlightIn &fl,
                                                 const CondRec *cond)
{
    L.m = &m;
#pragma unroll
    for (int k = 0; k < 3; ++k) { L.o[k] = fl.o[k]; L.li[k] = m.l_inv[k]; }
    L.seed = fl.noise_seed;
    L.sigma = m.sigma;
    L.cond = conditioned(m, fl);
    L.vs = L.gsz = L.ozc = 0.0f;
    L.ns = m.ls_kind != 0u;
    L.ls_o = 1.0f;
    L.mr_ow[0] = L.mr_ow[1] = 1.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) L.d[k] = fl.d[k];
    if (GENERAL && (m.flags & MF_MULTIRES) && L.cond) {
        const MrLevels lo = mr_levels(m, ls_value_precise(m, fl.o[0], fl.o[2]));
        L.mr_ow[0] = lo.w[0];
        L.mr_ow[1] = lo.w[1];
    }
    L.mean_kind = m.mean_kind;
#pragma unroll
    for (int k = 0; k < 6; ++k) L.mq[k] = m.mean_params[k];
    L.n_imp = m.n_imp;
    if (m.flags & MF_ONE_D) {
        Frame f;
        ray_frame(m, fl.d[0], fl.d[1], fl.d[2], f);
        L.n[0] = f.n[0]; L.n[1] = f.n[1]; L.n[2] = f.n[2];
        L.kr = m.kr_iso;
        L.kexp = m.kexp1d;
        L.inv_norm = m.inv_norm1d;
        if (L.cond) {
            if (GENERAL) L.ls_o = ns_scale_precise(m, L.o[0], L.o[2]);
            if (!GENERAL || m.n_oct == 1) {
                const CondOct c = cond->oct[0];
                L.vs = c.vs;
                L.gsz = c.gs[2];
                L.ozc = ray_coord_oct(m, L.n, L.o[0], L.o[1], L.o[2], 1.0f);
            } else {
                L.c3 = *cond;
            }
        }
    } else if (GENERAL && L.cond) {
        L.c3 = *cond;
    }
}

// mean_value with the parameters held in registers; the grid reads the medium table.
__device__ __forceinline__ float lane_mean(const LaneField &L, float x, float y, float z, int &id)
{
    id = 0;
    switch (L.mean_kind) {
    case 0: {
        const float dx = x - L.mq[0], dy = y - L.mq[1], dz = z - L.mq[2];
        return sqrtf(dx * dx + dy * dy + dz * dz) - L.mq[3];
    }
    case 1:
        return L.mq[0];
    case 3:
        return L.mq[0] * x + L.mq[1] * y + L.mq[2] * z - L.mq[3];
    case 4:
        return torus_sdf(L.mq, x, y, z);
    case 5: {
        const float t = torus_sdf(L.mq, x, y, z);
        const float pl = y - L.mq[5];
        if (pl < t) { id = 1; return pl; }
        return t;
    }
    default:
        return mean_value(*L.m, x, y, z, id);
    }
}

// Conditioning coefficients of octave k of a 1D lane: value scale, gradient
// scale along the ray (times the octave's length multiplier) and the origin's
// ray coordinate.  Single-octave flights keep them in registers.
__device__ __forceinline__ void lane_cond_1d(const LaneField &L, int k, float sc, float &vs, float &gz, float &oz)
{
    if (L.m->n_oct == 1) {
        vs = L.vs;
        gz = L.gsz;
        oz = L.ozc;
        return;
    }
    const CondOct &co = L.c3.oct[k];
    vs = co.vs;
    gz = __fmul_rn(sc, co.gs[2]);
    oz = ray_coord_oct(*L.m, L.n, L.o[0], L.o[1], L.o[2], sc);
}

// ---- precise evaluation ------------------------------------------------------
// The reference's float formulation op for op: every splat as
// exp(-((kr*t - kr*t_i)^2 / 2)) (GPFunctions.cpp:845-848) with the exp correctly
// rounded (cr_expf, as the oracle evaluates the reference's float exp), cell sums in impulse
// order, cells summed in order, division by the rounded normalisation, the
// conditioning splats of evaluateNoise1DNormalized, and the mean in double
// (emulated in float-float for the sphere) added as
// float(double(amplitude * noise) + mean) (SparseConvolutionNoise.cpp:114-130).
// The march uses it wherever a sign decision is close: the crossing step, the
// step before it and every refinement point.

// x / den rounded once; den is 2 ls^2, exactly 2 for a stationary medium, where the
// product with 0.5 is the same correctly rounded value without the division
__device__ __forceinline__ float div_den(float x, float den)
{
    return den == 2.0f ? __fmul_rn(x, 0.5f) : __fdiv_rn(x, den);
}

__device__ float noise1d_precise(const DevMedium &m, float z, uint32_t seed, float ls = 1.0f)
{
    const float kr = m.kr_iso;
    const float tg = __fdiv_rn(z, kr);
    const float fl = floorf(tg);
    const float frac = __fsub_rn(tg, fl);
    const int ci = (int)fl;
    const float den = __fmul_rn(2.0f, __fmul_rn(ls, ls));
    float sv = 0.0f;
    for (int dx = -1; dx <= 1; ++dx) {
        const float tl = __fsub_rn(frac, (float)dx);
        const float a = __fmul_rn(kr, tl);
        const uint32_t s = xxhash2((uint32_t)(ci + dx), seed) + 1u;
        float cv = 0.0f;
        for (uint32_t k = 0; k < m.n_imp; ++k) {
            const float ti = unit_float(pcg_draw(c_jump[2 + 2 * k], s));
            const uint32_t wr = pcg_draw(c_jump[3 + 2 * k], s);
            const float tp = __fsub_rn(tl, ti);
            if (fabsf(tp) < 1.0f) {
                const float ab = __fsub_rn(a, __fmul_rn(kr, ti));
                const float e = cr_expf(-div_den(__fmul_rn(ab, ab), den));
                cv = __fadd_rn(cv, (wr >> 31) ? e : -e);
            }
        }
        sv = __fadd_rn(sv, cv);
    }
    if (ls == 1.0f) return __fdiv_rn(sv, m.norm1d);
    // sparseConvNoiseVariance1D: impulseDensity/kernelRadius * sqrt(pi) * localScale
    const float var = (float)((double)m.var1d_c * (1.7724538509055159 * (double)ls));
    return __fdiv_rn(sv, __fsqrt_rn(var));
}

// a * b / c rounded once to float: the product exact as a float pair, the quotient
// carried with its remainder (the reference evaluates such terms in double and
// rounds the result to float; the two agree but where the exact value lies within
// about 2^-46 of a rounding boundary)
__device__ __forceinline__ float rn_mul_div(float a, float b, float c)
{
    const float ph = __fmul_rn(a, b);
    const float pl = __fmaf_rn(a, b, -ph);
    const float qh = __fdiv_rn(ph, c);
    const float rem = __fadd_rn(__fmaf_rn(-qh, c, ph), pl);
    return __fadd_rn(qh, __fdiv_rn(rem, c));
}

// noise1d_precise with the derivative d/dz of the normalized noise: per splat
// (float)(-2.0 * ab / den * f) as the reference's splattingKernel1D1stGrad
// evaluates it in double (GPFunctions.cpp:859-863), summed as the value.  The
// conditioning at a flight's origin takes both from here.
__device__ void noise1d_precise_vd(const DevMedium &m, float z, uint32_t seed, float ls, float &value, float &deriv)
{
    const float kr = m.kr_iso;
    const float tg = __fdiv_rn(z, kr);
    const float fl = floorf(tg);
    const float frac = __fsub_rn(tg, fl);
    const int ci = (int)fl;
    const float den = __fmul_rn(2.0f, __fmul_rn(ls, ls));
    float sv = 0.0f, sg = 0.0f;
    for (int dx = -1; dx <= 1; ++dx) {
        const float tl = __fsub_rn(frac, (float)dx);
        const float a = __fmul_rn(kr, tl);
        const uint32_t s = xxhash2((uint32_t)(ci + dx), seed) + 1u;
        float cv = 0.0f, cg = 0.0f;
        for (uint32_t k = 0; k < m.n_imp; ++k) {
            const float ti = unit_float(pcg_draw(c_jump[2 + 2 * k], s));
            const uint32_t wr = pcg_draw(c_jump[3 + 2 * k], s);
            const float tp = __fsub_rn(tl, ti);
            if (fabsf(tp) < 1.0f) {
                const float ab = __fsub_rn(a, __fmul_rn(kr, ti));
                const float e = cr_expf(-div_den(__fmul_rn(ab, ab), den));
                const float gr = rn_mul_div(__fmul_rn(-2.0f, ab), e, den);
                cv = __fadd_rn(cv, (wr >> 31) ? e : -e);
                cg = __fadd_rn(cg, (wr >> 31) ? gr : -gr);
            }
        }
        sv = __fadd_rn(sv, cv);
        sg = __fadd_rn(sg, cg);
    }
    float nrm = m.norm1d;
    if (ls != 1.0f) nrm = __fsqrt_rn((float)((double)m.var1d_c * (1.7724538509055159 * (double)ls)));
    value = __fdiv_rn(sv, nrm);
    deriv = __fdiv_rn(sg, nrm);
}

// noise3d_precise with the world gradient of the normalized noise: per splat
// (-2 (ab_c M_c)) f as the reference's splattingKernel3D1stGrad (GPFunctions.cpp:
// 814-821), summed per cell and over the cells in the value's order.
__device__ void noise3d_precise_grad(const DevMedium &m, float px, float py, float pz, uint32_t seed, float &value,
                                     float g[3])
{
    const float kr = m.kr_world;
    const float p[3] = {px, py, pz};
    float fr[3];
    int ijk[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float q = __fdiv_rn(p[i], kr);
        const float fl = floorf(q);
        fr[i] = __fsub_rn(q, fl);
        ijk[i] = (int)fl;
    }
    const bool xfirst = (m.flags & MF_XYZ_ORDER) != 0;
    float sv = 0.0f, s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                const float t0 = __fsub_rn(fr[0], (float)dx), t1 = __fsub_rn(fr[1], (float)dy),
                            t2 = __fsub_rn(fr[2], (float)dz);
                const uint32_t s = xxhash4((uint32_t)(ijk[2] + dz), (uint32_t)(ijk[1] + dy),
                                           (uint32_t)(ijk[0] + dx), seed) + 1u;
                float cv = 0.0f, c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
                for (uint32_t k = 0; k < m.n_imp; ++k) {
                    const int b = 2 + 4 * (int)k;
                    const float r0 = unit_float(pcg_draw(c_jump[b], s));
                    const float r1 = unit_float(pcg_draw(c_jump[b + 1], s));
                    const float r2 = unit_float(pcg_draw(c_jump[b + 2], s));
                    const uint32_t wr = pcg_draw(c_jump[b + 3], s);
                    const float ix = xfirst ? r0 : r2, iy = r1, iz = xfirst ? r2 : r0;
                    const float a0 = __fsub_rn(t0, ix), a1 = __fsub_rn(t1, iy), a2 = __fsub_rn(t2, iz);
                    const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(a0, a0), __fmul_rn(a1, a1)), __fmul_rn(a2, a2));
                    if (l2 < 1.0f) {
                        const float b0 = __fsub_rn(__fmul_rn(kr, t0), __fmul_rn(kr, ix));
                        const float b1 = __fsub_rn(__fmul_rn(kr, t1), __fmul_rn(kr, iy));
                        const float b2 = __fsub_rn(__fmul_rn(kr, t2), __fmul_rn(kr, iz));
                        float q = __fmul_rn(__fmul_rn(b0, m.m3[0]), b0);
                        q = __fadd_rn(q, __fmul_rn(__fmul_rn(b1, m.m3[1]), b1));
                        q = __fadd_rn(q, __fmul_rn(__fmul_rn(b2, m.m3[2]), b2));
                        const float e = cr_expf(-q);
                        const float g0 = __fmul_rn(__fmul_rn(-2.0f, __fmul_rn(b0, m.m3[0])), e);
                        const float g1 = __fmul_rn(__fmul_rn(-2.0f, __fmul_rn(b1, m.m3[1])), e);
                        const float g2 = __fmul_rn(__fmul_rn(-2.0f, __fmul_rn(b2, m.m3[2])), e);
                        const bool pos = (wr >> 31) != 0;
                        cv = __fadd_rn(cv, pos ? e : -e);
                        c0 = __fadd_rn(c0, pos ? g0 : -g0);
                        c1 = __fadd_rn(c1, pos ? g1 : -g1);
                        c2 = __fadd_rn(c2, pos ? g2 : -g2);
                    }
                }
                sv = __fadd_rn(sv, cv);
                s0 = __fadd_rn(s0, c0);
                s1 = __fadd_rn(s1, c1);
                s2 = __fadd_rn(s2, c2);
            }
    value = __fdiv_rn(sv, m.norm3d);
    g[0] = __fdiv_rn(s0, m.norm3d);
    g[1] = __fdiv_rn(s1, m.norm3d);
    g[2] = __fdiv_rn(s2, m.norm3d);
}

// ---- 3D noise outside the stationary world form --------------------------------
// Isotropic ray space (isotropic_3D_sampling: evaluateNoise3DIsotropicRayNormalized,
// SparseConvolutionNoise.cpp:348-377), the brute-force nonstationary length scale
// and the multi-resolution grid (evaluateNoise3D, :142-165), world or isotropic.
// One evaluation runs per level: the point in the level's space, the lattice of
// 27 cells with the level's kernel radius and inverse covariance, the
// normalisation, the gradient back to world space and the conditioning splats.
// PRECISE repeats the reference's float operations (cr_expf, unfused); the march's
// decisions near zero, the conditioning and the end-point gradient take it.

// One level: kernelRadius, kernelSpatialScale and its noise-seed offset.
struct Lv3 {
    float kr, ks;
    uint32_t seed_add;
};

// The levels at p with their weights (one, or the two of the multi-resolution
// grid around ls(p)).  kernelRadius: the isotropic localScale, or in world space
// (kernelScale * localScale) * the largest anisotropic length, localScale being
// the level's scale or, by brute force, the largest lateral scale
// (GPFunctions.cpp:711-719, 1253-1258).
__device__ __forceinline__ int levels3(const DevMedium &m, float px, float pz, bool precise, Lv3 lv[2], float w[2])
{
    const bool iso = (m.flags & MF_ISO3D) != 0;
    const float mtx = fmaxf(fmaxf(m.l_aniso[0], m.l_aniso[1]), m.l_aniso[2]);
    if (m.flags & MF_MULTIRES) {
        const MrLevels L = mr_levels(m, precise ? ls_value_precise(m, px, pz) : ls_value(m, px, pz));
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            lv[j].ks = L.s[j];
            lv[j].seed_add = L.seed[j];
            lv[j].kr = iso ? m.kr_iso : __fmul_rn(__fmul_rn(m.kr_iso, L.s[j]), mtx);
            w[j] = L.w[j];
        }
        return 2;
    }
    const bool ns = m.ls_kind != 0u;
    lv[0].kr = iso ? m.kr_iso : __fmul_rn(__fmul_rn(m.kr_iso, ns ? m.ls_max : 1.0f), mtx);
    lv[0].ks = (!iso && ns) ? m.ls_max : 1.0f;
    lv[0].seed_add = (!iso && ns) ? (uint32_t)m.ns3_seed : 0u;
    w[0] = 1.0f;
    w[1] = 0.0f;
    return 1;
}

// getInvCovMtx's diagonal (GPFunctions.cpp:784-812): world space (the inverse
// squared length scales over sqr(globalScale)) or isotropic space (identity), times
// 0.5 for a covariance splat, over sqr(localScale), times 0.5.
__device__ __forceinline__ void inv_cov3(const DevMedium &m, bool iso, bool is_cov, float a, float gs, float M[3])
{
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float v = iso ? 1.0f : __fmul_rn(m.l_inv[i], m.l_inv[i]);
        if (!iso && gs != 1.0f) v = __fdiv_rn(v, __fmul_rn(gs, gs));
        if (is_cov) v = __fmul_rn(v, 0.5f);
        v = __fdiv_rn(v, __fmul_rn(a, a));
        M[i] = __fmul_rn(v, 0.5f);
    }
}

// noise3D + cell3D (SparseConvolutionNoise.cpp:419-452) at the point q of a level's
// space: the raw sum and its gradient (q units).
template <bool GRAD, bool PRECISE>
__device__ void lattice3(const DevMedium &m, const float q[3], float kr, const float M[3], uint32_t seed, float &v,
                         float g[3])
{
    float fr[3];
    int ijk[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float t = __fdiv_rn(q[i], kr);
        const float fl = floorf(t);
        fr[i] = __fsub_rn(t, fl);
        ijk[i] = (int)fl;
    }
    const bool xfirst = (m.flags & MF_XYZ_ORDER) != 0;
    float sv = 0.0f, s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                const float t0 = __fsub_rn(fr[0], (float)dx), t1 = __fsub_rn(fr[1], (float)dy),
                            t2 = __fsub_rn(fr[2], (float)dz);
                const uint32_t s = xxhash4((uint32_t)(ijk[2] + dz), (uint32_t)(ijk[1] + dy),
                                           (uint32_t)(ijk[0] + dx), seed) + 1u;
                float cv = 0.0f, c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
                for (uint32_t k = 0; k < m.n_imp; ++k) {
                    const int b = 2 + 4 * (int)k;
                    const float r0 = unit_float(pcg_draw(c_jump[b], s));
                    const float r1 = unit_float(pcg_draw(c_jump[b + 1], s));
                    const float r2 = unit_float(pcg_draw(c_jump[b + 2], s));
                    const uint32_t wr = pcg_draw(c_jump[b + 3], s);
                    const float ix = xfirst ? r0 : r2, iy = r1, iz = xfirst ? r2 : r0;
                    const float a0 = __fsub_rn(t0, ix), a1 = __fsub_rn(t1, iy), a2 = __fsub_rn(t2, iz);
                    const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(a0, a0), __fmul_rn(a1, a1)), __fmul_rn(a2, a2));
                    if (l2 < 1.0f) {
                        const bool pos = (wr >> 31) != 0;
                        if (PRECISE) {
                            const float b0 = __fsub_rn(__fmul_rn(kr, t0), __fmul_rn(kr, ix));
                            const float b1 = __fsub_rn(__fmul_rn(kr, t1), __fmul_rn(kr, iy));
                            const float b2 = __fsub_rn(__fmul_rn(kr, t2), __fmul_rn(kr, iz));
                            float qq = __fmul_rn(__fmul_rn(b0, M[0]), b0);
                            qq = __fadd_rn(qq, __fmul_rn(__fmul_rn(b1, M[1]), b1));
                            qq = __fadd_rn(qq, __fmul_rn(__fmul_rn(b2, M[2]), b2));
                            const float e = cr_expf(-qq);
                            cv = __fadd_rn(cv, pos ? e : -e);
                            if (GRAD) {
                                const float g0 = __fmul_rn(__fmul_rn(-2.0f, __fmul_rn(b0, M[0])), e);
                                const float g1 = __fmul_rn(__fmul_rn(-2.0f, __fmul_rn(b1, M[1])), e);
                                const float g2 = __fmul_rn(__fmul_rn(-2.0f, __fmul_rn(b2, M[2])), e);
                                c0 = __fadd_rn(c0, pos ? g0 : -g0);
                                c1 = __fadd_rn(c1, pos ? g1 : -g1);
                                c2 = __fadd_rn(c2, pos ? g2 : -g2);
                            }
                        } else {
                            const float b0 = kr * a0, b1 = kr * a1, b2 = kr * a2;
                            const float e = ex2_approx(-LOG2E * (M[0] * b0 * b0 + M[1] * b1 * b1 + M[2] * b2 * b2));
                            const float w = pos ? 1.0f : -1.0f;
                            cv += w * e;
                            if (GRAD) {
                                c0 += w * (-2.0f * (b0 * M[0]) * e);
                                c1 += w * (-2.0f * (b1 * M[1]) * e);
                                c2 += w * (-2.0f * (b2 * M[2]) * e);
                            }
                        }
                    }
                }
                if (PRECISE) {
                    sv = __fadd_rn(sv, cv);
                    if (GRAD) { s0 = __fadd_rn(s0, c0); s1 = __fadd_rn(s1, c1); s2 = __fadd_rn(s2, c2); }
                } else {
                    sv += cv;
                    if (GRAD) { s0 += c0; s1 += c1; s2 += c2; }
                }
            }
    v = sv;
    if (GRAD) { g[0] = s0; g[1] = s1; g[2] = s2; }
}

// sqrt(sparseConvNoiseVariance3D) as the reference rounds it (GPFunctions.cpp:751-764,
// 1260-1263): impulseDensity / kr^3 in float, the determinant and the scales' cubes
// in double, pi^1.5 = pow(M_PI, 1.5).
__device__ __forceinline__ float norm3(const DevMedium &m, bool iso, float kr, float gs, float a)
{
    const float ud = __fdiv_rn(m.imp_density, __fmul_rn(__fmul_rn(kr, kr), kr));
    double det = 1.0;
    if (!iso) {
        const float detf = __fmul_rn(__fmul_rn(m.l_aniso[0], m.l_aniso[1]), m.l_aniso[2]);
        det = __dmul_rn((double)detf, __dmul_rn(__dmul_rn((double)gs, (double)gs), (double)gs));
    }
    det = __dmul_rn(det, __dmul_rn(__dmul_rn((double)a, (double)a), (double)a));
    const double pi15 = 0x1.645f7c63f2c6bp+2;
    return __fsqrt_rn((float)__dmul_rn((double)ud, __dmul_rn(pi15, det)));
}

// One level: the normalized noise value (and world gradient) at p with the
// conditioning splats of c (null: none) about the flight's origin o.
template <bool GRAD, bool PRECISE>
__device__ __noinline__ void noise3d_level_gen(const DevMedium &m, const float p[3], const float d[3], const CondRec *c,
                                  const float o[3], const Lv3 &lv, uint32_t seed, float &v, float g[3])
{
    const bool iso = (m.flags & MF_ISO3D) != 0;
    const float a = m.ls_kind ? (PRECISE ? ns_scale_precise(m, p[0], p[2]) : ns_scale(m, p[0], p[2])) : 1.0f;
    const float gs = iso ? 1.0f : lv.ks;
    // transformPosDirWorldtoLocal / transformGradLocaltoWorld scale: the largest
    // lateral scale by brute force, else the level's scale
    const float S = m.ls_kind ? m.ls_max : lv.ks;
    float q[3];
    Frame f;
    if (iso) {
        ray_frame(m, d[0], d[1], d[2], f);
        float pi[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) pi[i] = __fdiv_rn(__fmul_rn(m.l_inv[i], p[i]), S);
        q[0] = dot3_rn(f.t[0], f.t[1], f.t[2], pi[0], pi[1], pi[2]);
        q[1] = dot3_rn(f.b[0], f.b[1], f.b[2], pi[0], pi[1], pi[2]);
        q[2] = dot3_rn(f.n[0], f.n[1], f.n[2], pi[0], pi[1], pi[2]);
    } else {
        q[0] = p[0]; q[1] = p[1]; q[2] = p[2];
    }
    float M[3];
    inv_cov3(m, iso, false, a, gs, M);
    float sv, sg[3];
    lattice3<GRAD, PRECISE>(m, q, lv.kr, M, seed + lv.seed_add, sv, sg);
    const float nf = norm3(m, iso, lv.kr, gs, a);
    v = __fdiv_rn(sv, nf);
    // a vector of the level's space to world space (TangentFrame::toGlobal, then
    // transformGradLocaltoWorld)
    auto to_world = [&](const float x[3], float y[3]) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float gi = __fadd_rn(__fadd_rn(__fmul_rn(f.t[i], x[0]), __fmul_rn(f.b[i], x[1])),
                                       __fmul_rn(f.n[i], x[2]));
            y[i] = __fdiv_rn(__fmul_rn(m.l_inv[i], gi), S);
        }
    };
    if (GRAD) {
        float gw[3] = {sg[0], sg[1], sg[2]};
        if (iso) to_world(sg, gw);
#pragma unroll
        for (int i = 0; i < 3; ++i) g[i] = __fdiv_rn(gw[i], nf);
    }
    if (!c) return;
    float Mc[3];
    inv_cov3(m, iso, true, a, gs, Mc);
    float ab[3];
    if (iso) {
        float oi[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) oi[i] = __fdiv_rn(__fmul_rn(m.l_inv[i], o[i]), S);
        ab[0] = __fsub_rn(q[0], dot3_rn(f.t[0], f.t[1], f.t[2], oi[0], oi[1], oi[2]));
        ab[1] = __fsub_rn(q[1], dot3_rn(f.b[0], f.b[1], f.b[2], oi[0], oi[1], oi[2]));
        ab[2] = __fsub_rn(q[2], dot3_rn(f.n[0], f.n[1], f.n[2], oi[0], oi[1], oi[2]));
    } else {
#pragma unroll
        for (int i = 0; i < 3; ++i) ab[i] = __fsub_rn(p[i], o[i]);
    }
    float absq = __fmul_rn(__fmul_rn(ab[0], Mc[0]), ab[0]);
    absq = __fadd_rn(absq, __fmul_rn(__fmul_rn(ab[1], Mc[1]), ab[1]));
    absq = __fadd_rn(absq, __fmul_rn(__fmul_rn(ab[2], Mc[2]), ab[2]));
    const float fk = PRECISE ? cr_expf(-absq) : ex2_approx(-LOG2E * absq);
    const CondOct &co = c->oct[0];
    float dp[3], g1[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        dp[i] = __fmul_rn(-2.0f, __fmul_rn(ab[i], Mc[i]));
        g1[i] = __fmul_rn(dp[i], fk);
    }
    float gv = 0.0f;
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) gv = __fadd_rn(gv, __fmul_rn(g1[cc], co.gs[cc]));
    v = __fadd_rn(v, __fadd_rn(__fmul_rn(fk, co.vs), gv));
    if (GRAD) {
        float dg[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float gg = 0.0f;
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                const float h = __fsub_rn(__fmul_rn(dp[cc], dp[j]), cc == j ? __fmul_rn(2.0f, Mc[cc]) : 0.0f);
                gg = __fadd_rn(gg, __fmul_rn(__fmul_rn(h, fk), co.gs[cc]));
            }
            dg[j] = __fadd_rn(__fmul_rn(g1[j], co.vs), gg);
        }
        float dw[3] = {dg[0], dg[1], dg[2]};
        if (iso) to_world(dg, dw);
#pragma unroll
        for (int j = 0; j < 3; ++j) g[j] = __fadd_rn(g[j], dw[j]);
    }
}

// The normalized 3D noise (and world gradient) at p: one level or the blend of two.
// Returns the cells regenerated.
template <bool GRAD, bool PRECISE>
__device__ int noise3d_gen(const DevMedium &m, const float p[3], const float d[3], const CondRec *c, const float o[3],
                           uint32_t seed, float &v, float g[3])
{
    Lv3 lv[2];
    float w[2];
    const int n = levels3(m, p[0], p[2], PRECISE, lv, w);
    if (n == 1) {
        noise3d_level_gen<GRAD, PRECISE>(m, p, d, c, o, lv[0], seed, v, g);
        return 27;
    }
    float v0, v1, g0[3] = {0.0f, 0.0f, 0.0f}, g1[3] = {0.0f, 0.0f, 0.0f};
    noise3d_level_gen<GRAD, PRECISE>(m, p, d, c, o, lv[0], seed, v0, g0);
    noise3d_level_gen<GRAD, PRECISE>(m, p, d, c, o, lv[1], seed, v1, g1);
    v = __fadd_rn(__fmul_rn(w[0], v0), __fmul_rn(w[1], v1));
    if (GRAD) {
#pragma unroll
        for (int i = 0; i < 3; ++i) g[i] = __fadd_rn(__fmul_rn(w[0], g0[i]), __fmul_rn(w[1], g1[i]));
    }
    return 54;
}

__device__ float noise3d_precise(const DevMedium &m, float px, float py, float pz, uint32_t seed)
{
    const float kr = m.kr_world;
    const float p[3] = {px, py, pz};
    float fr[3];
    int ijk[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float q = __fdiv_rn(p[i], kr);
        const float fl = floorf(q);
        fr[i] = __fsub_rn(q, fl);
        ijk[i] = (int)fl;
    }
    const bool xfirst = (m.flags & MF_XYZ_ORDER) != 0;
    float sv = 0.0f;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                const float t0 = __fsub_rn(fr[0], (float)dx), t1 = __fsub_rn(fr[1], (float)dy),
                            t2 = __fsub_rn(fr[2], (float)dz);
                const uint32_t s = xxhash4((uint32_t)(ijk[2] + dz), (uint32_t)(ijk[1] + dy),
                                           (uint32_t)(ijk[0] + dx), seed) + 1u;
                float cv = 0.0f;
                for (uint32_t k = 0; k < m.n_imp; ++k) {
                    const int b = 2 + 4 * (int)k;
                    const float r0 = unit_float(pcg_draw(c_jump[b], s));
                    const float r1 = unit_float(pcg_draw(c_jump[b + 1], s));
                    const float r2 = unit_float(pcg_draw(c_jump[b + 2], s));
                    const uint32_t wr = pcg_draw(c_jump[b + 3], s);
                    const float ix = xfirst ? r0 : r2, iy = r1, iz = xfirst ? r2 : r0;
                    const float a0 = __fsub_rn(t0, ix), a1 = __fsub_rn(t1, iy), a2 = __fsub_rn(t2, iz);
                    const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(a0, a0), __fmul_rn(a1, a1)), __fmul_rn(a2, a2));
                    if (l2 < 1.0f) {
                        const float b0 = __fsub_rn(__fmul_rn(kr, t0), __fmul_rn(kr, ix));
                        const float b1 = __fsub_rn(__fmul_rn(kr, t1), __fmul_rn(kr, iy));
                        const float b2 = __fsub_rn(__fmul_rn(kr, t2), __fmul_rn(kr, iz));
                        float q = __fmul_rn(__fmul_rn(b0, m.m3[0]), b0);
                        q = __fadd_rn(q, __fmul_rn(__fmul_rn(b1, m.m3[1]), b1));
                        q = __fadd_rn(q, __fmul_rn(__fmul_rn(b2, m.m3[2]), b2));
                        const float e = cr_expf(-q);
                        cv = __fadd_rn(cv, (wr >> 31) ? e : -e);
                    }
                }
                sv = __fadd_rn(sv, cv);
            }
    return __fdiv_rn(sv, m.norm3d);
}

// float(double(an) + mean(p)) with the mean evaluated as the reference does in
// double; the sphere's distance is emulated in float-float.
__device__ float mean_plus_precise(const DevMedium &m, float an, float x, float y, float z, int &id)
{
    const float *q = m.mean_params;
    id = 0;
    if (m.mean_kind == 0) {
        float e0, e1, e2;
        const float h0 = two_sum(x, -q[0], e0), h1 = two_sum(y, -q[1], e1), h2 = two_sum(z, -q[2], e2);
        FF s = ff_add(ff_add(ff_sq({h0, e0}), ff_sq({h1, e1})), ff_sq({h2, e2}));
        FF len = ff_sqrt(s);
        FF mean = ff_add_f(len, -q[3]);
        FF tot = ff_add_f(mean, an);
        return __fadd_rn(tot.h, tot.l);
    }
    if (m.mean_kind == 3) {
        FF d = ff_add(ff_add(ff_prod(q[0], x), ff_prod(q[1], y)), ff_prod(q[2], z));
        FF tot = ff_add_f(ff_add_f(d, -q[3]), an);
        return __fadd_rn(tot.h, tot.l);
    }
    if (m.mean_kind == 4 || m.mean_kind == 5) {
        // the torus (and the union with the plane y = q[5]), which the reference evaluates
        // in double, in float-float: the differences are exact pairs, the square roots
        // good to about 46 bits, the sum with the noise rounded to float once
        float e0, e1, e2;
        const float h0 = two_sum(x, -q[0], e0), h1 = two_sum(y, -q[1], e1), h2 = two_sum(z, -q[2], e2);
        const FF dy = {h1, e1};
        const FF rxz = ff_add_f(ff_sqrt(ff_add(ff_sq({h0, e0}), ff_sq({h2, e2}))), -q[3]);
        FF mean = ff_add_f(ff_sqrt(ff_add(ff_sq(rxz), ff_sq(dy))), -q[4]);
        if (m.mean_kind == 5) {
            float e5;
            const FF pl = {two_sum(y, -q[5], e5), e5};
            if (pl.h < mean.h || (pl.h == mean.h && pl.l < mean.l)) {
                id = 1;
                mean = pl;
            }
        }
        const FF tot = ff_add_f(mean, an);
        return __fadd_rn(tot.h, tot.l);
    }
    // float means (homogeneous, grid): (float)((double)an + mean) is the rounded exact sum
    const float mv = mean_value(m, x, y, z, id);
    float e;
    const float s = two_sum(an, mv, e);
    return __fadd_rn(s, e);
}

// The 3D conditioning splats' value at p as the reference's float expressions give
// it: splattingKernel3D(p, origin, isCov) * value_scale plus splattingKernel3DGrad's
// value row sum_c gs_c * (-2 (ab_c M_c)) f (GPFunctions.cpp:555-580, 784-843).
__device__ __forceinline__ float cond3d_value_precise(const DevMedium &m, const CondRec &c, const float o[3],
                                                      const float p[3])
{
    float ab[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) ab[i] = __fsub_rn(p[i], o[i]);
    float absq = __fmul_rn(__fmul_rn(ab[0], m.m3c[0]), ab[0]);
    absq = __fadd_rn(absq, __fmul_rn(__fmul_rn(ab[1], m.m3c[1]), ab[1]));
    absq = __fadd_rn(absq, __fmul_rn(__fmul_rn(ab[2], m.m3c[2]), ab[2]));
    const float f = cr_expf(-absq);
    const CondOct &co = c.oct[0];
    float gv = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float g1 = __fmul_rn(__fmul_rn(-2.0f, __fmul_rn(ab[i], m.m3c[i])), f);
        gv = __fadd_rn(gv, __fmul_rn(g1, co.gs[i]));
    }
    return __fadd_rn(__fmul_rn(f, co.vs), gv);
}

__device__ float field_precise(const LaneField &L, float px, float py, float pz, int &id)
{
    const DevMedium &m = *L.m;
    if (general_3d(m)) {
        const float p[3] = {px, py, pz};
        float v, g[3];
        noise3d_gen<false, true>(m, p, L.d, L.cond ? &L.c3 : nullptr, L.o, L.seed, v, g);
        return mean_plus_precise(m, __fmul_rn(L.sigma, v), px, py, pz, id);
    }
    if (!(m.flags & MF_ONE_D)) {
        float noise = noise3d_precise(m, px, py, pz, L.seed);
        if (L.cond) {
            const float p[3] = {px, py, pz};
            noise = __fadd_rn(noise, cond3d_value_precise(m, L.c3, L.o, p));
        }
        return mean_plus_precise(m, __fmul_rn(L.sigma, noise), px, py, pz, id);
    }
    if (m.flags & MF_MULTIRES) {
        // evaluateValueNoise1D on the multi-resolution grid (SparseConvolutionNoise.cpp:156-165)
        const MrLevels lv = mr_levels(m, ls_value_precise(m, px, pz));
        float nl[2];
#pragma unroll 1
        for (int j = 0; j < 2; ++j) {
            const float z = ray_coord_oct(m, L.n, px, py, pz, lv.s[j]);
            float noise = noise1d_precise(m, z, L.seed + lv.seed[j], 1.0f);
            if (L.cond) {
                const float oz = ray_coord_oct(m, L.n, L.o[0], L.o[1], L.o[2], lv.s[j]);
                const float d = __fsub_rn(z, oz);
                const float den2 = m.cov_den2;
                const float k0 = cr_expf(-__fdiv_rn(__fmul_rn(d, d), den2));
                const float r = -2.0f * d;
                const float qh = __fdiv_rn(r, den2);
                const float ql = __fdiv_rn(__fmaf_rn(-qh, den2, r), den2);
                const float ph = __fmul_rn(qh, k0);
                const float k1 = __fadd_rn(ph, __fmaf_rn(ql, k0, __fmaf_rn(qh, k0, -ph)));
                const float vs0 = __fmul_rn(L.vs, k0);
                const float gz0 = __fmul_rn(__fmul_rn(lv.s[j], L.gsz), k1);
                noise = __fadd_rn(noise, __fmul_rn(L.mr_ow[j], __fadd_rn(vs0, gz0)));
            }
            nl[j] = noise;
        }
        const float nb = __fadd_rn(__fmul_rn(lv.w[0], nl[0]), __fmul_rn(lv.w[1], nl[1]));
        return mean_plus_precise(m, __fmul_rn(L.sigma, nb), px, py, pz, id);
    }
    const float ls = ns_scale_precise(m, px, pz);
    float an = 0.0f;
    for (int k = 0; k < (int)m.n_oct; ++k) {
        const float sc = oct_scale(m, k);
        const float z = m.n_oct == 1 && m.ls_kind == 0u ? ray_coord(L.li, L.n, px, py, pz)
                                                          : ray_coord_oct(m, L.n, px, py, pz, sc);
        float noise = noise1d_precise(m, z, L.seed + oct_seed(m, k), ls);
        if (L.cond) {
            // covarianceKernel1DVal / 1stGrad (GPFunctions.cpp:850-862) at the local
            // scale a: den2 = 2 (a sqrt2)^2 in float, the derivative in double
            float vs, gz, oz;
            lane_cond_1d(L, k, sc, vs, gz, oz);
            const float a = splat_cov_1d(ls, L.ls_o);
            float den2 = m.cov_den2;
            if (a != 1.0f) {
                const float s2 = (float)((double)a * 1.4142135623730951);
                den2 = (float)(2.0 * (double)__fmul_rn(s2, s2));
            }
            const float d = __fsub_rn(z, oz);
            const float k0 = cr_expf(-__fdiv_rn(__fmul_rn(d, d), den2));
            // (float)(-2 d / den2 * k0) with the quotient and product carried in
            // float-float: the double expression's rounding without FP64 division
            const float r = -2.0f * d;
            const float qh = __fdiv_rn(r, den2);
            const float ql = __fdiv_rn(__fmaf_rn(-qh, den2, r), den2);
            const float ph = __fmul_rn(qh, k0);
            const float k1 = __fadd_rn(ph, __fmaf_rn(ql, k0, __fmaf_rn(qh, k0, -ph)));
            const float vs0 = __fmul_rn(vs, k0);
            const float gz0 = __fmul_rn(gz, k1);
            noise = __fadd_rn(noise, __fmul_rn(1.0f, __fadd_rn(vs0, gz0)));
        }
        an = m.n_oct == 1 ? __fmul_rn(L.sigma, noise) : __fadd_rn(an, __fmul_rn(oct_sigma(m, k), noise));
    }
    return mean_plus_precise(m, an, px, py, pz, id);
}

// ---- fast evaluators ----------------------------------------------------------
// Generic evaluator: recomputes every impulse (any impulse count, 1D or 3D).
struct EvalGeneric {
    static constexpr bool kCollective = false;
    static constexpr int kMinBlocks = 2;
    static constexpr bool kGeneral = true;
    static constexpr bool kSkip = false;
    __device__ __forceinline__ void reset() {}
    __device__ __forceinline__ void bind(const PcgJump *) {}
    __device__ __forceinline__ float value(const LaneField &L, float px, float py, float pz,
                                           int &id, uint32_t &refills, bool)
    {
        const DevMedium &m = *L.m;
        float noise;
        if ((m.flags & MF_MULTIRES) && (m.flags & MF_ONE_D)) {
            const MrLevels lv = mr_levels(m, ls_value(m, px, pz));
            noise = 0.0f;
#pragma unroll 1
            for (int j = 0; j < 2; ++j) {
                const float z = ray_coord_oct(m, L.n, px, py, pz, lv.s[j]);
                float v, dv;
                noise1d_generic<false>(m, z, L.seed + lv.seed[j], v, dv, 1.0f);
                float nk = v * m.inv_norm1d;
                if (L.cond) {
                    const float oz = ray_coord_oct(m, L.n, L.o[0], L.o[1], L.o[2], lv.s[j]);
                    const Cov1D c = cov1d(z - oz);
                    nk += L.mr_ow[j] * (L.vs * c.k0 + (lv.s[j] * L.gsz) * c.k1);
                }
                noise += lv.w[j] * nk;
                refills += 3;
            }
            return L.sigma * noise + lane_mean(L, px, py, pz, id);
        }
        if (m.flags & MF_ONE_D) {
            const float ls = ns_scale(m, px, pz);
            noise = 0.0f;
            for (int k = 0; k < (int)m.n_oct; ++k) {
                const float sc = oct_scale(m, k);
                const float z = ray_coord_oct(m, L.n, px, py, pz, sc);
                float v, dv;
                noise1d_generic<false>(m, z, L.seed + oct_seed(m, k), v, dv, ls);
                float nk = v * inv_norm_1d(m, ls);
                if (L.cond) {
                    float vs, gz, oz;
                    lane_cond_1d(L, k, sc, vs, gz, oz);
                    const Cov1D c = cov1d(z - oz, splat_cov_1d(ls, L.ls_o));
                    nk += vs * c.k0 + gz * c.k1;
                }
                noise += oct_sigma(m, k) * nk;
                refills += 3;
            }
            return noise + lane_mean(L, px, py, pz, id);
        }
        float v, g[3];
        if (general_3d(m)) {
            const float p[3] = {px, py, pz};
            refills += noise3d_gen<false, false>(m, p, L.d, L.cond ? &L.c3 : nullptr, L.o, L.seed, v, g);
            return L.sigma * v + lane_mean(L, px, py, pz, id);
        }
        noise3d_generic<false>(m, px, py, pz, L.seed, v, g);
        noise = v * m.inv_norm3d;
        if (L.cond) {
            float cv, cg[3];
            const float p[3] = {px, py, pz};
            cond3d(m, L.c3, L.o, p, cv, cg);
            noise += cv;
        }
        refills += 27;
        return L.sigma * noise + lane_mean(L, px, py, pz, id);
    }
};

// The resume passes of batches whose media all use 1D noise: the generic evaluator
// compiled for 4 blocks of 256 per SM (64 registers, with spills).  For the precise
// pass that decides every crossing it hides the precise evaluator's dependent
// float-float chains better than 2 blocks at 128 registers (15.93 against 16.57 ms
// per bench step; 3 blocks: 16.07); the certified pass runs it too.  3D media keep
// 2 blocks: their 27-cell evaluations spill too much at 64 registers.
struct EvalGeneric4 : EvalGeneric {
    static constexpr int kMinBlocks = 4;
};

// Certified crossing decisions of the resume pass.  The refinement after a crossing
// (SparseConvolutionNoiseMedium.cpp:296-330) decides the sign of the field at
// t = ta + fac * step, fac = f(ta) / (f(ta) - f(tb)), and then fac <= 0.01 after each
// x0.9 back-off.  The reference takes those values in float at its own points.  For
// 1D stationary single-octave media with an analytic mean the pass decides them on
// EvalGeneric's fast values instead whenever the decision is certain:
//  * a fast value differs from the reference's float value at the same point by less
//    than kPreciseBand (the margin the fast pass's sign decisions use), so fac is
//    within dfac = 1.1 eps (|f(ta)| + |f(tb)|) / (f(ta) - f(tb))^2 of the reference's
//    (for |f(ta) - f(tb)| >= 64 eps) and the refinement point within step * dfac;
//  * the two points differ by d dt plus the rounding of each (pu: four float ulps of
//    the largest coordinate); between them the field moves by at most the ray's
//    slope bound (the step-skipping Lipschitz constant) times dt plus the gradient
//    bound times pu, both of which hold away from the splats' truncation edges, and
//    no truncation edge or cell face lies between them when the query's margin to
//    the nearest one exceeds their distance in cells.
// A sign is certain when |f| exceeds 2 eps plus that movement with the margin clear;
// a back-off comparison when |fac - 0.01| exceeds dfac.  Anything else restarts the
// crossing at tb with the precise evaluator, as without certification.
__device__ __forceinline__ bool cert_medium(const DevMedium &m)
{
    return (m.flags & MF_ONE_D) && m.n_oct == 1 && !(m.flags & MF_MULTIRES) && m.ls_kind == 0u &&
           m.mean_kind != GPIS_MEAN_GRID && m.skip_mean_lip >= 0.0f;
}

// true when the sign of the reference's value at its refinement point is that of
// the fast value f at this one (dt: the bound on their distance in t)
__device__ __forceinline__ bool cert_sign(const DevMedium &m, const LaneField &L, const float d[3], const float p[3],
                                          float step, float f, float margin, float dt, float eps)
{
    float lip, j0, j1;
    skip_params(m, d, L.sigma, L.cond, L.vs, L.gsz, step, lip, j0, j1);
    const float lmax = fmaxf(fabsf(m.l_inv[0]), fmaxf(fabsf(m.l_inv[1]), fabsf(m.l_inv[2])));
    const float lx = m.l_inv[0] * d[0], ly = m.l_inv[1] * d[1], lz = m.l_inv[2] * d[2];
    const float dz = sqrtf(lx * lx + ly * ly + lz * lz) * 1.0001f / m.kr_iso;   // cells per unit of t
    const float cslope = L.cond ? 0.42888194f * fabsf(L.vs) + 0.5f * fabsf(L.gsz) : 0.0f;
    const float grad = (m.skip_mean_lip + fabsf(L.sigma) * (m.skip_noise_lip + cslope) * lmax) * 1.01f;
    const float pu = 0x1p-21f * fmaxf(fabsf(p[0]), fmaxf(fabsf(p[1]), fabsf(p[2])));
    const float move = lip * dt + grad * pu;
    const float cells = dz * dt + lmax * 1.0001f / m.kr_iso * pu;
    return lip >= 0.0f && fabsf(f) > 2.0f * eps + move && margin > cells && isfinite(move) && isfinite(cells);
}

// EvalGeneric's value of such a medium, with the query's margin in cells
__device__ __forceinline__ float value_1d_cert(const LaneField &L, float px, float py, float pz, int &id, float &margin)
{
    const DevMedium &m = *L.m;
    const float ls = ns_scale(m, px, pz);
    const float z = ray_coord_oct(m, L.n, px, py, pz, oct_scale(m, 0));
    float v, dv;
    noise1d_generic<false, true>(m, z, L.seed + oct_seed(m, 0), v, dv, ls, &margin);
    float nk = v * inv_norm_1d(m, ls);
    if (L.cond) {
        const Cov1D c = cov1d(z - L.ozc, splat_cov_1d(ls, L.ls_o));
        nk += L.vs * c.k0 + L.gsz * c.k1;
    }
    return oct_sigma(m, 0) * nk + lane_mean(L, px, py, pz, id);
}

// the bound on fac's distance from the reference's (false: too close to call)
__device__ __forceinline__ bool cert_fac(float pf, float fb, float eps, float &dfac)
{
    const float den = fabsf(pf - fb);
    if (!(den >= 64.0f * eps)) return false;
    dfac = 1.1f * eps * (fabsf(pf) + fabsf(fb)) / (den * den) + 0x1p-40f;
    return isfinite(dfac);
}

// 3D stationary single-octave media with step skipping.  The value is EvalGeneric's
// (the same arithmetic); a march step that plans a segment [p, p + D d] also gets the
// range of the field over it: the raw noise sum's range (noise3d_core), the
// conditioning splat's exact range along the segment (its exponent is a quadratic in
// the segment parameter; the Renewal+ gradient terms bounded by their largest
// magnitude), and the mean within its Lipschitz slope times the segment length.  The
// segment ends inside p's cell (less kSupportEps of a cell), where the 27 cells hold
// every impulse that reaches it.  When the range keeps the sign of f with a margin
// above the float evaluations' error, every step on the segment keeps it too and the
// reference would march past: those steps are skipped.
struct EvalSkip3D {
    static constexpr bool kCollective = false;
    static constexpr int kMinBlocks = 2;
    static constexpr bool kGeneral = true;
    static constexpr bool kSkip = false;
    static constexpr bool kSkip3D = true;
    float want;          // planned segment length (world units along d; 0: none)
    float dlen;          // the segment's length actually bounded
    float f_lo, f_hi;    // the field's range over it

    __device__ __forceinline__ void reset() { want = 0.0f; dlen = 0.0f; }
    __device__ __forceinline__ void bind(const PcgJump *) {}
    __device__ __forceinline__ void plan(float len) { want = len; }

    __device__ __forceinline__ float value(const LaneField &L, const float d[3], float px, float py, float pz, int &id,
                                           uint32_t &refills, bool)
    {
        const DevMedium &m = *L.m;
        refills += 27;
        float len = want;
        want = 0.0f;
        dlen = 0.0f;
        const float kr = m.kr_world;
        // the segment's end inside p's cell: the distance to the cell's faces along d
        if (len > 0.0f && m.skip_mean_lip >= 0.0f) {
            const float p[3] = {px, py, pz};
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float q = __fdiv_rn(p[i], kr);
                const float fr = __fsub_rn(q, floorf(q));
                const float di = d[i] / kr;   // cells per unit of t
                float room = 1e30f;
                if (di > 0.0f) room = (1.0f - kSupportEps - fr) / di;
                else if (di < 0.0f) room = (fr - kSupportEps) / -di;
                len = fminf(len, room);
            }
        } else {
            len = 0.0f;
        }
        float v, g[3], lo = 0.0f, hi = 0.0f;
        if (len > 0.0f) {
            const float E[3] = {len * d[0] / kr, len * d[1] / kr, len * d[2] / kr};
            const float ee = E[0] * E[0] + E[1] * E[1] + E[2] * E[2];
            const float kr2 = kr * kr;
            const float kmax2 = fmaxf(fmaxf(m.kexp3d[0], m.kexp3d[1]), m.kexp3d[2]) * kr2;
            const float kmin2 = fminf(fminf(m.kexp3d[0], m.kexp3d[1]), m.kexp3d[2]) * kr2;
            noise3d_core<false, true>(m, px, py, pz, L.seed, v, g, E, ee, kmax2, kmin2, lo, hi);
        } else {
            noise3d_generic<false>(m, px, py, pz, L.seed, v, g);
        }
        float noise = v * m.inv_norm3d;
        float nlo = lo * m.inv_norm3d, nhi = hi * m.inv_norm3d;
        const float p[3] = {px, py, pz};
        if (L.cond) {
            float cv, cg[3];
            cond3d(m, L.c3, L.o, p, cv, cg);
            noise += cv;
            if (len > 0.0f) {
                // exponent -log2e Q(s), Q(s) = C + 2 B s + A s^2 over s in [0, 1]
                float A = 0.0f, B = 0.0f, C = 0.0f, gh = 0.0f, eh = 0.0f;
                const CondOct &co = L.c3.oct[0];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const float ab = p[i] - L.o[i], ew = len * d[i];
                    A += m.m3c[i] * ew * ew;
                    B += m.m3c[i] * ab * ew;
                    C += m.m3c[i] * ab * ab;
                    gh += ab * m.m3c[i] * co.gs[i];
                    eh += ew * m.m3c[i] * co.gs[i];
                }
                const float sn = A > 0.0f ? fminf(fmaxf(-B / A, 0.0f), 1.0f) : 0.0f;
                const float qmin = fmaxf(C + sn * (2.0f * B + sn * A), 0.0f);
                const float qmax = fmaxf(C, C + 2.0f * B + A);
                const float fmax = ex2_approx(-LOG2E * qmin) * 1.00001f;
                const float fmin = ex2_approx(-LOG2E * qmax) * 0.99999f;
                const float vlo = co.vs >= 0.0f ? co.vs * fmin : co.vs * fmax;
                const float vhi = co.vs >= 0.0f ? co.vs * fmax : co.vs * fmin;
                const float gb = 2.0f * fmax * (fabsf(gh) + fabsf(eh)) * 1.00001f;
                nlo += vlo - gb;
                nhi += vhi + gb;
            }
        }
        const float mu = lane_mean(L, px, py, pz, id);
        if (len > 0.0f) {
            const float dn = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            const float dm = m.skip_mean_lip * len * dn * 1.0001f;
            const float sg = L.sigma;
            f_lo = (sg >= 0.0f ? sg * nlo : sg * nhi) + mu - dm;
            f_hi = (sg >= 0.0f ? sg * nhi : sg * nlo) + mu + dm;
            dlen = len;
        }
        return L.sigma * noise + mu;
    }

    // steps of length `step` after p that keep the sign of f (f the value at p)
    __device__ __forceinline__ int skips(float f, float step, int cap) const
    {
        if (!(dlen > 0.0f)) return 0;
        const float margin = 1e-5f + 1e-6f * fmaxf(fabsf(f_lo), fabsf(f_hi));
        const bool keep = f > 0.0f ? f_lo > margin : (f < 0.0f && f_hi < -margin);
        if (!keep) return 0;
        return (int)fminf(floorf(dlen / step * (1.0f - 1e-6f)), (float)cap);
    }
};

// 1D evaluator with the three-cell impulse window in registers and a
// warp-cooperative refill: the lanes whose query entered a new cell are
// gathered by a ballot and the whole warp generates their cells, one impulse per
// lane (the jump-ahead PCG draws any impulse of a cell independently), 32/NMAX
// cells per pass; shuffles deliver each cell into its owner's registers.  Every
// lane of the warp must call value() (idle lanes pass live = false).
// SM: the three-cell window lives in dynamic shared memory as a ring of slots
// (kSmem1D bytes per 256-thread block, float4 rows per lane as EvalCoopOct lays
// them out) instead of 24 registers per lane; a one-cell move then refills one
// slot without shifting the others.
constexpr int kC1Threads = 256;
constexpr size_t kSmem1D = (size_t)3 * 8 * sizeof(float) * kC1Threads;

template <int NMAX, bool GRID = false, bool NS = false, bool SM = false>
struct EvalCoop1D {
    static constexpr bool kCollective = true;
    // CTAs per SM for the stationary analytic-mean kernel: with the window in shared
    // memory 3 (80 registers; 14.34 ms per bench step against 14.72 for 4 CTAs at 64
    // registers, whose spills feed long-scoreboard stalls, and 15.44 for 2 at 128),
    // with the window in registers 4 (64 registers, 2 % faster than 2 CTAs at 128
    // despite spills); the grid and nonstationary variants keep 2
    static constexpr int kMinBlocks = (GRID || NS) ? 2 : (SM ? 3 : 4);
    static constexpr bool kGeneral = NS;   // stationary, single octave, 1D otherwise
    static constexpr bool kSkip = !NS;
    float cache[SM ? 1 : 3][SM ? 1 : NMAX];
    int base;
    bool valid;
    const PcgJump *sj;      // the jump table in shared memory
    float last_ls;          // nonstationary: the local scale at the last evaluated point
    float *cbase;           // SM: the window's shared memory
    int rot;                // SM: logical cell j (0: ci - 1, 1: ci, 2: ci + 1) sits in slot (rot + j) mod 3

    __device__ __forceinline__ void reset() { valid = false; base = 0; last_ls = 1.0f; rot = 0; }
    __device__ __forceinline__ void bind(const PcgJump *t)
    {
        sj = t;
        if (SM) {
            extern __shared__ float4 dsm_c1[];
            cbase = reinterpret_cast<float *>(dsm_c1);
        }
    }
    __device__ __forceinline__ float *slot_ptr(int tid, int slot, int k) const
    {
        return cbase + (((slot * 2 + (k >> 2)) * kC1Threads + tid) << 2) + (k & 3);
    }

    // SM: cooperative generation of one cell per requesting lane, each impulse written
    // by the lane that draws it straight into the owner's ring slot
    __device__ __forceinline__ void fill_sm(bool need, int cell, int slot, const LaneField &L, int lane)
    {
        unsigned mask = __ballot_sync(FULL, need);
        const int rq = lane >> 3;
        const int k = lane & 7;
        const int warp0 = threadIdx.x & ~31;
        while (mask) {
            unsigned pass = 0u, mm = mask;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                pass |= mm & (0u - mm);
                mm &= mm - 1u;
            }
            mask = mm;
            unsigned pm = pass;
            for (int r = 0; r < rq; ++r) pm &= pm - 1u;
            const int owner = pm ? __ffs(pm) - 1 : 0;
            const int ocell = __shfl_sync(FULL, cell, owner);
            const uint32_t oseed = __shfl_sync(FULL, L.seed, owner);
            const int oslot = __shfl_sync(FULL, slot, owner);
            const uint32_t onimp = __shfl_sync(FULL, L.n_imp, owner);
            if (pm != 0u) {
                float v = __int_as_float(0x7f800000);
                if ((uint32_t)k < onimp) {
                    const uint32_t s = xxhash2((uint32_t)ocell, oseed) + 1u;
                    const uint32_t r1 = pcg_draw(sj[2 + 2 * k], s);
                    const uint32_t r2 = pcg_draw(sj[3 + 2 * k], s);
                    v = __uint_as_float(__float_as_uint(unit_float(r1)) | (~r2 & 0x80000000u));
                }
                *slot_ptr(warp0 + owner, oslot, k) = v;
            }
        }
        __syncwarp();
    }

    template <int S>
    __device__ __forceinline__ void fill_slot(bool need, int cell, const LaneField &L, int lane)
    {
        unsigned mask = __ballot_sync(FULL, need);
        const int rq = lane / NMAX;
        const int k = lane % NMAX;
        while (mask) {
            unsigned pass = 0u, m = mask;
#pragma unroll
            for (int r = 0; r < 32 / NMAX; ++r) {
                pass |= m & (0u - m);
                m &= m - 1u;
            }
            mask = m;
            // the request this lane produces an impulse for
            unsigned pm = pass;
            for (int r = 0; r < rq; ++r) pm &= pm - 1u;
            const int owner = pm ? __ffs(pm) - 1 : 0;
            const int ocell = __shfl_sync(FULL, cell, owner);
            const uint32_t oseed = __shfl_sync(FULL, L.seed, owner);
            const uint32_t onimp = __shfl_sync(FULL, L.n_imp, owner);
            float v = __int_as_float(0x7f800000);
            if (pm != 0u && (uint32_t)k < onimp) {
                const uint32_t s = xxhash2((uint32_t)ocell, oseed) + 1u;
                const uint32_t r1 = pcg_draw(sj[2 + 2 * k], s);
                const uint32_t r2 = pcg_draw(sj[3 + 2 * k], s);
                v = __uint_as_float(__float_as_uint(unit_float(r1)) | (~r2 & 0x80000000u));
            }
            const bool mine = (pass >> lane) & 1u;
            const int myrq = __popc(pass & ((1u << lane) - 1u));
#pragma unroll
            for (int kk = 0; kk < NMAX; ++kk) {
                const float x = __shfl_sync(FULL, v, myrq * NMAX + kk);
                if (mine) cache[S][kk] = x;
            }
        }
    }

    __device__ __forceinline__ float value(const LaneField &L, float px, float py, float pz,
                                           int &id, uint32_t &refills, bool live)
    {
        const int lane = threadIdx.x & 31;
        // a grid mean's voxel loads go first so that their latency overlaps the noise
        GridTap tap;
        const bool on_grid = GRID && L.mean_kind == GPIS_MEAN_GRID;
        if (on_grid) grid_fetch(*L.m, px, py, pz, tap);
        // nonstationary: coordinate in the ls_max-scaled space, kernel width,
        // normalisation and conditioning scale at the query
        float z, kexp = L.kexp, inv_norm = L.inv_norm, ca = 1.0f;
        if (NS && L.ns) {
            const float ls = ns_scale(*L.m, px, pz);
            last_ls = ls;
            z = ray_coord_oct(*L.m, L.n, px, py, pz, 1.0f);
            kexp = L.kexp / (ls * ls);
            inv_norm = inv_norm_1d(*L.m, ls);
            ca = splat_cov_1d(ls, L.ls_o);
        } else {
            z = ray_coord(L.li, L.n, px, py, pz);
        }
        const float tg = __fdiv_rn(z, L.kr);
        const float fl = floorf(tg);
        const float frac = __fsub_rn(tg, fl);
        const int ci = (int)fl;
        const bool changed = live && (!valid || ci != base);
        const bool up = changed && valid && ci == base + 1;
        const bool down = changed && valid && ci == base - 1;
        const bool full = changed && !up && !down;
        float acc0 = 0.0f, acc1 = 0.0f;
        if constexpr (SM) {
            int r = rot;
            if (up) r = r == 2 ? 0 : r + 1;          // the old middle becomes the low cell
            if (down) r = r == 0 ? 2 : r - 1;
            if (full) r = 0;
            const int s0 = r, s1 = r == 2 ? 0 : r + 1, s2 = r == 0 ? 2 : r - 1;
            fill_sm(full || down, ci - 1, s0, L, lane);
            fill_sm(full, ci, s1, L, lane);
            fill_sm(full || up, ci + 1, s2, L, lane);
            if (changed) {
                base = ci;
                rot = r;
                valid = true;
                refills += full ? 3u : 1u;
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float tl = __fsub_rn(frac, (float)(c - 1));
                const int slot = c == 0 ? s0 : (c == 1 ? s1 : s2);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float4 q4 = *reinterpret_cast<const float4 *>(slot_ptr(threadIdx.x, slot, 4 * h));
                    const float qs[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float sv = qs[j];
                        const float tp = __fsub_rn(tl, fabsf(sv));
                        const float e = ex2_approx(kexp * (tp * tp));
                        const float w = __uint_as_float(__float_as_uint(e) | (__float_as_uint(sv) & 0x80000000u));
                        if (j & 1) acc1 += fabsf(tp) < 1.0f ? w : 0.0f;
                        else acc0 += fabsf(tp) < 1.0f ? w : 0.0f;
                    }
                }
            }
        } else {
            if (up) {
#pragma unroll
                for (int k = 0; k < NMAX; ++k) { cache[0][k] = cache[1][k]; cache[1][k] = cache[2][k]; }
            }
            if (down) {
#pragma unroll
                for (int k = 0; k < NMAX; ++k) { cache[2][k] = cache[1][k]; cache[1][k] = cache[0][k]; }
            }
            fill_slot<0>(full || down, ci - 1, L, lane);
            fill_slot<1>(full, ci, L, lane);
            fill_slot<2>(full || up, ci + 1, L, lane);
            if (changed) {
                base = ci;
                valid = true;
                refills += full ? 3u : 1u;
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float tl = __fsub_rn(frac, (float)(c - 1));
#pragma unroll
                for (int k = 0; k < NMAX; ++k) {
                    const float sv = cache[c][k];
                    const float tp = __fsub_rn(tl, fabsf(sv));
                    const float e = ex2_approx(kexp * (tp * tp));
                    const float w = __uint_as_float(__float_as_uint(e) | (__float_as_uint(sv) & 0x80000000u));
                    if (k & 1) acc1 += fabsf(tp) < 1.0f ? w : 0.0f;
                    else acc0 += fabsf(tp) < 1.0f ? w : 0.0f;
                }
            }
        }
        float noise = (acc0 + acc1) * inv_norm;
        if (L.cond) {
            const Cov1D k = NS ? cov1d(z - L.ozc, ca) : cov1d(z - L.ozc);
            noise += L.vs * k.k0 + L.gsz * k.k1;
        }
        if (on_grid) {
            id = 0;
            return L.sigma * noise + grid_combine(*L.m, tap);
        }
        return L.sigma * noise + lane_mean(L, px, py, pz, id);
    }
};

// 1D evaluator for media with several octaves (and any length scale): each
// octave's three-cell impulse window (8 impulses per cell) lives in shared
// memory, 96 floats per lane, laid out [octave][cell slot][k / 4][lane] in
// float4 so that a warp's loads are contiguous.  A ring index per octave turns
// a one-cell move into one refill; refills are warp-cooperative as in
// EvalCoop1D, with the producing lane writing the impulse straight into the
// owner's slot.  Every lane of the warp must call value().
constexpr int kOctMax = 4;
constexpr int kOctThreads = 256;
constexpr size_t kSmemOct = (size_t)kOctMax * 3 * 8 * sizeof(float) * kOctThreads;

struct EvalCoopOct {
    static constexpr bool kCollective = true;
    static constexpr int kMinBlocks = 2;
    static constexpr bool kGeneral = true;
    static constexpr bool kSkip = false;
    float *cbase;           // float index ((o * 3 + slot) * 8 + k) maps to cbase[(((o*3+slot)*2 + k/4)*256 + tid)*4 + k%4]
    int base[kOctMax];
    int rot[kOctMax];
    uint32_t valid;         // bit o: octave o's window is filled
    const PcgJump *sj;
    float last_ls;          // the local scale at the last evaluated point

    __device__ __forceinline__ void reset() { valid = 0u; last_ls = 1.0f; }
    __device__ __forceinline__ void bind(const PcgJump *t)
    {
        extern __shared__ float4 dsm_oct[];
        cbase = reinterpret_cast<float *>(dsm_oct);
        sj = t;
    }
    __device__ __forceinline__ float *slot_ptr(int tid, int o, int slot, int k) const
    {
        return cbase + ((((o * 3 + slot) * 2 + (k >> 2)) * kOctThreads + tid) << 2) + (k & 3);
    }

    // cooperative generation of one cell per requesting lane into its ring slot
    __device__ __forceinline__ void fill(bool need, int cell, uint32_t seed, int o, int slot, int lane, uint32_t n_imp)
    {
        unsigned mask = __ballot_sync(FULL, need);
        const int rq = lane >> 3;
        const int k = lane & 7;
        const int warp0 = threadIdx.x & ~31;
        while (mask) {
            unsigned pass = 0u, mm = mask;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                pass |= mm & (0u - mm);
                mm &= mm - 1u;
            }
            mask = mm;
            unsigned pm = pass;
            for (int r = 0; r < rq; ++r) pm &= pm - 1u;
            const int owner = pm ? __ffs(pm) - 1 : 0;
            const int ocell = __shfl_sync(FULL, cell, owner);
            const uint32_t oseed = __shfl_sync(FULL, seed, owner);
            const int oslot = __shfl_sync(FULL, slot, owner);
            const uint32_t onimp = __shfl_sync(FULL, n_imp, owner);
            if (pm != 0u) {
                float v = __int_as_float(0x7f800000);
                if ((uint32_t)k < onimp) {
                    const uint32_t s = xxhash2((uint32_t)ocell, oseed) + 1u;
                    const uint32_t r1 = pcg_draw(sj[2 + 2 * k], s);
                    const uint32_t r2 = pcg_draw(sj[3 + 2 * k], s);
                    v = __uint_as_float(__float_as_uint(unit_float(r1)) | (~r2 & 0x80000000u));
                }
                *slot_ptr(warp0 + owner, o, oslot, k) = v;
            }
        }
        __syncwarp();
    }

    __device__ __forceinline__ float value(const LaneField &L, float px, float py, float pz,
                                           int &id, uint32_t &refills, bool live)
    {
        const int lane = threadIdx.x & 31;
        const DevMedium &m = *L.m;
        const int n_oct = live ? (int)m.n_oct : 0;
        const float ls = live ? ns_scale(m, px, pz) : 1.0f;
        last_ls = ls;
        const float kexp = L.kexp / (ls * ls);
        const float inv_norm = inv_norm_1d(m, ls);
        const float ca = splat_cov_1d(ls, L.ls_o);
        // the isotropic position (divided by the maximum lateral scale) once; each
        // octave divides it by its length multiplier, a multiply when that is a
        // power of two (the same rounding as ray_coord_oct's division)
        float bx = __fmul_rn(m.l_inv[0], px), by = __fmul_rn(m.l_inv[1], py), bz = __fmul_rn(m.l_inv[2], pz);
        if (m.ls_kind) {
            bx = __fdiv_rn(bx, m.ls_max);
            by = __fdiv_rn(by, m.ls_max);
            bz = __fdiv_rn(bz, m.ls_max);
        }
        float total = 0.0f;
        const int warp_oct = __reduce_max_sync(FULL, (unsigned)n_oct);
#pragma unroll
        for (int o = 0; o < kOctMax; ++o) {
            if (o >= warp_oct) break;
            const bool act = o < n_oct;
            const float sc = act ? oct_scale(m, o) : 1.0f;
            float qx = bx, qy = by, qz = bz;
            if (sc != 1.0f) {
                if ((m.oct_pow2 >> o) & 1u) {
                    const float inv = m.oct_inv[o];
                    qx = __fmul_rn(qx, inv); qy = __fmul_rn(qy, inv); qz = __fmul_rn(qz, inv);
                } else {
                    qx = __fdiv_rn(qx, sc); qy = __fdiv_rn(qy, sc); qz = __fdiv_rn(qz, sc);
                }
            }
            const float z = act ? dot3_rn(L.n[0], L.n[1], L.n[2], qx, qy, qz) : 0.0f;
            const float tg = __fdiv_rn(z, L.kr);
            const float fl = floorf(tg);
            const float frac = __fsub_rn(tg, fl);
            const int ci = (int)fl;
            const bool ok = (valid >> o) & 1u;
            const bool changed = act && (!ok || ci != base[o]);
            const bool up = changed && ok && ci == base[o] + 1;
            const bool down = changed && ok && ci == base[o] - 1;
            const bool full = changed && !up && !down;
            const uint32_t seed = L.seed + oct_seed(m, o);
            int r = rot[o];
            if (up) r = r == 2 ? 0 : r + 1;          // the old middle becomes the low cell
            if (down) r = r == 0 ? 2 : r - 1;
            if (full) r = 0;
            // logical cell j (0: ci - 1, 1: ci, 2: ci + 1) sits in slot (r + j) mod 3
            const int s0 = r, s1 = r == 2 ? 0 : r + 1, s2 = r == 0 ? 2 : r - 1;
            fill(full || down, ci - 1, seed, o, s0, lane, L.n_imp);
            fill(full, ci, seed, o, s1, lane, L.n_imp);
            fill(full || up, ci + 1, seed, o, s2, lane, L.n_imp);
            if (changed) {
                base[o] = ci;
                rot[o] = r;
                valid |= 1u << o;
                refills += full ? 3u : 1u;
            }
            if (!act) continue;
            float acc0 = 0.0f, acc1 = 0.0f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float tl = __fsub_rn(frac, (float)(c - 1));
                const int slot = c == 0 ? s0 : (c == 1 ? s1 : s2);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float4 q4 = *reinterpret_cast<const float4 *>(slot_ptr(threadIdx.x, o, slot, 4 * h));
                    const float qs[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float sgn = qs[j];
                        const float tp = __fsub_rn(tl, fabsf(sgn));
                        const float e = ex2_approx(kexp * (tp * tp));
                        const float w = __uint_as_float(__float_as_uint(e) | (__float_as_uint(sgn) & 0x80000000u));
                        if (j & 1) acc1 += fabsf(tp) < 1.0f ? w : 0.0f;
                        else acc0 += fabsf(tp) < 1.0f ? w : 0.0f;
                    }
                }
            }
            float nk = (acc0 + acc1) * inv_norm;
            if (L.cond) {
                float vs, gz, oz;
                lane_cond_1d(L, o, sc, vs, gz, oz);
                const Cov1D kc = cov1d(z - oz, ca);
                nk += vs * kc.k0 + gz * kc.k1;
            }
            total += (m.n_oct == 1 ? L.sigma : oct_sigma(m, o)) * nk;
        }
        return total + lane_mean(L, px, py, pz, id);
    }
};

// Phases of a lane's flight.  The fast evaluator marches; a precise evaluation
// re-decides every step whose fast value is within the band of zero or changed
// sign, evaluates the step before a crossing (when that one was fast) and every
// refinement point.
enum : int { PH_IDLE = 0, PH_F0, PH_F0_P, PH_MARCH, PH_MARCH_P, PH_PF, PH_REFINE, PH_FAR };

// most march steps one evaluation may skip (fast pass; the skipped steps cost one
// jump when t_direct_ok holds, a loop that the warp runs for its longest lane
// otherwise)
constexpr int kMaxSkip = 16;
// at most this many steps skipped per evaluation of a 3D medium (the segment also ends
// inside the query's cell)
constexpr int kMaxSkip3D = 32;

// Step skipping for multi-octave and nonstationary 1D media (EvalCoopOct, and
// EvalCoop1D's nonstationary form): a Lipschitz bound along the ray over the next
// `cap` steps, from the local scale's range there (multi-octave evaluations cost
// more than the warp's skip loop, so they may skip 16 steps; single-octave ones 8).  Octave k's noise is A(ls) S_k + C_k with S_k the sum of at
// most 3N truncated splats exp(-(z_k - z_i)^2 / (2 ls^2)) in the octave's iso
// coordinate z_k (|dz_k/dt| <= |l_inv o d| / (ls_max sc_k)), A(ls) = inv_norm1d
// ls^-1/2 the normalisation and C_k the conditioning splats.  Per splat |dK/dz| <=
// e^-1/2 / ls and |dK/dls| <= 2 / (e ls); |S_k| <= 3N; |dA/dls| = A / (2 ls); the
// conditioning kernels k0 = exp(-ia2 d^2 / 4), k1 = -ia2 d k0 / 2 with ia2 = 2 /
// (ls^2 + ls_o^2) (1 when stationary) have |dk0/dd| <= 0.42888 sqrt(ia2), |dk1/dd|
// <= ia2 / 2, |dk0/dia2| <= 1 / (e ia2), |dk1/dia2| <= 0.84 / sqrt(ia2) and
// |dia2/dls| <= 4 ls / (ls^2 + ls_o^2)^2; ls changes by at most |q1| sqrt(q2^2 +
// q3^2) / ls_max per unit of lateral (x, z) travel.  Every bound takes the worst
// local scale of the range.  A splat jumps by at most exp(-kr^2 / (2 ls_hi^2)) where
// the query crosses its support, and 2N (cells crossed + 1) crossings per octave
// are allowed for, as for single-octave media.  Returns the steps after the
// evaluated point that keep the sign of f (margins as for single-octave media).
__device__ __forceinline__ int oct_skip_count(const DevMedium &m, const LaneField &L, const float d[3], float ls_p,
                                              float f, float step, int cap)
{
    if (m.skip_mean_lip < 0.0f) return 0;
    const float span = (float)cap * step;
    float ls_lo = ls_p, ls_hi = ls_p, dls = 0.0f;
    const float lx = m.l_inv[0] * d[0], ly = m.l_inv[1] * d[1], lz = m.l_inv[2] * d[2];
    float dn = sqrtf(lx * lx + ly * ly + lz * lz) * 1.0001f;
    if (m.ls_kind) {
        const float *q = m.ls_params;
        dls = fabsf(q[1]) * sqrtf(q[2] * q[2] + q[3] * q[3]) / m.ls_max * sqrtf(d[0] * d[0] + d[2] * d[2]) * 1.0001f;
        const float glo = (q[0] - fabsf(q[1])) / m.ls_max, ghi = (q[0] + fabsf(q[1])) / m.ls_max;
        ls_lo = fmaxf(ls_p - dls * span - 1e-6f, glo * 0.9999f);
        ls_hi = fminf(ls_p + dls * span + 1e-6f, ghi * 1.0001f);
        if (!(ls_lo > 0.0f)) return 0;
        dn /= m.ls_max;
    }
    const float n3 = 3.0f * (float)m.n_imp;
    const float a_lo = m.inv_norm1d * rsqrtf(ls_lo) * 1.0001f;    // the largest normalisation
    const float e_h = 0.60653066f, e_1 = 0.36787944f;
    const float jump = expf(-0.5f * m.kr_iso * m.kr_iso / (ls_hi * ls_hi)) * 1.0001f;
    const float ia_hi = m.ls_kind ? 2.0f / (ls_lo * ls_lo + L.ls_o * L.ls_o) : 1.0f;
    const float ia_lo = m.ls_kind ? 2.0f / (ls_hi * ls_hi + L.ls_o * L.ls_o) : 1.0f;
    const float dia = m.ls_kind ? 4.0f * ls_hi / ((ls_lo * ls_lo + L.ls_o * L.ls_o) * (ls_lo * ls_lo + L.ls_o * L.ls_o))
                                : 0.0f;
    float lip = m.skip_mean_lip * sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    float j0 = 0.0f, j1 = 0.0f;
#pragma unroll
    for (int k = 0; k < kOctMax; ++k) {
        if (k >= (int)m.n_oct) break;
        const float sg = fabsf(oct_sigma(m, k));
        const float sc = oct_scale(m, k);
        const float dz = dn / sc;
        float slope = a_lo * n3 * (e_h / ls_lo * dz + 2.0f * e_1 / ls_lo * dls) + n3 * a_lo / (2.0f * ls_lo) * dls;
        if (L.cond) {
            float vs, gz, oz;
            lane_cond_1d(L, k, sc, vs, gz, oz);
            slope += (0.42888194f * sqrtf(ia_hi) * fabsf(vs) + 0.5f * ia_hi * fabsf(gz)) * dz;
            if (m.ls_kind)
                slope += (fabsf(vs) * e_1 / ia_lo + fabsf(gz) * 0.84f * rsqrtf(ia_lo)) * dia * dls;
        }
        lip += sg * slope;
        const float jn = sg * a_lo * jump * 2.0f * (float)m.n_imp * 1.01f;
        j0 += 3.0f * jn;
        j1 += jn * (step * dz / m.kr_iso);
    }
    lip *= 1.01f;
    const float af = fabsf(f) * (1.0f - 1e-6f) - 1e-5f - j0;
    const float per = lip * step + j1;
    if (!(af > per)) return 0;
    return (int)fminf(af / per, (float)cap);
}

// the evaluators whose fast pass skips by oct_skip_count, and the cap of each
template <class E> struct IsOct { static constexpr bool value = false; static constexpr int cap = 0; };
template <> struct IsOct<EvalCoopOct> { static constexpr bool value = true; static constexpr int cap = 16; };
template <> struct IsOct<EvalCoop1D<8, false, true>> { static constexpr bool value = true; static constexpr int cap = 8; };

template <class E> struct IsSkip3D { static constexpr bool value = false; };
template <> struct IsSkip3D<EvalSkip3D> { static constexpr bool value = true; };

template <class Eval>
__device__ __forceinline__ float eval_at(Eval &ev, const LaneField &L, const float *, const float p[3], int &id,
                                         uint32_t &refills, bool live)
{
    return ev.value(L, p[0], p[1], p[2], id, refills, live);
}
__device__ __forceinline__ float eval_at(EvalSkip3D &ev, const LaneField &L, const float *d, const float p[3],
                                         int &id, uint32_t &refills, bool live)
{
    return ev.value(L, d, p[0], p[1], p[2], id, refills, live);
}
// before a proposed crossing interval the cap is this by default (every skipped step is
// still certified; GPIS_TUNE_PROPOSED_SKIP_CAP sets it)
constexpr int kMaxSkipProposed = 32;

// Fast values farther than this from zero have the sign of the precise value
// (the fast evaluator differs from the precise one by a few 1e-8).
constexpr float kPreciseBand = 1e-6f;

// FlightArgs::work: the passes' fetch counters (fast 0, certified 1, precise 2),
// then the lengths of the two hand-off queues.
constexpr int kWorkQueueLen = 3;

// Appends v to a hand-off queue: one atomic per group of lanes that push together.
__device__ __forceinline__ void queue_push(uint32_t *q, uint32_t *len, uint32_t v)
{
    namespace cg = cooperative_groups;
    const cg::coalesced_group g = cg::coalesced_threads();
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(len, g.size());
    base = g.shfl(base, 0);
    q[base + g.thread_rank()] = v;
}

// Saved march state of a flight handed to the resume pass (phase 0: none); bit 26
// marks a crossing that the certified pass could not decide.
constexpr uint32_t kResumeNoCert = 1u << 26;
__device__ __forceinline__ uint4 pack_resume(float th, float tl, float pf, uint32_t steps, int sign0,
                                             bool pf_precise, int phase, bool no_cert = false)
{
    const uint32_t bits = (steps & 0xFFFFFFu) | (sign0 < 0 ? (1u << 24) : 0u) | (pf_precise ? (1u << 25) : 0u) |
                          (no_cert ? kResumeNoCert : 0u) | ((uint32_t)phase << 28);
    return make_uint4(__float_as_uint(th), __float_as_uint(tl), __float_as_uint(pf), bits);
}

__device__ __forceinline__ bool t_less(float hi, float lo, float far_t)
{
    return hi < far_t || (hi == far_t && lo < 0.0f);
}

// The march parameter after k steps, t0 + k step, straight from k: with t0 and step
// floats the exact sum is a multiple of q = min(ulp(t0), ulp(step)); while every t
// of the flight spans at most 45 bits above q, the product's two parts, their sum
// with t0 and the low parts' sum are all exact, so the result is the normalised
// float-float of the exact sum, which is what k sequential ff_add steps produce
// under the same condition (t_direct_ok).
__device__ __forceinline__ bool t_direct_ok(float t0, float step, float far_t)
{
    if (!(step > 0.0f) || !isfinite(t0) || !isfinite(far_t)) return false;
    const int top = ilogbf(fmaxf(fabsf(far_t), fabsf(t0)) + 4.0f * step);
    const int es = ilogbf(step);
    const int q = (t0 == 0.0f ? es : min(ilogbf(t0), es)) - 23;
    return top - q <= 44;
}

__device__ __forceinline__ void t_after(float t0, float step, uint32_t k, float &hi, float &lo)
{
    const float kf = (float)k;   // exact: k < 2^24
    const float p = __fmul_rn(kf, step);
    const float pe = __fmaf_rn(kf, step, -p);
    float e;
    const float s = two_sum(t0, p, e);
    const float l = __fadd_rn(e, pe);
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}

__device__ __forceinline__ unsigned long long warp_sum(uint32_t v)
{
    unsigned long long x = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    return x;
}

// ---------------------------------------------------------------------------
// k_march: persistent warps with per-lane refill.
// ---------------------------------------------------------------------------
// RESUME = false: the fast pass.  Lanes march with the fast evaluator only; a
// flight whose value comes within the band of zero or changes sign is saved to
// its resume record and left to the resume pass.
// RESUME = true: the resume pass over the saved flights, with precise decisions,
// the refinement and, after a rejected crossing candidate, the rest of the march.
// RESUME: the resume pass; with CERT the certified pass before it, which takes the
// saved crossings of the media cert_medium accepts, decides them on fast values
// where that is certain and hands the rest on (kResumeNoCert) to the precise pass,
// so that no warp runs both evaluators.
template <class Eval, bool RESUME, bool CERT = false>
__global__ void __launch_bounds__(256, Eval::kMinBlocks) k_march(FlightArgs a)
{
    static_assert(!CERT || RESUME, "the certified pass is a resume pass");
    const int lane = threadIdx.x & 31;
    uint32_t *work = a.work + (RESUME ? (CERT ? 1 : 2) : 0);
    const unsigned lt_mask = (1u << lane) - 1u;
    // 0.9 and 0.01 as float-float pairs (the reference's double constants)
    const FF kNine = {0.9f, -2.38418579e-08f};
    const float kHundredthH = 0.01f, kHundredthL = -2.23517418e-10f;
    __shared__ PcgJump s_jump[2 + 2 * 8];
    if (threadIdx.x < 2 + 2 * 8) s_jump[threadIdx.x] = c_jump[threadIdx.x];
    __syncthreads();
    Eval ev;
    ev.reset();
    ev.bind(s_jump);
    // the resume pass marches 3D flights on with the range-bounded evaluator
    EvalSkip3D ev3;
    ev3.reset();
    LaneField L;
    lane_field_idle(L, a.media);
    int phase = PH_IDLE;
    bool drained = false, first = true, pf_precise = false;
    uint32_t fid = 0, steps = 0, max_steps = 1, refine_iter = 0;
    float d[3] = {0, 0, 0}, near_t = 0, far_t = 0, step = 0, t0 = 0, th = 0, tl = 0, pf = 0, fb = 0;
    int sign0 = 1, gpid = 0;
    FF ta = {0, 0}, fac = {0, 0}, tprev = {0, 0}, ttest = {0, 0};
    uint32_t c_flights = 0, c_steps = 0, c_refine = 0, c_hits = 0, c_limit = 0, c_invalid = 0, c_refills = 0;
    uint32_t c_skipped = 0;
    // step skipping (fast pass): the field's Lipschitz constant along this ray and
    // its truncation-jump allowance, fixed and per step
    float skip_lip = -1.0f, skip_j0 = 0.0f, skip_j1 = 0.0f;
    bool t_direct = false;      // skipped steps jump to t0 + k step (t_direct_ok)
    float prop_a = -INFINITY;   // start of the proposed crossing interval (learned proposal)
    // certified pass: the bound on fac's distance from the reference's (cert_fac)
    float dfac = 0.0f;
    const int prop_cap = a.prop_cap ? (int)a.prop_cap : kMaxSkipProposed;
    // the flights this pass takes: every flight, or the queue the pass before filled
    const int q_in = RESUME && a.queue ? a.queue_in : 0;
    const uint32_t *queue_in = q_in ? a.queue + (size_t)(q_in - 1) * a.n : nullptr;
    const uint32_t n_live = q_in ? a.work[kWorkQueueLen + q_in - 1] : live_n(a);
    // the queue this pass hands its saved flights on to
    uint32_t *queue_out = a.queue ? a.queue + (CERT ? (size_t)a.n : 0) : nullptr;
    uint32_t *queue_len = a.work + kWorkQueueLen + (CERT ? 1 : 0);

    for (;;) {
        const bool need = phase == PH_IDLE && !drained;
        const unsigned need_mask = __ballot_sync(FULL, need);
        if (need_mask) {
            const int leader = __ffs(need_mask) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(work, (uint32_t)__popc(need_mask));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                const uint32_t item = base + (uint32_t)__popc(need_mask & lt_mask);
                if (item >= n_live) {
                    drained = true;
                } else {
                    const uint32_t idx = q_in ? queue_in[item] : item;
                    fid = idx;
                    if (!RESUME) c_flights++;
                    prop_a = (!RESUME && a.proposal) ? a.proposal[idx].x : -INFINITY;
                    bool mok;
                    L.m = medium_of(a, idx, mok);
                    const DevMedium &m = *L.m;
                    uint4 rs = make_uint4(0u, 0u, 0u, 0u);
                    if (RESUME) rs = a.resume[idx];
                    if (RESUME && (rs.w >> 28) == 0u) {
                        // finished by the fast pass
                    } else if (CERT && ((rs.w >> 28) != (uint32_t)PH_MARCH_P || (rs.w & kResumeNoCert) || !mok ||
                                        !cert_medium(m))) {
                        // left to the precise pass
                        if (queue_out) queue_push(queue_out, queue_len, idx);
                    } else if (Eval::kSkip && !RESUME && a.setup) {
                        // the set-up k_prepare computed for this flight
                        const float4 s0 = a.setup[4 * (size_t)idx], s1 = a.setup[4 * (size_t)idx + 1];
                        const float4 s2 = a.setup[4 * (size_t)idx + 2], s3 = a.setup[4 * (size_t)idx + 3];
                        const uint32_t flags = __float_as_uint(s3.y);
                        const float4 on = a.origin_near[idx], df = a.dir_far[idx];
                        if (!mok || !(flags & SF_VALID)) {
                            write_status(a, idx, 0.0f, 0.0f, 1.0f, 0u, GPIS_FLIGHT_INVALID_INPUT);
                            a.t_end[idx] = 0.0;
                            a.resume[idx] = make_uint4(0u, 0u, 0u, 0u);
                            c_invalid++;
                        } else {
#pragma unroll
                            for (int k = 0; k < 3; ++k) L.li[k] = m.l_inv[k];
                            L.o[0] = on.x; L.o[1] = on.y; L.o[2] = on.z;
                            d[0] = df.x; d[1] = df.y; d[2] = df.z;
                            near_t = on.w;
                            far_t = df.w;
                            first = (flags & SF_FIRST) != 0;
                            L.seed = __float_as_uint(s3.x);
                            L.sigma = m.sigma;
                            L.cond = (flags & SF_COND) != 0;
                            L.n[0] = s0.x; L.n[1] = s0.y; L.n[2] = s0.z;
                            L.ozc = s0.w;
                            L.vs = s1.x;
                            L.gsz = s1.y;
                            L.ns = false;
                            L.ls_o = 1.0f;
                            L.mean_kind = m.mean_kind;
#pragma unroll
                            for (int k = 0; k < 6; ++k) L.mq[k] = m.mean_params[k];
                            L.n_imp = m.n_imp;
                            L.kr = m.kr_iso;
                            L.kexp = m.kexp1d;
                            L.inv_norm = m.inv_norm1d;
                            step = s1.z;
                            t0 = s1.w;
                            skip_lip = s2.x;
                            skip_j0 = s2.y;
                            skip_j1 = s2.z;
                            max_steps = m.max_steps;
                            t_direct = t_direct_ok(t0, step, far_t);
                            th = near_t;
                            tl = 0.0f;
                            steps = 0;
                            ev.reset();
                            phase = PH_F0;
                        }
                    } else if (const FlightIn fl = load_flight(a, idx); !mok || !flight_valid(fl)) {
                        write_status(a, idx, 0.0f, 0.0f, 1.0f, 0u, GPIS_FLIGHT_INVALID_INPUT);
                        a.t_end[idx] = 0.0;
                        a.resume[idx] = make_uint4(0u, 0u, 0u, 0u);
                        c_invalid++;
                    } else {
#pragma unroll
                        for (int k = 0; k < 3; ++k) d[k] = fl.d[k];
                        near_t = fl.near_t;
                        far_t = fl.far_t;
                        first = (fl.flags & GPIS_FLAG_FIRST_SCATTER) != 0;
                        lane_field_setup<Eval::kGeneral>(L, m, fl, a.cond + idx);
                        step = __fdiv_rn(__fsub_rn(far_t, near_t), (float)m.min_step);
                        if (m.step_size < step) step = m.step_size;
                        t0 = __fadd_rn(near_t, __fmul_rn(step, fl.jitter));
                        max_steps = m.max_steps;
                        skip_lip = -1.0f;
                        if (Eval::kSkip && !RESUME)
                            skip_params(m, d, L.sigma, L.cond, L.vs, L.gsz, step, skip_lip, skip_j0, skip_j1);
                        t_direct = t_direct_ok(t0, step, far_t);
                        th = near_t;
                        tl = 0.0f;
                        steps = 0;
                        ev.reset();
                        phase = PH_F0;
                        if (RESUME) {
                            th = __uint_as_float(rs.x);
                            tl = __uint_as_float(rs.y);
                            pf = __uint_as_float(rs.z);
                            steps = rs.w & 0xFFFFFFu;
                            sign0 = (rs.w & (1u << 24)) ? -1 : 1;
                            pf_precise = (rs.w & (1u << 25)) != 0;
                            phase = (int)(rs.w >> 28);
                        }
                    }
                }
            }
        }
        const bool live = phase != PH_IDLE;
        if (!__any_sync(FULL, live)) {
            if (__all_sync(FULL, drained)) break;
            continue;
        }
        if (!Eval::kCollective && !live) continue;

        // evaluation point of this phase
        float eh = th, el = tl;
        if (phase == PH_REFINE || phase == PH_PF) { eh = ttest.h; el = ttest.l; }
        float p[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) p[k] = ff_point(L.o[k], d[k], eh, el);
        int id;
        // the value at farT of isotropic, nonstationary or multi-resolution 3D media
        // is the precise one too (their fast evaluator's normalisation and level
        // weights round differently)
        const bool decide = RESUME && (phase == PH_F0_P || phase == PH_MARCH_P || phase == PH_PF || phase == PH_REFINE);
        const bool cert_eval = CERT && decide;
        const bool precise = (!CERT && decide) ||
                             (std::is_same<Eval, EvalGeneric>::value && phase == PH_FAR && general_3d(*L.m));
        float margin = 0.0f;
        if constexpr (IsSkip3D<Eval>::value) {
            // a marching step of a 3D medium asks for the field's range over the next
            // steps: about half of |f| at the last step, and at least two steps
            if (!RESUME && phase == PH_MARCH) {
                const float len = fminf(0.5f * fabsf(pf), (float)kMaxSkip3D * step);
                ev.plan(len >= 2.0f * step ? len : 0.0f);
            }
        }
        bool use3 = false;
        if constexpr (RESUME) {
            const DevMedium &m3 = *L.m;
            use3 = !precise && phase == PH_MARCH && !(m3.flags & MF_ONE_D) && m3.n_oct == 1 && !general_3d(m3);
            if (use3) {
                const float len = fminf(0.5f * fabsf(pf), (float)kMaxSkip3D * step);
                ev3.plan(len >= 2.0f * step ? len : 0.0f);
            }
        }
        float f;
        if (CERT) {
            // every phase on the one evaluator (its value is EvalGeneric's), so that
            // the lanes of a warp never run two
            f = value_1d_cert(L, p[0], p[1], p[2], id, margin);
            c_refills += 3;
        } else {
            f = precise ? field_precise(L, p[0], p[1], p[2], id)
                        : (use3 ? ev3.value(L, d, p[0], p[1], p[2], id, c_refills, live)
                                : eval_at(ev, L, d, p, id, c_refills, live));
        }
        if (Eval::kCollective && !live) continue;
        gpid = id;
        const int sg = f < 0.0f ? -1 : 1;
        bool done = false;
        float t_out = 0.0f, v_out = 0.0f, trans = 1.0f;
        FF t_end = {0.0f, 0.0f};
        uint32_t status = GPIS_FLIGHT_OK;

        bool pend = false;
        // a certified decision that is not certain hands the crossing on to the
        // precise pass, from tb
        bool restart = false;
        if (cert_eval) {
            if (!isfinite(f)) {
                restart = true;
            } else if (phase == PH_MARCH_P) {
                restart = fabsf(f) < kPreciseBand;
            } else if (phase == PH_REFINE) {
                const float dt = step * dfac + 0x1p-44f * fabsf(ttest.h);
                restart = !cert_sign(*L.m, L, d, p, step, f, margin, dt, kPreciseBand);
                // the back-off comparison that follows a sign change
                if (!restart && sg != sign0) {
                    const FF nf = ff_mul(fac, kNine);
                    restart = fabsf(__fsub_rn(nf.h, kHundredthH)) <= 0.9f * dfac * 1.01f + 0x1p-40f;
                }
            }
        }
        if (CERT && restart) {
            // (t stays at tb through the refinement)
            if (phase != PH_MARCH_P) {
                steps--;
                c_steps--;
                pf_precise = false;
                phase = PH_MARCH_P;
            }
            pend = true;
        } else if (!isfinite(f)) {
            // a non-finite field value ends the flight (RaySegmentBatch.cu:228-229, 238-239)
            done = true;
            status = GPIS_FLIGHT_INVALID_INPUT;
            c_invalid++;
        } else if (phase == PH_F0 && first && fabsf(f) < kPreciseBand) {
            // the initial sign decides the crossing of a primary flight; a secondary
            // flight takes its sign from the first step instead
            phase = PH_F0_P;
            pend = !RESUME;
        } else if (phase == PH_F0 || phase == PH_F0_P) {
            sign0 = sg;
            pf = f;
            pf_precise = phase == PH_F0_P;
            th = t0;
            tl = 0.0f;
            if (t_less(th, tl, far_t)) {
                phase = PH_MARCH;
            } else {
                phase = PH_FAR;
                th = far_t;
            }
        } else if (phase == PH_MARCH && (fabsf(f) < kPreciseBand || (sg != sign0 && (first || steps != 0) && !CERT))) {
            // close to zero or a candidate crossing: decide on the precise value (a
            // certified resume lane decides a crossing on this value)
            phase = PH_MARCH_P;
            pend = !RESUME || CERT;
        } else if (phase == PH_MARCH || phase == PH_MARCH_P) {
            steps++;
            c_steps++;
            bool crossed = false;
            if (!first && steps == 1) {
                sign0 = sg;
            } else if (sg != sign0) {
                crossed = true;
            }
            if (crossed) {
                // tb = t, ta = t - step (exact); the back-off starts at the regula-falsi point
                ta = ff_add_f(ff_norm(th, tl), -step);
                fb = f;
                if (!pf_precise) {
                    // re-evaluate the previous value precisely first: it was taken at
                    // t - step, or at nearT for the first step (where the reference's
                    // interval [t - step, t] still starts at t - step)
                    ttest = steps == 1 ? FF{near_t, 0.0f} : ta;
                    phase = PH_PF;
                } else {
                    float e;
                    const float dh = two_sum(pf, -fb, e);
                    fac = ff_div_ff(pf, {dh, e});
                    ttest = ff_add(ta, ff_mul_f(fac, step));
                    tprev = ttest;
                    refine_iter = 0;
                    phase = PH_REFINE;
                    if (CERT && !cert_fac(pf, fb, kPreciseBand, dfac)) {
                        // too close to call: the precise pass, from tb
                        steps--;
                        c_steps--;
                        pf_precise = false;
                        phase = PH_MARCH_P;
                        pend = true;
                    }
                }
            } else {
                pf = f;
                pf_precise = phase == PH_MARCH_P;
                ff_add(th, tl, step);
                phase = PH_MARCH;
                // Step skipping: over the next k steps |f(t) - f| <= skip_lip |t - t_j| plus
                // the jump allowance, so while that stays below |f| (less a margin for the
                // fast value's error and the reference's float evaluation) every skipped
                // step has the sign of f and the reference would march past it.  Skipped
                // steps are counted as marched; the resume pass re-evaluates the step before
                // a crossing, so no skipped value is ever needed.
                int skip = 0;
                if (Eval::kSkip && !RESUME && skip_lip >= 0.0f) {
                    const float af = fabsf(f) * (1.0f - 1e-6f) - 1e-5f - skip_j0;
                    const float per = skip_lip * step + skip_j1;
                    // at most kMaxSkip per evaluation
                    const float cap = th < prop_a ? (float)prop_cap : (float)kMaxSkip;
                    if (af > per) skip = (int)fminf(af / per, cap);
                }
                if constexpr (IsSkip3D<Eval>::value) {
                    if (!RESUME) skip = ev.skips(f, step, kMaxSkip3D);
                }
                if constexpr (IsOct<Eval>::value) {
                    if (!RESUME)
                        skip = oct_skip_count(*L.m, L, d, ev.last_ls, f, step,
                                              th < prop_a ? max(IsOct<Eval>::cap, prop_cap) : IsOct<Eval>::cap);
                }
                if constexpr (RESUME) {
                    // a flight that marches on after a decision skips by the same slope bound
                    // (1D media) or range bound (3D media); the value before a later
                    // crossing is then no longer the last one evaluated, so the refinement
                    // re-evaluates it
                    if (L.m->flags & MF_ONE_D)
                        skip = oct_skip_count(*L.m, L, d, ns_scale(*L.m, p[0], p[2]), f, step, kMaxSkip);
                    else if (use3)
                        skip = ev3.skips(f, step, kMaxSkip3D);
                    if (skip > 0) pf_precise = false;
                }
                if (t_direct && skip > 0 && steps + (uint32_t)skip < max_steps) {
                    // the skipped steps in one jump when it stays before farT (else step by step)
                    float nh, nl;
                    t_after(t0, step, steps + (uint32_t)skip, nh, nl);
                    if (t_less(nh, nl, far_t)) {
                        th = nh;
                        tl = nl;
                        steps += (uint32_t)skip;
                        c_steps += (uint32_t)skip;
                        c_skipped += (uint32_t)skip;
                        skip = 0;
                    }
                }
                for (;;) {
                    if (!t_less(th, tl, far_t)) {
                        phase = PH_FAR;
                        th = far_t;
                        tl = 0.0f;
                        break;
                    }
                    if (steps >= max_steps) {
                        done = true;
                        status = GPIS_FLIGHT_STEP_LIMIT;
                        t_out = far_t;
                        t_end = {far_t, 0.0f};
                        c_limit++;
                        break;
                    }
                    if (skip == 0) break;
                    skip--;
                    steps++;
                    c_steps++;
                    c_skipped++;
                    ff_add(th, tl, step);
                }
            }
        } else if (phase == PH_PF) {
            // f: precise (or certified fast) value at the previous point; fb: the same at tb
            pf = f;
            float e;
            const float dh = two_sum(pf, -fb, e);
            fac = ff_div_ff(pf, {dh, e});
            ttest = ff_add(ta, ff_mul_f(fac, step));
            tprev = ttest;
            refine_iter = 0;
            phase = PH_REFINE;
            if (CERT && !cert_fac(pf, fb, kPreciseBand, dfac)) {
                steps--;
                c_steps--;
                pf_precise = false;
                phase = PH_MARCH_P;
                pend = true;
            }
        } else if (phase == PH_REFINE) {
            c_refine++;
            refine_iter++;
            bool hit = false;
            if (sg == sign0) {
                hit = true;
            } else {
                fac = ff_mul(fac, kNine);
                if (CERT) dfac *= 0.9f * 1.0001f;
                // 0.9^44 < 0.01: the back-off ends within 44 evaluations for any
                // factor <= 1; the explicit bound also covers a non-finite factor.
                if (ff_le(fac, kHundredthH, kHundredthL) || !(fac.h == fac.h) || refine_iter >= 64) {
                    tprev = {0.0f, 0.0f};
                    hit = true;
                } else {
                    tprev = ttest;
                    ttest = ff_add(ta, ff_mul_f(fac, step));
                }
            }
            if (hit) {
                done = true;
                t_end = tprev;
                t_out = __fadd_rn(tprev.h, tprev.l);
                v_out = 0.0f;
                trans = 0.0f;
                c_hits++;
            }
        } else {  // PH_FAR
            done = true;
            t_out = far_t;
            t_end = {far_t, 0.0f};
            v_out = f;
        }
        if (pend) {
            // (a value the certified pass took is never a precise one)
            a.resume[fid] = pack_resume(th, tl, pf, steps, sign0, pf_precise && !CERT, phase, CERT);
            if (queue_out) queue_push(queue_out, queue_len, fid);
            phase = PH_IDLE;
        } else if (done) {
            write_status(a, fid, t_out, v_out, trans, steps, status | ((uint32_t)gpid << 8));
            a.t_end[fid] = (double)t_end.h + (double)t_end.l;
            if (!RESUME || CERT) a.resume[fid] = make_uint4(0u, 0u, 0u, 0u);
            phase = PH_IDLE;
        }
    }
    // counters: one atomic per warp
    const unsigned long long s0 = warp_sum(c_flights), s1 = warp_sum(c_steps), s2 = warp_sum(c_refine),
                             s3 = warp_sum(c_hits), s4 = warp_sum(c_limit), s5 = warp_sum(c_invalid),
                             s6 = warp_sum(c_refills), s7 = warp_sum(c_skipped);
    if (lane == 0 && a.counters) {
        atomicAdd(a.counters + 0, s0);
        atomicAdd(a.counters + 1, s1);
        atomicAdd(a.counters + 2, s2);
        atomicAdd(a.counters + 3, s3);
        atomicAdd(a.counters + 4, s4);
        atomicAdd(a.counters + 5, s5);
        atomicAdd(a.counters + 6, s6);
        atomicAdd(a.counters + 7, s7);
    }
}

// ---------------------------------------------------------------------------
// k_finish: gradient sample at the end point.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void finish_one(const FlightArgs &a, uint32_t i)
{
    float4 r0 = a.out[2 * i];
    float4 r1 = a.out[2 * i + 1];
    const uint32_t status = __float_as_uint(r1.w) & 0xFFu;
    bool mok;
    const DevMedium &m = *medium_of(a, i, mok);
    const FlightIn fl = load_flight(a, i);
    const bool hit = r1.y == 0.0f;
    const bool shadow = (fl.flags & GPIS_FLAG_SHADOW) != 0;
    if (status != GPIS_FLIGHT_OK || (!hit && shadow) || !mok) {
        const bool keep = status != GPIS_FLIGHT_INVALID_INPUT;
        r0.z = keep ? fl.prev_g[0] : 0.0f;
        r0.w = keep ? fl.prev_g[1] : 0.0f;
        r1.x = keep ? fl.prev_g[2] : 0.0f;
        a.out[2 * i] = r0;
        a.out[2 * i + 1] = r1;
        return;
    }
    const double t = a.t_end[i];
    // ro + normalize(rd) * t in double, rounded to float (GaussianProcessMedium.cpp:307,
    // 401), carried in float-float: the squared length of rd is exact, its reciprocal
    // square root good to about 43 bits, and t splits exactly into two floats
    const float th = __double2float_rn(t);
    const FF tt = {th, __double2float_rn(t - (double)th)};
    const FF inv = ff_rsqrt(ff_add(ff_add(ff_prod(fl.d[0], fl.d[0]), ff_prod(fl.d[1], fl.d[1])),
                                   ff_prod(fl.d[2], fl.d[2])));
    float p[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const FF q = ff_add_f(ff_mul(ff_mul_f(inv, fl.d[j]), tt), fl.o[j]);
        p[j] = __fadd_rn(q.h, q.l);
    }
    const bool cond = conditioned(m, fl);
    CondRec c = {};
    if (cond) c = a.cond[i];
    // evaluateGradient (SparseConvolutionNoise.cpp:133-140): sum of the octaves'
    // amplitude-weighted noise gradients plus the mean gradient
    float gs[3] = {0.0f, 0.0f, 0.0f}, mg[3];
    const int n_oct = (m.flags & MF_ONE_D) ? (int)m.n_oct : 1;
    for (int k = 0; k < n_oct; ++k) {
        float v, g[3];
        noise_gradient_oct(m, fl, c, cond, p, (float)t, k, v, g);
        const float amp = oct_sigma(m, k);
#pragma unroll
        for (int j = 0; j < 3; ++j) gs[j] = __fadd_rn(gs[j], __fmul_rn(amp, g[j]));
    }
    mean_grad(m, p[0], p[1], p[2], mg);
    r0.z = __fadd_rn(gs[0], mg[0]);
    r0.w = __fadd_rn(gs[1], mg[1]);
    r1.x = __fadd_rn(gs[2], mg[2]);
    a.out[2 * i] = r0;
    a.out[2 * i + 1] = r1;
}

// MINB blocks of 128 per SM: 8 for batches of 1D media (0.62 against 0.79 ms per bench
// step at 128 registers), 4 when 3D media are present
template <int MINB>
__global__ void __launch_bounds__(128, MINB) k_finish(FlightArgs a)
{
    const uint32_t n = live_n(a);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) finish_one(a, i);
}

// ---------------------------------------------------------------------------
// Unit-level kernels.
// ---------------------------------------------------------------------------
// cr_expf at n arguments (its check against the correctly rounded exponential)
__global__ void k_debug_exp(const float *x, float *y, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = cr_expf(x[i]);
}

__global__ void k_debug_cells_1d(const uint32_t *cells, const uint32_t *seeds, uint32_t n,
                                 uint32_t imp, float *pos, float *weight)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s = xxhash2(cells[i], seeds[i]) + 1u;
    for (uint32_t k = 0; k < imp; ++k) {
        pos[(size_t)i * imp + k] = unit_float(pcg_draw(c_jump[2 + 2 * k], s));
        weight[(size_t)i * imp + k] = (pcg_draw(c_jump[3 + 2 * k], s) >> 31) ? 1.0f : -1.0f;
    }
}

__global__ void k_debug_cells_3d(const int32_t *cells, const uint32_t *seeds, uint32_t n, uint32_t imp,
                                 uint32_t order, float *pos, float *weight)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s = xxhash4((uint32_t)cells[3 * i + 2], (uint32_t)cells[3 * i + 1], (uint32_t)cells[3 * i],
                               seeds[i]) + 1u;
    for (uint32_t k = 0; k < imp; ++k) {
        const int b = 2 + 4 * (int)k;
        const float r0 = unit_float(pcg_draw(c_jump[b], s));
        const float r1 = unit_float(pcg_draw(c_jump[b + 1], s));
        const float r2 = unit_float(pcg_draw(c_jump[b + 2], s));
        const size_t o = ((size_t)i * imp + k) * 3;
        pos[o + 0] = order ? r0 : r2;
        pos[o + 1] = r1;
        pos[o + 2] = order ? r2 : r0;
        weight[(size_t)i * imp + k] = (pcg_draw(c_jump[b + 3], s) >> 31) ? 1.0f : -1.0f;
    }
}

// Field at arbitrary points: conditioning of the point's flight (as k_prepare),
// then the noise value/gradient and the field value.
__global__ void k_debug_field(const DevMedium *mp, const float4 *origins, const float4 *points,
                              const float4 *dirs, const uint4 *seeds, const float4 *prev,
                              uint32_t n, float4 *out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevMedium &m = *mp;
    FlightIn fl;
    const float4 o = origins[i], d = dirs[i], pp = points[i], pv = prev[i];
    const uint4 sd = seeds[i];
    fl.o[0] = o.x; fl.o[1] = o.y; fl.o[2] = o.z; fl.near_t = 0.0f;
    fl.d[0] = d.x; fl.d[1] = d.y; fl.d[2] = d.z; fl.far_t = 1.0f;
    fl.noise_seed = sd.x; fl.normal_seed = sd.y; fl.flags = sd.z; fl.jitter = 0.0f;
    fl.prev_v = pv.x; fl.prev_g[0] = pv.y; fl.prev_g[1] = pv.z; fl.prev_g[2] = pv.w;
    const bool cond = conditioned(m, fl);
    const CondRec c = cond ? make_condition(m, fl) : CondRec{};
    const float p[3] = {pp.x, pp.y, pp.z};
    float v = 0.0f, g[3] = {0.0f, 0.0f, 0.0f}, fv_noise;
    // value and derivative parts of the noise (the 1D xy entries are the
    // conditioning splats); several octaves report amplitude-weighted sums
    if ((m.flags & MF_MULTIRES) && (m.flags & MF_ONE_D)) {
        Frame f;
        ray_frame(m, fl.d[0], fl.d[1], fl.d[2], f);
        const MrLevels lv = mr_levels(m, ls_value_precise(m, p[0], p[2]));
        float ow[2] = {1.0f, 1.0f};
        if (cond) {
            const MrLevels lo = mr_levels(m, ls_value_precise(m, fl.o[0], fl.o[2]));
            ow[0] = lo.w[0];
            ow[1] = lo.w[1];
        }
        for (int j = 0; j < 2; ++j) {
            float vk, dv, gx, gy;
            noise1d_level(m, fl, c.oct[0], cond, f, p, lv.s[j], lv.seed[j], ow[j], vk, dv, gx, gy);
            v += lv.w[j] * vk;
            g[0] += lv.w[j] * gx;
            g[1] += lv.w[j] * gy;
            g[2] += lv.w[j] * dv;
        }
        fv_noise = m.sigma * v;
    } else if (m.flags & MF_ONE_D) {
        Frame f;
        ray_frame(m, fl.d[0], fl.d[1], fl.d[2], f);
        const float ls = ns_scale(m, p[0], p[2]);
        const float a = splat_cov_1d(ls, ns_scale(m, fl.o[0], fl.o[2]));
        for (int k = 0; k < (int)m.n_oct; ++k) {
            const float sc = oct_scale(m, k);
            const float z = ray_coord_oct(m, f.n, p[0], p[1], p[2], sc);
            float vk, dv;
            noise1d_generic<true>(m, z, fl.noise_seed + oct_seed(m, k), vk, dv, ls);
            const float inrm = inv_norm_1d(m, ls);
            vk *= inrm;
            dv *= inrm;
            float gx = 0.0f, gy = 0.0f;
            if (cond) {
                const CondOct &co = c.oct[k];
                const float oz = ray_coord_oct(m, f.n, fl.o[0], fl.o[1], fl.o[2], sc);
                const Cov1D kk = cov1d(z - oz, a);
                vk += co.vs * kk.k0 + (sc * co.gs[2]) * kk.k1;
                dv += co.vs * kk.k1 + (sc * co.gs[2]) * kk.k2;
                if (m.flags & MF_CORR_XY) { gx = (sc * co.gs[0]) * kk.k3; gy = (sc * co.gs[1]) * kk.k3; }
            }
            const float w = m.n_oct == 1 ? 1.0f : oct_sigma(m, k);
            v += w * vk;
            g[0] += w * gx;
            g[1] += w * gy;
            g[2] += w * dv;
        }
        fv_noise = m.n_oct == 1 ? m.sigma * v : v;
    } else {
        noise_gradient(m, fl, c, cond, p, 1.0f, v, g);
        fv_noise = m.sigma * v;
    }
    int id;
    const float mean = mean_value(m, p[0], p[1], p[2], id);
    // the march's precise evaluator at p (the value its decisions near zero use)
    LaneField L;
    lane_field_idle(L, &m);
    lane_field_setup(L, m, fl, &c);
    int pid;
    const float fp = field_precise(L, p[0], p[1], p[2], pid);
    out[2 * i] = make_float4(v, g[0], g[1], g[2]);
    out[2 * i + 1] = make_float4(fv_noise + mean, mean, fp, __int_as_float(pid));
}

// ---------------------------------------------------------------------------
// k_nee: 1D specular next-event estimation on the realization of a flight
// (neeShared / neeGrad / neePDF, SparseConvolutionNoise.cpp:662-821): the
// gradient plane of the ray's 1D derivative, the gradient that makes the world
// normal, and the solid-angle PDF of drawing it.  One thread per query; the
// realization's conditioning is rebuilt from the flight as k_prepare does.
// out = {pdf, gradient}; NaN pdf for media without 1D single-octave noise or
// non-finite inputs.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void inv3(const float A[9], float R[9])
{
    const float c00 = A[4] * A[8] - A[5] * A[7];
    const float c01 = A[5] * A[6] - A[3] * A[8];
    const float c02 = A[3] * A[7] - A[4] * A[6];
    const float id = 1.0f / (A[0] * c00 + A[1] * c01 + A[2] * c02);
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

// NEE for a field of several octaves (no reference form: the reference's NEE is for
// one realization).  Octave k contributes c_k (x_k, y_k, dv_k) in the common iso-ray
// frame, c_k = amplitude / length multiplier, with independent transverse draws of the
// law its gradient sample uses (noise_gradient_oct): N(base_k, 1 / (2 scx^2)) per
// component, or under Renewal+ with correlationXY away from the origin
// N(base_k + 2 fac x1_k, cov).  The summed transverse gradient is Gaussian with mean
// sum c_k m_k and variance v sum c_k^2; the along-ray component is Z = sum c_k dv_k.
// In double; returns {pdf, gradient}.
__device__ float4 nee_octaves(const DevMedium &m, const FlightIn &fl, const CondRec &c, bool cond, const Frame &f,
                              const float p[3], const float nw[3], float t_seg, const float mg[3])
{
    double A[9];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const double li = m.ls_kind ? (double)m.l_inv[r] / m.ls_max : (double)m.l_inv[r];
        A[3 * r + 0] = li * f.t[r];
        A[3 * r + 1] = li * f.b[r];
        A[3 * r + 2] = li * f.n[r];
    }
    const bool corr = (m.flags & MF_RENEWAL_PLUS) && (m.flags & MF_CORR_XY) && t_seg != 0.0f;
    float facf = 0.0f, covf = 0.0f;
    if (corr) corr_moments(t_seg, facf, covf);
    const float ls = ns_scale_precise(m, p[0], p[2]);
    const double scx = splat_cov_1d(ls, ls);
    const double v1 = corr ? (double)covf : 1.0 / (2.0 * scx * scx);
    double Z = 0.0, MX = 0.0, MY = 0.0, S2 = 0.0;
    const float ls_o = cond ? ns_scale_precise(m, fl.o[0], fl.o[2]) : 1.0f;
    for (int k = 0; k < (int)m.n_oct; ++k) {
        const float sc = oct_scale(m, k);
        const float z = ray_coord_oct(m, f.n, p[0], p[1], p[2], sc);
        float v, dv;
        noise1d_generic<true>(m, z, fl.noise_seed + oct_seed(m, k), v, dv, ls);
        dv *= inv_norm_1d(m, ls);
        double bx = 0.0, by = 0.0;
        if (cond) {
            const CondOct &co = c.oct[k];
            const float oz = ray_coord_oct(m, f.n, fl.o[0], fl.o[1], fl.o[2], sc);
            const Cov1D kk = cov1d(z - oz, splat_cov_1d(ls, ls_o));
            dv += co.vs * kk.k1 + (sc * co.gs[2]) * kk.k2;
            if (m.flags & MF_CORR_XY) {
                bx = (sc * co.gs[0]) * kk.k3;
                by = (sc * co.gs[1]) * kk.k3;
            }
        }
        if (corr) {
            float z0, z1;
            normal_draws(oct_normal_seed(m, fl.normal_seed, k), 0, z0, z1);
            bx += (double)facf * 2.0 * ((double)z0 / 1.41421354);
            by += (double)facf * 2.0 * ((double)z1 / 1.41421354);
        }
        const double ck = (double)oct_sigma(m, k) / sc;
        Z += ck * dv;
        MX += ck * bx;
        MY += ck * by;
        S2 += ck * ck;
    }
    const double V = v1 * S2;
    const double ax[3] = {A[0], A[3], A[6]}, ay[3] = {A[1], A[4], A[7]};
    double ppt[3], cr[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) ppt[r] = A[3 * r + 2] * Z + mg[r];
    cr[0] = ax[1] * ay[2] - ax[2] * ay[1];
    cr[1] = ax[2] * ay[0] - ax[0] * ay[2];
    cr[2] = ax[0] * ay[1] - ax[1] * ay[0];
    const double jac = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    const double pn[3] = {cr[0] / jac, cr[1] / jac, cr[2] / jac};
    const double npn = nw[0] * pn[0] + nw[1] * pn[1] + nw[2] * pn[2];
    const double isect = (ppt[0] * pn[0] + ppt[1] * pn[1] + ppt[2] * pn[2]) / npn;
    const float g0 = (float)(isect * nw[0]), g1 = (float)(isect * nw[1]), g2 = (float)(isect * nw[2]);
    if (!(isect >= 0.0) || !(V > 0.0)) return make_float4(0.0f, g0, g1, g2);
    const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
    const double id = 1.0 / (A[0] * c00 + A[1] * c01 + A[2] * c02);
    const double i0 = c00 * id, i1 = (A[2] * A[7] - A[1] * A[8]) * id, i2 = (A[1] * A[5] - A[2] * A[4]) * id;
    const double i3 = c01 * id, i4 = (A[0] * A[8] - A[2] * A[6]) * id, i5 = (A[2] * A[3] - A[0] * A[5]) * id;
    const double gw0 = isect * nw[0] - mg[0], gw1 = isect * nw[1] - mg[1], gw2 = isect * nw[2] - mg[2];
    const double X = i0 * gw0 + i1 * gw1 + i2 * gw2;
    const double Y = i3 * gw0 + i4 * gw1 + i5 * gw2;
    const double dx = X - MX, dy = Y - MY;
    const double pdf_area = exp(-0.5 * (dx * dx + dy * dy) / V) / (6.283185307179586 * V);
    const double pdf_n = pdf_area * isect * isect / fabs(npn) / jac;
    const double ndr = -((double)nw[0] * fl.d[0] + (double)nw[1] * fl.d[1] + (double)nw[2] * fl.d[2]);
    return make_float4((float)(pdf_n / (4.0 * ndr)), g0, g1, g2);
}

__device__ __forceinline__ void nee_one(const FlightArgs &a, const float4 *point_t, const float4 *normal, float4 *out,
                                        uint32_t i)
{
    bool mok;
    const DevMedium &m = *medium_of(a, i, mok);
    FlightIn fl = load_flight(a, i);
    const float4 q = point_t[i], nv = normal[i];
    const float p[3] = {q.x, q.y, q.z}, nw[3] = {nv.x, nv.y, nv.z};
    const float t_seg = q.w;
    bool ok = mok && (m.flags & MF_ONE_D) && isfinite(t_seg);
#pragma unroll
    for (int k = 0; k < 3; ++k)
        ok = ok && isfinite(fl.o[k]) && isfinite(fl.d[k]) && isfinite(p[k]) && isfinite(nw[k]);
    const bool cond = conditioned(m, fl);
    if (cond) ok = ok && isfinite(fl.prev_v) && isfinite(fl.prev_g[0]) && isfinite(fl.prev_g[1]) && isfinite(fl.prev_g[2]);
    if (!ok) {
        out[i] = make_float4(__int_as_float(0x7fffffff), 0.0f, 0.0f, 0.0f);
        return;
    }
    const CondRec c = cond ? make_condition(m, fl) : CondRec{};
    const float amp = m.sigma;
    float mg[3];
    mean_grad(m, p[0], p[1], p[2], mg);
    Frame f;
    ray_frame(m, fl.d[0], fl.d[1], fl.d[2], f);
    if (m.n_oct > 1) {
        out[i] = nee_octaves(m, fl, c, cond, f, p, nw, t_seg, mg);
        return;
    }
    // mtx_pt = amplitude * localToWorldInvTransposeMatrix(p) * [t b n]
    float A[9], Ai[9];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float li = m.ls_kind ? __fdiv_rn(m.l_inv[r], m.ls_max) : m.l_inv[r];
        const float al = __fmul_rn(amp, li);
        A[3 * r + 0] = __fmul_rn(al, f.t[r]);
        A[3 * r + 1] = __fmul_rn(al, f.b[r]);
        A[3 * r + 2] = __fmul_rn(al, f.n[r]);
    }
    inv3(A, Ai);
    // grad_constraint_3d: the conditioned 1D noise's splat parts at p
    const float ls = ns_scale_precise(m, p[0], p[2]);
    const float z = ray_coord_oct(m, f.n, p[0], p[1], p[2], 1.0f);
    float v, dv;
    float gc[3] = {0.0f, 0.0f, 0.0f};
    const bool mr = (m.flags & MF_MULTIRES) != 0;
    MrLevels lv = {};
    if (mr) {
        // the levels' parts, each weighted by w / s (SparseConvolutionNoise.cpp:687-692)
        lv = mr_levels(m, ls_value_precise(m, p[0], p[2]));
        float ow[2] = {1.0f, 1.0f};
        if (cond) {
            const MrLevels lo = mr_levels(m, ls_value_precise(m, fl.o[0], fl.o[2]));
            ow[0] = lo.w[0];
            ow[1] = lo.w[1];
        }
        for (int j = 0; j < 2; ++j) {
            float gx, gy;
            noise1d_level(m, fl, c.oct[0], cond, f, p, lv.s[j], lv.seed[j], ow[j], v, dv, gx, gy);
            gc[0] += gx * lv.w[j] / lv.s[j];
            gc[1] += gy * lv.w[j] / lv.s[j];
            gc[2] += dv * lv.w[j] / lv.s[j];
        }
    } else {
    noise1d_generic<true>(m, z, fl.noise_seed, v, dv, ls);
    const float inrm = inv_norm_1d(m, ls);
    dv *= inrm;
    if (cond) {
        const CondOct &co = c.oct[0];
        const float oz = ray_coord_oct(m, f.n, fl.o[0], fl.o[1], fl.o[2], 1.0f);
        const Cov1D kk = cov1d(z - oz, splat_cov_1d(ls, ns_scale_precise(m, fl.o[0], fl.o[2])));
        dv += co.vs * kk.k1 + co.gs[2] * kk.k2;
        if (m.flags & MF_CORR_XY) {
            gc[0] = co.gs[0] * kk.k3;
            gc[1] = co.gs[1] * kk.k3;
        }
    }
    gc[2] = dv;
    }
    // the gradient plane and the gradient that points along the normal
    float ppt[3], px[3], py[3], cr[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        ppt[r] = A[3 * r + 2] * gc[2] + mg[r];
        px[r] = A[3 * r + 0];
        py[r] = A[3 * r + 1];
    }
    cr[0] = px[1] * py[2] - px[2] * py[1];
    cr[1] = px[2] * py[0] - px[0] * py[2];
    cr[2] = px[0] * py[1] - px[1] * py[0];
    const float jac = sqrtf(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    const float pn[3] = {cr[0] / jac, cr[1] / jac, cr[2] / jac};
    const float npn = nw[0] * pn[0] + nw[1] * pn[1] + nw[2] * pn[2];
    const float isect = (ppt[0] * pn[0] + ppt[1] * pn[1] + ppt[2] * pn[2]) / npn;
    float g[3], gw[3], g3[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        g[r] = isect * nw[r];
        gw[r] = g[r] - mg[r];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) g3[r] = Ai[3 * r + 0] * gw[0] + Ai[3 * r + 1] * gw[1] + Ai[3 * r + 2] * gw[2];
    float pdf = 0.0f;
    if (!(isect < 0.0f)) {
        const double two_pi = 6.283185307179586;
        double pdf_area;
        const uint32_t nseed = fl.normal_seed;
        if (m.flags & MF_TRANSVERSE) {
            float m0, m1, var;
            transverse_moments(m, c, fl.o, p, f, cond, m0, m1, var);
            if (!(var > 0.0f)) {
                pdf_area = -1.0;
            } else {
                const double dx = (double)g3[0] - m0, dy = (double)g3[1] - m1;
                pdf_area = exp(-0.5 * (dx * dx + dy * dy) / var) / (two_pi * var);
            }
        } else if (mr) {
            // the multi-resolution law (SparseConvolutionNoise.cpp:776-808): transverse
            // scales times 1 / sqrt((w_low / s_low)^2 + (w_high / s_high)^2)
            const float a0 = lv.w[0] / lv.s[0], a1 = lv.w[1] / lv.s[1];
            const float nss = (float)(1.0 / (double)sqrtf(a0 * a0 + a1 * a1));
            if (!((m.flags & MF_RENEWAL_PLUS) && (m.flags & MF_CORR_XY)) || t_seg == 0.0f) {
                const float sx = (float)((double)(g3[0] - gc[0]) * 1.4142135623730951 * nss);
                const float sy = (float)((double)(g3[1] - gc[1]) * 1.4142135623730951 * nss);
                pdf_area = exp(-(double)(sx * sx) / 2.0) * exp(-(double)(sy * sy) / 2.0) / two_pi * 2.0 * nss * nss;
            } else {
                float z0, z1, z2, z3, fac, cv;
                normal_draws(nseed, 0, z0, z1);
                normal_draws(nseed, 1, z2, z3);
                corr_moments(t_seg, fac, cv);
                const double s2 = 1.41421354;
                const double mx = fac * 2.0 * ((double)z0 / s2 * lv.w[0] / lv.s[0] + (double)z2 / s2 * lv.w[1] / lv.s[1]);
                const double my = fac * 2.0 * ((double)z1 / s2 * lv.w[0] / lv.s[0] + (double)z3 / s2 * lv.w[1] / lv.s[1]);
                const double sq = sqrt((double)cv);
                const float sx = (float)(((double)(g3[0] - gc[0]) - mx) / sq * nss);
                const float sy = (float)(((double)(g3[1] - gc[1]) - my) / sq * nss);
                pdf_area = exp(-(double)(sx * sx) / 2.0) * exp(-(double)(sy * sy) / 2.0) / (two_pi * cv) * (double)(nss * nss);
            }
        } else if (!((m.flags & MF_RENEWAL_PLUS) && (m.flags & MF_CORR_XY)) || t_seg == 0.0f) {
            const float sc = splat_cov_1d(ls, ls);
            const float sx = (float)((double)(g3[0] - gc[0]) * 1.4142135623730951 * sc);
            const float sy = (float)((double)(g3[1] - gc[1]) * 1.4142135623730951 * sc);
            pdf_area = exp(-(double)(sx * sx) / 2.0) * exp(-(double)(sy * sy) / 2.0) / two_pi * 2.0 * sc * sc;
        } else {
            float z0, z1, fac, cv;
            normal_draws(nseed, 0, z0, z1);
            corr_moments(t_seg, fac, cv);
            const double s2 = 1.41421354;
            const double x1 = z0 / s2, y1 = z1 / s2;
            const double sq = sqrt((double)cv);
            const float sx = (float)(((double)(g3[0] - gc[0]) - fac * 2.0 * x1) / sq);
            const float sy = (float)(((double)(g3[1] - gc[1]) - fac * 2.0 * y1) / sq);
            pdf_area = exp(-(double)(sx * sx) / 2.0) * exp(-(double)(sy * sy) / 2.0) / two_pi / cv;
        }
        if (pdf_area >= 0.0) {
            const float cos_l = fabsf(npn);
            const float pdf_n = (float)pdf_area * (isect * isect) / cos_l / jac;
            const float ndr = -(nw[0] * fl.d[0] + nw[1] * fl.d[1] + nw[2] * fl.d[2]);
            pdf = (float)(pdf_n / (4.0 * ndr));
        }
    }
    out[i] = make_float4(pdf, g[0], g[1], g[2]);
}

__global__ void __launch_bounds__(128) k_nee(FlightArgs a, const float4 *point_t, const float4 *normal, float4 *out)
{
    const uint32_t n = live_n(a);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        nee_one(a, point_t, normal, out, i);
}

// Corner table of a grid mean: cell c holds the 8 clamped corner voxels that
// grid_fetch would load for any point whose trilinear cell is c.
__global__ void k_pack_grid(DevMedium m, float4 *cells, size_t n)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int cx = m.cell_lo[0] + (int)(i % (size_t)m.cell_n[0]);
    const int cy = m.cell_lo[1] + (int)((i / (size_t)m.cell_n[0]) % (size_t)m.cell_n[1]);
    const int cz = m.cell_lo[2] + (int)(i / ((size_t)m.cell_n[0] * (size_t)m.cell_n[1]));
    float v[8];
#pragma unroll
    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            v[4 * dz + 2 * dy + 0] = grid_voxel(m, cx, cy + dy, cz + dz);
            v[4 * dz + 2 * dy + 1] = grid_voxel(m, cx + 1, cy + dy, cz + dz);
        }
    cells[2 * i] = make_float4(v[0], v[1], v[2], v[3]);
    cells[2 * i + 1] = make_float4(v[4], v[5], v[6], v[7]);
}

__global__ void k_se_splat_1d(const float *q, const float *c, float *v, float *d, size_t n, float scale)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float delta = q[i] - c[i];
    const float inv = 1.0f / (scale * scale);
    const float e = expf(-0.5f * delta * delta * inv);
    v[i] = e;
    d[i] = -delta * inv * e;
}

}  // namespace

cudaError_t launch_flights(const FlightArgs &a, int num_sms, cudaStream_t stream, cudaEvent_t *ev)
{
    if (a.n == 0) return cudaSuccess;
    // one thread per flight; with a live count in device memory, grid-stride over a
    // grid of at most 16 blocks per SM
    uint32_t blocks = (a.n + 127) / 128;
    if (a.n_dev) blocks = std::min<uint32_t>(blocks, (uint32_t)num_sms * 16u);
    if (ev) cudaEventRecord(ev[0], stream);
    // the stationary cooperative fast pass takes its per-flight set-up from k_prepare
    const bool coop_plain = a.one_d && a.max_imp <= 8 && a.max_oct == 1 && !a.any_ns && !a.all_grid && !a.any_mr;
    FlightArgs b = a;
    if (!coop_plain) b.setup = nullptr;     // the march kernels read set-up records only when written
    // hand-off queues only with the certified pass: a precise pass that takes a queue
    // loads its flights in the order they were saved, scattered, and measured slower
    // than one that scans every resume record in flight order (the uneven image batch
    // 512 against 496 ms)
    const bool certify = coop_plain && !a.precise_only;
    if (!certify) b.queue = nullptr;
    if (b.any_cond || b.setup) {
        if (a.one_d) k_prepare<8><<<blocks, 128, 0, stream>>>(b);
        else k_prepare<4><<<blocks, 128, 0, stream>>>(b);
    }
    if (ev) cudaEventRecord(ev[1], stream);
    cudaError_t err = cudaMemsetAsync(b.work, 0, kWorkCounters * sizeof(uint32_t), stream);
    if (err != cudaSuccess) return err;
    // persistent grids: exactly the CTAs that are resident at once, never more
    // warps than flights
    const uint32_t warps_needed = (a.n + 31) / 32;
    const uint32_t ctas_needed = (warps_needed + 7) / 8;
    auto grid = [&](const void *fn, size_t smem = 0, bool tuned = true) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        // the schedule's CTAs per SM (never more than are resident at once)
        if (tuned && a.ctas_per_sm > 0 && (int)a.ctas_per_sm < per_sm) per_sm = (int)a.ctas_per_sm;
        uint32_t c = (uint32_t)num_sms * (uint32_t)per_sm;
        if (c > ctas_needed) c = ctas_needed;
        return c == 0 ? 1u : c;
    };
    if (ev) cudaEventRecord(ev[2], stream);
    // multi-resolution media take the generic evaluator (two levels per evaluation)
    const bool coop = a.one_d && a.max_imp <= 8 && a.max_oct == 1 && !a.any_mr;
    if (a.any_mr) {
        const void *fn = (const void *)k_march<EvalGeneric, false>;
        k_march<EvalGeneric, false><<<grid(fn), 256, 0, stream>>>(b);
    } else if (a.one_d && a.max_imp <= 8 && a.max_oct > 1) {
        const void *fn = (const void *)k_march<EvalCoopOct, false>;
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemOct);
        if (e != cudaSuccess) return e;
        k_march<EvalCoopOct, false><<<grid(fn, kSmemOct), 256, kSmemOct, stream>>>(b);
    } else if (coop && a.any_ns) {
        const void *fn = (const void *)k_march<EvalCoop1D<8, false, true>, false>;
        k_march<EvalCoop1D<8, false, true>, false><<<grid(fn), 256, 0, stream>>>(b);
    } else if (coop && a.all_grid) {
        const void *fn = (const void *)k_march<EvalCoop1D<8, true>, false>;
        k_march<EvalCoop1D<8, true>, false><<<grid(fn), 256, 0, stream>>>(b);
    } else if (coop && a.fast_window == 0u) {
        // the impulse window in shared memory (the default)
        const void *fn = (const void *)k_march<EvalCoop1D<8, false, false, true>, false>;
        k_march<EvalCoop1D<8, false, false, true>, false><<<grid(fn, kSmem1D), 256, kSmem1D, stream>>>(b);
    } else if (coop) {
        const void *fn = (const void *)k_march<EvalCoop1D<8>, false>;
        k_march<EvalCoop1D<8>, false><<<grid(fn), 256, 0, stream>>>(b);
    } else if (a.three_d && a.max_oct == 1 && !a.any_ns && !a.any_gen3d) {
        // 3D stationary single-octave media: the generic evaluator with step skipping
        const void *fn = (const void *)k_march<EvalSkip3D, false>;
        k_march<EvalSkip3D, false><<<grid(fn), 256, 0, stream>>>(b);
    } else {
        const void *fn = (const void *)k_march<EvalGeneric, false>;
        k_march<EvalGeneric, false><<<grid(fn), 256, 0, stream>>>(b);
    }
    // the resume passes take the flights the pass before handed on (queue 1: the
    // fast pass's, 2: the certified pass's)
    b.queue_in = 1;
    if (certify) {
        // crossings of stationary single-octave media decided on certified fast values
        const void *fn = (const void *)k_march<EvalGeneric4, true, true>;
        k_march<EvalGeneric4, true, true><<<grid(fn, 0, false), 256, 0, stream>>>(b);
        b.queue_in = 2;
    }
    if (a.one_d && !certify) {
        const void *fn = (const void *)k_march<EvalGeneric4, true>;
        k_march<EvalGeneric4, true><<<grid(fn, 0, false), 256, 0, stream>>>(b);
    } else {
        // 3D media, and what the certified pass leaves (a fifth of the crossings: 2
        // CTAs at 128 registers without spills, 0.7 % faster per bench step than 4)
        const void *fn = (const void *)k_march<EvalGeneric, true>;
        k_march<EvalGeneric, true><<<grid(fn, 0, false), 256, 0, stream>>>(b);
    }
    if (ev) cudaEventRecord(ev[3], stream);
    if (ev) cudaEventRecord(ev[4], stream);
    if (a.one_d) k_finish<8><<<blocks, 128, 0, stream>>>(b);
    else k_finish<4><<<blocks, 128, 0, stream>>>(b);
    if (ev) cudaEventRecord(ev[5], stream);
    return cudaGetLastError();
}

cudaError_t launch_debug_exp(const float *x, float *y, uint32_t n, cudaStream_t s)
{
    if (n) k_debug_exp<<<(n + 255) / 256, 256, 0, s>>>(x, y, n);
    return cudaGetLastError();
}

cudaError_t launch_debug_cells_1d(const uint32_t *cells, const uint32_t *seeds, uint32_t n,
                                  uint32_t impulses, float *pos, float *weight, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_debug_cells_1d<<<(n + 127) / 128, 128, 0, s>>>(cells, seeds, n, impulses, pos, weight);
    return cudaGetLastError();
}

cudaError_t launch_debug_cells_3d(const int32_t *cells, const uint32_t *seeds, uint32_t n,
                                  uint32_t impulses, uint32_t order, float *pos, float *weight,
                                  cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_debug_cells_3d<<<(n + 127) / 128, 128, 0, s>>>(cells, seeds, n, impulses, order, pos, weight);
    return cudaGetLastError();
}

cudaError_t launch_debug_field(const DevMedium *m, const float4 *origins, const float4 *points,
                               const float4 *dirs, const uint4 *seeds, const float4 *prev,
                               uint32_t n, float4 *out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_debug_field<<<(n + 127) / 128, 128, 0, s>>>(m, origins, points, dirs, seeds, prev, n, out);
    return cudaGetLastError();
}

cudaError_t launch_nee(const FlightArgs &a, const float4 *point_t, const float4 *normal, float4 *out,
                       cudaStream_t stream)
{
    if (a.n == 0) return cudaSuccess;
    uint32_t blocks = (a.n + 127) / 128;
    if (a.n_dev) blocks = std::min<uint32_t>(blocks, 2048u);
    k_nee<<<blocks, 128, 0, stream>>>(a, point_t, normal, out);
    return cudaGetLastError();
}

cudaError_t launch_pack_grid(const DevMedium &m, float4 *cells, size_t n, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    DevMedium mm = m;
    mm.grid_cells = nullptr;
    k_pack_grid<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(mm, cells, n);
    return cudaGetLastError();
}

cudaError_t launch_se_splat_1d(const float *q, const float *c, float *v, float *d, size_t n,
                               float scale, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const size_t blocks = (n + 255) / 256;
    k_se_splat_1d<<<(unsigned)blocks, 256, 0, s>>>(q, c, v, d, n, scale);
    return cudaGetLastError();
}

}  // namespace gpis
