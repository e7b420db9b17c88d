// device_common.cuh -- device-side building blocks of the GPIS flight kernels:
// the medium table, cell hash, jump-ahead PCG32, tangent frame, means and the
// float-float march parameter.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gpis {

// Maximum impulses per cell the library accepts (RaySegmentBatch.cu:317-318 caps
// impulseDensity at 64).
constexpr int kMaxImpulses = 64;
// PCG draws a cell can consume: 2 warm-up + 4 per 3D impulse.
constexpr int kMaxDraws = 2 + 4 * kMaxImpulses;

// Medium flags.
enum : uint32_t {
    MF_ONE_D = 1u << 0,          // 1D sampling in isotropic ray space
    MF_COND = 1u << 1,           // Renewal / Renewal+ conditioning active
    MF_RENEWAL_PLUS = 1u << 2,   // gradient conditioning
    MF_CORR_XY = 1u << 3,        // 1D_gradient_correlationXY
    MF_TRANSVERSE = 1u << 4,     // exact SE transverse law applies
    MF_XYZ_ORDER = 1u << 5,      // next3D drawn x first
    MF_MULTIRES = 1u << 6,       // 2-level multi-resolution blend of the length scale
    MF_ISO3D = 1u << 7,          // 3D noise in isotropic ray space (isotropic_3D_sampling)
};

// Levels of the multi-resolution grid: scales 2.5^L for L in [-kMrLevels, kMrLevels).
constexpr int kMrLevels = 16;

// Per-medium constants derived on the host (all float values are rounded as the
// reference's float expressions round them).
struct DevMedium {
    float sigma;            // noise amplitude
    float l_inv[3];         // world -> isotropic (diagonal of _world_to_local)
    float l_aniso[3];       // isotropic -> world (diagonal of _local_to_world)
    float kr_iso;           // cell size of 1D noise in isotropic units (localScale)
    float kr_world;         // cell size of 3D world noise
    float inv_norm1d;       // 1 / sqrt(sparseConvNoiseVariance1D)
    float inv_norm3d;       // 1 / sqrt(sparseConvNoiseVariance3D)
    float norm1d;           // sqrt(sparseConvNoiseVariance1D) as the reference rounds it
    float norm3d;           // sqrt(sparseConvNoiseVariance3D)
    float cov_den2;         // 2 * sqr(float(sqrt(2))): covarianceKernel1DVal denominator
    float kexp1d;           // exp(-(kr*d)^2/2) = ex2(kexp1d * d * d)
    float kexp3d[3];        // 3D splat: ex2(sum_c kexp3d[c] * (kr*d_c)^2)
    float m3[3];            // 3D splat inverse covariance diagonal (isCov = false)
    float m3c[3];           // 3D conditioning inverse covariance diagonal (isCov = true)
    float d2inv3[3];        // 3D Renewal+: 1 / (-2 * 0.25 * l_inv^2)
    uint32_t n_imp;         // impulses per cell
    uint32_t flags;
    uint32_t seed_pad;
    uint32_t mean_kind;
    float mean_params[8];
    const float *grid;      // device voxels (GPIS_MEAN_GRID)
    int32_t grid_origin[3];
    int32_t grid_dims[3];
    float grid_w2i[12];
    float grid_cmin[3];
    float grid_cmax[3];
    float grid_offset;
    float grid_scale;
    // corner table: the 8 (clamped) corner voxels of every reachable trilinear
    // cell as two float4, cells lo..lo+n-1 per axis; null when not built
    const float4 *grid_cells;
    int32_t cell_lo[3];
    int32_t cell_n[3];
    float step_size;
    uint32_t min_step;
    uint32_t max_steps;
    uint32_t scheme;
    // nonstationary length scale ls(p) = a + b*sin(fx*x)*cos(fz*z) (brute force)
    uint32_t ls_kind;
    float ls_params[4];
    float ls_max;
    float var1d_c;          // impulseDensity / kernelRadius as the reference rounds it
    // octaves: noise = sum_k oct_sigma[k] * n_k with length scale x oct_scale[k]
    uint32_t n_oct;
    float oct_sigma[4];
    float oct_scale[4];
    uint32_t oct_seed[4];
    // march-step skipping in the fast pass (skip_mean_lip < 0: not available): the
    // mean's Lipschitz constant along a ray, the noise's per iso unit and the
    // largest jump of one truncated splat (noise units)
    float skip_mean_lip;
    float skip_noise_lip;   // 3 N e^{-1/2} / norm1d per iso unit
    float skip_jump;        // e^{-kr^2/2} / norm1d per truncation crossing
    float oct_inv[4];       // 1 / oct_scale[k], exact where the scale is a power of two
    uint32_t oct_pow2;      // bit k: oct_scale[k] is a power of two (x / s == x * oct_inv[k])
    // multi-resolution grid (MF_MULTIRES; ls_kind is 0 on the device so that the
    // transforms and splats take the stationary forms, ls_params hold ls(p)):
    // log(2.5f), the level scales powf(2.5f, L) and the per-level noise-seed
    // offsets floor(log(scale) / log(2.5f)) at index L + kMrLevels, as the host's
    // float library rounds them
    float mr_log_base;
    float mr_pow[2 * kMrLevels];
    int32_t mr_seed[2 * kMrLevels];
    // 3D brute-force nonstationary noise in world space: the noise-seed offset
    // floor(log(ls_max) / log(2.5f)) of its kernelSpatialScale ls_max
    int32_t ns3_seed;
    float imp_density;      // impulseDensity as given (the 3D normalisation's numerator)
};

// A 3D medium outside the stationary world-space form: isotropic ray space,
// a nonstationary length scale or the multi-resolution grid.
__host__ __device__ inline bool general_3d(const DevMedium &m)
{
    return !(m.flags & MF_ONE_D) && ((m.flags & (MF_ISO3D | MF_MULTIRES)) || m.ls_kind != 0u);
}

struct PcgJump {
    uint32_t alo, ahi;      // multiplier M^k
    uint32_t clo, chi;      // increment sum_{j<k} M^j
};

// ---- hashing (MathUtil::xxhash32, src/core/math/MathUtil.hpp:179-224) -------
__device__ __forceinline__ uint32_t rotl17(uint32_t h) { return __funnelshift_l(h, h, 17); }

__device__ __forceinline__ uint32_t xx_finish(uint32_t h)
{
    h = 2246822519u * (h ^ (h >> 15));
    h = 3266489917u * (h ^ (h >> 13));
    return h ^ (h >> 16);
}

__device__ __forceinline__ uint32_t xxhash2(uint32_t x, uint32_t y)
{
    uint32_t h = y + 374761393u + x * 3266489917u;
    h = 668265263u * rotl17(h);
    return xx_finish(h);
}

__device__ __forceinline__ uint32_t xxhash4(uint32_t x, uint32_t y, uint32_t z, uint32_t w)
{
    uint32_t h = w + 374761393u + x * 3266489917u;
    h = 668265263u * rotl17(h);
    h += y * 3266489917u;
    h = 668265263u * rotl17(h);
    h += z * 3266489917u;
    h = 668265263u * rotl17(h);
    return xx_finish(h);
}

// ---- PCG32 output of a 64-bit state (UniformSampler::nextI, UniformSampler.hpp:41-48)
__device__ __forceinline__ uint32_t pcg_output(uint32_t lo, uint32_t hi)
{
    // ((old >> 18) ^ old) >> 27 truncated to 32 bits == (old >> 27) ^ (old >> 45)
    const uint32_t xs = __funnelshift_r(lo, hi, 27) ^ (hi >> 13);
    return __funnelshift_r(xs, xs, hi >> 27);
}

// State k of the stream that set_state(s) starts: M^k * s + C_k (s < 2^32).
__device__ __forceinline__ uint32_t pcg_draw(const PcgJump &j, uint32_t s)
{
    const uint64_t prod = (uint64_t)j.alo * s + (((uint64_t)j.chi << 32) | j.clo);
    const uint32_t lo = (uint32_t)prod;
    const uint32_t hi = (uint32_t)(prod >> 32) + j.ahi * s;
    return pcg_output(lo, hi);
}

// BitManip::normalizedUint (BitManip.hpp:47-50)
__device__ __forceinline__ float unit_float(uint32_t r)
{
    return __fsub_rn(__uint_as_float((r >> 9) | 0x3F800000u), 1.0f);
}

// ---- exact IEEE float helpers (no contraction) --------------------------------
__device__ __forceinline__ float dot3_rn(float a0, float a1, float a2, float b0, float b1, float b2)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a0, b0), __fmul_rn(a1, b1)), __fmul_rn(a2, b2));
}

__device__ __forceinline__ void normalize3_rn(float &x, float &y, float &z)
{
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot3_rn(x, y, z, x, y, z)));
    x = __fmul_rn(x, inv);
    y = __fmul_rn(y, inv);
    z = __fmul_rn(z, inv);
}

// TangentFrame(n) (TangentFrame.hpp:74-98), IEEE-rounded like the reference.
struct Frame {
    float n[3], t[3], b[3];
};

__device__ __forceinline__ void make_frame(float nx, float ny, float nz, Frame &f)
{
    normalize3_rn(nx, ny, nz);
    f.n[0] = nx; f.n[1] = ny; f.n[2] = nz;
    const float sign = copysignf(1.0f, nz);
    const float a = __fdiv_rn(-1.0f, __fadd_rn(sign, nz));
    const float b = __fmul_rn(__fmul_rn(nx, ny), a);
    float tx = __fadd_rn(1.0f, __fmul_rn(__fmul_rn(__fmul_rn(sign, nx), nx), a));
    float ty = __fmul_rn(sign, b);
    float tz = -__fmul_rn(sign, nx);
    float bx = b;
    float by = __fadd_rn(sign, __fmul_rn(__fmul_rn(ny, ny), a));
    float bz = -ny;
    normalize3_rn(tx, ty, tz);
    normalize3_rn(bx, by, bz);
    f.t[0] = tx; f.t[1] = ty; f.t[2] = tz;
    f.b[0] = bx; f.b[1] = by; f.b[2] = bz;
}

// ---- float-float march parameter ----------------------------------------------
// t = hi + lo represents the reference's double t exactly for the march grid
// t_k = t0 + k*step (t0, step floats).
__device__ __forceinline__ float two_sum(float a, float b, float &err)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

__device__ __forceinline__ void ff_add(float &hi, float &lo, float b)
{
    float e;
    const float s = two_sum(hi, b, e);
    const float l = __fadd_rn(lo, e);
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}

// float(o + t*d) with o, d floats and t = hi + lo, rounded as the double
// expression Vec3f(Vec3d(o) + t * Vec3d(d)).
__device__ __forceinline__ float ff_point(float o, float d, float hi, float lo)
{
    const float a = __fmul_rn(hi, d);
    const float ae = __fmaf_rn(hi, d, -a);
    const float b = __fmul_rn(lo, d);
    float se;
    const float s = two_sum(o, a, se);
    const float r = __fadd_rn(se, __fadd_rn(ae, b));
    return __fadd_rn(s, r);
}

// ---- float-float arithmetic (about 48 significant bits) -------------------------
struct FF {
    float h, l;
};

__device__ __forceinline__ FF ff_norm(float h, float l)
{
    const float s = __fadd_rn(h, l);
    return {s, __fsub_rn(l, __fsub_rn(s, h))};
}

__device__ __forceinline__ FF ff_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    float e;
    const float s = two_sum(a.h, b.h, e);
    return ff_norm(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}

__device__ __forceinline__ FF ff_add_f(FF a, float b)
{
    float e;
    const float s = two_sum(a.h, b, e);
    return ff_norm(s, __fadd_rn(e, a.l));
}

__device__ __forceinline__ FF ff_mul(FF a, FF b)
{
    FF p = ff_prod(a.h, b.h);
    return ff_norm(p.h, __fadd_rn(p.l, __fadd_rn(__fmul_rn(a.h, b.l), __fmul_rn(a.l, b.h))));
}

__device__ __forceinline__ FF ff_mul_f(FF a, float b)
{
    FF p = ff_prod(a.h, b);
    return ff_norm(p.h, __fadd_rn(p.l, __fmul_rn(a.l, b)));
}

__device__ __forceinline__ FF ff_sq(FF a)
{
    FF p = ff_prod(a.h, a.h);
    return ff_norm(p.h, __fadd_rn(p.l, __fmul_rn(2.0f * a.h, a.l)));
}

__device__ __forceinline__ FF ff_sqrt(FF a)
{
    if (!(a.h > 0.0f)) return {__fsqrt_rn(a.h), 0.0f};   // 0 (or NaN below 0), no 0 / 0
    const float r = __fsqrt_rn(a.h);
    const FF r2 = ff_prod(r, r);
    const float e = __fadd_rn(__fsub_rn(__fsub_rn(a.h, r2.h), r2.l), a.l);
    return ff_norm(r, __fdiv_rn(e, __fmul_rn(2.0f, r)));
}

// a / b for floats a, b as a float-float quotient.
__device__ __forceinline__ FF ff_div_ff(float a, FF b)
{
    const float q = __fdiv_rn(a, b.h);
    const float r = __fsub_rn(__fmaf_rn(-q, b.h, a), __fmul_rn(q, b.l));
    return ff_norm(q, __fdiv_rn(r, b.h));
}

// 1 / sqrt(a) as a float-float pair (about 43 significant bits): the float reciprocal
// square root and one Newton step r + r (1 - a r^2) / 2 in float-float.  Replaces the
// double division by a double square root where the result is rounded to float.
__device__ __forceinline__ FF ff_rsqrt(FF a)
{
    const float r = rsqrtf(a.h);
    const FF ar2 = ff_mul(a, ff_prod(r, r));
    const FF e = ff_add_f({-ar2.h, -ar2.l}, 1.0f);
    return ff_add_f(ff_mul_f(e, 0.5f * r), r);
}

// a <= c for a float-float a and the double c = ch + cl.
__device__ __forceinline__ bool ff_le(FF a, float ch, float cl)
{
    return a.h < ch || (a.h == ch && a.l <= cl);
}

__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ---- correctly rounded exp ---------------------------------------------------
// e^x rounded to the nearest float, the exp of the precise evaluator (the oracle
// evaluates the reference's float exp as (float)exp((double)x), the correctly
// rounded value).  Tang's table-driven method (P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point arithmetic",
// ACM TOMS 15(2), 1989) carried in float-float: x = (64 m + j) ln2 / 64 + r with
// |r| <= ln2 / 128, e^x = 2^m 2^(j/64) e^r, the table 2^(j/64) as float pairs
// (hi + lo, generated from the definition to 60 digits), e^r - 1 as
// r + r^2/2 (exact products) + r^3/6 + r^4/24 + r^5/120, one rounding at the end.
// Relative error about 2^-46 before the rounding: it differs from the correctly
// rounded value on about 1e-8 of the arguments in [-90, 0] (checked exhaustively
// on every third float there).  Arguments below -87 (results near the denormal
// range, which never decide a sum) take expf.
static __device__ const float2 g_exp2_64[64] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f},
    {0x1.02c9a40000000p+0f, -0x1.887fa00000000p-28f},
    {0x1.059b0e0000000p+0f, -0x1.9d4f520000000p-25f},
    {0x1.0874520000000p+0f, -0x1.e2990e0000000p-26f},
    {0x1.0b55860000000p+0f, 0x1.9f31220000000p-25f},
    {0x1.0e3ec40000000p+0f, -0x1.a585cc0000000p-25f},
    {0x1.11301e0000000p+0f, -0x1.fdb4960000000p-25f},
    {0x1.1429aa0000000p+0f, 0x1.d525bc0000000p-25f},
    {0x1.172b840000000p+0f, -0x1.c157420000000p-27f},
    {0x1.1a35be0000000p+0f, 0x1.6df96e0000000p-25f},
    {0x1.1d48740000000p+0f, -0x1.d2e8ca0000000p-25f},
    {0x1.2063b80000000p+0f, 0x1.0c519a0000000p-25f},
    {0x1.2387a60000000p+0f, 0x1.ceac480000000p-25f},
    {0x1.26b4560000000p+0f, 0x1.789f380000000p-26f},
    {0x1.29e9e00000000p+0f, -0x1.5c04240000000p-25f},
    {0x1.2d285a0000000p+0f, 0x1.b900c20000000p-26f},
    {0x1.306fe00000000p+0f, 0x1.4636e20000000p-25f},
    {0x1.33c08c0000000p+0f, -0x1.b37d200000000p-25f},
    {0x1.371a740000000p+0f, -0x1.18aac60000000p-25f},
    {0x1.3a7db40000000p+0f, -0x1.634c020000000p-25f},
    {0x1.3dea640000000p+0f, 0x1.8246840000000p-25f},
    {0x1.4160a20000000p+0f, 0x1.f72e2a0000000p-28f},
    {0x1.44e0860000000p+0f, 0x1.8624b40000000p-30f},
    {0x1.486a2c0000000p+0f, -0x1.47d8660000000p-25f},
    {0x1.4bfdae0000000p+0f, -0x1.593abc0000000p-25f},
    {0x1.4f9b280000000p+0f, -0x1.2c5a6c0000000p-25f},
    {0x1.5342b60000000p+0f, -0x1.2c56100000000p-25f},
    {0x1.56f4740000000p+0f, -0x1.295b040000000p-25f},
    {0x1.5ab07e0000000p+0f, -0x1.5bd5ec0000000p-27f},
    {0x1.5e76f20000000p+0f, -0x1.4a5bd60000000p-25f},
    {0x1.6247ec0000000p+0f, -0x1.f8b5500000000p-25f},
    {0x1.6623880000000p+0f, 0x1.2a91120000000p-27f},
    {0x1.6a09e60000000p+0f, 0x1.9fcef40000000p-26f},
    {0x1.6dfb240000000p+0f, -0x1.cd72e80000000p-27f},
    {0x1.71f75e0000000p+0f, 0x1.1d8bee0000000p-25f},
    {0x1.75feb60000000p+0f, -0x1.37b3060000000p-25f},
    {0x1.7a11480000000p+0f, -0x1.829fd00000000p-25f},
    {0x1.7e2f340000000p+0f, -0x1.2616340000000p-25f},
    {0x1.82589a0000000p+0f, -0x1.accc7c0000000p-26f},
    {0x1.868d9a0000000p+0f, -0x1.2edb440000000p-26f},
    {0x1.8ace540000000p+0f, 0x1.15506e0000000p-27f},
    {0x1.8f1aea0000000p+0f, -0x1.baa2320000000p-26f},
    {0x1.93737c0000000p+0f, -0x1.e647440000000p-25f},
    {0x1.97d82a0000000p+0f, -0x1.0d8d840000000p-31f},
    {0x1.9c49180000000p+0f, 0x1.51f8480000000p-27f},
    {0x1.a0c6680000000p+0f, -0x1.2886a60000000p-26f},
    {0x1.a5503c0000000p+0f, -0x1.b83b540000000p-25f},
    {0x1.a9e6b60000000p+0f, -0x1.50c0480000000p-25f},
    {0x1.ae89fa0000000p+0f, -0x1.a94b140000000p-26f},
    {0x1.b33a2c0000000p+0f, -0x1.ec3a820000000p-26f},
    {0x1.b7f7700000000p+0f, -0x1.a094380000000p-25f},
    {0x1.bcc1ea0000000p+0f, -0x1.f687c60000000p-25f},
    {0x1.c199be0000000p+0f, -0x1.3d56b20000000p-27f},
    {0x1.c67f120000000p+0f, 0x1.cafa2a0000000p-25f},
    {0x1.cb720e0000000p+0f, -0x1.8837cc0000000p-27f},
    {0x1.d072d40000000p+0f, 0x1.40f1300000000p-25f},
    {0x1.d5818e0000000p+0f, -0x1.822dbc0000000p-27f},
    {0x1.da9e600000000p+0f, 0x1.ed99420000000p-27f},
    {0x1.dfc9740000000p+0f, -0x1.908c940000000p-25f},
    {0x1.e502ee0000000p+0f, 0x1.e2cffe0000000p-26f},
    {0x1.ea4afa0000000p+0f, 0x1.52486c0000000p-27f},
    {0x1.efa1be0000000p+0f, 0x1.cc2b440000000p-25f},
    {0x1.f507660000000p+0f, -0x1.246eb00000000p-26f},
    {0x1.fa7c180000000p+0f, 0x1.9e90d80000000p-28f},
};

__device__ __forceinline__ float cr_expf(float x)
{
    if (!(x > -87.0f)) return expf(x);
    const float kf = rintf(x * 0x1.715476p+6f);   // 64 / ln2
    const int k = (int)kf;
    const float c_hi = 0x1.62e43p-7f, c_lo = -0x1.05c61p-35f;   // ln2 / 64 = c_hi + c_lo + O(2^-60)
    const float ph = __fmul_rn(kf, c_hi);
    float pl = __fmaf_rn(kf, c_hi, -ph);
    pl = __fmaf_rn(kf, c_lo, pl);
    const float rh = __fsub_rn(x, ph);   // exact (Sterbenz)
    const float r = __fsub_rn(rh, pl);
    const float rl = __fsub_rn(__fsub_rn(rh, r), pl);
    const float s2h = __fmul_rn(r, r);
    float s2l = __fmaf_rn(r, r, -s2h);
    s2l = __fmaf_rn(__fmul_rn(2.0f, r), rl, s2l);
    const float h2h = __fmul_rn(0.5f, s2h), h2l = __fmul_rn(0.5f, s2l);
    const float tail = __fmul_rn(__fmul_rn(r, s2h),
                                 __fmaf_rn(r, __fmaf_rn(r, 0x1.111112p-7f, 0x1.555556p-5f), 0x1.555556p-3f));
    // |h2h| <= 0.003 |r|: the fast two-sum is exact
    const float qh = __fadd_rn(r, h2h);
    float ql = __fsub_rn(h2h, __fsub_rn(qh, r));
    ql = __fadd_rn(ql, __fadd_rn(rl, __fadd_rn(h2l, tail)));
    const float2 t = __ldg(&g_exp2_64[k & 63]);
    const float ah = __fmul_rn(t.x, qh);
    float al = __fmaf_rn(t.x, qh, -ah);
    al = __fadd_rn(al, __fmaf_rn(t.x, ql, __fmaf_rn(t.y, qh, t.y)));
    // |ah| < 0.011 <= t.x: the fast two-sum is exact
    const float sh = __fadd_rn(t.x, ah);
    const float sl = __fsub_rn(ah, __fsub_rn(sh, t.x));
    const float y = __fadd_rn(sh, __fadd_rn(sl, al));
    return __fmul_rn(y, __int_as_float(((k >> 6) + 127) << 23));
}

// ---- means (MeanFunction::mean / dmean_da) -------------------------------------
__device__ __forceinline__ float grid_voxel(const DevMedium &m, int x, int y, int z)
{
    x = min(max(x - m.grid_origin[0], 0), m.grid_dims[0] - 1);
    y = min(max(y - m.grid_origin[1], 0), m.grid_dims[1] - 1);
    z = min(max(z - m.grid_origin[2], 0), m.grid_dims[2] - 1);
    const size_t idx = ((size_t)z * (size_t)m.grid_dims[1] + (size_t)y) * (size_t)m.grid_dims[0] + (size_t)x;
    return __ldg(m.grid + idx);
}

// The eight corner voxels of the trilinear cell of p and its fractions: the
// loads of grid_mean, issued apart from the arithmetic so that a caller can
// overlap their latency with other work.
struct GridTap {
    float v[8];
    float fx, fy, fz;
};

__device__ __forceinline__ void grid_fetch(const DevMedium &m, float px, float py, float pz, GridTap &g)
{
    float q[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float v = __fmul_rn(m.grid_w2i[4 * r + 0], px);
        v = __fadd_rn(v, __fmul_rn(m.grid_w2i[4 * r + 1], py));
        v = __fadd_rn(v, __fmul_rn(m.grid_w2i[4 * r + 2], pz));
        v = __fadd_rn(v, m.grid_w2i[4 * r + 3]);
        q[r] = fminf(fmaxf(v, m.grid_cmin[r]), m.grid_cmax[r]);
    }
    const int x = (int)floorf(q[0]), y = (int)floorf(q[1]), z = (int)floorf(q[2]);
    g.fx = q[0] - (float)x;
    g.fy = q[1] - (float)y;
    g.fz = q[2] - (float)z;
    if (m.grid_cells) {
        // the clamps keep (x, y, z) inside the table: floor of [cmin, cmax]
        const size_t c = ((size_t)(z - m.cell_lo[2]) * (size_t)m.cell_n[1] + (size_t)(y - m.cell_lo[1])) *
                             (size_t)m.cell_n[0] + (size_t)(x - m.cell_lo[0]);
        const float4 a = __ldg(m.grid_cells + 2 * c), b = __ldg(m.grid_cells + 2 * c + 1);
        g.v[0] = a.x; g.v[1] = a.y; g.v[2] = a.z; g.v[3] = a.w;
        g.v[4] = b.x; g.v[5] = b.y; g.v[6] = b.z; g.v[7] = b.w;
        return;
    }
    // clamp each axis' two indices once (grid_voxel's rule), then 8 loads
    const int nx = m.grid_dims[0], ny = m.grid_dims[1], nz = m.grid_dims[2];
    const int x0 = min(max(x - m.grid_origin[0], 0), nx - 1), x1 = min(max(x + 1 - m.grid_origin[0], 0), nx - 1);
    const int y0 = min(max(y - m.grid_origin[1], 0), ny - 1), y1 = min(max(y + 1 - m.grid_origin[1], 0), ny - 1);
    const int z0 = min(max(z - m.grid_origin[2], 0), nz - 1), z1 = min(max(z + 1 - m.grid_origin[2], 0), nz - 1);
    const float *r00 = m.grid + ((size_t)z0 * ny + y0) * nx;
    const float *r01 = m.grid + ((size_t)z0 * ny + y1) * nx;
    const float *r10 = m.grid + ((size_t)z1 * ny + y0) * nx;
    const float *r11 = m.grid + ((size_t)z1 * ny + y1) * nx;
    g.v[0] = __ldg(r00 + x0); g.v[1] = __ldg(r00 + x1);
    g.v[2] = __ldg(r01 + x0); g.v[3] = __ldg(r01 + x1);
    g.v[4] = __ldg(r10 + x0); g.v[5] = __ldg(r10 + x1);
    g.v[6] = __ldg(r11 + x0); g.v[7] = __ldg(r11 + x1);
}

__device__ __forceinline__ float grid_combine(const DevMedium &m, const GridTap &g)
{
    float layer[2];
#pragma unroll
    for (int dz = 0; dz < 2; ++dz) {
        float row[2];
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            const float a = g.v[4 * dz + 2 * dy + 0];
            const float b = g.v[4 * dz + 2 * dy + 1];
            row[dy] = a + g.fx * (b - a);
        }
        layer[dz] = row[0] + g.fy * (row[1] - row[0]);
    }
    return (layer[0] + g.fz * (layer[1] - layer[0]) + m.grid_offset) * m.grid_scale;
}

// Dense trilinear grid mean (RaySegmentBatch.cu:73-95 semantics).
__device__ __forceinline__ float grid_mean(const DevMedium &m, float px, float py, float pz)
{
    GridTap g;
    grid_fetch(m, px, py, pz, g);
    return grid_combine(m, g);
}

__device__ __forceinline__ float torus_sdf(const float *q, float x, float y, float z)
{
    x -= q[0]; y -= q[1]; z -= q[2];
    const float rxz = sqrtf(x * x + z * z) - q[3];
    return sqrtf(rxz * rxz + y * y) - q[4];
}

// mean_weight_space: value and GP id (0 unless the union picks its second surface).
__device__ __forceinline__ float mean_value(const DevMedium &m, float x, float y, float z, int &id)
{
    const float *q = m.mean_params;
    id = 0;
    switch (m.mean_kind) {
    case 0: {  // sphere
        const float dx = x - q[0], dy = y - q[1], dz = z - q[2];
        return sqrtf(dx * dx + dy * dy + dz * dz) - q[3];
    }
    case 1:
        return q[0];
    case 2:
        return grid_mean(m, x, y, z);
    case 3:
        return q[0] * x + q[1] * y + q[2] * z - q[3];
    case 4:
        return torus_sdf(q, x, y, z);
    case 5: {
        const float t = torus_sdf(q, x, y, z);
        const float pl = y - q[5];
        if (pl < t) { id = 1; return pl; }
        return t;
    }
    default:
        return 0.0f;
    }
}

// Mean gradient as the reference evaluates it (in double for the sphere, to float).
__device__ __forceinline__ void mean_grad(const DevMedium &m, float x, float y, float z, float g[3])
{
    const float *q = m.mean_params;
    int id;
    switch (m.mean_kind) {
    case 0: {
        // (p - c).normalized() in double, rounded to float: the differences are exact
        // float-float pairs, the squared length and its reciprocal square root are
        // carried in float-float (the double path's FP64 division and square root run
        // at a small fraction of the FP32 rate)
        float ex, ey, ez;
        const FF dx = {two_sum(x, -q[0], ex), 0.0f}, dy = {two_sum(y, -q[1], ey), 0.0f},
                 dz = {two_sum(z, -q[2], ez), 0.0f};
        const FF ddx = {dx.h, ex}, ddy = {dy.h, ey}, ddz = {dz.h, ez};
        const FF inv = ff_rsqrt(ff_add(ff_add(ff_sq(ddx), ff_sq(ddy)), ff_sq(ddz)));
        const FF gx = ff_mul(ddx, inv), gy = ff_mul(ddy, inv), gz = ff_mul(ddz, inv);
        g[0] = __fadd_rn(gx.h, gx.l); g[1] = __fadd_rn(gy.h, gy.l); g[2] = __fadd_rn(gz.h, gz.l);
        return;
    }
    case 1:
        g[0] = g[1] = g[2] = 0.0f;
        return;
    case 2: {  // TabulatedMean::dmean_da forward difference, eps 0.001 in double
        const double eps = 0.001;
        const float v0 = grid_mean(m, x, y, z);
        const float vx = grid_mean(m, (float)((double)x + eps), y, z);
        const float vy = grid_mean(m, x, (float)((double)y + eps), z);
        const float vz = grid_mean(m, x, y, (float)((double)z + eps));
        g[0] = (float)(((double)vx - v0) / eps);
        g[1] = (float)(((double)vy - v0) / eps);
        g[2] = (float)(((double)vz - v0) / eps);
        return;
    }
    case 3:
        g[0] = q[0]; g[1] = q[1]; g[2] = q[2];
        return;
    case 4:
    case 5: {
        (void)mean_value(m, x, y, z, id);
        if (m.mean_kind == 5 && id == 1) {
            g[0] = 0.0f; g[1] = 1.0f; g[2] = 0.0f;
            return;
        }
        const float px = x - q[0], py = y - q[1], pz = z - q[2];
        const float rxz = sqrtf(px * px + pz * pz);
        const float s = rxz - q[3];
        const float len = sqrtf(s * s + py * py);
        const float dr = s / len;
        g[0] = rxz > 0.0f ? dr * px / rxz : 0.0f;
        g[1] = py / len;
        g[2] = rxz > 0.0f ? dr * pz / rxz : 0.0f;
        return;
    }
    default:
        g[0] = g[1] = g[2] = 0.0f;
    }
}

}  // namespace gpis
