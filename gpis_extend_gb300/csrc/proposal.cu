// proposal.cu -- the learned crossing proposal of the flight path.
//
// A small network predicts, per flight, where along [near, far] the first
// downcrossing lies: a GRU (hidden 32) over eight samples of the mean SDF and its
// slope along the ray, then a 3 x 64 GELU MLP over the GRU state and eight
// per-flight features, emitting an 8-component logistic mixture over
// u = (t - near) / (far - near) and a miss logit.  Every contraction runs on the
// tensor cores as BF16 x BF16 -> FP32 (tcgen05 with tensor-memory accumulators; the
// warp-level mma.sync m16n8k16 kernels remain selectable); the elementwise parts,
// the loss and Adam are FP32.  Training uses an unfused layer-by-layer forward
// that keeps its activations and a hand-written backward, its GEMMs on tcgen05;
// inference is one persistent fused tcgen05 kernel with the weights in shared memory.
//
// The proposal never changes a flight's result: gpis_flights_submit_proposed lets
// the march take longer certified skips before the proposed interval, and every
// skipped step is still proven free of a sign change by the same bound as the
// plain march's step skipping.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/gpis.h"
#include "device_common.cuh"
#include "flights.cuh"
#include "umma.cuh"

extern "C" int gpis_internal_set_error(int code, const char *msg);

namespace gpis {
namespace prop {

constexpr int HID = 32, NIN = 16, MLPIN = 48, WID = 64, NOUT = 32, NHIST = 8, NFEAT = 24, NCOMP = 8;
// offsets into the flat parameter vector (weights row-major [out][in])
constexpr int O_WIH = 0, O_BIH = O_WIH + 3 * HID * NIN, O_WHH = O_BIH + 3 * HID, O_BHH = O_WHH + 3 * HID * HID,
              O_W1 = O_BHH + 3 * HID, O_B1 = O_W1 + WID * MLPIN, O_W2 = O_B1 + WID, O_B2 = O_W2 + WID * WID,
              O_W3 = O_B2 + WID, O_B3 = O_W3 + WID * WID, O_W4 = O_B3 + WID, O_B4 = O_W4 + NOUT * WID,
              N_PARAMS = O_B4 + NOUT;
static_assert(N_PARAMS == 18336, "parameter layout");

typedef __nv_bfloat16 bf;

__device__ __forceinline__ uint32_t bf_bits(bf x) { return (uint32_t)__bfloat16_as_ushort(x); }
__device__ __forceinline__ uint32_t pack2(bf lo, bf hi) { return bf_bits(lo) | (bf_bits(hi) << 16); }
__device__ __forceinline__ uint32_t pack2f(float lo, float hi)
{
    return pack2(__float2bfloat16_rn(lo), __float2bfloat16_rn(hi));
}

// D = A(16x16, row) * B(16x8, col) + D, BF16 inputs, FP32 accumulators.
// Fragments (g = lane / 4, t = lane % 4): a0 (g, 2t..2t+1), a1 (g+8, 2t..), a2 (g, 2t+8..),
// a3 (g+8, 2t+8..); b0 (k 2t..2t+1, n g), b1 (k 2t+8.., n g); d0,d1 (g, 2t..2t+1),
// d2,d3 (g+8, 2t..2t+1).  The lower half of each register holds the lower index.
__device__ __forceinline__ void mma_bf16(float d[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float sigm(float x) { return 1.0f / (1.0f + expf(-x)); }
// inference forms: the proposal only steers the march, so the fused kernel takes the
// hardware approximations (tanh.approx, ex2.approx, approximate division)
__device__ __forceinline__ float tanh_fast(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sigm_fast(float x) { return 0.5f + 0.5f * tanh_fast(0.5f * x); }
__device__ __forceinline__ float gelu_fast(float x)
{
    return 0.5f * x * (1.0f + tanh_fast(0.7978845608028654f * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float softplus(float x) { return x > 20.0f ? x : log1pf(expf(x)); }
constexpr float kGeluC = 0.7978845608028654f;
__device__ __forceinline__ float gelu(float x)
{
    return 0.5f * x * (1.0f + tanhf(kGeluC * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float gelu_grad(float x)
{
    const float t = tanhf(kGeluC * (x + 0.044715f * x * x * x));
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * kGeluC * (1.0f + 3.0f * 0.044715f * x * x);
}

// ---- generic strided GEMM: C(m, n) (+)= sum_k A(m, k) B(k, n) --------------------------
// A(m, k) = A[m * lam + k * lak], B(k, n) = B[k * lbk + n * lbn]; one warp per 16 x 8 tile
// of C and K chunk; M % 16 == 0, N % 8 == 0, K % 16 == 0.  ksplit > 1 adds into C
// with atomics (C zeroed or holding the sum to add to).
struct Gemm {
    const bf *A;
    long lam, lak;
    const bf *B;
    long lbk, lbn;
    float *C;
    long ldc;
    int M, N, K, accumulate, ksplit;
};

__global__ void __launch_bounds__(128) k_gemm(Gemm g)
{
    const long warp = (long)blockIdx.x * 4 + (threadIdx.x >> 5);
    const int tn_count = g.N / 8;
    const long total = (long)(g.M / 16) * tn_count * g.ksplit;
    if (warp >= total) return;
    const int lane = threadIdx.x & 31, gi = lane >> 2, ti = lane & 3;
    const int kc = (int)(warp % g.ksplit);
    const long tile = warp / g.ksplit;
    const int m0 = (int)(tile / tn_count) * 16, n0 = (int)(tile % tn_count) * 8;
    const int ktiles = g.K / 16;
    const int per = (ktiles + g.ksplit - 1) / g.ksplit;
    const int kt0 = kc * per, kt1 = min(ktiles, kt0 + per);
    float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const bf *A = g.A, *B = g.B;
    for (int kt = kt0; kt < kt1; ++kt) {
        const long k = (long)kt * 16 + 2 * ti;
        const long r0 = (long)(m0 + gi) * g.lam, r1 = (long)(m0 + gi + 8) * g.lam;
        const uint32_t a0 = pack2(A[r0 + k * g.lak], A[r0 + (k + 1) * g.lak]);
        const uint32_t a1 = pack2(A[r1 + k * g.lak], A[r1 + (k + 1) * g.lak]);
        const uint32_t a2 = pack2(A[r0 + (k + 8) * g.lak], A[r0 + (k + 9) * g.lak]);
        const uint32_t a3 = pack2(A[r1 + (k + 8) * g.lak], A[r1 + (k + 9) * g.lak]);
        const long c = (long)(n0 + gi) * g.lbn;
        const uint32_t b0 = pack2(B[k * g.lbk + c], B[(k + 1) * g.lbk + c]);
        const uint32_t b1 = pack2(B[(k + 8) * g.lbk + c], B[(k + 9) * g.lbk + c]);
        mma_bf16(d, a0, a1, a2, a3, b0, b1);
    }
    float *c0 = g.C + (long)(m0 + gi) * g.ldc + n0 + 2 * ti;
    float *c1 = g.C + (long)(m0 + gi + 8) * g.ldc + n0 + 2 * ti;
    if (g.ksplit > 1) {
        atomicAdd(c0, d[0]);
        atomicAdd(c0 + 1, d[1]);
        atomicAdd(c1, d[2]);
        atomicAdd(c1 + 1, d[3]);
    } else if (g.accumulate) {
        c0[0] += d[0]; c0[1] += d[1]; c1[0] += d[2]; c1[1] += d[3];
    } else {
        c0[0] = d[0]; c0[1] = d[1]; c1[0] = d[2]; c1[1] = d[3];
    }
}

// ---- elementwise kernels ---------------------------------------------------------------
// GRU inputs of every step, the globals part of the MLP input, h_0 = 0.
__global__ void k_prep(const float *feat, uint32_t n, bf *xb, bf *ub, float *h0, bf *h0b)
{
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const float *f = feat + (size_t)m * NFEAT;
    for (int j = 0; j < NHIST; ++j) {
        bf *x = xb + ((size_t)j * n + m) * NIN;
        x[0] = __float2bfloat16_rn(f[2 * j]);
        x[1] = __float2bfloat16_rn(f[2 * j + 1]);
        for (int c = 2; c < NIN; ++c) x[c] = __float2bfloat16_rn(0.0f);
    }
    bf *u = ub + (size_t)m * MLPIN;
    for (int c = 0; c < 8; ++c) u[HID + c] = __float2bfloat16_rn(f[16 + c]);
    for (int c = HID + 8; c < MLPIN; ++c) u[c] = __float2bfloat16_rn(0.0f);
    for (int c = 0; c < HID; ++c) {
        h0[(size_t)m * HID + c] = 0.0f;
        h0b[(size_t)m * HID + c] = __float2bfloat16_rn(0.0f);
    }
}

// GRU cell (PyTorch gate order r, z, n) from the raw products gi = x W_ih^T, gh = h W_hh^T.
__global__ void k_gru_cell(const float *gi, const float *gh, const float *P, const float *hprev, uint32_t n,
                           float *r_o, float *z_o, float *n_o, float *ghn_o, float *hnew, bf *hnewb, bf *ub)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * HID) return;
    const uint32_t m = i / HID, c = i % HID;
    const float *bih = P + O_BIH, *bhh = P + O_BHH;
    const float *a = gi + (size_t)m * 3 * HID, *b = gh + (size_t)m * 3 * HID;
    const float r = sigm(a[c] + bih[c] + b[c] + bhh[c]);
    const float z = sigm(a[HID + c] + bih[HID + c] + b[HID + c] + bhh[HID + c]);
    const float ghn = b[2 * HID + c] + bhh[2 * HID + c];
    const float nn = tanhf(a[2 * HID + c] + bih[2 * HID + c] + r * ghn);
    const float h = (1.0f - z) * nn + z * hprev[i];
    r_o[i] = r; z_o[i] = z; n_o[i] = nn; ghn_o[i] = ghn;
    hnew[i] = h;
    hnewb[i] = __float2bfloat16_rn(h);
    if (ub) ub[(size_t)m * MLPIN + c] = __float2bfloat16_rn(h);
}

// a += bias in place, y = bf16(gelu(a))
__global__ void k_bias_gelu(float *a, const float *bias, uint32_t n, int width, bf *y)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * (uint32_t)width) return;
    const float v = a[i] + bias[i % width];
    a[i] = v;
    y[i] = __float2bfloat16_rn(gelu(v));
}

// the mixture's negative log-likelihood and its gradient w.r.t. the 32 outputs, / n
__global__ void k_loss(float *o, const float *bias, const float2 *tgt, uint32_t n, float inv_n, float *dof, bf *dob,
                       float *loss)
{
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    float nll = 0.0f;
    if (m < n) {
        float *x = o + (size_t)m * NOUT;
        for (int c = 0; c < NOUT; ++c) x[c] += bias[c];
        const float us = tgt[m].x;
        const bool hit = tgt[m].y != 0.0f;
        float g[NOUT];
        for (int c = 0; c < NOUT; ++c) g[c] = 0.0f;
        const float ql = x[24];
        if (hit) {
            float lmax = x[0];
            for (int k = 1; k < NCOMP; ++k) lmax = fmaxf(lmax, x[k]);
            float se = 0.0f;
            for (int k = 0; k < NCOMP; ++k) se += expf(x[k] - lmax);
            const float lse_pi = lmax + logf(se);
            float comp[NCOMP], y[NCOMP], s[NCOMP], mu[NCOMP];
            float cmax = -INFINITY;
            for (int k = 0; k < NCOMP; ++k) {
                mu[k] = sigm(x[8 + k]);
                s[k] = softplus(x[16 + k]) + 1e-3f;
                y[k] = (us - mu[k]) / s[k];
                const float logf_k = -softplus(-y[k]) - softplus(y[k]) - logf(s[k]);
                comp[k] = x[k] - lse_pi + logf_k;
                cmax = fmaxf(cmax, comp[k]);
            }
            float cs = 0.0f;
            for (int k = 0; k < NCOMP; ++k) cs += expf(comp[k] - cmax);
            const float lse = cmax + logf(cs);
            nll = softplus(ql) - lse;
            for (int k = 0; k < NCOMP; ++k) {
                const float w = expf(comp[k] - lse);
                const float pk = expf(x[k] - lse_pi);
                g[k] = pk - w;
                const float dldy = tanhf(0.5f * y[k]);
                const float dm = w * dldy * (-1.0f / s[k]);
                const float ds = w * (dldy * (-y[k] / s[k]) + 1.0f / s[k]);
                g[8 + k] = dm * mu[k] * (1.0f - mu[k]);
                g[16 + k] = ds * sigm(x[16 + k]);
            }
            g[24] = sigm(ql);
        } else {
            nll = softplus(-ql);
            g[24] = -sigm(-ql);
        }
        for (int c = 0; c < NOUT; ++c) {
            const float v = g[c] * inv_n;
            dof[(size_t)m * NOUT + c] = v;
            dob[(size_t)m * NOUT + c] = __float2bfloat16_rn(v);
        }
    }
    // one atomic per warp
    for (int off = 16; off > 0; off >>= 1) nll += __shfl_xor_sync(0xffffffffu, nll, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, nll);
}

// out[c] += sum over rows of x[m * ld + c], c < width
__global__ void k_colsum(const float *x, uint32_t n, int width, long ld, float *out)
{
    const int c = threadIdx.x % width;
    const int rows_per = blockDim.x / width;
    float s = 0.0f;
    for (uint32_t m = blockIdx.x * rows_per + threadIdx.x / width; m < n; m += gridDim.x * rows_per)
        s += x[(size_t)m * ld + c];
    if ((int)threadIdx.x < rows_per * width) atomicAdd(out + c, s);
}

// da = dy * gelu'(a) (fp32 and bf16)
__global__ void k_gelu_back(const float *dy, const float *a, uint32_t n, int width, float *daf, bf *dab)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * (uint32_t)width) return;
    const float v = dy[i] * gelu_grad(a[i]);
    daf[i] = v;
    dab[i] = __float2bfloat16_rn(v);
}

// one GRU step backward: gate gradients and dh * z
__global__ void k_gru_back(const float *dh, long ldh, const float *r_, const float *z_, const float *n_,
                           const float *ghn_, const float *hprev, uint32_t n, float *dgif, bf *dgib, float *dghf,
                           bf *dghb, float *dhpart)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * HID) return;
    const uint32_t m = i / HID, c = i % HID;
    const float d = dh[(size_t)m * ldh + c];
    const float r = r_[i], z = z_[i], nn = n_[i], ghn = ghn_[i];
    const float dz = d * (hprev[i] - nn) * z * (1.0f - z);
    const float dn = d * (1.0f - z) * (1.0f - nn * nn);
    const float dr = dn * ghn * r * (1.0f - r);
    float *gi = dgif + (size_t)m * 3 * HID, *gh = dghf + (size_t)m * 3 * HID;
    bf *gib = dgib + (size_t)m * 3 * HID, *ghb = dghb + (size_t)m * 3 * HID;
    gi[c] = dr; gi[HID + c] = dz; gi[2 * HID + c] = dn;
    gh[c] = dr; gh[HID + c] = dz; gh[2 * HID + c] = dn * r;
    gib[c] = __float2bfloat16_rn(dr); gib[HID + c] = __float2bfloat16_rn(dz); gib[2 * HID + c] = __float2bfloat16_rn(dn);
    ghb[c] = __float2bfloat16_rn(dr); ghb[HID + c] = __float2bfloat16_rn(dz);
    ghb[2 * HID + c] = __float2bfloat16_rn(dn * r);
    dhpart[i] = d * z;
}

// Adam on the FP32 master parameters, then their BF16 copies
__global__ void k_adam(float *p, const float *g, float *m1, float *m2, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2, bf *pb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.0f - b1) * gi;
    const float b = b2 * m2[i] + (1.0f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float v = p[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    p[i] = v;
    pb[i] = __float2bfloat16_rn(v);
}

// out = o + bias over the 32 outputs of n flights
__global__ void k_add_bias(const float *o, const float *bias, uint32_t n, float *out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n * NOUT) out[i] = o[i] + bias[i % NOUT];
}

__global__ void k_to_bf16(const float *p, int n, bf *pb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pb[i] = __float2bfloat16_rn(p[i]);
}

// ---- features --------------------------------------------------------------------------
// 24 per flight: the mean SDF and its slope along the ray at the centres of eight
// equal parts of [near, far] (clamped to +-4), then t_max / 4, 10 x the local length
// scale at near, the conditioned value and derivative along the ray (clamped to +-4),
// the first-scatter flag, 10 x the amplitude, step / t_max and the mean at near.
__device__ __forceinline__ void features_one(const DevMedium *media, int n_media, const float4 *on, const float4 *df,
                                             const uint4 *sd, const float4 *pv, const uint32_t *mid, uint32_t i,
                                             float *feat)
{
    const uint32_t mi = mid ? mid[i] : 0u;
    const DevMedium &m = media[mi < (uint32_t)n_media ? mi : 0u];
    const float4 o = on[i], d = df[i];
    const float near_t = o.w, far_t = d.w, tm = fmaxf(far_t - near_t, 0.0f);
    float *f = feat + (size_t)i * NFEAT;
    for (int j = 0; j < NHIST; ++j) {
        const float t = near_t + ((float)j + 0.5f) * 0.125f * tm;
        const float x = o.x + t * d.x, y = o.y + t * d.y, z = o.z + t * d.z;
        int id;
        const float mv = mean_value(m, x, y, z, id);
        float g[3];
        if (m.mean_kind == GPIS_MEAN_SPHERE) {
            // float form of the sphere's gradient (mean_grad emulates the reference's double path)
            const float *c = m.mean_params;
            const float dx = x - c[0], dy = y - c[1], dz = z - c[2];
            const float inv = rsqrtf(dx * dx + dy * dy + dz * dz);
            g[0] = dx * inv; g[1] = dy * inv; g[2] = dz * inv;
        } else {
            mean_grad(m, x, y, z, g);
        }
        const float sl = g[0] * d.x + g[1] * d.y + g[2] * d.z;
        f[2 * j] = fminf(fmaxf(mv, -4.0f), 4.0f);
        f[2 * j + 1] = fminf(fmaxf(sl, -4.0f), 4.0f);
    }
    const float *q = m.ls_params;
    const bool varying = m.ls_kind != 0u || (m.flags & MF_MULTIRES);
    const float ls_here = varying ? q[0] + q[1] * sinf(q[2] * o.x) * cosf(q[3] * o.z) : 1.0f;
    const float ell = ls_here * m.l_aniso[0] * 1.41421356f;
    const bool first = (sd[i].z & GPIS_FLAG_FIRST_SCATTER) != 0u;
    const float4 p = pv ? pv[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float amp = m.sigma;
    if (m.n_oct > 1) {
        amp = 0.0f;
        for (int k = 0; k < (int)m.n_oct; ++k) amp += m.oct_sigma[k];
    }
    float step = tm / (float)m.min_step;
    if (m.step_size < step) step = m.step_size;
    int id;
    f[16] = tm * 0.25f;
    f[17] = 10.0f * ell;
    f[18] = first ? 0.0f : fminf(fmaxf(p.x, -4.0f), 4.0f);
    f[19] = first ? 0.0f : fminf(fmaxf(p.y * d.x + p.z * d.y + p.w * d.z, -4.0f), 4.0f);
    f[20] = first ? 1.0f : 0.0f;
    f[21] = 10.0f * amp;
    f[22] = tm > 0.0f ? fminf(step / tm, 1.0f) : 1.0f;
    f[23] = fminf(fmaxf(mean_value(m, o.x + near_t * d.x, o.y + near_t * d.y, o.z + near_t * d.z, id), -4.0f), 4.0f);
}

// n flights, or the live count in device memory (grid-stride)
__global__ void k_features(const DevMedium *media, int n_media, const float4 *on, const float4 *df, const uint4 *sd,
                           const float4 *pv, const uint32_t *mid, uint32_t n, const uint32_t *n_dev, float *feat)
{
    const uint32_t nl = n_dev ? min(*n_dev, n) : n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nl; i += gridDim.x * blockDim.x)
        features_one(media, n_media, on, df, sd, pv, mid, i, feat);
}

// ---- fused inference -------------------------------------------------------------------
// 4 warps x 16 flights per block; BF16 weights and FP32 biases in shared memory.
constexpr int kWeights = 3 * HID * NIN + 3 * HID * HID + WID * MLPIN + 2 * WID * WID + NOUT * WID;
constexpr int S_WIH = 0, S_WHH = S_WIH + 3 * HID * NIN, S_W1 = S_WHH + 3 * HID * HID, S_W2 = S_W1 + WID * MLPIN,
              S_W3 = S_W2 + WID * WID, S_W4 = S_W3 + WID * WID;
constexpr int kBiases = 6 * HID + 3 * WID + NOUT;

// b0, b1 of output tile nt and K tile kt of a [out][in] weight in shared memory
__device__ __forceinline__ void bfrag(const bf *w, int in, int nt, int kt, int gi, int ti, uint32_t &b0, uint32_t &b1)
{
    const uint32_t *row = reinterpret_cast<const uint32_t *>(w + (nt * 8 + gi) * in + kt * 16);
    b0 = row[ti];
    b1 = row[ti + 4];
}

// one dense layer: acc[NT][4] = A (KT K-tiles of fragments) * W^T
template <int NT, int KT>
__device__ __forceinline__ void dense(const uint32_t (&a)[KT][4], const bf *w, int in, int gi, int ti,
                                      float (&acc)[NT][4])
{
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < KT; ++kt) {
            uint32_t b0, b1;
            bfrag(w, in, nt, kt, gi, ti, b0, b1);
            mma_bf16(acc[nt], a[kt][0], a[kt][1], a[kt][2], a[kt][3], b0, b1);
        }
    }
}

// bias, GELU and the C -> A fragment reuse of a 64-wide layer
__device__ __forceinline__ void gelu_frag(float (&acc)[8][4], const float *bias, int ti, uint32_t (&a)[4][4])
{
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int nt = 2 * kt + h;
            const int c = nt * 8 + 2 * ti;
            const float v0 = gelu_fast(acc[nt][0] + bias[c]), v1 = gelu_fast(acc[nt][1] + bias[c + 1]);
            const float v2 = gelu_fast(acc[nt][2] + bias[c]), v3 = gelu_fast(acc[nt][3] + bias[c + 1]);
            a[kt][2 * h] = pack2f(v0, v1);
            a[kt][2 * h + 1] = pack2f(v2, v3);
        }
    }
}

// Persistent: each block loads the weights once and its warps walk 16-flight tiles.
__global__ void __launch_bounds__(128) k_propose(const bf *wb, const float *params, const float *feat,
                                                 const float4 *on, const float4 *df, uint32_t n_cap,
                                                 const uint32_t *n_dev, float4 *out)
{
    __shared__ __align__(16) bf sw[kWeights];
    __shared__ float sb[kBiases];
    const int tid = threadIdx.x;
    // weights: w_ih, w_hh, w1, w2, w3, w4 (each contiguous in the flat vector)
    const int src[6] = {O_WIH, O_WHH, O_W1, O_W2, O_W3, O_W4};
    const int dst[6] = {S_WIH, S_WHH, S_W1, S_W2, S_W3, S_W4};
    const int len[6] = {3 * HID * NIN, 3 * HID * HID, WID * MLPIN, WID * WID, WID * WID, NOUT * WID};
    for (int s = 0; s < 6; ++s)
        for (int k = tid; k < len[s]; k += blockDim.x) sw[dst[s] + k] = wb[src[s] + k];
    for (int k = tid; k < 3 * HID; k += blockDim.x) {
        sb[k] = params[O_BIH + k];
        sb[3 * HID + k] = params[O_BHH + k];
    }
    for (int k = tid; k < WID; k += blockDim.x) {
        sb[6 * HID + k] = params[O_B1 + k];
        sb[6 * HID + WID + k] = params[O_B2 + k];
        sb[6 * HID + 2 * WID + k] = params[O_B3 + k];
    }
    for (int k = tid; k < NOUT; k += blockDim.x) sb[6 * HID + 3 * WID + k] = params[O_B4 + k];
    __syncthreads();
    const int lane = tid & 31, gi = lane >> 2, ti = lane & 3;
    const uint32_t n = n_dev ? min(*n_dev, n_cap) : n_cap;
    const long tiles = ((long)n + 15) / 16;
    // the GRU's B fragments and this lane's gate biases stay in registers for every
    // tile: the recurrence would otherwise reload them from shared memory 8 times
    // per tile (the kernel is bound by those loads)
    uint32_t wih[12][2], whh[12][2][2];
    float brz[2][4][2], bin_[4][2], bhn_[4][2];
#pragma unroll
    for (int t = 0; t < 12; ++t) {
        bfrag(sw + S_WIH, NIN, t, 0, gi, ti, wih[t][0], wih[t][1]);
#pragma unroll
        for (int kt = 0; kt < 2; ++kt) bfrag(sw + S_WHH, HID, t, kt, gi, ti, whh[t][kt][0], whh[t][kt][1]);
    }
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int c = nt * 8 + 2 * ti + q;
            brz[0][nt][q] = sb[c] + sb[3 * HID + c];
            brz[1][nt][q] = sb[HID + c] + sb[3 * HID + HID + c];
            bin_[nt][q] = sb[2 * HID + c];
            bhn_[nt][q] = sb[3 * HID + 2 * HID + c];
        }
    for (long tile = (long)blockIdx.x * 4 + (tid >> 5); tile < tiles; tile += (long)gridDim.x * 4) {
    const long row0 = tile * 16;
    const long ra = min(row0 + gi, (long)n - 1), rb = min(row0 + gi + 8, (long)n - 1);
    const float *fa = feat + ra * NFEAT, *fb = feat + rb * NFEAT;
    const float *b1 = sb + 6 * HID, *b2 = b1 + WID, *b3 = b2 + WID, *b4 = b3 + WID;
    // GRU
    float h[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) h[nt][0] = h[nt][1] = h[nt][2] = h[nt][3] = 0.0f;
    for (int j = 0; j < NHIST; ++j) {
        uint32_t ha[2][4];
#pragma unroll
        for (int kt = 0; kt < 2; ++kt) {
            ha[kt][0] = pack2f(h[2 * kt][0], h[2 * kt][1]);
            ha[kt][1] = pack2f(h[2 * kt][2], h[2 * kt][3]);
            ha[kt][2] = pack2f(h[2 * kt + 1][0], h[2 * kt + 1][1]);
            ha[kt][3] = pack2f(h[2 * kt + 1][2], h[2 * kt + 1][3]);
        }
        const uint32_t xa0 = ti == 0 ? pack2f(fa[2 * j], fa[2 * j + 1]) : 0u;
        const uint32_t xa1 = ti == 0 ? pack2f(fb[2 * j], fb[2 * j + 1]) : 0u;
        float hn[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            float gr[4] = {0, 0, 0, 0}, gz[4] = {0, 0, 0, 0}, gin[4] = {0, 0, 0, 0}, ghn[4] = {0, 0, 0, 0};
            mma_bf16(gr, xa0, xa1, 0u, 0u, wih[nt][0], wih[nt][1]);
            mma_bf16(gz, xa0, xa1, 0u, 0u, wih[4 + nt][0], wih[4 + nt][1]);
            mma_bf16(gin, xa0, xa1, 0u, 0u, wih[8 + nt][0], wih[8 + nt][1]);
#pragma unroll
            for (int kt = 0; kt < 2; ++kt) {
                mma_bf16(gr, ha[kt][0], ha[kt][1], ha[kt][2], ha[kt][3], whh[nt][kt][0], whh[nt][kt][1]);
                mma_bf16(gz, ha[kt][0], ha[kt][1], ha[kt][2], ha[kt][3], whh[4 + nt][kt][0], whh[4 + nt][kt][1]);
                mma_bf16(ghn, ha[kt][0], ha[kt][1], ha[kt][2], ha[kt][3], whh[8 + nt][kt][0], whh[8 + nt][kt][1]);
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int q = e & 1;
                const float r = sigm_fast(gr[e] + brz[0][nt][q]);
                const float z = sigm_fast(gz[e] + brz[1][nt][q]);
                const float nn = tanh_fast(gin[e] + bin_[nt][q] + r * (ghn[e] + bhn_[nt][q]));
                hn[nt][e] = (1.0f - z) * nn + z * h[nt][e];
            }
        }
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) h[nt][e] = hn[nt][e];
    }
    // MLP input: [h (2 K tiles), globals (K tile 2: columns 32..39, zeros 40..47)]
    uint32_t u[3][4];
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
        u[kt][0] = pack2f(h[2 * kt][0], h[2 * kt][1]);
        u[kt][1] = pack2f(h[2 * kt][2], h[2 * kt][3]);
        u[kt][2] = pack2f(h[2 * kt + 1][0], h[2 * kt + 1][1]);
        u[kt][3] = pack2f(h[2 * kt + 1][2], h[2 * kt + 1][3]);
    }
    u[2][0] = pack2f(fa[16 + 2 * ti], fa[17 + 2 * ti]);
    u[2][1] = pack2f(fb[16 + 2 * ti], fb[17 + 2 * ti]);
    u[2][2] = 0u;
    u[2][3] = 0u;
    float acc[8][4];
    uint32_t y[4][4];
    dense<8, 3>(u, sw + S_W1, MLPIN, gi, ti, acc);
    gelu_frag(acc, b1, ti, y);
    dense<8, 4>(y, sw + S_W2, WID, gi, ti, acc);
    gelu_frag(acc, b2, ti, y);
    dense<8, 4>(y, sw + S_W3, WID, gi, ti, acc);
    gelu_frag(acc, b3, ti, y);
    float o[4][4];
    dense<4, 4>(y, sw + S_W4, WID, gi, ti, o);
    // per row (g: e = 0, 1; g + 8: e = 2, 3): the dominant component over the 4 lanes of the group
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        float best = -INFINITY, bm = 0.0f, bs = 1.0f;
        int bk = 0;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int k = 2 * ti + e;
            const float lg = o[0][2 * half + e] + b4[k];
            if (lg > best) {
                best = lg;
                bk = k;
                bm = sigm(o[1][2 * half + e] + b4[8 + k]);
                bs = softplus(o[2][2 * half + e] + b4[16 + k]) + 1e-3f;
            }
        }
#pragma unroll
        for (int off = 1; off < 4; off <<= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, off);
            const int ok = __shfl_xor_sync(0xffffffffu, bk, off);
            const float om = __shfl_xor_sync(0xffffffffu, bm, off);
            const float os = __shfl_xor_sync(0xffffffffu, bs, off);
            if (ob > best || (ob == best && ok < bk)) {
                best = ob;
                bk = ok;
                bm = om;
                bs = os;
            }
        }
        const float q = sigm(o[3][2 * half] + b4[24]);   // column 24 sits at lane t = 0
        const long r = row0 + gi + 8 * half;
        if (ti == 0 && r < (long)n) {
            const float4 a = on[r], b = df[r];
            const float tm = b.w - a.w;
            const float ua = fminf(fmaxf(bm - 3.0f * bs, 0.0f), 1.0f);
            const float ub = fminf(fmaxf(bm + 3.0f * bs, 0.0f), 1.0f);
            out[r] = make_float4(a.w + ua * tm, a.w + ub * tm, q, bm);
        }
    }
    }
}

// ---- fused inference on the tensor-memory path ------------------------------------------
// Each group of four warps walks 128-flight tiles: thread = flight = accumulator row.
// One GRU step is one N = 128, K = 48 product of the operand [bf16(h_{j-1}) | x_j | 0]
// with the gate matrix G, whose 128 rows are r, z (hidden and input weights side by
// side, so the product sums both parts), the input part of n (hidden columns zero) and
// the hidden part of n (input columns zero); the accumulator's four 32-column blocks
// are those pre-activations.  The MLP layers are N = 64, 64, 64, 32 products.  One
// thread of the group issues the MMAs; their completion arrives on the group's
// mbarrier, the epilogues (gates, GELU, the dominant component) read the accumulator
// rows with tcgen05.ld and write the next operand into shared memory.
//
// The GRU biases and the first layer's bias ride in the products: operand columns 34,
// 35 (GRU) and 40, 41 (first layer) hold 1.0, and the matching weight columns the
// bias split into two BF16 parts, hi = bf16(b) and lo = bf16(b - hi) (16 significant
// bits; those weight columns multiply zero inputs in the network, which has two
// inputs per step and 40 MLP inputs).  The other layers' biases are FP32 in shared memory.
constexpr int TC_KG = 48;  // GRU / first-layer operand width: 32 hidden + 16 input columns
constexpr uint32_t TC_GB = 0, TC_W1 = TC_GB + 128 * TC_KG * 2, TC_W2 = TC_W1 + WID * MLPIN * 2,
                   TC_W3 = TC_W2 + WID * WID * 2, TC_W4 = TC_W3 + WID * WID * 2, TC_WEND = TC_W4 + NOUT * WID * 2,
                   TC_A = 128 * TC_KG * 2, TC_Y = 128 * WID * 2, TC_GROUP = TC_A + TC_Y, TC_BIAS = (3 * WID + NOUT) * 4;
constexpr uint32_t tc_smem_bytes(int groups) { return TC_WEND + groups * TC_GROUP + TC_BIAS; }
constexpr uint32_t kTcWaitLimit = GPIS_PROPOSAL_WAIT_DEFAULT;

// the operand row chunk of 8 BF16 columns starting at column 8 kb of row `row`
__device__ __forceinline__ void put_chunk(unsigned char *tile, uint32_t row, uint32_t kb, uint32_t kdim, uint4 v)
{
    *reinterpret_cast<uint4 *>(tile + umma::tile_offset(row, kb * 8u, kdim)) = v;
}

// generic-proxy writes -> tensor core; group barrier; the group's first thread issues
// D = A B^T (K / 16 MMAs) and commits to `bar`; every thread waits (bounded) and the
// group agrees on the outcome, so that a time-out ends the tile loop of all 128
// threads together (false, `fail` set, `phase` left at the outstanding commit)
__device__ __forceinline__ bool tc_round(uint32_t gid, bool leader, uint32_t tmem, const unsigned char *a,
                                         const unsigned char *b, uint32_t kdim, uint32_t n, uint64_t *bar,
                                         uint32_t &phase, bool &fail, uint32_t wait_limit)
{
    umma::fence_async_smem();
    umma::fence_before_sync();
    umma::sync_or(1 + gid, 128, false);
    umma::fence_after_sync();
    if (leader) {
        for (uint32_t kb = 0; kb < kdim / 16; ++kb)
            umma::mma(tmem, umma::tile_desc(a, 0, kb, kdim), umma::tile_desc(b, 0, kb, kdim),
                      umma::idesc_bf16_m128(n), kb > 0);
        umma::commit(bar);
    }
    const bool done = umma::bar_wait(bar, phase, wait_limit);
    if (umma::sync_or(1 + gid, 128, !done)) {
        fail = true;
        return false;
    }
    phase ^= 1u;
    umma::fence_after_sync();
    return true;
}

// four FP32 values of shared memory; volatile, so that the loads stay in the loop
// (hoisted out of the tile loop, the biases would take 224 registers)
__device__ __forceinline__ float4 lds4(const float *p)
{
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0,%1,%2,%3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(umma::smem_u32(p)));
    return v;
}

// GELU of 64 accumulator columns (+ bias from shared memory, or none: the bias is in the
// product) into the next operand (K = 64)
__device__ __forceinline__ void tc_gelu64(uint32_t t, const float *bias, unsigned char *y, uint32_t row)
{
#pragma unroll
    for (uint32_t c0 = 0; c0 < 64; c0 += 32) {
        float v[32];
        umma::ld32(t + c0, v);
        if (bias) {
#pragma unroll
            for (uint32_t c = 0; c < 32; c += 4) {
                const float4 b = lds4(bias + c0 + c);
                v[c] += b.x;
                v[c + 1] += b.y;
                v[c + 2] += b.z;
                v[c + 3] += b.w;
            }
        }
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q) {
            uint32_t w[4];
#pragma unroll
            for (uint32_t e = 0; e < 4; ++e) {
                const uint32_t c = q * 8 + 2 * e;
                w[e] = pack2f(gelu_fast(v[c]), gelu_fast(v[c + 1]));
            }
            put_chunk(y, row, c0 / 8 + q, WID, make_uint4(w[0], w[1], w[2], w[3]));
        }
    }
}

// the two BF16 parts of a bias, hi = bf16(b) and lo = bf16(b - hi)
__device__ __forceinline__ bf bias_part(float b, uint32_t part)
{
    const bf hi = __float2bfloat16_rn(b);
    return part ? __float2bfloat16_rn(b - __bfloat162float(hi)) : hi;
}

template <int GROUPS>
__global__ void __launch_bounds__(128 * GROUPS, GROUPS == 1 ? 3 : 2) k_propose_tc(const bf *wb, const float *params,
                                                                         const float *feat, const float4 *on,
                                                                         const float4 *df, uint32_t n_cap,
                                                                         const uint32_t *n_dev, float4 *out,
                                                                         uint32_t *err, uint32_t wait_limit)
{
    extern __shared__ __align__(128) unsigned char tsm[];
    __shared__ __align__(8) uint64_t bars[GROUPS];
    __shared__ uint32_t tslot;
    const uint32_t tid = threadIdx.x, gid = tid >> 7, row = tid & 127u;
    unsigned char *gsh = tsm + TC_GB, *w1 = tsm + TC_W1, *w2 = tsm + TC_W2, *w3 = tsm + TC_W3, *w4 = tsm + TC_W4;
    unsigned char *A = tsm + TC_WEND + gid * TC_GROUP, *Y = A + TC_A;
    float *bm = reinterpret_cast<float *>(tsm + TC_WEND + GROUPS * TC_GROUP);  // b2, b3 (64), b4 (32)
    // gate matrix: rows r (0..31), z (32..63), n input (64..95), n hidden (96..127);
    // columns 0..31 hidden weights, 32, 33 input weights, 34, 35 the bias parts
    const bf zero = __float2bfloat16_rn(0.0f);
    for (uint32_t i = tid; i < 128u * TC_KG; i += blockDim.x) {
        const uint32_t r = i / TC_KG, k = i % TC_KG, g = r >> 5, u = r & 31u;
        bf v = zero;
        if (k < HID) {
            if (g != 2) v = wb[O_WHH + ((g == 3 ? 2u : g) * HID + u) * HID + k];
        } else if (k < HID + 2) {
            if (g != 3) v = wb[O_WIH + (g * HID + u) * NIN + (k - HID)];
        } else if (k < HID + 4) {
            const float b = g < 2 ? params[O_BIH + g * HID + u] + params[O_BHH + g * HID + u]
                                  : (g == 2 ? params[O_BIH + 2 * HID + u] : params[O_BHH + 2 * HID + u]);
            v = bias_part(b, k - HID - 2);
        }
        *reinterpret_cast<bf *>(gsh + umma::tile_offset(r, k, TC_KG)) = v;
    }
    // first layer: columns 0..39 weights, 40, 41 the bias parts, 42..47 zero
    for (uint32_t i = tid; i < WID * MLPIN; i += blockDim.x) {
        const uint32_t r = i / MLPIN, k = i % MLPIN;
        const bf v = k < 40 ? wb[O_W1 + i] : (k < 42 ? bias_part(params[O_B1 + r], k - 40) : zero);
        *reinterpret_cast<bf *>(w1 + umma::tile_offset(r, k, MLPIN)) = v;
    }
    for (uint32_t i = tid; i < WID * WID; i += blockDim.x) {
        *reinterpret_cast<bf *>(w2 + umma::tile_offset(i / WID, i % WID, WID)) = wb[O_W2 + i];
        *reinterpret_cast<bf *>(w3 + umma::tile_offset(i / WID, i % WID, WID)) = wb[O_W3 + i];
    }
    for (uint32_t i = tid; i < NOUT * WID; i += blockDim.x)
        *reinterpret_cast<bf *>(w4 + umma::tile_offset(i / WID, i % WID, WID)) = wb[O_W4 + i];
    for (uint32_t k = tid; k < WID; k += blockDim.x) {
        bm[k] = params[O_B2 + k];
        bm[WID + k] = params[O_B3 + k];
    }
    for (uint32_t k = tid; k < NOUT; k += blockDim.x) bm[2 * WID + k] = params[O_B4 + k];
    // operand columns 40..47: (1, 1, 0 ..) for every product (the GRU's weight columns
    // there are zero)
    const uint32_t one2 = pack2f(1.0f, 1.0f);
    put_chunk(A, row, 5, TC_KG, make_uint4(one2, 0u, 0u, 0u));
    if (tid < GROUPS) umma::bar_init(&bars[tid], 1);
    if (tid < 32) umma::tmem_alloc(&tslot, 128 * GROUPS);
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tslot + gid * 128u + (((tid >> 5) & 3u) << 21);  // lanes 32 (warp % 4) ..
    const bool leader = row == 0;
    uint64_t *bar = &bars[gid];
    const uint32_t n = n_dev ? min(*n_dev, n_cap) : n_cap;
    const uint32_t tiles = (n + 127u) / 128u;
    uint32_t phase = 0;
    bool fail = false;
    for (uint32_t tile = blockIdx.x * GROUPS + gid; tile < tiles; tile += gridDim.x * GROUPS) {
        const uint32_t r = tile * 128u + row;
        const float *fr = feat + (size_t)min(r, n - 1) * NFEAT;
        float h[HID];
#pragma unroll
        for (int u = 0; u < HID; ++u) h[u] = 0.0f;
        bool ok = true;
#pragma unroll 1
        for (int j = 0; j < NHIST && ok; ++j) {
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q)
                put_chunk(A, row, q, TC_KG,
                          make_uint4(pack2f(h[8 * q], h[8 * q + 1]), pack2f(h[8 * q + 2], h[8 * q + 3]),
                                     pack2f(h[8 * q + 4], h[8 * q + 5]), pack2f(h[8 * q + 6], h[8 * q + 7])));
            const float2 x = reinterpret_cast<const float2 *>(fr)[j];
            put_chunk(A, row, 4, TC_KG, make_uint4(pack2f(x.x, x.y), one2, 0u, 0u));
            ok = tc_round(gid, leader, tmem, A, gsh, TC_KG, 128, bar, phase, fail, wait_limit);
            if (!ok) break;
#pragma unroll
            for (uint32_t c0 = 0; c0 < HID; c0 += 8) {
                float v[32];
                umma::ld4x8(tmem + c0, tmem + 32 + c0, tmem + 64 + c0, tmem + 96 + c0, v);
#pragma unroll
                for (uint32_t i = 0; i < 8; ++i) {
                    const float rg = sigm_fast(v[i]);
                    const float zg = sigm_fast(v[8 + i]);
                    const float nn = tanh_fast(fmaf(rg, v[24 + i], v[16 + i]));
                    h[c0 + i] = fmaf(zg, h[c0 + i] - nn, nn);
                }
            }
        }
        if (!ok) break;
        // MLP input: [h | globals | 0]
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q)
            put_chunk(A, row, q, TC_KG,
                      make_uint4(pack2f(h[8 * q], h[8 * q + 1]), pack2f(h[8 * q + 2], h[8 * q + 3]),
                                 pack2f(h[8 * q + 4], h[8 * q + 5]), pack2f(h[8 * q + 6], h[8 * q + 7])));
        const float4 g0 = reinterpret_cast<const float4 *>(fr)[4], g1 = reinterpret_cast<const float4 *>(fr)[5];
        put_chunk(A, row, 4, TC_KG,
                  make_uint4(pack2f(g0.x, g0.y), pack2f(g0.z, g0.w), pack2f(g1.x, g1.y), pack2f(g1.z, g1.w)));
        if (!tc_round(gid, leader, tmem, A, w1, MLPIN, WID, bar, phase, fail, wait_limit)) break;
        tc_gelu64(tmem, nullptr, Y, row);
        if (!tc_round(gid, leader, tmem, Y, w2, WID, WID, bar, phase, fail, wait_limit)) break;
        tc_gelu64(tmem, bm, Y, row);
        if (!tc_round(gid, leader, tmem, Y, w3, WID, WID, bar, phase, fail, wait_limit)) break;
        tc_gelu64(tmem, bm + WID, Y, row);
        if (!tc_round(gid, leader, tmem, Y, w4, WID, NOUT, bar, phase, fail, wait_limit)) break;
        float o[32];
        umma::ld32(tmem, o);
#pragma unroll
        for (int c = 0; c < 28; c += 4) {
            const float4 b = lds4(bm + 2 * WID + c);
            o[c] += b.x;
            o[c + 1] += b.y;
            o[c + 2] += b.z;
            o[c + 3] += b.w;
        }
        // the dominant component: the first of the largest logits
        float best = -INFINITY, mlog = 0.0f, slog = 0.0f;
        bool found = false;
#pragma unroll
        for (int k = 0; k < NCOMP; ++k) {
            if (o[k] > best) {
                best = o[k];
                found = true;
                mlog = o[8 + k];
                slog = o[16 + k];
            }
        }
        const float bmean = found ? sigm(mlog) : 0.0f;
        const float bs = found ? softplus(slog) + 1e-3f : 1.0f;
        const float q = sigm(o[24]);
        if (r < n) {
            const float4 a = on[r], b = df[r];
            const float tm = b.w - a.w;
            const float ua = fminf(fmaxf(bmean - 3.0f * bs, 0.0f), 1.0f);
            const float ub = fminf(fmaxf(bmean + 3.0f * bs, 0.0f), 1.0f);
            out[r] = make_float4(a.w + ua * tm, a.w + ub * tm, q, bmean);
        }
    }
    // a group that gave up waits once more for the MMAs it committed before the
    // tensor memory is released, with the default bound whatever wait_limit was
    if (fail) {
        if (leader) atomicExch(err, 1u);
        umma::bar_wait(bar, phase, kTcWaitLimit);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (tid < 32) umma::tmem_free(tslot, 128 * GROUPS);
}

// ---- tcgen05 self-check --------------------------------------------------------------
// D[128 x N] = A[128 x K] B[N x K]^T through the tensor-memory path, one CTA: the
// operands staged in the K-major no-swizzle layout, K / 16 MMAs issued by one
// thread, completion on an mbarrier (bounded wait: err = 1 on time-out), the
// accumulator read back by the four warps (32 rows each).  N % 32 == 0, N <= 128,
// K % 16 == 0.
__global__ void __launch_bounds__(128) k_tc_gemm_check(const bf *A, const bf *B, uint32_t N, uint32_t K, float *D,
                                                        uint32_t *err)
{
    extern __shared__ __align__(128) unsigned char tc_smem[];
    bf *sa = reinterpret_cast<bf *>(tc_smem);
    bf *sbm = reinterpret_cast<bf *>(tc_smem + 128u * K * 2u);
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tslot;
    const uint32_t tid = threadIdx.x;
    for (uint32_t i = tid; i < 128u * K; i += 128u) sa[umma::tile_offset(i / K, i % K, K) / 2] = A[i];
    for (uint32_t i = tid; i < N * K; i += 128u) sbm[umma::tile_offset(i / K, i % K, K) / 2] = B[i];
    if (tid == 0) umma::bar_init(&bar, 1);
    if (tid < 32) umma::tmem_alloc(&tslot, 128);
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tslot;
    if (tid == 0) {
        for (uint32_t kb = 0; kb < K / 16; ++kb)
            umma::mma(tmem, umma::tile_desc(sa, 0, kb, K), umma::tile_desc(sbm, 0, kb, K), umma::idesc_bf16_m128(N),
                      kb > 0);
        umma::commit(&bar);
    }
    const bool ok = umma::bar_wait(&bar, 0, 1u << 24);
    umma::fence_after_sync();
    if (ok) {
        const uint32_t w = tid >> 5;
        for (uint32_t c0 = 0; c0 < N; c0 += 32) {
            float v[32];
            umma::ld32(tmem + ((w * 32u) << 16) + c0, v);
#pragma unroll
            for (int i = 0; i < 32; ++i) D[(size_t)tid * N + c0 + i] = v[i];
        }
    } else if (tid == 0) {
        atomicExch(err, 1u);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (tid < 32) umma::tmem_free(tmem, 128);
}

// ---- training GEMMs on the tensor cores --------------------------------------------------
// C(m, n) (+)= sum_k A(m, k) B(k, n) with the strides of Gemm, through tcgen05: one
// 128-thread CTA per 128-row tile of C, slice of 32 (or 16) columns and K chunk
// (ksplit), so that even these small GEMMs spread over the SMs.  Per 64-deep step of K
// the threads stage the A tile (128 x 64; rows beyond M are zero) and B^T (32 x 64) in the
// K-major no-swizzle layout, whatever the operands' strides in global memory; one thread
// issues the step's K = 16 MMAs into the tensor-memory accumulator (128 lanes x 32 FP32
// columns) and commits them to an mbarrier, which every thread waits for (bounded) before
// the next step overwrites the tiles.  The epilogue reads each thread's row (tcgen05.ld
// 32x32b) and stores, adds or, with several K chunks, atomically adds it into C.
// N % 16 == 0, N <= 128, K % 16 == 0.
constexpr int TCG_KC = 64, TCG_NMAX = 128;
constexpr uint32_t kTcgSmem = 128u * TCG_KC * 2u + 32u * TCG_KC * 2u;

__global__ void __launch_bounds__(128) k_gemm_tc(Gemm g, uint32_t wait_limit, uint32_t *err)
{
    extern __shared__ __align__(128) unsigned char gsm[];
    unsigned char *sa = gsm, *sb = gsm + 128u * TCG_KC * 2u;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tslot;
    const uint32_t tid = threadIdx.x;
    // the CTA's tile: 128 rows, a slice of 32 (or 16) columns, a K chunk
    const int N = g.N % 32 == 0 ? 32 : 16;
    const int nslices = g.N / N;
    const int kc = (int)(blockIdx.x % (unsigned)g.ksplit);
    const int rest = (int)(blockIdx.x / (unsigned)g.ksplit);
    const int n0 = (rest % nslices) * N, mt = rest / nslices;
    const long m0 = (long)mt * 128;
    const uint32_t cols = 32u;
    const int ktiles = g.K / 16;
    const int per = (ktiles + g.ksplit - 1) / g.ksplit;
    const int kt0 = kc * per, kt1 = min(ktiles, kt0 + per);
    if (tid == 0) umma::bar_init(&bar, 1);
    if (tid < 32) umma::tmem_alloc(&tslot, cols);
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tslot;
    const bf zero = __float2bfloat16_rn(0.0f);
    uint32_t phase = 0;
    bool fail = false, issued = false;
    for (int k16 = kt0; k16 < kt1; k16 += TCG_KC / 16) {
        const int kn = min(TCG_KC, (kt1 - k16) * 16);
        const long kbase = (long)k16 * 16;
        // operands contiguous along K (row-major activations, weights as [N][K]) move as
        // 16-byte core-matrix rows; the others element by element
        if (g.lak == 1 && g.lam % 8 == 0 && (reinterpret_cast<uintptr_t>(g.A) & 15u) == 0) {
            const int kq = kn / 8;
            for (int i = (int)tid; i < 128 * kq; i += 128) {
                const int r = i / kq, k = (i - r * kq) * 8;
                const long row = m0 + r;
                const uint4 v = row < g.M ? *reinterpret_cast<const uint4 *>(g.A + row * g.lam + kbase + k)
                                          : make_uint4(0u, 0u, 0u, 0u);
                *reinterpret_cast<uint4 *>(sa + umma::tile_offset((uint32_t)r, (uint32_t)k, TCG_KC)) = v;
            }
        } else {
            for (int i = (int)tid; i < 128 * kn; i += 128) {
                const int r = i / kn, k = i - r * kn;
                const long row = m0 + r;
                const bf v = row < g.M ? g.A[row * g.lam + (kbase + k) * g.lak] : zero;
                *reinterpret_cast<bf *>(sa + umma::tile_offset((uint32_t)r, (uint32_t)k, TCG_KC)) = v;
            }
        }
        if (g.lbk == 1 && g.lbn % 8 == 0 && (reinterpret_cast<uintptr_t>(g.B) & 15u) == 0) {
            const int kq = kn / 8;
            for (int i = (int)tid; i < N * kq; i += 128) {
                const int c = i / kq, k = (i - c * kq) * 8;
                *reinterpret_cast<uint4 *>(sb + umma::tile_offset((uint32_t)c, (uint32_t)k, TCG_KC)) =
                    *reinterpret_cast<const uint4 *>(g.B + (long)(n0 + c) * g.lbn + kbase + k);
            }
        } else {
            for (int i = (int)tid; i < N * kn; i += 128) {
                const int c = i / kn, k = i - c * kn;
                *reinterpret_cast<bf *>(sb + umma::tile_offset((uint32_t)c, (uint32_t)k, TCG_KC)) =
                    g.B[(kbase + k) * g.lbk + (long)(n0 + c) * g.lbn];
            }
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if (tid == 0) {
            for (int kb = 0; kb < kn / 16; ++kb)
                umma::mma(tmem, umma::tile_desc(sa, 0, (uint32_t)kb, TCG_KC), umma::tile_desc(sb, 0, (uint32_t)kb, TCG_KC),
                          umma::idesc_bf16_m128((uint32_t)N), issued || kb > 0);
            umma::commit(&bar);
        }
        issued = true;
        const bool done = umma::bar_wait(&bar, phase, wait_limit);
        if (umma::sync_or(1, 128, !done)) {
            fail = true;
            break;
        }
        phase ^= 1u;
        umma::fence_after_sync();
    }
    if (fail) {
        // wait (default bound) for the MMAs committed before the tensor memory is released
        if (tid == 0) atomicExch(err, 1u);
        umma::bar_wait(&bar, phase, kTcWaitLimit);
    } else if (issued) {
        const uint32_t w = tid >> 5;
        const long row = m0 + tid;
        float *c = g.C + row * g.ldc + n0;
        float v[32];
        umma::ld32(tmem + ((w * 32u) << 16), v);
        if (row < g.M) {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                if (j < N) {
                    if (g.ksplit > 1) atomicAdd(c + j, v[j]);
                    else if (g.accumulate) c[j] += v[j];
                    else c[j] = v[j];
                }
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (tid < 32) umma::tmem_free(tmem, cols);
}

}  // namespace prop
}  // namespace gpis

using namespace gpis::prop;

// ---- host objects ----------------------------------------------------------------------
struct gpis_proposal {
    float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;
    bf *pb = nullptr;
    uint32_t step = 0;
    cudaStream_t stream = nullptr;
    // activations of the unfused pass for a batch of `cap` flights
    uint32_t cap = 0;
    std::vector<void *> act;
    bf *xb = nullptr, *ub = nullptr, *hb = nullptr, *y1 = nullptr, *y2 = nullptr, *y3 = nullptr, *dob = nullptr,
       *dab = nullptr, *dgib = nullptr, *dghb = nullptr;
    float *h = nullptr, *gi = nullptr, *gh = nullptr, *r = nullptr, *z = nullptr, *nn = nullptr, *ghn = nullptr,
          *a1 = nullptr, *a2 = nullptr, *a3 = nullptr, *o = nullptr, *dof = nullptr, *dy = nullptr, *daf = nullptr,
          *du = nullptr, *dgif = nullptr, *dghf = nullptr, *dh = nullptr, *loss = nullptr;
    // fused inference: GPIS_PROPOSAL_KERNEL_*, resident blocks per SM of each form, and
    // the tensor-memory kernel's time-out flag (host-mapped, read by the next call)
    int kernel = GPIS_PROPOSAL_KERNEL_TC2;
    int sms = 1, per_sm_tc1 = 1, per_sm_tc2 = 1, per_sm_mma = 1;
    uint32_t *tc_err_host = nullptr, *tc_err_dev = nullptr;
    // polls of the tensor-memory kernel's completion wait per MMA round
    uint32_t wait_limit = GPIS_PROPOSAL_WAIT_DEFAULT;
};

namespace {

int cfail(cudaError_t e, const char *what)
{
    static thread_local char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return gpis_internal_set_error(GPIS_EIO, buf);
}

#define PTRY(expr, what)                                    \
    do {                                                    \
        cudaError_t e_ = (expr);                            \
        if (e_ != cudaSuccess) return cfail(e_, what);      \
    } while (0)

template <class T>
cudaError_t palloc(gpis_proposal *p, T *&ptr, size_t count)
{
    void *v = nullptr;
    cudaError_t e = cudaMalloc(&v, count * sizeof(T));
    if (e == cudaSuccess) p->act.push_back(v);
    ptr = static_cast<T *>(v);
    return e;
}

int ensure_batch(gpis_proposal *p, uint32_t n)
{
    if (n <= p->cap) return GPIS_OK;
    for (void *v : p->act) cudaFree(v);
    p->act.clear();
    p->cap = 0;
    const size_t N = n;
    PTRY(palloc(p, p->xb, N * NHIST * NIN), "allocate proposal activations");
    PTRY(palloc(p, p->ub, N * MLPIN), "allocate proposal activations");
    PTRY(palloc(p, p->hb, N * (NHIST + 1) * HID), "allocate proposal activations");
    PTRY(palloc(p, p->h, N * (NHIST + 1) * HID), "allocate proposal activations");
    PTRY(palloc(p, p->gi, N * 3 * HID), "allocate proposal activations");
    PTRY(palloc(p, p->gh, N * 3 * HID), "allocate proposal activations");
    for (float **q : {&p->r, &p->z, &p->nn, &p->ghn}) PTRY(palloc(p, *q, N * NHIST * HID), "allocate proposal activations");
    for (float **q : {&p->a1, &p->a2, &p->a3, &p->dy, &p->daf}) PTRY(palloc(p, *q, N * WID), "allocate proposal activations");
    for (bf **q : {&p->y1, &p->y2, &p->y3, &p->dab}) PTRY(palloc(p, *q, N * WID), "allocate proposal activations");
    PTRY(palloc(p, p->o, N * NOUT), "allocate proposal activations");
    PTRY(palloc(p, p->dof, N * NOUT), "allocate proposal activations");
    PTRY(palloc(p, p->dob, N * NOUT), "allocate proposal activations");
    PTRY(palloc(p, p->du, N * MLPIN), "allocate proposal activations");
    PTRY(palloc(p, p->dgif, N * 3 * HID), "allocate proposal activations");
    PTRY(palloc(p, p->dghf, N * 3 * HID), "allocate proposal activations");
    PTRY(palloc(p, p->dgib, N * 3 * HID), "allocate proposal activations");
    PTRY(palloc(p, p->dghb, N * 3 * HID), "allocate proposal activations");
    PTRY(palloc(p, p->dh, N * HID), "allocate proposal activations");
    PTRY(palloc(p, p->loss, 1), "allocate proposal activations");
    p->cap = n;
    return GPIS_OK;
}

// The training GEMMs: tcgen05 (k_gemm_tc) unless the proposal selects the warp-level
// mma.sync kernels (GPIS_PROPOSAL_KERNEL_MMA) or N is outside its shapes.
void gemm(gpis_proposal *p, cudaStream_t s, const bf *A, long lam, long lak, const bf *B, long lbk, long lbn, float *C,
          long ldc, int M, int N, int K, int accumulate, int ksplit = 1)
{
    Gemm g{A, lam, lak, B, lbk, lbn, C, ldc, M, N, K, accumulate, ksplit};
    if (p->kernel != GPIS_PROPOSAL_KERNEL_MMA && N % 16 == 0 && N <= TCG_NMAX) {
        const int nslices = N % 32 == 0 ? N / 32 : N / 16;
        const unsigned blocks = (unsigned)(((long)M + 127) / 128 * nslices * ksplit);
        k_gemm_tc<<<blocks, 128, kTcgSmem, s>>>(g, p->wait_limit, p->tc_err_dev);
        return;
    }
    const long warps = (long)(M / 16) * (N / 8) * ksplit;
    k_gemm<<<(unsigned)((warps + 3) / 4), 128, 0, s>>>(g);
}

inline unsigned nb(size_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

// the unfused forward over the batch: activations kept for backward; outputs o (+ b4 in k_loss)
void forward(gpis_proposal *p, const float *feat, uint32_t n, cudaStream_t s)
{
    const bf *wb = p->pb;
    k_prep<<<nb(n), 256, 0, s>>>(feat, n, p->xb, p->ub, p->h, p->hb);
    for (int j = 0; j < NHIST; ++j) {
        const bf *x = p->xb + (size_t)j * n * NIN;
        const bf *hb = p->hb + (size_t)j * n * HID;
        gemm(p, s, x, NIN, 1, wb + O_WIH, 1, NIN, p->gi, 3 * HID, n, 3 * HID, NIN, 0);
        gemm(p, s, hb, HID, 1, wb + O_WHH, 1, HID, p->gh, 3 * HID, n, 3 * HID, HID, 0);
        const size_t o = (size_t)j * n * HID;
        k_gru_cell<<<nb((size_t)n * HID), 256, 0, s>>>(p->gi, p->gh, p->p, p->h + o, n, p->r + o, p->z + o, p->nn + o,
                                                        p->ghn + o, p->h + o + (size_t)n * HID, p->hb + o + (size_t)n * HID,
                                                        j == NHIST - 1 ? p->ub : nullptr);
    }
    gemm(p, s, p->ub, MLPIN, 1, wb + O_W1, 1, MLPIN, p->a1, WID, n, WID, MLPIN, 0);
    k_bias_gelu<<<nb((size_t)n * WID), 256, 0, s>>>(p->a1, p->p + O_B1, n, WID, p->y1);
    gemm(p, s, p->y1, WID, 1, wb + O_W2, 1, WID, p->a2, WID, n, WID, WID, 0);
    k_bias_gelu<<<nb((size_t)n * WID), 256, 0, s>>>(p->a2, p->p + O_B2, n, WID, p->y2);
    gemm(p, s, p->y2, WID, 1, wb + O_W3, 1, WID, p->a3, WID, n, WID, WID, 0);
    k_bias_gelu<<<nb((size_t)n * WID), 256, 0, s>>>(p->a3, p->p + O_B3, n, WID, p->y3);
    gemm(p, s, p->y3, WID, 1, wb + O_W4, 1, WID, p->o, NOUT, n, NOUT, WID, 0);
}

int ksplit_for(uint32_t n) { return (int)std::max(1u, std::min(64u, n / 128)); }

// loss and gradient of the mean loss into p->g (zeroed here)
void backward(gpis_proposal *p, const float2 *tgt, uint32_t n, cudaStream_t s)
{
    const bf *wb = p->pb;
    float *G = p->g;
    const int ks = ksplit_for(n);
    cudaMemsetAsync(G, 0, N_PARAMS * sizeof(float), s);
    cudaMemsetAsync(p->loss, 0, sizeof(float), s);
    k_loss<<<nb(n), 256, 0, s>>>(p->o, p->p + O_B4, tgt, n, 1.0f / (float)n, p->dof, p->dob, p->loss);
    // output layer
    gemm(p, s, p->dob, 1, NOUT, p->y3, WID, 1, G + O_W4, WID, NOUT, WID, n, 1, ks);
    k_colsum<<<64, 256, 0, s>>>(p->dof, n, NOUT, NOUT, G + O_B4);
    gemm(p, s, p->dob, NOUT, 1, wb + O_W4, WID, 1, p->dy, WID, n, WID, NOUT, 0);
    // hidden layers 3, 2, 1
    const float *acts[3] = {p->a3, p->a2, p->a1};
    const bf *ins[3] = {p->y2, p->y1, p->ub};
    const int ow[3] = {O_W3, O_W2, O_W1}, ob[3] = {O_B3, O_B2, O_B1}, inw[3] = {WID, WID, MLPIN};
    for (int l = 0; l < 3; ++l) {
        k_gelu_back<<<nb((size_t)n * WID), 256, 0, s>>>(p->dy, acts[l], n, WID, p->daf, p->dab);
        gemm(p, s, p->dab, 1, WID, ins[l], inw[l], 1, G + ow[l], inw[l], WID, inw[l], n, 1, ks);
        k_colsum<<<64, 256, 0, s>>>(p->daf, n, WID, WID, G + ob[l]);
        if (l < 2) gemm(p, s, p->dab, WID, 1, wb + ow[l], WID, 1, p->dy, WID, n, WID, WID, 0);
        else gemm(p, s, p->dab, WID, 1, wb + ow[l], MLPIN, 1, p->du, MLPIN, n, MLPIN, WID, 0);
    }
    // GRU, through time
    const float *dh = p->du;
    long ldh = MLPIN;
    for (int j = NHIST - 1; j >= 0; --j) {
        const size_t o = (size_t)j * n * HID;
        k_gru_back<<<nb((size_t)n * HID), 256, 0, s>>>(dh, ldh, p->r + o, p->z + o, p->nn + o, p->ghn + o, p->h + o,
                                                        n, p->dgif, p->dgib, p->dghf, p->dghb, p->dh);
        const bf *x = p->xb + (size_t)j * n * NIN;
        const bf *hb = p->hb + o;
        gemm(p, s, p->dgib, 1, 3 * HID, x, NIN, 1, G + O_WIH, NIN, 3 * HID, NIN, n, 1, ks);
        gemm(p, s, p->dghb, 1, 3 * HID, hb, HID, 1, G + O_WHH, HID, 3 * HID, HID, n, 1, ks);
        k_colsum<<<64, 192, 0, s>>>(p->dgif, n, 3 * HID, 3 * HID, G + O_BIH);
        k_colsum<<<64, 192, 0, s>>>(p->dghf, n, 3 * HID, 3 * HID, G + O_BHH);
        gemm(p, s, p->dghb, 3 * HID, 1, wb + O_WHH, HID, 1, p->dh, HID, n, HID, 3 * HID, 1);
        dh = p->dh;
        ldh = HID;
    }
}

// Resident blocks per SM of a kernel with `dyn` bytes of dynamic shared memory (opted in
// above 48 KB, with the shared-memory carveout at its maximum); at least 1.  Kernels
// without tensor memory take the occupancy API's answer.  For the tensor-memory
// kernels the count follows from their resources: registers (allocated per warp in
// units of 256), shared memory (1 KB reserved per block), threads, and the 512
// tensor-memory columns of an SM (the occupancy API answers 1 for them, which would
// leave half of the SM's register file and shared memory idle).
int resident_blocks(const void *fn, int threads, uint32_t dyn, int dev, int tmem_cols)
{
    cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    if (dyn > 48u * 1024u) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    int n = 0;
    if (tmem_cols > 0 || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, dyn) != cudaSuccess ||
        n < 1) {
        cudaFuncAttributes a{};
        int smem = 0, regs = 0, max_threads = 0;
        cudaFuncGetAttributes(&a, fn);
        cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&regs, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&max_threads, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
        const long warps = (threads + 31) / 32;
        const long per_warp = (((long)std::max(a.numRegs, 1) * 32 + 255) / 256) * 256;
        const long per_block = (long)dyn + (long)a.sharedSizeBytes + 1024;
        long m = std::min<long>(regs / (per_warp * warps), smem / per_block);
        m = std::min<long>(m, max_threads / threads);
        if (tmem_cols > 0) m = std::min<long>(m, 512 / tmem_cols);
        n = (int)m;
    }
    cudaGetLastError();
    return std::max(n, 1);
}

// The fused inference launch: the tensor-memory kernel (two 128-flight groups or one
// per block) unless the proposal selects the warp-MMA kernel or the features are not
// 16-byte aligned (the tensor-memory kernel reads feature rows as float4).  A time-out
// recorded by an earlier tensor-memory launch is reported here.
int launch_infer(gpis_proposal *p, const gpis_flight_soa *in, const float *features, float *intervals, uint32_t cap,
                 const uint32_t *n_dev, cudaStream_t s)
{
    volatile uint32_t *flag = p->tc_err_host;   // written by the device through the mapping
    if (*flag) {
        *flag = 0;
        return gpis_internal_set_error(GPIS_EIO, "proposal inference: tensor-core completion wait timed out");
    }
    const float4 *on = reinterpret_cast<const float4 *>(in->origin_near);
    const float4 *df = reinterpret_cast<const float4 *>(in->dir_far);
    float4 *out = reinterpret_cast<float4 *>(intervals);
    int kernel = p->kernel;
    if (reinterpret_cast<uintptr_t>(features) & 15u) kernel = GPIS_PROPOSAL_KERNEL_MMA;
    if (kernel == GPIS_PROPOSAL_KERNEL_MMA) {
        const unsigned blocks = (unsigned)std::min<long>(((long)cap + 63) / 64, (long)p->sms * p->per_sm_mma);
        k_propose<<<blocks, 128, 0, s>>>(p->pb, p->p, features, on, df, cap, n_dev, out);
    } else if (kernel == GPIS_PROPOSAL_KERNEL_TC1) {
        const unsigned blocks = (unsigned)std::min<long>(((long)cap + 127) / 128, (long)p->sms * p->per_sm_tc1);
        k_propose_tc<1><<<blocks, 128, tc_smem_bytes(1), s>>>(p->pb, p->p, features, on, df, cap, n_dev, out,
                                                              p->tc_err_dev, p->wait_limit);
    } else {
        const unsigned blocks = (unsigned)std::min<long>(((long)cap + 255) / 256, (long)p->sms * p->per_sm_tc2);
        k_propose_tc<2><<<blocks, 256, tc_smem_bytes(2), s>>>(p->pb, p->p, features, on, df, cap, n_dev, out,
                                                              p->tc_err_dev, p->wait_limit);
    }
    PTRY(cudaGetLastError(), "proposal inference kernel");
    return GPIS_OK;
}

}  // namespace

extern "C" {

uint32_t gpis_proposal_n_params(void) { return (uint32_t)N_PARAMS; }

void gpis_proposal_destroy(gpis_proposal *p)
{
    if (!p) return;
    if (p->tc_err_host) cudaFreeHost(p->tc_err_host);
    for (void *v : p->act) cudaFree(v);
    cudaFree(p->p);
    cudaFree(p->g);
    cudaFree(p->m1);
    cudaFree(p->m2);
    cudaFree(p->pb);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

int gpis_proposal_set_params(gpis_proposal *p, const float *params)
{
    if (!p || !params) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    PTRY(cudaMemcpy(p->p, params, N_PARAMS * sizeof(float), cudaMemcpyHostToDevice), "upload proposal parameters");
    k_to_bf16<<<nb(N_PARAMS), 256, 0, p->stream>>>(p->p, N_PARAMS, p->pb);
    PTRY(cudaMemsetAsync(p->m1, 0, N_PARAMS * sizeof(float), p->stream), "reset Adam state");
    PTRY(cudaMemsetAsync(p->m2, 0, N_PARAMS * sizeof(float), p->stream), "reset Adam state");
    p->step = 0;
    PTRY(cudaStreamSynchronize(p->stream), "set proposal parameters");
    return GPIS_OK;
}

int gpis_proposal_create(const float *params, gpis_proposal **out)
{
    if (!out) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    *out = nullptr;
    gpis_proposal *p = new gpis_proposal;
    // a blocking stream: the training kernels run after the work the caller queued on
    // the legacy default stream (the batch it gathered) and that stream's later work
    // (which may reuse the batch's memory) waits for them
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamDefault) != cudaSuccess ||
        cudaMalloc(&p->p, N_PARAMS * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&p->g, N_PARAMS * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&p->m1, N_PARAMS * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&p->m2, N_PARAMS * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&p->pb, N_PARAMS * sizeof(bf)) != cudaSuccess) {
        gpis_proposal_destroy(p);
        return gpis_internal_set_error(GPIS_ENOMEM, "allocate proposal parameters");
    }
    if (cudaHostAlloc(reinterpret_cast<void **>(&p->tc_err_host), sizeof(uint32_t), cudaHostAllocMapped) !=
            cudaSuccess ||
        cudaHostGetDevicePointer(reinterpret_cast<void **>(&p->tc_err_dev), p->tc_err_host, 0) != cudaSuccess) {
        gpis_proposal_destroy(p);
        return gpis_internal_set_error(GPIS_ENOMEM, "allocate proposal status flag");
    }
    *p->tc_err_host = 0;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, dev);
        p->per_sm_tc1 =
            resident_blocks(reinterpret_cast<const void *>(k_propose_tc<1>), 128, tc_smem_bytes(1), dev, 128);
        p->per_sm_tc2 =
            resident_blocks(reinterpret_cast<const void *>(k_propose_tc<2>), 256, tc_smem_bytes(2), dev, 256);
        p->per_sm_mma = resident_blocks(reinterpret_cast<const void *>(k_propose), 128, 0, dev, 0);
    }
    std::vector<float> zero;
    if (!params) {
        zero.assign(N_PARAMS, 0.0f);
        params = zero.data();
    }
    const int rc = gpis_proposal_set_params(p, params);
    if (rc) {
        gpis_proposal_destroy(p);
        return rc;
    }
    *out = p;
    return GPIS_OK;
}

int gpis_proposal_get_params(gpis_proposal *p, float *params)
{
    if (!p || !params) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    PTRY(cudaStreamSynchronize(p->stream), "synchronize proposal");
    PTRY(cudaMemcpy(params, p->p, N_PARAMS * sizeof(float), cudaMemcpyDeviceToHost), "read proposal parameters");
    return GPIS_OK;
}

// a tensor-core wait that ran out in an earlier call (inference or training): reported
// once, as GPIS_EIO
static int check_tc_flag(gpis_proposal *p)
{
    volatile uint32_t *flag = p->tc_err_host;
    if (*flag) {
        *flag = 0;
        return gpis_internal_set_error(GPIS_EIO, "proposal: tensor-core completion wait timed out");
    }
    return GPIS_OK;
}

static int check_batch(gpis_proposal *p, const float *feat, uint32_t n)
{
    if (!p || !feat) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    if (n == 0 || n % 16) return gpis_internal_set_error(GPIS_EINVAL, "the batch must be a positive multiple of 16");
    const int rc = check_tc_flag(p);
    if (rc) return rc;
    return ensure_batch(p, n);
}

int gpis_proposal_forward(gpis_proposal *p, const float *features, uint32_t n, float *outputs)
{
    int rc = check_batch(p, features, n);
    if (rc) return rc;
    if (!outputs) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    forward(p, features, n, p->stream);
    // the output bias (the loss kernel adds it in place during training)
    k_add_bias<<<nb((size_t)n * NOUT), 256, 0, p->stream>>>(p->o, p->p + O_B4, n, outputs);
    PTRY(cudaStreamSynchronize(p->stream), "proposal forward");
    PTRY(cudaGetLastError(), "proposal forward kernels");
    return check_tc_flag(p);
}

int gpis_proposal_gradient(gpis_proposal *p, const float *features, const float *targets, uint32_t n, float *grad,
                           float *loss)
{
    int rc = check_batch(p, features, n);
    if (rc) return rc;
    if (!targets || !grad) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    forward(p, features, n, p->stream);
    backward(p, reinterpret_cast<const float2 *>(targets), n, p->stream);
    PTRY(cudaStreamSynchronize(p->stream), "proposal gradient");
    PTRY(cudaGetLastError(), "proposal gradient kernels");
    rc = check_tc_flag(p);
    if (rc) return rc;
    PTRY(cudaMemcpy(grad, p->g, N_PARAMS * sizeof(float), cudaMemcpyDeviceToHost), "read gradient");
    float l = 0.0f;
    PTRY(cudaMemcpy(&l, p->loss, sizeof(float), cudaMemcpyDeviceToHost), "read loss");
    if (loss) *loss = l / (float)n;
    return GPIS_OK;
}

int gpis_proposal_train_step(gpis_proposal *p, const float *features, const float *targets, uint32_t n, float lr,
                             float *loss)
{
    int rc = check_batch(p, features, n);
    if (rc) return rc;
    if (!targets) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    cudaStream_t s = p->stream;
    forward(p, features, n, s);
    backward(p, reinterpret_cast<const float2 *>(targets), n, s);
    p->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)p->step), c2 = 1.0f - std::pow(b2, (float)p->step);
    k_adam<<<nb(N_PARAMS), 256, 0, s>>>(p->p, p->g, p->m1, p->m2, N_PARAMS, lr, b1, b2, 1e-8f, c1, c2, p->pb);
    PTRY(cudaGetLastError(), "proposal training kernels");
    if (loss) {
        float l = 0.0f;
        PTRY(cudaMemcpyAsync(&l, p->loss, sizeof(float), cudaMemcpyDeviceToHost, s), "read loss");
        PTRY(cudaStreamSynchronize(s), "proposal training step");
        *loss = l / (float)n;
        return check_tc_flag(p);
    }
    return GPIS_OK;
}

int gpis_debug_tc_gemm(const uint16_t *a_bf16, const uint16_t *b_bf16, uint32_t n, uint32_t k, float *d)
{
    if (!a_bf16 || !b_bf16 || !d) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    if (n == 0 || n > 128 || n % 32 || k == 0 || k > 128 || k % 16)
        return gpis_internal_set_error(GPIS_EINVAL, "n must be a multiple of 32 up to 128, k of 16 up to 128");
    void *da = nullptr, *db = nullptr, *dd = nullptr, *de = nullptr;
    const size_t sa = 128u * k * 2u, sbb = (size_t)n * k * 2u, sd = 128u * n * 4u;
    int rc = GPIS_OK;
    if (cudaMalloc(&da, sa) != cudaSuccess || cudaMalloc(&db, sbb) != cudaSuccess || cudaMalloc(&dd, sd) != cudaSuccess ||
        cudaMalloc(&de, 4) != cudaSuccess) {
        rc = gpis_internal_set_error(GPIS_ENOMEM, "allocate check buffers");
    } else {
        cudaMemcpy(da, a_bf16, sa, cudaMemcpyHostToDevice);
        cudaMemcpy(db, b_bf16, sbb, cudaMemcpyHostToDevice);
        cudaMemset(de, 0, 4);
        cudaFuncSetAttribute(k_tc_gemm_check, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sa + sbb));
        k_tc_gemm_check<<<1, 128, sa + sbb>>>(static_cast<const bf *>(da), static_cast<const bf *>(db), n, k,
                                              static_cast<float *>(dd), static_cast<uint32_t *>(de));
        uint32_t err = 0;
        cudaError_t e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(&err, de, 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(d, dd, sd, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cfail(e, "tensor-core check");
        else if (err) rc = gpis_internal_set_error(GPIS_EIO, "tensor-core check: MMA completion wait timed out");
    }
    cudaFree(da);
    cudaFree(db);
    cudaFree(dd);
    cudaFree(de);
    return rc;
}

int gpis_proposal_set_kernel(gpis_proposal *p, int kernel)
{
    if (!p) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    if (kernel != GPIS_PROPOSAL_KERNEL_TC2 && kernel != GPIS_PROPOSAL_KERNEL_TC1 && kernel != GPIS_PROPOSAL_KERNEL_MMA)
        return gpis_internal_set_error(GPIS_EINVAL, "unknown proposal kernel");
    p->kernel = kernel;
    return GPIS_OK;
}

int gpis_proposal_set_wait_limit(gpis_proposal *p, uint32_t polls)
{
    if (!p) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    p->wait_limit = polls;
    return GPIS_OK;
}

int gpis_proposal_occupancy(const gpis_proposal *p, int kernel)
{
    if (!p) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    if (kernel == GPIS_PROPOSAL_KERNEL_TC2) return p->per_sm_tc2;
    if (kernel == GPIS_PROPOSAL_KERNEL_TC1) return p->per_sm_tc1;
    if (kernel == GPIS_PROPOSAL_KERNEL_MMA) return p->per_sm_mma;
    return gpis_internal_set_error(GPIS_EINVAL, "unknown proposal kernel");
}

int gpis_proposal_infer(gpis_proposal *p, const gpis_flight_soa *in, const float *features, float *intervals,
                        uint32_t n, void *cuda_stream)
{
    if (!p || !in || !features || !intervals) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    if (n == 0) return GPIS_OK;
    if (!in->origin_near || !in->dir_far) return gpis_internal_set_error(GPIS_EINVAL, "origin_near and dir_far are required");
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    // the parameters are written on the proposal's own stream
    cudaEvent_t ev;
    PTRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "create event");
    cudaEventRecord(ev, p->stream);
    cudaStreamWaitEvent(s, ev, 0);
    cudaEventDestroy(ev);
    return launch_infer(p, in, features, intervals, n, nullptr, s);
}

// Inference on a batch whose live count is in device memory (the path tracer's
// rounds); the parameters must be quiescent (gpis_internal_proposal_quiesce).
__attribute__((visibility("hidden"))) int gpis_internal_infer_live(gpis_proposal *p, const gpis_flight_soa *in,
                                                                   const float *features, float *intervals,
                                                                   uint32_t cap, const uint32_t *n_dev,
                                                                   void *cuda_stream)
{
    if (!p || !in || !features || !intervals || !n_dev) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    if (cap == 0) return GPIS_OK;
    return launch_infer(p, in, features, intervals, cap, n_dev, static_cast<cudaStream_t>(cuda_stream));
}

__attribute__((visibility("hidden"))) int gpis_internal_proposal_quiesce(gpis_proposal *p)
{
    if (!p) return GPIS_EINVAL;
    PTRY(cudaStreamSynchronize(p->stream), "synchronize proposal");
    return GPIS_OK;
}

}  // extern "C"

namespace gpis {
cudaError_t launch_features(const DevMedium *media, int n_media, const gpis_flight_soa &in, uint32_t n, float *feat,
                            cudaStream_t s, const uint32_t *n_dev)
{
    if (n == 0) return cudaSuccess;
    unsigned blocks = (n + 127) / 128;
    if (n_dev) blocks = std::min(blocks, 4096u);
    k_features<<<blocks, 128, 0, s>>>(media, n_media, reinterpret_cast<const float4 *>(in.origin_near),
                                      reinterpret_cast<const float4 *>(in.dir_far),
                                      reinterpret_cast<const uint4 *>(in.seeds),
                                      reinterpret_cast<const float4 *>(in.prev), in.medium, n, n_dev, feat);
    return cudaGetLastError();
}
}  // namespace gpis
