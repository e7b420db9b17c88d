// gpis_abi.cu -- the C ABI of libgpis_gb300.so (include/gpis.h): medium
// tables, contexts, flight submission and the unit-level entry points.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/gpis.h"
#include "flights.cuh"

namespace {

thread_local std::string g_error;

int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    return fail(GPIS_EIO, "%s: %s", what, cudaGetErrorString(e));
}

#define CUDA_TRY(expr, what)                                 \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) return cuda_fail(_e, what);   \
    } while (0)

bool finite3(const float *v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

// Host derivation of the device medium constants.  Float expressions follow
// the reference's rounding: _l_conv = l * sqrt(2.f) / 2 (GPFunctions.cpp:661),
// _l_aniso_inv = 1 / (l_conv * aniso) with inf -> 0 (GPFunctions.hpp:153-162),
// kernel radii (GPFunctions.cpp:706-719) and the noise variances (:751-770).
int derive_medium(const gpis_medium_desc &d, gpis::DevMedium &m)
{
    std::memset(&m, 0, sizeof(m));
    if (!(std::isfinite(d.length_scale) && d.length_scale > 0.0f))
        return fail(GPIS_EINVAL, "length_scale must be finite and > 0");
    if (!(std::isfinite(d.kernel_scale) && d.kernel_scale > 0.0f))
        return fail(GPIS_EINVAL, "kernel_scale (localScale) must be finite and > 0");
    if (!(std::isfinite(d.impulse_density) && d.impulse_density > 0.0f && d.impulse_density <= 64.0f))
        return fail(GPIS_EINVAL, "impulse_density must be in (0, 64]");
    if (!(std::isfinite(d.step_size) && d.step_size > 0.0f))
        return fail(GPIS_EINVAL, "step_size must be finite and > 0");
    if (!std::isfinite(d.sigma) || !finite3(d.aniso))
        return fail(GPIS_EINVAL, "sigma and aniso must be finite");
    if (d.correlation_context > GPIS_CTX_NONE) return fail(GPIS_EINVAL, "unknown correlation_context");
    if (d.sampling_scheme > GPIS_SCHEME_MIS) return fail(GPIS_EINVAL, "unknown 1D_sampling_scheme");
    for (int i = 0; i < 8; ++i)
        if (!std::isfinite(d.mean_params[i])) return fail(GPIS_EINVAL, "mean parameters must be finite");
    if (d.n_octaves < 1 || d.n_octaves > 4) return fail(GPIS_EINVAL, "n_octaves must be in 1..4");
    if (d.ls_kind > GPIS_LS_SINCOS) return fail(GPIS_EINVAL, "unknown ls_kind");
    if (d.n_octaves != 1 && !d.one_d_sampling)
        return fail(GPIS_ENOTSUP, "multi-octave fields need 1D_sampling");
    if (d.ls_kind != GPIS_LS_CONSTANT) {
        if (!(std::isfinite(d.ls_max) && d.ls_max > 0.0f)) return fail(GPIS_EINVAL, "ls_max must be finite and > 0");
        for (int i = 0; i < 4; ++i)
            if (!std::isfinite(d.ls_params[i])) return fail(GPIS_EINVAL, "ls parameters must be finite");
    }
    // _multiResolutionGrid = !isStationaryKernel() && useMultiResolutionGrid() (SparseConvolutionNoise.cpp:47)
    const bool multires = d.multires && d.ls_kind != GPIS_LS_CONSTANT;
    if (multires) {
        if (d.n_octaves != 1) return fail(GPIS_ENOTSUP, "multi-resolution fields take one octave");
        const float lo = d.ls_params[0] - std::fabs(d.ls_params[1]), hi = d.ls_params[0] + std::fabs(d.ls_params[1]);
        if (!(lo > 0.0f) || !std::isfinite(hi))
            return fail(GPIS_EINVAL, "multi-resolution fields need ls(p) > 0 everywhere");
        const float lb = std::log(2.5f);
        if (std::floor(std::log(lo) / lb) < -gpis::kMrLevels || std::floor(std::log(hi) / lb) >= gpis::kMrLevels - 1)
            return fail(GPIS_ERANGE, "multi-resolution length scales outside 2.5^[-16, 15)");
    }
    if (d.n_octaves > 1)
        for (uint32_t k = 0; k < d.n_octaves; ++k)
            if (!std::isfinite(d.octave_sigma[k]) || !(std::isfinite(d.octave_scale[k]) && d.octave_scale[k] > 0.0f))
                return fail(GPIS_EINVAL, "octave sigma must be finite and octave scale finite and > 0");
    if (d.mean_kind > GPIS_MEAN_TORUS_PLANE) return fail(GPIS_EINVAL, "unknown mean kind");
    if (d.mean_kind == GPIS_MEAN_GRID) {
        const gpis_mean_grid *g = d.grid;
        if (!g || !g->voxels || g->dims[0] < 2 || g->dims[1] < 2 || g->dims[2] < 2)
            return fail(GPIS_EINVAL, "grid mean needs voxels and dims >= 2");
    }

    const float lc = d.length_scale * std::sqrt(2.f) / 2;
    for (int i = 0; i < 3; ++i) {
        m.l_aniso[i] = lc * d.aniso[i];
        float inv = 1.0f / m.l_aniso[i];
        if (std::isinf(inv) || std::isnan(inv)) inv = 0.0f;
        m.l_inv[i] = inv;
    }
    const float mtx = std::max(std::max(m.l_aniso[0], m.l_aniso[1]), m.l_aniso[2]);
    m.kr_iso = d.kernel_scale;
    m.kr_world = d.kernel_scale * 1.0f * mtx;
    m.sigma = d.sigma;
    m.n_imp = (uint32_t)d.impulse_density;
    m.var1d_c = d.impulse_density / m.kr_iso;
    const float var1 = (float)((double)m.var1d_c * (std::sqrt(M_PI) * 1.0));
    m.norm1d = std::sqrt(var1);
    m.inv_norm1d = 1.0f / m.norm1d;
    {
        // covarianceKernel1DVal(ab, 1) = exp(-(ab*ab / (2 * sqr(float(1 * sqrt(2)))))), GPFunctions.cpp:845-852
        const float s2 = (float)(1.0 * std::sqrt(2.0));
        m.cov_den2 = (float)(2.0 * (double)(s2 * s2));
    }
    const float kr = m.kr_world;
    const float ud = d.impulse_density / (kr * kr * kr);
    const float det = m.l_aniso[0] * m.l_aniso[1] * m.l_aniso[2];
    const float var3 = (float)((double)ud * (std::pow(M_PI, 1.5) * (double)det));
    m.norm3d = std::sqrt(var3);
    m.inv_norm3d = 1.0f / m.norm3d;
    const double log2e = 1.4426950408889634;
    m.kexp1d = (float)(-0.5 * (double)m.kr_iso * (double)m.kr_iso * log2e);
    for (int i = 0; i < 3; ++i) {
        const float inv2 = m.l_inv[i] * m.l_inv[i];
        m.m3[i] = inv2 * 0.5f;
        m.m3c[i] = (inv2 * 0.5f) * 0.5f;
        m.kexp3d[i] = (float)(-(double)m.m3[i] * log2e);
        m.d2inv3[i] = inv2 > 0.0f ? 1.0f / (-2.0f * (inv2 * 0.25f)) : 0.0f;
    }
    const bool activate = !d.single_realization &&
        (d.correlation_context == GPIS_CTX_RENEWAL || d.correlation_context == GPIS_CTX_RENEWAL_PLUS);
    uint32_t flags = 0;
    if (d.one_d_sampling) flags |= gpis::MF_ONE_D;
    if (activate) flags |= gpis::MF_COND;
    if (d.correlation_context == GPIS_CTX_RENEWAL_PLUS) flags |= gpis::MF_RENEWAL_PLUS;
    if (d.correlation_xy) flags |= gpis::MF_CORR_XY;
    // seTransverseGradientMoments applies to one stationary SE realization only
    if (d.one_d_sampling && d.correlation_xy && d.correlation_context == GPIS_CTX_RENEWAL_PLUS && !d.multires &&
        d.ls_kind == GPIS_LS_CONSTANT && d.n_octaves == 1)
        flags |= gpis::MF_TRANSVERSE;
    if (d.impulse_xyz_order) flags |= gpis::MF_XYZ_ORDER;
    if (multires) flags |= gpis::MF_MULTIRES;
    if (d.isotropic_3d_sampling && !d.one_d_sampling) flags |= gpis::MF_ISO3D;
    m.flags = flags;
    m.mean_kind = d.mean_kind;
    std::memcpy(m.mean_params, d.mean_params, sizeof(m.mean_params));
    if (d.mean_kind == GPIS_MEAN_GRID) {
        const gpis_mean_grid *g = d.grid;
        std::memcpy(m.grid_origin, g->origin, sizeof(m.grid_origin));
        std::memcpy(m.grid_dims, g->dims, sizeof(m.grid_dims));
        std::memcpy(m.grid_w2i, g->world_to_index, sizeof(m.grid_w2i));
        std::memcpy(m.grid_cmin, g->clamp_min, sizeof(m.grid_cmin));
        std::memcpy(m.grid_cmax, g->clamp_max, sizeof(m.grid_cmax));
        m.grid_offset = g->offset;
        m.grid_scale = g->scale;
    }
    m.ls_kind = multires ? 0u : d.ls_kind;
    for (int i = 0; i < 4; ++i) m.ls_params[i] = d.ls_params[i];
    m.ls_max = d.ls_kind != GPIS_LS_CONSTANT && !multires ? d.ls_max : 1.0f;
    // kernelScaleLevelRatio's float log / pow (SparseConvolutionNoise.cpp:101-111, 385),
    // evaluated by the float library at run time (no compile-time folding), as the
    // CPU restatement evaluates them
    volatile float base = 2.5f;
    m.mr_log_base = std::log((float)base);
    for (int l = -gpis::kMrLevels; l < gpis::kMrLevels; ++l) {
        const float sc = std::pow((float)base, (float)l);
        m.mr_pow[l + gpis::kMrLevels] = sc;
        m.mr_seed[l + gpis::kMrLevels] = (int32_t)std::floor(std::log(sc) / m.mr_log_base);
    }
    m.imp_density = d.impulse_density;
    m.ns3_seed = 0;
    if (d.ls_kind != GPIS_LS_CONSTANT && !multires)
        m.ns3_seed = (int32_t)std::floor(std::log((float)m.ls_max) / m.mr_log_base);
    m.n_oct = d.n_octaves;
    for (int k = 0; k < 4; ++k) {
        const bool on = (uint32_t)k < d.n_octaves && d.n_octaves > 1;
        m.oct_sigma[k] = on ? d.octave_sigma[k] : 0.0f;
        m.oct_scale[k] = on ? d.octave_scale[k] : 1.0f;
        m.oct_seed[k] = on ? d.octave_seed[k] : 0u;
        int ex = 0;
        const bool pow2 = std::frexp(m.oct_scale[k], &ex) == 0.5f;
        m.oct_inv[k] = 1.0f / m.oct_scale[k];
        if (pow2) m.oct_pow2 |= 1u << k;
    }
    // The mean's slope bound for step skipping (SDFs are 1-Lipschitz; a linear mean
    // has the slope of its scaled normal); not for multi-resolution media
    m.skip_mean_lip = -1.0f;
    if (!multires) {
        switch (d.mean_kind) {
        case GPIS_MEAN_SPHERE: case GPIS_MEAN_TORUS: case GPIS_MEAN_TORUS_PLANE: m.skip_mean_lip = 1.0f; break;
        case GPIS_MEAN_HOMOGENEOUS: m.skip_mean_lip = 0.0f; break;
        case GPIS_MEAN_PLANE:
            m.skip_mean_lip = (float)std::sqrt((double)d.mean_params[0] * d.mean_params[0] +
                                               (double)d.mean_params[1] * d.mean_params[1] +
                                               (double)d.mean_params[2] * d.mean_params[2]);
            break;
        case GPIS_MEAN_GRID: {
            // trilinear interpolation of the voxels: |dv/dq_a| <= the largest difference of
            // neighbours along a, and q = W p + t, so |d mean / dp| <= |scale| |W^T g| with
            // g_a that largest difference (clamping q only flattens the mean)
            const gpis_mean_grid *g = d.grid;
            const int nx = g->dims[0], ny = g->dims[1], nz = g->dims[2];
            double md[3] = {0.0, 0.0, 0.0};
            bool finite = true;
            for (int z = 0; z < nz && finite; ++z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x) {
                        const size_t i = ((size_t)z * ny + y) * nx + x;
                        const double v = g->voxels[i];
                        if (!std::isfinite(v)) { finite = false; break; }
                        if (x + 1 < nx) md[0] = std::max(md[0], std::fabs((double)g->voxels[i + 1] - v));
                        if (y + 1 < ny) md[1] = std::max(md[1], std::fabs((double)g->voxels[i + nx] - v));
                        if (z + 1 < nz) md[2] = std::max(md[2], std::fabs((double)g->voxels[i + (size_t)nx * ny] - v));
                    }
            if (!finite) break;
            double b = 0.0;
            for (int j = 0; j < 3; ++j) {
                double c = 0.0;
                for (int a = 0; a < 3; ++a) c += std::fabs((double)g->world_to_index[4 * a + j]) * md[a];
                b += c * c;
            }
            m.skip_mean_lip = (float)(std::fabs((double)g->scale) * std::sqrt(b) * 1.001);
            break;
        }
        default: break;
        }
    }
    m.skip_noise_lip = (float)(3.0 * m.n_imp * std::exp(-0.5) / (double)m.norm1d);
    m.skip_jump = (float)(std::exp(-0.5 * (double)m.kr_iso * m.kr_iso) / (double)m.norm1d);
    m.step_size = d.step_size;
    m.min_step = d.min_step;
    m.max_steps = d.max_steps ? d.max_steps : 16384u;
    if (m.max_steps > 0xFFFFFFu) return fail(GPIS_ERANGE, "max_steps must be below 2^24");
    m.scheme = (!d.single_realization && d.one_d_sampling) ? d.sampling_scheme : GPIS_SCHEME_UNI;
    return GPIS_OK;
}

}  // namespace

namespace gpis {
// Medium derivation for the allocation-free entry point (gpis_static.cu).
int derive_medium_host(const gpis_medium_desc &d, DevMedium &m) { return derive_medium(d, m); }
}  // namespace gpis

constexpr uint32_t kMaxChunks = 64;  // chunks of gpis_flights_trace_host's pipeline

struct gpis_ctx {
    int device = 0;
    int num_sms = 1;
    int n_media = 0;
    gpis::DevMedium *d_media = nullptr;
    std::vector<float *> d_grids;
    bool any_cond = false, all_one_d = true, all_three_d = true, all_grid = true, any_ns = false, any_mr = false,
         any_gen3d = false;
    uint32_t max_imp = 0, max_oct = 1;
    // scratch of the flight kernels
    gpis::CondRec *d_cond = nullptr;
    double *d_tend = nullptr;
    uint4 *d_resume = nullptr;
    float4 *d_setup = nullptr;
    uint32_t *d_queue = nullptr;
    uint32_t *d_work = nullptr;
    unsigned long long *d_counters = nullptr;
    size_t cap = 0;
    // staging of the host entry point
    char *d_stage = nullptr;
    size_t stage_cap = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t h2d_stream = nullptr, d2h_stream = nullptr;  // gpis_flights_trace_host's copies
    cudaStream_t stream2 = nullptr;                            // its second compute stream
    std::vector<cudaEvent_t> ev_chunks;
    // per-kernel event timing (gpis_profile_*)
    std::vector<gpis_medium_desc> host_media;  // host copies for the medium queries
    bool profiling = false;
    std::vector<cudaEvent_t> ev_pool;      // free events
    std::vector<cudaEvent_t> ev_pending;   // groups of 6 recorded events
    double prof_ms[3] = {0, 0, 0};
    uint64_t prof_launches[3] = {0, 0, 0};
    // schedule knobs (gpis_tune_set; 0 = default)
    uint64_t tune[7] = {0, 0, 0, 0, 0, 0, 0};
};

namespace {

void release(gpis_ctx *c)
{
    if (!c) return;
    cudaFree(c->d_media);
    for (float *g : c->d_grids) cudaFree(g);
    cudaFree(c->d_cond);
    cudaFree(c->d_tend);
    cudaFree(c->d_resume);
    cudaFree(c->d_setup);
    cudaFree(c->d_queue);
    cudaFree(c->d_work);
    cudaFree(c->d_counters);
    cudaFree(c->d_stage);
    for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : c->ev_pending) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->h2d_stream) cudaStreamDestroy(c->h2d_stream);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->d2h_stream) cudaStreamDestroy(c->d2h_stream);
    for (cudaEvent_t e : c->ev_chunks) cudaEventDestroy(e);
    delete c;
}

// page-locked host memory the device maps at the same address (the kernels can use
// the pointer as it is)
bool host_mapped(const void *p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost && a.devicePointer == p;
}

int ensure_scratch(gpis_ctx *c, size_t n)
{
    if (n <= c->cap) return GPIS_OK;
    size_t cap = std::max<size_t>(n, 1024);
    cudaFree(c->d_cond);
    cudaFree(c->d_tend);
    cudaFree(c->d_resume);
    cudaFree(c->d_setup);
    cudaFree(c->d_queue);
    c->d_cond = nullptr;
    c->d_tend = nullptr;
    c->d_resume = nullptr;
    c->d_setup = nullptr;
    c->d_queue = nullptr;
    c->cap = 0;
    CUDA_TRY(cudaMalloc(&c->d_cond, cap * sizeof(gpis::CondRec)), "allocate conditioning scratch");
    CUDA_TRY(cudaMalloc(&c->d_tend, cap * sizeof(double)), "allocate end-parameter scratch");
    CUDA_TRY(cudaMalloc(&c->d_resume, cap * sizeof(uint4)), "allocate resume scratch");
    CUDA_TRY(cudaMalloc(&c->d_setup, cap * 4 * sizeof(float4)), "allocate set-up scratch");
    CUDA_TRY(cudaMalloc(&c->d_queue, cap * 2 * sizeof(uint32_t)), "allocate hand-off queues");
    c->cap = cap;
    return GPIS_OK;
}

}  // namespace

extern "C" {

__attribute__((visibility("hidden"))) int gpis_internal_set_error(int code, const char *msg)
{
    g_error = msg ? msg : "";
    return code;
}

__attribute__((visibility("hidden"))) const gpis_medium_desc *gpis_internal_ctx_medium(gpis_ctx *ctx, uint32_t index)
{
    if (!ctx || index >= ctx->host_media.size()) return nullptr;
    return &ctx->host_media[index];
}

void gpis_medium_desc_init(gpis_medium_desc *d)
{
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    d->sigma = 1.0f;
    d->length_scale = 1.0f;
    d->aniso[0] = d->aniso[1] = d->aniso[2] = 1.0f;
    d->kernel_scale = 3.0f;
    d->ls_kind = GPIS_LS_CONSTANT;
    d->ls_params[0] = 1.0f;
    d->ls_max = 1.0f;
    d->n_octaves = 1;
    d->octave_sigma[0] = 1.0f;
    for (int i = 0; i < 4; ++i) d->octave_scale[i] = 1.0f;
    d->mean_kind = GPIS_MEAN_SPHERE;
    d->mean_params[3] = 1.0f;
    d->step_size = 0.01f;
    d->min_step = 8;
    d->seed = 0;
    d->impulse_density = 3.0f;
    d->correlation_context = GPIS_CTX_RENEWAL_PLUS;
    d->sampling_scheme = GPIS_SCHEME_UNI;
    d->density = 1.0f;
    d->max_bounces = 1024;
}

const char *gpis_last_error(void) { return g_error.c_str(); }

int gpis_ctx_create(const gpis_medium_desc *media, int n_media, gpis_ctx **out)
{
    if (!out) return fail(GPIS_EINVAL, "out is null");
    *out = nullptr;
    if (!media || n_media <= 0) return fail(GPIS_EINVAL, "need at least one medium");
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return fail(GPIS_ENODEV, "no CUDA device");
    std::vector<gpis::DevMedium> host((size_t)n_media);
    for (int i = 0; i < n_media; ++i) {
        int rc = derive_medium(media[i], host[(size_t)i]);
        if (rc) return fail(rc, "medium %d: %s", i, g_error.c_str());
    }
    gpis_ctx *c = new (std::nothrow) gpis_ctx();
    if (!c) return fail(GPIS_ENOMEM, "out of host memory");
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    c->n_media = n_media;
    c->host_media.assign(media, media + n_media);
    int rc = GPIS_OK;
    do {
        if ((e = gpis::upload_pcg_table()) != cudaSuccess) { rc = cuda_fail(e, "upload PCG table"); break; }
        for (int i = 0; i < n_media; ++i) {
            gpis::DevMedium &m = host[(size_t)i];
            if (m.mean_kind == GPIS_MEAN_GRID) {
                const gpis_mean_grid *g = media[i].grid;
                const size_t cnt = (size_t)g->dims[0] * g->dims[1] * g->dims[2];
                float *dg = nullptr;
                if ((e = cudaMalloc(&dg, cnt * sizeof(float))) != cudaSuccess) { rc = cuda_fail(e, "allocate grid"); break; }
                c->d_grids.push_back(dg);
                if ((e = cudaMemcpy(dg, g->voxels, cnt * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess) {
                    rc = cuda_fail(e, "upload grid");
                    break;
                }
                m.grid = dg;
                // corner table over the cells the clamps can reach, when it stays
                // small enough to live in L2 (32 MiB); a larger table would turn
                // the L2 hits of a grid that fits there into DRAM reads
                size_t cells = 1;
                for (int k = 0; k < 3; ++k) {
                    const double lo = std::floor((double)g->clamp_min[k]), hi = std::floor((double)g->clamp_max[k]);
                    const double span = hi - lo + 1.0;
                    if (!(span >= 1.0 && span < 2147483647.0 && lo > -2147483647.0)) { cells = 0; break; }
                    m.cell_lo[k] = (int32_t)lo;
                    m.cell_n[k] = (int32_t)span;
                    cells *= (size_t)span;
                }
                const size_t table = cells * 2 * sizeof(float4);
                if (cells && table <= ((size_t)32 << 20)) {
                    float4 *dc = nullptr;
                    if ((e = cudaMalloc(&dc, table)) != cudaSuccess) { rc = cuda_fail(e, "allocate grid corner table"); break; }
                    c->d_grids.push_back(reinterpret_cast<float *>(dc));
                    if ((e = gpis::launch_pack_grid(m, dc, cells, nullptr)) != cudaSuccess ||
                        (e = cudaDeviceSynchronize()) != cudaSuccess) {
                        rc = cuda_fail(e, "build grid corner table");
                        break;
                    }
                    m.grid_cells = dc;
                }
            }
            c->any_cond = c->any_cond || (m.flags & gpis::MF_COND);
            c->all_one_d = c->all_one_d && (m.flags & gpis::MF_ONE_D);
            c->all_three_d = c->all_three_d && !(m.flags & gpis::MF_ONE_D);
            c->max_imp = std::max(c->max_imp, m.n_imp);
            c->max_oct = std::max(c->max_oct, m.n_oct);
            c->all_grid = c->all_grid && m.mean_kind == GPIS_MEAN_GRID;
            c->any_ns = c->any_ns || m.ls_kind != 0u;
            c->any_mr = c->any_mr || (m.flags & gpis::MF_MULTIRES) != 0u;
            c->any_gen3d = c->any_gen3d || gpis::general_3d(m);
        }
        if (rc) break;
        if ((e = cudaMalloc(&c->d_media, host.size() * sizeof(gpis::DevMedium))) != cudaSuccess) { rc = cuda_fail(e, "allocate media"); break; }
        if ((e = cudaMemcpy(c->d_media, host.data(), host.size() * sizeof(gpis::DevMedium), cudaMemcpyHostToDevice)) != cudaSuccess) {
            rc = cuda_fail(e, "upload media");
            break;
        }
        if ((e = cudaMalloc(&c->d_work, gpis::kWorkCounters * kMaxChunks * sizeof(uint32_t))) != cudaSuccess) { rc = cuda_fail(e, "allocate work counters"); break; }
        if ((e = cudaMalloc(&c->d_counters, sizeof(gpis_counters))) != cudaSuccess) { rc = cuda_fail(e, "allocate counters"); break; }
        if ((e = cudaMemset(c->d_counters, 0, sizeof(gpis_counters))) != cudaSuccess) { rc = cuda_fail(e, "clear counters"); break; }
        if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) { rc = cuda_fail(e, "create stream"); break; }
        if ((e = cudaStreamCreateWithFlags(&c->h2d_stream, cudaStreamNonBlocking)) != cudaSuccess) { rc = cuda_fail(e, "create stream"); break; }
        if ((e = cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking)) != cudaSuccess) { rc = cuda_fail(e, "create stream"); break; }
        if ((e = cudaStreamCreateWithFlags(&c->d2h_stream, cudaStreamNonBlocking)) != cudaSuccess) { rc = cuda_fail(e, "create stream"); break; }
    } while (false);
    if (rc) {
        release(c);
        return rc;
    }
    *out = c;
    return GPIS_OK;
}

void gpis_ctx_destroy(gpis_ctx *ctx)
{
    if (!ctx) return;
    cudaDeviceSynchronize();
    release(ctx);
}

namespace {

// gpis_flights_submit on the scratch slice [offset, offset + n) with its own four
// work counters, so that batches on different streams may run at the same time
int submit_slice(gpis_ctx *ctx, const gpis_flight_soa *in, const gpis_result_soa *out, uint32_t n,
                 cudaStream_t stream, size_t offset, uint32_t *work, const float *proposal = nullptr,
                 const uint32_t *n_dev = nullptr)
{
    gpis::FlightArgs a = {};
    a.proposal = reinterpret_cast<const float4 *>(proposal);
    a.n_dev = n_dev;
    a.ctas_per_sm = (uint32_t)ctx->tune[GPIS_TUNE_MARCH_CTAS_PER_SM];
    a.prop_cap = ctx->tune[GPIS_TUNE_PROPOSED_SKIP_CAP] ? (uint32_t)ctx->tune[GPIS_TUNE_PROPOSED_SKIP_CAP] : 32u;
    a.fast_window = (uint32_t)ctx->tune[GPIS_TUNE_FAST_WINDOW];
    a.precise_only = (uint32_t)ctx->tune[GPIS_TUNE_PRECISE_DECISIONS];
    a.origin_near = reinterpret_cast<const float4 *>(in->origin_near);
    a.dir_far = reinterpret_cast<const float4 *>(in->dir_far);
    a.seeds = reinterpret_cast<const uint4 *>(in->seeds);
    a.prev = reinterpret_cast<const float4 *>(in->prev);
    a.medium = in->medium;
    a.out = reinterpret_cast<float4 *>(out->rec);
    a.media = ctx->d_media;
    a.n_media = ctx->n_media;
    a.n = n;
    a.cond = ctx->d_cond + offset;
    a.t_end = ctx->d_tend + offset;
    a.work = work;
    a.resume = ctx->d_resume + offset;
    a.setup = ctx->d_setup + 4 * offset;
    a.queue = ctx->d_queue + 2 * offset;
    a.counters = ctx->d_counters;
    a.any_cond = ctx->any_cond;
    a.one_d = ctx->all_one_d;
    a.three_d = ctx->all_three_d;
    a.max_imp = ctx->max_imp;
    a.max_oct = ctx->max_oct;
    a.all_grid = ctx->all_grid;
    a.any_ns = ctx->any_ns;
    a.any_mr = ctx->any_mr;
    a.any_gen3d = ctx->any_gen3d;
    for (const void *p : {(const void *)in->origin_near, (const void *)in->dir_far, (const void *)in->seeds,
                          (const void *)in->prev, (const void *)out->rec})
        if (p && (reinterpret_cast<uintptr_t>(p) & 15u))
            return fail(GPIS_EINVAL, "flight and result streams must be 16-byte aligned");
    cudaEvent_t *ev = nullptr;
    cudaEvent_t evs[6];
    if (ctx->profiling) {
        for (int k = 0; k < 6; ++k) {
            if (ctx->ev_pool.empty()) {
                cudaEvent_t e;
                CUDA_TRY(cudaEventCreate(&e), "create profiling event");
                ctx->ev_pool.push_back(e);
            }
            evs[k] = ctx->ev_pool.back();
            ctx->ev_pool.pop_back();
            ctx->ev_pending.push_back(evs[k]);
        }
        ev = evs;
    }
    CUDA_TRY(gpis::launch_flights(a, ctx->num_sms, stream, ev), "launch flights");
    if (ctx->profiling) {
        ctx->prof_launches[0] += a.any_cond ? 1 : 0;
        ctx->prof_launches[1] += 1;
        ctx->prof_launches[2] += 1;
    }
    return GPIS_OK;
}

}  // namespace

int gpis_flights_submit(gpis_ctx *ctx, const gpis_flight_soa *in, const gpis_result_soa *out, uint32_t n,
                        void *cuda_stream)
{
    if (!ctx || !in || !out) return fail(GPIS_EINVAL, "null argument");
    if (n == 0) return GPIS_OK;
    if (!in->origin_near || !in->dir_far || !in->seeds || !out->rec)
        return fail(GPIS_EINVAL, "flight streams origin_near, dir_far, seeds and rec are required");
    if (ctx->any_cond && !in->prev) return fail(GPIS_EINVAL, "conditioning media need the prev stream");
    int rc = ensure_scratch(ctx, n);
    if (rc) return rc;
    return submit_slice(ctx, in, out, n, static_cast<cudaStream_t>(cuda_stream), 0, ctx->d_work);
}

int gpis_flights_submit_proposed(gpis_ctx *ctx, const gpis_flight_soa *in, const float *intervals,
                                 const gpis_result_soa *out, uint32_t n, void *cuda_stream)
{
    if (!ctx || !in || !out || (n && !intervals)) return fail(GPIS_EINVAL, "null argument");
    if (n == 0) return GPIS_OK;
    if (!in->origin_near || !in->dir_far || !in->seeds || !out->rec)
        return fail(GPIS_EINVAL, "flight streams origin_near, dir_far and seeds and rec are required");
    if (ctx->any_cond && !in->prev) return fail(GPIS_EINVAL, "conditioning media need the prev stream");
    if (reinterpret_cast<uintptr_t>(intervals) & 15u) return fail(GPIS_EINVAL, "intervals must be 16-byte aligned");
    int rc = ensure_scratch(ctx, n);
    if (rc) return rc;
    return submit_slice(ctx, in, out, n, static_cast<cudaStream_t>(cuda_stream), 0, ctx->d_work, intervals);
}

// Flight and NEE batches whose live count sits in device memory (n_dev <= cap), for
// callers that capture whole rounds in a CUDA graph (the path tracer).
__attribute__((visibility("hidden"))) int gpis_internal_submit_live(gpis_ctx *ctx, const gpis_flight_soa *in,
                                                                    const gpis_result_soa *out, uint32_t cap,
                                                                    const uint32_t *n_dev, void *cuda_stream,
                                                                    const float *intervals)
{
    if (!ctx || !in || !out || !n_dev) return fail(GPIS_EINVAL, "null argument");
    if (cap == 0) return GPIS_OK;
    int rc = ensure_scratch(ctx, cap);
    if (rc) return rc;
    return submit_slice(ctx, in, out, cap, static_cast<cudaStream_t>(cuda_stream), 0, ctx->d_work, intervals, n_dev);
}

__attribute__((visibility("hidden"))) int gpis_internal_features_live(gpis_ctx *ctx, const gpis_flight_soa *in,
                                                                      float *features, uint32_t cap,
                                                                      const uint32_t *n_dev, void *cuda_stream)
{
    if (!ctx || !in || !features || !n_dev) return fail(GPIS_EINVAL, "null argument");
    CUDA_TRY(gpis::launch_features(ctx->d_media, ctx->n_media, *in, cap, features,
                                   static_cast<cudaStream_t>(cuda_stream), n_dev),
             "proposal features");
    return GPIS_OK;
}

__attribute__((visibility("hidden"))) int gpis_internal_nee_live(gpis_ctx *ctx, const gpis_nee_soa *in, float *out,
                                                                 uint32_t cap, const uint32_t *n_dev,
                                                                 void *cuda_stream)
{
    if (!ctx || !in || !out || !n_dev) return fail(GPIS_EINVAL, "null argument");
    if (cap == 0) return GPIS_OK;
    const gpis_flight_soa &f = in->flight;
    gpis::FlightArgs a = {};
    a.origin_near = reinterpret_cast<const float4 *>(f.origin_near);
    a.dir_far = reinterpret_cast<const float4 *>(f.dir_far);
    a.seeds = reinterpret_cast<const uint4 *>(f.seeds);
    a.prev = reinterpret_cast<const float4 *>(f.prev);
    a.medium = f.medium;
    a.media = ctx->d_media;
    a.n_media = ctx->n_media;
    a.n = cap;
    a.n_dev = n_dev;
    CUDA_TRY(gpis::launch_nee(a, reinterpret_cast<const float4 *>(in->point_t),
                              reinterpret_cast<const float4 *>(in->normal), reinterpret_cast<float4 *>(out),
                              static_cast<cudaStream_t>(cuda_stream)),
             "launch NEE");
    return GPIS_OK;
}

// SM count, whether per-kernel profiling is on, and whether a flight batch runs the
// prepare kernel (conditioning media, or the stationary cooperative fast pass's set-up)
int gpis_tune_set(gpis_ctx *ctx, uint32_t key, uint64_t value)
{
    if (!ctx) return fail(GPIS_EINVAL, "null context");
    if (key > GPIS_TUNE_PRECISE_DECISIONS) return fail(GPIS_EINVAL, "unknown schedule knob");
    if (key == GPIS_TUNE_HOST_DIRECT && value > 1) return fail(GPIS_ERANGE, "host direct mode is 0 or 1");
    if (key == GPIS_TUNE_FAST_WINDOW && value > 1) return fail(GPIS_ERANGE, "fast window is 0 or 1");
    if (key == GPIS_TUNE_PRECISE_DECISIONS && value > 1) return fail(GPIS_ERANGE, "precise decisions is 0 or 1");
    if (key == GPIS_TUNE_PROPOSED_SKIP_CAP && value && (value < 8 || value > 256))
        return fail(GPIS_ERANGE, "proposed skip cap must be in [8, 256]");
    if (key == GPIS_TUNE_MARCH_CTAS_PER_SM && value > 64) return fail(GPIS_ERANGE, "CTAs per SM must be <= 64");
    if (key == GPIS_TUNE_RENDER_PASS_PATHS && value && (value < 4096 || value > (1ull << 26)))
        return fail(GPIS_ERANGE, "render pass size must be in [4096, 2^26]");
    if (key == GPIS_TUNE_HOST_CHUNK && value && (value < 4096 || value > (1ull << 26)))
        return fail(GPIS_ERANGE, "host chunk must be in [4096, 2^26]");
    ctx->tune[key] = value;
    return GPIS_OK;
}

int gpis_tune_get(gpis_ctx *ctx, uint32_t key, uint64_t *value)
{
    if (!ctx || !value) return fail(GPIS_EINVAL, "null argument");
    if (key > GPIS_TUNE_PRECISE_DECISIONS) return fail(GPIS_EINVAL, "unknown schedule knob");
    *value = ctx->tune[key];
    return GPIS_OK;
}

__attribute__((visibility("hidden"))) uint32_t gpis_internal_render_pass(gpis_ctx *ctx)
{
    return ctx && ctx->tune[GPIS_TUNE_RENDER_PASS_PATHS] ? (uint32_t)ctx->tune[GPIS_TUNE_RENDER_PASS_PATHS]
                                                         : (1u << 22);
}

__attribute__((visibility("hidden"))) int gpis_internal_ctx_info(gpis_ctx *ctx, int *num_sms, int *profiling,
                                                                 int *prepare_runs)
{
    if (!ctx) return GPIS_EINVAL;
    if (num_sms) *num_sms = ctx->num_sms;
    if (profiling) *profiling = ctx->profiling ? 1 : 0;
    if (prepare_runs) {
        const bool coop_plain = ctx->all_one_d && ctx->max_imp <= 8 && ctx->max_oct == 1 && !ctx->any_ns &&
                                !ctx->all_grid && !ctx->any_mr;
        *prepare_runs = (ctx->any_cond || coop_plain) ? 1 : 0;
    }
    return GPIS_OK;
}

int gpis_proposal_features(gpis_ctx *ctx, const gpis_flight_soa *in, float *features, uint32_t n, void *cuda_stream)
{
    if (!ctx || !in || (n && !features)) return fail(GPIS_EINVAL, "null argument");
    if (n == 0) return GPIS_OK;
    if (!in->origin_near || !in->dir_far || !in->seeds)
        return fail(GPIS_EINVAL, "flight streams origin_near, dir_far and seeds are required");
    CUDA_TRY(gpis::launch_features(ctx->d_media, ctx->n_media, *in, n, features,
                                   static_cast<cudaStream_t>(cuda_stream)),
             "proposal features");
    return GPIS_OK;
}

int gpis_profile_enable(gpis_ctx *ctx, int on)
{
    if (!ctx) return fail(GPIS_EINVAL, "null context");
    ctx->profiling = on != 0;
    return GPIS_OK;
}

int gpis_profile_read(gpis_ctx *ctx, double ms[3], uint64_t launches[3], int reset)
{
    if (!ctx || !ms || !launches) return fail(GPIS_EINVAL, "null argument");
    for (size_t g = 0; g + 6 <= ctx->ev_pending.size(); g += 6) {
        for (int k = 0; k < 3; ++k) {
            CUDA_TRY(cudaEventSynchronize(ctx->ev_pending[g + 2 * k + 1]), "synchronize profiling event");
            float t = 0.0f;
            CUDA_TRY(cudaEventElapsedTime(&t, ctx->ev_pending[g + 2 * k], ctx->ev_pending[g + 2 * k + 1]),
                     "read profiling event");
            ctx->prof_ms[k] += t;
        }
    }
    for (cudaEvent_t e : ctx->ev_pending) ctx->ev_pool.push_back(e);
    ctx->ev_pending.clear();
    for (int k = 0; k < 3; ++k) {
        ms[k] = ctx->prof_ms[k];
        launches[k] = ctx->prof_launches[k];
    }
    if (reset)
        for (int k = 0; k < 3; ++k) { ctx->prof_ms[k] = 0.0; ctx->prof_launches[k] = 0; }
    return GPIS_OK;
}

int gpis_flights_trace_host(gpis_ctx *ctx, const gpis_flight_soa *in, const gpis_result_soa *out, uint32_t n)
{
    if (!ctx || !in || !out) return fail(GPIS_EINVAL, "null argument");
    if (n == 0) return GPIS_OK;
    if (!in->origin_near || !in->dir_far || !in->seeds || !out->rec)
        return fail(GPIS_EINVAL, "flight streams origin_near, dir_far, seeds and rec are required");
    if (ctx->tune[GPIS_TUNE_HOST_DIRECT] && host_mapped(in->origin_near) && host_mapped(in->dir_far) &&
        host_mapped(in->seeds) && (!in->prev || host_mapped(in->prev)) && (!in->medium || host_mapped(in->medium)) &&
        host_mapped(out->rec)) {
        // in place: the kernels read the flights and write the records over the host link
        int rc = ensure_scratch(ctx, n);
        if (rc) return rc;
        gpis_flight_soa din = *in;
        float *zero_prev = nullptr;
        if (!din.prev) {
            // the prev stream is read for every flight: zeros in the staging area
            const size_t need = (size_t)n * 16;
            if (need > ctx->stage_cap) {
                cudaFree(ctx->d_stage);
                ctx->d_stage = nullptr;
                ctx->stage_cap = 0;
                CUDA_TRY(cudaMalloc(&ctx->d_stage, need), "allocate staging");
                ctx->stage_cap = need;
            }
            zero_prev = reinterpret_cast<float *>(ctx->d_stage);
            CUDA_TRY(cudaMemsetAsync(zero_prev, 0, need, ctx->stream), "clear prev");
            din.prev = zero_prev;
        }
        rc = submit_slice(ctx, &din, out, n, ctx->stream, 0, ctx->d_work);
        if (rc) return rc;
        CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize flights");
        return GPIS_OK;
    }
    const size_t rec16 = (size_t)n * 16;
    const size_t need = rec16 * 4 + (size_t)n * 4 + 64 + rec16 * 2;
    if (need > ctx->stage_cap) {
        cudaFree(ctx->d_stage);
        ctx->d_stage = nullptr;
        ctx->stage_cap = 0;
        CUDA_TRY(cudaMalloc(&ctx->d_stage, need), "allocate staging");
        ctx->stage_cap = need;
    }
    char *base = ctx->d_stage;
    float *d_on = reinterpret_cast<float *>(base);
    float *d_df = reinterpret_cast<float *>(base + rec16);
    uint32_t *d_sd = reinterpret_cast<uint32_t *>(base + 2 * rec16);
    float *d_pv = reinterpret_cast<float *>(base + 3 * rec16);
    uint32_t *d_md = reinterpret_cast<uint32_t *>(base + 4 * rec16);
    float *d_rec = reinterpret_cast<float *>(base + ((4 * rec16 + (size_t)n * 4 + 63) & ~(size_t)63));
    // Pipelined in chunks: the copies of the next chunk in (one stream) and of the
    // previous chunk out (another) overlap the flight kernels, and the chunks'
    // kernels alternate between two compute streams on disjoint slices of the
    // scratch, so one chunk's tail overlaps the next chunk's start.
    const uint32_t chunk = ctx->tune[GPIS_TUNE_HOST_CHUNK] ? (uint32_t)ctx->tune[GPIS_TUNE_HOST_CHUNK] : (1u << 20);
    uint32_t per = n > 3 * (uint64_t)chunk ? chunk : n;
    if ((n + per - 1) / per > kMaxChunks) per = (n + kMaxChunks - 1) / kMaxChunks;
    const uint32_t chunks = (n + per - 1) / per;
    int rc0 = ensure_scratch(ctx, n);
    if (rc0) return rc0;
    while (ctx->ev_chunks.size() < 2 * (size_t)chunks) {
        cudaEvent_t e;
        CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "create chunk event");
        ctx->ev_chunks.push_back(e);
    }
    cudaStream_t s = ctx->stream, hs = ctx->h2d_stream, ds = ctx->d2h_stream;
    for (uint32_t k = 0; k < chunks; ++k) {
        const size_t o = (size_t)k * per, m = std::min<size_t>(per, n - o);
        const size_t b16 = m * 16;
        CUDA_TRY(cudaMemcpyAsync(d_on + 4 * o, in->origin_near + 4 * o, b16, cudaMemcpyHostToDevice, hs), "copy origins");
        CUDA_TRY(cudaMemcpyAsync(d_df + 4 * o, in->dir_far + 4 * o, b16, cudaMemcpyHostToDevice, hs), "copy directions");
        CUDA_TRY(cudaMemcpyAsync(d_sd + 4 * o, in->seeds + 4 * o, b16, cudaMemcpyHostToDevice, hs), "copy seeds");
        if (in->prev)
            CUDA_TRY(cudaMemcpyAsync(d_pv + 4 * o, in->prev + 4 * o, b16, cudaMemcpyHostToDevice, hs), "copy prev");
        else
            CUDA_TRY(cudaMemsetAsync(d_pv + 4 * o, 0, b16, hs), "clear prev");
        if (in->medium)
            CUDA_TRY(cudaMemcpyAsync(d_md + o, in->medium + o, m * 4, cudaMemcpyHostToDevice, hs), "copy media");
        CUDA_TRY(cudaEventRecord(ctx->ev_chunks[2 * k], hs), "record copy event");
        cudaStream_t cs = (k & 1) ? ctx->stream2 : s;
        CUDA_TRY(cudaStreamWaitEvent(cs, ctx->ev_chunks[2 * k], 0), "wait for copies");
        gpis_flight_soa din{d_on + 4 * o, d_df + 4 * o, d_sd + 4 * o, d_pv + 4 * o, in->medium ? d_md + o : nullptr};
        gpis_result_soa dout{d_rec + 8 * o};
        int rc = submit_slice(ctx, &din, &dout, (uint32_t)m, cs, o, ctx->d_work + gpis::kWorkCounters * k);
        if (rc) return rc;
        CUDA_TRY(cudaEventRecord(ctx->ev_chunks[2 * k + 1], cs), "record kernel event");
    }
    // results out after every chunk is enqueued: a copy to pageable memory blocks the
    // calling thread until it is done, which must not hold back the later chunks
    for (uint32_t k = 0; k < chunks; ++k) {
        const size_t o = (size_t)k * per, m = std::min<size_t>(per, n - o);
        CUDA_TRY(cudaStreamWaitEvent(ds, ctx->ev_chunks[2 * k + 1], 0), "wait for kernels");
        CUDA_TRY(cudaMemcpyAsync(out->rec + 8 * o, d_rec + 8 * o, 2 * m * 16, cudaMemcpyDeviceToHost, ds),
                 "copy results");
    }
    CUDA_TRY(cudaStreamSynchronize(ds), "synchronize flights");
    return GPIS_OK;
}

int gpis_nee_submit(gpis_ctx *ctx, const gpis_nee_soa *in, float *out, uint32_t n, void *cuda_stream)
{
    if (!ctx || !in || !out) return fail(GPIS_EINVAL, "null argument");
    if (n == 0) return GPIS_OK;
    const gpis_flight_soa &f = in->flight;
    if (!f.origin_near || !f.dir_far || !f.seeds || !in->point_t || !in->normal)
        return fail(GPIS_EINVAL, "streams origin_near, dir_far, seeds, point_t and normal are required");
    if (ctx->any_cond && !f.prev) return fail(GPIS_EINVAL, "conditioning media need the prev stream");
    for (const void *p : {(const void *)f.origin_near, (const void *)f.dir_far, (const void *)f.seeds,
                          (const void *)f.prev, (const void *)in->point_t, (const void *)in->normal, (const void *)out})
        if (p && (reinterpret_cast<uintptr_t>(p) & 15u)) return fail(GPIS_EINVAL, "NEE streams must be 16-byte aligned");
    gpis::FlightArgs a = {};
    a.origin_near = reinterpret_cast<const float4 *>(f.origin_near);
    a.dir_far = reinterpret_cast<const float4 *>(f.dir_far);
    a.seeds = reinterpret_cast<const uint4 *>(f.seeds);
    a.prev = reinterpret_cast<const float4 *>(f.prev);
    a.medium = f.medium;
    a.media = ctx->d_media;
    a.n_media = ctx->n_media;
    a.n = n;
    CUDA_TRY(gpis::launch_nee(a, reinterpret_cast<const float4 *>(in->point_t),
                              reinterpret_cast<const float4 *>(in->normal), reinterpret_cast<float4 *>(out),
                              static_cast<cudaStream_t>(cuda_stream)),
             "launch NEE");
    return GPIS_OK;
}

int gpis_nee_host(gpis_ctx *ctx, const gpis_nee_soa *in, float *out, uint32_t n)
{
    if (!ctx || !in || !out) return fail(GPIS_EINVAL, "null argument");
    if (n == 0) return GPIS_OK;
    const gpis_flight_soa &f = in->flight;
    if (!f.origin_near || !f.dir_far || !f.seeds || !in->point_t || !in->normal)
        return fail(GPIS_EINVAL, "streams origin_near, dir_far, seeds, point_t and normal are required");
    const size_t q16 = (size_t)n * 16;
    const size_t need = q16 * 7 + (((size_t)n * 4 + 15) & ~(size_t)15);
    if (need > ctx->stage_cap) {
        cudaFree(ctx->d_stage);
        ctx->d_stage = nullptr;
        ctx->stage_cap = 0;
        CUDA_TRY(cudaMalloc(&ctx->d_stage, need), "allocate staging");
        ctx->stage_cap = need;
    }
    char *b = ctx->d_stage;
    gpis_nee_soa d;
    d.flight.origin_near = reinterpret_cast<float *>(b);
    d.flight.dir_far = reinterpret_cast<float *>(b + q16);
    d.flight.seeds = reinterpret_cast<uint32_t *>(b + 2 * q16);
    d.flight.prev = reinterpret_cast<float *>(b + 3 * q16);
    d.point_t = reinterpret_cast<float *>(b + 4 * q16);
    d.normal = reinterpret_cast<float *>(b + 5 * q16);
    float *dout = reinterpret_cast<float *>(b + 6 * q16);
    d.flight.medium = f.medium ? reinterpret_cast<uint32_t *>(b + 7 * q16) : nullptr;
    cudaStream_t s = ctx->stream;
    CUDA_TRY(cudaMemcpyAsync((void *)d.flight.origin_near, f.origin_near, q16, cudaMemcpyHostToDevice, s), "copy origins");
    CUDA_TRY(cudaMemcpyAsync((void *)d.flight.dir_far, f.dir_far, q16, cudaMemcpyHostToDevice, s), "copy directions");
    CUDA_TRY(cudaMemcpyAsync((void *)d.flight.seeds, f.seeds, q16, cudaMemcpyHostToDevice, s), "copy seeds");
    if (f.prev)
        CUDA_TRY(cudaMemcpyAsync((void *)d.flight.prev, f.prev, q16, cudaMemcpyHostToDevice, s), "copy prev");
    else
        CUDA_TRY(cudaMemsetAsync((void *)d.flight.prev, 0, q16, s), "clear prev");
    CUDA_TRY(cudaMemcpyAsync((void *)d.point_t, in->point_t, q16, cudaMemcpyHostToDevice, s), "copy points");
    CUDA_TRY(cudaMemcpyAsync((void *)d.normal, in->normal, q16, cudaMemcpyHostToDevice, s), "copy normals");
    if (f.medium)
        CUDA_TRY(cudaMemcpyAsync((void *)d.flight.medium, f.medium, (size_t)n * 4, cudaMemcpyHostToDevice, s), "copy media");
    int rc = gpis_nee_submit(ctx, &d, dout, n, s);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(out, dout, q16, cudaMemcpyDeviceToHost, s), "copy NEE results");
    CUDA_TRY(cudaStreamSynchronize(s), "synchronize NEE");
    return GPIS_OK;
}

int gpis_status(gpis_ctx *ctx, gpis_counters *out, int reset)
{
    if (!ctx || !out) return fail(GPIS_EINVAL, "null argument");
    CUDA_TRY(cudaDeviceSynchronize(), "synchronize");
    CUDA_TRY(cudaMemcpy(out, ctx->d_counters, sizeof(gpis_counters), cudaMemcpyDeviceToHost), "read counters");
    if (reset) CUDA_TRY(cudaMemset(ctx->d_counters, 0, sizeof(gpis_counters)), "reset counters");
    return GPIS_OK;
}

static uint32_t h_xx1(uint32_t p)
{
    uint32_t h = p + 374761393u;
    h = 668265263u * ((h << 17) | (h >> 15));
    h = 2246822519u * (h ^ (h >> 15));
    h = 3266489917u * (h ^ (h >> 13));
    return h ^ (h >> 16);
}

static uint32_t h_xx4(uint32_t x, uint32_t y, uint32_t z, uint32_t w)
{
    uint32_t h = w + 374761393u + x * 3266489917u;
    h = 668265263u * ((h << 17) | (h >> 15));
    h += y * 3266489917u;
    h = 668265263u * ((h << 17) | (h >> 15));
    h += z * 3266489917u;
    h = 668265263u * ((h << 17) | (h >> 15));
    h = 2246822519u * (h ^ (h >> 15));
    h = 3266489917u * (h ^ (h >> 13));
    return h ^ (h >> 16);
}

void gpis_flight_seeds(const gpis_medium_desc *d, const uint32_t pss[4], uint32_t scene_seed,
                       uint32_t *noise_seed, uint32_t *normal_seed)
{
    if (!d || !pss) return;
    const uint32_t w = d->correlation_context == GPIS_CTX_GLOBAL ? 0u : pss[3];
    uint32_t seed = d->seed;
    if (!d->single_realization) seed += h_xx4(pss[0], pss[1], pss[2], w) + h_xx1(scene_seed);
    if (noise_seed) *noise_seed = seed;
    if (normal_seed) *normal_seed = h_xx4(pss[0], pss[1], pss[2], pss[3]) + h_xx1(scene_seed) + 1u;
}

int gpis_debug_exp(const float *x, float *y, uint32_t n)
{
    if (n && (!x || !y)) return fail(GPIS_EINVAL, "null argument");
    CUDA_TRY(gpis::launch_debug_exp(x, y, n, 0), "launch");
    CUDA_TRY(cudaDeviceSynchronize(), "synchronize");
    return GPIS_OK;
}

int gpis_debug_cells_1d(const uint32_t *cells, const uint32_t *seeds, uint32_t n, uint32_t impulses,
                        float *pos, float *weight)
{
    if (impulses > (uint32_t)gpis::kMaxImpulses) return fail(GPIS_ERANGE, "at most %d impulses", gpis::kMaxImpulses);
    if (n && (!cells || !seeds || !pos || !weight)) return fail(GPIS_EINVAL, "null argument");
    CUDA_TRY(gpis::upload_pcg_table(), "upload PCG table");
    CUDA_TRY(gpis::launch_debug_cells_1d(cells, seeds, n, impulses, pos, weight, 0), "launch");
    CUDA_TRY(cudaDeviceSynchronize(), "synchronize");
    return GPIS_OK;
}

int gpis_debug_cells_3d(const int32_t *cells, const uint32_t *seeds, uint32_t n, uint32_t impulses,
                        uint32_t xyz_order, float *pos, float *weight)
{
    if (impulses > (uint32_t)gpis::kMaxImpulses) return fail(GPIS_ERANGE, "at most %d impulses", gpis::kMaxImpulses);
    if (n && (!cells || !seeds || !pos || !weight)) return fail(GPIS_EINVAL, "null argument");
    CUDA_TRY(gpis::upload_pcg_table(), "upload PCG table");
    CUDA_TRY(gpis::launch_debug_cells_3d(cells, seeds, n, impulses, xyz_order, pos, weight, 0), "launch");
    CUDA_TRY(cudaDeviceSynchronize(), "synchronize");
    return GPIS_OK;
}

int gpis_debug_field(gpis_ctx *ctx, const float *origins, const float *points, const float *dirs,
                     const uint32_t *seeds, const float *prev, uint32_t n, float *out)
{
    if (!ctx) return fail(GPIS_EINVAL, "null context");
    if (n && (!origins || !points || !dirs || !seeds || !prev || !out)) return fail(GPIS_EINVAL, "null argument");
    CUDA_TRY(gpis::launch_debug_field(ctx->d_media, reinterpret_cast<const float4 *>(origins),
                                      reinterpret_cast<const float4 *>(points), reinterpret_cast<const float4 *>(dirs),
                                      reinterpret_cast<const uint4 *>(seeds), reinterpret_cast<const float4 *>(prev), n,
                                      reinterpret_cast<float4 *>(out), 0),
             "launch");
    CUDA_TRY(cudaDeviceSynchronize(), "synchronize");
    return GPIS_OK;
}

int gpis_se_splat_1d(const float *queries, const float *centers, float *values, float *derivatives, size_t count,
                     float local_scale, void *cuda_stream)
{
    if (!(std::isfinite(local_scale) && local_scale > 0.0f)) return fail(GPIS_EINVAL, "local_scale must be finite and > 0");
    if (count == 0) return GPIS_OK;
    if (!queries || !centers || !values || !derivatives) return fail(GPIS_EINVAL, "null argument");
    CUDA_TRY(gpis::launch_se_splat_1d(queries, centers, values, derivatives, count, local_scale,
                                      static_cast<cudaStream_t>(cuda_stream)),
             "launch");
    return GPIS_OK;
}

}  // extern "C"
