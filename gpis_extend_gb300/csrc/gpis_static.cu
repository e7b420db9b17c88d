// gpis_static.cu -- gpis_flights_submit_static: the flight batch without any
// device allocation.
//
// Some callers of this library cannot call cudaMalloc.  A renderer's
// per-frame thread must not make the device synchronize, and cudaMalloc and
// cudaFree can do that.  Some plugin hosts also own every byte of device memory
// themselves and forbid plugins from allocating.  For them this entry point keeps
// all of its device working memory in one fixed array in this file, sized for at
// most GPIS_STATIC_MAX_FLIGHTS flights per call, which every GPU that loads the
// library holds until the process exits.  The caller still provides the flight
// and result streams.
#include <cmath>
#include <cstring>
#include <cstdint>
#include <mutex>

#include "../../include/gpis.h"
#include "flights.cuh"

namespace gpis {
int derive_medium_host(const gpis_medium_desc &d, DevMedium &m);
}

// error channel of the C ABI (gpis_abi.cu)
extern "C" int gpis_internal_set_error(int code, const char *msg);

namespace {

// Layout of the working array: the medium table, the work counters, the counter
// block, then the per-flight conditioning records, end parameters, saved march
// states, fast-pass set-up records and the two hand-off queues.
constexpr size_t kMax = GPIS_STATIC_MAX_FLIGHTS;
constexpr size_t kOffMedium = 0;
constexpr size_t kOffWork = 1024;
constexpr size_t kOffCounters = kOffWork + 256;
constexpr size_t kOffCond = kOffCounters + 256;
constexpr size_t kOffTEnd = kOffCond + kMax * sizeof(gpis::CondRec);
constexpr size_t kOffResume = kOffTEnd + kMax * sizeof(double);
constexpr size_t kOffSetup = kOffResume + kMax * sizeof(uint4);
constexpr size_t kOffQueue = kOffSetup + kMax * 4 * sizeof(float4);
constexpr size_t kBytes = kOffQueue + kMax * 2 * sizeof(uint32_t);
static_assert(sizeof(gpis::DevMedium) <= kOffWork, "medium table must fit its slot");
static_assert(gpis::kWorkCounters * sizeof(uint32_t) <= kOffCounters - kOffWork, "work counters must fit their slot");

// The working memory.  In host code this name is only a stand-in for the
// device array: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_scratch[kBytes];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
void *g_scratch_ptr[kMaxDevices] = {};

int fail(int code, const char *msg) { return gpis_internal_set_error(code, msg); }

// Writes the medium table into the working array from a kernel parameter, so no
// host staging buffer is involved.
__global__ void k_store_medium(gpis::DevMedium m, gpis::DevMedium *dst)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = m;
}

// One-time set-up per device, with that device current: the device address of
// the working array and the PCG jump table in constant memory.
int setup_device(int dev, void **ptr)
{
    std::lock_guard<std::mutex> g(g_lock);
    if (g_scratch_ptr[dev]) {
        *ptr = g_scratch_ptr[dev];
        return GPIS_OK;
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) return fail(GPIS_EIO, "cudaGetSymbolAddress of the static working array failed");
    e = gpis::upload_pcg_table();
    if (e != cudaSuccess) return fail(GPIS_EIO, "upload of the PCG jump table failed");
    g_scratch_ptr[dev] = p;
    *ptr = p;
    return GPIS_OK;
}

}  // namespace

extern "C" int gpis_flights_submit_static(const gpis_medium_desc *medium, const gpis_flight_soa *in,
                                          const gpis_result_soa *out, uint32_t n, void *cuda_stream)
{
    if (!medium || !in || !out) return fail(GPIS_EINVAL, "null argument");
    if (n > GPIS_STATIC_MAX_FLIGHTS)
        return fail(GPIS_ERANGE, "gpis_flights_submit_static takes at most GPIS_STATIC_MAX_FLIGHTS (65536) flights per call");
    if (n == 0) return GPIS_OK;
    if (!in->origin_near || !in->dir_far || !in->seeds || !out->rec)
        return fail(GPIS_EINVAL, "flight streams origin_near, dir_far, seeds and rec are required");
    // the kernels move these streams as 16-byte vectors: a misaligned pointer is
    // an error here, before anything is launched
    for (const void *p : {(const void *)in->origin_near, (const void *)in->dir_far, (const void *)in->seeds,
                          (const void *)in->prev, (const void *)out->rec})
        if (p && (reinterpret_cast<uintptr_t>(p) & 15u))
            return fail(GPIS_EINVAL, "flight and result streams must be 16-byte aligned");
    if (medium->mean_kind == GPIS_MEAN_GRID)
        return fail(GPIS_ENOTSUP, "a grid mean needs device memory; use gpis_ctx_create instead");
    gpis::DevMedium m;
    int rc = gpis::derive_medium_host(*medium, m);
    if (rc) return rc;
    const bool cond = (m.flags & gpis::MF_COND) != 0;
    if (cond && !in->prev) return fail(GPIS_EINVAL, "conditioning media need the prev stream");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return fail(GPIS_ENODEV, "no usable CUDA device");
    void *base = nullptr;
    rc = setup_device(dev, &base);
    if (rc) return rc;
    // the fast pass's persistent grid is the occupancy maximum (ctas_per_sm 0):
    // there is no context here to carry an autotuned value
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return fail(GPIS_ENODEV, "querying the device's multiprocessor count failed");
    char *b = static_cast<char *>(base);
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    // The array keeps the previous call's contents: the medium table is written
    // and the counters cleared before every launch.
    k_store_medium<<<1, 32, 0, s>>>(m, reinterpret_cast<gpis::DevMedium *>(b + kOffMedium));
    if (cudaGetLastError() != cudaSuccess || cudaMemsetAsync(b + kOffCounters, 0, sizeof(gpis_counters), s) != cudaSuccess)
        return fail(GPIS_EIO, "initialising the static working array failed");
    gpis::FlightArgs a = {};
    a.origin_near = reinterpret_cast<const float4 *>(in->origin_near);
    a.dir_far = reinterpret_cast<const float4 *>(in->dir_far);
    a.seeds = reinterpret_cast<const uint4 *>(in->seeds);
    a.prev = reinterpret_cast<const float4 *>(in->prev);
    a.medium = in->medium;
    a.out = reinterpret_cast<float4 *>(out->rec);
    a.media = reinterpret_cast<const gpis::DevMedium *>(b + kOffMedium);
    a.n_media = 1;
    a.n = n;
    a.cond = reinterpret_cast<gpis::CondRec *>(b + kOffCond);
    a.t_end = reinterpret_cast<double *>(b + kOffTEnd);
    a.work = reinterpret_cast<uint32_t *>(b + kOffWork);
    a.resume = reinterpret_cast<uint4 *>(b + kOffResume);
    a.setup = reinterpret_cast<float4 *>(b + kOffSetup);
    a.queue = reinterpret_cast<uint32_t *>(b + kOffQueue);
    a.counters = reinterpret_cast<unsigned long long *>(b + kOffCounters);
    a.any_cond = cond;
    a.one_d = (m.flags & gpis::MF_ONE_D) != 0;
    a.three_d = !a.one_d;
    a.max_imp = m.n_imp;
    a.max_oct = m.n_oct;
    a.all_grid = m.mean_kind == GPIS_MEAN_GRID;
    a.any_ns = m.ls_kind != 0u;
    a.any_mr = (m.flags & gpis::MF_MULTIRES) != 0u;
    a.any_gen3d = gpis::general_3d(m);
    if (gpis::launch_flights(a, sms, s) != cudaSuccess) return fail(GPIS_EIO, "launching the flight kernels failed");
    return GPIS_OK;
}
