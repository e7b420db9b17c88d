// ref_gpu_runner.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Loads the reference's own GPU kernel, traceSegments of
// src/gpu/cuda/RaySegmentBatch.cu (compiled unmodified, device code only, to
// oracle/_ref/ray_segment_batch.cubin), through the CUDA driver API and
// launches it the way launchSe1DRaySegments does (RaySegmentBatch.cu:297-331:
// 128 threads per block, one thread per segment), so that tests can compare
// the reference GPU baseline with the flight kernels on the same flights and
// time it.  The argument structs restate the layouts of RaySegmentBatch.hpp:12-84
// (RaySegmentInput 64 B, RaySegmentOutput 32 B, DeviceMeanGrid 112 B,
// Se1DRayParameters 28 B).
#include <cuda.h>

#include <cstdint>
#include <cstring>
#include <string>

namespace {

struct RefInput {        // RaySegmentInput, RaySegmentBatch.hpp:42-53
    float origin[3];
    float direction[3];
    float near_t, far_t, jitter;
    uint32_t noise_seed, normal_seed, first_scatter;
    float prev_value;
    float prev_gradient[3];
};
static_assert(sizeof(RefInput) == 64, "RaySegmentInput layout");

struct RefOutput {       // RaySegmentOutput, RaySegmentBatch.hpp:61-68
    float t, value, gradient[3];
    uint32_t hit, steps, status;
};
static_assert(sizeof(RefOutput) == 32, "RaySegmentOutput layout");

struct RefGrid {         // DeviceMeanGrid, RaySegmentBatch.hpp:70-79
    CUdeviceptr voxels;
    int origin[3];
    int dims[3];
    float world_to_index[12];
    float clamp_min[3];
    float clamp_max[3];
    float offset;
    float scale;
};
static_assert(sizeof(RefGrid) == 112, "DeviceMeanGrid layout");

struct RefParams {       // Se1DRayParameters, RaySegmentBatch.hpp:32-40
    float length_scale, amplitude, kernel_radius, impulse_density, max_step_size;
    uint32_t min_steps, max_steps;
};
static_assert(sizeof(RefParams) == 28, "Se1DRayParameters layout");

CUmodule g_module = nullptr;
CUfunction g_trace = nullptr;
CUcontext g_ctx = nullptr;

}  // namespace

extern "C" {

// Load the cubin on device 0 (primary context) and find traceSegments.
// Returns 0, a CUresult, or -1 when the module has no traceSegments kernel.
int refgpu_init(const char *cubin_path)
{
    if (g_trace) return 0;
    CUresult r = cuInit(0);
    if (r != CUDA_SUCCESS) return (int)r;
    CUdevice dev;
    if ((r = cuDeviceGet(&dev, 0)) != CUDA_SUCCESS) return (int)r;
    if ((r = cuDevicePrimaryCtxRetain(&g_ctx, dev)) != CUDA_SUCCESS) return (int)r;
    if ((r = cuCtxSetCurrent(g_ctx)) != CUDA_SUCCESS) return (int)r;
    if ((r = cuModuleLoad(&g_module, cubin_path)) != CUDA_SUCCESS) return (int)r;
    unsigned int count = 0;
    if ((r = cuModuleGetFunctionCount(&count, g_module)) != CUDA_SUCCESS) return (int)r;
    CUfunction fns[64];
    if (count > 64) count = 64;
    if ((r = cuModuleEnumerateFunctions(fns, count, g_module)) != CUDA_SUCCESS) return (int)r;
    for (unsigned int i = 0; i < count; ++i) {
        const char *name = nullptr;
        if (cuFuncGetName(&name, fns[i]) == CUDA_SUCCESS && name && std::strstr(name, "traceSegments")) {
            g_trace = fns[i];
            return 0;
        }
    }
    return -1;
}

// Trace n segments (host AoS inputs/outputs) over a dense mean grid with
// `reps` timed launches on device-resident inputs; ms_kernel gets the mean
// launch time (CUDA events), ms_e2e one host-to-host pass (copies included).
int refgpu_run(const void *inputs, void *outputs, uint64_t n, const float *voxels, const int dims[3],
               const int origin[3], const float world_to_index[12], const float clamp_min[3],
               const float clamp_max[3], float offset, float scale, const float params_f[5],
               const uint32_t params_u[2], int reps, double *ms_kernel, double *ms_e2e)
{
    if (!g_trace) return -1;
    if (n == 0) return 0;
    CUresult r = cuCtxSetCurrent(g_ctx);
    if (r != CUDA_SUCCESS) return (int)r;
    const size_t nvox = (size_t)dims[0] * dims[1] * dims[2];
    CUdeviceptr d_in = 0, d_out = 0, d_vox = 0;
    CUevent e0 = nullptr, e1 = nullptr;
    int rc = 0;
    do {
        if ((r = cuMemAlloc(&d_in, n * sizeof(RefInput))) != CUDA_SUCCESS) break;
        if ((r = cuMemAlloc(&d_out, n * sizeof(RefOutput))) != CUDA_SUCCESS) break;
        if ((r = cuMemAlloc(&d_vox, nvox * sizeof(float))) != CUDA_SUCCESS) break;
        if ((r = cuMemcpyHtoD(d_vox, voxels, nvox * sizeof(float))) != CUDA_SUCCESS) break;
        if ((r = cuEventCreate(&e0, CU_EVENT_DEFAULT)) != CUDA_SUCCESS) break;
        if ((r = cuEventCreate(&e1, CU_EVENT_DEFAULT)) != CUDA_SUCCESS) break;
        RefGrid grid;
        grid.voxels = d_vox;
        std::memcpy(grid.origin, origin, sizeof(grid.origin));
        std::memcpy(grid.dims, dims, sizeof(grid.dims));
        std::memcpy(grid.world_to_index, world_to_index, sizeof(grid.world_to_index));
        std::memcpy(grid.clamp_min, clamp_min, sizeof(grid.clamp_min));
        std::memcpy(grid.clamp_max, clamp_max, sizeof(grid.clamp_max));
        grid.offset = offset;
        grid.scale = scale;
        RefParams prm;
        prm.length_scale = params_f[0];
        prm.amplitude = params_f[1];
        prm.kernel_radius = params_f[2];
        prm.impulse_density = params_f[3];
        prm.max_step_size = params_f[4];
        prm.min_steps = params_u[0];
        prm.max_steps = params_u[1];
        size_t count = (size_t)n;
        void *args[] = {&d_in, &d_out, &count, &grid, &prm};
        const unsigned int blocks = (unsigned int)((n - 1) / 128 + 1);
        // one host-to-host pass: copy in, trace, copy out
        if ((r = cuEventRecord(e0, nullptr)) != CUDA_SUCCESS) break;
        if ((r = cuMemcpyHtoDAsync(d_in, inputs, n * sizeof(RefInput), nullptr)) != CUDA_SUCCESS) break;
        if ((r = cuLaunchKernel(g_trace, blocks, 1, 1, 128, 1, 1, 0, nullptr, args, nullptr)) != CUDA_SUCCESS) break;
        if ((r = cuMemcpyDtoHAsync(outputs, d_out, n * sizeof(RefOutput), nullptr)) != CUDA_SUCCESS) break;
        if ((r = cuEventRecord(e1, nullptr)) != CUDA_SUCCESS) break;
        if ((r = cuEventSynchronize(e1)) != CUDA_SUCCESS) break;
        float ms = 0.0f;
        if ((r = cuEventElapsedTime(&ms, e0, e1)) != CUDA_SUCCESS) break;
        if (ms_e2e) *ms_e2e = ms;
        // device-resident launches
        double total = 0.0;
        for (int k = 0; k < reps; ++k) {
            if ((r = cuEventRecord(e0, nullptr)) != CUDA_SUCCESS) break;
            if ((r = cuLaunchKernel(g_trace, blocks, 1, 1, 128, 1, 1, 0, nullptr, args, nullptr)) != CUDA_SUCCESS) break;
            if ((r = cuEventRecord(e1, nullptr)) != CUDA_SUCCESS) break;
            if ((r = cuEventSynchronize(e1)) != CUDA_SUCCESS) break;
            if ((r = cuEventElapsedTime(&ms, e0, e1)) != CUDA_SUCCESS) break;
            total += ms;
        }
        if (r != CUDA_SUCCESS) break;
        if (ms_kernel) *ms_kernel = reps > 0 ? total / reps : 0.0;
    } while (false);
    if (r != CUDA_SUCCESS) rc = (int)r;
    if (e0) cuEventDestroy(e0);
    if (e1) cuEventDestroy(e1);
    if (d_vox) cuMemFree(d_vox);
    if (d_out) cuMemFree(d_out);
    if (d_in) cuMemFree(d_in);
    return rc;
}

}  // extern "C"
