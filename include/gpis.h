/*
 * gpis.h -- C ABI of the GB300 GPIS ray-flight library (libgpis_gb300.so).
 *
 * One "ray-flight" is one sparse-convolution-noise medium segment query:
 * Renewal / Renewal+ conditioning at the segment origin, the fixed-step march
 * for the first sign change of the field, the regula-falsi back-off
 * refinement, and the gradient sample at the end point.  It is the unit of
 * work behind SparseConvolutionNoiseMedium::intersectGP
 * (src/core/media/SparseConvolutionNoiseMedium.cpp:188-347) and the
 * GpRayBatchBackend request/reply pair
 * (src/core/media/GpRayBatchBackend.hpp:15-40).
 *
 * All signatures use plain pointers and sizes.  Device pointers are CUDA
 * device addresses; "host" entry points take ordinary (preferably pinned)
 * host arrays.  Every function returns an int status (GPIS_OK = 0, otherwise
 * a positive errno-style code) and gpis_last_error() describes the last
 * failure of the calling thread.
 *
 * Threading: a context is not thread-safe; use one context (or one stream)
 * per host thread.  Contexts own their device-side medium tables; callers
 * own every flight/result buffer.
 */
#ifndef GPIS_GB300_H_
#define GPIS_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GPIS_OK        0
#define GPIS_EIO       5    /* a CUDA runtime call failed                    */
#define GPIS_ENOMEM   12    /* device or host allocation failed             */
#define GPIS_ENODEV   19    /* no CUDA device                               */
#define GPIS_EINVAL   22    /* invalid argument or medium description       */
#define GPIS_ERANGE   34    /* a size exceeds a documented maximum          */
#define GPIS_ENOTSUP  95    /* medium feature not supported by this build   */

/* ---- per-flight status (RaySegmentStatus, src/gpu/cuda/RaySegmentBatch.hpp:55-59) */
#define GPIS_FLIGHT_OK             0u
#define GPIS_FLIGHT_INVALID_INPUT  1u
#define GPIS_FLIGHT_STEP_LIMIT     2u
#define GPIS_FLIGHT_PROPOSAL_MISS  3u  /* learned proposal rejected; plain march answered */

/* ---- enumerations (values equal the reference enums) ------------------- */
/* GPCorrelationContext, src/core/math/GaussianProcess.hpp:26-31 */
#define GPIS_CTX_GLOBAL        0u
#define GPIS_CTX_RENEWAL_PLUS  1u
#define GPIS_CTX_RENEWAL       2u
#define GPIS_CTX_NONE          3u
/* SparseConv1DSamplingScheme, src/core/media/Medium.hpp:42-46 */
#define GPIS_SCHEME_UNI        0u
#define GPIS_SCHEME_NEE        1u
#define GPIS_SCHEME_MIS        2u

/* Mean functions (src/core/math/GPFunctions.hpp:915-996, GPFunctions.cpp:165-299). */
#define GPIS_MEAN_SPHERE       0u  /* |p-c| - r            params: cx cy cz r            */
#define GPIS_MEAN_HOMOGENEOUS  1u  /* offset               params: offset                */
#define GPIS_MEAN_GRID         2u  /* dense trilinear grid (TabulatedMean baked to a grid) */
#define GPIS_MEAN_PLANE        3u  /* n.p - d              params: nx ny nz d            */
#define GPIS_MEAN_TORUS        4u  /* torus about y        params: cx cy cz R r          */
#define GPIS_MEAN_TORUS_PLANE  5u  /* min(torus, y - h)    params: cx cy cz R r h; GP id 0 torus, 1 plane */

/* Length-scale fields of a nonstationary SE covariance
 * (ProceduralNonstationaryCovariance, src/core/math/GPFunctions.cpp:1600-1758). */
#define GPIS_LS_CONSTANT       0u  /* ls(p) = 1                                       */
#define GPIS_LS_SINCOS         1u  /* ls(p) = a + b*sin(fx*x)*cos(fz*z); ls_max given  */

/* Flight flag bits (word 2 of the seed stream). */
#define GPIS_FLAG_FIRST_SCATTER  1u  /* no preceding GPIS event: no conditioning      */
#define GPIS_FLAG_SHADOW         2u  /* transmittance query: no gradient on a miss     */

/* ---- dense mean grid (HostMeanGrid, src/gpu/cuda/RaySegmentBatch.hpp:21-30) */
typedef struct gpis_mean_grid {
    const float *voxels;        /* host array, x fastest, then y, then z          */
    int32_t origin[3];
    int32_t dims[3];            /* each >= 2                                     */
    float world_to_index[12];   /* row-major 3x4 affine                          */
    float clamp_min[3];
    float clamp_max[3];
    float offset;               /* mean = (trilinear + offset) * scale            */
    float scale;
} gpis_mean_grid;

/* ---- medium description ------------------------------------------------
 * Field names follow the scene-JSON keys of the "sparse_conv_noise" medium
 * (SparseConvolutionNoiseMedium::fromJson, SparseConvolutionNoiseMedium.cpp:102-118;
 * GaussianProcessMedium::fromJson, GaussianProcessMedium.cpp:98-127) and of the
 * squared-exponential covariance (GPFunctions.cpp:657-685).
 * gpis_medium_desc_init() fills the reference defaults.                       */
typedef struct gpis_medium_desc {
    /* squared-exponential covariance */
    float sigma;                /* "sigma" (noise amplitude)                      */
    float length_scale;         /* "lengthScale"                                   */
    float aniso[3];             /* "aniso" (diagonal anisotropy)                  */
    float kernel_scale;         /* "localScale": truncation radius in conv units  */
    /* nonstationary length scale (1.0 everywhere for GPIS_LS_CONSTANT) */
    uint32_t ls_kind;
    float ls_params[4];         /* a, b, fx, fz                                   */
    float ls_max;               /* supremum of ls(p); cell size follows it        */
    uint32_t multires;          /* 2-level multi-resolution blend (base 2.5)      */
    /* octaves: f = mean + sum_k octave_sigma[k] * noise_k; n_octaves = 1 means the
       single reference realization with amplitude "sigma" */
    uint32_t n_octaves;         /* 1..4                                           */
    float octave_sigma[4];
    float octave_scale[4];      /* length-scale multiplier of octave k            */
    uint32_t octave_seed[4];    /* seed offset of octave k                        */
    /* mean */
    uint32_t mean_kind;
    float mean_params[8];
    const gpis_mean_grid *grid; /* GPIS_MEAN_GRID only (host memory)             */
    /* sparse_conv_noise keys */
    float step_size;            /* "step_size"                                     */
    uint32_t min_step;          /* "min_step"                                      */
    uint32_t seed;              /* "seed" (global seed)                            */
    float impulse_density;      /* "impulse_density" (truncated to an integer)    */
    uint32_t single_realization;    /* "single_realization"                       */
    uint32_t isotropic_3d_sampling; /* "isotropic_3D_sampling"                    */
    uint32_t one_d_sampling;        /* "1D_sampling"                              */
    uint32_t sampling_scheme;       /* "1D_sampling_scheme"                       */
    uint32_t correlation_xy;        /* "1D_gradient_correlationXY"                */
    /* gaussian process medium keys */
    uint32_t correlation_context;   /* "correlation_context"                      */
    float sigma_a, sigma_s, density;
    /* device-side limits */
    uint32_t max_steps;         /* march give-up bound (StepLimit); 0 = 16384     */
    uint32_t impulse_xyz_order; /* 0: z drawn first (right-to-left argument
                                   evaluation of next3D, GCC/MSVC x86-64);
                                   1: x drawn first                               */
    int32_t max_bounces;        /* "max_bounces" (Medium::fromJson, Medium.cpp:37) */
    uint32_t reserved_;
} gpis_medium_desc;

/* ---- flight streams (structure of arrays, 16-byte records) ---------------
 * Record i of each stream belongs to flight i.  Requests follow
 * GpRaySegmentRequest (GpRayBatchBackend.hpp:15-29).                         */
typedef struct gpis_flight_soa {
    const float *origin_near;   /* n x {ox, oy, oz, nearT}                         */
    const float *dir_far;       /* n x {dx, dy, dz, farT}  (unit direction)         */
    const uint32_t *seeds;      /* n x {noiseSeed, normalSeed, flags, jitter bits}  */
    const float *prev;          /* n x {previousValue, gx, gy, gz} (world gradient) */
    const uint32_t *medium;     /* n medium indices, or NULL for medium 0           */
} gpis_flight_soa;

/* Results: two 16-byte records per flight.
 *   rec0 = {t, value, gx, gy}, rec1 = {gz, transmittance, steps(u32), status(u32)}
 * value is 0 at a hit and the field value at farT on a miss (lastVal);
 * (gx,gy,gz) is the sampled world gradient at the end point (at a hit, and at
 * farT for a distance miss; previous gradient for a shadow miss).
 * status = GPIS_FLIGHT_* | (gp_id << 8).                                     */
typedef struct gpis_result_soa {
    float *rec;                 /* n x 8 words                                      */
} gpis_result_soa;

/* Device counter block, summed over all flights since the last reset. */
typedef struct gpis_counters {
    uint64_t flights;
    uint64_t steps;             /* march steps (field evaluations in the march)    */
    uint64_t refine_evals;      /* field evaluations in the refinement             */
    uint64_t hits;
    uint64_t step_limit;
    uint64_t invalid;
    uint64_t cell_refills;      /* impulse-cache cell regenerations                */
    uint64_t skipped_steps;     /* march steps decided by the field bound, unevaluated */
} gpis_counters;

typedef struct gpis_ctx gpis_ctx;

/* ---- medium queries (GaussianProcessMedium state machines) -------------------
 * A ray (Ray: pos, dir, nearT, farT; farT may be +inf).                       */
typedef struct gpis_ray {
    float pos[3];
    float dir[3];
    float near_t;
    float far_t;
} gpis_ray;

/* The MediumState fields the GPIS medium reads and writes (Medium.hpp:70-108,
 * RayInfo): path coordinates and scene seed, firstScatter, bounce, lastGPId,
 * lastVal, lastAniso, info.t and the 1D sampling scheme of the last event.    */
typedef struct gpis_medium_state {
    uint32_t pixel_sample_segment[4];
    uint32_t scene_seed;
    uint32_t first_scatter;
    int32_t bounce;
    int32_t last_gp_id;
    float last_val;
    float last_aniso[3];
    double info_t;
    uint32_t sampling_scheme;
    uint32_t reserved_;
} gpis_medium_state;

/* MediumSample fields set by sampleDistance (MediumSample.hpp; resumeDistance,
 * GaussianProcessMedium.cpp:289-381).  status: 1 Finished, 0 Failed.       */
typedef struct gpis_medium_sample {
    float t;
    float p[3];
    float weight[3];
    float pdf;
    float aniso[3];
    float continued_t;
    float continued_weight[3];
    int32_t exited;
    int32_t gp_id;
    int32_t status;
    uint32_t sampling_scheme;
    uint32_t reserved_;
} gpis_medium_sample;

/* Reference defaults: SparseConvolutionNoiseMedium() (SparseConvolutionNoiseMedium.cpp:62-79),
 * GaussianProcessMedium() (GaussianProcessMedium.cpp:87-96), SE covariance with
 * localScale 3 (GPFunctions.hpp:1816) and a unit sphere mean.                 */
void gpis_medium_desc_init(gpis_medium_desc *desc);

/* Parse a Tungsten "sparse_conv_noise" medium JSON object (with an inline
 * "gaussian_process" {"mean", "covariance"}) into desc.  Replaces
 * SparseConvolutionNoiseMedium::fromJson for the supported subset.           */
int gpis_medium_desc_from_json(const char *json, gpis_medium_desc *desc);

/* Create a context on the current CUDA device with n_media medium tables
 * (replaces Se1DRayBatcher::setMeanGrid + SeBatchBackend set-up,
 * src/gpu/cuda/RaySegmentBatch.cpp:16-62, PathTracerSeBatchBackend.cpp:402-416). */
int gpis_ctx_create(const gpis_medium_desc *media, int n_media, gpis_ctx **out);
void gpis_ctx_destroy(gpis_ctx *ctx);

/* Asynchronous flight batch on a CUDA stream; all stream pointers are device
 * pointers (replaces launchSe1DRaySegments, RaySegmentBatch.cu:305-331).
 * Returns after enqueueing.  n == 0 is a successful no-op.                   */
int gpis_flights_submit(gpis_ctx *ctx, const gpis_flight_soa *in,
                        const gpis_result_soa *out, uint32_t n, void *cuda_stream);

/* Blocking flight batch on host arrays: copies in, traces, copies out and
 * synchronizes once (replaces Se1DRayBatcher::trace, RaySegmentBatch.hpp:124-126
 * and GpRayBatchBackend::trace, GpRayBatchBackend.hpp:43-47).                */
int gpis_flights_trace_host(gpis_ctx *ctx, const gpis_flight_soa *in,
                            const gpis_result_soa *out, uint32_t n);

/* Batched Medium::sampleDistance for n rays of one medium of the context
 * (GaussianProcessMedium::sampleDistance / beginDistance / resumeDistance /
 * finishDistance, GaussianProcessMedium.cpp:222-381).  jitter[i] is the one
 * PathSampleGenerator draw of ray i's segment (SparseConvolutionNoiseMedium.cpp:234).
 * Host arrays; states are updated in place; blocking.                         */
int gpis_medium_sample_distance(gpis_ctx *ctx, uint32_t medium, const gpis_ray *rays,
                                gpis_medium_state *states, const float *jitter,
                                gpis_medium_sample *samples, uint32_t n);

/* Batched Medium::transmittance (GaussianProcessMedium.cpp:383-440): writes 0 or 1
 * per ray and updates the states (lastAniso and firstScatter at a hit).      */
int gpis_medium_transmittance(gpis_ctx *ctx, uint32_t medium, const gpis_ray *rays,
                              gpis_medium_state *states, const float *jitter,
                              float *transmittance, uint32_t n);

/* ---- 1D specular next-event estimation ----------------------------------
 * neeGrad / neePDF on the realization of a hit (SparseConvolutionNoiseRealization::
 * neeShared / neeGrad / neePDF, SparseConvolutionNoise.cpp:662-821), as MirrorBsdf
 * (MirrorBsdf.cpp:45, 69, 79, 109) and ConductorBsdf (ConductorBsdf.cpp:73, 97,
 * 107, 137) call them.  Query i uses the realization of flight i of `flight`
 * (origin, direction = the ray direction info->w, seeds, prev, medium; near,
 * far and jitter are not read), the point and segment parameter
 * point_t[i] = {p, info->t} and the world normal normal[i] = {n, unused}.
 * out[i] = {pdf (neePDF), gradient (neeGrad, 3 floats)}.  Media must use 1D
 * sampling; with several octaves the law is the octave sum's (the transverse
 * gradient is the sum of the octaves' independent Gaussian draws, weighted by
 * amplitude / length multiplier).  A query on a 3D medium or with non-finite
 * inputs gets a NaN pdf.  All streams 16-byte aligned.                      */
typedef struct {
    gpis_flight_soa flight;
    const float *point_t;       /* float4 per query                           */
    const float *normal;        /* float4 per query                           */
} gpis_nee_soa;

/* Asynchronous, device pointers, n == 0 is a no-op. */
int gpis_nee_submit(gpis_ctx *ctx, const gpis_nee_soa *in, float *out, uint32_t n, void *cuda_stream);
/* Blocking, host pointers. */
int gpis_nee_host(gpis_ctx *ctx, const gpis_nee_soa *in, float *out, uint32_t n);

/* ---- schedule knobs (the autotuner's outputs) ------------------------------
 * 0 restores a knob's default.                                               */
#define GPIS_TUNE_MARCH_CTAS_PER_SM 0u   /* fast-pass persistent grid: CTAs per SM
                                            (default: every CTA that is resident)   */
#define GPIS_TUNE_RENDER_PASS_PATHS 1u   /* paths per render pass (default 2^22)     */
#define GPIS_TUNE_HOST_CHUNK        2u   /* flights per chunk of the host pipeline
                                            (default 2^20)                          */
#define GPIS_TUNE_HOST_DIRECT       3u   /* 1: gpis_flights_trace_host runs the kernels on
                                            page-locked host streams in place (the GPU
                                            reads and writes them over the host link, no
                                            staging copies) when every stream is
                                            page-locked and mapped; 0 (default): staged,
                                            chunked copies                             */
#define GPIS_TUNE_PROPOSED_SKIP_CAP 4u   /* gpis_flights_submit_proposed: the most steps
                                            one evaluation may skip before a flight's
                                            proposed interval, 8..256 (default 32; every
                                            skipped step is still certified)            */
#define GPIS_TUNE_FAST_WINDOW       5u   /* stationary 1D fast pass: 0 (default) keeps
                                            each lane's three-cell impulse window in
                                            shared memory, 1 in registers              */
#define GPIS_TUNE_PRECISE_DECISIONS 6u   /* 1: every crossing of a stationary 1D single-
                                            octave medium is decided on the precise
                                            evaluator; 0 (default): on fast values where
                                            error bounds make the decision certain (the
                                            refinement point may then differ from the
                                            reference's by that bound, far below the
                                            march's tolerance), the precise evaluator
                                            for the rest                                */
int gpis_tune_set(gpis_ctx *ctx, uint32_t key, uint64_t value);
int gpis_tune_get(gpis_ctx *ctx, uint32_t key, uint64_t *value);

/* Read (and optionally reset) the device counter block. */
int gpis_status(gpis_ctx *ctx, gpis_counters *out, int reset);

/* Per-kernel timing with CUDA events recorded on the launch stream of every
 * gpis_flights_submit while enabled.  gpis_profile_read synchronizes on the
 * recorded events and returns the accumulated milliseconds and launch counts
 * of the prepare (0), march (1) and finish (2) kernels.  Replaces the
 * TUNGSTEN_GPIS_PROFILE counters (SparseConvolutionNoiseMedium.cpp:23-60). */
int gpis_profile_enable(gpis_ctx *ctx, int on);
int gpis_profile_read(gpis_ctx *ctx, double ms[3], uint64_t launches[3], int reset);

/* Seeds of a flight from its path coordinates (computeSeed,
 * SparseConvolutionNoise.cpp:57-66, and the request seeds of
 * prepareGpisSegment, SparseConvolutionNoiseMedium.cpp:235-238).             */
void gpis_flight_seeds(const gpis_medium_desc *desc, const uint32_t pixel_sample_segment[4],
                       uint32_t scene_seed, uint32_t *noise_seed, uint32_t *normal_seed);

/* ---- unit-level device entry points (used by the parity tests) ---------- */
/* Impulses of n 1D cells (cell index, seed) on the device: pos[n*k], weight[n*k],
 * k = impulses per cell (cell1D, SparseConvolutionNoise.cpp:465-485).
 * All pointers are device pointers; synchronous.                             */
int gpis_debug_cells_1d(const uint32_t *cells, const uint32_t *seeds, uint32_t n,
                        uint32_t impulses, float *pos, float *weight);
/* Impulses of n 3D cells: cells = n x {i, j, k}; pos = n*k x {x,y,z}.        */
int gpis_debug_cells_3d(const int32_t *cells, const uint32_t *seeds, uint32_t n,
                        uint32_t impulses, uint32_t xyz_order, float *pos, float *weight);

/* The precise evaluator's exponential at n arguments (device pointers,
 * blocking): e^x rounded to the nearest float (the oracle's definition of the
 * reference's float exp).  Unit-level check; no counterpart in the reference. */
int gpis_debug_exp(const float *x, float *y, uint32_t n);

/* Field evaluation at n points (device pointers): points/dirs n x 4 floats,
 * seeds n x 4 words as in the flight seed stream, prev n x 4 floats.  The
 * conditioning of each point's flight is built from (origin = points of the
 * "origins" stream) exactly as a flight would.  out = n x 8 floats:
 * {noise value (normalized), n1, n2, n3, field value, mean, precise field
 * value, GP id (int bits)} where (n1, n2, n3) is, for 1D noise, (conditioning
 * x splat, conditioning y splat, dnoise/dz) and, for 3D noise, the world
 * gradient of the normalized noise; with several octaves the noise entries are
 * amplitude-weighted sums.  The precise value is the one the march decides
 * crossings with (the reference's float formulation operation for operation). */
int gpis_debug_field(gpis_ctx *ctx, const float *origins, const float *points,
                     const float *dirs, const uint32_t *seeds, const float *prev,
                     uint32_t n, float *out);

/* Elementwise squared-exponential splat (launchKernel1D / seSplat1D,
 * src/gpu/cuda/Kernel1D.hpp:26-29, SeSplat1D.cu:12-44): device pointers,
 * asynchronous on the stream; local_scale must be finite and > 0.            */
int gpis_se_splat_1d(const float *queries, const float *centers, float *values,
                     float *derivatives, size_t count, float local_scale, void *cuda_stream);

/* ---- allocation-free flight batch ------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc: a
 * renderer thread that must never make the device synchronize (cudaMalloc and
 * cudaFree can), or a plugin host that owns all device memory and forbids
 * plugins to allocate.  The same flight kernels as gpis_flights_submit run on
 * one medium description (no grid mean), with all working memory in a fixed
 * array of this library (about 12 MB for GPIS_STATIC_MAX_FLIGHTS flights)
 * that every GPU which loads the library keeps until the process exits.  The
 * caller provides device flight and result streams as for gpis_flights_submit.
 * Larger batches fail with GPIS_ERANGE.  The first call on a device, with that
 * device current, looks up the array's device address and uploads a constant
 * table; make that first call before any stream capture.  That set-up is kept
 * for the life of the process: after cudaDeviceReset (or anything else that
 * destroys the device's primary context) this entry point must not be called
 * again on that device.  All calls share the array, so calls that overlap on
 * the GPU (other streams, other host threads) race: serialize them.  Streams
 * must be 16-byte aligned (GPIS_EINVAL otherwise, before any launch).  The
 * march grid is the occupancy maximum, not a context's autotuned value.     */
#define GPIS_STATIC_MAX_FLIGHTS 65536u
int gpis_flights_submit_static(const gpis_medium_desc *medium, const gpis_flight_soa *in,
                               const gpis_result_soa *out, uint32_t n, void *cuda_stream);

/* ---- asynchronous batch backend -------------------------------------------
 * The GpRayBatchBackend contract (GpRayBatchBackend.hpp:43-55,
 * PathTracerSeBatchBackend.cpp:358-397) over flights: gpis_backend_submit
 * copies the n requests (host streams as gpis_flight_soa) before it returns,
 * traces them on the backend's own stream and, when the n result records are
 * in out_rec (host memory the caller keeps until then), calls done(user,
 * status) once: status GPIS_OK, or an error code with out_rec untouched (the
 * caller may then trace the requests on the CPU).  done runs on a CUDA
 * callback thread or the backend's dispatcher thread and must not call CUDA.
 * Batches complete in submission order.  One dispatcher thread per backend;
 * submit is thread-safe.  gpis_backend_destroy waits for every batch.      */
typedef struct gpis_backend gpis_backend;
typedef void (*gpis_batch_done_fn)(void *user, int status);
int gpis_backend_create(const gpis_medium_desc *media, int n_media, gpis_backend **out);
void gpis_backend_destroy(gpis_backend *backend);
int gpis_backend_submit(gpis_backend *backend, const gpis_flight_soa *in, float *out_rec, uint32_t n,
                        gpis_batch_done_fn done, void *user);

/* ---- wavefront path tracer around the medium (images) -------------------
 * The subset of PathTracer::traceSample (PathTracer.cpp:49-292) that the image
 * workloads use: a pinhole camera, the medium inside the cube [-h, h]^3 (a
 * forward-scattering boundary: entering and leaving count no bounce), one
 * one-sided quad light outside the cube, and the GP surface events of
 * GaussianProcessMedium::sampleDistance shaded by BRDFPhaseFunction over a
 * Lambert, mirror or conductor BSDF (BRDFPhaseFunction.cpp:29-119,
 * LambertBsdf, MirrorBsdf.cpp:31-109, ConductorBsdf.cpp:58-137).  Medium events
 * take volume direct lighting as TraceBase::handleVolume does
 * (TraceBase.cpp:993-1014, 798-874): one light sample and one phase sample,
 * each with a transmittance query through the medium, with the medium state of
 * the next bounce.  Lambert: both, power heuristic.  Mirror and conductor
 * follow the event's 1D sampling scheme (the medium's sampling_scheme through
 * samplingScheme): UNI takes the phase sample only, at MIS weight 1; NEE takes
 * the light sample only, its BSDF value albedo * F * neePDF at the half-vector
 * normal and its transmittance flight conditioned on neeGrad; MIS takes both
 * under the power heuristic with neePDF as the phase density (1D media).  No
 * Russian roulette; no environment light.
 *
 * Path decisions draw from a counter RNG keyed (sampler_seed, path, bounce,
 * dimension) with path = (y * width + x) * spp + sample; directions are sampled
 * without trigonometry (rejection in the unit disk), so the CUDA path and the
 * CPU restatement make the same decisions.  GP seeds follow the reference:
 * pixelSampleSegment = (x, y, sample, bounce), sceneSeed = scene_seed.       */
#define GPIS_PHASE_LAMBERT   0u
#define GPIS_PHASE_MIRROR    1u
#define GPIS_PHASE_CONDUCTOR 2u

typedef struct {
    uint32_t width, height, spp, max_bounces;
    float cam_pos[3];
    float cam_target[3];
    float cam_up[3];
    float tan_half_fov;         /* tangent of half the vertical field of view    */
    float box_half;             /* the medium fills the cube [-h, h]^3            */
    float light_center[3];
    float light_u[3];           /* the quad is center + s*u + t*v, |s|,|t| <= 1/2 */
    float light_v[3];
    float light_emission[3];    /* radiance emitted toward u x v                  */
    uint32_t phase;             /* GPIS_PHASE_*                                   */
    float albedo[3];
    uint32_t scene_seed;
    uint32_t sampler_seed;
    uint32_t medium;            /* medium index in the context                    */
    float eta[3];               /* conductor: complex index of refraction eta + ik; */
    float k[3];                 /* eta = k = 0 reflects everything (Fresnel.hpp:102-123) */
    uint32_t reserved_;
} gpis_scene_desc;

typedef struct {
    uint64_t paths;
    uint64_t distance_flights;  /* sampleDistance flights                         */
    uint64_t shadow_flights;    /* transmittance flights of direct lighting       */
    uint64_t medium_events;
    uint64_t failed;            /* paths ended by a failed medium or phase sample */
    double ms;                  /* device time of the render (CUDA events)        */
    uint64_t launches;          /* kernels launched by the render                 */
    uint64_t nee_queries;       /* neePDF / neeGrad queries of specular events    */
    uint32_t graphed;           /* 1: the bounce loop ran as a captured CUDA graph */
    uint32_t passes;            /* passes of up to 2^22 paths                     */
} gpis_render_stats;

/* Render into image_rgb (host, height x width x 3 floats, row 0 at the top):
 * the mean radiance of spp paths per pixel.  Blocking.                       */
int gpis_render(gpis_ctx *ctx, const gpis_scene_desc *scene, float *image_rgb, gpis_render_stats *stats);
/* Render n_scenes scenes (each with its own medium of the context, image size,
 * spp and bounces) in one wavefront: their paths share every flight batch.
 * images[k] as image_rgb of scene k; each image equals its own gpis_render.
 * The bounce loop keeps its queue lengths on the device and runs as one
 * captured CUDA graph per round (direct launches while the context profiles). */
int gpis_render_batch(gpis_ctx *ctx, const gpis_scene_desc *scenes, uint32_t n_scenes, float *const *images,
                      gpis_render_stats *stats);

/* ---- learned crossing proposal -------------------------------------------
 * A GRU (hidden 32) over eight samples of the mean SDF and its slope along the
 * flight, then a 3 x 64 GELU MLP over its state and eight per-flight features,
 * emitting an 8-component logistic mixture over u = (t - near) / (far - near)
 * of the first downcrossing and a miss logit.  BF16 tensor-core contractions,
 * FP32 accumulation, elementwise parts, loss and Adam.  The parameters are one
 * float vector of gpis_proposal_n_params() values: w_ih (96 x 16), b_ih (96),
 * w_hh (96 x 32), b_hh (96), w1 (64 x 48), b1, w2 (64 x 64), b2, w3 (64 x 64),
 * b3, w4 (32 x 64), b4 (32), weights row-major [out][in]; the padded input
 * columns (w_ih 2..15, w1 40..47) and output rows (w4, b4 25..31) are unused.
 * Outputs: 0..7 mixture logits, 8..15 locations (through a sigmoid), 16..23
 * scales (softplus + 1e-3), 24 the miss logit.
 * The proposal never changes a flight's result: gpis_flights_submit_proposed
 * lets the march take longer certified skips before the proposed interval.   */
typedef struct gpis_proposal gpis_proposal;
uint32_t gpis_proposal_n_params(void);
/* params: host vector, NULL for zeros.  One CUDA stream per proposal. */
int gpis_proposal_create(const float *params, gpis_proposal **out);
void gpis_proposal_destroy(gpis_proposal *prop);
int gpis_proposal_set_params(gpis_proposal *prop, const float *params);    /* resets Adam */
int gpis_proposal_get_params(gpis_proposal *prop, float *params);
/* 24 features per flight (device pointers, asynchronous): the mean SDF and its
 * slope along the ray at the centres of eight equal parts of [near, far], then
 * t_max / 4, 10 x the local length scale, the conditioned value and derivative,
 * the first-scatter flag, 10 x the amplitude, step / t_max, the mean at near. */
int gpis_proposal_features(gpis_ctx *ctx, const gpis_flight_soa *in, float *features, uint32_t n,
                           void *cuda_stream);
/* Training on device batches: features (24 per flight), targets (u*, hit) per
 * flight; n a positive multiple of 16.  train_step: one Adam step (lr), loss =
 * mean negative log-likelihood before the step (NULL: no synchronization: the
 * step runs on the proposal's own blocking stream, ordered with the legacy
 * default stream; a caller that fills or reuses the batch on another stream
 * synchronizes first).
 * gradient: the gradient of the mean loss (host vector) without a step.
 * forward: the 32 raw outputs per flight (device).  Blocking.               */
int gpis_proposal_train_step(gpis_proposal *prop, const float *features, const float *targets, uint32_t n,
                             float lr, float *loss);
int gpis_proposal_gradient(gpis_proposal *prop, const float *features, const float *targets, uint32_t n,
                           float *grad, float *loss);
int gpis_proposal_forward(gpis_proposal *prop, const float *features, uint32_t n, float *outputs);
/* Fused inference (asynchronous, device pointers): per flight the dominant
 * component's interval [m - 3s, m + 3s] in t, the miss probability and m:
 * intervals[4 i .. 4 i + 3] = (t_a, t_b, q, m).  A time-out of the tensor
 * cores' completion wait in an earlier call is returned as GPIS_EIO.        */
int gpis_proposal_infer(gpis_proposal *prop, const gpis_flight_soa *in, const float *features, float *intervals,
                        uint32_t n, void *cuda_stream);
/* The fused inference kernel: tcgen05 MMAs with tensor-memory accumulators, two
 * 128-flight tiles per block (default) or one, or warp-level mma.sync (also
 * taken when features is not 16-byte aligned).  The training GEMMs (forward,
 * gradient, train_step) run on tcgen05 too, unless GPIS_PROPOSAL_KERNEL_MMA
 * selects the warp-level mma.sync kernels for them as well.                  */
#define GPIS_PROPOSAL_KERNEL_TC2 0
#define GPIS_PROPOSAL_KERNEL_TC1 1
#define GPIS_PROPOSAL_KERNEL_MMA 2
int gpis_proposal_set_kernel(gpis_proposal *prop, int kernel);
/* Polls of the tensor-memory kernels' bounded completion wait per
 * MMA round (default GPIS_PROPOSAL_WAIT_DEFAULT; each poll is one
 * mbarrier.try_wait).  When a round's wait runs out, the kernel's threads stop
 * together, wait for the MMAs already committed with the default bound, free
 * their tensor memory and set a flag; the next gpis_proposal_infer returns
 * GPIS_EIO and clears it.  0 makes every wait run out at once: the way to
 * exercise that path.  No counterpart in the reference.                      */
#define GPIS_PROPOSAL_WAIT_DEFAULT (1u << 22)
int gpis_proposal_set_wait_limit(gpis_proposal *prop, uint32_t polls);
/* Resident blocks per SM of a fused inference kernel (its persistent grid is
 * SMs x this); negative on error.                                           */
int gpis_proposal_occupancy(const gpis_proposal *prop, int kernel);
/* gpis_flights_submit with proposals: identical results; intervals from
 * gpis_proposal_infer (16-byte aligned).                                    */
int gpis_flights_submit_proposed(gpis_ctx *ctx, const gpis_flight_soa *in, const float *intervals,
                                 const gpis_result_soa *out, uint32_t n, void *cuda_stream);
/* gpis_render_batch with the learned arm: every distance-flight batch takes
 * features, inference and the proposed march (identical images).            */
int gpis_render_batch_proposed(gpis_ctx *ctx, gpis_proposal *prop, const gpis_scene_desc *scenes,
                               uint32_t n_scenes, float *const *images, gpis_render_stats *stats);

/* Tensor-core self-check: d[128 x n] = a[128 x k] * b[n x k]^T with BF16 inputs
 * (row-major bit patterns) through the tcgen05 / tensor-memory path the proposal
 * kernels use.  n a multiple of 32 up to 128, k of 16 up to 128.  Blocking.   */
int gpis_debug_tc_gemm(const uint16_t *a_bf16, const uint16_t *b_bf16, uint32_t n, uint32_t k, float *d);

/* Last error message of the calling thread ("" when none). */
const char *gpis_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* GPIS_GB300_H_ */
