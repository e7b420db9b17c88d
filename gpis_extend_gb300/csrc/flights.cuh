// flights.cuh -- launch interface between the C ABI (gpis_abi.cu) and the
// flight kernels (flights.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gpis.h"
#include "device_common.cuh"

namespace gpis {

// Per-flight conditioning coefficients (SparseConvConditioningCoefficients1D/3D,
// SparseConvolutionNoise.hpp:7-24), written by the prepare kernel.
// One realization's coefficients; several octaves each have their own.
struct CondOct {
    float vs;               // value_scale
    float gs[3];            // gradient_scale (iso-ray space for 1D, world for 3D)
};

struct CondRec {
    CondOct oct[4];
    float tgn[3];           // target_gradient_noise (1D transverse law)
    uint32_t has_obs;       // has_gradient_observation
};
static_assert(sizeof(CondRec) == 80 && offsetof(CondRec, tgn) == 64, "conditioning record layout (k_prepare "
                                                                      "writes 1D single-octave records by float4)");

// counters per FlightArgs::work block
constexpr int kWorkCounters = 8;

struct FlightArgs {
    const float4 *origin_near;
    const float4 *dir_far;
    const uint4 *seeds;
    const float4 *prev;
    const uint32_t *medium;     // may be null
    float4 *out;                // 2 float4 per flight
    const DevMedium *media;
    int n_media;
    uint32_t n;
    CondRec *cond;              // scratch, n records
    double *t_end;              // scratch, n values (double march parameter at the end point)
    uint32_t *work;             // scratch, kWorkCounters counters zeroed before the march: the
                                // passes' work counters and the hand-off queues' lengths
    uint4 *resume;              // scratch, n saved march states
    uint32_t *queue;            // scratch, 2 n flight indices (may be null: the resume passes then
                                // scan every flight): the flights the fast pass hands on, then
                                // those the certified resume pass hands on
    int queue_in;               // set by launch_flights for each resume pass
    float4 *setup;              // scratch, 4 per flight: the fast pass's per-flight set-up, written by
                                // k_prepare when the stationary cooperative evaluator runs (else unused)
    unsigned long long *counters;  // gpis_counters block (8 x u64)
    int any_cond;               // some medium conditions (run the prepare kernel)
    int one_d;                  // all media use 1D noise
    int three_d;                // all media use 3D noise
    uint32_t max_imp;           // max impulses per cell over the media
    uint32_t max_oct;           // max octaves over the media
    int all_grid;               // all media have a grid mean
    int any_ns;                 // some medium has a nonstationary length scale
    int any_mr;                 // some medium blends multi-resolution levels
    int any_gen3d;              // some 3D medium is isotropic, nonstationary or multi-resolution
                                // (the general 3D evaluator, no 3D step skipping)
    uint32_t ctas_per_sm;       // fast-pass persistent grid: CTAs per SM (0: every resident CTA)
    uint32_t prop_cap;          // most steps one evaluation skips before a proposed interval (0: 32)
    uint32_t fast_window;       // stationary 1D fast pass: 0 impulse window in shared memory, 1 in registers
    uint32_t precise_only;      // 1: no certified resume pass (every crossing on the precise evaluator)
    const uint32_t *n_dev;      // may be null: the live flight count in device memory (<= n,
                                // which is then the capacity the grids are sized for)
    const float4 *proposal;     // may be null: per flight the proposed crossing interval
                                // (t_a, t_b, miss probability, -); the fast pass may skip
                                // further than its usual cap before t_a
};

// Per-flight features of the learned proposal (proposal.cu).
cudaError_t launch_features(const DevMedium *media, int n_media, const gpis_flight_soa &in, uint32_t n, float *feat,
                            cudaStream_t s, const uint32_t *n_dev = nullptr);

// Upload the jump-ahead PCG table to the current device (once per device).
cudaError_t upload_pcg_table();

// Enqueue the flight kernels on the stream.  ev, when not null, holds start/stop
// events for the prepare, march (march + resume) and finish kernels (ev[2k], ev[2k+1]).
cudaError_t launch_flights(const FlightArgs &a, int num_sms, cudaStream_t stream, cudaEvent_t *ev = nullptr);
// Fill the corner table of a grid mean (m holds the device voxel pointer and cell_lo/cell_n)
cudaError_t launch_pack_grid(const DevMedium &m, float4 *cells, size_t n, cudaStream_t stream);
// 1D specular NEE queries on the realizations of the flights in a (one thread each)
cudaError_t launch_nee(const FlightArgs &a, const float4 *point_t, const float4 *normal, float4 *out,
                       cudaStream_t stream);

// Unit-level kernels (synchronous wrappers live in gpis_abi.cu).
cudaError_t launch_debug_exp(const float *x, float *y, uint32_t n, cudaStream_t s);
cudaError_t launch_debug_cells_1d(const uint32_t *cells, const uint32_t *seeds, uint32_t n,
                                  uint32_t impulses, float *pos, float *weight, cudaStream_t s);
cudaError_t launch_debug_cells_3d(const int32_t *cells, const uint32_t *seeds, uint32_t n,
                                  uint32_t impulses, uint32_t order, float *pos, float *weight,
                                  cudaStream_t s);
cudaError_t launch_debug_field(const DevMedium *m, const float4 *origins, const float4 *points,
                               const float4 *dirs, const uint4 *seeds, const float4 *prev,
                               uint32_t n, float4 *out, cudaStream_t s);
cudaError_t launch_se_splat_1d(const float *q, const float *c, float *v, float *d, size_t n,
                               float scale, cudaStream_t s);

}  // namespace gpis
