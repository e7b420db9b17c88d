/*
 * gpis_oracle.h -- CPU restatement of the reference sparse-convolution-noise
 * GPIS ray-flight path.  TEST INFRASTRUCTURE ONLY: the parity tests, the
 * smoke check and the CPU baseline of the benchmark call it as the checker;
 * the product library never links it.
 *
 * Every function follows the reference file:line cited beside it and keeps
 * the reference's float/double precision choices ("float mode").  The
 * "double mode" noise entry points evaluate the same impulse sums in FP64 on
 * the same cell decomposition; they are the FP64 anchor of the noise-value
 * parity bar.
 */
#ifndef GPIS_ORACLE_H_
#define GPIS_ORACLE_H_

#include <stdint.h>
#include "../include/gpis.h"

#ifdef __cplusplus
extern "C" {
#endif

/* MathUtil::xxhash32 (src/core/math/MathUtil.hpp:179-224) */
uint32_t gor_xxhash32_1(uint32_t p);
uint32_t gor_xxhash32_2(uint32_t x, uint32_t y);
uint32_t gor_xxhash32_4(uint32_t x, uint32_t y, uint32_t z, uint32_t w);

/* UniformSampler PCG32 stream after set_state(state) (UniformSampler.hpp:41-75):
 * writes n next1D() floats and their raw 32-bit outputs. */
void gor_pcg_stream(uint64_t state, uint32_t n, float *out_float, uint32_t *out_raw);

/* Box-Muller pair from a sampler set to state (Gaussian.cpp:23-35). */
void gor_normal_pair(uint64_t state, uint32_t pairs, double *out);

/* Impulses of one 1D cell (cell1D, SparseConvolutionNoise.cpp:465-485). */
void gor_cell_1d(uint32_t cell, uint32_t seed, uint32_t impulses, float *pos, float *weight);
/* Impulses of one 3D cell (cell3D, SparseConvolutionNoise.cpp:432-452);
 * pos gets x,y,z per impulse in the pinned next3D order. */
void gor_cell_3d(int32_t i, int32_t j, int32_t k, uint32_t seed, uint32_t impulses,
                 uint32_t xyz_order, float *pos, float *weight);

/* Noise evaluation at one point of a flight.
 *   origin/dir: the flight's ray; p: query point; seeds: {noiseSeed, normalSeed,
 *   flags, jitter bits}; prev: {value, gx, gy, gz}.
 *   out[0] = normalized noise (conditioned as the flight would be),
 *   out[1..3] = 1D: {cond. x splat, cond. y splat, dnoise/dz}; 3D: world gradient,
 *   out[4] = field value, out[5] = mean.
 * double_mode != 0 evaluates every impulse and splat sum in FP64 on the same
 * float cell decomposition (the FP64 anchor). */
int gor_field(const gpis_medium_desc *desc, const float origin[3], const float dir[3],
              const float p[3], const uint32_t seeds[4], const float prev[4],
              int double_mode, double out[6]);

/* World gradient sample at a point (evaluateGradient, SparseConvolutionNoise.cpp:133-140)
 * with t_segment the segment parameter of the point. */
int gor_gradient(const gpis_medium_desc *desc, const float origin[3], const float dir[3],
                 const float p[3], float t_segment, const uint32_t seeds[4],
                 const float prev[4], float out[3]);

/* Flights in float mode (prepareGpisSegment + finishGpisSegment + the gradient
 * sample of resumeDistance/resumeTransmittance).  Streams as in gpis.h; host
 * memory.  n_threads <= 0 uses all online cores. */
int gor_trace_flights(const gpis_medium_desc *media, int n_media, const gpis_flight_soa *in,
                      const gpis_result_soa *out, uint32_t n, int n_threads);

/* Seeds as gpis_flight_seeds (computeSeed, SparseConvolutionNoise.cpp:57-66). */
void gor_flight_seeds(const gpis_medium_desc *desc, const uint32_t pss[4], uint32_t scene_seed,
                      uint32_t *noise_seed, uint32_t *normal_seed);

/* Transverse gradient moments of the stationary SE 1D Renewal+ law with
 * correlationXY (seTransverseGradientMoments, SparseConvolutionNoise.cpp:78-99).
 * Returns 1 when the law applies; mean[2], var out. */
int gor_transverse_moments(const gpis_medium_desc *desc, const float origin[3],
                           const float dir[3], const float p[3], const uint32_t seeds[4],
                           const float prev[4], int conditioning, double mean[2], double *var);

/* Multi-resolution levels at p (kernelScaleLevelRatio, SparseConvolutionNoise.cpp:101-111):
 * info = (low scale, high scale, low weight, high weight) and the two levels'
 * noise-seed offsets.  EINVAL for a medium without the multi-resolution grid. */
int gor_level_ratio(const gpis_medium_desc *desc, const float p[3], float info[4], uint32_t level_seeds[2]);

/* 1D NEE PDF and gradient (neePDF / neeGrad, SparseConvolutionNoise.cpp:662-821). */
int gor_nee(const gpis_medium_desc *desc, const float origin[3], const float dir[3],
            const float p[3], const float normal[3], float t_segment, const uint32_t seeds[4],
            const float prev[4], float *pdf, float grad[3]);

/* Sampling scheme at a point (samplingScheme, SparseConvolutionNoise.cpp:68-76). */
int gor_sampling_scheme(const gpis_medium_desc *desc, const float origin[3], const float p[3],
                        const uint32_t seeds[4]);

/* Medium queries over oracle flights (GaussianProcessMedium state machines,
 * GaussianProcessMedium.cpp:222-440); single-threaded. */
int gor_medium_sample_distance(const gpis_medium_desc *desc, const gpis_ray *rays, gpis_medium_state *states,
                               const float *jitter, gpis_medium_sample *samples, uint32_t n);
int gor_medium_transmittance(const gpis_medium_desc *desc, const gpis_ray *rays, gpis_medium_state *states,
                             const float *jitter, float *transmittance, uint32_t n);

/* Path tracer restatement (gpis_render): rows [row0, row0 + rows) of the image;
 * counts[4] += {distance flights, shadow flights, medium events, failed paths}. */
int gor_render(const gpis_medium_desc *md, const gpis_scene_desc *sc, float *image, uint64_t counts[4],
               uint32_t row0, uint32_t rows);
int gor_render_span(const gpis_medium_desc *md, const gpis_scene_desc *sc, float *image, uint64_t counts[4],
                    uint32_t row, uint32_t col0, uint32_t cols);

/* Elementwise SE splat in FP64 (the SeSplat1DTest expectation, SeSplat1DTest.cpp:72-84). */
void gor_se_splat_1d(const float *q, const float *c, uint32_t n, float scale,
                     double *values, double *derivatives);

#ifdef __cplusplus
}
#endif

#endif
