/*
 * Synthetic NLOS captures for benchmarks and tests (no counterpart in the reference,
 * which reads captures from the Zaragoza HDF5 dataset, dataset_loader.hpp:175-234).
 * Host code (OpenMP), deterministic for a given input and seed.
 */
#ifndef BPGB_SYNTH_H
#define BPGB_SYNTH_H

#include <stdint.h>

#include "backprojector_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* out[p, t] (P x T floats, overwritten): sum over scatterers q with
 *   t = round((lw_p + |l_p - q| + |q - c_p| + cw_p - t0) / deltaT) in [0, T)
 * of albedo_q / (|l_p - q|^2 |q - c_p|^2) (1/r^2 per leg).  Geometry in double. */
int bpgb_synth_render(const bpgb_pair *pairs, uint64_t num_pairs, uint32_t T, float t0,
                      float deltaT, const float *points, const float *albedo,
                      uint64_t num_points, float *out);

/* Device form of bpgb_synth_render for training scenes: pairs, points (xyz), albedo and
 * out ([P, pitch] floats; bins T..pitch-1 written as zero) in device memory, launched on
 * `stream`.  Geometry in FP32 (|l - q| + |q - c| + lw + cw, bin = round((d - t0) * (1 /
 * deltaT))), 1/r^2 weights and per-bin sums in FP64, added in scatterer order, so the
 * result is deterministic; it differs from the host renderer's FP64 bins only where a
 * path lies within FP32 rounding of a bin edge.  T <= 25,600. */
int bpgb_synth_render_device(const bpgb_pair *d_pairs, uint64_t num_pairs, uint32_t T, float t0,
                             float deltaT, const float *d_points, const float *d_albedo,
                             uint64_t num_points, float *d_out, uint32_t pitch, void *stream);

/* Scales H so that its maximum equals `peak` and replaces every bin by a Poisson sample
 * of that mean (Knuth's method below 30, rounded Gaussian above), from a counter-based
 * generator keyed by (seed, bin index).  peak <= 0 only rescales nothing and returns. */
int bpgb_synth_poisson(float *H, uint64_t n, float peak, uint64_t seed);

#ifdef __cplusplus
}
#endif

#endif /* BPGB_SYNTH_H */
