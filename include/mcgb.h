/*
 * mcgb — GB300-native lattice Monte Carlo hot path: the C ABI.
 *
 * Every entry point takes plain device pointers and sizes, enqueues its work
 * on `stream` (a cudaStream_t passed as void*; NULL = legacy default stream)
 * and returns an int status: 0 on success, a negative MCGB_E* code on error
 * (message in mcgb_last_error(), per host thread).  Nothing here synchronises
 * the stream or copies to the host unless stated.
 *
 * Layouts are the reference's (JinhaoR/GPU-monte-carlo), C order:
 *   Ising    int8     (R, L, L)
 *   XY       float32  (R, L, L)            angles in [-pi, pi)
 *   Kawamura float32  (R, L, L, 5)         theta, tau, dx, dy, dz
 *   He3      complex64 (R, L, L, 3, 2)     as interleaved float pairs
 *   RNG      16-byte records {uint64 s0, uint64 s1}, stream r*L*L + i*L + j
 *   betas    float32 (R,) inverse temperatures, physical walker order
 *   measure  float64 (C, R); column = temperature_indices[r] when given
 * Each declaration names the reference interface it replaces (file:line).
 */
#ifndef MCGB_H
#define MCGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MCGB_OK = 0,
    MCGB_EINVAL = -1,   /* bad argument (sizes, null pointers, ranges) */
    MCGB_ECUDA = -2,    /* CUDA runtime error at launch or in an API call */
    MCGB_ENOMEM = -3,   /* device allocation failed */
    MCGB_ETIMEOUT = -4, /* a bounded device-side wait gave up */
};

/* Last error message of the calling host thread ("" after success). */
const char *mcgb_last_error(void);
/* Library version string. */
const char *mcgb_version(void);

/* ------------------------------------------------------------ RNG
 * Replaces numba.cuda.random.create_xoroshiro128p_states(n, seed,
 * subsequence_start) as called at core/runtime.py:51-53 and
 * core/parallel_tempering.py:177-179.  Stream k equals stream 0 advanced by
 * (subsequence_start + k) * 2^64 steps; computed on the device by GF(2)
 * jump-ahead instead of n sequential host jumps. */
int mcgb_rng_init(void *states, int64_t n, uint64_t seed, uint64_t subsequence_start,
                  void *stream);
/* Draw `count` consecutive float32 (kind 0) or float64 (kind 1) uniforms
 * from stream `index`, advancing it (numba xoroshiro128p_uniform_float32/64).
 * Writes `out` (device, count elements). Diagnostic/parity use. */
int mcgb_rng_draw(void *states, int64_t index, int count, int kind, void *out, void *stream);
/* out[k] = expf(x[k]) with CUDA's non-fast-math expf (the Metropolis
 * acceptance exponential). Diagnostic/parity use. */
int mcgb_expf(const float *x, float *out, int64_t n, void *stream);

/* ------------------------------------------------------------ Ising
 * models/ising/update.py:7-29 metropolis_color (Model.update_color,
 * core/model.py:16-23): one checkerboard colour, one uniform per visit. */
int mcgb_ising_update_color(int8_t *spins, void *rng, const float *betas, int R, int L,
                            int color, float J, void *stream);
/* Fused sweep: colours 0, {1, 2}, 3 of n_sweeps sweeps (bit-identical to four
 * update_color calls per sweep: colours 1 and 2 share no bond). */
int mcgb_ising_sweep(int8_t *spins, void *rng, const float *betas, int R, int L, float J,
                     int n_sweeps, void *stream);
/* models/ising/measure.py:71-99 ising_energy_kernel: out (R,) float64. */
int mcgb_ising_energy(const int8_t *spins, int R, int L, float J, double *out, void *stream);
/* models/ising/measure.py:10-68 (plain / ordered / cached / ordered+cached):
 * out (2, R) = energy, magnetization; temperature_indices and cached_energies
 * may be NULL. */
int mcgb_ising_measure(const int8_t *spins, int R, int L, float J,
                       const int32_t *temperature_indices, const double *cached_energies,
                       double *out, void *stream);

/* ------------------------------------------------------------ XY
 * models/xy/update.py:6-54: uniform proposal theta + delta*(2u-1). */
int mcgb_xy_update_color(float *theta, void *rng, const float *betas, int R, int L, int color,
                         float J, float delta, void *stream);
/* Gaussian proposal theta + sigma_r * z (per-walker sigma), same acceptance
 * rule; three draws per visit.  No reference counterpart (configuration
 * option "Gaussian MH proposals"); oracle: orc_xy_update_color_gauss. */
int mcgb_xy_update_color_gauss(float *theta, void *rng, const float *betas,
                               const float *sigmas, int R, int L, int color, float J,
                               void *stream);
/* Plain FP64 form: one lattice (replica r) per launch, float64 state,
 * float64 betas and sigmas, float64 uniforms; sigmas NULL = uniform delta. */
int mcgb_xy64_update_color(double *theta, void *rng, const double *betas,
                           const double *sigmas, int R, int L, int r, int color, double J,
                           double delta, void *stream);
/* FP64 energy of one lattice (replica r) into out[r]. */
int mcgb_xy64_energy(const double *theta, int R, int L, int r, double J, double *out,
                     void *stream);
/* models/xy/measure.py:104-134 xy_energy_kernel. */
int mcgb_xy_energy(const float *theta, int R, int L, float J, double *out, void *stream);
/* models/xy/measure.py:17-101: out (5, R) = energy, mx, my, twist_cos_x,
 * twist_sin_x. */
int mcgb_xy_measure(const float *theta, int R, int L, float J,
                    const int32_t *temperature_indices, const double *cached_energies,
                    double *out, void *stream);

/* ------------------------------------------------------------ Kawamura
 * models/kawamura/update.py:21-65 (three sub-moves, six draws per visit). */
int mcgb_kawamura_update_color(float *state, void *rng, const float *betas, int R, int L,
                               int color, float J, float delta, void *stream);
/* models/kawamura/measure.py:96-122. */
int mcgb_kawamura_energy(const float *state, int R, int L, float J, double *out, void *stream);
/* models/kawamura/measure.py:14-93: out (7, R) = energy, chirality, px, py,
 * spin2, twist_cos_x, twist_sin_x. */
int mcgb_kawamura_measure(const float *state, int R, int L, float J,
                          const int32_t *temperature_indices, const double *cached_energies,
                          double *out, void *stream);
/* For n rows (r, i, j) of `positions` (int32, n x 3) and proposed site
 * values (float32, n x 5): out (2, n) float32 = local energy of the stored
 * site and of the proposal (models/kawamura/update.py:7-18 local_energy).
 * Diagnostic/parity use. */
int mcgb_kawamura_local_energies(const float *state, int R, int L, const int32_t *positions,
                                 const float *proposed, int n, float J, float *out,
                                 void *stream);

/* ------------------------------------------------------------ He3
 * coefficients: 5 float32 GL betas (He3Model.betas, host array).
 * models/he3/update.py:178-227: Cartesian proposal, 13 draws per visit. */
int mcgb_he3_update_color(float *state, void *rng, const float *betas, int R, int L, int color,
                          const float *coefficients, float K, float delta, float g_d,
                          void *stream);
/* models/he3/gaussian_fast.py:91-119 fast_gaussian_color: conditional
 * Gaussian AR proposal with MH correction; counts (3, R, L, L) int64
 * (attempted, accepted, nonfinite). */
int mcgb_he3_gaussian_update_color(float *state, void *rng, const float *betas, int R, int L,
                                   int color, const float *coefficients, float K, float rho,
                                   float mass, float g_d, int64_t *counts, void *stream);
/* models/he3/measure.py:115-143. */
int mcgb_he3_energy(const float *state, int R, int L, const float *coefficients, float K,
                    float g_d, double *out, void *stream);
/* models/he3/measure.py:22-113: out (10, R) = energy, density, chirality,
 * phase_real, phase_imag, current_x, curvature_x, current_y, curvature_y,
 * spin_alignment. */
int mcgb_he3_measure(const float *state, int R, int L, const float *coefficients, float K,
                     float g_d, const int32_t *temperature_indices,
                     const double *cached_energies, double *out, void *stream);
/* For n rows (r, i, j) of `positions` (int32, n x 3) and proposed site
 * values (complex64, n x 3 x 2): out (3, n) float64 = gradient difference,
 * potential difference, potential difference + K * gradient difference
 * (models/he3/update.py:32-63 potential, :95-175 gradient_difference).
 * Diagnostic/parity use. */
int mcgb_he3_local_differences(const float *state, int R, int L, const int32_t *positions,
                               const float *proposed, int n, const float *coefficients,
                               float K, float g_d, double *out, void *stream);

/* ------------------------------------------------------------ PT
 * core/parallel_tempering.py:35-91 _exchange_kernel: one matching of
 * neighbouring temperatures at `parity`; swaps betas and both maps on
 * acceptance; swap_counts (3, R-1) int64, trips (5, R) int64. */
int mcgb_pt_exchange(const double *energies, float *betas, int32_t *walker_to_temperature,
                     int32_t *temperature_to_walker, void *rng, int64_t *swap_counts,
                     int64_t *trips, int R, int parity, int64_t sweep, void *stream);
/* core/parallel_tempering.py:28-32 _record_walkers_kernel:
 * history_row[k] = walker_to_temperature[walker_ids[k]]. */
int mcgb_pt_record_walkers(const int32_t *walker_to_temperature, const int32_t *walker_ids,
                           int32_t *history_row, int n, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MCGB_H */
