/*
 * CPU oracle for the lattice Monte Carlo hot path (test infrastructure only).
 *
 * This library restates, in plain C, the reference's Numba-CUDA kernels for
 * the checkerboard Metropolis sweeps, the per-site xoroshiro128+ streams,
 * the measurement/energy reductions and the parallel-tempering exchange.
 * It is the checker for the CUDA library and the timed CPU baseline; the
 * product path never links or calls it.
 *
 * Parity pins (see tests/test_oracle_*.py):
 *   - SplitMix64 seeding checked against a published SplitMix64 test vector;
 *   - the xoroshiro128+ jump constant checked against x^(2^64) mod the
 *     engine's characteristic polynomial (derived from the output stream by
 *     Berlekamp-Massey), so stream k really is stream 0 advanced by k*2^64;
 *   - the reference tests' deterministic known-answer cases (Ising beta
 *     limits, ordered-state observables, NumPy formula references).
 * The RNG itself lives in a third-party package (numba.cuda.random, Numba
 * 0.68.0) that is absent here; no reference test pins raw RNG outputs.
 */
#ifndef MC_ORACLE_H
#define MC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- xoroshiro128+ per-site streams (numba.cuda.random restated) ---- */
void orc_rng_init(uint64_t *states, int64_t n, uint64_t seed, uint64_t subsequence_start);
uint64_t orc_rng_next(uint64_t *state);
void orc_rng_jump(uint64_t *state);
float orc_rng_uniform_f32(uint64_t *state);
double orc_rng_uniform_f64(uint64_t *state);
uint64_t orc_splitmix64_first(uint64_t seed);

/* ---- Ising: int8 spins (R, L, L) ---- */
void orc_ising_update_color(int8_t *spins, uint64_t *rng, const float *betas,
                            int R, int L, int color, float J);
void orc_ising_sweeps(int8_t *spins, uint64_t *rng, const float *betas,
                      int R, int L, float J, int n_sweeps, int n_threads);
/* As orc_ising_sweeps with a per-replica table (R x 5) of the acceptance
 * exponentials exp(-beta * float32(k) * J), k = -8, -4, 0, 4, 8. */
void orc_ising_sweeps_tab(int8_t *spins, uint64_t *rng, const float *betas, const float *tab,
                          int R, int L, float J, int n_sweeps, int n_threads);
void orc_ising_energy(const int8_t *spins, int R, int L, float J, double *out);
void orc_ising_measure(const int8_t *spins, int R, int L, float J,
                       const int32_t *temperature_indices, const double *cached,
                       double *out);

/* ---- XY: float32 angles (R, L, L) ---- */
void orc_xy_update_color(float *theta, uint64_t *rng, const float *betas,
                         int R, int L, int color, float J, float delta);
void orc_xy_update_color_gauss(float *theta, uint64_t *rng, const float *betas,
                               const float *sigmas, int R, int L, int color, float J);
void orc_xy_sweeps(float *theta, uint64_t *rng, const float *betas, const float *sigmas,
                   int R, int L, float J, float delta, int n_sweeps, int n_threads);
void orc_xy_energy(const float *theta, int R, int L, float J, double *out);
void orc_xy_measure(const float *theta, int R, int L, float J,
                    const int32_t *temperature_indices, const double *cached,
                    double *out);

/* ---- Kawamura: float32 (R, L, L, 5) = theta, tau, dx, dy, dz ---- */
float orc_kawamura_local_energy(const float *state, int L, int r, int i, int j,
                                float theta, float tau, float dx, float dy, float dz,
                                float J);
void orc_kawamura_update_color(float *state, uint64_t *rng, const float *betas,
                               int R, int L, int color, float J, float delta);
void orc_kawamura_sweeps(float *state, uint64_t *rng, const float *betas,
                         int R, int L, float J, float delta, int n_sweeps, int n_threads);
void orc_kawamura_update_color_gauss(float *state, uint64_t *rng, const float *betas,
                                     const float *sigmas, int R, int L, int color, float J);
void orc_kawamura_sweeps_gauss(float *state, uint64_t *rng, const float *betas, const float *sigmas,
                               int R, int L, float J, int n_sweeps, int n_threads);
void orc_kawamura_energy(const float *state, int R, int L, float J, double *out);
void orc_kawamura_measure(const float *state, int R, int L, float J,
                          const int32_t *temperature_indices, const double *cached,
                          double *out);

/* ---- He3: complex64 (R, L, L, 3, 2) stored as float pairs ---- */
float orc_he3_potential(const float *psi, const float *coeff, float g_d);
float orc_he3_gradient_difference(const float *state, int L, int r, int i, int j,
                                  const float *proposed);
void orc_he3_update_color(float *state, uint64_t *rng, const float *betas,
                          int R, int L, int color, const float *coeff, float K,
                          float delta, float g_d);
void orc_he3_gaussian_update_color(float *state, uint64_t *rng, const float *betas,
                                   int R, int L, int color, const float *coeff, float K,
                                   float rho, float mass, float g_d, int64_t *counts);
void orc_he3_sweeps(float *state, uint64_t *rng, const float *betas, int R, int L,
                    const float *coeff, float K, float delta, float g_d,
                    int gaussian, float rho, float mass, int64_t *counts,
                    int n_sweeps, int n_threads);
void orc_he3_energy(const float *state, int R, int L, const float *coeff, float K,
                    float g_d, double *out);
void orc_he3_measure(const float *state, int R, int L, const float *coeff, float K,
                     float g_d, const int32_t *temperature_indices,
                     const double *cached, double *out);

/* ---- Parallel tempering exchange ---- */
void orc_pt_exchange(const double *energies, float *betas, int32_t *walker_to_temperature,
                     int32_t *temperature_to_walker, uint64_t *rng, int64_t *swap_counts,
                     int64_t *trips, int R, int parity, int64_t sweep);

#ifdef __cplusplus
}
#endif

#endif
