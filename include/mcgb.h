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
 * rule; one draw per visit: u1 = (2k+1) 2^-22 from bits 63..43, u2 = k 2^-21
 * from bits 42..22 (the Box-Muller pair) and the acceptance uniform
 * k 2^-21 from bits 21..1.  No reference counterpart (configuration option
 * "Gaussian MH proposals"); oracle: orc_xy_update_color_gauss. */
int mcgb_xy_update_color_gauss(float *theta, void *rng, const float *betas,
                               const float *sigmas, int R, int L, int color, float J,
                               void *stream);
/* A whole sweep (core/runtime.py:87-99: colours 0, 1, 2, 3 of
 * models/xy/update.py:6-54, or of the Gaussian proposal when sigmas is not
 * NULL) in three launches per sweep -- colours 0, {1, 2}, 3: colours 1 and
 * 2 share no bond -- bit-identical to four update_color calls; n_sweeps
 * sweeps. */
int mcgb_xy_sweep(float *theta, void *rng, const float *betas, const float *sigmas, int R, int L,
                  float J, float delta, int n_sweeps, void *stream);
/* Plain FP64 form: one lattice (replica r) per launch, float64 state,
 * float64 betas and sigmas, float64 uniforms; sigmas NULL = uniform delta.
 * With w2t NULL, betas and sigmas are per walker; otherwise they are per
 * temperature slot and walker r reads entry w2t[r] (a PT ladder whose
 * exchanges permute w2t).  No reference counterpart: the float64 baseline
 * the mixed-precision batch is compared with. */
int mcgb_xy64_update_color(double *theta, void *rng, const double *betas,
                           const double *sigmas, const int32_t *w2t, int R, int L, int r,
                           int color, double J, double delta, void *stream);
/* FP64 energy of one lattice (replica r) into out[r]. */
int mcgb_xy64_energy(const double *theta, int R, int L, int r, double J, double *out,
                     void *stream);
/* The five channels of models/xy/measure.py:17-101 (energy, mx, my,
 * twist_cos_x, twist_sin_x) of one lattice of the plain FP64 form, summed in
 * float64, into column w2t[r] (w2t NULL: r) of out (5, R). */
int mcgb_xy64_measure(const double *theta, int R, int L, int r, double J, const int32_t *w2t,
                      double *out, void *stream);
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
/* A whole sweep (core/runtime.py:87-99 over models/kawamura/update.py:7-65)
 * in three launches, colours 0, {1, 2}, 3, bit-identical to four
 * update_color calls; n_sweeps sweeps. */
int mcgb_kawamura_sweep(float *state, void *rng, const float *betas, int R, int L, float J, float delta,
                        int n_sweeps, void *stream);
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
/* core/parallel_tempering.py:35-91 _exchange_kernel with the schedule
 * arguments it takes from ParallelTempering.attempt_exchanges
 * (core/parallel_tempering.py:255-269: `self._parity`, `self.sweeps`) read
 * from a device clock int64 {sweeps, rounds} instead: the round runs after
 * clock[0] + advance sweeps at parity rounds % 2 (0 when R == 2), then the
 * clock becomes {clock[0] + advance, rounds + 1}.  Same results as
 * mcgb_pt_exchange; a captured CUDA graph of it replays each round at its
 * own sweep and parity. */
int mcgb_pt_exchange_clocked(const double *energies, float *betas, int32_t *walker_to_temperature,
                             int32_t *temperature_to_walker, void *rng, int64_t *swap_counts,
                             int64_t *trips, int R, int64_t *clock, int advance, void *stream);
/* core/parallel_tempering.py:206-216 _record_walker_history into a device
 * ring: row head[0] % capacity of ring [capacity][n] receives
 * walker_to_temperature[walker_ids[k]], then head[0] += 1 (replaces the
 * per-row pointer of mcgb_pt_record_walkers inside captured graphs). */
int mcgb_pt_record_walkers_ring(const int32_t *walker_to_temperature, const int32_t *walker_ids,
                                int32_t *ring, int64_t *head, int n, int64_t capacity, void *stream);
/* core/simulation.py:39-66 sample accumulation (`samples[name].append`)
 * on the device: copy n float64 values from src to slot head[0] % capacity
 * of ring [capacity][n], then head[0] += 1.  One bulk copy of the ring
 * replaces a host copy per sample. */
int mcgb_ring_push(const double *src, double *ring, int64_t *head, int64_t n, int64_t capacity, void *stream);

/* ------------------------------------------------------------ Handle API
 * One reference Runtime (core/runtime.py:8-135) with its ParallelTempering
 * state (core/parallel_tempering.py:94-317) behind an opaque handle that
 * owns its device buffers, for C callers that want the reference's object
 * model instead of raw kernels.  Replicas may differ in L (runs of equal L
 * in table order).  Every call is asynchronous on the handle's stream (but
 * mc_create, mc_copy_in/out and mc_destroy, which synchronise it) and
 * returns MCGB_OK or a negative status; mc_get_error repeats the handle's
 * last status, mcgb_last_error() the message.  Models: MCGB_MODEL_ISING,
 * _XY (uniform, or Gaussian with params->sigmas), _KAWAMURA, _HE3 and
 * _HE3_GAUSS. */
typedef struct mc_handle mc_handle;

typedef struct mc_params {
    float J;                  /* coupling (Ising, XY, Kawamura) */
    float delta;              /* uniform proposal width (XY, Kawamura) / He3 Cartesian step */
    const float *sigmas;      /* XY: host (R,) Gaussian widths per replica, NULL = uniform delta */
    float coefficients[5];    /* He3: GL betas */
    float K, g_d;             /* He3: gradient coupling, dipole */
    float rho, mass;          /* He3 conditional Gaussian sampler */
} mc_params;

enum {
    MC_STATE = 0,         /* reference layout, runs concatenated: int8 / float / 5 floats / 6 floats a site */
    MC_RNG = 1,           /* 16-byte streams, stream index = global site index */
    MC_BETAS = 2,         /* float (R,), walker order */
    MC_ENERGIES = 3,      /* double (R,), walker order, as of the last mc_energy / mc_exchange */
    MC_W2T = 4,           /* int32 (R,) walker_to_temperature */
    MC_T2W = 5,           /* int32 (R,) temperature_to_walker */
    MC_SWAP_COUNTS = 6,   /* int64 (3, R-1) attempts, accepted, nonfinite */
    MC_TRIPS = 7,         /* int64 (5, R) round-trip bookkeeping */
    MC_EXCHANGE_RNG = 8,  /* 16-byte streams (R-1,), one per neighbouring pair */
};

/* Runtime(model, L, temperatures, seed) + ParallelTempering(seed + 1):
 * site streams seeded with `seed` (stream = global site index), exchange
 * streams with seed + 1, betas 1/T, identity maps, the ordered state (Ising
 * +1, XY 0, Kawamura theta 0, tau +1, d = z; He3 zero) until mc_copy_in.
 * stream NULL: the legacy default stream. */
int mc_create(int model_id, const mc_params *params, const int32_t *L_table, int R,
              const double *temperatures, uint64_t seed, void *stream, mc_handle **out);
/* n_sweeps sweeps, colours 0, 1, 2, 3 each (core/runtime.py:87-99). */
int mc_sweep(mc_handle *h, int n_sweeps);
/* One colour of every replica (Model.update_color, core/model.py:16-23). */
int mc_update_color(mc_handle *h, int color);
/* Energies (R,) float64 in walker order into device `out`, or into the
 * handle's MC_ENERGIES buffer when out is NULL (Model.measure_energy). */
int mc_energy(mc_handle *h, double *out);
/* Model.measure: out device (channels, R) float64; temperature_index
 * (device, int32 (R,), nullable) puts walker w's values in column
 * temperature_index[w]; cached_energy (device, float64 (R,) walker order,
 * nullable) replaces the energy channel (core/model.py:25-48).  Channels:
 * Ising 2, XY 5, Kawamura 7, He3 10 (mcgb_batch_channels). */
int mc_measure(mc_handle *h, const int32_t *temperature_index, const double *cached_energy,
               double *out);
/* One exchange round at `parity` after sweep `sweep`: the energies, then
 * core/parallel_tempering.py:35-91 on the handle's maps and counters. */
int mc_exchange(mc_handle *h, int parity, int64_t sweep);
/* Reseed the site streams: create_xoroshiro128p_states(sites, seed,
 * subsequence) (core/runtime.py:51-53). */
int mc_rng_init(mc_handle *h, uint64_t seed, uint64_t subsequence);
/* The handle's last status (MCGB_EINVAL for a NULL handle). */
int mc_get_error(const mc_handle *h);
/* Synchronous host copies of a buffer (MC_STATE ... MC_EXCHANGE_RNG); n_bytes
 * must equal its size. */
int mc_copy_in(mc_handle *h, int buffer, const void *host, int64_t n_bytes);
int mc_copy_out(mc_handle *h, int buffer, void *host, int64_t n_bytes);
/* Frees the handle and its buffers (after its stream's work). */
int mc_destroy(mc_handle *h);

/* ------------------------------------------------------------ Batched engine
 * No single reference counterpart: these run what the reference does with
 * one Runtime per (L, ladder) and four launches per sweep
 * (core/runtime.py:87-99, core/parallel_tempering.py:245-269,
 * core/simulation.py:36-72) as one launch per exchange window over a table
 * of replicas of any mix of L.  Inside a window the lattice of each replica
 * lives in the shared memory of one thread-block cluster (one strip of rows
 * per CTA) and its RNG streams in registers.
 *
 * Batch layout ("colour-major"): per replica, four planes (one per
 * checkerboard colour c = 2*(i%2) + j%2) of (L/2) x (L/2) sites each; the
 * RNG array has one 16-byte stream per site in the same order.  The
 * permutation kernels below convert from/to the reference layout, keeping
 * each site's stream. */

enum {
    MCGB_MODEL_ISING = 0,
    MCGB_MODEL_XY = 1,
    MCGB_MODEL_KAWAMURA = 2,
    MCGB_MODEL_HE3 = 3,       /* Cartesian proposals */
    MCGB_MODEL_HE3_GAUSS = 4, /* conditional Gaussian MH proposals */
    MCGB_MODEL_KAWAMURA_GAUSS = 5, /* Gaussian MH proposals (theta and d), widths sigma_t;
                                      no reference counterpart */
    /* Windows over replicas stored in the reference layout instead: (R, L, L)
     * states, the stream of site (i, j) of replica r at r*L*L + i*L + j, one
     * replica of size L per table entry with state_offset = r*L*L.  Only
     * mcgb_batch_smem_bytes, mcgb_batch_max_clusters and mcgb_batch_window_run
     * take them, without samples; every strip must hold at most two
     * plaquettes per thread.  The sweeps are bit-identical to four
     * mcgb_ising_update_color / mcgb_xy_update_color (uniform proposal)
     * launches each (models/ising/update.py:7-29, models/xy/update.py:6-54). */
    MCGB_MODEL_ISING_REF = 6,
    MCGB_MODEL_XY_REF = 7,
};

typedef struct mcgb_replica {
    int32_t L;             /* even, >= 4; held by the largest divisor of L/2 not above
                              cluster_size CTAs of a cluster (the others idle for it) */
    int32_t ladder;        /* ladder index */
    int32_t ladder_start;  /* first replica index (= temperature slot 0) of the ladder */
    int32_t n_temps;       /* replicas in the ladder */
    int64_t state_offset;  /* first site of the replica in the batch arrays */
} mcgb_replica;

typedef struct mcgb_batch_window {
    const mcgb_replica *table;      /* device, n_replicas entries */
    const mcgb_replica *host_table; /* host copy (validated on every call) */
    int32_t n_replicas;
    const int32_t *work_ptr;        /* device, n_clusters + 1: cluster k runs */
    const int32_t *work_idx;        /*   work_idx[work_ptr[k] .. work_ptr[k+1]) */
    int32_t n_clusters, cluster_size, threads;
    void *state;                    /* colour-major: int8 / float / 5 floats / 6 complex64 per site */
    void *rng;                      /* colour-major 16-byte streams */
    void *aux;                      /* XY, Kawamura: colour-major (cos theta, sin theta) float pairs
                                       kept with the state so every window sees the values the
                                       updates computed; NULL for other models */
    const float *betas;             /* per replica, walker order */
    const int32_t *w2t;             /* per replica: temperature slot within its ladder */
    float *e_run;                   /* 2 per replica: compensated running energy (hi, lo) */
    double *energies;               /* out, per replica: energy after the window */
    long long *accepted;            /* per replica: += accepted moves (He3: all sub-counters) */
    long long *counters;            /* He3 Gaussian: (3, n_replicas) attempts/accepted/nonfinite, else NULL */
    double *samples;                /* ring of [n_slots][channels][n_temps_total] or NULL; the
                                       sample after cumulative sweep s lands in slot
                                       ((s - first_sample_sweep) / sample_interval) % n_slots */
    double *staging;                /* [channels][n_replicas]: when not NULL, a sample due at the
                                       window's last sweep goes here (walker order) for the exchange
                                       to scatter with the updated temperature map */
    int32_t n_temps_total, n_slots;
    const int64_t *clock;           /* device {sweeps completed, exchange rounds} before the window */
    int64_t first_sample_sweep;     /* cumulative sweep number of sample slot 0 */
    int32_t sample_interval;        /* 0 = no samples; at most 2^24 */
    int32_t n_sweeps;               /* sweeps in this window, 0 .. 2^24 (a resident launch: at
                                       most 2^28 over its windows) */
    float J, delta;                 /* Ising/XY/Kawamura coupling, uniform proposal width */
    const float *sigma_t;           /* XY: Gaussian width per temperature slot (NULL = uniform delta) */
    float coefficients[5], K, g_d, rho, mass; /* He3 */
    const int32_t *host_work_idx;   /* host copy of work_idx (n_work entries), or NULL: the work
                                       lists hold every replica of the table; a launch over part of
                                       the table (one size group) sizes shared memory and picks its
                                       variant from the replicas listed here */
    int32_t n_work;                 /* entries in host_work_idx */
    int32_t hold_clock;             /* fused window + exchange launches: nonzero leaves the clock to
                                       another launch of the same window (several size groups each
                                       run the window over their replicas; the last one advances) */
} mcgb_batch_window;

/* Number of float64 sample channels a model writes per replica. */
int mcgb_batch_channels(int model);
/* Dynamic shared memory (bytes) a window needs for a replica of size L in
 * clusters of cluster_size CTAs (a batch needs the maximum over its L). */
int64_t mcgb_batch_smem_bytes(int model, int L, int cluster_size);
/* Largest number of co-resident clusters of `cluster_size` CTAs of `threads`
 * threads with `smem_bytes` dynamic shared memory (cudaOccupancyMaxActiveClusters). */
int mcgb_batch_max_clusters(int model, int cluster_size, int threads, int64_t smem_bytes, int *out);
/* One window of n_sweeps sweeps over every replica of the batch. */
int mcgb_batch_window_run(int model, const mcgb_batch_window *w, void *stream);
/* Reference layout <-> colour-major, elem_bytes per site (a multiple of 1, 4
 * or 16), for every replica of the table (device) with n_replicas entries and
 * max_L the largest L.  direction 0: reference -> batch, 1: batch -> reference.
 * `ref_offsets` (device, int64 per replica) gives each replica's first site in
 * the reference-layout array. */
int mcgb_batch_permute(const void *src, void *dst, int64_t elem_bytes, const mcgb_replica *table,
                       const int64_t *ref_offsets, int n_replicas, int max_L, int direction,
                       void *stream);
/* Recompute the (cos, sin) cache `aux` from the state (after the state was
 * written from outside a window). */
int mcgb_batch_refresh_aux(int model, const mcgb_batch_window *w, void *stream);
/* FP64 total energy of every replica from the colour-major state (the
 * periodic drift check): writes energies[r], drift[r] = running - exact, and
 * resets e_run[r] to the exact value. */
int mcgb_batch_recompute_energy(int model, const mcgb_batch_window *w, double *drift, void *stream);
/* Parallel-tempering bookkeeping of a batch: per ladder l, replicas
 * [ladder_starts[l], ladder_starts[l] + ladder_sizes[l]); t2w holds, per
 * ladder slot, the walker index local to the ladder (w2t in the window block
 * holds the slot per replica); rng has one stream per neighbouring pair
 * (pair index = ladder_start - l + left); swap_counts is (3, n_pairs_total),
 * trips (5, n_replicas). */
typedef struct mcgb_batch_pt {
    int32_t *t2w;
    void *rng;
    int64_t *swap_counts;
    int64_t *trips;
    const int32_t *ladder_starts;
    const int32_t *ladder_sizes;
    int32_t n_ladders;
    int32_t channels;               /* sample channels of the model (staging rows) */
} mcgb_batch_pt;

/* Replica exchange for every ladder (one thread block per ladder,
 * core/parallel_tempering.py:35-91 per ladder) after a window described by
 * `w` (energies, betas, w2t, clock, n_sweeps; samples/staging for the
 * deferred window-end sample).  The trip sweep is clock[0] + n_sweeps and the
 * matching parity of a ladder with more than two replicas is clock[1] % 2
 * (two-replica ladders always use 0), as core/parallel_tempering.py:245-269
 * schedules them.  A staged window-end sample is then written to the slots
 * of the updated map, matching a measurement taken after the exchange. */
int mcgb_batch_exchange(const mcgb_batch_window *w, const mcgb_batch_pt *pt, void *stream);
/* No counterpart in the reference.  mcgb_batch_window_run then
 * mcgb_batch_exchange in one call that allocates nothing, for callers that
 * cannot allocate device memory: a program inside a host runtime that owns
 * every device allocation (a pool sized to the whole GPU, or a binding whose
 * allocator must not be bypassed), or a latency-critical loop that cannot
 * afford cudaMalloc's implicit device synchronisation.  w->staging must be
 * NULL: the deferred-sample scratch is a fixed array in the library of 32768
 * doubles, so channels x n_replicas must not exceed 32768 (else MCGB_EINVAL).
 * One launch over the whole replica table only: host_work_idx NULL, n_work 0
 * and hold_clock 0 (size-group windows are rejected with MCGB_EINVAL).  All
 * calls on one device share that array and must not overlap on the GPU
 * (serialise them on one stream); each device has its own copy.  The first
 * call in a CUDA context looks up the array's address; make it before any
 * stream capture.  The caller ticks the clock as with the two separate calls. */
int mcgb_batch_window_exchange_noalloc(int model, const mcgb_batch_window *w, const mcgb_batch_pt *pt,
                                       void *stream);
/* No counterpart in the reference (it launches four colour kernels per sweep
 * and one exchange kernel per round, core/parallel_tempering.py:245-269).
 * mcgb_batch_window_run, mcgb_batch_exchange and
 * mcgb_batch_clock_tick(clock, n_sweeps, 1) in ONE launch: each pair of the
 * matching is decided by the second of its two walkers to finish (with the
 * same result as mcgb_batch_exchange), and the last cluster to finish
 * advances the clock.  At most 32 sample channels.  `sync` is
 * 5 * n_replicas + 2 int32, 16-byte aligned, zero before the first call:
 * per-pair mailboxes and decision words (tagged with the exchange-round
 * count clock[1]), a launch counter and an error flag.  One `sync` array per
 * batch, kept for its lifetime; zero all of it if clock[1] is ever set back.
 * Calls sharing it must not overlap on the GPU. */
int mcgb_batch_window_exchange(int model, const mcgb_batch_window *w, const mcgb_batch_pt *pt,
                               int32_t *sync, void *stream);
/* No counterpart in the reference.  n_windows consecutive windows of
 * w->n_sweeps sweeps, each followed by every ladder's exchange and a clock
 * tick, in ONE cooperative launch that keeps every strip, its halos and its
 * RNG streams on chip between windows (loaded once, written back once).
 * Needs one cluster per replica (w->n_clusters == w->n_replicas, one replica
 * in every work list) and every cluster resident at once: otherwise the
 * launch fails (a CUDA error, MCGB_ECUDA) and nothing runs.  Between
 * windows each walker waits only for its own pair's decision.  `sync` is the
 * array of mcgb_batch_window_exchange; its last entry is an error flag the
 * kernel sets (and leaves set) if such a wait gave up after about a second:
 * check it after the run.  After a failed launch the slot maps may disagree
 * (t2w not the inverse of w2t): rebuild them and zero `sync` before going on.
 * n_windows = 1 is mcgb_batch_window_exchange. */
int mcgb_batch_run_resident(int model, const mcgb_batch_window *w, const mcgb_batch_pt *pt,
                            int32_t *sync, int n_windows, void *stream);
/* No counterpart in the reference.  Polls of a resident launch's wait
 * between windows before it gives up and raises the error flag (default
 * 2^22, about a second; negative restores the default); a walker whose wait
 * gave up runs the launch's later windows at the slot and beta it had.
 * Applies to later calls; returns the previous value.  With 0 every such
 * wait gives up before its first poll, which is how the timeout path is
 * tested. */
int64_t mcgb_batch_set_wait_limit(int64_t polls);
/* Advance the device clock: clock[0] += n_sweeps, clock[1] += exchanged, so
 * a captured graph of windows and exchanges can be replayed. */
int mcgb_batch_clock_tick(int64_t *clock, int n_sweeps, int exchanged, void *stream);
/* Robbins-Monro step of the per-temperature Gaussian widths towards a target
 * acceptance: sigma_t[slot] *= exp(gain * (rate - target)), clamped to
 * [lo, hi], rate = (accepted - accepted_prev) / (L^2 * n_sweeps) of the
 * replica at that slot; then accepted_prev = accepted. */
int mcgb_batch_tune_sigma(float *sigma_t, const long long *accepted, long long *accepted_prev,
                          const int32_t *w2t, const mcgb_replica *table, int n_replicas, int n_sweeps,
                          float target, float gain, float lo, float hi, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MCGB_H */
