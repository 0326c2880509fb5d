/*
 * CPU oracle for the lattice Monte Carlo hot path — TEST INFRASTRUCTURE.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this file's library, and only as the checker (or as the timed CPU baseline,
 * which is a restatement of the reference's algorithm: the reference has no
 * CPU sweep of its own).  Nothing in the product path calls it.
 *
 * Every function restates a kernel of the reference project
 * (JinhaoR/GPU-monte-carlo); citations are file:line in that project.  The
 * per-site RNG restates the published xoroshiro128+ (Blackman & Vigna,
 * 2016 parameters a=55, b=14, c=36) with SplitMix64 seeding, as packaged by
 * numba.cuda.random (Numba 0.68.0, third party, not vendored by the
 * reference).  Arithmetic follows the reference's precision: float32 where the
 * Numba kernels use float32, float64 where they accumulate in float64.
 * Compile with -ffp-contract=off so no fused multiply-add changes rounding.
 */
#include "mc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* xoroshiro128+ and SplitMix64 seeding                                     */
/* call sites: core/runtime.py:51-53 (create_xoroshiro128p_states(R*L*L,    */
/* seed)), core/parallel_tempering.py:177-179 (R-1 exchange streams),       */
/* draws in every update kernel and core/parallel_tempering.py:60.          */
/* ------------------------------------------------------------------------ */

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

uint64_t orc_splitmix64_first(uint64_t seed)
{
    uint64_t z = seed + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t orc_rng_next(uint64_t *s)
{
    uint64_t s0 = s[0], s1 = s[1];
    uint64_t result = s0 + s1;
    s1 ^= s0;
    s[0] = rotl64(s0, 55) ^ s1 ^ (s1 << 14);
    s[1] = rotl64(s1, 36);
    return result;
}

/* Advance by 2^64 steps: the published jump polynomial for (55, 14, 36). */
void orc_rng_jump(uint64_t *s)
{
    static const uint64_t JUMP[2] = {0xbeac0467eba5facbull, 0xd86b048b86aa9922ull};
    uint64_t a = 0, b = 0;
    for (int w = 0; w < 2; ++w)
        for (int bit = 0; bit < 64; ++bit) {
            if (JUMP[w] & (1ull << bit)) {
                a ^= s[0];
                b ^= s[1];
            }
            orc_rng_next(s);
        }
    s[0] = a;
    s[1] = b;
}

/* Stream 0 is SplitMix64(seed) in both words, advanced subsequence_start
 * jumps; stream k is stream k-1 advanced by one jump. */
void orc_rng_init(uint64_t *states, int64_t n, uint64_t seed, uint64_t subsequence_start)
{
    if (n < 1) return;
    uint64_t z = orc_splitmix64_first(seed);
    states[0] = z;
    states[1] = z;
    for (uint64_t k = 0; k < subsequence_start; ++k) orc_rng_jump(states);
    for (int64_t i = 1; i < n; ++i) {
        states[2 * i] = states[2 * i - 2];
        states[2 * i + 1] = states[2 * i - 1];
        orc_rng_jump(states + 2 * i);
    }
}

/* (x >> 11) * 2^-53 in float64, rounded to float32 (can round up to 1.0f). */
double orc_rng_uniform_f64(uint64_t *s)
{
    uint64_t x = orc_rng_next(s);
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

float orc_rng_uniform_f32(uint64_t *s) { return (float)orc_rng_uniform_f64(s); }

static inline int wrap(int i, int L) { return (i % L + L) % L; }

#ifdef _OPENMP
#define OMP_FOR_R _Pragma("omp parallel for schedule(static) num_threads(n_threads)")
#else
#define OMP_FOR_R
#endif

/* ------------------------------------------------------------------------ */
/* Ising: models/ising/update.py:7-29, models/ising/measure.py:10-99        */
/* ------------------------------------------------------------------------ */

/* `tab` (5 floats, may be NULL) supplies exp(-beta*dE) for the five
 * possible dE = float32(k) * J, k = -8, -4, 0, 4, 8 (index (k + 8) / 4).  The
 * reference evaluates this with CUDA's float32 expf (libdevice), which is not
 * always correctly rounded; a test can pass the values a GPU's expf produced
 * so that the lattices stay bit-exact.  NULL evaluates libm expf. */
static void ising_color_replica(int8_t *spins, uint64_t *rng, float beta, const float *tab, int r,
                                int L, int color, float J)
{
    const int8_t *base = spins + (int64_t)r * L * L;
    for (int i = color / 2; i < L; i += 2)
        for (int j = color % 2; j < L; j += 2) {
            int s = base[i * L + j];
            int up = base[wrap(i - 1, L) * L + j];
            int down = base[wrap(i + 1, L) * L + j];
            int left = base[i * L + wrap(j - 1, L)];
            int right = base[i * L + wrap(j + 1, L)];
            /* float32(2*s*sum) * J, then a float32 exp of -beta*dE. */
            int k = 2 * s * (up + down + left + right);
            float dE = (float)k * J;
            int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
            float u = orc_rng_uniform_f32(rng + 2 * idx);
            if (dE <= 0.0f || u < (tab ? tab[(k + 8) / 4] : expf(-beta * dE)))
                spins[(int64_t)r * L * L + i * L + j] = (int8_t)(-s);
        }
}

void orc_ising_update_color(int8_t *spins, uint64_t *rng, const float *betas, int R, int L,
                            int color, float J)
{
    for (int r = 0; r < R; ++r) ising_color_replica(spins, rng, betas[r], NULL, r, L, color, J);
}

void orc_ising_sweeps(int8_t *spins, uint64_t *rng, const float *betas, int R, int L,
                      float J, int n_sweeps, int n_threads)
{
    orc_ising_sweeps_tab(spins, rng, betas, NULL, R, L, J, n_sweeps, n_threads);
}

void orc_ising_sweeps_tab(int8_t *spins, uint64_t *rng, const float *betas, const float *tab,
                          int R, int L, float J, int n_sweeps, int n_threads)
{
    (void)n_threads;
    OMP_FOR_R
    for (int r = 0; r < R; ++r)
        for (int s = 0; s < n_sweeps; ++s)
            for (int c = 0; c < 4; ++c)
                ising_color_replica(spins, rng, betas[r], tab ? tab + 5 * r : NULL, r, L, c, J);
}

void orc_ising_energy(const int8_t *spins, int R, int L, float J, double *out)
{
    for (int r = 0; r < R; ++r) {
        const int8_t *b = spins + (int64_t)r * L * L;
        double e = 0.0;
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
                int s = b[i * L + j];
                int down = b[wrap(i + 1, L) * L + j];
                int right = b[i * L + wrap(j + 1, L)];
                e += -(double)J * s * (down + right);
            }
        out[r] = e;
    }
}

void orc_ising_measure(const int8_t *spins, int R, int L, float J,
                       const int32_t *tidx, const double *cached, double *out)
{
    for (int r = 0; r < R; ++r) {
        const int8_t *b = spins + (int64_t)r * L * L;
        double e = 0.0, m = 0.0;
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
                int s = b[i * L + j];
                if (!cached) {
                    int down = b[wrap(i + 1, L) * L + j];
                    int right = b[i * L + wrap(j + 1, L)];
                    e += -(double)J * s * (down + right);
                }
                m += s;
            }
        int d = tidx ? tidx[r] : r;
        out[0 * R + d] = cached ? cached[r] : e;
        out[1 * R + d] = m;
    }
}

/* ------------------------------------------------------------------------ */
/* XY: models/xy/update.py:6-54, models/xy/measure.py:17-134                */
/* The Gaussian-proposal variant is this project's extension (symmetric     */
/* proposal theta + sigma*z, Box-Muller z, full wrap); it reuses the       */
/* reference's acceptance rule.  Two draws per visit: the Box-Muller pair  */
/* u1, u2 are bits 63..41 and 40..18 of the first (23-bit uniforms), the   */
/* acceptance uniform is the float32 uniform of the second.                */
/* ------------------------------------------------------------------------ */

static const float PI_F = 3.14159265358979323846f;
static const float TWO_PI_F = 6.28318530717958647692f;

static inline float xy_bond_sum(const float *b, int L, int i, int j, float t)
{
    float up = b[wrap(i - 1, L) * L + j];
    float down = b[wrap(i + 1, L) * L + j];
    float left = b[i * L + wrap(j - 1, L)];
    float right = b[i * L + wrap(j + 1, L)];
    return ((cosf(t - up) + cosf(t - down)) + cosf(t - left)) + cosf(t - right);
}

static void xy_color_replica(float *theta, uint64_t *rng, float beta, int r, int L, int color,
                             float J, float delta, int gaussian, float sigma)
{
    float *b = theta + (int64_t)r * L * L;
    for (int i = color / 2; i < L; i += 2)
        for (int j = color % 2; j < L; j += 2) {
            float t = b[i * L + j];
            int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
            uint64_t *st = rng + 2 * idx;
            float proposed, v;
            if (!gaussian) {
                float u = orc_rng_uniform_f32(st);
                proposed = t + delta * (2.0f * u - 1.0f);
                if (proposed >= PI_F) proposed -= TWO_PI_F;
                else if (proposed < -PI_F) proposed += TWO_PI_F;
                v = orc_rng_uniform_f32(st);
            } else {
                /* one draw per visit: u1 = (2k+1) 2^-22 (bits 63..43), u2 = k 2^-21
                   (bits 42..22), acceptance v = k 2^-21 (bits 21..1) */
                uint64_t x = orc_rng_next(st);
                float u1 = (float)(2u * (uint32_t)(x >> 43) + 1u) * 0x1p-22f;
                float u2 = (float)((uint32_t)(x >> 22) & 0x1fffffu) * 0x1p-21f;
                v = (float)((uint32_t)(x >> 1) & 0x1fffffu) * 0x1p-21f;
                float z = sqrtf(-2.0f * logf(u1)) * cosf(TWO_PI_F * u2);
                proposed = t + sigma * z;
                proposed -= TWO_PI_F * floorf((proposed + PI_F) / TWO_PI_F);
                if (proposed >= PI_F) proposed -= TWO_PI_F;
                if (proposed < -PI_F) proposed += TWO_PI_F;
            }
            float e_old = -J * xy_bond_sum(b, L, i, j, t);
            float e_new = -J * xy_bond_sum(b, L, i, j, proposed);
            float dE = e_new - e_old;
            if (dE <= 0.0f || v < expf(-beta * dE)) b[i * L + j] = proposed;
        }
}

void orc_xy_update_color(float *theta, uint64_t *rng, const float *betas, int R, int L,
                         int color, float J, float delta)
{
    for (int r = 0; r < R; ++r) xy_color_replica(theta, rng, betas[r], r, L, color, J, delta, 0, 0.f);
}

void orc_xy_update_color_gauss(float *theta, uint64_t *rng, const float *betas,
                               const float *sigmas, int R, int L, int color, float J)
{
    for (int r = 0; r < R; ++r)
        xy_color_replica(theta, rng, betas[r], r, L, color, J, 0.f, 1, sigmas[r]);
}

void orc_xy_sweeps(float *theta, uint64_t *rng, const float *betas, const float *sigmas,
                   int R, int L, float J, float delta, int n_sweeps, int n_threads)
{
    (void)n_threads;
    OMP_FOR_R
    for (int r = 0; r < R; ++r)
        for (int s = 0; s < n_sweeps; ++s)
            for (int c = 0; c < 4; ++c)
                xy_color_replica(theta, rng, betas[r], r, L, c, J, delta, sigmas != NULL,
                                 sigmas ? sigmas[r] : 0.f);
}

void orc_xy_energy(const float *theta, int R, int L, float J, double *out)
{
    for (int r = 0; r < R; ++r) {
        const float *b = theta + (int64_t)r * L * L;
        double e = 0.0;
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
                double t = b[i * L + j];
                double tx = b[wrap(i + 1, L) * L + j];
                double ty = b[i * L + wrap(j + 1, L)];
                e += -(double)J * (cos(t - tx) + cos(t - ty));
            }
        out[r] = e;
    }
}

void orc_xy_measure(const float *theta, int R, int L, float J, const int32_t *tidx,
                    const double *cached, double *out)
{
    for (int r = 0; r < R; ++r) {
        const float *b = theta + (int64_t)r * L * L;
        double e = 0, mx = 0, my = 0, cx = 0, qx = 0;
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
                double t = b[i * L + j];
                double tx = b[wrap(i + 1, L) * L + j];
                double dx = t - tx;
                double cos_x = cos(dx);
                if (!cached) {
                    double ty = b[i * L + wrap(j + 1, L)];
                    e += -(double)J * (cos_x + cos(t - ty));
                }
                mx += cos(t);
                my += sin(t);
                cx += cos_x;
                qx += sin(dx);
            }
        int d = tidx ? tidx[r] : r;
        out[0 * R + d] = cached ? cached[r] : e;
        out[1 * R + d] = mx;
        out[2 * R + d] = my;
        out[3 * R + d] = cx;
        out[4 * R + d] = qx;
    }
}

/* ------------------------------------------------------------------------ */
/* Kawamura: models/kawamura/update.py:7-65, models/kawamura/measure.py     */
/* ------------------------------------------------------------------------ */

float orc_kawamura_local_energy(const float *state, int L, int r, int i, int j, float theta,
                                float tau, float dx, float dy, float dz, float J)
{
    const float *b = state + (int64_t)r * L * L * 5;
    int ni[4] = {wrap(i - 1, L), wrap(i + 1, L), i, i};
    int nj[4] = {j, j, wrap(j - 1, L), wrap(j + 1, L)};
    float energy = 0.0f;
    for (int k = 0; k < 4; ++k) {
        const float *n = b + ((int64_t)ni[k] * L + nj[k]) * 5;
        float dot = (dx * n[2] + dy * n[3]) + dz * n[4];
        energy -= ((J * (1.0f + tau * n[1])) * dot) * cosf(theta - n[0]);
    }
    return energy;
}

static void kawamura_color_replica(float *state, uint64_t *rng, float beta, int r, int L,
                                   int color, float J, float delta)
{
    for (int i = color / 2; i < L; i += 2)
        for (int j = color % 2; j < L; j += 2) {
            float *site = state + (((int64_t)r * L + i) * L + j) * 5;
            int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
            uint64_t *st = rng + 2 * idx;
            float theta = site[0], tau = site[1], dx = site[2], dy = site[3], dz = site[4];
            float energy = orc_kawamura_local_energy(state, L, r, i, j, theta, tau, dx, dy, dz, J);

            float pt = theta + delta * (2.0f * orc_rng_uniform_f32(st) - 1.0f);
            if (pt >= PI_F) pt -= TWO_PI_F;
            else if (pt < -PI_F) pt += TWO_PI_F;
            float pe = orc_kawamura_local_energy(state, L, r, i, j, pt, tau, dx, dy, dz, J);
            float dE = pe - energy;
            float u = orc_rng_uniform_f32(st);
            if (dE <= 0.0f || u < expf(-beta * dE)) {
                theta = pt;
                energy = pe;
            }

            float ptau = -tau;
            pe = orc_kawamura_local_energy(state, L, r, i, j, theta, ptau, dx, dy, dz, J);
            dE = pe - energy;
            u = orc_rng_uniform_f32(st);
            if (dE <= 0.0f || u < expf(-beta * dE)) {
                tau = ptau;
                energy = pe;
            }

            float z = 2.0f * orc_rng_uniform_f32(st) - 1.0f;
            float phi = TWO_PI_F * orc_rng_uniform_f32(st);
            float radius = sqrtf(1.0f - z * z);
            float x = radius * cosf(phi), y = radius * sinf(phi);
            pe = orc_kawamura_local_energy(state, L, r, i, j, theta, tau, x, y, z, J);
            dE = pe - energy;
            u = orc_rng_uniform_f32(st);
            if (dE <= 0.0f || u < expf(-beta * dE)) {
                dx = x;
                dy = y;
                dz = z;
            }
            site[0] = theta;
            site[1] = tau;
            site[2] = dx;
            site[3] = dy;
            site[4] = dz;
        }
}

/* Gaussian proposals (this project's extension; the three sub-moves and   */
/* their acceptance rule are the reference's): theta' = theta + sigma*z0,   */
/* wrapped; tau flipped; d' = (d + sigma*g)/|d + sigma*g| with g three      */
/* standard normals (symmetric: its density depends only on the angle       */
/* between d and d').  Five draws per visit: two Box-Muller pairs (z0, gx)  */
/* and (gy, gz), each from bits 63..41 and 40..18 of one draw, then the     */
/* three acceptance uniforms.                                               */
static void box_muller_pair(uint64_t x, float *z1, float *z2)
{
    float u1 = (float)(x >> 41) * 0x1p-23f;
    float u2 = (float)((x >> 18) & 0x7fffffu) * 0x1p-23f;
    if (u1 <= 0.0f) u1 = 1.1102230246251565e-16f;
    float rad = sqrtf(-2.0f * logf(u1));
    float ang = TWO_PI_F * u2;
    *z1 = rad * cosf(ang);
    *z2 = rad * sinf(ang);
}

static void kawamura_gauss_color_replica(float *state, uint64_t *rng, float beta, int r, int L,
                                         int color, float J, float sigma)
{
    for (int i = color / 2; i < L; i += 2)
        for (int j = color % 2; j < L; j += 2) {
            float *site = state + (((int64_t)r * L + i) * L + j) * 5;
            int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
            uint64_t *st = rng + 2 * idx;
            float theta = site[0], tau = site[1], dx = site[2], dy = site[3], dz = site[4];
            float z0, gx, gy, gz;
            box_muller_pair(orc_rng_next(st), &z0, &gx);
            box_muller_pair(orc_rng_next(st), &gy, &gz);
            float energy = orc_kawamura_local_energy(state, L, r, i, j, theta, tau, dx, dy, dz, J);

            float pt = theta + sigma * z0;
            pt -= TWO_PI_F * floorf((pt + PI_F) / TWO_PI_F);
            if (pt >= PI_F) pt -= TWO_PI_F;
            if (pt < -PI_F) pt += TWO_PI_F;
            float pe = orc_kawamura_local_energy(state, L, r, i, j, pt, tau, dx, dy, dz, J);
            float dE = pe - energy;
            float u = orc_rng_uniform_f32(st);
            if (dE <= 0.0f || u < expf(-beta * dE)) {
                theta = pt;
                energy = pe;
            }

            float ptau = -tau;
            pe = orc_kawamura_local_energy(state, L, r, i, j, theta, ptau, dx, dy, dz, J);
            dE = pe - energy;
            u = orc_rng_uniform_f32(st);
            if (dE <= 0.0f || u < expf(-beta * dE)) {
                tau = ptau;
                energy = pe;
            }

            float x = dx + sigma * gx, y = dy + sigma * gy, z = dz + sigma * gz;
            float inv = 1.0f / sqrtf((x * x + y * y) + z * z);
            x *= inv;
            y *= inv;
            z *= inv;
            pe = orc_kawamura_local_energy(state, L, r, i, j, theta, tau, x, y, z, J);
            dE = pe - energy;
            u = orc_rng_uniform_f32(st);
            if (dE <= 0.0f || u < expf(-beta * dE)) {
                dx = x;
                dy = y;
                dz = z;
            }
            site[0] = theta;
            site[1] = tau;
            site[2] = dx;
            site[3] = dy;
            site[4] = dz;
        }
}

void orc_kawamura_update_color_gauss(float *state, uint64_t *rng, const float *betas, const float *sigmas,
                                     int R, int L, int color, float J)
{
    for (int r = 0; r < R; ++r) kawamura_gauss_color_replica(state, rng, betas[r], r, L, color, J, sigmas[r]);
}

void orc_kawamura_sweeps_gauss(float *state, uint64_t *rng, const float *betas, const float *sigmas, int R,
                               int L, float J, int n_sweeps, int n_threads)
{
    (void)n_threads;
    OMP_FOR_R
    for (int r = 0; r < R; ++r)
        for (int s = 0; s < n_sweeps; ++s)
            for (int c = 0; c < 4; ++c) kawamura_gauss_color_replica(state, rng, betas[r], r, L, c, J, sigmas[r]);
}

void orc_kawamura_update_color(float *state, uint64_t *rng, const float *betas, int R, int L,
                               int color, float J, float delta)
{
    for (int r = 0; r < R; ++r) kawamura_color_replica(state, rng, betas[r], r, L, color, J, delta);
}

void orc_kawamura_sweeps(float *state, uint64_t *rng, const float *betas, int R, int L,
                         float J, float delta, int n_sweeps, int n_threads)
{
    (void)n_threads;
    OMP_FOR_R
    for (int r = 0; r < R; ++r)
        for (int s = 0; s < n_sweeps; ++s)
            for (int c = 0; c < 4; ++c) kawamura_color_replica(state, rng, betas[r], r, L, c, J, delta);
}

static double kawamura_bond64(const float *a, const float *n, double *weight_out, double *angle_out)
{
    double dot = (double)a[2] * n[2] + (double)a[3] * n[3] + (double)a[4] * n[4];
    double weight = (1.0 + (double)a[1] * n[1]) * dot;
    double angle = (double)a[0] - (double)n[0];
    if (weight_out) *weight_out = weight;
    if (angle_out) *angle_out = angle;
    return weight * cos(angle);
}

void orc_kawamura_energy(const float *state, int R, int L, float J, double *out)
{
    for (int r = 0; r < R; ++r) {
        const float *b = state + (int64_t)r * L * L * 5;
        double e = 0.0;
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
                const float *a = b + ((int64_t)i * L + j) * 5;
                e -= (double)J * kawamura_bond64(a, b + ((int64_t)wrap(i + 1, L) * L + j) * 5, 0, 0);
                e -= (double)J * kawamura_bond64(a, b + ((int64_t)i * L + wrap(j + 1, L)) * 5, 0, 0);
            }
        out[r] = e;
    }
}

void orc_kawamura_measure(const float *state, int R, int L, float J, const int32_t *tidx,
                          const double *cached, double *out)
{
    for (int r = 0; r < R; ++r) {
        const float *b = state + (int64_t)r * L * L * 5;
        double e = 0, chir = 0, px = 0, py = 0, cx = 0, qx = 0;
        double xx = 0, yy = 0, zz = 0, xy = 0, xz = 0, yz = 0;
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
                const float *a = b + ((int64_t)i * L + j) * 5;
                double th = a[0], dx = a[2], dy = a[3], dz = a[4];
                chir += a[1];
                px += cos(2 * th);
                py += sin(2 * th);
                xx += dx * dx - 1.0 / 3;
                yy += dy * dy - 1.0 / 3;
                zz += dz * dz - 1.0 / 3;
                xy += dx * dy;
                xz += dx * dz;
                yz += dy * dz;
                double w, ang;
                double cosine = kawamura_bond64(a, b + ((int64_t)wrap(i + 1, L) * L + j) * 5, &w, &ang);
                if (!cached) e -= (double)J * cosine;
                cx += cosine;
                qx += w * sin(ang);
                if (!cached)
                    e -= (double)J * kawamura_bond64(a, b + ((int64_t)i * L + wrap(j + 1, L)) * 5, 0, 0);
            }
        int d = tidx ? tidx[r] : r;
        out[0 * R + d] = cached ? cached[r] : e;
        out[1 * R + d] = chir;
        out[2 * R + d] = px;
        out[3 * R + d] = py;
        out[4 * R + d] = (xx * xx + yy * yy + zz * zz + 2 * (xy * xy + xz * xz + yz * yz)) / 3;
        out[5 * R + d] = cx;
        out[6 * R + d] = qx;
    }
}

/* ------------------------------------------------------------------------ */
/* He3 thin film: models/he3/update.py:9-227, models/he3/gaussian_fast.py,  */
/* models/he3/measure.py.  complex64 values are (re, im) float pairs; the  */
/* state is (R, L, L, 3, 2) complex64 = 12 floats per site.                */
/* ------------------------------------------------------------------------ */

typedef struct { float re, im; } c32;

static inline c32 cmk(float a, float b) { c32 z = {a, b}; return z; }
static inline c32 cadd(c32 a, c32 b) { return cmk(a.re + b.re, a.im + b.im); }
static inline c32 csub(c32 a, c32 b) { return cmk(a.re - b.re, a.im - b.im); }
static inline c32 cmul(c32 a, c32 b) { return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline c32 cconj(c32 a) { return cmk(a.re, -a.im); }
static inline c32 cscale(float s, c32 a) { return cmk(s * a.re, s * a.im); }
static inline c32 cneg(c32 a) { return cmk(-a.re, -a.im); }
static inline float norm2(c32 z) { return z.re * z.re + z.im * z.im; }

static inline c32 site_c(const float *state, int L, int r, int i, int j, int mu, int a)
{
    const float *p = state + ((((int64_t)r * L + i) * L + j) * 6 + mu * 2 + a) * 2;
    return cmk(p[0], p[1]);
}

/* models/he3/update.py:14-28 */
static float he3_dipole(const c32 *psi, float n)
{
    c32 a = psi[0], b = psi[1], c = psi[2], d = psi[3];
    return norm2(cadd(a, d)) + norm2(a) + norm2(d) + 2.0f * cmul(b, cconj(c)).re
           - (float)(2.0 / 3.0) * n;
}

/* models/he3/update.py:32-63 ; psi[mu*2 + a] */
static float he3_potential_c(const c32 *psi, const float *beta, float g_d)
{
    float nx = norm2(psi[0]), ny = norm2(psi[1]);
    c32 xx = cmul(psi[0], psi[0]), yy = cmul(psi[1], psi[1]);
    c32 xy = cmul(psi[0], psi[1]);
    c32 overlap = cmul(cconj(psi[0]), psi[1]);
    for (int mu = 1; mu < 3; ++mu) {
        c32 x = psi[2 * mu], y = psi[2 * mu + 1];
        nx += norm2(x);
        ny += norm2(y);
        xx = cadd(xx, cmul(x, x));
        yy = cadd(yy, cmul(y, y));
        xy = cadd(xy, cmul(x, y));
        overlap = cadd(overlap, cmul(cconj(x), y));
    }
    float n = nx + ny, two = 2.0f;
    float i1 = norm2(cadd(xx, yy));
    float i2 = n * n;
    float i3 = nx * nx + ny * ny + two * cmul(overlap, overlap).re;
    float i4 = nx * nx + ny * ny + two * norm2(overlap);
    float i5 = norm2(xx) + norm2(yy) + two * norm2(xy);
    float dip = he3_dipole(psi, n);
    return -two * n + beta[0] * i1 + beta[1] * i2 + beta[2] * i3 + beta[3] * i4 + beta[4] * i5
           + g_d * dip;
}

float orc_he3_potential(const float *psi_f, const float *coeff, float g_d)
{
    c32 psi[6];
    for (int k = 0; k < 6; ++k) psi[k] = cmk(psi_f[2 * k], psi_f[2 * k + 1]);
    return he3_potential_c(psi, coeff, g_d);
}

/* models/he3/update.py:66-72 */
static float he3_gradient(c32 dx_x, c32 dx_y, c32 dy_x, c32 dy_y)
{
    return 3.0f * (norm2(dx_x) + norm2(dy_y)) + norm2(dx_y) + norm2(dy_x)
           + 2.0f * cadd(cmul(cconj(dx_x), dy_y), cmul(cconj(dx_y), dy_x)).re;
}

/* models/he3/update.py:95-175 */
static float he3_gradient_difference_c(const float *state, int L, int r, int i, int j,
                                       const c32 *proposed)
{
    int ip = wrap(i + 1, L), im = wrap(i - 1, L), jp = wrap(j + 1, L), jm = wrap(j - 1, L);
    float delta_g = 0.0f;
    for (int mu = 0; mu < 3; ++mu) {
        c32 x = site_c(state, L, r, i, j, mu, 0), y = site_c(state, L, r, i, j, mu, 1);
        c32 ex = csub(proposed[2 * mu], x), ey = csub(proposed[2 * mu + 1], y);
        c32 rx = site_c(state, L, r, ip, j, mu, 0), ry = site_c(state, L, r, ip, j, mu, 1);
        c32 ux = site_c(state, L, r, i, jp, mu, 0), uy = site_c(state, L, r, i, jp, mu, 1);
        c32 lx = site_c(state, L, r, im, j, mu, 0), ly = site_c(state, L, r, im, j, mu, 1);
        c32 dx = site_c(state, L, r, i, jm, mu, 0), dy = site_c(state, L, r, i, jm, mu, 1);
        c32 lux = site_c(state, L, r, im, jp, mu, 0), luy = site_c(state, L, r, im, jp, mu, 1);
        c32 drx = site_c(state, L, r, ip, jm, mu, 0), dry = site_c(state, L, r, ip, jm, mu, 1);
        c32 a = csub(rx, x), b = csub(ry, y), c = csub(ux, x), d = csub(uy, y);
        c32 al = csub(x, lx), bl = csub(y, ly), cl = csub(lux, lx), dl = csub(luy, ly);
        c32 ad = csub(drx, dx), bd = csub(dry, dy), cd = csub(x, dx), dd = csub(y, dy);
        c32 fx = cadd(cadd(cneg(cadd(cadd(cadd(cscale(3.0f, a), b), c), d)),
                           cadd(cscale(3.0f, al), dl)),
                      cadd(cd, bd));
        c32 fy = cadd(cadd(cneg(cadd(cadd(cadd(a, b), c), cscale(3.0f, d))), cadd(bl, cl)),
                      cadd(cscale(3.0f, dd), ad));
        float linear = 2.0f * cadd(cmul(cconj(ex), fx), cmul(cconj(ey), fy)).re;
        float quadratic = 8.0f * (norm2(ex) + norm2(ey)) + 4.0f * cmul(cconj(ex), ey).re;
        delta_g += linear + quadratic;
    }
    return delta_g;
}

float orc_he3_gradient_difference(const float *state, int L, int r, int i, int j,
                                  const float *proposed_f)
{
    c32 p[6];
    for (int k = 0; k < 6; ++k) p[k] = cmk(proposed_f[2 * k], proposed_f[2 * k + 1]);
    return he3_gradient_difference_c(state, L, r, i, j, p);
}

static void he3_load(const float *state, int L, int r, int i, int j, c32 *psi)
{
    for (int mu = 0; mu < 3; ++mu)
        for (int a = 0; a < 2; ++a) psi[2 * mu + a] = site_c(state, L, r, i, j, mu, a);
}

static void he3_store(float *state, int L, int r, int i, int j, const c32 *psi)
{
    float *p = state + (((int64_t)r * L + i) * L + j) * 12;
    for (int k = 0; k < 6; ++k) {
        p[2 * k] = psi[k].re;
        p[2 * k + 1] = psi[k].im;
    }
}

/* models/he3/update.py:178-227 */
static void he3_color_replica(float *state, uint64_t *rng, float beta, int r, int L, int color,
                              const float *coeff, float K, float delta, float g_d)
{
    for (int i = color / 2; i < L; i += 2)
        for (int j = color % 2; j < L; j += 2) {
            uint64_t *st = rng + 2 * ((int64_t)r * L * L + (int64_t)i * L + j);
            c32 psi[6];
            he3_load(state, L, r, i, j, psi);
            float old_potential = he3_potential_c(psi, coeff, g_d);
            for (int k = 0; k < 6; ++k) {
                float re = delta * (2.0f * orc_rng_uniform_f32(st) - 1.0f);
                float im = delta * (2.0f * orc_rng_uniform_f32(st) - 1.0f);
                psi[k] = cmk(psi[k].re + re, psi[k].im + im);
            }
            float dv = he3_potential_c(psi, coeff, g_d) - old_potential;
            float dg = he3_gradient_difference_c(state, L, r, i, j, psi);
            float difference = dv + K * dg;
            float u = orc_rng_uniform_f32(st);
            if (difference <= 0.0f || u < expf(-beta * difference)) he3_store(state, L, r, i, j, psi);
        }
}

void orc_he3_update_color(float *state, uint64_t *rng, const float *betas, int R, int L,
                          int color, const float *coeff, float K, float delta, float g_d)
{
    for (int r = 0; r < R; ++r) he3_color_replica(state, rng, betas[r], r, L, color, coeff, K, delta, g_d);
}

/* models/he3/gaussian_fast.py:26-40 */
static void he3_neighbor_field(const float *state, int L, int r, int i, int j, c32 *field)
{
    int ip = wrap(i + 1, L), im = wrap(i - 1, L), jp = wrap(j + 1, L), jm = wrap(j - 1, L);
    for (int mu = 0; mu < 3; ++mu) {
        c32 rx = site_c(state, L, r, ip, j, mu, 0), ry = site_c(state, L, r, ip, j, mu, 1);
        c32 ux = site_c(state, L, r, i, jp, mu, 0), uy = site_c(state, L, r, i, jp, mu, 1);
        c32 lx = site_c(state, L, r, im, j, mu, 0), ly = site_c(state, L, r, im, j, mu, 1);
        c32 dx = site_c(state, L, r, i, jm, mu, 0), dy = site_c(state, L, r, i, jm, mu, 1);
        c32 lux = site_c(state, L, r, im, jp, mu, 0), luy = site_c(state, L, r, im, jp, mu, 1);
        c32 drx = site_c(state, L, r, ip, jm, mu, 0), dry = site_c(state, L, r, ip, jm, mu, 1);
        c32 f0 = cscale(-3.0f, cadd(rx, lx));
        f0 = csub(f0, ux); f0 = csub(f0, uy); f0 = csub(f0, ry); f0 = csub(f0, ly);
        f0 = csub(f0, dx); f0 = csub(f0, dy); f0 = cadd(f0, luy); f0 = cadd(f0, dry);
        c32 f1 = cneg(rx);
        f1 = csub(f1, ry); f1 = csub(f1, ux); f1 = csub(f1, lx); f1 = csub(f1, ly);
        f1 = csub(f1, dx); f1 = csub(f1, cscale(3.0f, cadd(uy, dy)));
        f1 = cadd(f1, lux); f1 = cadd(f1, drx);
        field[2 * mu] = f0;
        field[2 * mu + 1] = f1;
    }
}

/* models/he3/gaussian_fast.py:42-50 */
static c32 he3_normal_pair(uint64_t *st)
{
    float u = orc_rng_uniform_f32(st);
    if (u <= 0.0f) u = 1.1102230246251565e-16f;
    float angle = 6.283185307179586f * orc_rng_uniform_f32(st);
    float radius = sqrtf(-2.0f * logf(u));
    return cmk(radius * cosf(angle), radius * sinf(angle));
}

/* models/he3/gaussian_fast.py:53-88 */
static float he3_gaussian_proposal(c32 *psi, const c32 *field, float beta, float K, float rho,
                                   float mass, uint64_t *st)
{
    const float one = 1.0f, two = 2.0f, root = 0.7071067811865475f;
    float plus = 10.0f * K + mass, minus = 6.0f * K + mass;
    float vf = one - rho * rho;
    float sp = sqrtf(vf / (two * beta * plus));
    float sm = sqrtf(vf / (two * beta * minus));
    float qp = vf / (8.0f * root * root * sp * sp);
    float qm = vf / (8.0f * root * root * sm * sm);
    float log_ratio = 0.0f;
    for (int mu = 0; mu < 3; ++mu) {
        c32 x = psi[2 * mu], y = psi[2 * mu + 1];
        c32 hp = cscale(root, cadd(field[2 * mu], field[2 * mu + 1]));
        c32 hm = cscale(root, csub(field[2 * mu], field[2 * mu + 1]));
        c32 mp = cscale(-K, hp), mm = cscale(-K, hm);
        mp = cmk(mp.re / plus, mp.im / plus);
        mm = cmk(mm.re / minus, mm.im / minus);
        c32 mx = cscale(root, cadd(mp, mm)), my = cscale(root, csub(mp, mm));
        c32 zp = cscale(sp, he3_normal_pair(st));
        c32 zm = cscale(sm, he3_normal_pair(st));
        c32 nx = cadd(cadd(mx, cscale(rho, csub(x, mx))), cscale(root, cadd(zp, zm)));
        c32 ny = cadd(cadd(my, cscale(rho, csub(y, my))), cscale(root, csub(zp, zm)));
        psi[2 * mu] = nx;
        psi[2 * mu + 1] = ny;
        c32 old_plus = cadd(csub(x, mx), csub(y, my)), old_minus = csub(csub(x, mx), csub(y, my));
        c32 new_plus = cadd(csub(nx, mx), csub(ny, my)), new_minus = csub(csub(nx, mx), csub(ny, my));
        log_ratio += qp * (norm2(new_plus) - norm2(old_plus));
        log_ratio += qm * (norm2(new_minus) - norm2(old_minus));
    }
    return log_ratio;
}

/* models/he3/gaussian_fast.py:91-119 ; counts is (3, R, L, L) int64 */
static void he3_gauss_color_replica(float *state, uint64_t *rng, float beta, int R, int r, int L,
                                    int color, const float *coeff, float K, float rho, float mass,
                                    float g_d, int64_t *counts)
{
    int64_t plane = (int64_t)R * L * L;
    for (int i = color / 2; i < L; i += 2)
        for (int j = color % 2; j < L; j += 2) {
            int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
            uint64_t *st = rng + 2 * idx;
            c32 field[6], psi[6];
            he3_neighbor_field(state, L, r, i, j, field);
            he3_load(state, L, r, i, j, psi);
            float old_potential = he3_potential_c(psi, coeff, g_d);
            float lpr = he3_gaussian_proposal(psi, field, beta, K, rho, mass, st);
            float delta_h = he3_potential_c(psi, coeff, g_d) - old_potential
                            + K * he3_gradient_difference_c(state, L, r, i, j, psi);
            float log_ratio = -beta * delta_h + lpr;
            float u = orc_rng_uniform_f32(st);
            counts[idx] += 1;
            if (!isfinite(log_ratio)) {
                counts[2 * plane + idx] += 1;
            } else if (log_ratio >= 0.0f || u < expf(log_ratio)) {
                counts[plane + idx] += 1;
                he3_store(state, L, r, i, j, psi);
            }
        }
}

void orc_he3_gaussian_update_color(float *state, uint64_t *rng, const float *betas, int R, int L,
                                   int color, const float *coeff, float K, float rho, float mass,
                                   float g_d, int64_t *counts)
{
    for (int r = 0; r < R; ++r)
        he3_gauss_color_replica(state, rng, betas[r], R, r, L, color, coeff, K, rho, mass, g_d, counts);
}

void orc_he3_sweeps(float *state, uint64_t *rng, const float *betas, int R, int L,
                    const float *coeff, float K, float delta, float g_d, int gaussian, float rho,
                    float mass, int64_t *counts, int n_sweeps, int n_threads)
{
    (void)n_threads;
    OMP_FOR_R
    for (int r = 0; r < R; ++r)
        for (int s = 0; s < n_sweeps; ++s)
            for (int c = 0; c < 4; ++c) {
                if (gaussian)
                    he3_gauss_color_replica(state, rng, betas[r], R, r, L, c, coeff, K, rho, mass, g_d,
                                            counts);
                else
                    he3_color_replica(state, rng, betas[r], r, L, c, coeff, K, delta, g_d);
            }
}

/* models/he3/measure.py:115-143 */
void orc_he3_energy(const float *state, int R, int L, const float *coeff, float K, float g_d,
                    double *out)
{
    for (int r = 0; r < R; ++r) {
        double energy = 0.0;
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
                c32 psi[6];
                he3_load(state, L, r, i, j, psi);
                energy += he3_potential_c(psi, coeff, g_d);
                for (int mu = 0; mu < 3; ++mu) {
                    c32 a = csub(site_c(state, L, r, wrap(i + 1, L), j, mu, 0), psi[2 * mu]);
                    c32 b = csub(site_c(state, L, r, wrap(i + 1, L), j, mu, 1), psi[2 * mu + 1]);
                    c32 c = csub(site_c(state, L, r, i, wrap(j + 1, L), mu, 0), psi[2 * mu]);
                    c32 d = csub(site_c(state, L, r, i, wrap(j + 1, L), mu, 1), psi[2 * mu + 1]);
                    energy += K * he3_gradient(a, b, c, d);
                }
            }
        out[r] = energy;
    }
}

/* models/he3/measure.py:22-89 ; 10 channels */
void orc_he3_measure(const float *state, int R, int L, const float *coeff, float K, float g_d,
                     const int32_t *tidx, const double *cached, double *out)
{
    for (int r = 0; r < R; ++r) {
        double energy = 0, density = 0, chirality = 0, pr = 0, pim = 0;
        double ix = 0, kx = 0, iy = 0, ky = 0, szd = 0;
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
                c32 psi[6];
                he3_load(state, L, r, i, j, psi);
                if (!cached) energy += he3_potential_c(psi, coeff, g_d);
                for (int mu = 0; mu < 3; ++mu) {
                    c32 x = psi[2 * mu], y = psi[2 * mu + 1];
                    c32 xpx = site_c(state, L, r, wrap(i + 1, L), j, mu, 0);
                    c32 xpy = site_c(state, L, r, wrap(i + 1, L), j, mu, 1);
                    c32 ypx = site_c(state, L, r, i, wrap(j + 1, L), mu, 0);
                    c32 ypy = site_c(state, L, r, i, wrap(j + 1, L), mu, 1);
                    c32 a = csub(xpx, x), b = csub(xpy, y), c = csub(ypx, x), d = csub(ypy, y);
                    if (!cached) energy += K * he3_gradient(a, b, c, d);
                    float rd = norm2(x) + norm2(y);
                    density += rd;
                    if (mu == 2) szd += rd;
                    chirality += 2.0 * (double)cmul(cconj(x), y).im;
                    c32 ph = csub(cmul(x, x), cmul(y, y));
                    pr += ph.re;
                    pim += ph.im;
                    /* Twist derivatives: models/he3/measure.py:54-60 (complex128 in Numba,
                     * since int64 * complex64 promotes). */
                    double ar = a.re, ai = -a.im, br = b.re, bi = -b.im;
                    double cr = c.re, ci = -c.im, dr = d.re, di = -d.im;
                    double zx_r = (3 * ar + dr) * xpx.re - (3 * ai + di) * xpx.im
                                  + (br + cr) * xpy.re - (bi + ci) * xpy.im;
                    double zx_i = (3 * ar + dr) * xpx.im + (3 * ai + di) * xpx.re
                                  + (br + cr) * xpy.im + (bi + ci) * xpy.re;
                    double zy_r = (cr + br) * ypx.re - (ci + bi) * ypx.im
                                  + (3 * dr + ar) * ypy.re - (3 * di + ai) * ypy.im;
                    double zy_i = (cr + br) * ypx.im + (ci + bi) * ypx.re
                                  + (3 * dr + ar) * ypy.im + (3 * di + ai) * ypy.re;
                    double K2 = 2.0 * (double)K;
                    ix += K2 * zx_i;
                    kx += K2 * (3.0 * norm2(xpx) + (double)norm2(xpy) - zx_r);
                    iy += K2 * zy_i;
                    ky += K2 * ((double)norm2(ypx) + 3.0 * norm2(ypy) - zy_r);
                }
            }
        int dst = tidx ? tidx[r] : r;
        out[0 * R + dst] = cached ? cached[r] : energy;
        out[1 * R + dst] = density;
        out[2 * R + dst] = chirality;
        out[3 * R + dst] = pr;
        out[4 * R + dst] = pim;
        out[5 * R + dst] = ix;
        out[6 * R + dst] = kx;
        out[7 * R + dst] = iy;
        out[8 * R + dst] = ky;
        out[9 * R + dst] = density == 0.0 ? 0.0 : 0.5 * (3 * szd / density - 1);
    }
}

/* ------------------------------------------------------------------------ */
/* Parallel tempering: core/parallel_tempering.py:35-91                     */
/* Pairs at one parity are disjoint, so a sequential loop equals the GPU's  */
/* concurrent threads.  swap_counts is (3, R-1), trips is (5, R).           */
/* ------------------------------------------------------------------------ */

void orc_pt_exchange(const double *energies, float *betas, int32_t *w2t, int32_t *t2w,
                     uint64_t *rng, int64_t *swap_counts, int64_t *trips, int R, int parity,
                     int64_t sweep)
{
    int64_t *attempts = swap_counts, *accepted = swap_counts + (R - 1),
            *nonfinite = swap_counts + 2 * (R - 1);
    for (int left = parity; left < R - 1; left += 2) {
        int right = left + 1;
        int a = t2w[left], b = t2w[right];
        double ea = energies[a], eb = energies[b];
        attempts[left] += 1;
        if (!isfinite(ea) || !isfinite(eb)) {
            nonfinite[left] += 1;
            continue;
        }
        double log_ratio = ((double)betas[a] - (double)betas[b]) * (ea - eb);
        double u = orc_rng_uniform_f64(rng + 2 * left);
        if (log_ratio >= 0.0 || u == 0.0 || log(u) < log_ratio) {
            t2w[left] = b;
            t2w[right] = a;
            w2t[a] = right;
            w2t[b] = left;
            float tmp = betas[a];
            betas[a] = betas[b];
            betas[b] = tmp;
            accepted[left] += 1;
        }
    }
    int64_t *origin = trips, *visited = trips + R, *start = trips + 2 * R, *nrt = trips + 3 * R,
            *rts = trips + 4 * R;
    for (int w = 0; w < R; ++w) {
        int t = w2t[w];
        if (t != 0 && t != R - 1) continue;
        if (origin[w] < 0) {
            origin[w] = t;
            start[w] = sweep;
        } else if (t != origin[w]) {
            visited[w] = 1;
        } else if (visited[w]) {
            nrt[w] += 1;
            rts[w] += sweep - start[w];
            start[w] = sweep;
            visited[w] = 0;
        }
    }
}
