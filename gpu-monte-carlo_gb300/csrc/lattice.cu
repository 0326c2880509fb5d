// Per-colour Metropolis updates and per-replica reductions for the Ising, XY
// and Kawamura models, on the reference's own layouts.  These are the kernels
// behind the drop-in Model plugin interface (core/model.py:16-62): one launch
// per checkerboard colour, any number of replicas per launch.
//
// Colour c visits sites i = 2*row + c/2, j = 2*col + c%2 (e.g.
// models/ising/update.py:12-13); one thread per visited site, consecutive
// threads on consecutive columns.  Site (r, i, j) draws from RNG stream
// r*L*L + i*L + j, every draw is taken whether or not the move is accepted,
// and each acceptance test is `dE <= 0 or u < expf(-beta*dE)` in float32, as
// in the reference kernels.  Reductions accumulate in float64 with one
// thread-block cluster per replica (warp shuffles, a pass over warp sums,
// then the CTAs' sums in rank order through distributed shared memory).
#include "ffmath.h"
#include "mcgb_common.cuh"

namespace mcgb {

constexpr int kReduceThreads = 256;

inline unsigned grid_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

inline int check_lattice(const char *who, int R, int L)
{
    MCGB_REQUIRE(R >= 1, "%s: R must be >= 1", who);
    MCGB_REQUIRE(L >= 4 && L % 2 == 0, "%s: L must be even and >= 4", who);
    MCGB_REQUIRE((int64_t)R * L * L < (1ll << 40), "%s: lattice too large", who);
    MCGB_REQUIRE(R <= 32767, "%s: at most 32767 replicas (one grid layer per replica and colour)", who);
    return MCGB_OK;
}

// ============================================================== Ising
// models/ising/update.py:7-29

__global__ void ising_phase_kernel(int8_t *__restrict__ spins, ulonglong2 *__restrict__ rng,
                                   const float *__restrict__ betas, int R, int L, int c0, int ncol,
                                   float J)
{
    int r, i, j;
    if (!colour_grid_site(R, L, c0, r, i, j)) return;
    const int8_t *b = spins + (int64_t)r * L * L;
    const int s = b[i * L + j];
    const int up = b[wrapi(i - 1, L) * L + j];
    const int down = b[wrapi(i + 1, L) * L + j];
    const int left = b[i * L + wrapi(j - 1, L)];
    const int right = b[i * L + wrapi(j + 1, L)];
    const float dE = (float)(2 * s * (up + down + left + right)) * J;
    const int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
    ulonglong2 st = rng[idx];
    const float u = xoro_uniform_f32(st);
    rng[idx] = st;
    if (dE <= 0.0f || u < expf(-betas[r] * dE)) spins[idx] = (int8_t)(-s);
}

// models/ising/measure.py:10-99.  mode bit 0: energy channel, bit 1: magnetization.
__global__ void ising_reduce_kernel(const int8_t *__restrict__ spins, int R, int L, float J,
                                    const int32_t *__restrict__ tidx, const double *__restrict__ cached,
                                    double *__restrict__ out, int energy_only)
{
    __shared__ double scratch[2 * 32], part[2];
    const ReplicaSpan sp = replica_span();
    const int r = sp.r;
    const int8_t *b = spins + (int64_t)r * L * L;
    // Integer partial sums are exact; J is applied once at the end, which
    // equals the reference's per-bond float64 products for |sum| < 2^53.
    long long e = 0, m = 0;
    const bool need_e = cached == nullptr;
    for (int k = sp.first; k < L * L; k += sp.step) {
        int i = k / L, j = k - i * L;
        int s = b[k];
        if (need_e) e += s * (b[wrapi(i + 1, L) * L + j] + b[i * L + wrapi(j + 1, L)]);
        m += s;
    }
    double v[2] = {(double)e, (double)m};
    cluster_sum<2>(v, scratch, part);
    if (sp.rank == 0 && threadIdx.x == 0) {
        double energy = need_e ? -(double)J * v[0] : cached[r];
        if (energy_only) {
            out[r] = energy;
        } else {
            int d = tidx ? tidx[r] : r;
            out[d] = energy;
            out[R + d] = v[1];
        }
    }
}

// ============================================================== XY
// models/xy/update.py:6-54 (uniform proposal) and the Gaussian variant.

__device__ __forceinline__ float xy_bond_sum(const float *b, int L, int i, int j, float t)
{
    const float up = b[wrapi(i - 1, L) * L + j];
    const float down = b[wrapi(i + 1, L) * L + j];
    const float left = b[i * L + wrapi(j - 1, L)];
    const float right = b[i * L + wrapi(j + 1, L)];
    return ((cosf(t - up) + cosf(t - down)) + cosf(t - left)) + cosf(t - right);
}

// Colour `color` (ncol = 1) or colours `color` and `color` + 1 (ncol = 2:
// colours 1 and 2 share no bond, so one launch of both equals two).
template <bool kGauss>
__global__ void xy_color_kernel(float *__restrict__ theta, ulonglong2 *__restrict__ rng,
                                const float *__restrict__ betas, const float *__restrict__ sigmas,
                                int R, int L, int color, int ncol, float J, float delta)
{
    const float pi = 3.14159265358979323846f, two_pi = 6.28318530717958647692f;
    int r, i, j;
    if (!colour_grid_site(R, L, color, r, i, j)) return;
    float *b = theta + (int64_t)r * L * L;
    const float th = b[i * L + j];
    const int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
    ulonglong2 st = rng[idx];
    float proposed, v;
    if (!kGauss) {
        // The reference's rule, shared with the reference-layout window.
        proposed = xy_ref_propose(th, st, delta, v);
        const int up = wrapi(i - 1, L) * L + j, down = wrapi(i + 1, L) * L + j;
        const int left = i * L + wrapi(j - 1, L), right = i * L + wrapi(j + 1, L);
        float dE;
        const bool acc = xy_ref_accept(th, proposed, v, b[up], b[down], b[left], b[right], betas[r], J, dE);
        rng[idx] = st;
        if (acc) b[i * L + j] = proposed;
        return;
    } else {
        // One draw per visit: u1, u2 and the acceptance v (mcgb_visit_*).
        const uint64_t x = xoro_next(st);
        const float u1 = mcgb_visit_u1(x), u2 = mcgb_visit_u2(x);
        v = mcgb_visit_v(x);
        const float z = sqrtf(-2.0f * logf(u1)) * cosf(two_pi * u2);
        proposed = th + sigmas[r] * z;
        proposed -= two_pi * floorf((proposed + pi) / two_pi);
        if (proposed >= pi) proposed -= two_pi;
        if (proposed < -pi) proposed += two_pi;
    }
    const float e_old = -J * xy_bond_sum(b, L, i, j, th);
    const float e_new = -J * xy_bond_sum(b, L, i, j, proposed);
    const float dE = e_new - e_old;
    rng[idx] = st;
    if (dE <= 0.0f || v < expf(-betas[r] * dE)) b[i * L + j] = proposed;
}

// Plain FP64 form: one replica per launch, float64 everywhere.
__global__ void xy64_color_kernel(double *__restrict__ theta, ulonglong2 *__restrict__ rng,
                                  const double *__restrict__ betas, const double *__restrict__ sigmas,
                                  const int32_t *__restrict__ w2t, int L, int r, int color, double J,
                                  double delta)
{
    const double pi = 3.14159265358979323846, two_pi = 6.28318530717958647692;
    int rr, i, j;
    if (!colour_grid_site(1, L, color, rr, i, j)) return;
    double *b = theta + (int64_t)r * L * L;
    const double th = b[i * L + j];
    const int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
    ulonglong2 st = rng[idx];
    const int slot = w2t != nullptr ? w2t[r] : r;
    double proposed;
    if (sigmas == nullptr) {
        proposed = th + delta * (2.0 * xoro_uniform_f64(st) - 1.0);
        if (proposed >= pi) proposed -= two_pi;
        else if (proposed < -pi) proposed += two_pi;
    } else {
        double u1 = xoro_uniform_f64(st);
        const double u2 = xoro_uniform_f64(st);
        if (u1 <= 0.0) u1 = 1.1102230246251565e-16;
        proposed = th + sigmas[slot] * (sqrt(-2.0 * log(u1)) * cos(two_pi * u2));
        proposed -= two_pi * floor((proposed + pi) / two_pi);
    }
    const double up = b[wrapi(i - 1, L) * L + j], down = b[wrapi(i + 1, L) * L + j];
    const double left = b[i * L + wrapi(j - 1, L)], right = b[i * L + wrapi(j + 1, L)];
    const double e_old = -J * (cos(th - up) + cos(th - down) + cos(th - left) + cos(th - right));
    const double e_new = -J * (cos(proposed - up) + cos(proposed - down) + cos(proposed - left) +
                               cos(proposed - right));
    const double dE = e_new - e_old;
    const double v = xoro_uniform_f64(st);
    rng[idx] = st;
    if (dE <= 0.0 || v < exp(-betas[slot] * dE)) b[i * L + j] = proposed;
}

// models/xy/measure.py:17-134.  NC = 1: energy only; NC = 5: all channels.
// The reference evaluates cos and sin of every bond angle and spin angle in
// float64.  GB300's float64 pipe issues a small fraction of the float32
// rate, so the terms come from float-float arithmetic on the float32 pipe
// (ff_sincos of the exact float-float difference of two float angles, error
// below 1e-14) and accumulate per thread as float-float; only the per-thread
// totals enter the float64 cluster reduction.  The result differs from a
// float64 evaluation by about 1e-14 per term.
template <int NC>
__global__ void xy_reduce_kernel(const float *__restrict__ theta, int R, int L, float J,
                                 const int32_t *__restrict__ tidx, const double *__restrict__ cached,
                                 double *__restrict__ out)
{
    __shared__ double scratch[NC * 32], part[NC];
    const ReplicaSpan sp = replica_span();
    const int r = sp.r;
    const float *b = theta + (int64_t)r * L * L;
    ff acc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] = ff_make(0.0f, 0.0f);
    const bool need_e = cached == nullptr;
    for (int k = sp.first; k < L * L; k += sp.step) {
        const int i = k / L, j = k - i * L;
        const float t = b[k];
        ff sin_x, cos_x;
        ff_sincos(ff_diff(t, b[wrapi(i + 1, L) * L + j]), &sin_x, &cos_x);
        if (need_e) {
            ff sin_y, cos_y;
            ff_sincos(ff_diff(t, b[i * L + wrapi(j + 1, L)]), &sin_y, &cos_y);
            acc[0] = ff_add(acc[0], ff_add(cos_x, cos_y));
        }
        if (NC == 5) {
            ff sn, cs;
            ff_sincos(ff_make(t, 0.0f), &sn, &cs);
            acc[NC == 5 ? 1 : 0] = ff_add(acc[NC == 5 ? 1 : 0], cs);
            acc[NC == 5 ? 2 : 0] = ff_add(acc[NC == 5 ? 2 : 0], sn);
            acc[NC == 5 ? 3 : 0] = ff_add(acc[NC == 5 ? 3 : 0], cos_x);
            acc[NC == 5 ? 4 : 0] = ff_add(acc[NC == 5 ? 4 : 0], sin_x);
        }
    }
    double v[NC];
    v[0] = -(double)J * ff_to_double(acc[0]);
#pragma unroll
    for (int c = 1; c < NC; ++c) v[c] = ff_to_double(acc[c]);
    cluster_sum<NC>(v, scratch, part);
    if (sp.rank == 0 && threadIdx.x == 0) {
        const int d = tidx ? tidx[r] : r;
        out[d] = need_e ? v[0] : cached[r];
#pragma unroll
        for (int c = 1; c < NC; ++c) out[c * R + d] = v[c];
    }
}

__global__ void xy64_energy_kernel(const double *__restrict__ theta, int L, int r, double J,
                                   double *__restrict__ out)
{
    __shared__ double scratch[32];
    const double *b = theta + (int64_t)r * L * L;
    double v[1] = {0.0};
    for (int k = threadIdx.x; k < L * L; k += blockDim.x) {
        const int i = k / L, j = k - i * L;
        const double t = b[k];
        v[0] += -J * (cos(t - b[wrapi(i + 1, L) * L + j]) + cos(t - b[i * L + wrapi(j + 1, L)]));
    }
    block_sum<1>(v, scratch);
    if (threadIdx.x == 0) out[r] = v[0];
}

// The five channels of models/xy/measure.py:17-134 (energy, mx, my,
// twist_cos_x, twist_sin_x) of lattice r of the plain float64 form, into
// column w2t[r] (or r) of out (5, n_out).
__global__ void xy64_measure_kernel(const double *__restrict__ theta, int L, int r, double J,
                                    const int32_t *__restrict__ w2t, double *__restrict__ out, int n_out)
{
    __shared__ double scratch[32 * 5];
    const double *b = theta + (int64_t)r * L * L;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < L * L; k += blockDim.x) {
        const int i = k / L, j = k - i * L;
        const double t = b[k];
        const double dx = t - b[wrapi(i + 1, L) * L + j];
        const double cx = cos(dx);
        v[0] += -J * (cx + cos(t - b[i * L + wrapi(j + 1, L)]));
        v[1] += cos(t);
        v[2] += sin(t);
        v[3] += cx;
        v[4] += sin(dx);
    }
    block_sum<5>(v, scratch);
    if (threadIdx.x == 0) {
        const int col = w2t != nullptr ? w2t[r] : r;
        for (int c = 0; c < 5; ++c) out[(int64_t)c * n_out + col] = v[c];
    }
}

// ============================================================== Kawamura
// models/kawamura/update.py:7-65

__device__ __forceinline__ float kaw_local_energy(const float *b, int L, int i, int j, float theta,
                                                  float tau, float dx, float dy, float dz, float J)
{
    const int ni[4] = {wrapi(i - 1, L), wrapi(i + 1, L), i, i};
    const int nj[4] = {j, j, wrapi(j - 1, L), wrapi(j + 1, L)};
    float energy = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float *n = b + ((int64_t)ni[k] * L + nj[k]) * 5;
        const float dot = (dx * n[2] + dy * n[3]) + dz * n[4];
        energy -= ((J * (1.0f + tau * n[1])) * dot) * cosf(theta - n[0]);
    }
    return energy;
}

// Colour `color`, or colours `color` and `color` + 1 with ncol = 2 (as xy_color_kernel).
__global__ void kawamura_color_kernel(float *__restrict__ state, ulonglong2 *__restrict__ rng,
                                      const float *__restrict__ betas, int R, int L, int color, int ncol,
                                      float J, float delta)
{
    const float pi = 3.14159265358979323846f, two_pi = 6.28318530717958647692f;
    int r, i, j;
    if (!colour_grid_site(R, L, color, r, i, j)) return;
    const float *b = state + (int64_t)r * L * L * 5;
    float *site = state + (((int64_t)r * L + i) * L + j) * 5;
    const int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
    const float beta = betas[r];
    ulonglong2 st = rng[idx];
    float theta = site[0], tau = site[1], dx = site[2], dy = site[3], dz = site[4];
    float energy = kaw_local_energy(b, L, i, j, theta, tau, dx, dy, dz, J);

    float pt = theta + delta * (2.0f * xoro_uniform_f32(st) - 1.0f);
    if (pt >= pi) pt -= two_pi;
    else if (pt < -pi) pt += two_pi;
    float pe = kaw_local_energy(b, L, i, j, pt, tau, dx, dy, dz, J);
    float dE = pe - energy;
    float u = xoro_uniform_f32(st);
    if (dE <= 0.0f || u < expf(-beta * dE)) {
        theta = pt;
        energy = pe;
    }
    const float ptau = -tau;
    pe = kaw_local_energy(b, L, i, j, theta, ptau, dx, dy, dz, J);
    dE = pe - energy;
    u = xoro_uniform_f32(st);
    if (dE <= 0.0f || u < expf(-beta * dE)) {
        tau = ptau;
        energy = pe;
    }
    const float z = 2.0f * xoro_uniform_f32(st) - 1.0f;
    const float phi = two_pi * xoro_uniform_f32(st);
    const float radius = sqrtf(1.0f - z * z);
    const float x = radius * cosf(phi), y = radius * sinf(phi);
    pe = kaw_local_energy(b, L, i, j, theta, tau, x, y, z, J);
    dE = pe - energy;
    u = xoro_uniform_f32(st);
    if (dE <= 0.0f || u < expf(-beta * dE)) {
        dx = x;
        dy = y;
        dz = z;
    }
    rng[idx] = st;
    site[0] = theta;
    site[1] = tau;
    site[2] = dx;
    site[3] = dy;
    site[4] = dz;
}

__global__ void kawamura_local_kernel(const float *__restrict__ state, int L,
                                      const int32_t *__restrict__ pos, const float *__restrict__ prop,
                                      int n, float J, float *__restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int r = pos[3 * k], i = pos[3 * k + 1], j = pos[3 * k + 2];
    const float *b = state + (int64_t)r * L * L * 5;
    const float *s = b + ((int64_t)i * L + j) * 5;
    const float *p = prop + 5 * k;
    out[k] = kaw_local_energy(b, L, i, j, s[0], s[1], s[2], s[3], s[4], J);
    out[n + k] = kaw_local_energy(b, L, i, j, p[0], p[1], p[2], p[3], p[4], J);
}

// One bond of models/kawamura/measure.py:29-42 as float-float:
// weight = (1 + tau tau_n) (d . d_n) and cos, sin of theta - theta_n (the
// reference's float64 terms, to about 1e-14; GB300's float64 pipe issues at
// a small fraction of the float32 rate).  Returns weight * cos.
__device__ __forceinline__ ff kaw_bond_ff(const float *a, const float *n, ff &weight, ff &sin_term)
{
    const ff dot = ff_add(ff_add(ff_two_prod(a[2], n[2]), ff_two_prod(a[3], n[3])), ff_two_prod(a[4], n[4]));
    weight = ff_mul(dot, ff_add_f(ff_two_prod(a[1], n[1]), 1.0f));
    ff sn, cs;
    ff_sincos(ff_diff(a[0], n[0]), &sn, &cs);
    sin_term = ff_mul(weight, sn);
    return ff_mul(weight, cs);
}

// models/kawamura/measure.py:14-122.  NC = 1 energy only; NC = 12 sums for
// the 7 output channels (spin2 is formed from 6 tensor sums at the end).
// Every per-site term is evaluated and accumulated per thread as
// float-float on the float32 pipe (within about 1e-14 of the reference's
// float64 terms); only the per-thread totals enter the float64 reduction.
template <int NC>
__global__ void kawamura_reduce_kernel(const float *__restrict__ state, int R, int L, float J,
                                       const int32_t *__restrict__ tidx,
                                       const double *__restrict__ cached, double *__restrict__ out)
{
    __shared__ double scratch[NC * 32], part[NC];
    const ReplicaSpan sp = replica_span();
    const int r = sp.r;
    const float *b = state + (int64_t)r * L * L * 5;
    const ff third = ff_make(0x1.555556p-2f, -0x1.555556p-27f);  // 1/3
    ff acc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] = ff_make(0.0f, 0.0f);
    const bool need_e = cached == nullptr;
    for (int k = sp.first; k < L * L; k += sp.step) {
        const int i = k / L, j = k - i * L;
        const float *a = b + (int64_t)k * 5;
        ff w, sin_x;
        const ff cos_x = kaw_bond_ff(a, b + ((int64_t)wrapi(i + 1, L) * L + j) * 5, w, sin_x);
        if (need_e) {
            ff w2, s2;
            const ff cos_y = kaw_bond_ff(a, b + ((int64_t)i * L + wrapi(j + 1, L)) * 5, w2, s2);
            acc[0] = ff_add(acc[0], ff_add(cos_x, cos_y));
        }
        if (NC == 12) {
            constexpr int q = NC == 12 ? 1 : 0;  // channel offsets valid for NC == 12 only
            const float dx = a[2], dy = a[3], dz = a[4];
            ff s2t, c2t;
            ff_sincos(ff_make(2.0f * a[0], 0.0f), &s2t, &c2t);  // 2 theta is exact
            acc[q * 1] = ff_add_f(acc[q * 1], a[1]);
            acc[q * 2] = ff_add(acc[q * 2], c2t);
            acc[q * 3] = ff_add(acc[q * 3], s2t);
            acc[q * 4] = ff_add(acc[q * 4], ff_add(ff_two_prod(dx, dx), ff_neg(third)));
            acc[q * 5] = ff_add(acc[q * 5], ff_add(ff_two_prod(dy, dy), ff_neg(third)));
            acc[q * 6] = ff_add(acc[q * 6], ff_add(ff_two_prod(dz, dz), ff_neg(third)));
            acc[q * 7] = ff_add(acc[q * 7], ff_two_prod(dx, dy));
            acc[q * 8] = ff_add(acc[q * 8], ff_two_prod(dx, dz));
            acc[q * 9] = ff_add(acc[q * 9], ff_two_prod(dy, dz));
            acc[q * 10] = ff_add(acc[q * 10], cos_x);
            acc[q * 11] = ff_add(acc[q * 11], sin_x);
        }
    }
    double v[NC];
    v[0] = -(double)J * ff_to_double(acc[0]);
#pragma unroll
    for (int c = 1; c < NC; ++c) v[c] = ff_to_double(acc[c]);
    cluster_sum<NC>(v, scratch, part);
    if (sp.rank == 0 && threadIdx.x == 0) {
        const int d = tidx ? tidx[r] : r;
        out[d] = need_e ? v[0] : cached[r];
        if (NC == 12) {
            out[1 * R + d] = v[1];
            out[2 * R + d] = v[2];
            out[3 * R + d] = v[3];
            out[4 * R + d] = (v[4] * v[4] + v[5] * v[5] + v[6] * v[6] +
                              2 * (v[7] * v[7] + v[8] * v[8] + v[9] * v[9])) / 3;
            out[5 * R + d] = v[10];
            out[6 * R + d] = v[11];
        }
    }
}

}  // namespace mcgb

using namespace mcgb;

// ------------------------------------------------------------------ C ABI

extern "C" int mcgb_ising_update_color(int8_t *spins, void *rng, const float *betas, int R, int L,
                                       int color, float J, void *stream)
{
    if (int st = check_lattice("ising_update_color", R, L)) return st;
    MCGB_REQUIRE(spins && rng && betas, "ising_update_color: null pointer");
    MCGB_REQUIRE(color >= 0 && color < 4, "ising_update_color: color must be 0..3");
    const ColourGrid cg = colour_grid(R, L, 1);
    ising_phase_kernel<<<cg.grid, cg.block, 0, as_stream(stream)>>>(
        spins, static_cast<ulonglong2 *>(rng), betas, R, L, color, 1, J);
    return check_launch("ising_phase_kernel");
}

extern "C" int mcgb_ising_sweep(int8_t *spins, void *rng, const float *betas, int R, int L, float J,
                                int n_sweeps, void *stream)
{
    if (int st = check_lattice("ising_sweep", R, L)) return st;
    MCGB_REQUIRE(spins && rng && betas, "ising_sweep: null pointer");
    MCGB_REQUIRE(n_sweeps >= 0, "ising_sweep: n_sweeps must be >= 0");
    const ColourGrid one = colour_grid(R, L, 1), two = colour_grid(R, L, 2);
    cudaStream_t s = as_stream(stream);
    for (int k = 0; k < n_sweeps; ++k) {
        ising_phase_kernel<<<one.grid, one.block, 0, s>>>(
            spins, static_cast<ulonglong2 *>(rng), betas, R, L, 0, 1, J);
        ising_phase_kernel<<<two.grid, two.block, 0, s>>>(
            spins, static_cast<ulonglong2 *>(rng), betas, R, L, 1, 2, J);
        ising_phase_kernel<<<one.grid, one.block, 0, s>>>(
            spins, static_cast<ulonglong2 *>(rng), betas, R, L, 3, 1, J);
    }
    return check_launch("ising_phase_kernel");
}

extern "C" int mcgb_ising_energy(const int8_t *spins, int R, int L, float J, double *out, void *stream)
{
    if (int st = check_lattice("ising_energy", R, L)) return st;
    MCGB_REQUIRE(spins && out, "ising_energy: null pointer");
    return launch_replica_reduce(ising_reduce_kernel, R, L, kReduceThreads, as_stream(stream), "ising_reduce_kernel",
                                 spins, R, L, J, (const int32_t *)nullptr, (const double *)nullptr, out, 1);
}

extern "C" int mcgb_ising_measure(const int8_t *spins, int R, int L, float J, const int32_t *tidx,
                                  const double *cached, double *out, void *stream)
{
    if (int st = check_lattice("ising_measure", R, L)) return st;
    MCGB_REQUIRE(spins && out, "ising_measure: null pointer");
    return launch_replica_reduce(ising_reduce_kernel, R, L, kReduceThreads, as_stream(stream), "ising_reduce_kernel",
                                 spins, R, L, J, tidx, cached, out, 0);
}

extern "C" int mcgb_xy_update_color(float *theta, void *rng, const float *betas, int R, int L, int color,
                                    float J, float delta, void *stream)
{
    if (int st = check_lattice("xy_update_color", R, L)) return st;
    MCGB_REQUIRE(theta && rng && betas, "xy_update_color: null pointer");
    MCGB_REQUIRE(color >= 0 && color < 4, "xy_update_color: color must be 0..3");
    const ColourGrid cg = colour_grid(R, L, 1);
    xy_color_kernel<false><<<cg.grid, cg.block, 0, as_stream(stream)>>>(
        theta, static_cast<ulonglong2 *>(rng), betas, nullptr, R, L, color, 1, J, delta);
    return check_launch("xy_color_kernel");
}

extern "C" int mcgb_xy_update_color_gauss(float *theta, void *rng, const float *betas, const float *sigmas,
                                          int R, int L, int color, float J, void *stream)
{
    if (int st = check_lattice("xy_update_color_gauss", R, L)) return st;
    MCGB_REQUIRE(theta && rng && betas && sigmas, "xy_update_color_gauss: null pointer");
    MCGB_REQUIRE(color >= 0 && color < 4, "xy_update_color_gauss: color must be 0..3");
    const ColourGrid cg = colour_grid(R, L, 1);
    xy_color_kernel<true><<<cg.grid, cg.block, 0, as_stream(stream)>>>(
        theta, static_cast<ulonglong2 *>(rng), betas, sigmas, R, L, color, 1, J, 0.0f);
    return check_launch("xy_color_kernel");
}

extern "C" int mcgb_xy_sweep(float *theta, void *rng, const float *betas, const float *sigmas, int R, int L,
                             float J, float delta, int n_sweeps, void *stream)
{
    if (int st = check_lattice("xy_sweep", R, L)) return st;
    MCGB_REQUIRE(theta && rng && betas, "xy_sweep: null pointer");
    MCGB_REQUIRE(n_sweeps >= 0, "xy_sweep: n_sweeps must be >= 0");
    cudaStream_t s = as_stream(stream);
    ulonglong2 *st = static_cast<ulonglong2 *>(rng);
    for (int k = 0; k < n_sweeps; ++k) {
        for (int ph = 0; ph < 3; ++ph) {
            const int c0 = ph == 0 ? 0 : (ph == 1 ? 1 : 3), ncol = ph == 1 ? 2 : 1;
            const ColourGrid cg = colour_grid(R, L, ncol);
            if (sigmas)
                xy_color_kernel<true><<<cg.grid, cg.block, 0, s>>>(
                    theta, st, betas, sigmas, R, L, c0, ncol, J, 0.0f);
            else
                xy_color_kernel<false><<<cg.grid, cg.block, 0, s>>>(
                    theta, st, betas, nullptr, R, L, c0, ncol, J, delta);
        }
    }
    return check_launch("xy_color_kernel");
}

extern "C" int mcgb_xy64_update_color(double *theta, void *rng, const double *betas, const double *sigmas,
                                      const int32_t *w2t, int R, int L, int r, int color, double J, double delta,
                                      void *stream)
{
    if (int st = check_lattice("xy64_update_color", R, L)) return st;
    MCGB_REQUIRE(theta && rng && betas, "xy64_update_color: null pointer");
    MCGB_REQUIRE(r >= 0 && r < R, "xy64_update_color: replica out of range");
    MCGB_REQUIRE(color >= 0 && color < 4, "xy64_update_color: color must be 0..3");
    const ColourGrid cg = colour_grid(1, L, 1);
    xy64_color_kernel<<<cg.grid, cg.block, 0, as_stream(stream)>>>(
        theta, static_cast<ulonglong2 *>(rng), betas, sigmas, w2t, L, r, color, J, delta);
    return check_launch("xy64_color_kernel");
}

extern "C" int mcgb_xy64_energy(const double *theta, int R, int L, int r, double J, double *out, void *stream)
{
    if (int st = check_lattice("xy64_energy", R, L)) return st;
    MCGB_REQUIRE(theta && out, "xy64_energy: null pointer");
    MCGB_REQUIRE(r >= 0 && r < R, "xy64_energy: replica out of range");
    xy64_energy_kernel<<<1, 1024, 0, as_stream(stream)>>>(theta, L, r, J, out);
    return check_launch("xy64_energy_kernel");
}

extern "C" int mcgb_xy64_measure(const double *theta, int R, int L, int r, double J, const int32_t *w2t,
                                  double *out, void *stream)
{
    if (int st = check_lattice("xy64_measure", R, L)) return st;
    MCGB_REQUIRE(theta && out, "xy64_measure: null pointer");
    MCGB_REQUIRE(r >= 0 && r < R, "xy64_measure: replica out of range");
    xy64_measure_kernel<<<1, 1024, 0, as_stream(stream)>>>(theta, L, r, J, w2t, out, R);
    return check_launch("xy64_measure_kernel");
}

extern "C" int mcgb_xy_energy(const float *theta, int R, int L, float J, double *out, void *stream)
{
    if (int st = check_lattice("xy_energy", R, L)) return st;
    MCGB_REQUIRE(theta && out, "xy_energy: null pointer");
    return launch_replica_reduce(xy_reduce_kernel<1>, R, L, kReduceThreads, as_stream(stream), "xy_reduce_kernel",
                                 theta, R, L, J, (const int32_t *)nullptr, (const double *)nullptr, out);
}

extern "C" int mcgb_xy_measure(const float *theta, int R, int L, float J, const int32_t *tidx,
                               const double *cached, double *out, void *stream)
{
    if (int st = check_lattice("xy_measure", R, L)) return st;
    MCGB_REQUIRE(theta && out, "xy_measure: null pointer");
    return launch_replica_reduce(xy_reduce_kernel<5>, R, L, kReduceThreads, as_stream(stream), "xy_reduce_kernel",
                                 theta, R, L, J, tidx, cached, out);
}

extern "C" int mcgb_kawamura_update_color(float *state, void *rng, const float *betas, int R, int L,
                                          int color, float J, float delta, void *stream)
{
    if (int st = check_lattice("kawamura_update_color", R, L)) return st;
    MCGB_REQUIRE(state && rng && betas, "kawamura_update_color: null pointer");
    MCGB_REQUIRE(color >= 0 && color < 4, "kawamura_update_color: color must be 0..3");
    const ColourGrid cg = colour_grid(R, L, 1);
    kawamura_color_kernel<<<cg.grid, cg.block, 0, as_stream(stream)>>>(
        state, static_cast<ulonglong2 *>(rng), betas, R, L, color, 1, J, delta);
    return check_launch("kawamura_color_kernel");
}

extern "C" int mcgb_kawamura_sweep(float *state, void *rng, const float *betas, int R, int L, float J,
                                   float delta, int n_sweeps, void *stream)
{
    if (int st = check_lattice("kawamura_sweep", R, L)) return st;
    MCGB_REQUIRE(state && rng && betas, "kawamura_sweep: null pointer");
    MCGB_REQUIRE(n_sweeps >= 0, "kawamura_sweep: n_sweeps must be >= 0");
    cudaStream_t s = as_stream(stream);
    for (int k = 0; k < n_sweeps; ++k) {
        for (int ph = 0; ph < 3; ++ph) {
            const int c0 = ph == 0 ? 0 : (ph == 1 ? 1 : 3), ncol = ph == 1 ? 2 : 1;
            const ColourGrid cg = colour_grid(R, L, ncol);
            kawamura_color_kernel<<<cg.grid, cg.block, 0, s>>>(
                state, static_cast<ulonglong2 *>(rng), betas, R, L, c0, ncol, J, delta);
        }
    }
    return check_launch("kawamura_color_kernel");
}

extern "C" int mcgb_kawamura_energy(const float *state, int R, int L, float J, double *out, void *stream)
{
    if (int st = check_lattice("kawamura_energy", R, L)) return st;
    MCGB_REQUIRE(state && out, "kawamura_energy: null pointer");
    return launch_replica_reduce(kawamura_reduce_kernel<1>, R, L, kReduceThreads, as_stream(stream),
                                 "kawamura_reduce_kernel", state, R, L, J, (const int32_t *)nullptr,
                                 (const double *)nullptr, out);
}

extern "C" int mcgb_kawamura_measure(const float *state, int R, int L, float J, const int32_t *tidx,
                                     const double *cached, double *out, void *stream)
{
    if (int st = check_lattice("kawamura_measure", R, L)) return st;
    MCGB_REQUIRE(state && out, "kawamura_measure: null pointer");
    return launch_replica_reduce(kawamura_reduce_kernel<12>, R, L, kReduceThreads, as_stream(stream),
                                 "kawamura_reduce_kernel", state, R, L, J, tidx, cached, out);
}

extern "C" int mcgb_kawamura_local_energies(const float *state, int R, int L, const int32_t *positions,
                                            const float *proposed, int n, float J, float *out, void *stream)
{
    if (int st = check_lattice("kawamura_local_energies", R, L)) return st;
    MCGB_REQUIRE(n >= 0, "kawamura_local_energies: n must be >= 0");
    if (n == 0) return MCGB_OK;
    MCGB_REQUIRE(state && positions && proposed && out, "kawamura_local_energies: null pointer");
    kawamura_local_kernel<<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(state, L, positions, proposed, n, J, out);
    return check_launch("kawamura_local_kernel");
}
