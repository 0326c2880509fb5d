// He3 thin-film model: per-colour Cartesian Metropolis and conditional
// Gaussian MH updates, energy and measurement reductions, on the reference's
// complex64 (R, L, L, 3, 2) layout (12 floats = 48 bytes per site).
//
// Local algebra is float32 complex arithmetic in the reference's operation
// order (models/he3/update.py:9-175, models/he3/gaussian_fast.py:26-119);
// lattice sums accumulate in float64 (models/he3/measure.py).  The site
// neighbourhood is the 3 forward gradient cells that contain the site:
// (i+-1, j), (i, j+-1), (i-1, j+1), (i+1, j-1) — six neighbours, so all four
// colours must run in sequence.
#include "mcgb_common.cuh"

namespace mcgb {

struct Coeff5 {
    float b[5];
};

__device__ __forceinline__ c32 ld_c(const float *state, int L, int r, int i, int j, int k)
{
    const float2 v = reinterpret_cast<const float2 *>(state)[(((int64_t)r * L + i) * L + j) * 6 + k];
    return cmk(v.x, v.y);
}

// models/he3/update.py:14-28
__device__ __forceinline__ float he3_dipole(const c32 *psi, float n)
{
    const c32 a = psi[0], b = psi[1], c = psi[2], d = psi[3];
    return norm2(a + d) + norm2(a) + norm2(d) + 2.0f * (b * conj(c)).re - (float)(2.0 / 3.0) * n;
}

// models/he3/update.py:32-63
__device__ __forceinline__ float he3_potential(const c32 *psi, const Coeff5 &beta, float g_d)
{
    float nx = norm2(psi[0]), ny = norm2(psi[1]);
    c32 xx = psi[0] * psi[0], yy = psi[1] * psi[1], xy = psi[0] * psi[1];
    c32 overlap = conj(psi[0]) * psi[1];
#pragma unroll
    for (int mu = 1; mu < 3; ++mu) {
        const c32 x = psi[2 * mu], y = psi[2 * mu + 1];
        nx += norm2(x);
        ny += norm2(y);
        xx = xx + x * x;
        yy = yy + y * y;
        xy = xy + x * y;
        overlap = overlap + conj(x) * y;
    }
    const float n = nx + ny, two = 2.0f;
    const float i1 = norm2(xx + yy);
    const float i2 = n * n;
    const float i3 = nx * nx + ny * ny + two * (overlap * overlap).re;
    const float i4 = nx * nx + ny * ny + two * norm2(overlap);
    const float i5 = norm2(xx) + norm2(yy) + two * norm2(xy);
    const float dip = he3_dipole(psi, n);
    return -two * n + beta.b[0] * i1 + beta.b[1] * i2 + beta.b[2] * i3 + beta.b[3] * i4 +
           beta.b[4] * i5 + g_d * dip;
}

// models/he3/update.py:66-72
__device__ __forceinline__ float he3_gradient(c32 dx_x, c32 dx_y, c32 dy_x, c32 dy_y)
{
    return 3.0f * (norm2(dx_x) + norm2(dy_y)) + norm2(dx_y) + norm2(dy_x) +
           2.0f * (conj(dx_x) * dy_y + conj(dx_y) * dy_x).re;
}

// models/he3/update.py:95-175 — exact change of the three affected cells.
__device__ __forceinline__ float he3_gradient_difference(const float *state, int L, int r, int i, int j,
                                                         const c32 *proposed)
{
    const int ip = wrapi(i + 1, L), im = wrapi(i - 1, L), jp = wrapi(j + 1, L), jm = wrapi(j - 1, L);
    float delta_g = 0.0f;
#pragma unroll
    for (int mu = 0; mu < 3; ++mu) {
        const int kx = 2 * mu, ky = 2 * mu + 1;
        const c32 x = ld_c(state, L, r, i, j, kx), y = ld_c(state, L, r, i, j, ky);
        const c32 ex = proposed[kx] - x, ey = proposed[ky] - y;
        const c32 rx = ld_c(state, L, r, ip, j, kx), ry = ld_c(state, L, r, ip, j, ky);
        const c32 ux = ld_c(state, L, r, i, jp, kx), uy = ld_c(state, L, r, i, jp, ky);
        const c32 lx = ld_c(state, L, r, im, j, kx), ly = ld_c(state, L, r, im, j, ky);
        const c32 dx = ld_c(state, L, r, i, jm, kx), dy = ld_c(state, L, r, i, jm, ky);
        const c32 lux = ld_c(state, L, r, im, jp, kx), luy = ld_c(state, L, r, im, jp, ky);
        const c32 drx = ld_c(state, L, r, ip, jm, kx), dry = ld_c(state, L, r, ip, jm, ky);
        const c32 a = rx - x, b = ry - y, c = ux - x, d = uy - y;
        const c32 al = x - lx, dl = luy - ly, bl = y - ly, cl = lux - lx;
        const c32 ad = drx - dx, bd = dry - dy, cd = x - dx, dd = y - dy;
        const c32 fx = (-(3.0f * a + b + c + d) + (3.0f * al + dl)) + (cd + bd);
        const c32 fy = (-(a + b + c + 3.0f * d) + (bl + cl)) + (3.0f * dd + ad);
        const float linear = 2.0f * (conj(ex) * fx + conj(ey) * fy).re;
        const float quadratic = 8.0f * (norm2(ex) + norm2(ey)) + 4.0f * (conj(ex) * ey).re;
        delta_g += linear + quadratic;
    }
    return delta_g;
}

// models/he3/update.py:178-227
__global__ void he3_color_kernel(float *__restrict__ state, ulonglong2 *__restrict__ rng,
                                 const float *__restrict__ betas, int R, int L, int color, Coeff5 coeff,
                                 float K, float delta, float g_d)
{
    int r, i, j;
    if (!colour_grid_site(R, L, color, r, i, j)) return;
    const int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
    ulonglong2 st = rng[idx];
    c32 psi[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) psi[k] = ld_c(state, L, r, i, j, k);
    const float old_potential = he3_potential(psi, coeff, g_d);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float re = delta * (2.0f * xoro_uniform_f32(st) - 1.0f);
        const float im = delta * (2.0f * xoro_uniform_f32(st) - 1.0f);
        psi[k] = cmk(psi[k].re + re, psi[k].im + im);
    }
    const float dv = he3_potential(psi, coeff, g_d) - old_potential;
    const float dg = he3_gradient_difference(state, L, r, i, j, psi);
    const float difference = dv + K * dg;
    const float u = xoro_uniform_f32(st);
    rng[idx] = st;
    if (difference <= 0.0f || u < expf(-betas[r] * difference)) {
        float2 *p = reinterpret_cast<float2 *>(state) + idx * 6;
#pragma unroll
        for (int k = 0; k < 6; ++k) p[k] = make_float2(psi[k].re, psi[k].im);
    }
}

// models/he3/gaussian_fast.py:42-50
__device__ __forceinline__ c32 he3_normal_pair(ulonglong2 &st)
{
    float u = xoro_uniform_f32(st);
    if (u <= 0.0f) u = 1.1102230246251565e-16f;
    const float angle = 6.283185307179586f * xoro_uniform_f32(st);
    const float radius = sqrtf(-2.0f * logf(u));
    float s, c;
    sincosf(angle, &s, &c);
    return cmk(radius * c, radius * s);
}

// models/he3/gaussian_fast.py:91-119 (with :26-40 neighbor field, :53-88 proposal)
__global__ void he3_gauss_color_kernel(float *__restrict__ state, ulonglong2 *__restrict__ rng,
                                       const float *__restrict__ betas, int R, int L, int color,
                                       Coeff5 coeff, float K, float rho, float mass, float g_d,
                                       long long *__restrict__ counts)
{
    int r, i, j;
    if (!colour_grid_site(R, L, color, r, i, j)) return;
    const int64_t idx = (int64_t)r * L * L + (int64_t)i * L + j;
    const int64_t plane = (int64_t)R * L * L;
    const int ip = wrapi(i + 1, L), im = wrapi(i - 1, L), jp = wrapi(j + 1, L), jm = wrapi(j - 1, L);
    c32 field[6], psi[6];
#pragma unroll
    for (int mu = 0; mu < 3; ++mu) {
        const int kx = 2 * mu, ky = 2 * mu + 1;
        const c32 rx = ld_c(state, L, r, ip, j, kx), ry = ld_c(state, L, r, ip, j, ky);
        const c32 ux = ld_c(state, L, r, i, jp, kx), uy = ld_c(state, L, r, i, jp, ky);
        const c32 lx = ld_c(state, L, r, im, j, kx), ly = ld_c(state, L, r, im, j, ky);
        const c32 dx = ld_c(state, L, r, i, jm, kx), dy = ld_c(state, L, r, i, jm, ky);
        const c32 lux = ld_c(state, L, r, im, jp, kx), luy = ld_c(state, L, r, im, jp, ky);
        const c32 drx = ld_c(state, L, r, ip, jm, kx), dry = ld_c(state, L, r, ip, jm, ky);
        field[kx] = -3.0f * (rx + lx) - ux - uy - ry - ly - dx - dy + luy + dry;
        field[ky] = -rx - ry - ux - lx - ly - dx - 3.0f * (uy + dy) + lux + drx;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) psi[k] = ld_c(state, L, r, i, j, k);
    const float beta = betas[r];
    ulonglong2 st = rng[idx];
    const float old_potential = he3_potential(psi, coeff, g_d);

    // gaussian_proposal_float32
    const float one = 1.0f, two = 2.0f, root = 0.7071067811865475f;
    const float plus = 10.0f * K + mass, minus = 6.0f * K + mass;
    const float vf = one - rho * rho;
    const float sp = sqrtf(vf / (two * beta * plus));
    const float sm = sqrtf(vf / (two * beta * minus));
    const float qp = vf / (8.0f * root * root * sp * sp);
    const float qm = vf / (8.0f * root * root * sm * sm);
    float lpr = 0.0f;
#pragma unroll
    for (int mu = 0; mu < 3; ++mu) {
        const int kx = 2 * mu, ky = 2 * mu + 1;
        const c32 x = psi[kx], y = psi[ky];
        const c32 hp = root * (field[kx] + field[ky]);
        const c32 hm = root * (field[kx] - field[ky]);
        c32 mp = (-K) * hp, mm = (-K) * hm;
        mp = cmk(mp.re / plus, mp.im / plus);
        mm = cmk(mm.re / minus, mm.im / minus);
        const c32 mx = root * (mp + mm), my = root * (mp - mm);
        const c32 zp = sp * he3_normal_pair(st);
        const c32 zm = sm * he3_normal_pair(st);
        const c32 nx = (mx + rho * (x - mx)) + root * (zp + zm);
        const c32 ny = (my + rho * (y - my)) + root * (zp - zm);
        psi[kx] = nx;
        psi[ky] = ny;
        const c32 old_plus = (x - mx) + (y - my), old_minus = (x - mx) - (y - my);
        const c32 new_plus = (nx - mx) + (ny - my), new_minus = (nx - mx) - (ny - my);
        lpr += qp * (norm2(new_plus) - norm2(old_plus));
        lpr += qm * (norm2(new_minus) - norm2(old_minus));
    }
    const float delta_h = he3_potential(psi, coeff, g_d) - old_potential +
                          K * he3_gradient_difference(state, L, r, i, j, psi);
    const float log_ratio = -beta * delta_h + lpr;
    const float u = xoro_uniform_f32(st);
    rng[idx] = st;
    counts[idx] += 1;
    if (!isfinite(log_ratio)) {
        counts[2 * plane + idx] += 1;
    } else if (log_ratio >= 0.0f || u < expf(log_ratio)) {
        counts[plane + idx] += 1;
        float2 *p = reinterpret_cast<float2 *>(state) + idx * 6;
#pragma unroll
        for (int k = 0; k < 6; ++k) p[k] = make_float2(psi[k].re, psi[k].im);
    }
}

// models/he3/measure.py:22-143.  NC = 1: energy; NC = 10: all sums (channel 9
// holds the spin-z density until the spin-alignment ratio is formed).
template <int NC>
__global__ void he3_reduce_kernel(const float *__restrict__ state, int R, int L, Coeff5 coeff, float K,
                                  float g_d, const int32_t *__restrict__ tidx,
                                  const double *__restrict__ cached, double *__restrict__ out)
{
    __shared__ double scratch[NC * 32], part[NC];
    const ReplicaSpan sp = replica_span();
    const int r = sp.r;
    double v[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) v[c] = 0.0;
    const bool need_e = cached == nullptr;
    for (int k = sp.first; k < L * L; k += sp.step) {
        const int i = k / L, j = k - i * L;
        const int ip = wrapi(i + 1, L), jp = wrapi(j + 1, L);
        c32 psi[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) psi[q] = ld_c(state, L, r, i, j, q);
        if (need_e) v[0] += he3_potential(psi, coeff, g_d);
#pragma unroll
        for (int mu = 0; mu < 3; ++mu) {
            const c32 x = psi[2 * mu], y = psi[2 * mu + 1];
            const c32 xpx = ld_c(state, L, r, ip, j, 2 * mu), xpy = ld_c(state, L, r, ip, j, 2 * mu + 1);
            const c32 ypx = ld_c(state, L, r, i, jp, 2 * mu), ypy = ld_c(state, L, r, i, jp, 2 * mu + 1);
            const c32 a = xpx - x, b = xpy - y, c = ypx - x, d = ypy - y;
            if (need_e) v[0] += K * he3_gradient(a, b, c, d);
            if (NC == 10) {
                const float rd = norm2(x) + norm2(y);
                v[NC == 10 ? 1 : 0] += rd;
                if (mu == 2) v[NC == 10 ? 9 : 0] += rd;
                v[NC == 10 ? 2 : 0] += 2.0 * (double)(conj(x) * y).im;
                const c32 ph = x * x - y * y;
                v[NC == 10 ? 3 : 0] += ph.re;
                v[NC == 10 ? 4 : 0] += ph.im;
                // measure.py:54-60; Numba promotes int64 * complex64 to complex128.
                const double ar = a.re, ai = -(double)a.im, br = b.re, bi = -(double)b.im;
                const double cr = c.re, ci = -(double)c.im, dr = d.re, di = -(double)d.im;
                const double zx_r = (3 * ar + dr) * xpx.re - (3 * ai + di) * xpx.im + (br + cr) * xpy.re -
                                    (bi + ci) * xpy.im;
                const double zx_i = (3 * ar + dr) * xpx.im + (3 * ai + di) * xpx.re + (br + cr) * xpy.im +
                                    (bi + ci) * xpy.re;
                const double zy_r = (cr + br) * ypx.re - (ci + bi) * ypx.im + (3 * dr + ar) * ypy.re -
                                    (3 * di + ai) * ypy.im;
                const double zy_i = (cr + br) * ypx.im + (ci + bi) * ypx.re + (3 * dr + ar) * ypy.im +
                                    (3 * di + ai) * ypy.re;
                const double K2 = 2.0 * (double)K;
                v[NC == 10 ? 5 : 0] += K2 * zx_i;
                v[NC == 10 ? 6 : 0] += K2 * (3.0 * norm2(xpx) + (double)norm2(xpy) - zx_r);
                v[NC == 10 ? 7 : 0] += K2 * zy_i;
                v[NC == 10 ? 8 : 0] += K2 * ((double)norm2(ypx) + 3.0 * norm2(ypy) - zy_r);
            }
        }
    }
    cluster_sum<NC>(v, scratch, part);
    if (sp.rank == 0 && threadIdx.x == 0) {
        const int dst = tidx ? tidx[r] : r;
        out[dst] = need_e ? v[0] : cached[r];
        if (NC == 10) {
#pragma unroll
            for (int c = 1; c < 9; ++c) out[c * R + dst] = v[c];
            out[9 * R + dst] = v[1] == 0.0 ? 0.0 : 0.5 * (3 * v[NC == 10 ? 9 : 0] / v[1] - 1);
        }
    }
}

__global__ void he3_local_diff_kernel(const float *__restrict__ state, int L, const int32_t *__restrict__ pos,
                                      const float *__restrict__ proposed, int n, Coeff5 coeff, float K,
                                      float g_d, double *__restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int r = pos[3 * k], i = pos[3 * k + 1], j = pos[3 * k + 2];
    c32 oldp[6], newp[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        oldp[q] = ld_c(state, L, r, i, j, q);
        newp[q] = cmk(proposed[(6 * k + q) * 2], proposed[(6 * k + q) * 2 + 1]);
    }
    const float dg = he3_gradient_difference(state, L, r, i, j, newp);
    const float dv = he3_potential(newp, coeff, g_d) - he3_potential(oldp, coeff, g_d);
    out[k] = dg;
    out[n + k] = dv;
    out[2 * n + k] = dv + K * dg;
}

inline int check_he3(const char *who, int R, int L, const float *coeff)
{
    MCGB_REQUIRE(R >= 1, "%s: R must be >= 1", who);
    MCGB_REQUIRE(R <= 32767, "%s: at most 32767 replicas (one grid layer per replica)", who);
    MCGB_REQUIRE(L >= 4 && L % 2 == 0, "%s: L must be even and >= 4", who);
    MCGB_REQUIRE(coeff != nullptr, "%s: null coefficients", who);
    return MCGB_OK;
}

inline Coeff5 make_coeff(const float *c)
{
    Coeff5 k;
    for (int q = 0; q < 5; ++q) k.b[q] = c[q];
    return k;
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace mcgb

using namespace mcgb;

extern "C" int mcgb_he3_update_color(float *state, void *rng, const float *betas, int R, int L, int color,
                                     const float *coefficients, float K, float delta, float g_d, void *stream)
{
    if (int st = check_he3("he3_update_color", R, L, coefficients)) return st;
    MCGB_REQUIRE(state && rng && betas, "he3_update_color: null pointer");
    MCGB_REQUIRE(color >= 0 && color < 4, "he3_update_color: color must be 0..3");
    const ColourGrid cg = colour_grid(R, L, 1, 128);
    he3_color_kernel<<<cg.grid, cg.block, 0, as_stream(stream)>>>(
        state, static_cast<ulonglong2 *>(rng), betas, R, L, color, make_coeff(coefficients), K, delta, g_d);
    return check_launch("he3_color_kernel");
}

extern "C" int mcgb_he3_gaussian_update_color(float *state, void *rng, const float *betas, int R, int L,
                                              int color, const float *coefficients, float K, float rho,
                                              float mass, float g_d, int64_t *counts, void *stream)
{
    if (int st = check_he3("he3_gaussian_update_color", R, L, coefficients)) return st;
    MCGB_REQUIRE(state && rng && betas && counts, "he3_gaussian_update_color: null pointer");
    MCGB_REQUIRE(color >= 0 && color < 4, "he3_gaussian_update_color: color must be 0..3");
    const ColourGrid cg = colour_grid(R, L, 1, 128);
    he3_gauss_color_kernel<<<cg.grid, cg.block, 0, as_stream(stream)>>>(
        state, static_cast<ulonglong2 *>(rng), betas, R, L, color, make_coeff(coefficients), K, rho, mass, g_d,
        reinterpret_cast<long long *>(counts));
    return check_launch("he3_gauss_color_kernel");
}

extern "C" int mcgb_he3_energy(const float *state, int R, int L, const float *coefficients, float K, float g_d,
                               double *out, void *stream)
{
    if (int st = check_he3("he3_energy", R, L, coefficients)) return st;
    MCGB_REQUIRE(state && out, "he3_energy: null pointer");
    return launch_replica_reduce(he3_reduce_kernel<1>, R, L, 256, as_stream(stream), "he3_reduce_kernel", state, R,
                                 L, make_coeff(coefficients), K, g_d, (const int32_t *)nullptr,
                                 (const double *)nullptr, out);
}

extern "C" int mcgb_he3_measure(const float *state, int R, int L, const float *coefficients, float K, float g_d,
                                const int32_t *tidx, const double *cached, double *out, void *stream)
{
    if (int st = check_he3("he3_measure", R, L, coefficients)) return st;
    MCGB_REQUIRE(state && out, "he3_measure: null pointer");
    return launch_replica_reduce(he3_reduce_kernel<10>, R, L, 256, as_stream(stream), "he3_reduce_kernel", state, R,
                                 L, make_coeff(coefficients), K, g_d, tidx, cached, out);
}

extern "C" int mcgb_he3_local_differences(const float *state, int R, int L, const int32_t *positions,
                                          const float *proposed, int n, const float *coefficients, float K,
                                          float g_d, double *out, void *stream)
{
    if (int st = check_he3("he3_local_differences", R, L, coefficients)) return st;
    MCGB_REQUIRE(n >= 0, "he3_local_differences: n must be >= 0");
    if (n == 0) return MCGB_OK;
    MCGB_REQUIRE(state && positions && proposed && out, "he3_local_differences: null pointer");
    he3_local_diff_kernel<<<blocks_for(n, 64), 64, 0, as_stream(stream)>>>(
        state, L, positions, proposed, n, make_coeff(coefficients), K, g_d, out);
    return check_launch("he3_local_diff_kernel");
}
