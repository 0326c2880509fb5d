// Batched-engine policies for the Kawamura and He3 models (mixed precision).
//
// Kawamura (models/kawamura/update.py:7-65): a site carries (theta, tau, d);
// shared memory holds (cos theta, sin theta, tau, d) so that, with
//   w_n = d . d_n,  A = sum w_n cos_n,  B = sum w_n sin_n,
//   A' = sum tau_n w_n cos_n,  B' = sum tau_n w_n sin_n   (four neighbours),
// the local energy of (theta, tau, d) is
//   E = -J [ cos(theta) A + sin(theta) B + tau (cos(theta) A' + sin(theta) B') ],
// and the three sequential sub-moves (theta, tau flip, d on the sphere) cost
// two neighbour sums instead of sixteen cosines.  The six draws of a visit
// (theta proposal, theta accept, tau accept, z, phi, d accept) are all taken
// in propose, in that order.  The (cos, sin) cache persists in `aux`.
//
// He3 (models/he3/update.py:9-227, models/he3/gaussian_fast.py:26-119): the
// cell is the site's six complex64 components; neighbours are the four
// nearest plus (i-1, j+1) and (i+1, j-1), the corners of the three forward
// gradient cells that contain the site, so colours 1 and 2 are updated in
// separate phases.  Cartesian: propose draws the twelve offsets and the
// acceptance uniform and evaluates the on-site potential change; decide adds
// the exact gradient change.  Conditional Gaussian: propose draws the six
// Box-Muller pairs and the acceptance uniform; decide builds the neighbour
// field, the autoregressive proposal and its reverse/forward log density
// ratio, then the full Hamiltonian change.  Nonfinite log ratios are counted
// per replica (counters row 2) and rejected.
#include "batch_args.cuh"

namespace mcgb {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kTwoPi = 6.28318530717958647692f;

// =============================================================== Kawamura

struct KawCell {
    float c, s, tau, dx, dy, dz;
};

// kGauss: Gaussian proposals (this project's extension, no reference
// counterpart): theta' = theta + sigma z0 (wrapped), d' = normalise(d + sigma g)
// with g three standard normals -- symmetric, since its density depends only
// on the angle between d and d' -- and the reference's tau flip.  Five draws
// per visit: the normal pairs (z0, gx) and (gy, gz), each from bits 63..41
// and 40..18 of one draw, then the three acceptance uniforms.
template <bool kGauss>
struct KawamuraPolicy {
    using Args = BatchArgs;
    using Cell = KawCell;
    static constexpr int kOwnFloats = 1;  // theta
    static constexpr int kChannels = 7;   // energy, chirality, px, py, spin2, twist_cos_x, twist_sin_x
    static constexpr int kSums = 12;      // ... with the six spin-tensor sums in place of spin2
    static constexpr int kMaxThreads = 512;
    static constexpr int kPairThreads = 256;  // two plaquettes a thread spill at 128 registers
    static constexpr bool kSplitMiddle = false;
    static constexpr bool kPipeline = true;
    // Global-stream variant: sites whose visits one thread carries at once.
    static constexpr int kGlobalInFlight = 2;
    static constexpr bool kSmemStreams = false;
    static constexpr bool kEnergyFromDelta = true;
    static constexpr bool kExactEnergy = false;
    // The cell gathers (cos, sin) from the cache and tau, d from the state:
    // loaded site by site.
    static constexpr bool kRefLayout = false;  // colour-major batch arrays
    static constexpr bool kBulkLoad = false;

    struct Ctx {
        float beta, J, delta, sigma;
    };
    struct Prop {
        float tp, cp, sp;  // theta proposal and its (cos, sin)
        float x, y, z;     // sphere proposal
        float v1, v2, v3;  // acceptance uniforms of the three sub-moves
    };

    static __device__ __forceinline__ Ctx prepare(const Args &a, int, const mcgb_replica &, const Walker &wk)
    {
        return Ctx{wk.beta, a.J, a.delta, kGauss ? wk.sigma : 0.0f};
    }
    // A pair of standard normals from one draw (Box-Muller, fast intrinsics).
    static __device__ __forceinline__ float2 normal_pair(uint64_t bits)
    {
        float u = mcgb_fast_unit(bits);
        if (u <= 0.0f) u = 1.1102230246251565e-16f;
        const float t = -2.0f * __logf(u);
        const float rad = t * rsqrtf(t);
        float sn, cs;
        __sincosf(fmaf(kTwoPi, mcgb_fast_unit_mid(bits), -kPi), &sn, &cs);  // angle - pi
        return make_float2(-rad * cs, -rad * sn);
    }
    static __device__ __forceinline__ void load(const Args &a, int64_t site, Cell &cell, float *own)
    {
        const float *p = static_cast<const float *>(a.state) + 5 * site;
        own[0] = p[0];
        const float2 cs = a.aux[site];
        cell = KawCell{cs.x, cs.y, p[1], p[2], p[3], p[4]};
    }
    static __device__ __forceinline__ void store(const Args &a, int64_t site, const Cell &cell, const float *own)
    {
        float *p = static_cast<float *>(a.state) + 5 * site;
        p[0] = own[0];
        p[1] = cell.tau;
        p[2] = cell.dx;
        p[3] = cell.dy;
        p[4] = cell.dz;
        a.aux[site] = make_float2(cell.c, cell.s);
    }
    template <int C_>
    static __device__ __forceinline__ Prop propose(const Ctx &x, const Cell &me, const float *own, ulonglong2 &st)
    {
        Prop q;
        if (kGauss) {
            const float2 n0 = normal_pair(xoro_next(st));
            const float2 n1 = normal_pair(xoro_next(st));
            float tp = fmaf(x.sigma, n0.x, own[0]);
            tp -= kTwoPi * floorf((tp + kPi) * (1.0f / kTwoPi));
            if (tp >= kPi) tp -= kTwoPi;
            if (tp < -kPi) tp += kTwoPi;
            q.tp = tp;
            __sincosf(tp, &q.sp, &q.cp);
            q.v1 = mcgb_fast_unit(xoro_next(st));
            q.v2 = mcgb_fast_unit(xoro_next(st));
            const float gx = fmaf(x.sigma, n0.y, me.dx), gy = fmaf(x.sigma, n1.x, me.dy),
                        gz = fmaf(x.sigma, n1.y, me.dz);
            const float inv = rsqrtf(fmaf(gx, gx, fmaf(gy, gy, gz * gz)));
            q.x = gx * inv;
            q.y = gy * inv;
            q.z = gz * inv;
            q.v3 = mcgb_fast_unit(xoro_next(st));
            return q;
        }
        float tp = own[0] + x.delta * (2.0f * mcgb_fast_unit(xoro_next(st)) - 1.0f);
        if (tp >= kPi) tp -= kTwoPi;
        else if (tp < -kPi) tp += kTwoPi;
        q.tp = tp;
        __sincosf(tp, &q.sp, &q.cp);
        q.v1 = mcgb_fast_unit(xoro_next(st));
        q.v2 = mcgb_fast_unit(xoro_next(st));
        q.z = 2.0f * mcgb_fast_unit(xoro_next(st)) - 1.0f;
        const float phi = kTwoPi * mcgb_fast_unit(xoro_next(st));
        const float rad = sqrtf(fmaxf(1.0f - q.z * q.z, 0.0f));
        float sn, cs;
        __sincosf(phi - kPi, &sn, &cs);  // phi in [-pi, pi): cos(phi) = -cs, sin(phi) = -sn
        q.x = -rad * cs;
        q.y = -rad * sn;
        q.v3 = mcgb_fast_unit(xoro_next(st));
        return q;
    }

    struct Sums {
        float a, b, ap, bp;
    };
    static __device__ __forceinline__ Sums sums(const KawCell (&n)[4], float dx, float dy, float dz)
    {
        Sums r{0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float w = fmaf(dx, n[k].dx, fmaf(dy, n[k].dy, dz * n[k].dz));
            const float wc = w * n[k].c, ws = w * n[k].s;
            r.a += wc;
            r.b += ws;
            r.ap = fmaf(n[k].tau, wc, r.ap);
            r.bp = fmaf(n[k].tau, ws, r.bp);
        }
        return r;
    }
    static __device__ __forceinline__ float energy(const Sums &m, float c, float s, float tau, float J)
    {
        return -J * (fmaf(c, m.a, s * m.b) + tau * fmaf(c, m.ap, s * m.bp));
    }
    template <int C_>
    static __device__ __forceinline__ bool decide(const Ctx &x, const Nbrs<Cell> &nb, Cell &me, float *own,
                                                  const Prop &q, float &dE)
    {
        const KawCell n[4] = {MCGB_NBR(nb, kUp(C_)), MCGB_NBR(nb, kDown(C_)), MCGB_NBR(nb, kLeft(C_)),
                              MCGB_NBR(nb, kRight(C_))};
        const Sums m = sums(n, me.dx, me.dy, me.dz);
        const float e0 = energy(m, me.c, me.s, me.tau, x.J);
        float e = e0;
        bool changed = false;
        // theta
        float e1 = energy(m, q.cp, q.sp, me.tau, x.J);
        float d = e1 - e;
        if (d <= 0.0f || q.v1 < __expf(-x.beta * d)) {
            own[0] = q.tp;
            me.c = q.cp;
            me.s = q.sp;
            e = e1;
            changed = true;
        }
        // tau flip
        e1 = energy(m, me.c, me.s, -me.tau, x.J);
        d = e1 - e;
        if (d <= 0.0f || q.v2 < __expf(-x.beta * d)) {
            me.tau = -me.tau;
            e = e1;
            changed = true;
        }
        // d on the sphere
        const Sums m2 = sums(n, q.x, q.y, q.z);
        e1 = energy(m2, me.c, me.s, me.tau, x.J);
        d = e1 - e;
        if (d <= 0.0f || q.v3 < __expf(-x.beta * d)) {
            me.dx = q.x;
            me.dy = q.y;
            me.dz = q.z;
            e = e1;
            changed = true;
        }
        dE = e - e0;
        return changed;
    }
    template <int C_>
    static __device__ __forceinline__ void measure(const Ctx &, const Nbrs<Cell> &nb, const Cell &me,
                                                   const float *, FSum *v)
    {
        const KawCell dn = MCGB_NBR(nb, kDown(C_));
        const float third = 1.0f / 3.0f;
        v[1] += me.tau;
        v[2] += me.c * me.c - me.s * me.s;
        v[3] += 2.0f * me.c * me.s;
        v[4] += fmaf(me.dx, me.dx, -third);
        v[5] += fmaf(me.dy, me.dy, -third);
        v[6] += fmaf(me.dz, me.dz, -third);
        v[7] += me.dx * me.dy;
        v[8] += me.dx * me.dz;
        v[9] += me.dy * me.dz;
        const float w = (1.0f + me.tau * dn.tau) * fmaf(me.dx, dn.dx, fmaf(me.dy, dn.dy, me.dz * dn.dz));
        v[10] += w * fmaf(me.c, dn.c, me.s * dn.s);
        v[11] += w * fmaf(me.s, dn.c, -me.c * dn.s);
    }
    template <int C_>
    static __device__ __forceinline__ void energy_site(const Ctx &, const Nbrs<Cell> &, const Cell &, const float *,
                                                       FSum &)
    {
    }
    static __device__ __forceinline__ void finish_sample(const Ctx &, double *v)
    {
        // models/kawamura/measure.py:194-196: D = (dd^T - I/3); off-diagonal entries count twice.
        const double spin2 =
            (v[4] * v[4] + v[5] * v[5] + v[6] * v[6] + 2 * (v[7] * v[7] + v[8] * v[8] + v[9] * v[9])) / 3;
        v[4] = spin2;
        v[5] = v[10];
        v[6] = v[11];
    }
    static __device__ __forceinline__ double finish_energy(const Ctx &, double e) { return e; }
};

// =============================================================== He3

struct He3Cell {
    c32 z[6];  // index 2*mu + a: spin row mu (x, y, z), orbital column a (x, y)
};

__device__ __forceinline__ float he3_potential_f(const c32 *psi, const float *beta, float g_d)
{
    float nx = norm2(psi[0]), ny = norm2(psi[1]);
    c32 xx = psi[0] * psi[0], yy = psi[1] * psi[1], xy = psi[0] * psi[1];
    c32 ov = conj(psi[0]) * psi[1];
#pragma unroll
    for (int mu = 1; mu < 3; ++mu) {
        const c32 x = psi[2 * mu], y = psi[2 * mu + 1];
        nx += norm2(x);
        ny += norm2(y);
        xx = xx + x * x;
        yy = yy + y * y;
        xy = xy + x * y;
        ov = ov + conj(x) * y;
    }
    const float n = nx + ny;
    const float i1 = norm2(xx + yy);
    const float i2 = n * n;
    const float i3 = nx * nx + ny * ny + 2.0f * (ov * ov).re;
    const float i4 = nx * nx + ny * ny + 2.0f * norm2(ov);
    const float i5 = norm2(xx) + norm2(yy) + 2.0f * norm2(xy);
    const float dip = norm2(psi[0] + psi[3]) + norm2(psi[0]) + norm2(psi[3]) + 2.0f * (psi[1] * conj(psi[2])).re -
                      (float)(2.0 / 3.0) * n;
    return -2.0f * n + beta[0] * i1 + beta[1] * i2 + beta[2] * i3 + beta[3] * i4 + beta[4] * i5 + g_d * dip;
}

// The six neighbour cells a visit reads: the four nearest and the far
// corners (i-1, j+1), (i+1, j-1) of the site's three forward gradient cells.
struct He3Nbrs {
    const He3Cell *R, *U, *Lf, *D, *LU, *DR;  // (i+1,j) (i,j+1) (i-1,j) (i,j-1) (i-1,j+1) (i+1,j-1)
};

// Component mu of the exact change of the three gradient cells containing
// the site when it moves by (ex, ey) from (x, y) (models/he3/update.py:95-175):
//   2 Re(conj(ex) fx + conj(ey) fy) + 8 (|ex|^2 + |ey|^2) + 4 Re(conj(ex) ey)
// with fx, fy from neighbour differences (small in an ordered state, so
// little is lost to cancellation).  fx - 8x - 2y and fy - 2x - 8y are the
// neighbour field of the conditional Gaussian proposal
// (gaussian_fast.py:26-39): one set of neighbour reads serves both.
struct He3Grad {
    c32 fx, fy;
};

__device__ __forceinline__ He3Grad he3_grad_terms(const He3Nbrs &n, int kx, int ky, c32 x, c32 y)
{
    const c32 a = n.R->z[kx] - x, b = n.R->z[ky] - y, c = n.U->z[kx] - x, d = n.U->z[ky] - y;
    const c32 al = x - n.Lf->z[kx], bl = y - n.Lf->z[ky], cl = n.LU->z[kx] - n.Lf->z[kx],
              dl = n.LU->z[ky] - n.Lf->z[ky];
    const c32 ad = n.DR->z[kx] - n.D->z[kx], bd = n.DR->z[ky] - n.D->z[ky], cd = x - n.D->z[kx],
              dd = y - n.D->z[ky];
    He3Grad g;
    g.fx = (-(3.0f * a + b + c + d) + (3.0f * al + dl)) + (cd + bd);
    g.fy = (-(a + b + c + 3.0f * d) + (bl + cl)) + (3.0f * dd + ad);
    return g;
}

__device__ __forceinline__ float he3_grad_change(const He3Grad &g, c32 ex, c32 ey)
{
    const float linear = 2.0f * (conj(ex) * g.fx + conj(ey) * g.fy).re;
    const float quadratic = 8.0f * (norm2(ex) + norm2(ey)) + 4.0f * (conj(ex) * ey).re;
    return linear + quadratic;
}

// Per-replica constants of a window.  The conditional Gaussian's proposal
// widths and density coefficients depend on beta, K, rho and the proposal
// mass only (gaussian_fast.py:57-66), so they are evaluated once per window
// rather than per visit: sp, sm the widths of the (x+y) and (x-y) noise, qp,
// qm the coefficients of the reverse/forward log density ratio, kp = -K/plus,
// km = -K/minus the factors of the neighbour mean.
struct He3Ctx {
    float beta, K, delta, g_d, rho;
    float sp, sm, qp, qm, kp, km;
    float coeff[5];
    long long *nonfinite;  // counters row 2 entry of this replica
};

struct He3Visit {
    ulonglong2 st;
    float dE;
    int accepted;
};

// gaussian_fast.py:42-50 with fast intrinsics: a pair of standard normals.
__device__ __forceinline__ c32 he3_normal_pair(ulonglong2 &st)
{
    float u = mcgb_fast_unit(xoro_next(st));
    if (u <= 0.0f) u = 1.1102230246251565e-16f;
    const float ang = kTwoPi * mcgb_fast_unit(xoro_next(st));
    const float t = -2.0f * __logf(u);
    const float rad = t * rsqrtf(t);
    float sn, cs;
    __sincosf(ang - kPi, &sn, &cs);  // cos(ang) = -cs, sin(ang) = -sn
    return cmk(-rad * cs, -rad * sn);
}

// One visit of one site: every draw, in the reference's order, and the
// decision.  Independent of the colour (the neighbours come as pointers) and
// inlined into each colour's pass: the row-by-row body is short enough for
// the copies to share the instruction cache, and the inlined form ran 9-12 %
// faster than one out-of-line copy, whose call saved and restored the
// caller's live registers around every visit.  The visit walks the three spin rows mu in turn: it
// reads row mu of the six neighbours once, forms the gradient terms, draws
// and forms row mu of the proposal and adds that row's gradient change (and,
// for the Gaussian, its log density ratio), so only one row of neighbour
// values is live at a time.  The draws keep the reference's order, which is
// row by row too.
//   Cartesian (models/he3/update.py:178-227): twelve offsets, then the
//     acceptance uniform; potential change plus the exact gradient change.
//   Conditional Gaussian (gaussian_fast.py:26-119): six Box-Muller pairs, the
//     acceptance uniform; neighbour field, autoregressive proposal, reverse /
//     forward log density ratio, full Hamiltonian change.  Nonfinite log
//     ratios are counted per replica and rejected.
template <bool kGauss>
__device__ __forceinline__ He3Visit he3_visit(const He3Ctx x, const He3Nbrs n, He3Cell *site, ulonglong2 st)
{
    He3Visit out;
    out.accepted = 0;
    out.dE = 0.0f;
    const He3Cell me = *site;
    const float root = 0.7071067811865475f;
    c32 nxt[6];
    float dg = 0.0f, lpr = 0.0f;
#pragma unroll
    for (int mu = 0; mu < 3; ++mu) {
        const int kx = 2 * mu, ky = 2 * mu + 1;
        const c32 xo = me.z[kx], yo = me.z[ky];
        const He3Grad g = he3_grad_terms(n, kx, ky, xo, yo);
        c32 nx, ny;
        if constexpr (!kGauss) {
            const float xr = x.delta * (2.0f * mcgb_fast_unit(xoro_next(st)) - 1.0f);
            const float xi = x.delta * (2.0f * mcgb_fast_unit(xoro_next(st)) - 1.0f);
            const float yr = x.delta * (2.0f * mcgb_fast_unit(xoro_next(st)) - 1.0f);
            const float yi = x.delta * (2.0f * mcgb_fast_unit(xoro_next(st)) - 1.0f);
            nx = cmk(xo.re + xr, xo.im + xi);
            ny = cmk(yo.re + yr, yo.im + yi);
        } else {
            const c32 f0 = g.fx - (8.0f * xo + 2.0f * yo);
            const c32 f1 = g.fy - (2.0f * xo + 8.0f * yo);
            const c32 hp = root * (f0 + f1), hm = root * (f0 - f1);
            const c32 mp = x.kp * hp, mm = x.km * hm;
            const c32 mx = root * (mp + mm), my = root * (mp - mm);
            const c32 zp = x.sp * he3_normal_pair(st);
            const c32 zm = x.sm * he3_normal_pair(st);
            nx = (mx + x.rho * (xo - mx)) + root * (zp + zm);
            ny = (my + x.rho * (yo - my)) + root * (zp - zm);
            const c32 op = (xo - mx) + (yo - my), om = (xo - mx) - (yo - my);
            const c32 np = (nx - mx) + (ny - my), nm = (nx - mx) - (ny - my);
            lpr += x.qp * (norm2(np) - norm2(op));
            lpr += x.qm * (norm2(nm) - norm2(om));
        }
        dg += he3_grad_change(g, nx - xo, ny - yo);
        nxt[kx] = nx;
        nxt[ky] = ny;
    }
    const float v = mcgb_fast_unit(xoro_next(st));
    out.st = st;
    const float dh = he3_potential_f(nxt, x.coeff, x.g_d) - he3_potential_f(me.z, x.coeff, x.g_d) + x.K * dg;
    if constexpr (!kGauss) {
        if (dh <= 0.0f || v < __expf(-x.beta * dh)) {
#pragma unroll
            for (int k = 0; k < 6; ++k) site->z[k] = nxt[k];
            out.dE = dh;
            out.accepted = 1;
        }
        return out;
    } else {
        const float log_ratio = -x.beta * dh + lpr;
        if (!isfinite(log_ratio)) {
            if (x.nonfinite) atomicAdd(reinterpret_cast<unsigned long long *>(x.nonfinite), 1ull);
            return out;
        }
        if (log_ratio >= 0.0f || v < __expf(log_ratio)) {
#pragma unroll
            for (int k = 0; k < 6; ++k) site->z[k] = nxt[k];
            out.dE = dh;
            out.accepted = 1;
        }
        return out;
    }
}

template <bool kGauss>
struct He3Policy {
    using Args = BatchArgs;
    using Cell = He3Cell;
    static constexpr int kOwnFloats = 0;
    static constexpr int kChannels = 10;
    static constexpr int kSums = 10;  // the last sum is the spin-z density until finish_sample
    // The visit walks one spin row at a time and fits 128 registers without
    // spills, so CTAs of up to 512 threads (16 warps an SM, or two 256-thread
    // CTAs) run the one-plaquette and global-stream variants.  There is no
    // two-plaquette variant (kPairThreads = 0): strips with more plaquettes
    // than threads keep their streams in global memory, whose 32 bytes a
    // visit are small beside the visit's arithmetic.
    static constexpr int kMaxThreads = 512;
    static constexpr int kPairThreads = 0;
    static constexpr bool kSplitMiddle = true;
    static constexpr bool kPipeline = false;  // update<c>: one out-of-line visit
    // Global-stream variant: sites whose visits one thread carries at once.
    static constexpr int kGlobalInFlight = 1;
    static constexpr bool kSmemStreams = false;
    static constexpr bool kEnergyFromDelta = true;
    static constexpr bool kExactEnergy = false;

    // The cell is the site's twelve floats as stored: bulk strip loads.
    static constexpr bool kRefLayout = false;  // colour-major batch arrays
    static constexpr bool kBulkLoad = true;
    static __device__ __forceinline__ const void *bulk_cells(const Args &a) { return a.state; }

    using Ctx = He3Ctx;
    struct Prop {};

    static __device__ __forceinline__ Ctx prepare(const Args &a, int r, const mcgb_replica &, const Walker &wk)
    {
        Ctx x;
        x.beta = wk.beta;
        x.K = a.K;
        x.delta = a.delta;
        x.g_d = a.g_d;
        x.rho = a.rho;
        // gaussian_fast.py:57-66, once per window.
        const float root = 0.7071067811865475f;
        const float plus = 10.0f * a.K + a.mass, minus = 6.0f * a.K + a.mass;
        const float vf = 1.0f - a.rho * a.rho;
        x.sp = sqrtf(vf / (2.0f * x.beta * plus));
        x.sm = sqrtf(vf / (2.0f * x.beta * minus));
        x.qp = vf / (8.0f * root * root * x.sp * x.sp);
        x.qm = vf / (8.0f * root * root * x.sm * x.sm);
        x.kp = -a.K / plus;
        x.km = -a.K / minus;
#pragma unroll
        for (int q = 0; q < 5; ++q) x.coeff[q] = a.coeff[q];
        x.nonfinite = a.counters ? a.counters + 2 * (size_t)a.n_replicas + r : nullptr;
        return x;
    }
    static __device__ __forceinline__ void load(const Args &a, int64_t site, Cell &cell, float *)
    {
        const float4 *p = reinterpret_cast<const float4 *>(static_cast<const float *>(a.state) + 12 * site);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float4 v = p[q];
            cell.z[2 * q] = cmk(v.x, v.y);
            cell.z[2 * q + 1] = cmk(v.z, v.w);
        }
    }
    static __device__ __forceinline__ void store(const Args &a, int64_t site, const Cell &cell, const float *)
    {
        float4 *p = reinterpret_cast<float4 *>(static_cast<float *>(a.state) + 12 * site);
#pragma unroll
        for (int q = 0; q < 3; ++q)
            p[q] = make_float4(cell.z[2 * q].re, cell.z[2 * q].im, cell.z[2 * q + 1].re, cell.z[2 * q + 1].im);
    }
    template <int C_>
    static __device__ __forceinline__ bool update(const Ctx &x, const Nbrs<Cell> &nb, Cell &me, float *,
                                                  ulonglong2 &st, float &dE)
    {
        const He3Nbrs n{&MCGB_NBR(nb, kDown(C_)), &MCGB_NBR(nb, kRight(C_)), &MCGB_NBR(nb, kUp(C_)),
                        &MCGB_NBR(nb, kLeft(C_)), &MCGB_NBR(nb, kUpRight(C_)), &MCGB_NBR(nb, kDownLeft(C_))};
        const He3Visit v = he3_visit<kGauss>(x, n, &me, st);
        st = v.st;
        dE = v.dE;
        return v.accepted != 0;
    }
    template <int C_>
    static __device__ __forceinline__ void measure(const Ctx &x, const Nbrs<Cell> &nb, const Cell &me, const float *,
                                                   FSum *v)
    {
        // models/he3/measure.py:33-60 (energy comes from the running cache);
        // per-site terms in float32, sums compensated.
        const He3Cell &Xp = MCGB_NBR(nb, kDown(C_));   // (i+1, j)
        const He3Cell &Yp = MCGB_NBR(nb, kRight(C_));  // (i, j+1)
        const float K2 = 2.0f * x.K;
#pragma unroll
        for (int mu = 0; mu < 3; ++mu) {
            const c32 X = me.z[2 * mu], Y = me.z[2 * mu + 1];
            const c32 xpx = Xp.z[2 * mu], xpy = Xp.z[2 * mu + 1], ypx = Yp.z[2 * mu], ypy = Yp.z[2 * mu + 1];
            const c32 a = xpx - X, b = xpy - Y, c = ypx - X, d = ypy - Y;
            const float rd = norm2(X) + norm2(Y);
            v[1] += rd;
            if (mu == 2) v[9] += rd;
            v[2] += 2.0f * (conj(X) * Y).im;
            const c32 ph = X * X - Y * Y;
            v[3] += ph.re;
            v[4] += ph.im;
            const c32 A = 3.0f * conj(a) + conj(d), B = conj(b) + conj(c);
            const c32 zx = A * xpx + B * xpy;
            const c32 Cc = conj(c) + conj(b), Dd = 3.0f * conj(d) + conj(a);
            const c32 zy = Cc * ypx + Dd * ypy;
            v[5] += K2 * zx.im;
            v[6] += K2 * ((3.0f * norm2(xpx) + norm2(xpy)) - zx.re);
            v[7] += K2 * zy.im;
            v[8] += K2 * ((norm2(ypx) + 3.0f * norm2(ypy)) - zy.re);
        }
    }
    template <int C_>
    static __device__ __forceinline__ void energy_site(const Ctx &, const Nbrs<Cell> &, const Cell &, const float *,
                                                       FSum &)
    {
    }
    static __device__ __forceinline__ void finish_sample(const Ctx &, double *v)
    {
        v[9] = v[1] == 0.0 ? 0.0 : 0.5 * (3 * v[9] / v[1] - 1);
    }
    static __device__ __forceinline__ double finish_energy(const Ctx &, double e) { return e; }
};

// =============================================================== FP64 energies

template <typename T>
__device__ __forceinline__ const T *cm_site(const T *base, int i, int j, int L, int width)
{
    return base + cm_index(i, j, L) * width;
}

struct c64 {
    double re, im;
};
__device__ __forceinline__ c64 dmk(double a, double b) { return c64{a, b}; }
__device__ __forceinline__ c64 operator+(c64 a, c64 b) { return dmk(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ c64 operator-(c64 a, c64 b) { return dmk(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ c64 operator*(c64 a, c64 b)
{
    return dmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ c64 dconj(c64 a) { return dmk(a.re, -a.im); }
__device__ __forceinline__ double dnorm2(c64 z) { return z.re * z.re + z.im * z.im; }

__device__ double he3_potential_d(const c64 *p, const float *beta, double g_d)
{
    double nx = dnorm2(p[0]), ny = dnorm2(p[1]);
    c64 xx = p[0] * p[0], yy = p[1] * p[1], xy = p[0] * p[1], ov = dconj(p[0]) * p[1];
    for (int mu = 1; mu < 3; ++mu) {
        const c64 x = p[2 * mu], y = p[2 * mu + 1];
        nx += dnorm2(x);
        ny += dnorm2(y);
        xx = xx + x * x;
        yy = yy + y * y;
        xy = xy + x * y;
        ov = ov + dconj(x) * y;
    }
    const double n = nx + ny;
    const double dip = dnorm2(p[0] + p[3]) + dnorm2(p[0]) + dnorm2(p[3]) + 2.0 * (p[1] * dconj(p[2])).re -
                       (2.0 / 3.0) * n;
    return -2.0 * n + beta[0] * dnorm2(xx + yy) + beta[1] * n * n +
           beta[2] * (nx * nx + ny * ny + 2.0 * (ov * ov).re) + beta[3] * (nx * nx + ny * ny + 2.0 * dnorm2(ov)) +
           beta[4] * (dnorm2(xx) + dnorm2(yy) + 2.0 * dnorm2(xy)) + g_d * dip;
}

__device__ __forceinline__ double he3_gradient_d(c64 a, c64 b, c64 c, c64 d)
{
    return 3.0 * (dnorm2(a) + dnorm2(d)) + dnorm2(b) + dnorm2(c) + 2.0 * (dconj(a) * d + dconj(b) * c).re;
}

struct Coeff5f {
    float b[5];
};

__global__ void batch_energy64_continuum(int model, const void *state, const mcgb_replica *table, float J, float K,
                                         float g_d, Coeff5f coeff, float *e_run, double *energies, double *drift)
{
    __shared__ double scratch[32];
    const int r = blockIdx.x;
    const mcgb_replica rep = table[r];
    const int L = rep.L;
    double v[1] = {0.0};
    for (int k = threadIdx.x; k < L * L; k += blockDim.x) {
        const int i = k / L, j = k - i * L;
        const int id = i + 1 == L ? 0 : i + 1, jr = j + 1 == L ? 0 : j + 1;
        if (model == MCGB_MODEL_KAWAMURA || model == MCGB_MODEL_KAWAMURA_GAUSS) {
            const float *b = static_cast<const float *>(state) + 5 * rep.state_offset;
            const float *a = cm_site(b, i, j, L, 5);
            const float *nbs[2] = {cm_site(b, id, j, L, 5), cm_site(b, i, jr, L, 5)};
            for (int q = 0; q < 2; ++q) {
                const float *n = nbs[q];
                const double dot = (double)a[2] * n[2] + (double)a[3] * n[3] + (double)a[4] * n[4];
                v[0] -= (double)J * (1.0 + (double)a[1] * n[1]) * dot * cos((double)a[0] - (double)n[0]);
            }
        } else {
            const float *b = static_cast<const float *>(state) + 12 * rep.state_offset;
            const float *a = cm_site(b, i, j, L, 12);
            const float *xp = cm_site(b, id, j, L, 12);
            const float *yp = cm_site(b, i, jr, L, 12);
            c64 p[6];
            for (int q = 0; q < 6; ++q) p[q] = dmk(a[2 * q], a[2 * q + 1]);
            v[0] += he3_potential_d(p, coeff.b, g_d);
            for (int mu = 0; mu < 3; ++mu) {
                const c64 x = p[2 * mu], y = p[2 * mu + 1];
                const c64 ga = dmk(xp[4 * mu], xp[4 * mu + 1]) - x, gb = dmk(xp[4 * mu + 2], xp[4 * mu + 3]) - y;
                const c64 gc = dmk(yp[4 * mu], yp[4 * mu + 1]) - x, gd = dmk(yp[4 * mu + 2], yp[4 * mu + 3]) - y;
                v[0] += (double)K * he3_gradient_d(ga, gb, gc, gd);
            }
        }
    }
    block_sum<1>(v, scratch);
    if (threadIdx.x == 0) {
        const double e = v[0];
        if (drift) drift[r] = ((double)e_run[2 * r] + (double)e_run[2 * r + 1]) - e;
        const float hi = (float)e;
        e_run[2 * r] = hi;
        e_run[2 * r + 1] = (float)(e - (double)hi);
        energies[r] = e;
    }
}

// =============================================================== dispatch

// Both register variants are compiled for kMaxThreads threads per CTA; the
// two-plaquette variant serves strips of up to 2 * threads plaquettes.
template <class M>
int continuum_launch(const BatchArgs &a, const mcgb_batch_window &w, cudaStream_t s, const char *name)
{
    return launch_any<M>(a, w, s, name);
}

int continuum_window(int model, const mcgb_batch_window &w, cudaStream_t s, const FusedExchange *fx)
{
    if (int st = validate_window(w)) return st;
    MCGB_REQUIRE((model != MCGB_MODEL_KAWAMURA && model != MCGB_MODEL_KAWAMURA_GAUSS) || w.aux != nullptr,
                 "Kawamura window: null (cos, sin) cache");
    BatchArgs a = make_args(w);
    if (fx != nullptr) a.fx = *fx;
    switch (model) {
    case MCGB_MODEL_KAWAMURA: return continuum_launch<KawamuraPolicy<false>>(a, w, s, "kawamura window");
    case MCGB_MODEL_KAWAMURA_GAUSS:
        return continuum_launch<KawamuraPolicy<true>>(a, w, s, "kawamura gaussian window");
    case MCGB_MODEL_HE3: return continuum_launch<He3Policy<false>>(a, w, s, "he3 window");
    default: return continuum_launch<He3Policy<true>>(a, w, s, "he3 gaussian window");
    }
}

int64_t continuum_smem(int model, int L, int C)
{
    if (model == MCGB_MODEL_KAWAMURA || model == MCGB_MODEL_KAWAMURA_GAUSS)
        return (int64_t)single_smem<KawamuraPolicy<false>>(L, C);
    return (int64_t)single_smem<He3Policy<false>>(L, C);
}

template <class M>
int continuum_clusters(int C, int threads, size_t smem, int *out)
{
    return max_clusters_any<M>(C, threads, smem, out);
}

int continuum_max_clusters(int model, int C, int threads, size_t smem, int *out)
{
    switch (model) {
    case MCGB_MODEL_KAWAMURA: return continuum_clusters<KawamuraPolicy<false>>(C, threads, smem, out);
    case MCGB_MODEL_KAWAMURA_GAUSS: return continuum_clusters<KawamuraPolicy<true>>(C, threads, smem, out);
    case MCGB_MODEL_HE3: return continuum_clusters<He3Policy<false>>(C, threads, smem, out);
    default: return continuum_clusters<He3Policy<true>>(C, threads, smem, out);
    }
}

int continuum_energy64(int model, const mcgb_batch_window &w, double *drift, cudaStream_t s)
{
    Coeff5f c;
    for (int q = 0; q < 5; ++q) c.b[q] = w.coefficients[q];
    batch_energy64_continuum<<<w.n_replicas, 256, 0, s>>>(model, w.state, w.table, w.J, w.K, w.g_d, c, w.e_run,
                                                          w.energies, drift);
    return check_launch("batch_energy64_continuum");
}

}  // namespace mcgb
