// Batched-engine policies for the Ising and XY models (mixed precision).
//
// Ising (models/ising/update.py:7-29): int8 spins in shared memory, one RNG
// draw per visit, acceptance `dE <= 0 or u < expf(-beta*dE)` with the five
// possible expf values per replica evaluated once per window with the same
// float32 expf and turned into exact integer thresholds on the raw draw --
// bit-identical to the per-colour kernel.  The window's final energy is the
// exact integer bond count times J.
//
// XY (models/xy/update.py:6-54 and the Gaussian variant): shared memory
// holds (cos, sin) of every angle, so an update evaluates one sincos of the
// proposal instead of eight cosines:
//   dE = -J [ (cos t' - cos t) S_c + (sin t' - sin t) S_s ],
// S_c, S_s the sums over the four neighbours' cached (cos, sin).  Proposal,
// Box-Muller and acceptance use the fast float32 intrinsics and 23-bit
// uniforms; the draw sequence per visit is the oracle's (uniform: u, v;
// Gaussian: u1, u2, v), so the streams stay in step with it.
// Accepted changes accumulate per thread with compensation and update the
// replica's running energy; samples read it instead of re-summing bonds.
#include "batch_args.cuh"

namespace mcgb {

// ================================================================= Ising

struct IsingPolicy {
    using Args = BatchArgs;
    using Cell = int8_t;
    static constexpr int kOwnFloats = 0;
    static constexpr int kChannels = 2;  // energy, magnetization
    static constexpr int kSums = 2;
    static constexpr int kMaxThreads = 1024;
    static constexpr int kPairThreads = 512;
    static constexpr bool kSplitMiddle = false;
    static constexpr bool kPipeline = true;
    // Global-stream variant: sites whose visits one thread carries at once.
    static constexpr int kGlobalInFlight = 2;
    // One plaquette a thread (1024 threads): RNG streams in shared memory.
    static constexpr bool kSmemStreams = true;
    static constexpr bool kEnergyFromDelta = false;
    static constexpr bool kExactEnergy = true;
    // The strip's int8 spins are the global records: bulk strip loads.
    static constexpr bool kRefLayout = false;  // colour-major batch arrays
    static constexpr bool kBulkLoad = true;
    static __device__ __forceinline__ const void *bulk_cells(const Args &a) { return a.state; }

    // u < expf(-beta*dE) for the float32 uniform u of draw x is
    // (x >> 11) < M, with M the integer threshold of that float (exact, see
    // mcgb_unit_threshold); k = 2*s*sum in {-8, -4, 0, 4, 8}.
    struct Ctx {
        unsigned long long m[5];
        float J;
    };
    struct Prop {
        unsigned long long m;  // x >> 11 of the visit's draw
    };

    static __device__ __forceinline__ Ctx prepare(const Args &a, int, const mcgb_replica &, const Walker &wk)
    {
        Ctx x;
        x.J = a.J;
        const float beta = wk.beta;
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            const float dE = (float)(4 * q - 8) * a.J;
            // dE <= 0 accepts every draw: u <= 1 < 2.
            x.m[q] = mcgb_unit_threshold(dE <= 0.0f ? 2.0f : expf(-beta * dE));
        }
        return x;
    }
    static __device__ __forceinline__ void load(const Args &a, int64_t site, Cell &cell, float *)
    {
        cell = static_cast<const int8_t *>(a.state)[site];
    }
    static __device__ __forceinline__ void store(const Args &a, int64_t site, const Cell &cell, const float *)
    {
        static_cast<int8_t *>(a.state)[site] = cell;
    }
    template <int C_>
    static __device__ __forceinline__ Prop propose(const Ctx &, const Cell &, const float *, ulonglong2 &st)
    {
        return Prop{(unsigned long long)(xoro_next(st) >> 11)};
    }
    template <int C_>
    static __device__ __forceinline__ bool decide(const Ctx &x, const Nbrs<Cell> &nb, Cell &me, float *,
                                                  const Prop &pr, float &dE)
    {
        const int s = me;
        const int sum = MCGB_NBR(nb, kUp(C_)) + MCGB_NBR(nb, kDown(C_)) + MCGB_NBR(nb, kLeft(C_)) +
                        MCGB_NBR(nb, kRight(C_));
        const int k = 2 * s * sum;
        dE = (float)k * x.J;
        // Static indices keep the five thresholds in registers.
        unsigned long long t = x.m[0];
        t = k == -4 ? x.m[1] : t;
        t = k == 0 ? x.m[2] : t;
        t = k == 4 ? x.m[3] : t;
        t = k == 8 ? x.m[4] : t;
        if (pr.m < t) {
            me = (int8_t)(-s);
            return true;
        }
        return false;
    }
    template <int C_>
    static __device__ __forceinline__ void measure(const Ctx &, const Nbrs<Cell> &nb, const Cell &me,
                                                   const float *, FSum *v)
    {
        const int s = me;
        v[0] += (float)(s * (MCGB_NBR(nb, kDown(C_)) + MCGB_NBR(nb, kRight(C_))));
        v[1] += (float)s;
    }
    template <int C_>
    static __device__ __forceinline__ void energy_site(const Ctx &, const Nbrs<Cell> &nb, const Cell &me,
                                                       const float *, FSum &e)
    {
        e += (float)(me * (MCGB_NBR(nb, kDown(C_)) + MCGB_NBR(nb, kRight(C_))));
    }
    static __device__ __forceinline__ void finish_sample(const Ctx &x, double *v) { v[0] *= -(double)x.J; }
    static __device__ __forceinline__ double finish_energy(const Ctx &x, double bonds) { return -(double)x.J * bonds; }
};

// ================================================================= XY

struct XYPolicy {
    using Args = BatchArgs;
    using Cell = float2;  // (cos theta, sin theta)
    static constexpr int kOwnFloats = 1;  // theta
    static constexpr int kChannels = 5;   // energy, mx, my, twist_cos_x, twist_sin_x
    static constexpr int kSums = 5;
    static constexpr int kMaxThreads = 1024;
    static constexpr int kPairThreads = 512;
    static constexpr bool kSplitMiddle = false;
    static constexpr bool kPipeline = true;
    // Global-stream variant: sites whose visits one thread carries at once.
    static constexpr int kGlobalInFlight = 2;
    // One plaquette a thread (1024 threads): RNG streams in shared memory.
    static constexpr bool kSmemStreams = true;
    static constexpr bool kEnergyFromDelta = true;
    static constexpr bool kExactEnergy = false;
    // Cells are the (cos, sin) cache and the owner's float the angle, both
    // stored site by site: bulk strip loads.
    static constexpr bool kRefLayout = false;  // colour-major batch arrays
    static constexpr bool kBulkLoad = true;
    static __device__ __forceinline__ const void *bulk_cells(const Args &a) { return a.aux; }
    static __device__ __forceinline__ const float *bulk_own(const Args &a)
    {
        return static_cast<const float *>(a.state);
    }

    struct Ctx {
        float beta, sigma, J, delta;
        bool gauss;
    };
    // Proposal angle, its (cos, sin) and the acceptance uniform.
    struct Prop {
        float tp, cp, sp, v;
    };

    static __device__ __forceinline__ Ctx prepare(const Args &a, int, const mcgb_replica &, const Walker &wk)
    {
        Ctx x;
        x.beta = wk.beta;
        x.J = a.J;
        x.delta = a.delta;
        x.gauss = a.sigma_t != nullptr;
        x.sigma = x.gauss ? wk.sigma : 0.0f;
        return x;
    }
    // The (cos, sin) cache persists in `aux` between windows, so the chain
    // always evaluates the energy of the values its updates computed.
    static __device__ __forceinline__ void load(const Args &a, int64_t site, Cell &cell, float *own)
    {
        own[0] = static_cast<const float *>(a.state)[site];
        cell = a.aux[site];
    }
    static __device__ __forceinline__ void store(const Args &a, int64_t site, const Cell &cell, const float *own)
    {
        static_cast<float *>(a.state)[site] = own[0];
        a.aux[site] = cell;
    }
    // Draws: Gaussian -- one draw, its three visit uniforms (u1, u2, v;
    // mcgb_visit_*); uniform -- u, then the acceptance v (23-bit
    // mcgb_fast_unit in the mixed form).
    template <int C_>
    static __device__ __forceinline__ Prop propose(const Ctx &x, const Cell &, const float *own, ulonglong2 &st)
    {
        const float pi = 3.14159265358979323846f, two_pi = 6.28318530717958647692f;
        const float t = own[0];
        Prop q;
        if (x.gauss) {
            const uint64_t bits = xoro_next(st);
            const float u1 = mcgb_visit_u1(bits), u2 = mcgb_visit_u2(bits);
            q.v = mcgb_visit_v(bits);
            const float t2 = -2.0f * __logf(u1);
            // cos(2 pi u2) = -cos(2 pi u2 - pi), evaluated on [-pi, pi].
            const float z = -(t2 * rsqrtf(t2)) * __cosf(fmaf(two_pi, u2, -pi));
            float tp = fmaf(x.sigma, z, t);
            tp -= two_pi * floorf((tp + pi) * (1.0f / two_pi));
            if (tp >= pi) tp -= two_pi;
            if (tp < -pi) tp += two_pi;
            q.tp = tp;
        } else {
            const float u = mcgb_fast_unit(xoro_next(st));
            float tp = t + x.delta * (2.0f * u - 1.0f);
            if (tp >= pi) tp -= two_pi;
            else if (tp < -pi) tp += two_pi;
            q.tp = tp;
            q.v = mcgb_fast_unit(xoro_next(st));
        }
        __sincosf(q.tp, &q.sp, &q.cp);
        return q;
    }
    template <int C_>
    static __device__ __forceinline__ bool decide(const Ctx &x, const Nbrs<Cell> &nb, Cell &me, float *own,
                                                  const Prop &q, float &dE)
    {
        const float2 a = MCGB_NBR(nb, kUp(C_)), b = MCGB_NBR(nb, kDown(C_));
        const float2 c = MCGB_NBR(nb, kLeft(C_)), d = MCGB_NBR(nb, kRight(C_));
        const float sc = (a.x + b.x) + (c.x + d.x);
        const float ss = (a.y + b.y) + (c.y + d.y);
        dE = -x.J * ((q.cp - me.x) * sc + (q.sp - me.y) * ss);
        if (dE <= 0.0f || q.v < __expf(-x.beta * dE)) {
            own[0] = q.tp;
            me = make_float2(q.cp, q.sp);
            return true;
        }
        return false;
    }
    template <int C_>
    static __device__ __forceinline__ void measure(const Ctx &, const Nbrs<Cell> &nb, const Cell &me,
                                                   const float *, FSum *v)
    {
        const float2 dn = MCGB_NBR(nb, kDown(C_));
        v[1] += me.x;
        v[2] += me.y;
        v[3] += me.x * dn.x + me.y * dn.y;
        v[4] += me.y * dn.x - me.x * dn.y;
    }
    template <int C_>
    static __device__ __forceinline__ void energy_site(const Ctx &, const Nbrs<Cell> &, const Cell &,
                                                       const float *, FSum &)
    {
    }
    static __device__ __forceinline__ void finish_sample(const Ctx &, double *) {}
    static __device__ __forceinline__ double finish_energy(const Ctx &, double e) { return e; }
};

// ================================================================= reference layout
//
// The drop-in Runtime keeps the reference's arrays: (R, L, L) states and
// one stream per site at r*L*L + i*L + j.  These policies run the window
// kernel directly on them (strips gathered into colour planes on load,
// scattered back on write-back), so Simulation runs of the built-in Ising
// and XY (uniform proposal) models do a whole run of sweeps in one launch
// with the strip on chip, bit-identical to four update_color launches a
// sweep: Ising's window decision is already bit-identical to
// ising_phase_kernel, and XY's uses the same xy_ref_propose/xy_ref_accept
// as xy_color_kernel.  Windows only: no samples, no fused exchange.

struct IsingRefPolicy : IsingPolicy {
    static constexpr bool kRefLayout = true;
    static constexpr bool kBulkLoad = false;
};

// models/xy/update.py:6-54 on the angles themselves (the cell is theta).
struct XYRefPolicy {
    using Args = BatchArgs;
    using Cell = float;
    static constexpr int kOwnFloats = 0;
    static constexpr int kChannels = 5;
    static constexpr int kSums = 5;
    static constexpr int kMaxThreads = 1024;
    static constexpr int kPairThreads = 512;
    static constexpr bool kSplitMiddle = false;
    static constexpr bool kPipeline = true;
    static constexpr int kGlobalInFlight = 1;
    static constexpr bool kSmemStreams = true;
    static constexpr bool kEnergyFromDelta = true;
    static constexpr bool kExactEnergy = false;
    static constexpr bool kRefLayout = true;
    static constexpr bool kBulkLoad = false;

    struct Ctx {
        float beta, J, delta;
    };
    struct Prop {
        float tp, v;
    };

    static __device__ __forceinline__ Ctx prepare(const Args &a, int, const mcgb_replica &, const Walker &wk)
    {
        return Ctx{wk.beta, a.J, a.delta};
    }
    static __device__ __forceinline__ void load(const Args &a, int64_t site, Cell &cell, float *)
    {
        cell = static_cast<const float *>(a.state)[site];
    }
    static __device__ __forceinline__ void store(const Args &a, int64_t site, const Cell &cell, const float *)
    {
        static_cast<float *>(a.state)[site] = cell;
    }
    template <int C_>
    static __device__ __forceinline__ Prop propose(const Ctx &x, const Cell &me, const float *, ulonglong2 &st)
    {
        Prop q;
        q.tp = xy_ref_propose(me, st, x.delta, q.v);
        return q;
    }
    template <int C_>
    static __device__ __forceinline__ bool decide(const Ctx &x, const Nbrs<Cell> &nb, Cell &me, float *,
                                                  const Prop &q, float &dE)
    {
        if (xy_ref_accept(me, q.tp, q.v, MCGB_NBR(nb, kUp(C_)), MCGB_NBR(nb, kDown(C_)), MCGB_NBR(nb, kLeft(C_)),
                          MCGB_NBR(nb, kRight(C_)), x.beta, x.J, dE)) {
            me = q.tp;
            return true;
        }
        return false;
    }
    // Samples are not taken in this layout (the drop-in classes measure with
    // their own kernels); the sums below keep the skeleton complete.
    template <int C_>
    static __device__ __forceinline__ void measure(const Ctx &, const Nbrs<Cell> &nb, const Cell &me,
                                                   const float *, FSum *v)
    {
        const float dn = MCGB_NBR(nb, kDown(C_));
        float s, c, sd, cd;
        __sincosf(me, &s, &c);
        __sincosf(me - dn, &sd, &cd);
        v[1] += c;
        v[2] += s;
        v[3] += cd;
        v[4] += sd;
    }
    template <int C_>
    static __device__ __forceinline__ void energy_site(const Ctx &, const Nbrs<Cell> &, const Cell &,
                                                       const float *, FSum &)
    {
    }
    static __device__ __forceinline__ void finish_sample(const Ctx &, double *) {}
    static __device__ __forceinline__ double finish_energy(const Ctx &, double e) { return e; }
};

// ================================================================= FP64 energies

// Site (i, j) of a colour-major replica.
template <typename T>
__device__ __forceinline__ const T &cm_at(const T *base, int i, int j, int L)
{
    return base[cm_index(i, j, L)];
}

// Exact total energy of each replica (one block per replica), float64.
// model: 0 Ising (integer bond count times J), 1 XY (float64 cos).
__global__ void batch_energy64_kernel(int model, const void *state, const mcgb_replica *table, float J,
                                      float *e_run, double *energies, double *drift)
{
    __shared__ double scratch[32];
    const int r = blockIdx.x;
    const mcgb_replica rep = table[r];
    const int L = rep.L;
    double v[1] = {0.0};
    for (int k = threadIdx.x; k < L * L; k += blockDim.x) {
        const int i = k / L, j = k - i * L;
        const int id = i + 1 == L ? 0 : i + 1, jr = j + 1 == L ? 0 : j + 1;
        if (model == MCGB_MODEL_ISING) {
            const int8_t *b = static_cast<const int8_t *>(state) + rep.state_offset;
            v[0] += (double)(cm_at(b, i, j, L) * (cm_at(b, id, j, L) + cm_at(b, i, jr, L)));
        } else {
            const float *b = static_cast<const float *>(state) + rep.state_offset;
            const double t = cm_at(b, i, j, L);
            v[0] += -(double)J * (cos(t - (double)cm_at(b, id, j, L)) + cos(t - (double)cm_at(b, i, jr, L)));
        }
    }
    block_sum<1>(v, scratch);
    if (threadIdx.x == 0) {
        const double e = model == MCGB_MODEL_ISING ? -(double)J * v[0] : v[0];
        if (drift) drift[r] = ((double)e_run[2 * r] + (double)e_run[2 * r + 1]) - e;
        const float hi = (float)e;
        e_run[2 * r] = hi;
        e_run[2 * r + 1] = (float)(e - (double)hi);
        energies[r] = e;
    }
}

// The (cos, sin) cache from the angles, with the intrinsic the updates use
// when they store an accepted angle's pair: the cache is a function of the
// angles alone, so rebuilding it reproduces the evolved cache bit for bit.
__global__ void refresh_aux_kernel(const float *state, float2 *aux, int64_t n, int stride)
{
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    float sn, cs;
    __sincosf(state[k * stride], &sn, &cs);
    aux[k] = make_float2(cs, sn);
}

int refresh_aux(const mcgb_batch_window &w, int stride, cudaStream_t s)
{
    MCGB_REQUIRE(w.aux && w.state && w.host_table && w.n_replicas >= 1, "refresh_aux: null pointer");
    const mcgb_replica &last = w.host_table[w.n_replicas - 1];
    const int64_t n = last.state_offset + (int64_t)last.L * last.L;
    refresh_aux_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<const float *>(w.state),
                                                                    static_cast<float2 *>(w.aux), n, stride);
    return check_launch("refresh_aux_kernel");
}

int lattice_window(int model, const mcgb_batch_window &w, cudaStream_t s, const FusedExchange *fx)
{
    if (model == MCGB_MODEL_XY) MCGB_REQUIRE(w.aux != nullptr, "XY window: null (cos, sin) cache");
    if (model == MCGB_MODEL_ISING_REF || model == MCGB_MODEL_XY_REF)
        MCGB_REQUIRE(fx == nullptr && w.samples == nullptr,
                     "reference-layout window: no samples and no fused exchange");
    if (int st = validate_window(w)) return st;
    BatchArgs a = make_args(w);
    if (fx != nullptr) a.fx = *fx;
    switch (model) {
    case MCGB_MODEL_ISING: return launch_any<IsingPolicy>(a, w, s, "ising window");
    case MCGB_MODEL_ISING_REF: return launch_any<IsingRefPolicy>(a, w, s, "ising reference-layout window");
    case MCGB_MODEL_XY_REF: return launch_any<XYRefPolicy>(a, w, s, "xy reference-layout window");
    default: return launch_any<XYPolicy>(a, w, s, "xy window");
    }
}

int64_t lattice_smem(int model, int L, int C)
{
    switch (model) {
    case MCGB_MODEL_ISING: return (int64_t)single_smem<IsingPolicy>(L, C);
    case MCGB_MODEL_ISING_REF: return (int64_t)single_smem<IsingRefPolicy>(L, C);
    case MCGB_MODEL_XY_REF: return (int64_t)single_smem<XYRefPolicy>(L, C);
    default: return (int64_t)single_smem<XYPolicy>(L, C);
    }
}

int lattice_max_clusters(int model, int C, int threads, size_t smem, int *out)
{
    switch (model) {
    case MCGB_MODEL_ISING: return max_clusters_any<IsingPolicy>(C, threads, smem, out);
    case MCGB_MODEL_ISING_REF: return max_clusters_any<IsingRefPolicy>(C, threads, smem, out);
    case MCGB_MODEL_XY_REF: return max_clusters_any<XYRefPolicy>(C, threads, smem, out);
    default: return max_clusters_any<XYPolicy>(C, threads, smem, out);
    }
}

int lattice_energy64(int model, const mcgb_batch_window &w, double *drift, cudaStream_t s)
{
    batch_energy64_kernel<<<w.n_replicas, 256, 0, s>>>(model, w.state, w.table, w.J, w.e_run, w.energies, drift);
    return check_launch("batch_energy64_kernel");
}

}  // namespace mcgb
