// The window kernel skeleton of the batched engine, shared by every model.
//
// window_kernel<M, NPMAX> runs `n_sweeps` sweeps on every replica of a batch.
// Cluster k processes replicas work_idx[work_ptr[k] .. work_ptr[k+1]); for
// each, its C CTAs load their strips (colour-major planes) into shared
// memory, keep each thread's RNG streams in registers when the strip has at
// most NPMAX plaquettes per thread (otherwise the streams stay in global
// memory, where the window's reuse keeps them in L2), and run the sweeps:
// colour 0, cluster barrier, colours 1 and 2 together (they share no bond),
// barrier, colour 3, barrier -- the visit order of four sequential colour
// launches, since every site draws from its own stream.  Models whose sites
// couple colours 1 and 2 (He3's diagonal gradient cells) set kSplitMiddle and
// get a barrier between them.  Samples due inside the window are reduced
// over the cluster and written in temperature order.  At the end the
// accepted energy changes update the replica's compensated running energy.
//
// Policy M supplies: Args (with the common fields below), Cell (the
// per-site shared-memory record neighbours read), kOwnFloats (extra
// per-site floats only the owner reads), kChannels, kSplitMiddle, and
//   Ctx  prepare(const Args&, int r, const mcgb_replica&)
//   void load(const Args&, int64_t site, Cell&, float* own)
//   void store(const Args&, int64_t site, const Cell&, const float* own)
//   bool update<c>(const Ctx&, Nbrs, Cell&, float* own, ulonglong2&, float& dE)
//   void measure<c>(const Ctx&, Nbrs, const Cell&, const float* own, double* v)
//   void finish_sample(const Ctx&, double* v)  (channel 0 holds the energy)
// and two flags: kEnergyFromDelta (channel 0 = running energy + accepted
// changes; else measure<c> accumulates it) and kExactEnergy (the epilogue
// recomputes the energy exactly with energy_site<c>/finish_energy instead of
// adding the accepted changes to the running energy).
#pragma once

#include "batch_common.cuh"

namespace mcgb {

// Neighbour accessor handed to the policies.
template <typename Cell>
struct Nbrs {
    Cell *planes;
    Strip g;
    int pr, pc;

    __device__ __forceinline__ const Cell &at(NbrSpec s) const { return *nbr_ptr(planes, g, s, pr, pc); }
};

struct WindowCommon {
    const mcgb_replica *table;
    const int32_t *work_ptr;
    const int32_t *work_idx;
    void *rng;             // colour-major ulonglong2 per site
    const float *betas;    // per replica (walker order)
    const int32_t *w2t;    // per replica: temperature slot within its ladder
    float *e_run;          // 2 per replica: compensated running energy (hi, lo)
    double *energies;      // out: per replica, hi + lo after the window
    long long *accepted;   // per replica, += accepted moves
    double *samples;       // [n_slots][kChannels][n_temps_total] or null
    double *staging;       // [kChannels][n_replicas]: window-end sample, walker order
    int n_temps_total;
    int n_slots;
    const long long *clock; // device {sweeps completed, exchange rounds}
    long long first_sample_sweep;
    int sample_interval;
    int n_sweeps;
};

constexpr int kRedDoubles = 16;  // per-CTA cluster reduction slots

template <class M>
__host__ __device__ constexpr size_t cell_bytes()
{
    return sizeof(typename M::Cell) + sizeof(float) * M::kOwnFloats;
}

template <class M>
__host__ __device__ inline size_t window_smem_bytes(int max_npl)
{
    return sizeof(double) * (kRedDoubles + 32 * (M::kChannels + 2)) + (size_t)4 * max_npl * cell_bytes<M>();
}

template <class M, int NPMAX, int C_>
__device__ __forceinline__ void colour_pass(const typename M::Args &a, const typename M::Ctx &ctx,
                                            cg::cluster_group &cluster, typename M::Cell *cells,
                                            float *own, const Strip &g, ulonglong2 (&st)[NPMAX > 0 ? NPMAX : 1][4],
                                            bool regs, int64_t base, int64_t gplane, float &dsum,
                                            float &dcomp, int &nacc)
{
    const int T = blockDim.x;
    ulonglong2 *rng_g = static_cast<ulonglong2 *>(a.c.rng);
    if (regs) {
#pragma unroll
        for (int k = 0; k < NPMAX; ++k) {
            const int p = threadIdx.x + k * T;
            if (p < g.NPL) {
                Nbrs<typename M::Cell> nb{cells, g, p / g.LP, p % g.LP};
                float dE;
                if (M::template update<C_>(ctx, nb, cells[C_ * g.NPL + p], own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats,
                                           st[k][C_], dE)) {
                    comp_add(dsum, dcomp, dE);
                    ++nacc;
                }
            }
        }
    } else {
        for (int p = threadIdx.x; p < g.NPL; p += T) {
            const int64_t idx = base + C_ * gplane + p;
            ulonglong2 s = rng_g[idx];
            Nbrs<typename M::Cell> nb{cells, g, p / g.LP, p % g.LP};
            float dE;
            if (M::template update<C_>(ctx, nb, cells[C_ * g.NPL + p], own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats,
                                       s, dE)) {
                comp_add(dsum, dcomp, dE);
                ++nacc;
            }
            rng_g[idx] = s;
        }
    }
}

template <class M, int C_>
__device__ __forceinline__ void measure_colour(const typename M::Ctx &ctx, cg::cluster_group &cluster,
                                               typename M::Cell *cells, float *own, const Strip &g,
                                               double *v)
{
    for (int p = threadIdx.x; p < g.NPL; p += blockDim.x) {
        Nbrs<typename M::Cell> nb{cells, g, p / g.LP, p % g.LP};
        M::template measure<C_>(ctx, nb, cells[C_ * g.NPL + p], own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats, v);
    }
}

template <class M, int C_>
__device__ __forceinline__ void energy_colour(const typename M::Ctx &ctx, cg::cluster_group &cluster,
                                              typename M::Cell *cells, float *own, const Strip &g, double &e)
{
    for (int p = threadIdx.x; p < g.NPL; p += blockDim.x) {
        Nbrs<typename M::Cell> nb{cells, g, p / g.LP, p % g.LP};
        M::template energy_site<C_>(ctx, nb, cells[C_ * g.NPL + p], own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats, e);
    }
}

// Threads per block the NPMAX variant is compiled for: NPMAX streams of four
// colours live in registers (16 registers per plaquette).
template <int NPMAX>
constexpr int window_max_threads()
{
    return NPMAX <= 1 ? 1024 : 512;
}

template <class M, int NPMAX>
__global__ void __launch_bounds__(window_max_threads<NPMAX>(), 1) window_kernel(const typename M::Args a)
{
    using Cell = typename M::Cell;
    constexpr int NC = M::kChannels;
    cg::cluster_group cluster = cg::this_cluster();
    const int C = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int cid = blockIdx.x / C;
    const int T = blockDim.x, tid = threadIdx.x;

    extern __shared__ __align__(16) unsigned char smem[];
    double *red = reinterpret_cast<double *>(smem);              // kRedDoubles
    double *scratch = red + kRedDoubles;                           // 32 * (NC + 2)
    unsigned char *tail = reinterpret_cast<unsigned char *>(scratch + 32 * (NC + 2));

    const WindowCommon &cm = a.c;
    ulonglong2 *rng_g = static_cast<ulonglong2 *>(cm.rng);

    for (int w = cm.work_ptr[cid]; w < cm.work_ptr[cid + 1]; ++w) {
        const int r = cm.work_idx[w];
        const mcgb_replica rep = cm.table[r];
        Strip g;
        g.L = rep.L;
        g.LP = rep.L >> 1;
        g.HP = rep.L / (2 * C);
        g.NPL = g.HP * g.LP;
        g.rank = rank;
        g.C = C;
        Cell *cells = reinterpret_cast<Cell *>(tail);
        float *own = reinterpret_cast<float *>(cells + 4 * g.NPL);
        const int64_t gplane = (int64_t)g.LP * g.LP;
        const int64_t base = rep.state_offset + (int64_t)rank * g.NPL;

        const typename M::Ctx ctx = M::prepare(a, r, rep);
        for (int c = 0; c < 4; ++c)
            for (int p = tid; p < g.NPL; p += T)
                M::load(a, base + c * gplane + p, cells[c * g.NPL + p], own + (size_t)(c * g.NPL + p) * M::kOwnFloats);

        const bool regs = NPMAX > 0 && g.NPL <= NPMAX * T;
        ulonglong2 st[NPMAX > 0 ? NPMAX : 1][4];
        if (regs) {
#pragma unroll
            for (int k = 0; k < (NPMAX > 0 ? NPMAX : 1); ++k) {
                const int p = tid + k * T;
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (p < g.NPL) st[k][c] = rng_g[base + c * gplane + p];
            }
        }
        const float e_hi0 = cm.e_run[2 * r], e_lo0 = cm.e_run[2 * r + 1];
        const long long sweep0 = cm.clock[0];
        const int tslot = rep.ladder_start + cm.w2t[r];
        cluster.sync();

        float dsum = 0.0f, dcomp = 0.0f;
        int nacc = 0;
        for (int s = 0; s < cm.n_sweeps; ++s) {
            colour_pass<M, NPMAX, 0>(a, ctx, cluster, cells, own, g, st, regs, base, gplane, dsum, dcomp, nacc);
            cluster.sync();
            colour_pass<M, NPMAX, 1>(a, ctx, cluster, cells, own, g, st, regs, base, gplane, dsum, dcomp, nacc);
            if (M::kSplitMiddle) cluster.sync();
            colour_pass<M, NPMAX, 2>(a, ctx, cluster, cells, own, g, st, regs, base, gplane, dsum, dcomp, nacc);
            cluster.sync();
            colour_pass<M, NPMAX, 3>(a, ctx, cluster, cells, own, g, st, regs, base, gplane, dsum, dcomp, nacc);
            cluster.sync();

            const int slot = sample_slot(sweep0 + s + 1, cm.first_sample_sweep, cm.sample_interval, cm.n_slots);
            if (slot >= 0 && cm.samples != nullptr) {
                double v[NC];
#pragma unroll
                for (int q = 0; q < NC; ++q) v[q] = 0.0;
                v[0] = M::kEnergyFromDelta ? (double)dsum + (double)dcomp : 0.0;
                measure_colour<M, 0>(ctx, cluster, cells, own, g, v);
                measure_colour<M, 1>(ctx, cluster, cells, own, g, v);
                measure_colour<M, 2>(ctx, cluster, cells, own, g, v);
                measure_colour<M, 3>(ctx, cluster, cells, own, g, v);
                block_sum<NC>(v, scratch);
                if (tid == 0) {
#pragma unroll
                    for (int q = 0; q < NC; ++q) red[q] = v[q];
                }
                cluster.sync();
                if (rank == 0 && tid == 0) {
                    double tot[NC];
#pragma unroll
                    for (int q = 0; q < NC; ++q) tot[q] = 0.0;
                    for (int k = 0; k < C; ++k) {
                        const double *rr = cluster.map_shared_rank(red, k);
#pragma unroll
                        for (int q = 0; q < NC; ++q) tot[q] += rr[q];
                    }
                    if (M::kEnergyFromDelta) tot[0] += (double)e_hi0 + (double)e_lo0;
                    M::finish_sample(ctx, tot);
                    if (cm.staging != nullptr && s + 1 == cm.n_sweeps) {
                        // The exchange after this window scatters it with the new map.
#pragma unroll
                        for (int q = 0; q < NC; ++q) cm.staging[(size_t)q * a.n_replicas + r] = tot[q];
                    } else {
                        double *out = cm.samples + (size_t)slot * NC * cm.n_temps_total + tslot;
#pragma unroll
                        for (int q = 0; q < NC; ++q) out[(size_t)q * cm.n_temps_total] = tot[q];
                    }
                }
                cluster.sync();
            }
        }

        // Window epilogue: energy and acceptance bookkeeping, write back.
        double v2[3] = {(double)dsum + (double)dcomp, (double)nacc, 0.0};
        if (M::kExactEnergy) {
            energy_colour<M, 0>(ctx, cluster, cells, own, g, v2[2]);
            energy_colour<M, 1>(ctx, cluster, cells, own, g, v2[2]);
            energy_colour<M, 2>(ctx, cluster, cells, own, g, v2[2]);
            energy_colour<M, 3>(ctx, cluster, cells, own, g, v2[2]);
        }
        block_sum<3>(v2, scratch);
        if (tid == 0) {
            red[NC] = v2[0];
            red[NC + 1] = v2[1];
            red[NC + 2] = v2[2];
        }
        for (int c = 0; c < 4; ++c)
            for (int p = tid; p < g.NPL; p += T)
                M::store(a, base + c * gplane + p, cells[c * g.NPL + p], own + (size_t)(c * g.NPL + p) * M::kOwnFloats);
        if (regs) {
#pragma unroll
            for (int k = 0; k < (NPMAX > 0 ? NPMAX : 1); ++k) {
                const int p = tid + k * T;
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (p < g.NPL) rng_g[base + c * gplane + p] = st[k][c];
            }
        }
        cluster.sync();
        if (rank == 0 && tid == 0) {
            double de = 0.0, na = 0.0, ex = 0.0;
            for (int k = 0; k < C; ++k) {
                const double *rr = cluster.map_shared_rank(red, k);
                de += rr[NC];
                na += rr[NC + 1];
                ex += rr[NC + 2];
            }
            float hi, lo2;
            if (M::kExactEnergy) {
                const double e = M::finish_energy(ctx, ex);
                hi = (float)e;
                lo2 = (float)(e - (double)hi);
                cm.energies[r] = e;
            } else {
                // Compensated (hi, lo) float update of the running energy.
                const float de_hi = (float)de;
                const float de_lo = (float)(de - (double)de_hi);
                float s1, e1;
                two_sum(e_hi0, de_hi, s1, e1);
                const float lo = e_lo0 + e1 + de_lo;
                two_sum(s1, lo, hi, lo2);
                cm.energies[r] = (double)hi + (double)lo2;
            }
            cm.e_run[2 * r] = hi;
            cm.e_run[2 * r + 1] = lo2;
            cm.accepted[r] += (long long)na;
        }
        cluster.sync();
    }
}

}  // namespace mcgb
