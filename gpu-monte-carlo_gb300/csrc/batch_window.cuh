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
// get a barrier between them.  The others, whose colours 0 and 3 share no
// bond either, run colour 0 of the next sweep in the colour-3 phase within a
// window (two barriers a sweep instead of three).  A sample due after a sweep is measured by
// every CTA, reduced over the CTA in compensated float32 and pushed into
// rank 0's shared memory before the barrier that ends the sweep; one warp of
// rank 0 combines the partial sums after the next wait and writes the sample
// in temperature order (or stages it for the exchange when it falls on the
// window's last sweep).  With a FusedExchange the same launch also runs the
// replica exchange, pair by pair as both walkers of a pair finish
// (pair_finished), and advances the device clock.
//
// Halo rows.  Each colour plane of a strip is stored with one halo row above
// and one below, so every neighbour read is a local shared-memory load at a
// compile-time offset.  Only two halos are ever read: planes 2 and 3 (odd
// rows) are read one plaquette row above the strip, planes 0 and 1 (even
// rows) one row below.  When a thread accepts a move on its strip's last
// plaquette row of plane 2/3 it also stores the new cell into the top halo of
// the CTA below (DSMEM store); on the first row of plane 0/1, into the bottom
// halo of the CTA above.  The cluster barrier that ends the phase publishes
// those stores.  With C = 1 the neighbour CTA is the CTA itself.
//
// Pipelining across barriers.  An update is split into propose<c> (every
// random draw of the visit, in the reference's draw order, and whatever
// depends only on the site's own value) and decide<c> (neighbour reads,
// energy change, acceptance).  The cluster barrier is split into arrive and
// wait: a thread arrives after deciding a colour, proposes its next colour's
// moves, then waits, so the barrier latency hides behind independent work.
//
// Policy M supplies: Args (with the common fields below), Cell (the
// per-site shared-memory record neighbours read), kOwnFloats (extra
// per-site floats only the owner reads), kChannels, kSplitMiddle, Prop (the
// per-visit proposal), and
//   Ctx  prepare(const Args&, int r, const mcgb_replica&, const Walker&)  (the walker's
//        beta, proposal width and slot for the window)
//   void load(const Args&, int64_t site, Cell&, float* own)
//   void store(const Args&, int64_t site, const Cell&, const float* own)
//   Prop propose<c>(const Ctx&, const Cell&, const float* own, ulonglong2&)
//   bool decide<c>(const Ctx&, Nbrs, Cell&, float* own, const Prop&, float& dE)
// or, with kPipeline = false (no propose/decide split: every phase waits
// first, then each visit draws and decides in one call),
//   bool update<c>(const Ctx&, Nbrs, Cell&, float* own, ulonglong2&, float& dE)
//   void measure<c>(const Ctx&, Nbrs, const Cell&, const float* own, FSum* v)
//   void finish_sample(const Ctx&, double* v)  (turns kSums reduced sums, sum 0
//        the energy, into the kChannels output channels, in place)
// and two flags: kEnergyFromDelta (channel 0 = running energy + accepted
// changes; else measure<c> accumulates it) and kExactEnergy (the epilogue
// recomputes the energy exactly with energy_site<c>/finish_energy instead of
// adding the accepted changes to the running energy).
#pragma once

#include "batch_common.cuh"
#include "batch_exchange.cuh"

namespace mcgb {

// Compile-time neighbour specs (plane, dpr, dpc) of colour c.
__host__ __device__ constexpr NbrSpec kUp(int c) { return c < 2 ? NbrSpec{c + 2, -1, 0} : NbrSpec{c - 2, 0, 0}; }
__host__ __device__ constexpr NbrSpec kDown(int c) { return c < 2 ? NbrSpec{c + 2, 0, 0} : NbrSpec{c - 2, 1, 0}; }
__host__ __device__ constexpr NbrSpec kLeft(int c) { return (c & 1) ? NbrSpec{c - 1, 0, 0} : NbrSpec{c + 1, 0, -1}; }
__host__ __device__ constexpr NbrSpec kRight(int c) { return (c & 1) ? NbrSpec{c - 1, 0, 1} : NbrSpec{c + 1, 0, 0}; }
__host__ __device__ constexpr NbrSpec kUpRight(int c)
{
    return c == 0 ? NbrSpec{3, -1, 0} : c == 1 ? NbrSpec{2, -1, 1} : c == 2 ? NbrSpec{1, 0, 0} : NbrSpec{0, 0, 1};
}
__host__ __device__ constexpr NbrSpec kDownLeft(int c)
{
    return c == 0 ? NbrSpec{3, 0, -1} : c == 1 ? NbrSpec{2, 0, 0} : c == 2 ? NbrSpec{1, 1, -1} : NbrSpec{0, 1, 0};
}

// A thread's plaquette in the haloed strip: own row offset o = (pr + 1) * LP,
// rows above/below om/op, column pc and its periodic neighbours pcm/pcp.
struct Site {
    int o, om, op, pc, pcm, pcp;
    int pr;
};

__device__ __forceinline__ Site make_site(int p, int LP)
{
    Site s;
    s.pr = p / LP;
    s.pc = p - s.pr * LP;
    s.o = (s.pr + 1) * LP;
    s.om = s.o - LP;
    s.op = s.o + LP;
    s.pcm = s.pc == 0 ? LP - 1 : s.pc - 1;
    s.pcp = s.pc + 1 == LP ? 0 : s.pc + 1;
    return s;
}

// The plaquettes p, p + step, p + 2 step, ... of a strip with rows of LP:
// (row, column) advanced by additions, without a division per visit.
struct SiteWalk {
    int pr, pc, dq, dr, LP;
    __device__ __forceinline__ SiteWalk(int p, int step, int lp)
        : pr(p / lp), pc(p - (p / lp) * lp), dq(step / lp), dr(step - (step / lp) * lp), LP(lp)
    {
    }
    __device__ __forceinline__ void advance()
    {
        pc += dr;
        pr += dq;
        if (pc >= LP) {
            pc -= LP;
            ++pr;
        }
    }
    __device__ __forceinline__ Site site() const
    {
        Site s;
        s.pr = pr;
        s.pc = pc;
        s.o = (pr + 1) * LP;
        s.om = s.o - LP;
        s.op = s.o + LP;
        s.pcm = pc == 0 ? LP - 1 : pc - 1;
        s.pcp = pc + 1 == LP ? 0 : pc + 1;
        return s;
    }
};

// Neighbour accessor handed to the policies: every read is local.
template <typename Cell>
struct Nbrs {
    const Cell *planes;
    int PS;  // plane stride (HP + 2) * LP
    Site s;

    template <int P, int DR, int DC>
    __device__ __forceinline__ const Cell &get() const
    {
        const int row = DR < 0 ? s.om : (DR > 0 ? s.op : s.o);
        const int col = DC < 0 ? s.pcm : (DC > 0 ? s.pcp : s.pc);
        return planes[P * PS + row + col];
    }
};

// The neighbour of `nb` described by the constexpr NbrSpec `spec`.
#define MCGB_NBR(nb, spec) ((nb).template get<(spec).plane, (spec).dpr, (spec).dpc>())

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
    double *samples;       // ring [n_slots][kChannels][n_temps_total] or null
    double *staging;       // [kChannels][n_replicas]: window-end sample, walker order
    int n_temps_total;
    int n_slots;
    const long long *clock; // device {sweeps completed, exchange rounds}
    long long first_sample_sweep;
    int sample_interval;
    int n_sweeps;
    int cluster_size;       // the launch shape the work lists were built for:
    int n_clusters;         // a launch of another shape runs nothing (see below)
};

constexpr int kRedDoubles = 16;  // per-CTA cluster reduction slots
constexpr int kMaxCluster = 16;  // CTAs per cluster (non-portable maximum)

// Partial sums a CTA pushes into rank 0: a sample's kSums, then the window
// epilogue's three (energy change, acceptances, exact energy) in slots of
// their own -- the epilogue's pushes may land while rank 0 still merges the
// window's last sample.
template <class M>
__host__ __device__ constexpr int part_slots()
{
    return M::kSums + 3;
}

// A copy of the launch's exchange arguments in shared memory, read once per
// window by the exchange (its lines in the parameter bank go cold over a
// window's sweeps).
constexpr size_t kFusedCopyBytes = (sizeof(FusedExchange) + 15) & ~static_cast<size_t>(15);
// The mbarrier the bulk strip loads complete on (8 bytes, padded to 16).
constexpr size_t kStripBarBytes = 16;

// The walker a window runs: its beta, its proposal width (sigma_t of its
// slot with per-temperature widths, else 0) and its slot in the ladder.
struct Walker {
    float beta, sigma;
    int slot;
};

// What a resident launch carries in each CTA from one window of a replica to
// the next, so that no window starts or ends on a global load: the walker
// after the exchange (written into every CTA of the cluster by rank 0
// before the cluster barrier that ends the window; at a replica's first
// window each CTA's own copy of the walker it loaded), rank 0's running
// energy and acceptance count, and the launch's clock {sweeps, rounds},
// which stands still within a launch.
struct WindowCarry {
    Walker next;
    float e_hi, e_lo;
    long long accepted;
    long long clock0, rounds0;
};
constexpr size_t kCarryBytes = (sizeof(WindowCarry) + 15) & ~static_cast<size_t>(15);
// A launch's sample schedule with no sample due within the launch.
constexpr int kNoSample = 0x3fffffff;
// Sweeps a window may run, and sweeps a launch may run in all (the host
// refuses more), so that the schedule's int countdown -- at most a launch's
// sweeps plus one sample interval -- stays below kNoSample.
constexpr int kMaxWindowSweeps = 1 << 24;
constexpr long long kMaxLaunchSweeps = 1ll << 28;
static_assert(kMaxLaunchSweeps + kMaxWindowSweeps < kNoSample, "sample countdown range");

// The walker of replica r as the device tables hold it.
template <class Args>
__device__ __forceinline__ Walker load_walker(const Args &a, int r, const mcgb_replica &rep)
{
    Walker w;
    w.beta = __ldcg(a.c.betas + r);
    w.slot = __ldcg(a.c.w2t + r);
    w.sigma = a.sigma_t != nullptr ? __ldcg(a.sigma_t + rep.ladder_start + w.slot) : 0.0f;
    return w;
}

// Shared memory of a strip with npl plaquettes in rows of lp (with
// `streams`, also the strip's four colours of RNG streams, 16 B a site).
template <class M>
__host__ __device__ inline size_t window_smem_bytes(long long npl, long long lp, bool streams = false)
{
    return sizeof(double) * (kRedDoubles + 32 * (M::kSums + 3) + kMaxCluster * part_slots<M>()) + kFusedCopyBytes +
           kStripBarBytes + kCarryBytes +
           (size_t)4 * (npl + 2 * lp) * sizeof(typename M::Cell) + 16 +
           (size_t)4 * npl * sizeof(float) * M::kOwnFloats + (streams ? (size_t)4 * npl * 16 + 16 : 0);
}

// The one-plaquette variant (NPMAX = 1, up to 1024 threads, 64 registers)
// of a policy with kSmemStreams keeps the strip's RNG streams in shared
// memory instead of registers: each visit loads its stream and stores it
// back, and the 16 registers the four streams held go to the visit.
template <class M, int NPMAX>
constexpr bool smem_stream_variant()
{
    return NPMAX == 1 && M::kSmemStreams;
}

struct StripCtx {
    int LP, HP, NPL, PS, up, dn;
};

// Global index of plaquette p of colour c in the strip of CTA `rank`:
// colour-major (base + c * gplane + p, base = state_offset + rank * NPL), or,
// for a policy with kRefLayout, the reference layout, site (i, j) of the
// replica at state_offset + i * L + j (streams in the same order).
template <class M>
__device__ __forceinline__ int64_t strip_site(const mcgb_replica &rep, const StripCtx &g, int rank, int64_t base,
                                              int64_t gplane, int c, int p)
{
    if constexpr (M::kRefLayout) {
        const int pr = p / g.LP, pc = p - pr * g.LP;
        const int i = 2 * (rank * g.HP + pr) + (c >> 1), j = 2 * pc + (c & 1);
        return rep.state_offset + (int64_t)i * rep.L + j;
    } else {
        return base + c * gplane + p;
    }
}

// CTAs of a C-CTA cluster that hold a replica of size L: the largest divisor
// of L/2 (the plaquette rows) that does not exceed C.  The other CTAs of the
// cluster hold no rows of that replica and only take part in the barriers,
// so one cluster shape serves every L of a ragged batch.
__host__ __device__ __forceinline__ int effective_cluster(int L, int C)
{
    const int rows = L >> 1;
    for (int c = C; c > 1; --c)
        if (rows % c == 0) return c;
    return 1;
}

// After an accepted move on a boundary plaquette, copy the new cell into the
// halo of the neighbouring CTA that reads it.
template <int C_, typename Cell>
__device__ __forceinline__ void push_halo(Cell *cells, const StripCtx &g, const Site &s, const Cell &v)
{
    if (C_ < 2) {
        if (s.pr == 0) {
            Cell *dst = cells + C_ * g.PS + (g.HP + 1) * g.LP + s.pc;
            *static_cast<Cell *>(__cluster_map_shared_rank(dst, g.up)) = v;
        }
    } else {
        if (s.pr == g.HP - 1) {
            Cell *dst = cells + C_ * g.PS + s.pc;
            *static_cast<Cell *>(__cluster_map_shared_rank(dst, g.dn)) = v;
        }
    }
}

// Split cluster barrier: arrive publishes this thread's shared-memory and
// DSMEM stores (release); wait returns when every thread of the cluster has
// arrived and makes their stores visible (acquire).  Calls must alternate.
__device__ __forceinline__ void cluster_arrive()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait()
{
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// Bulk copies (the Blackwell tensor memory accelerator's untiled form,
// cp.async.bulk) of contiguous strip rows from global into shared memory,
// completing on an mbarrier that counts the bytes.  Addresses and sizes
// must be multiples of 16 bytes.
__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // Make the initialisation visible to the async proxy (the copies).
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_addr(dst)),
        "l"(static_cast<unsigned long long>(__cvta_generic_to_global(src))), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// Orders this thread's earlier shared-memory accesses (generic proxy) before
// later bulk copies into the same memory (async proxy).
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
__device__ __forceinline__ bool aligned16(const void *p)
{
    return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

// Polls of the strip load's mbarrier before a window gives up (each try_wait
// may itself suspend the thread for a while): far beyond any copy's time.
constexpr long long kStripWaitLimit = 1ll << 22;

// Whether this CTA's strip can arrive by bulk copies: policies whose
// shared-memory records are the global records byte for byte (kBulkLoad:
// M::bulk_cells, and M::bulk_own for the kOwnFloats), each colour's rows one
// contiguous run in both places, every run starting on 16 bytes with a
// length that is a multiple of 16.  Uniform over the CTA.
template <class M, bool SS>
__device__ __forceinline__ bool strip_bulk_ok(const typename M::Args &a, const typename M::Cell *cells,
                                              const float *own, const StripCtx &g, int64_t base, int64_t gplane)
{
    using Cell = typename M::Cell;
    if (g.NPL <= 0) return false;
    const Cell *gc = static_cast<const Cell *>(M::bulk_cells(a));
    bool ok = ((g.NPL * sizeof(Cell)) & 15u) == 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) ok = ok && aligned16(cells + c * g.PS + g.LP) && aligned16(gc + base + c * gplane);
    if constexpr (M::kOwnFloats > 0) {
        const float *go = M::bulk_own(a);
        ok = ok && ((g.NPL * M::kOwnFloats * sizeof(float)) & 15u) == 0;
#pragma unroll
        for (int c = 0; c < 4; ++c)
            ok = ok && aligned16(own + (size_t)c * g.NPL * M::kOwnFloats) &&
                 aligned16(go + (base + c * gplane) * M::kOwnFloats);
    }
    return ok;
}

// The strip by bulk copies: thread 0 issues one copy per colour and array
// (cells, the owner's floats, and with SS the RNG streams) into rows 1..HP of
// each haloed plane, completing on `bar`; every thread waits for the bytes
// (bounded: on giving up, error flag 2 and the window runs on, so no cluster
// barrier is left waiting), then the boundary rows go to the neighbours'
// halos as in the per-thread load.  Before the copies, every thread's earlier
// accesses to these buffers (the previous replica's sweeps and write-back)
// are ordered before the copies' writes by a proxy fence and a CTA barrier.
template <class M, bool SS>
__device__ __forceinline__ void load_strip_bulk(const typename M::Args &a, typename M::Cell *cells, float *own,
                                                ulonglong2 *sst, const StripCtx &g, int64_t base, int64_t gplane,
                                                uint64_t *bar, unsigned &phase, int32_t *error)
{
    using Cell = typename M::Cell;
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned cb = (unsigned)(g.NPL * sizeof(Cell));
        const unsigned ob = (unsigned)(g.NPL * M::kOwnFloats * sizeof(float));
        const unsigned sb = SS ? (unsigned)(g.NPL * sizeof(ulonglong2)) : 0u;
        mbar_arrive_expect_tx(bar, 4u * (cb + ob + sb));
        const Cell *gc = static_cast<const Cell *>(M::bulk_cells(a));
#pragma unroll
        for (int c = 0; c < 4; ++c) bulk_load(cells + c * g.PS + g.LP, gc + base + c * gplane, cb, bar);
        if constexpr (M::kOwnFloats > 0) {
            const float *go = M::bulk_own(a);
#pragma unroll
            for (int c = 0; c < 4; ++c)
                bulk_load(own + (size_t)c * g.NPL * M::kOwnFloats, go + (base + c * gplane) * M::kOwnFloats, ob,
                          bar);
        }
        if constexpr (SS) {
            const ulonglong2 *gr = static_cast<const ulonglong2 *>(a.c.rng);
#pragma unroll
            for (int c = 0; c < 4; ++c) bulk_load(sst + (size_t)c * g.NPL, gr + base + c * gplane, sb, bar);
        }
    }
    for (long long it = 0; !mbar_try_wait(bar, phase); ++it) {
        if (it >= kStripWaitLimit) {
            if (threadIdx.x == 0 && error != nullptr) atomicExch(error, 2);
            break;
        }
    }
    phase ^= 1u;
    for (int q = threadIdx.x; q < g.LP; q += blockDim.x) {
#pragma unroll
        for (int c = 0; c < 2; ++c)
            *static_cast<Cell *>(__cluster_map_shared_rank(cells + c * g.PS + (g.HP + 1) * g.LP + q, g.up)) =
                cells[c * g.PS + g.LP + q];
#pragma unroll
        for (int c = 2; c < 4; ++c)
            *static_cast<Cell *>(__cluster_map_shared_rank(cells + c * g.PS + q, g.dn)) =
                cells[c * g.PS + g.HP * g.LP + q];
    }
}

template <class M, int NK, int C_, bool SS = false>
__device__ __forceinline__ void propose_pass(const typename M::Ctx &ctx, const typename M::Cell *cells,
                                             const float *own, const StripCtx &g, const Site (&sites)[NK],
                                             ulonglong2 (&st)[NK][4], typename M::Prop (&prop)[NK],
                                             ulonglong2 *sst = nullptr)
{
#pragma unroll
    for (int k = 0; k < NK; ++k) {
        const int p = threadIdx.x + k * blockDim.x;
        if (p < g.NPL) {
            const typename M::Cell &me = cells[C_ * g.PS + sites[k].o + sites[k].pc];
            const float *o = own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats;
            if constexpr (SS) {
                // The stream of this site, from and back to shared memory.
                ulonglong2 v = sst[C_ * g.NPL + p];
                prop[k] = M::template propose<C_>(ctx, me, o, v);
                sst[C_ * g.NPL + p] = v;
            } else {
                prop[k] = M::template propose<C_>(ctx, me, o, st[k][C_]);
            }
        }
    }
}

template <class M, int NK, int C_>
__device__ __forceinline__ void decide_pass(const typename M::Ctx &ctx, typename M::Cell *cells, float *own,
                                            const StripCtx &g, const Site (&sites)[NK],
                                            const typename M::Prop (&prop)[NK], float &dacc,
                                            int &nacc)
{
#pragma unroll
    for (int k = 0; k < NK; ++k) {
        const int p = threadIdx.x + k * blockDim.x;
        if (p < g.NPL) {
            const Site &s = sites[k];
            const Nbrs<typename M::Cell> nb{cells, g.PS, s};
            typename M::Cell &me = cells[C_ * g.PS + s.o + s.pc];
            float dE;
            if (M::template decide<C_>(ctx, nb, me, own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats, prop[k], dE)) {
                dacc += dE;
                ++nacc;
                push_halo<C_>(cells, g, s, me);
            }
        }
    }
}

// Strips with more plaquettes than NK per thread keep their streams in
// global memory and run propose + decide per plaquette, with full barriers.
// A colour with the streams in global memory (strips with more plaquettes
// than the register path holds).  Each thread walks its plaquettes with the
// streams of the next two already requested, so the loads overlap with the
// updates instead of each visit waiting on its own.
template <class M, int C_, int IF>
__device__ __forceinline__ void global_rng_pass(const typename M::Args &a, const typename M::Ctx &ctx,
                                                typename M::Cell *cells, float *own, const StripCtx &g,
                                                int64_t base, int64_t gplane, float &dacc, int &nacc)
{
    ulonglong2 *rng_g = static_cast<ulonglong2 *>(a.c.rng) + base + C_ * gplane;
    const int T = blockDim.x;
    const ulonglong2 zero = make_ulonglong2(0, 0);
    int p = threadIdx.x;
    if constexpr (IF == 2) {
        // Two visits at a time (sites p and p + T; sites of a colour never
        // interact and each keeps its own stream, so the order is free):
        // two independent dependency chains, the next pair's streams in
        // flight meanwhile.  Site p + T is touched only when it exists.
        ulonglong2 c0 = p < g.NPL ? rng_g[p] : zero;
        ulonglong2 c1 = p + T < g.NPL ? rng_g[p + T] : zero;
        SiteWalk w0(p, 2 * T, g.LP), w1(p + T, 2 * T, g.LP);
#pragma unroll 1
        for (; p < g.NPL; p += 2 * T, w0.advance(), w1.advance()) {
            const int q = p + T;
            const bool has1 = q < g.NPL;
            const ulonglong2 n0 = p + 2 * T < g.NPL ? rng_g[p + 2 * T] : zero;
            const ulonglong2 n1 = p + 3 * T < g.NPL ? rng_g[p + 3 * T] : zero;
            const Site s0 = w0.site();
            const Site s1 = has1 ? w1.site() : s0;
            float *o0 = own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats;
            float *o1 = own + (size_t)(C_ * g.NPL + (has1 ? q : p)) * M::kOwnFloats;
            typename M::Cell &me0 = cells[C_ * g.PS + s0.o + s0.pc];
            typename M::Cell &me1 = cells[C_ * g.PS + s1.o + s1.pc];
            const typename M::Prop pr0 = M::template propose<C_>(ctx, me0, o0, c0);
            typename M::Prop pr1;
            if (has1) pr1 = M::template propose<C_>(ctx, me1, o1, c1);
            rng_g[p] = c0;
            if (has1) rng_g[q] = c1;
            float dE0, dE1;
            const Nbrs<typename M::Cell> nb0{cells, g.PS, s0};
            if (M::template decide<C_>(ctx, nb0, me0, o0, pr0, dE0)) {
                dacc += dE0;
                ++nacc;
                push_halo<C_>(cells, g, s0, me0);
            }
            if (has1) {
                const Nbrs<typename M::Cell> nb1{cells, g.PS, s1};
                if (M::template decide<C_>(ctx, nb1, me1, o1, pr1, dE1)) {
                    dacc += dE1;
                    ++nacc;
                    push_halo<C_>(cells, g, s1, me1);
                }
            }
            c0 = n0;
            c1 = n1;
        }
        return;
    }
    ulonglong2 cur = p < g.NPL ? rng_g[p] : zero;
    ulonglong2 nx1 = p + T < g.NPL ? rng_g[p + T] : zero;
    SiteWalk walk(p, T, g.LP);
#pragma unroll 1
    for (; p < g.NPL; p += T, walk.advance()) {
        const ulonglong2 nx2 = p + 2 * T < g.NPL ? rng_g[p + 2 * T] : zero;
        ulonglong2 sv = cur;
        const Site s = walk.site();
        float *o = own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats;
        typename M::Cell &me = cells[C_ * g.PS + s.o + s.pc];
        const Nbrs<typename M::Cell> nb{cells, g.PS, s};
        float dE;
        bool accepted;
        if constexpr (M::kPipeline) {
            const typename M::Prop pr = M::template propose<C_>(ctx, me, o, sv);
            rng_g[p] = sv;
            accepted = M::template decide<C_>(ctx, nb, me, o, pr, dE);
        } else {
            accepted = M::template update<C_>(ctx, nb, me, o, sv, dE);
            rng_g[p] = sv;
        }
        if (accepted) {
            dacc += dE;
            ++nacc;
            push_halo<C_>(cells, g, s, me);
        }
        cur = nx1;
        nx1 = nx2;
    }
}

// A colour of a non-pipelined policy (kPipeline = false) with the streams in
// registers: each visit draws and decides in one call, so nothing is held in
// registers across a cluster barrier.
template <class M, int NK, int C_>
__device__ __forceinline__ void fused_pass(const typename M::Ctx &ctx, typename M::Cell *cells, float *own,
                                           const StripCtx &g, const Site (&sites)[NK], ulonglong2 (&st)[NK][4],
                                           float &dacc, int &nacc)
{
#pragma unroll
    for (int k = 0; k < NK; ++k) {
        const int p = threadIdx.x + k * blockDim.x;
        if (p < g.NPL) {
            const Site &s = sites[k];
            const Nbrs<typename M::Cell> nb{cells, g.PS, s};
            typename M::Cell &me = cells[C_ * g.PS + s.o + s.pc];
            float dE;
            if (M::template update<C_>(ctx, nb, me, own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats, st[k][C_],
                                       dE)) {
                dacc += dE;
                ++nacc;
                push_halo<C_>(cells, g, s, me);
            }
        }
    }
}

template <class M, int C_>
__device__ __forceinline__ void measure_colour(const typename M::Ctx &ctx, typename M::Cell *cells, float *own,
                                               const StripCtx &g, FSum *v)
{
    // Long loops (strips of more than two plaquettes per thread) step by
    // additions; short ones divide once per plaquette, fewer in all.
    const bool long_loop = g.NPL > 2 * (int)blockDim.x;
    SiteWalk walk(long_loop ? threadIdx.x : 0, long_loop ? blockDim.x : 1, g.LP);
    for (int p = threadIdx.x; p < g.NPL; p += blockDim.x, walk.advance()) {
        const Site s = long_loop ? walk.site() : make_site(p, g.LP);
        const Nbrs<typename M::Cell> nb{cells, g.PS, s};
        M::template measure<C_>(ctx, nb, cells[C_ * g.PS + s.o + s.pc],
                                own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats, v);
    }
}

template <class M, int C_>
__device__ __forceinline__ void energy_colour(const typename M::Ctx &ctx, typename M::Cell *cells, float *own,
                                              const StripCtx &g, FSum &e)
{
    const bool long_loop = g.NPL > 2 * (int)blockDim.x;
    SiteWalk walk(long_loop ? threadIdx.x : 0, long_loop ? blockDim.x : 1, g.LP);
    for (int p = threadIdx.x; p < g.NPL; p += blockDim.x, walk.advance()) {
        const Site s = long_loop ? walk.site() : make_site(p, g.LP);
        const Nbrs<typename M::Cell> nb{cells, g.PS, s};
        M::template energy_site<C_>(ctx, nb, cells[C_ * g.PS + s.o + s.pc],
                                    own + (size_t)(C_ * g.NPL + p) * M::kOwnFloats, e);
    }
}

// A sample's first half, out of line (it runs once per sample interval and
// would otherwise crowd the sweep loop's instruction cache): measure the
// strip, reduce over the CTA, push the partial sums into rank 0's `parts`.
// With `epilogue` (a sample on the window's last sweep) the same reduction
// carries the window epilogue's three sums -- energy change, acceptances,
// exact energy -- into their slots after the sample's.  The caller arrives
// at the cluster barrier afterwards, which publishes them.
template <class M>
__device__ void window_epilogue_sums(const typename M::Ctx &ctx, typename M::Cell *cells, float *own,
                                     const StripCtx &g, float dsum, float dcomp, int nacc, FSum *v)
{
    v[0].hi = dsum;
    v[0].lo = dcomp;
    v[1].hi = (float)nacc;  // exact: a thread's count is far below 2^24
    if (M::kExactEnergy) {
        energy_colour<M, 0>(ctx, cells, own, g, v[2]);
        energy_colour<M, 1>(ctx, cells, own, g, v[2]);
        energy_colour<M, 2>(ctx, cells, own, g, v[2]);
        energy_colour<M, 3>(ctx, cells, own, g, v[2]);
    }
}

template <class M>
__device__ __noinline__ void push_sample(const typename M::Ctx ctx, typename M::Cell *cells, float *own,
                                         const StripCtx g, float dsum, float dcomp, int nacc, bool epilogue,
                                         float2 *scratch, float2 *parts, int rank)
{
    constexpr int NS = M::kSums;
    FSum v[NS + 3];
    if (M::kEnergyFromDelta) {
        v[0].hi = dsum;
        v[0].lo = dcomp;
    }
    measure_colour<M, 0>(ctx, cells, own, g, v);
    measure_colour<M, 1>(ctx, cells, own, g, v);
    measure_colour<M, 2>(ctx, cells, own, g, v);
    measure_colour<M, 3>(ctx, cells, own, g, v);
    float2 *dst = static_cast<float2 *>(__cluster_map_shared_rank(parts, 0)) + rank * part_slots<M>();
    if (epilogue) {
        window_epilogue_sums<M>(ctx, cells, own, g, dsum, dcomp, nacc, v + NS);
        block_fsum_push<NS + 3>(v, scratch, dst);
    } else {
        const FSum (&w)[NS] = *reinterpret_cast<const FSum (*)[NS]>(v);
        block_fsum_push<NS>(w, scratch, dst);
    }
}

// Warp 0 of the cluster's rank-0 CTA turns the C partial sums of a sample
// (pushed into its `parts` before the barrier that ended the sweep) into the
// sample: lane q merges channel q over the CTAs in rank order, lane 0
// finishes the sample and writes it to the staging row (pend == -2, a sample
// on the window's last sweep, scattered by the exchange) or the ring slot.
template <class M>
__device__ __noinline__ void combine_sample(const typename M::Ctx ctx, const WindowCommon &cm, const float2 *parts,
                                            double *red, int C, int pend, int r, int tslot, float e_hi0,
                                            float e_lo0, int n_replicas)
{
    constexpr int NS = M::kSums, NC = M::kChannels;
    const int lane = threadIdx.x;
    if (lane < NS) {
        FSum f;
        for (int k = 0; k < C; ++k) {
            const float2 q = parts[k * part_slots<M>() + lane];
            f.merge(q.x, q.y);
        }
        red[lane] = f.value();
    }
    __syncwarp();
    if (lane == 0) {
        double tot[NS];
#pragma unroll
        for (int q = 0; q < NS; ++q) tot[q] = red[q];
        if (M::kEnergyFromDelta) tot[0] += (double)e_hi0 + (double)e_lo0;
        M::finish_sample(ctx, tot);
        if (pend == -2) {
#pragma unroll
            for (int q = 0; q < NC; ++q) cm.staging[(size_t)q * n_replicas + r] = tot[q];
        } else {
            double *out = cm.samples + (size_t)pend * NC * cm.n_temps_total + tslot;
#pragma unroll
            for (int q = 0; q < NC; ++q) out[(size_t)q * cm.n_temps_total] = tot[q];
        }
    }
    __syncwarp();
}


// After a cluster's whole work list (thread 0 of its rank-0 CTA): the last
// cluster to finish advances the device clock by the launch's windows (every
// cluster has read it at its start; unless another launch of the same
// windows does) and resets the launch counter.
__device__ __forceinline__ void launch_finished(const FusedExchange &fx, const WindowCommon &cm, int n_clusters)
{
    __threadfence();
    if (atomicAdd(fx.launch_done, 1) == n_clusters - 1) {
        __threadfence();
        if (!fx.hold_clock) {
            long long *clock = const_cast<long long *>(cm.clock);
            clock[0] = __ldcg(clock) + (long long)cm.n_sweeps * fx.n_windows;
            clock[1] = __ldcg(clock + 1) + fx.n_windows;
        }
        *fx.launch_done = 0;
        __threadfence();
    }
}

__device__ __forceinline__ int load_acquire(const int32_t *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Default polls of a pair's decision (each sleeps 32..256 ns) before a wait
// between the windows of a resident launch gives up: ~1 s, far beyond a
// window's length.
constexpr long long kWaitSpinLimit = 1ll << 22;

// 16-byte atomic exchange with acquire-release semantics at GPU scope
// (PTX atom.exch.b128, sm_90 and later): stores (lo, hi) at p, returns the
// previous contents.
__device__ __forceinline__ void exchange16(double2 *p, unsigned long long lo, unsigned long long hi,
                                           unsigned long long &old_lo, unsigned long long &old_hi)
{
    asm volatile(
        "{\n\t.reg .b128 nv, ov;\n\t"
        "mov.b128 nv, {%2, %3};\n\t"
        "atom.acq_rel.gpu.global.exch.b128 ov, [%4], nv;\n\t"
        "mov.b128 {%0, %1}, ov;\n\t}"
        : "=l"(old_lo), "=l"(old_hi)
        : "l"(lo), "l"(hi), "l"(p)
        : "memory");
}

__device__ __forceinline__ void store_release(int32_t *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The exchange acceptance of core/parallel_tempering.py:76-80 for a draw u
// in (0, 1) and log_ratio < 0: log(u) < log_ratio, decided exactly as in
// double precision.  A float logf settles all but a sliver of cases: with
// u rounded to float (relative error 2^-24, so log moves by under 6.0e-8)
// and logf within a few ulp (under 3 * 2^-18 = 1.2e-5 for |log| < 37, the
// range of 53-bit draws), the float result lies within 1e-5 * (1 + |lr|) of
// log(u); only inside that margin is the double log computed.
__device__ __forceinline__ bool exchange_accepts(double u, double log_ratio)
{
    const float lf = logf((float)u);
    const double margin = 1e-5 * (1.0 - log_ratio);
    if ((double)lf < log_ratio - margin) return true;
    if ((double)lf > log_ratio + margin) return false;
    return log(u) < log_ratio;
}

// The fused replica exchange of walker r (slot s, beta b, energy e) of the
// ladder of R slots from global slot `start` (ladder index `ladder`), with
// `fx` the shared-memory copy of the exchange arguments, after
// the window that ends at sweep `sweep`, the exchange round after `rounds`
// earlier ones, with the window-end sample staged for ring slot `slot` (-1:
// none) and `wait` when more windows follow in this launch:
// core/parallel_tempering.py:35-91, decided pair by pair as soon as both
// walkers of a pair are done, so no walker waits for the rest of its
// ladder.  Lane 0 of the walker's rank-0 warp 0 swaps its post into the
// pair's mailbox in one atomic: finding it empty, the walker is first;
// finding the partner's post, it decides with the pair's stream, empties the
// mailbox and writes the swap counters, maps, betas and (released) the
// decision word of both.  Between the windows of a resident launch the first
// walker waits for that word, bounded: on giving up it raises the error flag
// and keeps its slot (the host then reports the launch as failed).  After
// the last window nobody waits: the decider settles both walkers.  A walker
// reaches a pair's next round only after the pair's decision, so the mailbox
// is empty at every round's first arrival, and the word carries the round's
// tag (the exchange-round count + 1).  The other lanes load the walker's
// staged sample and round-trip counters (and the pair's stream) meanwhile;
// settling them at the new slot is then stores.  Decisions, maps, counters,
// round trips and sample slots are exchange_ladder's on the same window.
// Called by the 32 threads of warp 0; kept light in registers, because the
// window kernel keeps its sweep state live across the call.  Returns, on
// every lane, the walker for the next window when `wait` (its slot, its
// beta: its own, the partner's known to the decider, or re-read by a waiter
// whose pair swapped; and the proposal width of the slot, from `sigma_t`
// when not null, both candidates loaded ahead of the decision).
static __device__ __noinline__ Walker pair_finished(const FusedExchange &fx, const float *sigma_t, int start, int R,
                                                    int ladder, int r, int s, float b, double e, long long sweep,
                                                    long long rounds, int slot, bool wait)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const ExchangeArgs &x = fx.ex;
    const int w = r - start, n = x.n_replicas;
    const int parity = R > 2 ? (int)(rounds & 1) : 0;
    int left = -1;
    if (R >= 2) {
        if (s >= parity && ((s - parity) & 1) == 0 && s < R - 1)
            left = s;
        else if (s >= 1 + parity && ((s - 1 - parity) & 1) == 0)
            left = s - 1;
    }
    const int partner = left < 0 ? s : (s == left ? left + 1 : left);
    const int poff = start - ladder;
    const int tag = (int)((rounds + 1) & 0x3fffffff);
    double2 *box = fx.mailbox + start + (left < 0 ? 0 : left);

    // Loads that do not depend on the decision, off lane 0.
    double own = 0.0;  // lane q < channels: channel q of the staged sample
    if (slot >= 0 && lane < x.channels) own = __ldcg(x.staging + (size_t)lane * n + r);
    long long *tr = x.trips + r;
    const bool ends = s == 0 || s == R - 1 || partner == 0 || partner == R - 1;
    long long origin = 0, visited = 0, sweep0 = 0, ntrips = 0, tsweeps = 0;  // lane 1
    if (lane == 1 && ends) {
        origin = __ldcg(tr);
        visited = __ldcg(tr + n);
        sweep0 = __ldcg(tr + 2 * n);
        ntrips = __ldcg(tr + 3 * n);
        tsweeps = __ldcg(tr + 4 * n);
    }
    // The pair's stream (lane 2): its last writer decided the pair's previous
    // round, which this walker's own rounds have ordered before this load.
    ulonglong2 st = make_ulonglong2(0, 0);
    if (lane == 2 && left >= 0) st = __ldcg(x.rng + poff + left);
    // The proposal widths of the walker's slot (lane 4) and its partner's
    // (lane 5): sigma_t does not change within a launch.
    float sg = 0.0f;
    if (sigma_t != nullptr && (lane == 4 || (lane == 5 && left >= 0)))
        sg = __ldcg(sigma_t + start + (lane == 4 ? s : partner));
    // Lane 0 posts; the stream travels to it while the atomic is in flight.
    unsigned long long got_lo = 0, got_hi = 0;
    if (lane == 0 && left >= 0)
        exchange16(box, (unsigned long long)__double_as_longlong(e),
                   (1ull << 63) | ((unsigned long long)(unsigned)w << 32) | __float_as_uint(b), got_lo, got_hi);
    st.x = __shfl_sync(full, st.x, 2);
    st.y = __shfl_sync(full, st.y, 2);

    // walker w ends at slot t0 (-1: unknown) with beta nb; walker w1 (-1:
    // none) at t1
    int t0 = -1, w1 = -1, t1 = -1;
    float nb = b;
    if (lane == 0) {
        if (left < 0) {
            t0 = s;  // no partner this round
        } else if (got_hi >> 63) {
            // Second to arrive: decide.
            const int wq = (int)((got_hi >> 32) & 0x7fffffffu);
            const double eq = __longlong_as_double((long long)got_lo);
            const float bq = __uint_as_float((unsigned)got_hi);
            const bool me_left = s == left;
            const double ea = me_left ? e : eq, eb = me_left ? eq : e;
            const float ba = me_left ? b : bq, bb = me_left ? bq : b;
            const int np = x.n_pairs_total;
            unsigned long long *cnt = reinterpret_cast<unsigned long long *>(x.counts + poff + left);
            int swapped = 0;
            atomicAdd(cnt, 1ull);
            if (!isfinite(ea) || !isfinite(eb)) {
                atomicAdd(cnt + 2 * np, 1ull);
            } else {
                const double log_ratio = ((double)ba - (double)bb) * (ea - eb);
                const double u = xoro_uniform_f64(st);
                x.rng[poff + left] = st;
                if (log_ratio >= 0.0 || u == 0.0 || exchange_accepts(u, log_ratio)) {
                    swapped = 1;
                    atomicAdd(cnt + np, 1ull);
                }
            }
            if (swapped) {
                const int wa = me_left ? w : wq, wb = me_left ? wq : w;
                x.t2w[start + left] = wb;
                x.t2w[start + left + 1] = wa;
                x.w2t[start + wa] = left + 1;
                x.w2t[start + wb] = left;
                x.betas[start + wa] = bb;
                x.betas[start + wb] = ba;
            }
            *box = make_double2(0.0, 0.0);
            store_release(fx.decided + start + left, tag << 1 | swapped);
            t0 = swapped ? partner : s;
            if (swapped) nb = bq;
            if (!wait) {
                w1 = wq;
                t1 = swapped ? s : partner;
            }
        } else if (wait) {
            unsigned ns = 32;
            for (long long it = 0;; ++it) {
                if (it >= fx.wait_limit) {
                    atomicExch(fx.error, 1);
                    break;
                }
                const int v = load_acquire(fx.decided + start + left);
                if ((v >> 1) == tag) {
                    t0 = (v & 1) ? partner : s;
                    // The decider wrote the swapped betas before its release.
                    if (v & 1) nb = __ldcg(x.betas + r);
                    break;
                }
                __nanosleep(ns);
                if (ns < 256) ns <<= 1;
            }
        }
    }
    t0 = __shfl_sync(full, t0, 0);
    w1 = __shfl_sync(full, w1, 0);
    t1 = __shfl_sync(full, t1, 0);
    // A waiter that gave up (error flag raised, t0 = -1) keeps its slot and
    // beta for the next window, so no index below ever goes out of the
    // ladder.
    Walker next;
    next.slot = t0 >= 0 ? t0 : s;
    next.beta = __shfl_sync(full, nb, 0);
    const float sg_own = __shfl_sync(full, sg, 4), sg_partner = __shfl_sync(full, sg, 5);
    next.sigma = next.slot == s ? sg_own : sg_partner;
    __syncwarp();  // orders lane 0's acquire before the other lanes' reads

    // Settle: round-trip counters (lane 1 for this walker, lane 3 for the
    // partner the decider settles), then the staged samples at the new slots.
    if ((lane == 1 && t0 >= 0 && ends) || (lane == 3 && t1 >= 0)) {
        const int t = lane == 1 ? t0 : t1;
        if (lane == 3) {
            tr = x.trips + start + w1;
            origin = __ldcg(tr);
            visited = __ldcg(tr + n);
            sweep0 = __ldcg(tr + 2 * n);
            ntrips = __ldcg(tr + 3 * n);
            tsweeps = __ldcg(tr + 4 * n);
        }
        if (t == 0 || t == R - 1) {
            if (origin < 0) {
                tr[0] = t;
                tr[2 * n] = sweep;
            } else if (t != origin) {
                tr[n] = 1;
            } else if (visited) {
                tr[3 * n] = ntrips + 1;
                tr[4 * n] = tsweeps + (sweep - sweep0);
                tr[2 * n] = sweep;
                tr[n] = 0;
            }
        }
    }
    if (slot < 0) return next;
    double *out = x.samples + (size_t)slot * x.channels * x.n_temps_total + start;
    if (t0 >= 0 && lane < x.channels) out[(size_t)lane * x.n_temps_total + t0] = own;
    if (t1 >= 0 && lane < x.channels)
        out[(size_t)lane * x.n_temps_total + t1] = __ldcg(x.staging + (size_t)lane * n + start + w1);
    return next;
}

// The global-stream variant with two visits in flight (policies with
// kGlobalInFlight = 2): like the two-plaquette variant it carries two visits
// per thread, so it shares that variant's thread cap (kPairThreads) and
// register budget.
constexpr int kGlobalPairVariant = -2;

// Threads per block the NPMAX variant is compiled for: NPMAX streams of four
// colours live in registers (16 registers per plaquette).  kMaxThreads caps
// every variant, kPairThreads the two-plaquette one (its launch bound sets
// the register budget: 256 threads leave 255 registers a thread).  NPMAX = 0 is the
// global-stream variant for up to 1024 threads (64 registers), one visit at
// a time.
template <class M, int NPMAX>
constexpr int window_max_threads()
{
    return NPMAX <= 1 && NPMAX != kGlobalPairVariant ? (1024 < M::kMaxThreads ? 1024 : M::kMaxThreads)
                                                    : (M::kPairThreads < M::kMaxThreads ? M::kPairThreads : M::kMaxThreads);
}

template <class M, int NPMAX>
__global__ void __launch_bounds__(window_max_threads<M, NPMAX>(), 1) window_kernel(const typename M::Args a)
{
    using Cell = typename M::Cell;
    constexpr int NS = M::kSums;  // reduced sums (>= the kChannels output channels)
    static_assert(NS + 3 <= kRedDoubles && NS <= 32, "too many reduced sums");
    constexpr int NK = NPMAX > 0 ? NPMAX : 1;
    constexpr int GIF = NPMAX == kGlobalPairVariant ? 2 : 1;  // global variant: visits in flight
    static_assert(!smem_stream_variant<M, NPMAX>() || M::kPipeline, "shared-memory streams need propose/decide");
    cg::cluster_group cluster = cg::this_cluster();
    const int C = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int cid = blockIdx.x / C;
    const int T = blockDim.x, tid = threadIdx.x;

    extern __shared__ __align__(16) unsigned char smem[];
    double *red = reinterpret_cast<double *>(smem);  // kRedDoubles
    double *scratch = red + kRedDoubles;               // 32 * (NS + 3)
    constexpr int NP = part_slots<M>();
    float2 *parts = reinterpret_cast<float2 *>(scratch + 32 * (NS + 3));  // [kMaxCluster][NP], rank 0's used
    FusedExchange *fxs = reinterpret_cast<FusedExchange *>(parts + kMaxCluster * NP);
    uint64_t *strip_bar = reinterpret_cast<uint64_t *>(reinterpret_cast<unsigned char *>(fxs) + kFusedCopyBytes);
    WindowCarry *carry =
        reinterpret_cast<WindowCarry *>(reinterpret_cast<unsigned char *>(strip_bar) + kStripBarBytes);
    Cell *cells = reinterpret_cast<Cell *>(reinterpret_cast<unsigned char *>(carry) + kCarryBytes);

    const WindowCommon &cm = a.c;
    // The work lists hold n_clusters entries for clusters of cluster_size
    // CTAs.  A launch of any other shape -- a re-issued launch that lost its
    // cluster attribute would run clusters of one CTA, with cluster indices
    // far past the work lists -- touches nothing: it raises the error flag
    // of a fused launch (the host reports it) and returns before its first
    // memory access or barrier.  The condition is uniform over the grid.
    if (C != cm.cluster_size || (int)gridDim.x != cm.n_clusters * cm.cluster_size) {
        if (a.fx.enabled && blockIdx.x == 0 && tid == 0) atomicExch(a.fx.error, 1);
        return;
    }
    ulonglong2 *rng_g = static_cast<ulonglong2 *>(cm.rng);
    if (a.fx.enabled && tid == 0) *fxs = a.fx;
    // A resident launch runs n_windows windows with the strip on chip,
    // exchanging between them (each walker waits for its pair's decision
    // only).
    const int n_windows = a.fx.enabled && a.fx.n_windows > 1 ? a.fx.n_windows : 1;
    // The launch's sample schedule (sample_slot's, once per launch: the clock
    // stands still within a launch): the sweeps from the launch's start to
    // the first one due a sample (kNoSample: none within the launch), and
    // that sample's ring slot.
    int sched_due0 = kNoSample, sched_slot0 = 0;
    if (cm.samples != nullptr && cm.sample_interval > 0 && cm.n_slots > 0) {
        const long long clock0 = __ldcg(cm.clock), first = cm.first_sample_sweep, from = clock0 + 1;
        const long long k = from <= first ? 0 : (from - first + cm.sample_interval - 1) / cm.sample_interval;
        const long long due = first + k * cm.sample_interval - clock0;
        if (due <= (long long)n_windows * cm.n_sweeps) sched_due0 = (int)due;
        sched_slot0 = (int)(k % cm.n_slots);
    }
    if (M::kBulkLoad && tid == 0) mbar_init(strip_bar, 1);
    if (tid == 0) {
        carry->clock0 = __ldcg(cm.clock);
        carry->rounds0 = __ldcg(cm.clock + 1);
    }
    [[maybe_unused]] unsigned strip_phase = 0;
    // DSMEM stores below need every CTA of the cluster to be running.
    cluster.sync();

    for (int w = cm.work_ptr[cid]; w < cm.work_ptr[cid + 1]; ++w) {
        const int r = cm.work_idx[w];
        const mcgb_replica rep = cm.table[r];
        // The next replica of this cluster's work list has another size: its
        // strip layout differs, so the halo rows its strip load pushes into
        // the neighbouring CTAs may land on cells they still write back.
        const bool relayout = w + 1 < cm.work_ptr[cid + 1] && cm.table[cm.work_idx[w + 1]].L != rep.L;
        const int Ce = effective_cluster(rep.L, C);
        StripCtx g;
        g.LP = rep.L >> 1;
        g.HP = rank < Ce ? rep.L / (2 * Ce) : 0;
        g.NPL = g.HP * g.LP;
        g.PS = (g.HP + 2) * g.LP;
        g.up = rank == 0 ? Ce - 1 : rank - 1;
        g.dn = rank + 1 >= Ce ? 0 : rank + 1;
        float *own = reinterpret_cast<float *>(
            (reinterpret_cast<uintptr_t>(cells + 4 * g.PS) + 15) & ~static_cast<uintptr_t>(15));
        [[maybe_unused]] ulonglong2 *sst = reinterpret_cast<ulonglong2 *>(
            (reinterpret_cast<uintptr_t>(own + (size_t)4 * g.NPL * M::kOwnFloats) + 15) & ~static_cast<uintptr_t>(15));
        const int64_t gplane = (int64_t)g.LP * g.LP;
        const int64_t base = rep.state_offset + (int64_t)rank * g.NPL;

        // Load the strip; boundary rows also go to the neighbours' halos.
        // Fused launches (which carry an error flag for the bounded wait)
        // take bulk copies where the layout allows.
        constexpr bool SS = smem_stream_variant<M, NPMAX>();
        bool bulk = false;
        if constexpr (M::kBulkLoad) {
            if (a.fx.enabled && strip_bulk_ok<M, SS>(a, cells, own, g, base, gplane)) {
                bulk = true;
                load_strip_bulk<M, SS>(a, cells, own, sst, g, base, gplane, strip_bar, strip_phase, a.fx.error);
            }
        }
        // Long loops step by additions (see measure_colour).
        const bool long_loop = g.NPL > 2 * T;
        if (!bulk)
        for (int c = 0; c < 4; ++c) {
            SiteWalk walk(long_loop ? tid : 0, long_loop ? T : 1, g.LP);
            for (int p = tid; p < g.NPL; p += T, walk.advance()) {
                const Site s = long_loop ? walk.site() : make_site(p, g.LP);
                Cell &me = cells[c * g.PS + s.o + s.pc];
                M::load(a, strip_site<M>(rep, g, rank, base, gplane, c, p), me,
                        own + (size_t)(c * g.NPL + p) * M::kOwnFloats);
                if (c < 2 && s.pr == 0)
                    *static_cast<Cell *>(
                        __cluster_map_shared_rank(cells + c * g.PS + (g.HP + 1) * g.LP + s.pc, g.up)) = me;
                if (c >= 2 && s.pr == g.HP - 1)
                    *static_cast<Cell *>(__cluster_map_shared_rank(cells + c * g.PS + s.pc, g.dn)) = me;
            }
        }

        // NPMAX > 0: the streams live in registers (the host launches this
        // variant only when every strip fits) or, for the shared-memory
        // stream variant, in shared memory; NPMAX = 0: global memory.
        constexpr bool regs = NPMAX > 0;
        ulonglong2 st[NK][4];
        Site sites[NK];
#pragma unroll
        for (int k = 0; k < NK; ++k) {
            const int p = tid + k * T;
            sites[k] = make_site(p < g.NPL ? p : 0, g.LP);
            if (regs && !SS) {
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (p < g.NPL) st[k][c] = rng_g[strip_site<M>(rep, g, rank, base, gplane, c, p)];
            }
        }
        if constexpr (SS) {
            if (!bulk)
                for (int c = 0; c < 4; ++c)
                    for (int p = tid; p < g.NPL; p += T)
                        sst[c * g.NPL + p] = rng_g[strip_site<M>(rep, g, rank, base, gplane, c, p)];
        }
        // The sample schedule: the sweeps from the window's start to the next
        // one due a sample (sweep s of the window is due when s + 1 == due)
        // and its ring slot, from the launch's schedule at the first window,
        // then carried from window to window.
        int due = sched_due0, next_slot = sched_slot0;
        for (int win = 0; win < n_windows; ++win) {
        // The walker and the running energy: from the device tables at a
        // replica's first window, then as the previous window's exchange
        // left them (carried on chip, published by the barrier that ended
        // that window).
        // Rank 0 reads the running energy and the walker's slot from its
        // carry where it needs them (in no register across the sweeps).
        Walker wk;
        if (win == 0) {
            wk = load_walker(a, r, rep);
            if (tid == 0) {
                carry->next = wk;
                if (rank == 0) {
                    carry->e_hi = __ldcg(cm.e_run + 2 * r);
                    carry->e_lo = __ldcg(cm.e_run + 2 * r + 1);
                }
            }
        } else {
            wk = carry->next;
        }
        const typename M::Ctx ctx = M::prepare(a, r, rep, wk);
        cluster_arrive();

        float dsum = 0.0f, dcomp = 0.0f;
        int nacc = 0;
        // A sample whose partial sums wait in rank 0's `parts`: -1 none, -2
        // the staged window-end sample, else its ring slot.
        int pend = -1;
#define MCGB_COMBINE_PENDING()                                                                              \
    if (pend != -1) {                                                                                       \
        if (rank == 0 && tid < 32)                                                                          \
            combine_sample<M>(ctx, cm, parts, red, C, pend, r, rep.ladder_start + carry->next.slot,        \
                              carry->e_hi, carry->e_lo, a.n_replicas);                                      \
        pend = -1;                                                                                          \
    }
        [[maybe_unused]] typename M::Prop pa[NK], pb[NK];
        // Colour 0 of this sweep already ran, in the last phase of the
        // previous sweep (see `merge` below).
        bool c0_done = false;
        for (int s = 0; s < cm.n_sweeps; ++s) {
            // This sweep's accepted energy changes (at most a few terms per
            // thread), folded into the compensated running sum once per sweep.
            float dacc = 0.0f;
            // Colours 0 and 3 share no bond when a site couples to its four
            // nearest neighbours only (every model without diagonal cells,
            // i.e. without kSplitMiddle): both read only planes 1 and 2.  So
            // colour 0 of the next sweep runs in this sweep's colour-3 phase
            // -- the same moves with the same streams against the same
            // neighbour values as in a phase of its own -- which saves one
            // cluster barrier a sweep.  Not after the window's last sweep
            // (an exchange may change the temperature before the next one)
            // nor after a sampled sweep (the sample reads the state between
            // the two).
            const bool sample_due = s + 1 == due;
            [[maybe_unused]] const bool merge =
                !M::kSplitMiddle && (M::kPipeline || !regs) && s + 1 < cm.n_sweeps && !sample_due;
            if constexpr (!M::kPipeline && regs) {
                {
                    cluster_wait();
                    MCGB_COMBINE_PENDING()
                    fused_pass<M, NK, 0>(ctx, cells, own, g, sites, st, dacc, nacc);
                    cluster_arrive();
                    cluster_wait();
                    fused_pass<M, NK, 1>(ctx, cells, own, g, sites, st, dacc, nacc);
                    if (M::kSplitMiddle) {
                        cluster_arrive();
                        cluster_wait();
                    }
                    fused_pass<M, NK, 2>(ctx, cells, own, g, sites, st, dacc, nacc);
                    cluster_arrive();
                    cluster_wait();
                    fused_pass<M, NK, 3>(ctx, cells, own, g, sites, st, dacc, nacc);
                }
            } else if constexpr (regs) {
                {
                // Invariant: this thread has arrived at the barrier that
                // follows the previous phase and not yet waited.
                if (!c0_done) {
                    propose_pass<M, NK, 0, SS>(ctx, cells, own, g, sites, st, pa, sst);
                    cluster_wait();
                    MCGB_COMBINE_PENDING()
                    decide_pass<M, NK, 0>(ctx, cells, own, g, sites, pa, dacc, nacc);
                    cluster_arrive();
                }
                propose_pass<M, NK, 1, SS>(ctx, cells, own, g, sites, st, pa, sst);
                propose_pass<M, NK, 2, SS>(ctx, cells, own, g, sites, st, pb, sst);
                cluster_wait();
                MCGB_COMBINE_PENDING()
                decide_pass<M, NK, 1>(ctx, cells, own, g, sites, pa, dacc, nacc);
                if (M::kSplitMiddle) {
                    cluster_arrive();
                    cluster_wait();
                }
                decide_pass<M, NK, 2>(ctx, cells, own, g, sites, pb, dacc, nacc);
                cluster_arrive();
                propose_pass<M, NK, 3, SS>(ctx, cells, own, g, sites, st, pa, sst);
                if (merge) propose_pass<M, NK, 0, SS>(ctx, cells, own, g, sites, st, pb, sst);
                cluster_wait();
                decide_pass<M, NK, 3>(ctx, cells, own, g, sites, pa, dacc, nacc);
                if (merge) decide_pass<M, NK, 0>(ctx, cells, own, g, sites, pb, dacc, nacc);
                }
            } else {
                (void)sites;
                if (!c0_done) {
                    cluster_wait();
                    MCGB_COMBINE_PENDING()
                    global_rng_pass<M, 0, GIF>(a, ctx, cells, own, g, base, gplane, dacc, nacc);
                    cluster_arrive();
                }
                cluster_wait();
                MCGB_COMBINE_PENDING()
                global_rng_pass<M, 1, GIF>(a, ctx, cells, own, g, base, gplane, dacc, nacc);
                if (M::kSplitMiddle) {
                    cluster_arrive();
                    cluster_wait();
                }
                global_rng_pass<M, 2, GIF>(a, ctx, cells, own, g, base, gplane, dacc, nacc);
                cluster_arrive();
                cluster_wait();
                global_rng_pass<M, 3, GIF>(a, ctx, cells, own, g, base, gplane, dacc, nacc);
                if (merge) global_rng_pass<M, 0, GIF>(a, ctx, cells, own, g, base, gplane, dacc, nacc);
            }
            c0_done = merge;

            comp_add(dsum, dcomp, dacc);
            if (sample_due) {
                const int slot = next_slot;
                due += cm.sample_interval;
                next_slot = next_slot + 1 == cm.n_slots ? 0 : next_slot + 1;
                // Measure the strip before arriving at the barrier that ends
                // the sweep.  Once this CTA's own colour-3 moves are done (a
                // CTA barrier) every cell the measurement reads is final: it
                // reads the cells below and to the right only, and the one
                // halo row among them (planes 0/1 below the strip) was last
                // written in the colour 0-1 phases, published by an earlier
                // barrier.  Reduce over the CTA, push into rank 0.
                __syncthreads();
                const bool last = s + 1 == cm.n_sweeps;
                push_sample<M>(ctx, cells, own, g, dsum, dcomp, nacc, last, reinterpret_cast<float2 *>(scratch),
                               parts, rank);
                pend = (cm.staging != nullptr && last) ? -2 : slot;
            }
            cluster_arrive();
        }
        // Ring slot of a sample staged on the window's last sweep (-1: none);
        // a sample on the last sweep has also pushed the epilogue's sums.
        const int end_slot = pend == -2 ? (next_slot == 0 ? cm.n_slots - 1 : next_slot - 1) : -1;
        const bool epilogue_pushed = pend != -1;
        cluster_wait();
        MCGB_COMBINE_PENDING()
#undef MCGB_COMBINE_PENDING
        // The acceptance count, and for the exchange the walker's beta and
        // the exchange rounds before this one.
        const long long acc_prev =
            rank == 0 && tid == 0 ? (win == 0 ? __ldcg(cm.accepted + r) : carry->accepted) : 0;
        const float beta_now = a.fx.enabled && rank == 0 && tid == 0 ? carry->next.beta : 0.0f;
        const long long rounds = a.fx.enabled && rank == 0 && tid < 32 ? carry->rounds0 + win : 0;
        double e_now = 0.0;
        float e_hi = 0.0f, e_lo = 0.0f;
        long long acc_now = 0;

        // Window epilogue: energy and acceptance bookkeeping (compensated
        // float32 partial sums pushed into rank 0, as for samples, unless a
        // sample on the last sweep carried them), write back.
        if (!epilogue_pushed) {
            FSum v2[3];
            window_epilogue_sums<M>(ctx, cells, own, g, dsum, dcomp, nacc, v2);
            block_fsum_push<3>(v2, reinterpret_cast<float2 *>(scratch),
                               static_cast<float2 *>(__cluster_map_shared_rank(parts, 0)) + rank * NP + NS);
        }
        if (win + 1 == n_windows) {
        for (int c = 0; c < 4; ++c) {
            SiteWalk walk(long_loop ? tid : 0, long_loop ? T : 1, g.LP);
            for (int p = tid; p < g.NPL; p += T, walk.advance()) {
                const Site s = long_loop ? walk.site() : make_site(p, g.LP);
                M::store(a, strip_site<M>(rep, g, rank, base, gplane, c, p), cells[c * g.PS + s.o + s.pc],
                         own + (size_t)(c * g.NPL + p) * M::kOwnFloats);
            }
        }
        if constexpr (SS) {
            for (int c = 0; c < 4; ++c)
                for (int p = tid; p < g.NPL; p += T)
                    rng_g[strip_site<M>(rep, g, rank, base, gplane, c, p)] = sst[c * g.NPL + p];
        } else if (regs) {
#pragma unroll
            for (int k = 0; k < NK; ++k) {
                const int p = tid + k * T;
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (p < g.NPL) rng_g[strip_site<M>(rep, g, rank, base, gplane, c, p)] = st[k][c];
            }
        }
        }
        // The epilogue's pushes land before rank 0 merges them: published by
        // this barrier, or already by the barrier ending the last sweep.  The
        // barrier also holds a replica of another size back until every CTA
        // has written this one back.
        if (!epilogue_pushed || (relayout && win + 1 == n_windows)) cluster.sync();
        if (rank == 0 && tid == 0) {
            FSum de, na, ex;
            for (int k = 0; k < C; ++k) {
                const float2 *pk = parts + k * NP + NS;
                de.merge(pk[0].x, pk[0].y);
                na.merge(pk[1].x, pk[1].y);
                ex.merge(pk[2].x, pk[2].y);
            }
            float hi, lo2;
            if (M::kExactEnergy) {
                const double e = M::finish_energy(ctx, ex.value());
                hi = (float)e;
                lo2 = (float)(e - (double)hi);
                e_now = e;
            } else {
                // Compensated (hi, lo) float update of the running energy.
                float s1, e1;
                two_sum(carry->e_hi, de.hi, s1, e1);
                const float lo = carry->e_lo + e1 + de.lo;
                two_sum(s1, lo, hi, lo2);
                e_now = (double)hi + (double)lo2;
            }
            e_hi = hi;
            e_lo = lo2;
            acc_now = acc_prev + (long long)na.value();
        }
        __syncwarp();
        Walker nw{};
        if (a.fx.enabled && rank == 0 && tid < 32)
            nw = pair_finished(*fxs, a.sigma_t, rep.ladder_start, rep.n_temps, rep.ladder, r,
                               carry->next.slot, beta_now, e_now, carry->clock0 + (long long)(win + 1) * cm.n_sweeps,
                               rounds, end_slot,
                               win + 1 < n_windows);
        // The next window's walker into every CTA of the cluster (lane k,
        // rank k), published by the cluster barrier below.
        if (win + 1 < n_windows && rank == 0 && tid < C)
            *static_cast<Walker *>(__cluster_map_shared_rank(&carry->next, tid)) = nw;
        // After the exchange, whose releasing atomic need not wait for them.
        if (rank == 0 && tid == 0) {
            cm.energies[r] = e_now;
            cm.e_run[2 * r] = e_hi;
            cm.e_run[2 * r + 1] = e_lo;
            cm.accepted[r] = acc_now;
            carry->e_hi = e_hi;
            carry->e_lo = e_lo;
            carry->accepted = acc_now;
        }
        __syncwarp();  // the aligned cluster barriers need warp 0 converged again
        // Between windows of a resident launch every CTA waits for the new
        // temperature.  After the last window nothing waits: no replica runs
        // twice in a launch, so the next replica of the work list reads
        // nothing the exchange writes, and its strip load (cells and halo
        // rows; the exchange reads neither) overlaps warp 0's exchange.  A
        // replica of the same size pushes only into halo rows, which the
        // write-back does not read; one of another size waited above.
        if (win + 1 < n_windows) cluster.sync();
        if (due != kNoSample) due -= cm.n_sweeps;
        }  // windows
    }
    if (a.fx.enabled && rank == 0 && tid == 0) launch_finished(a.fx, cm, (int)(gridDim.x / C));
}

}  // namespace mcgb
