// The handle API (include/mcgb.h): one reference Runtime (core/runtime.py:
// 8-135) with its ParallelTempering state (core/parallel_tempering.py:94-
// 317) behind an opaque handle that owns its device buffers.  Every call
// composes the per-colour, measure, energy, exchange and RNG entry points of
// this library over the handle's runs of equal L.
#include <cmath>
#include <cstdlib>
#include <new>
#include <vector>

#include "mcgb_common.cuh"

namespace mcgb {
namespace {

struct Run {
    int L, first, count;  // replicas [first, first + count) of size L
    int64_t site0;        // their first global site
};

int site_bytes(int model)
{
    switch (model) {
    case MCGB_MODEL_ISING: return 1;
    case MCGB_MODEL_XY: return 4;
    case MCGB_MODEL_KAWAMURA: return 20;
    case MCGB_MODEL_HE3:
    case MCGB_MODEL_HE3_GAUSS: return 24;
    default: return 0;
    }
}

int channels(int model)
{
    switch (model) {
    case MCGB_MODEL_ISING: return 2;
    case MCGB_MODEL_XY: return 5;
    case MCGB_MODEL_KAWAMURA: return 7;
    default: return 10;
    }
}

// Walker w's channel values (scratch, `count` columns) into out (C, R) at
// column tidx[first + w] (or first + w).
__global__ void scatter_columns(const double *__restrict__ scratch, double *__restrict__ out,
                                const int32_t *__restrict__ tidx, int first, int count, int C, int R)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count * C) return;
    const int c = k / count, w = k % count;
    const int d = tidx ? tidx[first + w] : first + w;
    out[(size_t)c * R + d] = scratch[(size_t)c * count + w];
}

// The ordered state a new handle starts from.
__global__ void ordered_state(void *state, int64_t n_sites, int model)
{
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n_sites) return;
    if (model == MCGB_MODEL_ISING) {
        static_cast<int8_t *>(state)[k] = 1;
    } else if (model == MCGB_MODEL_KAWAMURA) {
        float *s = static_cast<float *>(state) + 5 * k;
        s[0] = 0.0f;  // theta
        s[1] = 1.0f;  // tau
        s[2] = 0.0f;
        s[3] = 0.0f;
        s[4] = 1.0f;  // d = z
    }
    // XY and He3: zero (the allocation is cleared)
}

}  // namespace
}  // namespace mcgb

using namespace mcgb;

struct mc_handle {
    int model = 0, R = 0, last = MCGB_OK;
    mc_params p{};
    cudaStream_t s = nullptr;
    std::vector<Run> runs;
    int64_t n_sites = 0;
    int sbytes = 0, C = 0;
    void *state = nullptr, *rng = nullptr, *exrng = nullptr;
    float *betas = nullptr, *sigmas = nullptr;
    double *energies = nullptr, *scratch = nullptr;
    int32_t *w2t = nullptr, *t2w = nullptr;
    int64_t *swaps = nullptr, *trips = nullptr, *counts = nullptr;
};

namespace {

int record(mc_handle *h, int st)
{
    if (h) h->last = st;
    return st;
}

void free_all(mc_handle *h)
{
    void *ptrs[] = {h->state, h->rng, h->exrng, h->betas, h->sigmas, h->energies, h->scratch,
                    h->w2t, h->t2w, h->swaps, h->trips, h->counts};
    for (void *q : ptrs)
        if (q) cudaFree(q);
}

int alloc(void **p, size_t bytes)
{
    if (bytes == 0) return MCGB_OK;
    if (cudaMalloc(p, bytes) != cudaSuccess) {
        (void)cudaGetLastError();
        set_error("mc_create: cudaMalloc of %zu bytes failed", bytes);
        return MCGB_ENOMEM;
    }
    return MCGB_OK;
}

// Buffer `which`: device pointer and size in bytes.
int buffer_of(mc_handle *h, int which, void **ptr, int64_t *bytes)
{
    const int64_t R = h->R, np = R > 1 ? R - 1 : 0;
    switch (which) {
    case MC_STATE: *ptr = h->state, *bytes = h->n_sites * h->sbytes; break;
    case MC_RNG: *ptr = h->rng, *bytes = h->n_sites * 16; break;
    case MC_BETAS: *ptr = h->betas, *bytes = R * 4; break;
    case MC_ENERGIES: *ptr = h->energies, *bytes = R * 8; break;
    case MC_W2T: *ptr = h->w2t, *bytes = R * 4; break;
    case MC_T2W: *ptr = h->t2w, *bytes = R * 4; break;
    case MC_SWAP_COUNTS: *ptr = h->swaps, *bytes = 3 * np * 8; break;
    case MC_TRIPS: *ptr = h->trips, *bytes = 5 * R * 8; break;
    case MC_EXCHANGE_RNG: *ptr = h->exrng, *bytes = np * 16; break;
    default: MCGB_REQUIRE(false, "mc_copy: unknown buffer %d", which);
    }
    return MCGB_OK;
}

template <typename T>
T *at(void *base, int64_t elems_offset, int elem_bytes)
{
    return reinterpret_cast<T *>(static_cast<char *>(base) + elems_offset * elem_bytes);
}

int update_run(mc_handle *h, const Run &u, int color)
{
    void *st = at<void>(h->state, u.site0, h->sbytes);
    void *rng = at<void>(h->rng, u.site0, 16);
    const float *b = h->betas + u.first;
    switch (h->model) {
    case MCGB_MODEL_ISING:
        return mcgb_ising_update_color(static_cast<int8_t *>(st), rng, b, u.count, u.L, color, h->p.J, h->s);
    case MCGB_MODEL_XY:
        if (h->sigmas)
            return mcgb_xy_update_color_gauss(static_cast<float *>(st), rng, b, h->sigmas + u.first, u.count, u.L,
                                              color, h->p.J, h->s);
        return mcgb_xy_update_color(static_cast<float *>(st), rng, b, u.count, u.L, color, h->p.J, h->p.delta, h->s);
    case MCGB_MODEL_KAWAMURA:
        return mcgb_kawamura_update_color(static_cast<float *>(st), rng, b, u.count, u.L, color, h->p.J, h->p.delta,
                                          h->s);
    case MCGB_MODEL_HE3:
        return mcgb_he3_update_color(static_cast<float *>(st), rng, b, u.count, u.L, color, h->p.coefficients,
                                     h->p.K, h->p.delta, h->p.g_d, h->s);
    default:
        return mcgb_he3_gaussian_update_color(static_cast<float *>(st), rng, b, u.count, u.L, color,
                                              h->p.coefficients, h->p.K, h->p.rho, h->p.mass, h->p.g_d,
                                              h->counts + u.site0, h->s);
    }
}

int energy_run(mc_handle *h, const Run &u, double *out)
{
    const void *st = at<void>(h->state, u.site0, h->sbytes);
    switch (h->model) {
    case MCGB_MODEL_ISING:
        return mcgb_ising_energy(static_cast<const int8_t *>(st), u.count, u.L, h->p.J, out, h->s);
    case MCGB_MODEL_XY: return mcgb_xy_energy(static_cast<const float *>(st), u.count, u.L, h->p.J, out, h->s);
    case MCGB_MODEL_KAWAMURA:
        return mcgb_kawamura_energy(static_cast<const float *>(st), u.count, u.L, h->p.J, out, h->s);
    default:
        return mcgb_he3_energy(static_cast<const float *>(st), u.count, u.L, h->p.coefficients, h->p.K, h->p.g_d,
                               out, h->s);
    }
}

int measure_run(mc_handle *h, const Run &u, const int32_t *tidx, const double *cached, double *out)
{
    const void *st = at<void>(h->state, u.site0, h->sbytes);
    switch (h->model) {
    case MCGB_MODEL_ISING:
        return mcgb_ising_measure(static_cast<const int8_t *>(st), u.count, u.L, h->p.J, tidx, cached, out, h->s);
    case MCGB_MODEL_XY:
        return mcgb_xy_measure(static_cast<const float *>(st), u.count, u.L, h->p.J, tidx, cached, out, h->s);
    case MCGB_MODEL_KAWAMURA:
        return mcgb_kawamura_measure(static_cast<const float *>(st), u.count, u.L, h->p.J, tidx, cached, out, h->s);
    default:
        return mcgb_he3_measure(static_cast<const float *>(st), u.count, u.L, h->p.coefficients, h->p.K, h->p.g_d,
                                tidx, cached, out, h->s);
    }
}

}  // namespace

extern "C" int mc_create(int model_id, const mc_params *params, const int32_t *L_table, int R,
                         const double *temperatures, uint64_t seed, void *stream, mc_handle **out)
{
    MCGB_REQUIRE(out != nullptr && params != nullptr && L_table != nullptr && temperatures != nullptr,
                 "mc_create: null argument");
    *out = nullptr;
    MCGB_REQUIRE(site_bytes(model_id) > 0,
                 "mc_create: model %d has no per-colour form here (Ising, XY, Kawamura, He3, He3 Gaussian)",
                 model_id);
    MCGB_REQUIRE(R >= 1, "mc_create: R must be >= 1");
    mc_handle *h = new (std::nothrow) mc_handle;
    MCGB_REQUIRE(h != nullptr, "mc_create: out of host memory");
    h->model = model_id;
    h->p = *params;
    h->p.sigmas = nullptr;
    h->R = R;
    h->s = as_stream(stream);
    h->sbytes = site_bytes(model_id);
    h->C = channels(model_id);
    for (int r = 0; r < R; ++r) {
        const int L = L_table[r];
        if (L < 4 || L % 2 || !(std::isfinite(temperatures[r]) && temperatures[r] > 0)) {
            delete h;
            MCGB_REQUIRE(false, "mc_create: replica %d needs an even L >= 4 and a positive finite temperature", r);
        }
        if (h->runs.empty() || h->runs.back().L != L) h->runs.push_back(Run{L, r, 0, h->n_sites});
        h->runs.back().count += 1;
        h->n_sites += (int64_t)L * L;
    }
    int max_count = 0;
    for (const Run &u : h->runs) max_count = u.count > max_count ? u.count : max_count;
    const int64_t np = R > 1 ? R - 1 : 0;
    int st = MCGB_OK;
    const size_t sizes[] = {(size_t)(h->n_sites * h->sbytes), (size_t)(h->n_sites * 16), (size_t)(np * 16),
                            (size_t)R * 4, params->sigmas ? (size_t)R * 4 : 0, (size_t)R * 8,
                            (size_t)2 * h->C * (size_t)(R > max_count ? R : max_count) * 8, (size_t)R * 4,
                            (size_t)R * 4, (size_t)(3 * np * 8), (size_t)(5 * R * 8),
                            model_id == MCGB_MODEL_HE3_GAUSS ? (size_t)(3 * h->n_sites * 8) : 0};
    void **targets[] = {&h->state, &h->rng, &h->exrng, reinterpret_cast<void **>(&h->betas),
                        reinterpret_cast<void **>(&h->sigmas), reinterpret_cast<void **>(&h->energies),
                        reinterpret_cast<void **>(&h->scratch), reinterpret_cast<void **>(&h->w2t),
                        reinterpret_cast<void **>(&h->t2w), reinterpret_cast<void **>(&h->swaps),
                        reinterpret_cast<void **>(&h->trips), reinterpret_cast<void **>(&h->counts)};
    for (int k = 0; k < 12 && st == MCGB_OK; ++k) st = alloc(targets[k], sizes[k]);
    if (st == MCGB_OK) {
        std::vector<float> b(R), sg(params->sigmas ? R : 0);
        std::vector<int32_t> ident(R);
        std::vector<int64_t> trips((size_t)5 * R, 0);
        for (int r = 0; r < R; ++r) {
            b[r] = (float)(1.0 / temperatures[r]);
            ident[r] = r;
            trips[r] = -1;          // origin
            trips[2 * R + r] = -1;  // start sweep
            if (params->sigmas) sg[r] = params->sigmas[r];
        }
        trips[0] = 0;
        trips[R - 1] = R - 1;
        trips[2 * R] = 0;
        trips[2 * R + R - 1] = 0;
        cudaError_t e = cudaMemsetAsync(h->state, 0, sizes[0], h->s);
        if (e == cudaSuccess && np) e = cudaMemsetAsync(h->swaps, 0, sizes[9], h->s);
        if (e == cudaSuccess && h->counts) e = cudaMemsetAsync(h->counts, 0, sizes[11], h->s);
        if (e == cudaSuccess) e = cudaMemsetAsync(h->energies, 0, sizes[5], h->s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h->betas, b.data(), R * 4, cudaMemcpyHostToDevice, h->s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h->w2t, ident.data(), R * 4, cudaMemcpyHostToDevice, h->s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h->t2w, ident.data(), R * 4, cudaMemcpyHostToDevice, h->s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h->trips, trips.data(), sizes[10], cudaMemcpyHostToDevice, h->s);
        if (e == cudaSuccess && h->sigmas)
            e = cudaMemcpyAsync(h->sigmas, sg.data(), R * 4, cudaMemcpyHostToDevice, h->s);
        st = cuda_status(e, "mc_create: initial copies");
        if (st == MCGB_OK && model_id != MCGB_MODEL_XY && model_id != MCGB_MODEL_HE3 &&
            model_id != MCGB_MODEL_HE3_GAUSS) {
            ordered_state<<<(unsigned)((h->n_sites + 255) / 256), 256, 0, h->s>>>(h->state, h->n_sites, model_id);
            st = check_launch("ordered_state");
        }
        if (st == MCGB_OK) st = mcgb_rng_init(h->rng, h->n_sites, seed, 0, h->s);
        if (st == MCGB_OK && np) st = mcgb_rng_init(h->exrng, np, seed + 1, 0, h->s);
        if (st == MCGB_OK) st = cuda_status(cudaStreamSynchronize(h->s), "mc_create: synchronise");
    }
    if (st != MCGB_OK) {
        free_all(h);
        delete h;
        return st;
    }
    *out = h;
    return MCGB_OK;
}

extern "C" int mc_update_color(mc_handle *h, int color)
{
    MCGB_REQUIRE(h != nullptr, "mc_update_color: null handle");
    if (color < 0 || color > 3) {
        set_error("mc_update_color: color must be 0..3");
        return record(h, MCGB_EINVAL);
    }
    for (const Run &u : h->runs)
        if (int st = update_run(h, u, color)) return record(h, st);
    return record(h, MCGB_OK);
}

extern "C" int mc_sweep(mc_handle *h, int n_sweeps)
{
    MCGB_REQUIRE(h != nullptr, "mc_sweep: null handle");
    if (n_sweeps < 0) {
        set_error("mc_sweep: n_sweeps must be >= 0");
        return record(h, MCGB_EINVAL);
    }
    if (h->model == MCGB_MODEL_ISING) {
        // Replicas never interact within a sweep: each run sweeps on its own
        // with the fused kernel (bit-identical to four colour launches).
        for (const Run &u : h->runs)
            if (int st = mcgb_ising_sweep(at<int8_t>(h->state, u.site0, 1), at<void>(h->rng, u.site0, 16),
                                          h->betas + u.first, u.count, u.L, h->p.J, n_sweeps, h->s))
                return record(h, st);
        return record(h, MCGB_OK);
    }
    for (int n = 0; n < n_sweeps; ++n)
        for (int c = 0; c < 4; ++c)
            if (int st = mc_update_color(h, c)) return st;
    return record(h, MCGB_OK);
}

extern "C" int mc_energy(mc_handle *h, double *out)
{
    MCGB_REQUIRE(h != nullptr, "mc_energy: null handle");
    double *dst = out ? out : h->energies;
    for (const Run &u : h->runs)
        if (int st = energy_run(h, u, dst + u.first)) return record(h, st);
    return record(h, MCGB_OK);
}

extern "C" int mc_measure(mc_handle *h, const int32_t *temperature_index, const double *cached_energy, double *out)
{
    MCGB_REQUIRE(h != nullptr, "mc_measure: null handle");
    if (out == nullptr) {
        set_error("mc_measure: null output");
        return record(h, MCGB_EINVAL);
    }
    if (h->runs.size() == 1)
        return record(h, measure_run(h, h->runs[0], temperature_index, cached_energy, out));
    for (const Run &u : h->runs) {
        const double *c = cached_energy ? cached_energy + u.first : nullptr;
        if (int st = measure_run(h, u, nullptr, c, h->scratch)) return record(h, st);
        const int n = u.count * h->C;
        scatter_columns<<<(n + 255) / 256, 256, 0, h->s>>>(h->scratch, out, temperature_index, u.first, u.count, h->C,
                                                           h->R);
        if (int st = check_launch("scatter_columns")) return record(h, st);
    }
    return record(h, MCGB_OK);
}

extern "C" int mc_exchange(mc_handle *h, int parity, int64_t sweep)
{
    MCGB_REQUIRE(h != nullptr, "mc_exchange: null handle");
    if (h->R < 2 || (parity != 0 && parity != 1)) {
        set_error("mc_exchange: needs R >= 2 and parity 0 or 1");
        return record(h, MCGB_EINVAL);
    }
    if (int st = mc_energy(h, nullptr)) return st;
    return record(h, mcgb_pt_exchange(h->energies, h->betas, h->w2t, h->t2w, h->exrng, h->swaps, h->trips, h->R,
                                      parity, sweep, h->s));
}

extern "C" int mc_rng_init(mc_handle *h, uint64_t seed, uint64_t subsequence)
{
    MCGB_REQUIRE(h != nullptr, "mc_rng_init: null handle");
    return record(h, mcgb_rng_init(h->rng, h->n_sites, seed, subsequence, h->s));
}

extern "C" int mc_get_error(const mc_handle *h) { return h ? h->last : MCGB_EINVAL; }

static int copy_buffer(mc_handle *h, int which, void *host, int64_t n_bytes, bool in)
{
    MCGB_REQUIRE(h != nullptr && host != nullptr, "mc_copy: null argument");
    void *dev = nullptr;
    int64_t bytes = 0;
    if (int st = buffer_of(h, which, &dev, &bytes)) return record(h, st);
    if (n_bytes != bytes) {
        set_error("mc_copy: buffer %d holds %lld bytes, not %lld", which, (long long)bytes, (long long)n_bytes);
        return record(h, MCGB_EINVAL);
    }
    if (bytes == 0) return record(h, MCGB_OK);
    cudaError_t e = in ? cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, h->s)
                       : cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, h->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
    return record(h, cuda_status(e, in ? "mc_copy_in" : "mc_copy_out"));
}

extern "C" int mc_copy_in(mc_handle *h, int buffer, const void *host, int64_t n_bytes)
{
    return copy_buffer(h, buffer, const_cast<void *>(host), n_bytes, true);
}

extern "C" int mc_copy_out(mc_handle *h, int buffer, void *host, int64_t n_bytes)
{
    return copy_buffer(h, buffer, host, n_bytes, false);
}

extern "C" int mc_destroy(mc_handle *h)
{
    if (h == nullptr) return MCGB_OK;
    const int st = cuda_status(cudaStreamSynchronize(h->s), "mc_destroy: synchronise");
    free_all(h);
    delete h;
    return st;
}
