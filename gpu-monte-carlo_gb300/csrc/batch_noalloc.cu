// One exchange window of the batched engine that allocates nothing.
//
// mcgb_batch_window_run followed by mcgb_batch_exchange needs a caller-owned
// scratch buffer, `staging`: the window kernel parks a sample that falls on
// the window's last sweep there, and the exchange kernel scatters it to the
// temperature slots of the updated map.  Some callers cannot allocate device
// memory for it: a program embedded in a host runtime that owns every device
// allocation itself (a fixed memory pool sized to the whole GPU, or a language
// binding whose allocator the library must not bypass, so a cudaMalloc here
// would fail or escape its accounting), and a latency-critical driver loop in
// which cudaMalloc's implicit device synchronisation would stall the work
// other streams have in flight.  For them, mcgb_batch_window_exchange_noalloc
// runs the same two kernels with `staging` in a fixed array compiled into
// this library.
//
// The array holds kNoAllocStagingDoubles doubles (256 KB): channels x
// replicas must fit, so batches of up to 3276 replicas for the 10-channel
// He3 model, 6553 for XY.  Every GPU that loads the library keeps it until
// the process exits.  All calls share it and it keeps the last call's
// contents.  Nothing in it needs to start at zero: the call runs one window
// over every replica of the table (size-group windows, which cover only part
// of it, are rejected), so the exchange reads only entries the same call's
// window has just written.  Calls on one device share the one array, so they
// must not overlap on the GPU: serialise them on one stream.  Each device
// has its own copy of the array, so calls on different devices do not race.
//
// The array's name is a host-side stand-in, not a device address, so host
// code never passes it to a kernel.  The first call in each CUDA context,
// with that context's device current, looks up the device address with
// cudaGetSymbolAddress and caches it with the context handle; a later call
// in another context (after cudaDeviceReset, say) looks it up again.  Make
// that first call before any stream capture begins.
#include <cuda.h>

#include <mutex>

#include "batch_args.cuh"

namespace mcgb {

constexpr int kNoAllocStagingDoubles = 32768;
static __device__ __align__(256) double g_noalloc_staging[kNoAllocStagingDoubles];

// The current driver context, through the runtime's driver entry point
// (the library does not link libcuda directly).
static int current_context(CUcontext *ctx)
{
    using GetCurrent = CUresult (*)(CUcontext *);
    static GetCurrent fn = nullptr;
    if (fn == nullptr) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        int st = cuda_status(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q),
                             "cudaGetDriverEntryPointByVersion(cuCtxGetCurrent)");
        if (st) return st;
        MCGB_REQUIRE(q == cudaDriverEntryPointSuccess && p != nullptr, "no-alloc window: cuCtxGetCurrent not found");
        fn = reinterpret_cast<GetCurrent>(p);
    }
    *ctx = nullptr;
    MCGB_REQUIRE(fn(ctx) == CUDA_SUCCESS, "no-alloc window: cuCtxGetCurrent failed");
    return MCGB_OK;
}

static int noalloc_staging_address(double **out)
{
    struct Entry {
        CUcontext ctx;
        double *addr;
    };
    static std::mutex mu;
    static Entry cache[128] = {};
    int dev = 0;
    int st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (st) return st;
    MCGB_REQUIRE(dev >= 0 && dev < 128, "no-alloc window: device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(mu);
    CUcontext ctx = nullptr;
    if ((st = current_context(&ctx))) return st;
    if (ctx == nullptr || cache[dev].ctx != ctx) {
        // cudaGetSymbolAddress also makes the device's primary context
        // current if no runtime call has done so yet.
        void *p = nullptr;
        st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_staging), "cudaGetSymbolAddress(no-alloc staging)");
        if (st) return st;
        if ((st = current_context(&ctx))) return st;
        cache[dev] = Entry{ctx, static_cast<double *>(p)};
    }
    *out = cache[dev].addr;
    return MCGB_OK;
}

}  // namespace mcgb

using namespace mcgb;

extern "C" int mcgb_batch_window_exchange_noalloc(int model, const mcgb_batch_window *w, const mcgb_batch_pt *pt,
                                                  void *stream)
{
    MCGB_REQUIRE(w != nullptr && pt != nullptr, "no-alloc window: null argument block");
    MCGB_REQUIRE(w->staging == nullptr, "no-alloc window: staging must be NULL (the library supplies it)");
    MCGB_REQUIRE(w->host_work_idx == nullptr && w->n_work == 0,
                 "no-alloc window: one launch over the whole replica table only (host_work_idx must be NULL, "
                 "n_work 0): a size-group window would leave other replicas' scratch entries stale");
    MCGB_REQUIRE(w->hold_clock == 0, "no-alloc window: hold_clock must be 0 (one launch per window)");
    const int channels = mcgb_batch_channels(model);
    if (channels < 0) return channels;
    MCGB_REQUIRE(pt->channels == channels, "no-alloc window: pt->channels must be %d for model %d", channels,
                 model);
    MCGB_REQUIRE(w->n_replicas >= 1 && (long long)channels * w->n_replicas <= kNoAllocStagingDoubles,
                 "no-alloc window: %d replicas x %d channels exceed the fixed scratch of %d values", w->n_replicas,
                 channels, kNoAllocStagingDoubles);
    double *staging = nullptr;
    int st = noalloc_staging_address(&staging);
    if (st) return st;
    mcgb_batch_window local = *w;
    local.staging = w->samples != nullptr ? staging : nullptr;
    st = mcgb_batch_window_run(model, &local, stream);
    if (st) return st;
    return mcgb_batch_exchange(&local, pt, stream);
}
