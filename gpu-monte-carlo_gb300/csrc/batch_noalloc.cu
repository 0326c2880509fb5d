// One exchange window of the batched engine that allocates nothing.
//
// mcgb_batch_window_run followed by mcgb_batch_exchange needs a caller-owned
// scratch buffer, `staging`: the window kernel parks a sample that falls on
// the window's last sweep there, and the exchange kernel scatters it to the
// temperature slots of the updated map.  Some callers cannot allocate device
// memory for it: a host program that drives the library through the C ABI
// from inside a CUDA-graph capture (where cudaMalloc is not allowed), or one
// embedded in a runtime that owns every device allocation itself (a fixed
// memory pool, or a language binding whose allocator the library must not
// bypass).  For them, mcgb_batch_window_exchange_noalloc runs the same two
// kernels with `staging` in a fixed array compiled into this library.
//
// The array holds kNoAllocStagingDoubles doubles (256 KB): channels x
// replicas must fit, so batches of up to 3276 replicas for the 10-channel
// He3 model, 6553 for XY.  Every GPU that loads the library keeps it until
// the process exits.  All calls share it and it keeps the last call's
// contents; nothing in it needs to start at zero, because the exchange reads
// only entries the window of the same call has just written.  Calls whose
// work overlaps on the GPU (different streams, or different devices is fine)
// race on it: serialise them on one stream.
//
// The array's name is a host-side stand-in, not a device address, so host
// code must never pass it to a kernel.  The first call on each device, with
// that device current, looks up the device address with cudaGetSymbolAddress
// and caches it; make that first call before any stream capture begins.
#include <mutex>

#include "batch_args.cuh"

namespace mcgb {

constexpr int kNoAllocStagingDoubles = 32768;
static __device__ __align__(256) double g_noalloc_staging[kNoAllocStagingDoubles];

static int noalloc_staging_address(double **out)
{
    static std::mutex mu;
    static double *addr[128] = {};
    int dev = 0;
    int st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (st) return st;
    MCGB_REQUIRE(dev >= 0 && dev < 128, "no-alloc window: device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (addr[dev] == nullptr) {
        void *p = nullptr;
        st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_staging), "cudaGetSymbolAddress(no-alloc staging)");
        if (st) return st;
        addr[dev] = static_cast<double *>(p);
    }
    *out = addr[dev];
    return MCGB_OK;
}

}  // namespace mcgb

using namespace mcgb;

extern "C" int mcgb_batch_window_exchange_noalloc(int model, const mcgb_batch_window *w, const mcgb_batch_pt *pt,
                                                  void *stream)
{
    MCGB_REQUIRE(w != nullptr && pt != nullptr, "no-alloc window: null argument block");
    MCGB_REQUIRE(w->staging == nullptr, "no-alloc window: staging must be NULL (the library supplies it)");
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
