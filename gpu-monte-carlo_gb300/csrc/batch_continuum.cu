// Batched-engine policies for the Kawamura and He3 models.
#include "batch_args.cuh"

namespace mcgb {

int continuum_window(int model, const mcgb_batch_window &, cudaStream_t)
{
    set_error("batched engine: model %d is not available yet", model);
    return MCGB_EINVAL;
}

int64_t continuum_smem(int model, int, int)
{
    set_error("batched engine: model %d is not available yet", model);
    return MCGB_EINVAL;
}

int continuum_max_clusters(int model, int, int, size_t, int *)
{
    set_error("batched engine: model %d is not available yet", model);
    return MCGB_EINVAL;
}

int continuum_energy64(int model, const mcgb_batch_window &, double *, cudaStream_t)
{
    set_error("batched engine: model %d is not available yet", model);
    return MCGB_EINVAL;
}

}  // namespace mcgb
