/*
 * sampler_fast_num.cu - the fast sampler with the sampled PSF (OptModel 1).
 */
#include "sampler_kernel.cuh"
#include "sampler_launch.h"

namespace bamf {

cudaError_t launch_fast_num(const SamplerConsts &K, const SamplerBatch &B, size_t smem, int blocks, int threads,
                            int min_ctas, cudaStream_t stream)
{
    if (min_ctas == 1) return cudaErrorInvalidValue;
    return min_ctas == 3 ? launch_kernel(rjmcmc_kernel_sync<true, 3>, K, B, smem, blocks, threads, stream)
                         : launch_kernel(rjmcmc_kernel_sync<true, 2>, K, B, smem, blocks, threads, stream);
}

int occupancy_fast_num(size_t smem, int threads, int min_ctas)
{
    if (min_ctas == 1) return 0; /* the one-CTA build is instantiated for the Gaussian PSF only */
    return min_ctas == 3 ? resident_ctas(rjmcmc_kernel_sync<true, 3>, smem, threads)
                         : resident_ctas(rjmcmc_kernel_sync<true, 2>, smem, threads);
}

}  // namespace bamf
