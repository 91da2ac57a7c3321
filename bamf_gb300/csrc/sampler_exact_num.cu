/*
 * sampler_exact_num.cu - the exact (parity) sampler with the sampled PSF
 * (OptModel 1); built with -fmad=false like sampler_exact.cu.
 */
#include "sampler_kernel.cuh"
#include "sampler_launch.h"

namespace bamf {

cudaError_t launch_exact_num(const SamplerConsts &K, const SamplerBatch &B, size_t smem, int blocks, int threads,
                             cudaStream_t stream)
{
    return launch_kernel(rjmcmc_kernel<true, true>, K, B, smem, blocks, threads, stream);
}

int occupancy_exact_num(size_t smem, int threads) { return resident_ctas(rjmcmc_kernel<true, true>, smem, threads); }

}  // namespace bamf
