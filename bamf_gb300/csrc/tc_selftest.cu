/*
 * tc_selftest.cu - known-answer check of the tcgen05 path (tc_ptx.cuh): one
 * CTA computes D = A B^T for a 128 x 16 BF16 A and a 32 x 16 BF16 B of small
 * integers (exact in BF16 and FP32) with one tcgen05.mma into TMEM, reads D
 * back with tcgen05.ld and reports it; the host compares it with the exact
 * product.  Two operand layouts: K-major (the convolutions' forward and
 * input gradient) and MN-major (their weight gradient).  Every wait is
 * bounded: on a timeout the kernel records it, frees its TMEM and
 * returns.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "bamf.h"
#include "tc_ptx.cuh"

namespace {

__host__ __device__ inline float a_val(int m, int k) { return (float)((m * 3 + k * 5) % 7 - 3); }
__host__ __device__ inline float b_val(int n, int k) { return (float)((n * 2 + k) % 5 - 2); }

/* byte offset of element (row, k) in a K-major no-swizzle tile with K = 16:
 * core matrices 8 rows x 8 k (128 B), LBO = 128 (next 8 k), SBO = 256 */
__host__ __device__ inline int kmajor_off(int row, int k) { return (row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2; }

/* byte offset of element (row, k) in an MN-major no-swizzle tile with K =
 * 16 and `rows` rows: core matrices 8 k x 8 rows (128 B), SBO = 128 (next 8
 * rows), LBO = rows * 16 (next 8 k) */
__host__ __device__ inline int mnmajor_off(int row, int k, int rows)
{
    return (k >> 3) * (rows * 16) + (row >> 3) * 128 + (k & 7) * 16 + (row & 7) * 2;
}

template <bool MN>
__global__ void __launch_bounds__(128) tc_selftest_kernel(float *__restrict__ out, int *__restrict__ status)
{
    __shared__ __align__(1024) unsigned char As[128 * 16 * 2];
    __shared__ __align__(1024) unsigned char Bs[32 * 16 * 2];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, warp = t >> 5;
    if (warp == 0) bamf::tc::tmem_alloc(&tslot, 32);
    for (int i = t; i < 128 * 16; i += 128) {
        int m = i / 16, k = i % 16;
        *(__nv_bfloat16 *)(As + (MN ? mnmajor_off(m, k, 128) : kmajor_off(m, k))) = __float2bfloat16(a_val(m, k));
    }
    for (int i = t; i < 32 * 16; i += 128) {
        int n = i / 16, k = i % 16;
        *(__nv_bfloat16 *)(Bs + (MN ? mnmajor_off(n, k, 32) : kmajor_off(n, k))) = __float2bfloat16(b_val(n, k));
    }
    bamf::tc::fence_proxy_async();
    if (t == 0) bamf::tc::mbar_init(&mbar, 1);
    bamf::tc::fence_before_sync();
    __syncthreads();
    bamf::tc::fence_after_sync();
    const uint32_t taddr = tslot;
    if (t == 0) {
        const uint64_t ad = MN ? bamf::tc::smem_desc(bamf::tc::smem_addr(As), 128 * 16, 128)
                               : bamf::tc::smem_desc(bamf::tc::smem_addr(As), 128, 256);
        const uint64_t bd = MN ? bamf::tc::smem_desc(bamf::tc::smem_addr(Bs), 32 * 16, 128)
                               : bamf::tc::smem_desc(bamf::tc::smem_addr(Bs), 128, 256);
        bamf::tc::mma_bf16(taddr, ad, bd, MN ? bamf::tc::idesc_bf16_f32_mn(128, 32) : bamf::tc::idesc_bf16_f32(128, 32),
                           0u);
        bamf::tc::commit(&mbar);
    }
    const bool ok = bamf::tc::mbar_wait(&mbar, 0, 1u << 22);
    bamf::tc::fence_after_sync();
    if (ok) {
        float v[32];
        bamf::tc::tmem_ld32(taddr + ((uint32_t)(warp * 32) << 16), v);
        for (int n = 0; n < 32; ++n) out[t * 32 + n] = v[n];
    } else if (t == 0) {
        atomicExch(status, 1);
    }
    bamf::tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) bamf::tc::tmem_dealloc(taddr, 32);
}

}  // namespace

/* Runs the check for one operand layout (0 K-major, 1 MN-major);
 * *max_abs_err = max |D - exact| over the 128 x 32 product, *timed_out = 1
 * when the MMA's completion never arrived. */
extern "C" bamf_status bamf_tcgen05_selftest_layout(int layout, double *max_abs_err, int *timed_out)
{
    if (!max_abs_err || !timed_out || (layout != 0 && layout != 1)) return BAMF_ERR_INVALID_ARG;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    float *d_out = nullptr;
    int *d_status = nullptr;
    if (cudaMalloc(&d_out, 128 * 32 * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&d_status, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_out);
        return BAMF_ERR_CUDA;
    }
    cudaMemset(d_status, 0, sizeof(int));
    cudaMemset(d_out, 0xff, 128 * 32 * sizeof(float));
    if (layout) tc_selftest_kernel<true><<<1, 128>>>(d_out, d_status);
    else tc_selftest_kernel<false><<<1, 128>>>(d_out, d_status);
    std::vector<float> h(128 * 32);
    int st = 0;
    bool good = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
                cudaMemcpy(h.data(), d_out, h.size() * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess &&
                cudaMemcpy(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
    cudaFree(d_out);
    cudaFree(d_status);
    if (!good) {
        cudaGetLastError();
        return BAMF_ERR_CUDA;
    }
    double err = 0.0;
    for (int m = 0; m < 128; ++m)
        for (int n = 0; n < 32; ++n) {
            double e = 0.0;
            for (int k = 0; k < 16; ++k) e += (double)a_val(m, k) * b_val(n, k);
            double d = std::fabs((double)h[m * 32 + n] - e);
            if (!(d <= err)) err = d; /* NaN propagates */
        }
    *max_abs_err = err;
    *timed_out = st;
    return BAMF_OK;
}

extern "C" bamf_status bamf_tcgen05_selftest(double *max_abs_err, int *timed_out)
{
    return bamf_tcgen05_selftest_layout(0, max_abs_err, timed_out);
}
