/*
 * probe.cu - throughput probes for the sampler's roofline denominators:
 * FP32 FMA and MUFU log2 issue rates of the current device, measured with
 * independent chains so the pipes, not latency, set the rate.
 */
#include <cuda_runtime.h>

#include "bamf.h"
#include "bamf_parity_math.h"

/* a failed CUDA runtime call: clear its error so that a later call on this
 * thread does not report it again */
static inline bamf_status clear_cuda_error()
{
    cudaGetLastError();
    return BAMF_ERR_CUDA;
}

namespace {

__global__ void fma_probe(float *out, int iters, float a, float b)
{
    float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    float x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
        x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
    float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678f) out[blockIdx.x] = s;
}

__global__ void mufu_probe(float *out, int iters)
{
    float x0 = 1.5f + threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    for (int i = 0; i < iters; ++i) {
        x0 = __log2f(x0) + 2.0f; x1 = __log2f(x1) + 2.0f;
        x2 = __log2f(x2) + 2.0f; x3 = __log2f(x3) + 2.0f;
    }
    float s = x0 + x1 + x2 + x3;
    if (s == 12345.678f) out[blockIdx.x] = s;
}

}  // namespace

extern "C" bamf_status bamf_probe_peaks(double *fp32_flops, double *mufu_ops)
{
    if (!fp32_flops || !mufu_ops) return BAMF_ERR_INVALID_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return BAMF_ERR_NO_DEVICE;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *out = nullptr;
    if (cudaMalloc(&out, 65536 * sizeof(float)) != cudaSuccess) return clear_cuda_error();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256;
    const int it_fma = 4096, it_mufu = 2048;
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    float ms = 0.0f, best_fma = 1e30f, best_mufu = 1e30f;
    fma_probe<<<blocks, threads, 0, st>>>(out, 16, 1.0001f, 0.5f); /* warm-up */
    mufu_probe<<<blocks, threads, 0, st>>>(out, 16);
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0, st);
        fma_probe<<<blocks, threads, 0, st>>>(out, it_fma, 1.0001f, 0.5f);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        best_fma = ms < best_fma ? ms : best_fma;
        cudaEventRecord(e0, st);
        mufu_probe<<<blocks, threads, 0, st>>>(out, it_mufu);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        best_mufu = ms < best_mufu ? ms : best_mufu;
    }
    cudaStreamDestroy(st);
    *fp32_flops = 2.0 * 8.0 * it_fma * (double)blocks * threads / (best_fma * 1e-3);
    *mufu_ops = 4.0 * it_mufu * (double)blocks * threads / (best_mufu * 1e-3);
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return err == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}

/* The parity math of the exact sampler (include/bamf_parity_math.h) on the
 * device: out[i] = f(x[i]) for f = erf (0), log (1), exp (2); a host caller
 * compares with the same header compiled for the CPU. */
__global__ void parity_math_kernel(const float *__restrict__ x, int n, int fn, float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = x[i];
    out[i] = fn == 0 ? bamf_pm_erff(v) : (fn == 1 ? bamf_pm_logf(v) : bamf_pm_expf(v));
}

extern "C" bamf_status bamf_parity_math_device(int fn, const float *x, int n, float *out)
{
    if (!x || !out || n < 0 || fn < 0 || fn > 2) return BAMF_ERR_INVALID_ARG;
    if (n == 0) return BAMF_OK;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    float *d = nullptr;
    if (cudaMalloc(&d, 2 * (size_t)n * sizeof(float)) != cudaSuccess) return clear_cuda_error();
    bamf_status st = BAMF_OK;
    if (cudaMemcpy(d, x, (size_t)n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) st = BAMF_ERR_CUDA;
    if (!st) {
        parity_math_kernel<<<(n + 255) / 256, 256>>>(d, n, fn, d + n);
        if (cudaMemcpy(out, d + n, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
            st = BAMF_ERR_CUDA;
    }
    if (st) cudaGetLastError();
    cudaFree(d);
    return st;
}
