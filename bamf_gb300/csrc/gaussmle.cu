/*
 * gaussmle.cu - single-emitter maximum-likelihood fits of (x, y, N, bg)
 * (gaussMLE 'Basic'/'CCD': kernel_MLEFit_XYNB_, cuda_gaussMLEv2.cu:16-141,
 * with GPUgaussLib.cuh:14-258 and MatInvLib.h:15-75) for sm_103a.
 *
 * One thread per fit, ROIs staged through shared memory with coalesced
 * loads (the reference reads each ROI per thread, uncoalesced).  The model
 * is separable: the integrated PSF along x depends only on the column ii
 * and along y only on the row jj, and so do the x/y derivative factors up to
 * the final multiply by the other axis's PSF.  Those per-axis terms are
 * computed once per Newton iteration (2*sz values instead of sz^2), which
 * leaves every per-pixel value bit for bit what the direct evaluation gives.
 * The O(sz^4) start-up filter uses a table of the sz*2-1 distinct Gaussian
 * weights for the same reason.
 * Output layout as the reference: param-major P[Nfits*k + i], k = 0..3 for
 * (x along the contiguous axis, y, N, bg), CRLB likewise, LogLikelihood[i].
 */
#include <cuda_runtime.h>

#include "bamf.h"

/* a failed CUDA runtime call: clear its error so that a later call on this
 * thread does not report it again */
static inline bamf_status clear_cuda_error()
{
    cudaGetLastError();
    return BAMF_ERR_CUDA;
}

namespace {

constexpr int MAXSZ = 21;        /* IMSZBIG of definitions.h: largest fit window */
constexpr int FITS_PER_BLOCK = 64;
#define MLE_PI 3.141592f         /* definitions.h:13 */

/* kernel_IntGauss1D (GPUgaussLib.cuh:14-24) */
__device__ __forceinline__ float int_gauss(int ii, float x, float sigma)
{
    const float norm = 1.0f / 2.0f / sigma / sigma;
    return 1.0f / 2.0f * (erff((ii - x + 1.0f) * sqrtf(norm)) - erff((ii - x) * sqrtf(norm)));
}

/* the part of kernel_DerivativeIntGauss1D (:67-87) before "* PSFother" */
__device__ __forceinline__ void dgauss_axis(int ii, float x, float sigma, float N, float *d1, float *d2)
{
    float u = (ii + 1.0f - x) / sigma, v = (ii - x) / sigma;
    float a = expf(-1.0f / 2.0f * (u * u));
    float b = expf(-1.0f / 2.0f * (v * v));
    *d1 = -N / sqrtf(2.0f * MLE_PI) / sigma * (a - b);
    *d2 = -N / sqrtf(2.0f * MLE_PI) / (sigma * sigma * sigma) * ((ii + 1.0f - x) * a - (ii - x) * b);
}

__global__ void __launch_bounds__(FITS_PER_BLOCK) mle_xynb_kernel(
    const float *__restrict__ data, float sigma, int sz, int iterations,
    float *__restrict__ P, float *__restrict__ CRLB, float *__restrict__ LL, int nfits)
{
    extern __shared__ float sm[];
    const int npx = sz * sz;
    const int64_t first = (int64_t)blockIdx.x * FITS_PER_BLOCK;
    const int nblk = (int)min((int64_t)FITS_PER_BLOCK, (int64_t)nfits - first);
    /* coalesced staging of this block's ROIs */
    for (int i = threadIdx.x; i < nblk * npx; i += blockDim.x) sm[i] = data[first * npx + i];
    __syncthreads();
    if ((int)threadIdx.x >= nblk) return;
    const float *d = sm + threadIdx.x * npx;
    const int64_t fit = first + threadIdx.x;

    float theta[4];
    const float maxjump[4] = {1e0f, 1e0f, 1e2f, 2e0f};
    /* kernel_CenterofMass2D (GPUgaussLib.cuh:207-227) */
    float tx = 0.0f, ty = 0.0f, ts = 0.0f;
    for (int ii = 0; ii < sz; ii++)
        for (int jj = 0; jj < sz; jj++) {
            float v = d[sz * jj + ii];
            tx += v * ii;
            ty += v * jj;
            ts += v;
        }
    theta[0] = tx / ts;
    theta[1] = ty / ts;
    /* kernel_GaussFMaxMin2D (:230-258) with the distinct weights tabulated */
    float w[2 * MAXSZ - 1];
    {
        const float norm = 1.0f / 2.0f / sigma / sigma;
        for (int q = -(sz - 1); q <= sz - 1; ++q) w[q + sz - 1] = expf(-(float)(q * q) * norm);
    }
    float Nmax = 0.0f, MinBG = 10e10f;
    for (int kk = 0; kk < sz; kk++)
        for (int ll = 0; ll < sz; ll++) {
            float fp = 0.0f, sum = 0.0f;
            for (int ii = 0; ii < sz; ii++)
                for (int jj = 0; jj < sz; jj++) {
                    float ww = w[ii - kk + sz - 1] * w[ll - jj + sz - 1];
                    fp += ww * d[ii * sz + jj];
                    sum += ww;
                }
            fp /= sum;
            Nmax = fmaxf(Nmax, fp);
            MinBG = fminf(MinBG, fp);
        }
    theta[3] = MinBG;
    theta[2] = fmaxf(0.0f, (Nmax - theta[3]) * 2 * 2 * MLE_PI * sigma * sigma);

    float px[MAXSZ], py[MAXSZ], dx1[MAXSZ], dx2[MAXSZ], dy1[MAXSZ], dy2[MAXSZ];
    for (int kk = 0; kk < iterations; kk++) {
        float num[4] = {0.0f, 0.0f, 0.0f, 0.0f}, den[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int q = 0; q < sz; ++q) {
            px[q] = int_gauss(q, theta[0], sigma);
            py[q] = int_gauss(q, theta[1], sigma);
            dgauss_axis(q, theta[0], sigma, theta[2], &dx1[q], &dx2[q]);
            dgauss_axis(q, theta[1], sigma, theta[2], &dy1[q], &dy2[q]);
        }
        for (int ii = 0; ii < sz; ii++)
            for (int jj = 0; jj < sz; jj++) {
                float PSFx = px[ii], PSFy = py[jj];
                float model = theta[3] + theta[2] * PSFx * PSFy;
                float data_v = d[sz * jj + ii];
                float dudt[4], d2udt2[4];
                dudt[0] = dx1[ii] * PSFy;
                d2udt2[0] = dx2[ii] * PSFy;
                dudt[1] = dy1[jj] * PSFx;
                d2udt2[1] = dy2[jj] * PSFx;
                dudt[2] = PSFx * PSFy;
                d2udt2[2] = 0.0f;
                dudt[3] = 1.0f;
                d2udt2[3] = 0.0f;
                float cf = 0.0f, df = 0.0f;
                if (model > 10e-3f) cf = data_v / model - 1;
                if (model > 10e-3f) df = data_v / (model * model);
                cf = fminf(cf, 10e4f);
                df = fminf(df, 10e4f);
                for (int l = 0; l < 4; l++) {
                    num[l] += dudt[l] * cf;
                    den[l] += d2udt2[l] * cf - (dudt[l] * dudt[l]) * df;
                }
            }
        theta[0] -= fminf(fmaxf(num[0] / den[0], -maxjump[0]), maxjump[0]);
        theta[1] -= fminf(fmaxf(num[1] / den[1], -maxjump[1]), maxjump[1]);
        theta[2] -= fminf(fmaxf(num[2] / den[2], -theta[2]), theta[2]);
        theta[3] -= fminf(fmaxf(num[3] / den[3], -theta[3]), theta[3]);
        theta[2] = fmaxf(theta[2], 1.0f);
        theta[3] = fmaxf(theta[3], 0.01f);
    }

    /* Fisher information, log-likelihood (cuda_gaussMLEv2.cu:104-130) */
    float M[16];
    for (int q = 0; q < 16; ++q) M[q] = 0.0f;
    float Div = 0.0f;
    for (int q = 0; q < sz; ++q) {
        px[q] = int_gauss(q, theta[0], sigma);
        py[q] = int_gauss(q, theta[1], sigma);
        dgauss_axis(q, theta[0], sigma, theta[2], &dx1[q], &dx2[q]);
        dgauss_axis(q, theta[1], sigma, theta[2], &dy1[q], &dy2[q]);
    }
    for (int ii = 0; ii < sz; ii++)
        for (int jj = 0; jj < sz; jj++) {
            float PSFx = px[ii], PSFy = py[jj];
            float model = theta[3] + theta[2] * PSFx * PSFy;
            float data_v = d[sz * jj + ii];
            float dudt[4] = {dx1[ii] * PSFy, dy1[jj] * PSFx, PSFx * PSFy, 1.0f};
            for (int a = 0; a < 4; a++)
                for (int b = a; b < 4; b++) {
                    M[a * 4 + b] += dudt[b] * dudt[a] / model;
                    M[b * 4 + a] = M[a * 4 + b];
                }
            if (model > 0) {
                if (data_v > 0)
                    Div += data_v * logf(model) - model - data_v * logf(data_v) + data_v;
                else
                    Div += -model;
            }
        }
    /* kernel_MatInvN (MatInvLib.h:15-75): LU without pivoting, diagonal of
     * the inverse */
    const int n = 4;
    float Minv[16], yy[4], tmp1 = 0.0f;
    for (int jj = 0; jj < n; jj++) {
        for (int ii = 0; ii <= jj; ii++)
            if (ii > 0) {
                for (int q = 0; q <= ii - 1; q++) tmp1 += M[ii + q * n] * M[q + jj * n];
                M[ii + jj * n] -= tmp1;
                tmp1 = 0.0f;
            }
        for (int ii = jj + 1; ii < n; ii++)
            if (jj > 0) {
                for (int q = 0; q <= jj - 1; q++) tmp1 += M[ii + q * n] * M[q + jj * n];
                M[ii + jj * n] = (1 / M[jj + jj * n]) * (M[ii + jj * n] - tmp1);
                tmp1 = 0.0f;
            } else {
                M[ii + jj * n] = (1 / M[jj + jj * n]) * M[ii + jj * n];
            }
    }
    for (int num = 0; num < n; num++) {
        yy[0] = num == 0 ? 1.0f : 0.0f;
        for (int ii = 1; ii < n; ii++) {
            float b = ii == num ? 1.0f : 0.0f;
            for (int q = 0; q <= ii - 1; q++) tmp1 += M[ii + q * n] * yy[q];
            yy[ii] = b - tmp1;
            tmp1 = 0.0f;
        }
        Minv[n - 1 + num * n] = yy[n - 1] / M[(n - 1) + (n - 1) * n];
        for (int ii = n - 2; ii >= 0; ii--) {
            for (int q = ii + 1; q < n; q++) tmp1 += M[ii + q * n] * Minv[q + num * n];
            Minv[ii + num * n] = (1 / M[ii + ii * n]) * (yy[ii] - tmp1);
            tmp1 = 0.0f;
        }
    }
    for (int k = 0; k < 4; k++) {
        P[(int64_t)nfits * k + fit] = theta[k];
        CRLB[(int64_t)nfits * k + fit] = Minv[k * n + k];
    }
    LL[fit] = Div;
}

}  // namespace

extern "C" bamf_status bamf_gauss_mle_device(const float *rois, int sz, int nfits, float psf_sigma,
                                             int iterations, float *params, float *crlb,
                                             float *loglik, void *stream)
{
    if (!rois || !params || !crlb || !loglik || sz < 1 || nfits < 0 || iterations < 0)
        return BAMF_ERR_INVALID_ARG;
    if (sz > MAXSZ) return BAMF_ERR_TOO_LARGE;
    if (nfits == 0) return BAMF_OK;
    size_t smem = (size_t)FITS_PER_BLOCK * sz * sz * sizeof(float);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(mle_xynb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return clear_cuda_error();
    int blocks = (nfits + FITS_PER_BLOCK - 1) / FITS_PER_BLOCK;
    mle_xynb_kernel<<<blocks, FITS_PER_BLOCK, smem, (cudaStream_t)stream>>>(
        rois, psf_sigma, sz, iterations, params, crlb, loglik, nfits);
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}

extern "C" bamf_status bamf_gauss_mle_host(const float *rois, int sz, int nfits, float psf_sigma,
                                           int iterations, float *params, float *crlb,
                                           float *loglik)
{
    if (!rois || !params || !crlb || !loglik || sz < 1 || nfits < 0 || iterations < 0)
        return BAMF_ERR_INVALID_ARG;
    if (sz > MAXSZ) return BAMF_ERR_TOO_LARGE;
    if (nfits == 0) return BAMF_OK;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    float *dr = nullptr, *dp = nullptr, *dc = nullptr, *dl = nullptr;
    size_t nin = (size_t)nfits * sz * sz, nout = (size_t)nfits * 4;
    bamf_status st = BAMF_OK;
    if (cudaMalloc(&dr, nin * sizeof(float)) != cudaSuccess || cudaMalloc(&dp, nout * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&dc, nout * sizeof(float)) != cudaSuccess || cudaMalloc(&dl, nfits * sizeof(float)) != cudaSuccess)
        st = BAMF_ERR_CUDA;
    if (!st && cudaMemcpy(dr, rois, nin * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) st = BAMF_ERR_CUDA;
    if (!st) st = bamf_gauss_mle_device(dr, sz, nfits, psf_sigma, iterations, dp, dc, dl, nullptr);
    if (!st && cudaDeviceSynchronize() != cudaSuccess) st = BAMF_ERR_CUDA;
    if (!st && (cudaMemcpy(params, dp, nout * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(crlb, dc, nout * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(loglik, dl, nfits * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess))
        st = BAMF_ERR_CUDA;
    cudaFree(dr);
    cudaFree(dp);
    cudaFree(dc);
    cudaFree(dl);
    return st;
}
