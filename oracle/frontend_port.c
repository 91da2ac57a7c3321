/*
 * frontend_port.c - TEST INFRASTRUCTURE: CPU restatement of the findROI /
 * gaussMLE front end.
 *
 * findROI (@RJ/findROI.m + source/cuda/cuda_FindROI/cuda_FindROI.cu):
 *   The kernels see a frame as a row-major Ysize x Xsize array whose rows
 *   are the contiguous runs of Xsize floats (for the square frames BAMF uses
 *   this is the MATLAB frame transposed).  Per frame:
 *     kernel_gaussX  3rd-order recursive Gaussian (Young & van Vliet) along
 *                    each contiguous row, forward then backward  (:10-46)
 *     kernel_gaussY  the same along each strided column            (:48-83)
 *     (for sigma1 and sigma2 separately), kernel_subtract DoG      (:85-92)
 *     kernel_maxX    row-window max with floor minval, +max/-max   (:94-117)
 *     kernel_maxY    column-window max of |.|, flag if equal       (:119-147)
 *   The recurrence temp = w0*B + (b1*w1 + b2*w2 + b3*w3)/b0 is evaluated as
 *   nvcc contracts it for the reference kernel (default -fmad=true):
 *     q = fma(b3, w3, fma(b1, w1, b2*w2)); temp = fma(w0, B, q / b0).
 *   kernel_maxX forms its window bounds in float:
 *     start = (int)((fmaxf(0, c-k) + Xsize*row) + Xsize*Ysize*frame)
 *   which rounds once the linear index passes 2^24 (frame >= 256 at
 *   256x256); the port does the same float additions.
 *   IIR coefficients: findROI.m:169-182 in double, passed to the kernel as
 *   single (MATLAB's feval cast).
 *
 * gaussMLE _XYNB_ (cuda_gaussMLEv2.cu:16-141, GPUgaussLib.cuh:14-258,
 *   MatInvLib.h:15-75): one Newton-Raphson fit of (x, y, N, bg) per ROI,
 *   restated in float and in double.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* ------------------------------------------------------------------ IIR */
static void iir_coeffs(double Sigma, float c[5])
{
    double Q;
    if (Sigma > 2.5)
        Q = 0.98711 * Sigma - 0.96330;
    else
        Q = 3.97156 - 4.14554 * sqrt(1 - 0.26891 * Sigma);
    double Qq = Q * Q;
    double Qqq = Qq * Q;
    double B0 = 1.57825 + 2.44413 * Q + 1.4281 * Qq + 0.422205 * Qqq;
    double B1 = 2.44413 * Q + 2.85619 * Qq + 1.26661 * Qqq;
    double B2 = -1.4281 * Qq - 1.26661 * Qqq;
    double B3 = 0.422205 * Qqq;
    double B = 1 - (B1 + B2 + B3) / B0;
    c[0] = (float)B0;
    c[1] = (float)B1;
    c[2] = (float)B2;
    c[3] = (float)B3;
    c[4] = (float)B;
}

static inline float iir_step(float w0, float w1, float w2, float w3, const float c[5])
{
    float q = fmaf(c[3], w3, fmaf(c[1], w1, c[2] * w2));
    return fmaf(w0, c[4], q / c[0]);
}

/* in-place filter of n values at stride s (forward then backward pass) */
static void iir_line(float *d, int n, int s, const float c[5])
{
    float w1, w2, w3, t;
    w1 = w2 = w3 = d[0];
    for (int i = 0; i < n; ++i) {
        t = iir_step(d[(size_t)i * s], w1, w2, w3, c);
        d[(size_t)i * s] = t;
        w3 = w2; w2 = w1; w1 = t;
    }
    w1 = w2 = w3 = d[(size_t)(n - 1) * s];
    for (int i = n - 1; i >= 0; --i) {
        t = iir_step(d[(size_t)i * s], w1, w2, w3, c);
        d[(size_t)i * s] = t;
        w3 = w2; w2 = w1; w1 = t;
    }
}

typedef struct {
    float *frames, *flags, *tmpA, *tmpB;
    int ysize, xsize, zsize, boxsize;
    float minval;
    float cA[5], cB[5];
    int next;
    pthread_mutex_t lock;
} fr_job;

static void findroi_frame(fr_job *j, int z)
{
    const int X = j->xsize, Y = j->ysize;
    const size_t fs = (size_t)X * Y;
    const float *src = j->frames + z * fs;
    float *A = j->tmpA + z * fs, *Bf = j->tmpB + z * fs;
    memcpy(A, src, fs * sizeof(float));
    memcpy(Bf, src, fs * sizeof(float));
    /* gaussX on rows of X contiguous floats, then gaussY on columns */
    for (int r = 0; r < Y; ++r) iir_line(A + (size_t)r * X, X, 1, j->cA);
    for (int c = 0; c < X; ++c) iir_line(A + c, Y, X, j->cA);
    for (int r = 0; r < Y; ++r) iir_line(Bf + (size_t)r * X, X, 1, j->cB);
    for (int c = 0; c < X; ++c) iir_line(Bf + c, Y, X, j->cB);
    /* kernel_subtract: A = A - B (DoG) */
    for (size_t i = 0; i < fs; ++i) A[i] = A[i] - Bf[i];
    /* kernel_maxX: Bf := +-rowmax; window bounds formed in float as the
     * reference does, over the whole stack's linear index */
    const int k = j->boxsize;
    for (int r = 0; r < Y; ++r) {
        float rowbase = (float)((unsigned)X * (unsigned)r);
        float zbase = (float)((unsigned)X * (unsigned)Y * (unsigned)z);
        for (int c = 0; c < X; ++c) {
            size_t idx = (size_t)c + (size_t)X * r;
            float lo = fmaxf(0.0f, (float)(c - k));
            float hi = fminf((float)(X - 1), (float)(c + k));
            int64_t start = (int64_t)((lo + rowbase) + zbase);
            int64_t end = (int64_t)((hi + rowbase) + zbase);
            float maxval = j->minval;
            float inpixel = A[idx];
            const int64_t base = (int64_t)fs * z; /* A holds this frame only */
            for (int64_t ii = start; ii < end + 1; ++ii) {
                int64_t li = ii - base;
                float v;
                if (li >= 0 && li < (int64_t)fs)
                    v = A[li];
                else if (li == (int64_t)fs && z + 1 < j->zsize)
                    v = NAN; /* next frame's first DoG value: filled below */
                else
                    v = NAN; /* past the stack end: ignored (fmaxf drops NaN) */
                maxval = fmaxf(maxval, v);
            }
            float out;
            if (maxval > inpixel) out = -maxval;
            else if (maxval == inpixel) out = maxval;
            else out = 0.0f;
            Bf[idx] = out;
        }
    }
    /* kernel_maxY: flags */
    float *fl = j->flags + z * fs;
    for (int c = 0; c < X; ++c) {
        for (int r = 0; r < Y; ++r) {
            size_t idx = (size_t)c + (size_t)X * r;
            int start = (int)fmaxf(0.0f, (float)(r - k));
            int end = (int)fminf((float)(Y - 1), (float)(r + k));
            float maxval = j->minval;
            float inpixel = Bf[idx];
            for (int ii = start; ii <= end; ++ii) maxval = fmaxf(maxval, fabsf(Bf[(size_t)ii * X + c]));
            fl[idx] = (double)fabsf(maxval - inpixel) < 1e-6 ? 1.0f : 0.0f;
        }
    }
}

static void *findroi_worker(void *arg)
{
    fr_job *j = (fr_job *)arg;
    for (;;) {
        pthread_mutex_lock(&j->lock);
        int z = j->next++;
        pthread_mutex_unlock(&j->lock);
        if (z >= j->zsize) break;
        findroi_frame(j, z);
    }
    return NULL;
}

/* The difference of Gaussians alone (cuda_FindROI.cu kernel_gaussX,
 * kernel_gaussY for each sigma, kernel_subtract: the first half of
 * findroi_frame) into dog, frame by frame. */
int oracle_findroi_dog(const float *frames, int ysize, int xsize, int zsize, double sigma1, double sigma2,
                       float *dog)
{
    if (!frames || !dog || ysize < 1 || xsize < 1 || zsize < 1) return BAMF_ERR_INVALID_ARG;
    const int X = xsize, Y = ysize;
    const size_t fs = (size_t)X * Y;
    float cA[5], cB[5];
    iir_coeffs(sigma1, cA);
    iir_coeffs(sigma2, cB);
    float *Bf = (float *)malloc(fs * sizeof(float));
    if (!Bf) return BAMF_ERR_INVALID_ARG;
    for (int z = 0; z < zsize; ++z) {
        float *A = dog + z * fs;
        memcpy(A, frames + z * fs, fs * sizeof(float));
        memcpy(Bf, frames + z * fs, fs * sizeof(float));
        for (int r = 0; r < Y; ++r) iir_line(A + (size_t)r * X, X, 1, cA);
        for (int c = 0; c < X; ++c) iir_line(A + c, Y, X, cA);
        for (int r = 0; r < Y; ++r) iir_line(Bf + (size_t)r * X, X, 1, cB);
        for (int c = 0; c < X; ++c) iir_line(Bf + c, Y, X, cB);
        for (size_t i = 0; i < fs; ++i) A[i] = A[i] - Bf[i];
    }
    free(Bf);
    return 0;
}

/* flags: zsize*ysize*xsize floats (1 = local maximum), memory order of the
 * input stack.  The window of kernel_maxX may cross into the next frame's
 * first DoG value when its float bounds round up (frames >= 256 at
 * 256x256); those cases are resolved after all frames are filtered. */
int oracle_findroi_filter(float *frames, int ysize, int xsize, int zsize, double sigma1,
                          double sigma2, int boxsize, float minval, float *flags, int threads)
{
    if (!frames || !flags || ysize < 1 || xsize < 1 || zsize < 1 || boxsize < 0) return BAMF_ERR_INVALID_ARG;
    size_t n = (size_t)xsize * ysize * zsize;
    fr_job j;
    memset(&j, 0, sizeof j);
    j.frames = frames;
    j.flags = flags;
    j.tmpA = (float *)malloc(n * sizeof(float));
    j.tmpB = (float *)malloc(n * sizeof(float));
    if (!j.tmpA || !j.tmpB) {
        free(j.tmpA);
        free(j.tmpB);
        return BAMF_ERR_INVALID_ARG;
    }
    j.ysize = ysize;
    j.xsize = xsize;
    j.zsize = zsize;
    j.boxsize = boxsize;
    j.minval = minval;
    iir_coeffs(sigma1, j.cA);
    iir_coeffs(sigma2, j.cB);
    pthread_mutex_init(&j.lock, NULL);
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) pthread_create(&th[t], NULL, findroi_worker, &j);
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    free(th);
    /* cross-frame windows: redo the row-max of the last row's right edge
     * of frames whose rounded window end reaches the next frame */
    const size_t fs = (size_t)xsize * ysize;
    const int X = xsize, Y = ysize, k = boxsize;
    for (int z = 0; z + 1 < zsize; ++z) {
        int r = Y - 1;
        float rowbase = (float)((unsigned)X * (unsigned)r);
        float zbase = (float)((unsigned)X * (unsigned)Y * (unsigned)z);
        int changed = 0;
        float *Arow = j.tmpA + z * fs + (size_t)X * r;
        float *Brow = j.tmpB + z * fs + (size_t)X * r;
        for (int c = 0; c < X; ++c) {
            float hi = fminf((float)(X - 1), (float)(c + k));
            int64_t end = (int64_t)((hi + rowbase) + zbase);
            int64_t last = (int64_t)fs * z + (int64_t)fs - 1;
            if (end <= last) continue;
            float lo = fmaxf(0.0f, (float)(c - k));
            int64_t start = (int64_t)((lo + rowbase) + zbase);
            float maxval = minval;
            for (int64_t ii = start; ii < end + 1; ++ii) maxval = fmaxf(maxval, j.tmpA[ii]);
            float inpixel = Arow[c];
            Brow[c] = maxval > inpixel ? -maxval : (maxval == inpixel ? maxval : 0.0f);
            changed = 1;
        }
        if (!changed) continue;
        /* recompute this frame's column maxima that see row Y-1 */
        float *fl = flags + z * fs;
        float *Bf = j.tmpB + z * fs;
        for (int c = 0; c < X; ++c)
            for (int rr = Y - 1 - k; rr < Y; ++rr) {
                if (rr < 0) continue;
                size_t idx = (size_t)c + (size_t)X * rr;
                int start = (int)fmaxf(0.0f, (float)(rr - k));
                int end = (int)fminf((float)(Y - 1), (float)(rr + k));
                float maxval = minval;
                for (int ii = start; ii <= end; ++ii) maxval = fmaxf(maxval, fabsf(Bf[(size_t)ii * X + c]));
                fl[idx] = (double)fabsf(maxval - Bf[idx]) < 1e-6 ? 1.0f : 0.0f;
            }
    }
    free(j.tmpA);
    free(j.tmpB);
    return BAMF_OK;
}

/* --------------------------------------------------------------- gaussMLE */
#define MLE_PI_F 3.141592f /* definitions.h:13 */
#define NV 4

#define DEFINE_MLE(T, SUF, EXP, ERF, SQRT, LOG, PIV, FMAX, FMIN)                                           \
    static T int_gauss_##SUF(int ii, T x, T sigma)                                             \
    {                                                                                          \
        const T norm = (T)1 / (T)2 / sigma / sigma;                                            \
        return (T)1 / (T)2 * (ERF((ii - x + (T)1) * SQRT(norm)) - ERF((ii - x) * SQRT(norm))); \
    }                                                                                          \
    static void dint_gauss_##SUF(int ii, T x, T sigma, T N, T PSFy, T *dudt, T *d2udt2)        \
    {                                                                                          \
        T a = EXP((T)-0.5 * (((ii + (T)1 - x) / sigma) * ((ii + (T)1 - x) / sigma)));          \
        T b = EXP((T)-0.5 * (((ii - x) / sigma) * ((ii - x) / sigma)));                        \
        *dudt = -N / SQRT((T)2 * PIV) / sigma * (a - b) * PSFy;                                \
        if (d2udt2)                                                                            \
            *d2udt2 = -N / SQRT((T)2 * PIV) / (sigma * sigma * sigma) *                        \
                      ((ii + (T)1 - x) * a - (ii - x) * b) * PSFy;                             \
    }                                                                                          \
    static void fit_one_##SUF(const float *d, int sz, T sigma, int iterations, T *theta_out,   \
                              T *crlb, T *ll)                                                  \
    {                                                                                          \
        T theta[NV], M[NV * NV], Minv[NV * NV], Diag[NV];                                      \
        const T maxjump[NV] = {(T)1, (T)1, (T)100, (T)2};                                      \
        memset(M, 0, sizeof M);                                                                \
        memset(Minv, 0, sizeof Minv);                                                          \
        /* CenterofMass2D (GPUgaussLib.cuh:207-227) */                                          \
        T tx = 0, ty = 0, ts = 0;                                                              \
        for (int ii = 0; ii < sz; ii++)                                                        \
            for (int jj = 0; jj < sz; jj++) {                                                  \
                tx += d[sz * jj + ii] * ii;                                                    \
                ty += d[sz * jj + ii] * jj;                                                    \
                ts += d[sz * jj + ii];                                                         \
            }                                                                                  \
        theta[0] = tx / ts;                                                                    \
        theta[1] = ty / ts;                                                                    \
        /* GaussFMaxMin2D (:230-258) */                                                         \
        T Nmax = 0, MinBG = (T)10e10;                                                          \
        const T nrm = (T)1 / (T)2 / sigma / sigma;                                             \
        for (int kk = 0; kk < sz; kk++)                                                        \
            for (int l = 0; l < sz; l++) {                                                     \
                T fp = 0, sum = 0;                                                             \
                for (int ii = 0; ii < sz; ii++)                                                \
                    for (int jj = 0; jj < sz; jj++) {                                          \
                        T w = EXP(-(T)((ii - kk) * (ii - kk)) * nrm) *                         \
                              EXP(-(T)((l - jj) * (l - jj)) * nrm);                            \
                        fp += w * d[ii * sz + jj];                                             \
                        sum += w;                                                              \
                    }                                                                          \
                fp /= sum;                                                                     \
                Nmax = FMAX(Nmax, fp);                                                         \
                MinBG = FMIN(MinBG, fp);                                                       \
            }                                                                                  \
        theta[3] = MinBG;                                                                      \
        theta[2] = FMAX((T)0, (Nmax - theta[3]) * 2 * 2 * PIV * sigma * sigma);                \
        for (int kk = 0; kk < iterations; kk++) {                                              \
            T num[NV] = {0, 0, 0, 0}, den[NV] = {0, 0, 0, 0};                                  \
            for (int ii = 0; ii < sz; ii++)                                                    \
                for (int jj = 0; jj < sz; jj++) {                                              \
                    T PSFx = int_gauss_##SUF(ii, theta[0], sigma);                             \
                    T PSFy = int_gauss_##SUF(jj, theta[1], sigma);                             \
                    T model = theta[3] + theta[2] * PSFx * PSFy;                               \
                    T data = d[sz * jj + ii];                                                  \
                    T dudt[NV], d2[NV];                                                        \
                    dint_gauss_##SUF(ii, theta[0], sigma, theta[2], PSFy, &dudt[0], &d2[0]);   \
                    dint_gauss_##SUF(jj, theta[1], sigma, theta[2], PSFx, &dudt[1], &d2[1]);   \
                    dudt[2] = PSFx * PSFy;                                                     \
                    d2[2] = 0;                                                                 \
                    dudt[3] = 1;                                                               \
                    d2[3] = 0;                                                                 \
                    T cf = 0, df = 0;                                                          \
                    if (model > (T)10e-3) cf = data / model - 1;                               \
                    if (model > (T)10e-3) df = data / (model * model);                         \
                    cf = FMIN(cf, (T)10e4);                                                    \
                    df = FMIN(df, (T)10e4);                                                    \
                    for (int l = 0; l < NV; l++) {                                             \
                        num[l] += dudt[l] * cf;                                                \
                        den[l] += d2[l] * cf - dudt[l] * dudt[l] * df;                         \
                    }                                                                          \
                }                                                                              \
            for (int l = 0; l < 2; l++)                                                        \
                theta[l] -= FMIN(FMAX(num[l] / den[l], -maxjump[l]), maxjump[l]);              \
            for (int l = 2; l < 4; l++)                                                        \
                theta[l] -= FMIN(FMAX(num[l] / den[l], -theta[l]), theta[l]);                  \
            theta[2] = FMAX(theta[2], (T)1);                                                   \
            theta[3] = FMAX(theta[3], (T)0.01);                                                \
        }                                                                                      \
        T Div = 0;                                                                             \
        for (int ii = 0; ii < sz; ii++)                                                        \
            for (int jj = 0; jj < sz; jj++) {                                                  \
                T PSFx = int_gauss_##SUF(ii, theta[0], sigma);                                 \
                T PSFy = int_gauss_##SUF(jj, theta[1], sigma);                                 \
                T model = theta[3] + theta[2] * PSFx * PSFy;                                   \
                T data = d[sz * jj + ii];                                                      \
                T dudt[NV];                                                                    \
                dint_gauss_##SUF(ii, theta[0], sigma, theta[2], PSFy, &dudt[0], NULL);         \
                dint_gauss_##SUF(jj, theta[1], sigma, theta[2], PSFx, &dudt[1], NULL);         \
                dudt[2] = PSFx * PSFy;                                                         \
                dudt[3] = 1;                                                                   \
                for (int a = 0; a < NV; a++)                                                   \
                    for (int b = a; b < NV; b++) {                                             \
                        M[a * NV + b] += dudt[b] * dudt[a] / model;                            \
                        M[b * NV + a] = M[a * NV + b];                                         \
                    }                                                                          \
                if (model > 0) {                                                               \
                    if (data > 0)                                                              \
                        Div += data * LOG(model) - model - data * LOG(data) + data;            \
                    else                                                                       \
                        Div += -model;                                                         \
                }                                                                              \
            }                                                                                  \
        /* MatInvN (MatInvLib.h:15-75): LU without pivoting, then solves */                     \
        {                                                                                      \
            T tmp1 = 0, yy[NV];                                                                \
            int n = NV;                                                                        \
            for (int jj = 0; jj < n; jj++) {                                                   \
                for (int ii = 0; ii <= jj; ii++)                                               \
                    if (ii > 0) {                                                              \
                        for (int q = 0; q <= ii - 1; q++) tmp1 += M[ii + q * n] * M[q + jj * n]; \
                        M[ii + jj * n] -= tmp1;                                                \
                        tmp1 = 0;                                                              \
                    }                                                                          \
                for (int ii = jj + 1; ii < n; ii++)                                            \
                    if (jj > 0) {                                                              \
                        for (int q = 0; q <= jj - 1; q++) tmp1 += M[ii + q * n] * M[q + jj * n]; \
                        M[ii + jj * n] = ((T)1 / M[jj + jj * n]) * (M[ii + jj * n] - tmp1);   \
                        tmp1 = 0;                                                              \
                    } else {                                                                   \
                        M[ii + jj * n] = ((T)1 / M[jj + jj * n]) * M[ii + jj * n];             \
                    }                                                                          \
            }                                                                                  \
            tmp1 = 0;                                                                          \
            for (int num = 0; num < n; num++) {                                                \
                yy[0] = num == 0 ? 1 : 0;                                                      \
                for (int ii = 1; ii < n; ii++) {                                               \
                    int b = ii == num;                                                         \
                    for (int q = 0; q <= ii - 1; q++) tmp1 += M[ii + q * n] * yy[q];           \
                    yy[ii] = b - tmp1;                                                         \
                    tmp1 = 0;                                                                  \
                }                                                                              \
                Minv[n - 1 + num * n] = yy[n - 1] / M[(n - 1) + (n - 1) * n];                  \
                for (int ii = n - 2; ii >= 0; ii--) {                                          \
                    for (int q = ii + 1; q < n; q++) tmp1 += M[ii + q * n] * Minv[q + num * n]; \
                    Minv[ii + num * n] = ((T)1 / M[ii + ii * n]) * (yy[ii] - tmp1);            \
                    tmp1 = 0;                                                                  \
                }                                                                              \
            }                                                                                  \
            for (int ii = 0; ii < n; ii++) Diag[ii] = Minv[ii * n + ii];                       \
        }                                                                                      \
        for (int l = 0; l < NV; l++) {                                                         \
            theta_out[l] = theta[l];                                                           \
            crlb[l] = Diag[l];                                                                 \
        }                                                                                      \
        *ll = Div;                                                                             \
    }

DEFINE_MLE(float, f32, expf, erff, sqrtf, logf, MLE_PI_F, fmaxf, fminf)
DEFINE_MLE(double, f64, exp, erf, sqrt, log, (double)MLE_PI_F, fmax, fmin)

typedef struct {
    const float *rois;
    int sz, nfits, iterations, dbl;
    float sigf;
    double sigd;
    float *pf, *cf, *lf;
    double *pd, *cd, *ld;
    int next;
    pthread_mutex_t lock;
} mle_job;

static void *mle_worker(void *arg)
{
    mle_job *j = (mle_job *)arg;
    for (;;) {
        pthread_mutex_lock(&j->lock);
        int i0 = j->next;
        j->next += 256;
        pthread_mutex_unlock(&j->lock);
        if (i0 >= j->nfits) break;
        int i1 = i0 + 256 < j->nfits ? i0 + 256 : j->nfits;
        for (int i = i0; i < i1; ++i) {
            const float *d = j->rois + (size_t)i * j->sz * j->sz;
            if (j->dbl) {
                double th[NV], cr[NV], ll;
                fit_one_f64(d, j->sz, j->sigd, j->iterations, th, cr, &ll);
                for (int k = 0; k < NV; ++k) {
                    j->pd[(size_t)j->nfits * k + i] = th[k];
                    j->cd[(size_t)j->nfits * k + i] = cr[k];
                }
                j->ld[i] = ll;
            } else {
                float th[NV], cr[NV], ll;
                fit_one_f32(d, j->sz, j->sigf, j->iterations, th, cr, &ll);
                for (int k = 0; k < NV; ++k) {
                    j->pf[(size_t)j->nfits * k + i] = th[k];
                    j->cf[(size_t)j->nfits * k + i] = cr[k];
                }
                j->lf[i] = ll;
            }
        }
    }
    return NULL;
}

static int run_mle(mle_job *j, int threads)
{
    pthread_mutex_init(&j->lock, NULL);
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) pthread_create(&th[t], NULL, mle_worker, j);
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    free(th);
    return BAMF_OK;
}

int oracle_gaussmle_xynb(const float *rois, int sz, int nfits, float psf_sigma, int iterations,
                         float *params, float *crlb, float *loglik, int threads)
{
    if (!rois || !params || !crlb || !loglik || sz < 1 || nfits < 0) return BAMF_ERR_INVALID_ARG;
    mle_job j;
    memset(&j, 0, sizeof j);
    j.rois = rois; j.sz = sz; j.nfits = nfits; j.iterations = iterations; j.sigf = psf_sigma;
    j.pf = params; j.cf = crlb; j.lf = loglik;
    return run_mle(&j, threads);
}

int oracle_gaussmle_xynb_f64(const float *rois, int sz, int nfits, double psf_sigma,
                             int iterations, double *params, double *crlb, double *loglik,
                             int threads)
{
    if (!rois || !params || !crlb || !loglik || sz < 1 || nfits < 0) return BAMF_ERR_INVALID_ARG;
    mle_job j;
    memset(&j, 0, sizeof j);
    j.rois = rois; j.sz = sz; j.nfits = nfits; j.iterations = iterations; j.sigd = psf_sigma;
    j.dbl = 1;
    j.pd = params; j.cd = crlb; j.ld = loglik;
    return run_mle(&j, threads);
}
