/*
 * findroi.cu - the findROI front end (@RJ/findROI.m driving
 * source/cuda/cuda_FindROI/cuda_FindROI.cu) for sm_103a.
 *
 * Frames arrive as MATLAB hands them over: Ysize x Xsize x Zsize floats,
 * y fastest.  Like the reference kernels, the passes treat each frame as a
 * row-major Ysize x Xsize array whose rows are the contiguous runs of Xsize
 * floats; for square frames this is the MATLAB frame transposed, and the
 * separable filter and the two 1-D maxima make the result the same.
 *
 * Passes (all on the device, no host round trip between them):
 *   1. rows   - recursive Gaussian (Young & van Vliet, 3rd order) along the
 *               contiguous rows, forward then backward, for sigma1 and
 *               sigma2 from one read of the frame (cuda_FindROI.cu:10-46)
 *   2. cols   - the same along the strided columns, both sigmas, then the
 *               difference of Gaussians (:48-92); lanes own columns, so
 *               every access is coalesced
 *   3. maxima - window max along rows with floor minval, +max / -max
 *               (:94-117), window bounds formed in float over the stack's
 *               linear index exactly as the reference does, then window max
 *               of |.| along columns, flag where it equals the pixel within
 *               1e-6 (:119-147), fused through shared-memory tiles
 *   5. compaction of the flags in memory order (MATLAB find, findROI.m:125),
 *      box corners (:130-148) and the ROI crop (:157-160)
 * The recurrence is evaluated with explicit IEEE operations in the order
 * nvcc gives the reference expression w0*B + (b1*w1 + b2*w2 + b3*w3)/b0:
 *   q = fma(b3, w3, fma(b1, w1, b2*w2));  out = fma(w0, B, q / b0).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bamf.h"

namespace {

struct Coef {
    float b0, b1, b2, b3, B;
};

/* findROI.m:169-182 in double; the kernel receives singles. */
Coef iir_coef(double Sigma)
{
    double Q;
    if (Sigma > 2.5)
        Q = 0.98711 * Sigma - 0.96330;
    else
        Q = 3.97156 - 4.14554 * std::sqrt(1 - 0.26891 * Sigma);
    double Qq = Q * Q, Qqq = Qq * Q;
    double B0 = 1.57825 + 2.44413 * Q + 1.4281 * Qq + 0.422205 * Qqq;
    double B1 = 2.44413 * Q + 2.85619 * Qq + 1.26661 * Qqq;
    double B2 = -1.4281 * Qq - 1.26661 * Qqq;
    double B3 = 0.422205 * Qqq;
    double B = 1 - (B1 + B2 + B3) / B0;
    return Coef{(float)B0, (float)B1, (float)B2, (float)B3, (float)B};
}

__device__ __forceinline__ float iir_step(float w0, float w1, float w2, float w3, const Coef &c)
{
    float q = __fmaf_rn(c.b3, w3, __fmaf_rn(c.b1, w1, __fmul_rn(c.b2, w2)));
    return __fmaf_rn(w0, c.B, __fdiv_rn(q, c.b0));
}

/* Pass 1: one thread per (frame, row) runs the row's recurrence for both
 * sigmas, in the reference's sequential order.  Rows are contiguous, so the
 * warp moves its 32 rows through shared memory in chunks of 32 columns: a
 * [32][33] tile is loaded with 128-byte row segments (coalesced), each
 * thread walks its own tile row (stride 33: conflict-free), and the
 * results leave the same way.  The forward results go to out_a/out_b and
 * come back chunk by chunk, last chunk first, for the backward pass; the
 * grid is persistent with ROWS_CTAS_PER_SM CTAs per SM so that the rows in
 * flight (and their forward results) stay within L2. */
constexpr int ROWS_WARPS = 3;
constexpr int ROWS_CTAS_PER_SM = 5;

__global__ void __launch_bounds__(32 * ROWS_WARPS) rows_kernel(const float *__restrict__ in,
                                                               float *__restrict__ out_a,
                                                               float *__restrict__ out_b, int X, int Y,
                                                               int Z, Coef ca, Coef cb)
{
    __shared__ float tile[ROWS_WARPS][3][32][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float(*ti)[33] = tile[warp][0];
    float(*ta_)[33] = tile[warp][1];
    float(*tb_)[33] = tile[warp][2];
    const int64_t nrows = (int64_t)Y * Z;
    const int64_t ngroups = (nrows + 31) / 32;
    const int nch = (X + 31) / 32;
    for (int64_t g = (int64_t)blockIdx.x * ROWS_WARPS + warp; g < ngroups; g += (int64_t)gridDim.x * ROWS_WARPS) {
        const int64_t row0 = g * 32;
        const int rows_here = (int)min((int64_t)32, nrows - row0);
        const bool mine = lane < rows_here;
        float a1 = 0.0f, a2 = 0.0f, a3 = 0.0f, b1 = 0.0f, b2 = 0.0f, b3 = 0.0f;
        for (int c = 0; c < nch; ++c) {
            const int c0 = c * 32, w = min(32, X - c0);
            for (int r = 0; r < rows_here; ++r)
                if (lane < w) ti[r][lane] = in[(row0 + r) * X + c0 + lane];
            __syncwarp();
            if (mine) {
                if (c == 0) {
                    a1 = a2 = a3 = ti[lane][0];
                    b1 = b2 = b3 = ti[lane][0];
                }
                for (int j = 0; j < w; ++j) {
                    float w0 = ti[lane][j];
                    float ta = iir_step(w0, a1, a2, a3, ca);
                    float tb = iir_step(w0, b1, b2, b3, cb);
                    ta_[lane][j] = ta;
                    tb_[lane][j] = tb;
                    a3 = a2; a2 = a1; a1 = ta;
                    b3 = b2; b2 = b1; b1 = tb;
                }
            }
            __syncwarp();
            for (int r = 0; r < rows_here; ++r)
                if (lane < w) {
                    out_a[(row0 + r) * X + c0 + lane] = ta_[r][lane];
                    out_b[(row0 + r) * X + c0 + lane] = tb_[r][lane];
                }
            __syncwarp();
        }
        for (int c = nch - 1; c >= 0; --c) {
            const int c0 = c * 32, w = min(32, X - c0);
            for (int r = 0; r < rows_here; ++r)
                if (lane < w) {
                    ta_[r][lane] = out_a[(row0 + r) * X + c0 + lane];
                    tb_[r][lane] = out_b[(row0 + r) * X + c0 + lane];
                }
            __syncwarp();
            if (mine) {
                if (c == nch - 1) {
                    a1 = a2 = a3 = ta_[lane][w - 1];
                    b1 = b2 = b3 = tb_[lane][w - 1];
                }
                for (int j = w - 1; j >= 0; --j) {
                    float ta = iir_step(ta_[lane][j], a1, a2, a3, ca);
                    float tb = iir_step(tb_[lane][j], b1, b2, b3, cb);
                    ta_[lane][j] = ta;
                    tb_[lane][j] = tb;
                    a3 = a2; a2 = a1; a1 = ta;
                    b3 = b2; b2 = b1; b1 = tb;
                }
            }
            __syncwarp();
            for (int r = 0; r < rows_here; ++r)
                if (lane < w) {
                    out_a[(row0 + r) * X + c0 + lane] = ta_[r][lane];
                    out_b[(row0 + r) * X + c0 + lane] = tb_[r][lane];
                }
            __syncwarp();
        }
    }
}

/* Pass 2: one thread per (frame, column): column filters of both images in
 * place, then dog = a - b written over a. */
__global__ void __launch_bounds__(128) cols_kernel(float *__restrict__ a, float *__restrict__ b,
                                                   int X, int Y, int Z, Coef ca, Coef cb)
{
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)X * Z) return;
    int64_t z = t / X, c = t - z * X;
    float *pa = a + z * (int64_t)X * Y + c, *pb = b + z * (int64_t)X * Y + c;
    float a1, a2, a3, b1, b2, b3;
    a1 = a2 = a3 = pa[0];
    b1 = b2 = b3 = pb[0];
    /* the loads of a block of COLS_PF rows are issued before its
     * recurrence steps (they do not depend on it), hiding their latency */
    constexpr int COLS_PF = 8;
    int i = 0;
    for (; i + COLS_PF <= Y; i += COLS_PF) {
        float va[COLS_PF], vb[COLS_PF];
#pragma unroll
        for (int u = 0; u < COLS_PF; ++u) {
            va[u] = pa[(int64_t)(i + u) * X];
            vb[u] = pb[(int64_t)(i + u) * X];
        }
#pragma unroll
        for (int u = 0; u < COLS_PF; ++u) {
            float ta = iir_step(va[u], a1, a2, a3, ca);
            float tb = iir_step(vb[u], b1, b2, b3, cb);
            pa[(int64_t)(i + u) * X] = ta;
            pb[(int64_t)(i + u) * X] = tb;
            a3 = a2; a2 = a1; a1 = ta;
            b3 = b2; b2 = b1; b1 = tb;
        }
    }
    for (; i < Y; ++i) {
        float ta = iir_step(pa[(int64_t)i * X], a1, a2, a3, ca);
        float tb = iir_step(pb[(int64_t)i * X], b1, b2, b3, cb);
        pa[(int64_t)i * X] = ta;
        pb[(int64_t)i * X] = tb;
        a3 = a2; a2 = a1; a1 = ta;
        b3 = b2; b2 = b1; b1 = tb;
    }
    a1 = a2 = a3 = pa[(int64_t)(Y - 1) * X];
    b1 = b2 = b3 = pb[(int64_t)(Y - 1) * X];
    i = Y - 1;
    for (; i - COLS_PF + 1 >= 0; i -= COLS_PF) {
        float va[COLS_PF], vb[COLS_PF];
#pragma unroll
        for (int u = 0; u < COLS_PF; ++u) {
            va[u] = pa[(int64_t)(i - u) * X];
            vb[u] = pb[(int64_t)(i - u) * X];
        }
#pragma unroll
        for (int u = 0; u < COLS_PF; ++u) {
            float ta = iir_step(va[u], a1, a2, a3, ca);
            float tb = iir_step(vb[u], b1, b2, b3, cb);
            pa[(int64_t)(i - u) * X] = __fsub_rn(ta, tb); /* kernel_subtract */
            a3 = a2; a2 = a1; a1 = ta;
            b3 = b2; b2 = b1; b1 = tb;
        }
    }
    for (; i >= 0; --i) {
        float ta = iir_step(pa[(int64_t)i * X], a1, a2, a3, ca);
        float tb = iir_step(pb[(int64_t)i * X], b1, b2, b3, cb);
        pa[(int64_t)i * X] = __fsub_rn(ta, tb); /* kernel_subtract */
        a3 = a2; a2 = a1; a1 = ta;
        b3 = b2; b2 = b1; b1 = tb;
    }
}

/* Passes 3 and 4, fused: kernel_maxX (window max along rows with floor
 * minval, +max / -max) then kernel_maxY (window max of |.| along columns,
 * flag where it equals the pixel within 1e-6), cuda_FindROI.cu:94-147.
 * One CTA per (32-column strip, MAX_TH-row tile, frame): every row-max value
 * the tile's column windows need (its rows and k above and below, clamped to
 * the frame) is formed from a linear chunk of the DoG stack staged in shared
 * memory, with the window bounds formed in float over the stack's linear
 * index exactly as the reference does ((int)((fmaxf(0, c-k) + (float)(X*row))
 * + (float)(X*Y*frame))); a window that leaves the staged chunk (only where
 * the float spacing of the linear index exceeds the halo, stacks beyond
 * ~2^28 pixels) reads global memory.  An index past the stack's end (only in
 * the very last row) is left out of the max (the reference reads beyond its
 * buffer there).  The column maxima then run over the staged row maxima. */
constexpr int MAX_TW = 32, MAX_TH = 128, MAX_WARPS = 8, MAX_HALO_EXTRA = 32;

__host__ __device__ inline int maxima_smem_floats(int k)
{
    return MAX_WARPS * (MAX_TW + 2 * (k + MAX_HALO_EXTRA)) + (MAX_TH + 2 * k) * MAX_TW;
}

__global__ void __launch_bounds__(32 * MAX_WARPS) maxima_kernel(const float *__restrict__ dog,
                                                                uint8_t *__restrict__ flags, int X, int Y,
                                                                int Z, int k, float minval, float eps_hi)
{
    extern __shared__ float sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int H = k + MAX_HALO_EXTRA, CW = MAX_TW + 2 * H;
    float *chunk = sm + warp * CW;
    float *rmT = sm + MAX_WARPS * CW; /* [MAX_TH + 2k][MAX_TW] */
    const int64_t n = (int64_t)X * Y * Z;
    const int c0 = blockIdx.x * MAX_TW, r0 = blockIdx.y * MAX_TH, c = c0 + lane;
    const int rlo = max(0, r0 - k), rhi = min(Y - 1, r0 + MAX_TH - 1 + k);
    for (int z = blockIdx.z; z < Z; z += gridDim.z) {
        __syncthreads(); /* rmT of the previous frame is consumed */
        for (int r = rlo + warp; r <= rhi; r += MAX_WARPS) {
            const int64_t base = ((int64_t)z * Y + r) * X + c0, cbeg = base - H;
            for (int i = lane; i < CW; i += 32) {
                const int64_t g = cbeg + i;
                chunk[i] = (g >= 0 && g < n) ? __ldg(&dog[g]) : 0.0f; /* never inside a window */
            }
            __syncwarp();
            float rmv = 0.0f;
            if (c < X) {
                const float lo = fmaxf(0.0f, (float)(c - k));
                const float hi = fminf((float)(X - 1), (float)(c + k));
                const float rb = __uint2float_rn((unsigned)X * (unsigned)r);
                const float zb = __uint2float_rn((unsigned)X * (unsigned)Y * (unsigned)z);
                const int64_t start = (int64_t)__fadd_rn(__fadd_rn(lo, rb), zb);
                int64_t end = (int64_t)__fadd_rn(__fadd_rn(hi, rb), zb);
                if (end > n - 1) end = n - 1;
                float maxval = minval;
                if (start >= cbeg && end < cbeg + CW) {
                    const int s0 = (int)(start - cbeg), s1 = (int)(end - cbeg);
#pragma unroll 4
                    for (int i = s0; i <= s1; ++i) maxval = fmaxf(maxval, chunk[i]);
                } else {
                    for (int64_t i = start; i <= end; ++i) maxval = fmaxf(maxval, __ldg(&dog[i]));
                }
                const float inpixel = chunk[lane + H];
                rmv = maxval > inpixel ? -maxval : (maxval == inpixel ? maxval : 0.0f);
            }
            rmT[(r - rlo) * MAX_TW + lane] = rmv;
            __syncwarp(); /* the chunk is restaged for the warp's next row */
        }
        __syncthreads();
        if (c < X) {
            for (int r = r0 + warp; r < min(Y, r0 + MAX_TH); r += MAX_WARPS) {
                const int start = (int)fmaxf(0.0f, (float)(r - k));
                const int end = (int)fminf((float)(Y - 1), (float)(r + k));
                float maxval = minval;
                const float *col = rmT + (start - rlo) * MAX_TW + lane;
#pragma unroll 4
                for (int i = 0; i <= end - start; ++i) maxval = fmaxf(maxval, fabsf(col[i * MAX_TW]));
                const float inpixel = rmT[(r - rlo) * MAX_TW + lane];
                /* (double)d < 1e-6 for a float d is d < eps_hi, the float
                 * just above the double 1e-6 */
                flags[((int64_t)z * Y + r) * X + c] = fabsf(__fsub_rn(maxval, inpixel)) < eps_hi ? 1 : 0;
            }
        }
    }
}

/* Compaction: chunks of CHUNK pixels, one block of 256 threads each, a
 * thread owning 32 consecutive pixels (two 16-byte loads of flags where the
 * 32 lie inside the stack and are 16-byte aligned). */
constexpr int CHUNK = 256 * 32;

/* the flags of pixels [j0, j0 + 32) as a bit mask, bit q = pixel j0 + q
 * (flags are 0 or 1: byte i of a little-endian word holds pixel i's flag in
 * its lowest bit) */
__device__ __forceinline__ uint32_t flag_bits(const uint8_t *__restrict__ flags, int64_t n, int64_t j0)
{
    uint32_t m = 0;
    if (j0 + 32 <= n && (reinterpret_cast<uintptr_t>(flags + j0) & 15) == 0) {
        const uint4 *v = reinterpret_cast<const uint4 *>(flags + j0);
        const uint4 a = v[0], b = v[1];
        const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t x = w[k];
            m |= ((x & 1u) | ((x >> 7) & 2u) | ((x >> 14) & 4u) | ((x >> 21) & 8u)) << (4 * k);
        }
    } else {
        for (int q = 0; q < 32; ++q)
            if (j0 + q < n && flags[j0 + q]) m |= 1u << q;
    }
    return m;
}

/* phase 1: flags per chunk. */
__global__ void __launch_bounds__(256) count_kernel(const uint8_t *__restrict__ flags, int64_t n,
                                                    int32_t *__restrict__ counts)
{
    __shared__ int wsum[8];
    const int64_t j0 = (int64_t)blockIdx.x * CHUNK + (int64_t)threadIdx.x * 32;
    int local = __popc(flag_bits(flags, n, j0));
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int k = 0; k < 8; ++k) s += wsum[k];
        counts[blockIdx.x] = s;
    }
}

/* phase 2: exclusive scan of the chunk counts (one block, serial tiles). */
__global__ void scan_kernel(int32_t *__restrict__ counts, int64_t nchunks,
                            int64_t *__restrict__ total)
{
    __shared__ int64_t carry;
    __shared__ int64_t warp_sums[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t b0 = 0; b0 < nchunks; b0 += blockDim.x) {
        int64_t i = b0 + threadIdx.x;
        int64_t v = i < nchunks ? counts[i] : 0;
        int64_t x = v;
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += t;
        }
        if (lane == 31) warp_sums[w] = x;
        __syncthreads();
        if (w == 0) {
            int64_t s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int64_t t = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += t;
            }
            warp_sums[lane] = s;
        }
        __syncthreads();
        int64_t incl = x + (w > 0 ? warp_sums[w - 1] : 0) + carry;
        if (i < nchunks) counts[i] = (int32_t)(incl - v);
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

/* phase 3: write the flagged pixels of each chunk in memory order as MATLAB
 * 1-based (row, col, frame) = ind2sub([Ysize Xsize Zsize], m+1), plus the
 * clamped box corners of findROI.m:130-148. */
__global__ void __launch_bounds__(256) emit_kernel(const uint8_t *__restrict__ flags, int64_t n,
                                                   const int32_t *__restrict__ offs, int Ysz,
                                                   int Xsz, int box, int64_t capacity,
                                                   int32_t *__restrict__ coords,
                                                   int32_t *__restrict__ corners)
{
    __shared__ int wsum[8];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    /* each thread owns 32 consecutive pixels: keeps memory order */
    const int64_t j0 = (int64_t)blockIdx.x * CHUNK + (int64_t)threadIdx.x * 32;
    uint32_t bits = flag_bits(flags, n, j0);
    const int cnt = __popc(bits);
    int x = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    int before = 0;
    for (int i = 0; i < w; ++i) before += wsum[i];
    int64_t pos = (int64_t)offs[blockIdx.x] + before + x - cnt;
    const int half = (int)floor(box / 2.0 + 0.5);
    while (bits) {
        const int q = __ffs(bits) - 1;
        bits &= bits - 1;
        if (pos < capacity) {
            int64_t m = j0 + q;
            int64_t plane = (int64_t)Ysz * Xsz;
            int kk = (int)(m / plane);
            int64_t rem = m - (int64_t)kk * plane;
            int jj = (int)(rem / Ysz);
            int ii = (int)(rem - (int64_t)jj * Ysz);
            int Ii = ii + 1, Jj = jj + 1, Kk = kk + 1;
            coords[3 * pos + 0] = Ii;
            coords[3 * pos + 1] = Jj;
            coords[3 * pos + 2] = Kk;
            if (corners) {
                int sr = Ii - half + 1, sc = Jj - half + 1;
                bool mr = sr < 1, mc = sc < 1;
                if (mr) sr = 1;
                if (mc) sc = 1;
                int er = mr ? box : sr + box - 1;
                int ec = mc ? box : sc + box - 1;
                if (er > Ysz) sr = Ysz - box + 1;
                if (ec > Xsz) sc = Xsz - box + 1;
                corners[2 * pos + 0] = sr; /* YBoxCorner = StartRow */
                corners[2 * pos + 1] = sc; /* XBoxCorner = StartCol */
            }
        }
        pos++;
    }
}

/* ROI crop (findROI.m:157-160): ROIStack(:,:,b) = Image(rows, cols, Kk). */
__global__ void crop_kernel(const float *__restrict__ frames, int Ysz, int Xsz,
                            const int32_t *__restrict__ coords, const int32_t *__restrict__ corners,
                            const int64_t *__restrict__ count, int box, float *__restrict__ stack,
                            int64_t capacity)
{
    int64_t nroi = *count < capacity ? *count : capacity;
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t per = (int64_t)box * box;
    if (t >= nroi * per) return;
    int64_t b = t / per;
    int p = (int)(t - b * per);
    int col = p / box, row = p - col * box;
    int sr = corners[2 * b], sc = corners[2 * b + 1], kk = coords[3 * b + 2];
    int64_t src = (int64_t)(sr - 1 + row) + (int64_t)(sc - 1 + col) * Ysz + (int64_t)(kk - 1) * Ysz * Xsz;
    stack[t] = frames[src];
}

struct Scratch {
    void *p = nullptr;
    size_t n = 0;
    ~Scratch()
    {
        if (p) cudaFree(p);
    }
    bool ensure(size_t bytes)
    {
        if (bytes <= n) return true;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        n = bytes;
        return true;
    }
};

bamf_status launch_err()
{
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}

/* a failed runtime call: clear its error so that it is not reported again
 * by a later call on this thread */
bamf_status cuda_fail()
{
    cudaGetLastError();
    return BAMF_ERR_CUDA;
}

}  // namespace

struct bamf_findroi_ws {
    Scratch a, b, flags, chunks, total;
    cudaStream_t copy = nullptr; /* host-to-device chunks of bamf_find_roi_pinned */
    cudaEvent_t landed = nullptr;
    ~bamf_findroi_ws()
    {
        if (landed) cudaEventDestroy(landed);
        if (copy) cudaStreamDestroy(copy);
    }
};

extern "C" bamf_status bamf_findroi_workspace_create(bamf_findroi_ws **ws)
{
    if (!ws) return BAMF_ERR_INVALID_ARG;
    *ws = new bamf_findroi_ws();
    return BAMF_OK;
}

extern "C" void bamf_findroi_workspace_destroy(bamf_findroi_ws *ws) { delete ws; }

namespace {

/* Passes 1-5 on `frames` (device).  With host_frames, the frames are first
 * copied from there in chunks of chunk_frames on the workspace's copy
 * stream, and each chunk's row and column filters start on `s` as soon as
 * its copy has landed (the filters are frame-local, so a chunk is filtered
 * exactly as inside the whole stack); the window maxima and everything after
 * them run on the whole stack once every chunk is filtered. */
bamf_status find_roi(bamf_findroi_ws *ws, const float *host_frames, int chunk_frames, const float *frames,
                     int ysize, int xsize, int zsize, double sigma1, double sigma2, int boxsize, float minval,
                     int64_t capacity, int32_t *coords, int32_t *corners, float *roi_stack, int64_t *count,
                     uint8_t *flags_out, cudaStream_t s)
{
    if (!ws || !frames || !coords || !count || ysize < 1 || xsize < 1 || zsize < 1 || boxsize < 1 ||
        capacity < 0)
        return BAMF_ERR_INVALID_ARG;
    if ((roi_stack != nullptr) && corners == nullptr) return BAMF_ERR_INVALID_ARG;
    if (xsize > ysize * 64 || ysize > xsize * 64) return BAMF_ERR_INVALID_ARG;
    if (boxsize > 256) return BAMF_ERR_TOO_LARGE; /* the maxima tiles stage 2 boxsize + 96 rows */
    const int64_t n = (int64_t)xsize * ysize * zsize;
    /* kernel view (as the reference launches it): each frame is KY = Ysize
     * runs of KX = Xsize contiguous floats (size(Image,2), findROI.m:186-189) */
    const int KX = xsize, KY = ysize;
    Coef ca = iir_coef(sigma1), cb = iir_coef(sigma2);
    if (!ws->a.ensure(n * sizeof(float)) || !ws->b.ensure(n * sizeof(float))) return BAMF_ERR_CUDA;
    uint8_t *flags = flags_out;
    if (!flags) {
        if (!ws->flags.ensure(n)) return BAMF_ERR_CUDA;
        flags = (uint8_t *)ws->flags.p;
    }
    int64_t nchunks = (n + CHUNK - 1) / CHUNK;
    if (!ws->chunks.ensure(nchunks * sizeof(int32_t)) || !ws->total.ensure(sizeof(int64_t)))
        return BAMF_ERR_CUDA;
    float *A = (float *)ws->a.p, *Bb = (float *)ws->b.p;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (host_frames) {
        if (!ws->copy && cudaStreamCreateWithFlags(&ws->copy, cudaStreamNonBlocking) != cudaSuccess)
            return cuda_fail();
        if (!ws->landed && cudaEventCreateWithFlags(&ws->landed, cudaEventDisableTiming) != cudaSuccess)
            return cuda_fail();
        /* the copies start after the work already enqueued on s */
        if (cudaEventRecord(ws->landed, s) != cudaSuccess || cudaStreamWaitEvent(ws->copy, ws->landed, 0) != cudaSuccess)
            return cuda_fail();
    }
    const int step = host_frames ? std::max(1, chunk_frames) : zsize;
    const int64_t plane = (int64_t)KX * KY;
    for (int z0 = 0; z0 < zsize; z0 += step) {
        const int zc = std::min(step, zsize - z0);
        const int64_t off = z0 * plane;
        if (host_frames) {
            if (cudaMemcpyAsync((float *)frames + off, host_frames + off, (size_t)(zc * plane) * sizeof(float),
                                cudaMemcpyHostToDevice, ws->copy) != cudaSuccess ||
                cudaEventRecord(ws->landed, ws->copy) != cudaSuccess ||
                cudaStreamWaitEvent(s, ws->landed, 0) != cudaSuccess)
                return cuda_fail();
        }
        const int64_t nrows = (int64_t)KY * zc, ncols = (int64_t)KX * zc;
        const int64_t groups = (nrows + 31) / 32;
        const unsigned grid = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>((groups + ROWS_WARPS - 1) / ROWS_WARPS, (int64_t)sms * ROWS_CTAS_PER_SM));
        rows_kernel<<<grid, 32 * ROWS_WARPS, 0, s>>>(frames + off, A + off, Bb + off, KX, KY, zc, ca, cb);
        cols_kernel<<<(unsigned)((ncols + 127) / 128), 128, 0, s>>>(A + off, Bb + off, KX, KY, zc, ca, cb);
    }
    {
        const size_t smem = (size_t)maxima_smem_floats(boxsize) * sizeof(float);
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(maxima_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return cuda_fail();
        dim3 grid((unsigned)((KX + MAX_TW - 1) / MAX_TW), (unsigned)((KY + MAX_TH - 1) / MAX_TH),
                  (unsigned)std::min(zsize, 65535));
        /* the smallest float above the double 1e-6 */
        float eps_hi = (float)1e-6;
        if ((double)eps_hi <= 1e-6) eps_hi = std::nextafter(eps_hi, 1.0f);
        maxima_kernel<<<grid, 32 * MAX_WARPS, smem, s>>>(A, flags, KX, KY, zsize, boxsize, minval, eps_hi);
    }
    count_kernel<<<(unsigned)nchunks, 256, 0, s>>>(flags, n, (int32_t *)ws->chunks.p);
    scan_kernel<<<1, 1024, 0, s>>>((int32_t *)ws->chunks.p, nchunks, (int64_t *)ws->total.p);
    emit_kernel<<<(unsigned)nchunks, 256, 0, s>>>(flags, n, (int32_t *)ws->chunks.p, ysize, xsize,
                                                  boxsize, capacity, coords, corners);
    if (cudaMemcpyAsync(count, ws->total.p, sizeof(int64_t), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return cuda_fail();
    if (roi_stack) {
        int64_t work = capacity * boxsize * boxsize;
        if (work > 0)
            crop_kernel<<<(unsigned)((work + 255) / 256), 256, 0, s>>>(frames, ysize, xsize, coords, corners,
                                                                      (int64_t *)ws->total.p, boxsize,
                                                                      roi_stack, capacity);
    }
    return launch_err();
}

}  // namespace

extern "C" bamf_status bamf_find_roi_device(bamf_findroi_ws *ws, const float *frames, int ysize,
                                            int xsize, int zsize, double sigma1, double sigma2,
                                            int boxsize, float minval, int64_t capacity,
                                            int32_t *coords, int32_t *corners, float *roi_stack,
                                            int64_t *count, uint8_t *flags_out, void *stream)
{
    return find_roi(ws, nullptr, 0, frames, ysize, xsize, zsize, sigma1, sigma2, boxsize, minval, capacity,
                    coords, corners, roi_stack, count, flags_out, (cudaStream_t)stream);
}

extern "C" bamf_status bamf_find_roi_pinned(bamf_findroi_ws *ws, const float *host_frames, float *dev_frames,
                                            int chunk_frames, int ysize, int xsize, int zsize, double sigma1,
                                            double sigma2, int boxsize, float minval, int64_t capacity,
                                            int32_t *coords, int32_t *corners, float *roi_stack,
                                            int64_t *count, uint8_t *flags_out, void *stream)
{
    if (!host_frames || chunk_frames < 1) return BAMF_ERR_INVALID_ARG;
    return find_roi(ws, host_frames, chunk_frames, dev_frames, ysize, xsize, zsize, sigma1, sigma2, boxsize,
                    minval, capacity, coords, corners, roi_stack, count, flags_out, (cudaStream_t)stream);
}

extern "C" bamf_status bamf_find_roi_host(const float *frames, int ysize, int xsize, int zsize,
                                          double sigma1, double sigma2, int boxsize, float minval,
                                          int64_t capacity, int32_t *coords, int32_t *corners,
                                          float *roi_stack, int64_t *count)
{
    if (!frames || !coords || !count || ysize < 1 || xsize < 1 || zsize < 1 || boxsize < 1 || capacity < 0)
        return BAMF_ERR_INVALID_ARG;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    bamf_findroi_ws ws;
    const int64_t n = (int64_t)xsize * ysize * zsize;
    Scratch dframes, dcoords, dcorners, dstack, dcount;
    int64_t cap = capacity > 0 ? capacity : 1;
    if (!dframes.ensure(n * sizeof(float)) || !dcoords.ensure(cap * 3 * sizeof(int32_t)) ||
        !dcorners.ensure(cap * 2 * sizeof(int32_t)) || !dcount.ensure(sizeof(int64_t)))
        return BAMF_ERR_CUDA;
    if (roi_stack && !dstack.ensure(cap * boxsize * boxsize * sizeof(float))) return BAMF_ERR_CUDA;
    if (cudaMemcpy(dframes.p, frames, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
        return cuda_fail();
    bamf_status r = bamf_find_roi_device(&ws, (float *)dframes.p, ysize, xsize, zsize, sigma1, sigma2,
                                         boxsize, minval, capacity, (int32_t *)dcoords.p,
                                         (int32_t *)dcorners.p, roi_stack ? (float *)dstack.p : nullptr,
                                         (int64_t *)dcount.p, nullptr, nullptr);
    if (r) return r;
    if (cudaDeviceSynchronize() != cudaSuccess) return cuda_fail();
    int64_t c = 0;
    cudaMemcpy(&c, dcount.p, sizeof c, cudaMemcpyDeviceToHost);
    *count = c;
    int64_t m = c < capacity ? c : capacity;
    if (m > 0) {
        cudaMemcpy(coords, dcoords.p, m * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost);
        if (corners) cudaMemcpy(corners, dcorners.p, m * 2 * sizeof(int32_t), cudaMemcpyDeviceToHost);
        if (roi_stack)
            cudaMemcpy(roi_stack, dstack.p, m * boxsize * boxsize * sizeof(float), cudaMemcpyDeviceToHost);
    }
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}
