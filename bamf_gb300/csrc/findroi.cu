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
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

#include "bamf.h"
#include "frontend_launch.h"

namespace {

/* rb0 = RN(1/b0); the fused filter divides by b0 through rb0 (div_fast)
 * for |q| in [lo, hi], and with IEEE division elsewhere (lo = +inf: never
 * through rb0). */
struct Coef {
    float b0, b1, b2, b3, B, rb0, lo, hi;
};

/* Division by the constant b0 with one multiply and two FMAs (Markstein,
 * "Computation of elementary functions on the IBM RISC System/6000
 * processor", IBM J. Res. Dev. 34(1), 1990): q0 = RN(q*rb0), the residual
 * b0*q0 - q in one FMA, the corrected quotient RN(q0 - residual*rb0); a zero
 * q keeps its sign.  The sequence is invariant under scaling q by a power of
 * two while no intermediate leaves the normal range, which holds for |q| in
 * [2^-100, 2^100] and b0 in [2^-20, 2^20]; so it equals RN(q/b0) on that whole
 * range iff it does for the 2^23 significands of [1, 2), which
 * fast_division_exact checks on the host, once per divisor. */
__host__ __device__ __forceinline__ float div_fast(float q, float b0, float rb0)
{
#ifdef __CUDA_ARCH__
    const float q0 = __fmul_rn(q, rb0);
    return __fmaf_rn(-__fmaf_rn(b0, q0, -q), rb0, q0);
#else
    const float q0 = q * rb0;
    return std::fma(-std::fma(b0, q0, -q), rb0, q0);
#endif
}

bool fast_division_exact(float b0, float rb0)
{
    if (!(std::fabs(b0) >= 0x1p-20f && std::fabs(b0) <= 0x1p20f)) return false;
    static std::mutex mu;
    static std::vector<std::pair<float, bool>> seen;
    std::lock_guard<std::mutex> lock(mu);
    for (const auto &s : seen)
        if (std::memcmp(&s.first, &b0, sizeof b0) == 0) return s.second;
    constexpr int NT = 8;
    std::atomic<bool> ok{true};
    std::vector<std::thread> th;
    for (int k = 0; k < NT; ++k)
        th.emplace_back([&, k] {
            for (uint32_t m = (uint32_t)k; m < (1u << 23) && ok.load(std::memory_order_relaxed); m += NT) {
                const uint32_t bits = 0x3f800000u | m;
                float q;
                std::memcpy(&q, &bits, sizeof q);
                const float want = q / b0, got = div_fast(q, b0, rb0);
                if (std::memcmp(&want, &got, sizeof got) != 0) ok = false;
            }
        });
    for (auto &t : th) t.join();
    seen.emplace_back(b0, ok.load());
    return ok.load();
}

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
    Coef c{(float)B0, (float)B1, (float)B2, (float)B3, (float)B, 0.0f, INFINITY, 0.0f};
    c.rb0 = 1.0f / c.b0;
    if (fast_division_exact(c.b0, c.rb0)) {
        c.lo = 0x1p-100f;
        c.hi = 0x1p100f;
    }
    return c;
}

__device__ __forceinline__ float iir_q(float w1, float w2, float w3, const Coef &c)
{
    return __fmaf_rn(c.b3, w3, __fmaf_rn(c.b1, w1, __fmul_rn(c.b2, w2)));
}

__device__ __forceinline__ float iir_step(float w0, float w1, float w2, float w3, const Coef &c)
{
    return __fmaf_rn(w0, c.B, __fdiv_rn(iir_q(w1, w2, w3, c), c.b0));
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

/* Passes 1 and 2 fused, for whole frames (frames of up to FF_MAX_SLOT
 * pixels per intermediate image; larger frames take rows_kernel +
 * cols_kernel).  One CTA owns one frame at a time, persistent over the
 * stack, and keeps the frame's two intermediate images in its own slot of
 * `scratch`: column-major, pixel (r, j) at j*YP + r with YP = Y rounded up to
 * 32, 2*X*YP floats.  The grid's slots together stay within L2, so only the
 * frames are read from DRAM and only the DoG is written.  The recurrences
 * run exactly as in rows_kernel / cols_kernel (bit-identical results):
 *   rows, forward:  thread r walks its row through shared-memory chunks of
 *                   FF_CW columns (cp.async, double-buffered) and writes each
 *                   output to the slot (consecutive r: coalesced)
 *   rows, backward: the slot's chunks come back through shared memory, last
 *                   first; outputs overwrite the forward ones in place
 *   cols, forward:  tiles of FF_CW rows x FF_T columns, [column][FF_TS]:
 *                   thread c walks column c in float4 steps (conflict-free),
 *                   results go back into the tile and the tile to the slot
 *   cols, backward: the same, last tile first, the DoG written to `dog` in
 *                   frame layout (consecutive c: coalesced) */
constexpr int FF_T = 256;   /* threads: rows of a row group / columns of a column group */
constexpr int FF_CW = 32;   /* columns per row-pass chunk, rows per column-pass tile */
constexpr int FF_TS = 36;   /* tile row stride in floats: 16-byte rows, float4 reads conflict-free */
constexpr size_t FF_MAX_SLOT = 80 * 1024; /* pixels per image in a slot (X * YP) */
/* per warp: the largest phase, two buffers of column tiles [sigma][32 columns][FF_TS] */
constexpr int FF_WARP_FLOATS = 2 * 2 * 32 * FF_TS;
constexpr int FF_SMEM_FLOATS = (FF_T / 32) * FF_WARP_FLOATS;

/* L2 eviction priorities: the frames and the DoG stream through L2 once
 * (evict first); the slots are reused all the time (evict last) and are
 * discarded at the end of each frame instead of being written back. */
__device__ __forceinline__ uint64_t l2_evict_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint64_t l2_evict_last()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ void cp_async16(float *smem, const float *gmem, uint64_t pol)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "l"(pol)
                 : "memory");
}

__device__ __forceinline__ void cp_async4(float *smem, const float *gmem, uint64_t pol)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "l"(pol)
                 : "memory");
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

/* all but the most recent group landed */
__device__ __forceinline__ void cp_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

__device__ __forceinline__ void st_hint(float *g, float v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(g), "f"(v), "l"(pol));
}

/* st_hint at g + OFF bytes, the offset folded into the address */
template <int OFF>
__device__ __forceinline__ void st_hint_at(float *g, float v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.f32 [%0+%3], %1, %2;" ::"l"(g), "f"(v), "l"(pol), "n"(OFF));
}

/* v0..v3 to g[0], g[stride], g[2 stride], g[3 stride]; with the stride
 * known at compile time (S > 0) the offsets are immediates */
template <int S>
__device__ __forceinline__ void st_hint_4(float *g, int stride, float v0, float v1, float v2, float v3, uint64_t pol)
{
    if (S > 0) {
        st_hint_at<0>(g, v0, pol);
        st_hint_at<4 * S>(g, v1, pol);
        st_hint_at<8 * S>(g, v2, pol);
        st_hint_at<12 * S>(g, v3, pol);
    } else {
        st_hint(g, v0, pol);
        st_hint(g + stride, v1, pol);
        st_hint(g + 2 * (size_t)stride, v2, pol);
        st_hint(g + 3 * (size_t)stride, v3, pol);
    }
}

__device__ __forceinline__ void st4_hint(float *g, float4 v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(g), "f"(v.x), "f"(v.y),
                 "f"(v.z), "f"(v.w), "l"(pol));
}

__device__ __forceinline__ void discard_line(const float *g)
{
    asm volatile("discard.global.L2 [%0], 128;" ::"l"(g) : "memory");
}

struct IirState {
    float w1, w2, w3;
    __device__ __forceinline__ void init(float v) { w1 = w2 = w3 = v; }
    __device__ __forceinline__ void push(float o)
    {
        w3 = w2;
        w2 = w1;
        w1 = o;
    }
    /* one step, IEEE division */
    __device__ __forceinline__ float step(float w0, const Coef &c)
    {
        const float o = iir_step(w0, w1, w2, w3, c);
        push(o);
        return o;
    }
    /* one step, division through rb0; `slow` records a q outside [lo, hi] */
    __device__ __forceinline__ float step_fast(float w0, const Coef &c, bool &slow)
    {
        const float q = iir_q(w1, w2, w3, c);
        slow |= !(fabsf(q) >= c.lo && fabsf(q) <= c.hi);
        const float o = __fmaf_rn(w0, c.B, div_fast(q, c.b0, c.rb0));
        push(o);
        return o;
    }
};

/* Four steps of both recurrences, inputs xa / xb to outputs ya / yb in
 * processing order.  A block in which any q left [lo, hi] is redone from
 * its saved state with IEEE division, so every output is the one iir_step
 * gives. */
__device__ __forceinline__ void steps4(IirState &a, IirState &b, const Coef &ca, const Coef &cb,
                                       const float (&xa)[4], const float (&xb)[4], float (&ya)[4], float (&yb)[4])
{
    const IirState a0 = a, b0 = b;
    bool slow = false;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        ya[u] = a.step_fast(xa[u], ca, slow);
        yb[u] = b.step_fast(xb[u], cb, slow);
    }
    if (slow) {
        a = a0;
        b = b0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            ya[u] = a.step(xa[u], ca);
            yb[u] = b.step(xb[u], cb);
        }
    }
}

/* F > 0: frames of F x F pixels (YP = F), the strides compile-time */
template <bool VEC, int F>
__global__ void __launch_bounds__(FF_T, 1) filter_kernel(const float *__restrict__ in, float *__restrict__ dog,
                                                         float *__restrict__ scratch, int X_, int Y_, int Z, int YP_,
                                                         Coef ca, Coef cb)
{
    const int X = F > 0 ? F : X_, Y = F > 0 ? F : Y_, YP = F > 0 ? F : YP_;
    extern __shared__ __align__(16) float fsm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t pf = l2_evict_first(), pl = l2_evict_last();
    const size_t img = (size_t)X * YP;
    float *FA = scratch + (size_t)blockIdx.x * 2 * img, *FB = FA + img;
    float *wsm = fsm + warp * FF_WARP_FLOATS; /* this warp's chunks and tiles */
    const int nch = (X + FF_CW - 1) / FF_CW, nq = (Y + FF_CW - 1) / FF_CW;
    for (int z = blockIdx.x; z < Z; z += gridDim.x) {
        const float *fin = in + (size_t)z * X * Y;
        /* rows: the warp's 32 rows of each group of FF_T */
        for (int rg = 32 * warp; rg < Y; rg += FF_T) {
            const int nr = min(32, Y - rg), r = rg + lane;
            const bool mine = lane < nr;
            IirState a, b;
            /* ---- rows, forward: input chunk [row][FF_TS] */
            auto stage_in = [&](int c, float *buf) {
                const int c0 = c * FF_CW, w = min(FF_CW, X - c0);
                if (VEC) {
                    const int p = lane & 7;
                    if (4 * p < w)
                        for (int i = lane >> 3; i < nr; i += 4)
                            cp_async16(buf + i * FF_TS + 4 * p, fin + (size_t)(rg + i) * X + c0 + 4 * p, pf);
                } else if (lane < w) {
                    for (int i = 0; i < nr; ++i)
                        cp_async4(buf + i * FF_TS + lane, fin + (size_t)(rg + i) * X + c0 + lane, pf);
                }
            };
            stage_in(0, wsm);
            cp_commit();
            for (int c = 0; c < nch; ++c) {
                if (c + 1 < nch) stage_in(c + 1, wsm + ((c + 1) & 1) * 32 * FF_TS);
                cp_commit();
                cp_wait_prev();
                __syncwarp();
                const float *ti = wsm + (c & 1) * 32 * FF_TS + lane * FF_TS;
                const int c0 = c * FF_CW, w = min(FF_CW, X - c0);
                if (mine) {
                    if (c == 0) {
                        a.init(ti[0]);
                        b.init(ti[0]);
                    }
                    float *pa = FA + (size_t)c0 * YP + r, *pb = FB + (size_t)c0 * YP + r;
                    if (w == FF_CW) {
#pragma unroll 1
                        for (int j4 = 0; j4 < FF_CW; j4 += 4) {
                            const float4 v = *reinterpret_cast<const float4 *>(ti + j4);
                            const float x[4] = {v.x, v.y, v.z, v.w};
                            float ya[4], yb[4];
                            steps4(a, b, ca, cb, x, x, ya, yb);
                            st_hint_4<F>(pa + (size_t)j4 * YP, YP, ya[0], ya[1], ya[2], ya[3], pl);
                            st_hint_4<F>(pb + (size_t)j4 * YP, YP, yb[0], yb[1], yb[2], yb[3], pl);
                        }
                    } else {
                        for (int j = 0; j < w; ++j) {
                            st_hint(pa + (size_t)j * YP, a.step(ti[j], ca), pl);
                            st_hint(pb + (size_t)j * YP, b.step(ti[j], cb), pl);
                        }
                    }
                }
                __syncwarp(); /* buffer c & 1 is restaged for chunk c + 2; the slot stores are seen */
            }
            /* ---- rows, backward: the warp's rows of the slot's chunks,
             * [sigma][column][32 rows] */
            constexpr int BUF = 2 * FF_CW * 32;
            auto stage_f = [&](int c, float *buf) {
                const int c0 = c * FF_CW, w = min(FF_CW, X - c0), n4 = (nr + 3) >> 2;
                const int q4 = lane & 7;
                if (q4 < n4)
                    for (int j = lane >> 3; j < w; j += 4) {
                        cp_async16(buf + j * 32 + 4 * q4, FA + (size_t)(c0 + j) * YP + rg + 4 * q4, pl);
                        cp_async16(buf + (FF_CW + j) * 32 + 4 * q4, FB + (size_t)(c0 + j) * YP + rg + 4 * q4, pl);
                    }
            };
            stage_f(nch - 1, wsm);
            cp_commit();
            for (int ci = 0; ci < nch; ++ci) {
                const int c = nch - 1 - ci;
                if (c > 0) stage_f(c - 1, wsm + ((ci + 1) & 1) * BUF);
                cp_commit();
                cp_wait_prev();
                __syncwarp();
                const float *fa = wsm + (ci & 1) * BUF + lane, *fb = fa + FF_CW * 32;
                const int c0 = c * FF_CW, w = min(FF_CW, X - c0);
                if (mine) {
                    if (ci == 0) {
                        a.init(fa[(w - 1) * 32]);
                        b.init(fb[(w - 1) * 32]);
                    }
                    float *pa = FA + (size_t)c0 * YP + r, *pb = FB + (size_t)c0 * YP + r;
                    if (w == FF_CW) {
#pragma unroll 1
                        for (int j4 = FF_CW - 4; j4 >= 0; j4 -= 4) {
                            const float xa[4] = {fa[(j4 + 3) * 32], fa[(j4 + 2) * 32], fa[(j4 + 1) * 32],
                                                 fa[j4 * 32]};
                            const float xb[4] = {fb[(j4 + 3) * 32], fb[(j4 + 2) * 32], fb[(j4 + 1) * 32],
                                                 fb[j4 * 32]};
                            float ya[4], yb[4];
                            steps4(a, b, ca, cb, xa, xb, ya, yb);
                            st_hint_4<F>(pa + (size_t)j4 * YP, YP, ya[3], ya[2], ya[1], ya[0], pl);
                            st_hint_4<F>(pb + (size_t)j4 * YP, YP, yb[3], yb[2], yb[1], yb[0], pl);
                        }
                    } else {
                        for (int j = w - 1; j >= 0; --j) {
                            st_hint(pa + (size_t)j * YP, a.step(fa[j * 32], ca), pl);
                            st_hint(pb + (size_t)j * YP, b.step(fb[j * 32], cb), pl);
                        }
                    }
                }
                __syncwarp();
            }
        }
        __syncthreads(); /* every row of the frame is in the slot */
        /* columns: the warp's 32 columns of each group of FF_T, tiles
         * [sigma][column][FF_TS] of FF_CW rows */
        constexpr int TBUF = 2 * 32 * FF_TS;
        for (int cg = 32 * warp; cg < X; cg += FF_T) {
            const int nc = min(32, X - cg), col = cg + lane;
            const bool mine = lane < nc;
            auto stage_t = [&](int q, float *buf) {
                const int p = lane & 7;
                for (int c = lane >> 3; c < nc; c += 4) {
                    const size_t g = (size_t)(cg + c) * YP + q * FF_CW + 4 * p;
                    cp_async16(buf + c * FF_TS + 4 * p, FA + g, pl);
                    cp_async16(buf + (32 + c) * FF_TS + 4 * p, FB + g, pl);
                }
            };
            IirState a, b;
            /* ---- columns, forward */
            stage_t(0, wsm);
            cp_commit();
            for (int q = 0; q < nq; ++q) {
                if (q + 1 < nq) stage_t(q + 1, wsm + ((q + 1) & 1) * TBUF);
                cp_commit();
                cp_wait_prev();
                __syncwarp();
                float *buf = wsm + (q & 1) * TBUF;
                float *ta = buf + lane * FF_TS, *tb = ta + 32 * FF_TS;
                const int nr = min(FF_CW, Y - q * FF_CW);
                if (mine) {
                    if (q == 0) {
                        a.init(ta[0]);
                        b.init(tb[0]);
                    }
                    if (nr == FF_CW) {
#pragma unroll 1
                        for (int i4 = 0; i4 < FF_CW; i4 += 4) {
                            const float4 va = *reinterpret_cast<const float4 *>(ta + i4);
                            const float4 vb = *reinterpret_cast<const float4 *>(tb + i4);
                            const float xa[4] = {va.x, va.y, va.z, va.w}, xb[4] = {vb.x, vb.y, vb.z, vb.w};
                            float ya[4], yb[4];
                            steps4(a, b, ca, cb, xa, xb, ya, yb);
                            *reinterpret_cast<float4 *>(ta + i4) = make_float4(ya[0], ya[1], ya[2], ya[3]);
                            *reinterpret_cast<float4 *>(tb + i4) = make_float4(yb[0], yb[1], yb[2], yb[3]);
                        }
                    } else {
                        for (int i = 0; i < nr; ++i) {
                            ta[i] = a.step(ta[i], ca);
                            tb[i] = b.step(tb[i], cb);
                        }
                    }
                }
                __syncwarp();
                {
                    const int p = lane & 7;
                    for (int c = lane >> 3; c < nc; c += 4) {
                        const size_t g = (size_t)(cg + c) * YP + q * FF_CW + 4 * p;
                        st4_hint(FA + g, *reinterpret_cast<const float4 *>(buf + c * FF_TS + 4 * p), pl);
                        st4_hint(FB + g, *reinterpret_cast<const float4 *>(buf + (32 + c) * FF_TS + 4 * p), pl);
                    }
                }
                __syncwarp(); /* buffer q & 1 is restaged for tile q + 2; the slot stores are seen */
            }
            /* ---- columns, backward, DoG out */
            stage_t(nq - 1, wsm);
            cp_commit();
            for (int qi = 0; qi < nq; ++qi) {
                const int q = nq - 1 - qi;
                if (q > 0) stage_t(q - 1, wsm + ((qi + 1) & 1) * TBUF);
                cp_commit();
                cp_wait_prev();
                __syncwarp();
                const float *ta = wsm + (qi & 1) * TBUF + lane * FF_TS, *tb = ta + 32 * FF_TS;
                const int nr = min(FF_CW, Y - q * FF_CW);
                if (mine) {
                    if (qi == 0) {
                        a.init(ta[nr - 1]);
                        b.init(tb[nr - 1]);
                    }
                    float *pd = dog + ((size_t)z * Y + (size_t)q * FF_CW) * X + col;
                    if (nr == FF_CW) {
#pragma unroll 1
                        for (int i4 = FF_CW - 4; i4 >= 0; i4 -= 4) {
                            const float4 va = *reinterpret_cast<const float4 *>(ta + i4);
                            const float4 vb = *reinterpret_cast<const float4 *>(tb + i4);
                            const float xa[4] = {va.w, va.z, va.y, va.x}, xb[4] = {vb.w, vb.z, vb.y, vb.x};
                            float ya[4], yb[4];
                            steps4(a, b, ca, cb, xa, xb, ya, yb);
                            st_hint_4<F>(pd + (size_t)i4 * X, X, __fsub_rn(ya[3], yb[3]), __fsub_rn(ya[2], yb[2]),
                                         __fsub_rn(ya[1], yb[1]), __fsub_rn(ya[0], yb[0]), pf);
                        }
                    } else {
                        for (int i = nr - 1; i >= 0; --i)
                            st_hint(pd + (size_t)i * X, __fsub_rn(a.step(ta[i], ca), b.step(tb[i], cb)), pf);
                    }
                }
                __syncwarp();
            }
        }
        __syncthreads(); /* every read of the slot is done */
        /* the frame's slot is dead: drop its lines without writing them back */
        for (size_t off = (size_t)threadIdx.x * 32; off < 2 * img; off += (size_t)FF_T * 32) discard_line(FA + off);
        __syncthreads();
    }
}


/* Passes 3 and 4, fused: kernel_maxX (window max along rows with floor
 * minval, +max / -max) then kernel_maxY (window max of |.| along columns,
 * flag where it equals the pixel within 1e-6), cuda_FindROI.cu:94-147.
 * One CTA per (32-column strip, MAX_TH-row tile, frame), over the frames
 * [z0, z1) of the Z-frame stack.
 * Row maxima: every row-max value the tile's column windows need (its rows
 * and k above and below, clamped to the frame) is formed by a warp from a
 * linear chunk of the DoG stack staged in shared memory, the strip and H =
 * k + hr values either side of it, where hr bounds how far the reference's
 * float-rounded window bounds stray from the nominal ones (0 while the
 * stack has at most 2^24 pixels; the host derives it from the float spacing
 * near n).  The bounds are formed in float over the stack's linear index
 * exactly as the reference does ((int)((fmaxf(0, c-k) + (float)(X*row)) +
 * (float)(X*Y*frame))); a window that leaves the chunk anyway (a stack past
 * 2^32 pixels, whose 32-bit frame offset wraps as the reference's does)
 * reads global memory.  An index past the stack's end (only in the very
 * last row) is left out of the max (the reference reads beyond its buffer
 * there).  The window max takes the chunk's quad maxima (max of 4
 * consecutive values) in steps of 4 and closes with the quad, pair or value
 * that ends the window (overlaps are harmless: max is idempotent).
 * Column maxima: van Herk / Gil-Werman over the tile's rows of |row max|,
 * blocks of W = 2k+1 rows from the tile's first row: g (max from the block
 * start) and h (max to the block end) per (block, column) task; a window
 * [s, e] of at most W rows is max(h[s], g[e]) across two blocks, g[e] when
 * it starts a block and h[s] when it ends one (only windows clamped to the
 * frame are shorter than W: they start at row 0 or end at the frame's last
 * row, the tile's last).  Both maxima are exact, so the flags are the
 * reference's.  WORDS (X a multiple of 32): the flags as a bit mask in
 * memory order, a warp's 32 columns of a row one word; else one byte per
 * pixel. */
constexpr int MAX_TW = 32, MAX_TH = 128, MAX_WARPS = 8, MAX_BOXSIZE = 128;

__host__ __device__ inline int maxima_cwp(int k, int hr) { return (MAX_TW + 2 * (k + hr) + 31) / 32 * 32; }

/* shared memory of maxima_kernel in 4-byte words: per warp two chunks
 * (double-buffered) and the pair and quad maxima, then the rm, g and h tiles
 * [MAX_TH + 2k][MAX_TW] and the row -> block table */
__host__ __device__ inline int maxima_smem_floats(int k, int hr)
{
    return MAX_WARPS * 4 * maxima_cwp(k, hr) + 3 * (MAX_TH + 2 * k) * MAX_TW + (MAX_TH + 2 * k);
}

template <bool IDX64, bool WORDS>
__global__ void __launch_bounds__(32 * MAX_WARPS) maxima_kernel(const float *__restrict__ dog,
                                                                uint8_t *__restrict__ flags, int X, int Y,
                                                                int Z, int z0, int z1, int k, float minval,
                                                                float eps_hi, int hr)
{
    using Idx = typename std::conditional<IDX64, int64_t, int>::type;
    extern __shared__ float sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int H = k + hr, CW = MAX_TW + 2 * H, CWP = maxima_cwp(k, hr), NR = MAX_TH + 2 * k;
    float *ch0 = sm + warp * 4 * CWP, *p1 = ch0 + 2 * CWP, *p2 = p1 + CWP;
    float *rmT = sm + MAX_WARPS * 4 * CWP, *gT = rmT + NR * MAX_TW, *hT = gT + NR * MAX_TW;
    int *bdiv = reinterpret_cast<int *>(hT + NR * MAX_TW); /* i / W for the tile's rows */
    const Idx n = (Idx)((int64_t)X * Y * Z);
    const int c0 = blockIdx.x * MAX_TW, r0 = blockIdx.y * MAX_TH, c = c0 + lane;
    const int r1 = min(Y, r0 + MAX_TH) - 1;
    const int rlo = max(0, r0 - k), rhi = min(Y - 1, r1 + k), nrows = rhi - rlo + 1;
    const int W = 2 * k + 1, nblk = (nrows + W - 1) / W;
    for (int i = threadIdx.x; i < NR; i += blockDim.x) bdiv[i] = i / W;
    const float lo = fmaxf(0.0f, (float)(c - k));
    const float hi = fminf((float)(X - 1), (float)(c + k));
    /* the chunk of row r: [cbeg, cbeg + CW) of the stack, zero outside it */
    auto stage = [&](int z, int r, float *buf) {
        const Idx cbeg = ((Idx)z * Y + r) * X + c0 - H;
        for (int i = lane; i < CW; i += 32) {
            const Idx g = cbeg + i;
            const bool in = g >= 0 && g < n;
            const unsigned d = (unsigned)__cvta_generic_to_shared(buf + i);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(in ? dog + g : dog),
                         "r"(in ? 4 : 0)
                         : "memory");
        }
    };
    for (int z = z0 + blockIdx.z; z < z1; z += gridDim.z) {
        __syncthreads(); /* the tiles of the previous frame are consumed */
        const float zb = __uint2float_rn((unsigned)X * (unsigned)Y * (unsigned)z);
        int j = 0;
        if (rlo + warp <= rhi) stage(z, rlo + warp, ch0);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        for (int r = rlo + warp; r <= rhi; r += MAX_WARPS, ++j) {
            float *ch = ch0 + (j & 1) * CWP;
            if (r + MAX_WARPS <= rhi) stage(z, r + MAX_WARPS, ch0 + ((j + 1) & 1) * CWP);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            __syncwarp();
            for (int i = lane; i < CW - 1; i += 32) p1[i] = fmaxf(ch[i], ch[i + 1]);
            __syncwarp();
            for (int i = lane; i < CW - 3; i += 32) p2[i] = fmaxf(p1[i], p1[i + 2]);
            __syncwarp();
            float rmv = 0.0f;
            if (c < X) {
                const Idx cbeg = ((Idx)z * Y + r) * X + c0 - H;
                const float rb = __uint2float_rn((unsigned)X * (unsigned)r);
                const Idx start = (Idx)__fadd_rn(__fadd_rn(lo, rb), zb);
                Idx end = (Idx)__fadd_rn(__fadd_rn(hi, rb), zb);
                if (end > n - 1) end = n - 1;
                float maxval = minval;
                const Idx s = start - cbeg, e = end - cbeg;
                if (s >= 0 && e < CW) {
                    const int si = (int)s, ei = (int)e;
                    /* the first six quads unrolled and predicated (windows
                     * of up to 2k+1+2*(float spacing/2): 23 values at 2000
                     * frames of 256x256, k = 7), then any further quads */
#pragma unroll
                    for (int q = 0; q < 6; ++q)
                        if (si + 4 * q + 3 <= ei) maxval = fmaxf(maxval, p2[si + 4 * q]);
                    int i = si + 4 * min(6, (ei - si + 1) >> 2);
                    for (; i + 3 <= ei; i += 4) maxval = fmaxf(maxval, p2[i]);
                    if (i <= ei)
                        maxval = fmaxf(maxval, ei - 3 >= si ? p2[ei - 3] : (ei > si ? fmaxf(p1[si], p1[ei - 1]) : ch[si]));
                } else {
                    for (Idx i = start; i <= end; ++i) maxval = fmaxf(maxval, __ldg(&dog[i]));
                }
                const float inpixel = ch[lane + H];
                rmv = maxval > inpixel ? -maxval : (maxval == inpixel ? maxval : 0.0f);
            }
            rmT[(r - rlo) * MAX_TW + lane] = rmv;
            __syncwarp(); /* p1, p2 and this chunk are rewritten for the warp's next rows */
        }
        __syncthreads();
        for (int task = threadIdx.x; task < nblk * MAX_TW; task += blockDim.x) {
            const int col = task & (MAX_TW - 1), i0 = (task / MAX_TW) * W, i1 = min(nrows, i0 + W) - 1;
            float m = fabsf(rmT[i0 * MAX_TW + col]);
            gT[i0 * MAX_TW + col] = m;
            for (int i = i0 + 1; i <= i1; ++i) {
                m = fmaxf(m, fabsf(rmT[i * MAX_TW + col]));
                gT[i * MAX_TW + col] = m;
            }
            m = fabsf(rmT[i1 * MAX_TW + col]);
            hT[i1 * MAX_TW + col] = m;
            for (int i = i1 - 1; i >= i0; --i) {
                m = fmaxf(m, fabsf(rmT[i * MAX_TW + col]));
                hT[i * MAX_TW + col] = m;
            }
        }
        __syncthreads();
        if (c < X) { /* the whole warp or none of it where WORDS */
            uint8_t *fl = flags + ((int64_t)z * Y) * X + c;
            for (int r = r0 + warp; r <= r1; r += MAX_WARPS) {
                const int s = max(0, r - k) - rlo, e = min(Y - 1, r + k) - rlo;
                const int bs = bdiv[s];
                const float m = bs != bdiv[e] ? fmaxf(hT[s * MAX_TW + lane], gT[e * MAX_TW + lane])
                                              : (s == bs * W ? gT[e * MAX_TW + lane] : hT[s * MAX_TW + lane]);
                const float maxval = fmaxf(minval, m);
                const float inpixel = rmT[(r - rlo) * MAX_TW + lane];
                /* (double)d < 1e-6 for a float d is d < eps_hi, the float
                 * just above the double 1e-6 */
                const bool f = fabsf(__fsub_rn(maxval, inpixel)) < eps_hi;
                if (WORDS) {
                    const unsigned b = __ballot_sync(0xffffffffu, f);
                    if (lane == 0)
                        reinterpret_cast<uint32_t *>(flags)[(((int64_t)z * Y + r) * X + c0) >> 5] = b;
                } else {
                    fl[(int64_t)r * X] = f ? 1 : 0;
                }
            }
        }
    }
}

/* Passes 3 and 4 for rows of a multiple of 4 floats, Boxsize up to 12 and
 * stacks indexed in 32 bits (maxima_kernel takes the others): the same
 * flags from a CTA per (WIDE_TW-column strip, TH-row tile, frame) in which
 * a lane owns 4 adjacent columns.
 * Row maxima: a warp stages the strip's chunk of a row and H = k + hr values
 * either side of it (16-byte copies from the multiple of 4 at or below the
 * chunk's start), then a sparse table over it: level L holds, from each
 * index, the maximum of the 2^L values starting there; levels 1 to 3 come
 * from one pass over three staged quads in registers, higher ones from the
 * level below, up to the longest window among the warp's columns.  A window
 * [s, e], its bounds formed in float over the stack's linear index as the
 * reference forms them, is max(T_L[s], T_L[e + 1 - 2^L]) with
 * 2^L <= e - s + 1 < 2^(L+1): two overlapping halves, exact because max is
 * idempotent.  A window outside the chunk, or longer than the levels built,
 * reads global memory.
 * Column maxima: van Herk / Gil-Werman in registers, a thread per (column,
 * half of the tile's windows), blocks of W = 2k+1 rows from the half's first
 * window start: the window starting at offset j of a block is the block's
 * maximum for j = 0 and else max(h_j, g_(j-1)), h the maximum from offset j
 * to the block's end (kept from the previous block) and g the maximum from
 * the next block's start (accumulated while it is read).  Windows clamped to
 * the frame's first or last row are scanned directly.
 * KT > 0 fixes k = KT at compile time; KT = 0 takes k up to 12 at run time.
 * F > 0 fixes X = Y = F.  WORDS (X a multiple of 32): the flags as a bit
 * mask in memory order, bit p % 32 of word p / 32 for pixel p, a warp's 32
 * columns of a row being one word; else one byte per pixel. */
constexpr int WIDE_TW = 128, WIDE_WARPS = 8, WIDE_TH = 128;

/* 16-byte units staged per row: the chunk [start - H, start + WIDE_TW + H)
 * from the multiple of 4 at or below its first index */
__host__ __device__ inline int wide_units(int H) { return (((-H) & 3) + WIDE_TW + 2 * H + 3) >> 2; }
/* words per staged row or table level (level builds read up to 8 words
 * past the staged ones) */
__host__ __device__ inline int wide_cwp(int H) { return 4 * wide_units(H) + 8; }
/* per warp: two staged rows (slots 0 and 1, level 0) and level L in slot
 * L + 1 for L = 1..max(LV, 3) */
__host__ __device__ inline int wide_slots(int LV) { return (LV > 3 ? LV : 3) + 2; }
/* shared memory of maxima_wide_kernel in 4-byte words: the warps' slots,
 * then the row-max tile [TH + 2k][WIDE_TW] */
__host__ __device__ inline int wide_smem_floats(int k, int H, int LV, int TH)
{
    return WIDE_WARPS * wide_slots(LV) * wide_cwp(H) + (TH + 2 * k) * WIDE_TW;
}

__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float a, float b, float c, float d)
{
    *reinterpret_cast<float4 *>(p) = make_float4(a, b, c, d);
}

template <int KT, int F, bool WORDS>
__global__ void __launch_bounds__(32 * WIDE_WARPS, 2)
    maxima_wide_kernel(const float *__restrict__ dog, uint8_t *__restrict__ flags, int X_, int Y_, int Z, int z0,
                       int z1, int k_arg, float minval, float eps_hi, int H, int LV, int TH)
{
    const int X = F > 0 ? F : X_, Y = F > 0 ? F : Y_;
    constexpr int WMAX = KT > 0 ? 2 * KT + 1 : 25;
    const int k = KT > 0 ? KT : k_arg, W = KT > 0 ? WMAX : 2 * k + 1;
    extern __shared__ __align__(16) float sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sh = (-H) & 3, units = wide_units(H), CWP = wide_cwp(H), staged = 4 * units;
    float *wb = sm + warp * wide_slots(LV) * CWP;
    float *rmT = sm + WIDE_WARPS * wide_slots(LV) * CWP;
    const int n = X * Y * Z;
    const int c0 = blockIdx.x * WIDE_TW, r0 = blockIdx.y * TH;
    const int r1 = min(Y, r0 + TH) - 1;
    const int rlo = max(0, r0 - k), rhi = min(Y - 1, r1 + k);
    float lo[4], hi[4];
    bool on[4];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
        const int c = c0 + 4 * lane + jj;
        on[jj] = c < X;
        lo[jj] = fmaxf(0.0f, (float)(c - k));
        hi[jj] = fminf((float)(X - 1), (float)(c + k));
    }
    /* row r's chunk from index cb4 = its strip start - H - sh (a multiple of
     * 4, as is n: a unit lies wholly inside or outside the stack) */
    auto stage = [&](int z, int r, float *buf) {
        const int cb4 = (z * Y + r) * X + c0 - H - sh;
        for (int u = lane; u < units; u += 32) {
            const int g = cb4 + 4 * u;
            const bool in = g >= 0 && g < n;
            const unsigned d = (unsigned)__cvta_generic_to_shared(buf + 4 * u);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(in ? dog + g : dog),
                         "r"(in ? 16 : 0)
                         : "memory");
        }
    };
    for (int z = z0 + blockIdx.z; z < z1; z += gridDim.z) {
        __syncthreads(); /* the tile of the previous frame is consumed */
        const float zb = __uint2float_rn((unsigned)X * (unsigned)Y * (unsigned)z);
        int j = 0;
        if (rlo + warp <= rhi) stage(z, rlo + warp, wb);
        cp_commit();
        for (int r = rlo + warp; r <= rhi; r += WIDE_WARPS, ++j) {
            float *ch = wb + (j & 1) * CWP;
            if (r + WIDE_WARPS <= rhi) stage(z, r + WIDE_WARPS, wb + ((j + 1) & 1) * CWP);
            cp_commit();
            cp_wait_prev();
            __syncwarp();
            const int cb4 = (z * Y + r) * X + c0 - H - sh;
            const float rb = __uint2float_rn((unsigned)X * (unsigned)r);
            int s[4], e[4];
            int lmax = 1;
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
                const int start = (int)__fadd_rn(__fadd_rn(lo[jj], rb), zb);
                const int end = min((int)__fadd_rn(__fadd_rn(hi[jj], rb), zb), n - 1);
                s[jj] = start - cb4;
                e[jj] = end - cb4;
                if (on[jj]) lmax = max(lmax, e[jj] - s[jj] + 1);
            }
            lmax = __reduce_max_sync(0xffffffffu, lmax);
            const int nl = min(LV, 31 - __clz(lmax));
            if (nl >= 1) {
                float *t1 = wb + 2 * CWP, *t2 = wb + 3 * CWP, *t3 = wb + 4 * CWP;
                for (int q = lane; q < units; q += 32) {
                    const float4 a = ld4(ch + 4 * q), b = ld4(ch + 4 * q + 4), c = ld4(ch + 4 * q + 8);
                    const float x[11] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z};
                    float p[10], f[8];
#pragma unroll
                    for (int i = 0; i < 10; ++i) p[i] = fmaxf(x[i], x[i + 1]);
#pragma unroll
                    for (int i = 0; i < 8; ++i) f[i] = fmaxf(p[i], p[i + 2]);
                    st4(t1 + 4 * q, p[0], p[1], p[2], p[3]);
                    st4(t2 + 4 * q, f[0], f[1], f[2], f[3]);
                    st4(t3 + 4 * q, fmaxf(f[0], f[4]), fmaxf(f[1], f[5]), fmaxf(f[2], f[6]), fmaxf(f[3], f[7]));
                }
                __syncwarp();
                for (int L = 4; L <= nl; ++L) {
                    const float *prev = wb + L * CWP;
                    float *cur = wb + (L + 1) * CWP;
                    const int d = 1 << (L - 1), nq = (staged - (1 << L) + 4) >> 2;
                    for (int q = lane; q < nq; q += 32) {
                        const float4 a = ld4(prev + 4 * q), b = ld4(prev + 4 * q + d);
                        st4(cur + 4 * q, fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), fmaxf(a.w, b.w));
                    }
                    __syncwarp();
                }
            }
            /* the maximum of chunk values [a, b], 1 <= b - a + 1 < 2^(nl+1) */
            auto window = [&](int a, int b) {
                const int L = 31 - __clz(b - a + 1);
                const float *t = L == 0 ? ch : wb + (L + 1) * CWP;
                return fmaxf(t[a], t[b + 1 - (1 << L)]);
            };
            /* a lane's 4 columns are all inside the frame or all outside it
             * (X and c0 are multiples of 4), and their bounds grow with the
             * column: every window of the warp lies in the chunk, is not
             * empty and has its level built, or the per-column path runs */
            const bool fast =
                __all_sync(0xffffffffu, !on[0] || (s[0] >= 0 && e[3] < staged &&
                                                   min(min(e[0] - s[0], e[1] - s[1]), min(e[2] - s[2], e[3] - s[3])) >= 0)) &&
                lmax < (2 << nl);
            const float4 px = ld4(ch + 4 * lane + H + sh);
            const float pix[4] = {px.x, px.y, px.z, px.w};
            float rm[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (on[0]) {
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) {
                    const int a = s[jj], b = e[jj], len = b - a + 1;
                    float m = -INFINITY;
                    if (fast) {
                        m = window(a, b);
                    } else if (len > 0) {
                        if (a >= 0 && b < staged && len < (2 << nl))
                            m = window(a, b);
                        else
                            for (int i = cb4 + a; i <= cb4 + b; ++i) m = fmaxf(m, __ldg(&dog[i]));
                    }
                    const float maxval = fmaxf(minval, m);
                    rm[jj] = maxval > pix[jj] ? -maxval : (maxval == pix[jj] ? maxval : 0.0f);
                }
            }
            st4(rmT + (r - rlo) * WIDE_TW + 4 * lane, rm[0], rm[1], rm[2], rm[3]);
            __syncwarp(); /* this buffer and the levels are rewritten for the warp's next rows */
        }
        __syncthreads();
        const int cl = threadIdx.x & (WIDE_TW - 1), part = threadIdx.x / WIDE_TW;
        const int c = c0 + cl;
        if (c < X) { /* the whole warp or none of it where WORDS */
            const int64_t fl = (int64_t)z * Y * X + c; /* pixel (z, 0, c) */
            const float *col = rmT + cl;
            /* (double)d < 1e-6 for a float d is d < eps_hi, the float just
             * above the double 1e-6 */
            auto flag = [&](int64_t px, int i, float m) {
                const bool f = fabsf(__fsub_rn(fmaxf(minval, m), col[i * WIDE_TW])) < eps_hi;
                if (WORDS) {
                    const unsigned b = __ballot_sync(0xffffffffu, f);
                    if (lane == 0) reinterpret_cast<uint32_t *>(flags)[px >> 5] = b;
                } else {
                    flags[px] = f ? 1 : 0;
                }
            };
            /* rows whose window [r - k, r + k] lies in the frame; window
             * starts (tile rows) [s_lo, s_lo + cnt), split in two halves */
            const int ia = max(r0, k), ib = min(r1, Y - 1 - k);
            if (ib >= ia) {
                const int s_lo = ia - k - rlo, cnt = ib - ia + 1, half = (cnt + 1) >> 1;
                const int sb = s_lo + part * half, se = min(s_lo + cnt - 1, sb + half - 1), emax = se + 2 * k;
                if (sb <= se) {
                    /* rows past emax are read as emax: they reach only g
                     * values and blocks that no emitted window uses */
                    float v[WMAX], hp[WMAX];
#pragma unroll
                    for (int q = 0; q < WMAX; ++q)
                        if (q < W) v[q] = fabsf(col[min(sb + q, emax) * WIDE_TW]);
                    float m = -INFINITY;
#pragma unroll
                    for (int q = WMAX - 1; q >= 0; --q)
                        if (q < W) {
                            m = fmaxf(m, v[q]);
                            hp[q] = m;
                        }
                    for (int base = sb + W; base - W <= se; base += W) {
#pragma unroll
                        for (int q = 0; q < WMAX; ++q)
                            if (q < W) v[q] = fabsf(col[min(base + q, emax) * WIDE_TW]);
                        float g = -INFINITY;
                        /* this block's first output row: its byte, or the
                         * word of the warp's 32 columns, rows X apart */
                        const int64_t px0 = fl + (int64_t)(base - W + k + rlo) * X;
                        uint8_t *fb = flags + px0;
                        uint32_t *fw = reinterpret_cast<uint32_t *>(flags) + (px0 >> 5);
                        const float *ctr = col + (base - W + k) * WIDE_TW;
#pragma unroll
                        for (int q = 0; q < WMAX; ++q)
                            if (q < W) {
                                if (base - W + q <= se) {
                                    const bool f =
                                        fabsf(__fsub_rn(fmaxf(minval, fmaxf(hp[q], g)), ctr[q * WIDE_TW])) < eps_hi;
                                    if (WORDS) {
                                        const unsigned b = __ballot_sync(0xffffffffu, f);
                                        if (lane == 0) fw[q * (X >> 5)] = b;
                                    } else {
                                        fb[q * X] = f ? 1 : 0;
                                    }
                                }
                                g = fmaxf(g, v[q]);
                            }
                        m = -INFINITY;
#pragma unroll
                        for (int q = WMAX - 1; q >= 0; --q)
                            if (q < W) {
                                m = fmaxf(m, v[q]);
                                hp[q] = m;
                            }
                    }
                }
            }
            /* windows clamped to the frame: rows above k, then rows within
             * k of the last one (and not above k) */
            auto direct = [&](int r) {
                const int s = max(0, r - k) - rlo, e = min(Y - 1, r + k) - rlo;
                float m = -INFINITY;
                for (int i = s; i <= e; ++i) m = fmaxf(m, fabsf(col[i * WIDE_TW]));
                flag(fl + (int64_t)r * X, r - rlo, m);
            };
            for (int r = r0 + part; r <= min(r1, k - 1); r += 2) direct(r);
            for (int r = max(max(r0, Y - k), k) + part; r <= r1; r += 2) direct(r);
        }
    }
}

/* Compaction: chunks of CHUNK pixels, one block of 256 threads each, a
 * thread owning 32 consecutive pixels: one word of the bit mask (WORDS; n a
 * multiple of 32), or two 16-byte loads of byte flags where the 32 lie inside
 * the stack and are 16-byte aligned. */
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

template <bool WORDS>
__device__ __forceinline__ uint32_t flag_word(const uint8_t *__restrict__ flags, int64_t n, int64_t j0)
{
    if (WORDS) return j0 < n ? reinterpret_cast<const uint32_t *>(flags)[j0 >> 5] : 0u;
    return flag_bits(flags, n, j0);
}

/* phase 1: flags per chunk, chunks chunk0 + blockIdx.x. */
template <bool WORDS>
__global__ void __launch_bounds__(256) count_kernel(const uint8_t *__restrict__ flags, int64_t n,
                                                    int32_t *__restrict__ counts, int64_t chunk0)
{
    __shared__ int wsum[8];
    const int64_t c = chunk0 + blockIdx.x;
    const int64_t j0 = c * CHUNK + (int64_t)threadIdx.x * 32;
    int local = __popc(flag_word<WORDS>(flags, n, j0));
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int k = 0; k < 8; ++k) s += wsum[k];
        counts[c] = s;
    }
}

/* phase 2: exclusive scan of the chunk counts (one block, serial tiles),
 * from *total on (accumulate) or from 0; *total becomes the sum, and range,
 * when given, the [first, end) of the maxima these chunks hold. */
__global__ void scan_kernel(int32_t *__restrict__ counts, int64_t nchunks, int64_t *__restrict__ total,
                            bool accumulate, int64_t *__restrict__ range)
{
    __shared__ int64_t carry;
    __shared__ int64_t warp_sums[32];
    int64_t start = 0;
    if (threadIdx.x == 0) {
        start = accumulate ? *total : 0;
        carry = start;
    }
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
    if (threadIdx.x == 0) {
        *total = carry;
        if (range) {
            range[0] = start;
            range[1] = carry;
        }
    }
}

/* phase 3: write the flagged pixels of each chunk in memory order as MATLAB
 * 1-based (row, col, frame) = ind2sub([Ysize Xsize Zsize], m+1), plus the
 * clamped box corners of findROI.m:130-148. */
template <bool WORDS>
__global__ void __launch_bounds__(256) emit_kernel(const uint8_t *__restrict__ flags, int64_t n,
                                                   const int32_t *__restrict__ offs, int64_t chunk0, int Ysz,
                                                   int Xsz, int box, int64_t capacity,
                                                   int32_t *__restrict__ coords,
                                                   int32_t *__restrict__ corners)
{
    __shared__ int wsum[8];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    /* each thread owns 32 consecutive pixels: keeps memory order */
    const int64_t c = chunk0 + blockIdx.x;
    const int64_t j0 = c * CHUNK + (int64_t)threadIdx.x * 32;
    uint32_t bits = flag_word<WORDS>(flags, n, j0);
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
    int64_t pos = (int64_t)offs[c] + before + x - cnt;
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

/* ROI crop (findROI.m:157-160): ROIStack(:,:,b) = Image(rows, cols, Kk).
 * A warp per ROI, grid-stride over the ROIs found (the count, or the range
 * [range[0], range[1]) when given, is read on the device): the box's pixels
 * in stack order, each column's run of box pixels contiguous in the frame;
 * stores coalesced. */
__global__ void crop_kernel(const float *__restrict__ frames, int Ysz, int Xsz,
                            const int32_t *__restrict__ coords, const int32_t *__restrict__ corners,
                            const int64_t *__restrict__ count, const int64_t *__restrict__ range, int box,
                            float *__restrict__ stack, int64_t capacity)
{
    const int64_t b0 = range ? range[0] : 0, b1 = range ? range[1] : *count;
    const int64_t nroi = b1 < capacity ? b1 : capacity;
    const int lane = threadIdx.x & 31, per = box * box;
    const int64_t plane = (int64_t)Ysz * Xsz;
    for (int64_t b = b0 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); b < nroi;
         b += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const int sr = corners[2 * b], sc = corners[2 * b + 1], kk = coords[3 * b + 2];
        const float *src = frames + (int64_t)(kk - 1) * plane + (int64_t)(sc - 1) * Ysz + (sr - 1);
        float *dst = stack + b * per;
        for (int q = lane; q < per; q += 32) {
            const int col = q / box, row = q - col * box;
            dst[q] = src[(int64_t)col * Ysz + row];
        }
    }
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
    Scratch a, b, flags, chunks, total, ranges;
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

/* Passes 1-2 (the DoG) of `frames` (device) into `dog`.  With host_frames,
 * the frames are first copied from there in chunks of chunk_frames on the
 * workspace's copy stream, and each chunk's filters start on `s` as soon as
 * its copy has landed (the filters are frame-local, so a chunk is filtered
 * exactly as inside the whole stack).  Frames whose two intermediate images
 * fit a slot take the fused filter (one slot per CTA, one CTA per SM, the
 * slots in ws->b); larger frames take rows_kernel + cols_kernel (the second
 * image in ws->b).  after_chunk, when given, is called with the number of
 * frames filtered so far after each chunk's launches. */
bamf_status run_filter(bamf_findroi_ws *ws, const float *host_frames, int chunk_frames, const float *frames,
                       int KX, int KY, int zsize, double sigma1, double sigma2, float *dog, cudaStream_t s,
                       const std::function<bamf_status(int)> *after_chunk = nullptr)
{
    const Coef ca = iir_coef(sigma1), cb = iir_coef(sigma2);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int step = host_frames ? std::max(1, chunk_frames) : zsize;
    const int64_t plane = (int64_t)KX * KY, n = plane * zsize;
    const int YP = (KY + FF_CW - 1) / FF_CW * FF_CW;
    const bool fused = (size_t)KX * YP <= FF_MAX_SLOT;
    const int ff_grid = std::min(step, sms);
    const size_t b_bytes = fused ? (size_t)ff_grid * 2 * KX * YP * sizeof(float) : n * sizeof(float);
    if (!ws->b.ensure(b_bytes)) return BAMF_ERR_CUDA;
    float *Bb = (float *)ws->b.p;
    const bool vec = KX % 4 == 0 && (reinterpret_cast<uintptr_t>(frames) & 15) == 0;
    const size_t ff_smem = (size_t)FF_SMEM_FLOATS * sizeof(float);
    /* 256 x 256 frames (the common camera region) have their own build */
    auto ff = vec ? (KX == 256 && KY == 256 ? filter_kernel<true, 256> : filter_kernel<true, 0>)
                  : filter_kernel<false, 0>;
    if (fused && cudaFuncSetAttribute(ff, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ff_smem) != cudaSuccess)
        return cuda_fail();
    if (host_frames) {
        if (!ws->copy && cudaStreamCreateWithFlags(&ws->copy, cudaStreamNonBlocking) != cudaSuccess)
            return cuda_fail();
        if (!ws->landed && cudaEventCreateWithFlags(&ws->landed, cudaEventDisableTiming) != cudaSuccess)
            return cuda_fail();
        /* the copies start after the work already enqueued on s */
        if (cudaEventRecord(ws->landed, s) != cudaSuccess || cudaStreamWaitEvent(ws->copy, ws->landed, 0) != cudaSuccess)
            return cuda_fail();
    }
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
        if (fused) {
            const unsigned grid = (unsigned)std::min(zc, ff_grid);
            ff<<<grid, FF_T, ff_smem, s>>>(frames + off, dog + off, Bb, KX, KY, zc, YP, ca, cb);
        } else {
            const int64_t nrows = (int64_t)KY * zc, ncols = (int64_t)KX * zc;
            const int64_t groups = (nrows + 31) / 32;
            const unsigned grid = (unsigned)std::max<int64_t>(
                1, std::min<int64_t>((groups + ROWS_WARPS - 1) / ROWS_WARPS, (int64_t)sms * ROWS_CTAS_PER_SM));
            rows_kernel<<<grid, 32 * ROWS_WARPS, 0, s>>>(frames + off, dog + off, Bb + off, KX, KY, zc, ca, cb);
            cols_kernel<<<(unsigned)((ncols + 127) / 128), 128, 0, s>>>(dog + off, Bb + off, KX, KY, zc, ca, cb);
        }
        if (after_chunk) {
            const bamf_status r = (*after_chunk)(z0 + zc);
            if (r) return r;
        }
    }
    return launch_err();
}

/* gaussMLE of the ROIs found (bamf_find_roi_fit_pinned) */
struct FitArgs {
    float psf_sigma;
    int iterations;
    float *params, *crlb, *loglik; /* [4][capacity], [4][capacity], [capacity] */
};

/* Passes 1-5 on `frames` (device), copied first from host_frames when given
 * (run_filter; each chunk's window maxima start once it is filtered).  The
 * compaction and crop run on the whole stack at the end; with `fit`, the
 * compaction, crops and fits run after each chunk's maxima on the flag
 * chunks those complete, appended in memory order. */
bamf_status find_roi(bamf_findroi_ws *ws, const float *host_frames, int chunk_frames, const float *frames,
                     int ysize, int xsize, int zsize, double sigma1, double sigma2, int boxsize, float minval,
                     int64_t capacity, int32_t *coords, int32_t *corners, float *roi_stack, int64_t *count,
                     uint8_t *flags_out, cudaStream_t s, const FitArgs *fit = nullptr)
{
    if (!ws || !frames || !coords || !count || ysize < 1 || xsize < 1 || zsize < 1 || boxsize < 1 ||
        capacity < 0)
        return BAMF_ERR_INVALID_ARG;
    if ((roi_stack != nullptr) && corners == nullptr) return BAMF_ERR_INVALID_ARG;
    if (xsize > ysize * 64 || ysize > xsize * 64) return BAMF_ERR_INVALID_ARG;
    /* the maxima tiles hold 2 boxsize + 128 rows: boxsize up to 128 */
    if (boxsize > MAX_BOXSIZE) return BAMF_ERR_TOO_LARGE;
    const int64_t n = (int64_t)xsize * ysize * zsize;
    /* kernel view (as the reference launches it): each frame is KY = Ysize
     * runs of KX = Xsize contiguous floats (size(Image,2), findROI.m:186-189) */
    const int KX = xsize, KY = ysize;
    if (!ws->a.ensure(n * sizeof(float))) return BAMF_ERR_CUDA;
    uint8_t *flags = flags_out;
    /* without byte flags asked for, rows of a multiple of 32 pixels keep the
     * flags as a bit mask (a warp's 32 columns of a row are one word) */
    const bool words = !flags_out && KX % 32 == 0;
    if (!flags) {
        if (!ws->flags.ensure(words ? (size_t)(n / 8) : (size_t)n)) return BAMF_ERR_CUDA;
        flags = (uint8_t *)ws->flags.p;
    }
    int64_t nchunks = (n + CHUNK - 1) / CHUNK;
    if (!ws->chunks.ensure(nchunks * sizeof(int32_t)) || !ws->total.ensure(sizeof(int64_t)))
        return BAMF_ERR_CUDA;
    float *A = (float *)ws->a.p;
    /* the smallest float above the double 1e-6 */
    float eps_hi = (float)1e-6;
    if ((double)eps_hi <= 1e-6) eps_hi = std::nextafter(eps_hi, 1.0f);
    /* how far the float-rounded window bounds can stray from the nominal
     * ones: exact up to 2^24 stack pixels; above, each of the reference's two
     * float additions and its float frame offset moves a bound by at most
     * half the float spacing near n (halved while the tiles would not fit
     * shared memory: windows that stray further read global memory) */
    int hr = 0;
    if (n > (int64_t(1) << 24)) hr = 2 * (1 << std::min(7, std::max(0, std::ilogb((float)n) - 23)));
    const int hr_bound = hr;
    const bool idx64 = n > (int64_t(1) << 31) - 4096;
    /* maxima_wide_kernel where it applies: row-max tiles of WIDE_TH rows or
     * fewer and table levels for windows up to 2k + 1 + hr, within two CTAs
     * per SM (hr halved last) */
    bool wide = KX % 4 == 0 && boxsize <= 12 && !idx64 && (reinterpret_cast<uintptr_t>(A) & 15) == 0;
    int wth = WIDE_TH, wlv = 0;
    size_t wsmem = 0;
    if (wide) {
        constexpr size_t limit = 112 * 1024;
        auto size_for = [&](int th, int h) {
            wlv = 0;
            while ((2 << wlv) <= 2 * boxsize + 1 + h) ++wlv;
            return (size_t)wide_smem_floats(boxsize, boxsize + h, wlv, th) * sizeof(float);
        };
        while (wth > 32 && size_for(wth, hr) > limit) wth /= 2;
        while (hr > 0 && size_for(wth, hr) > limit) hr /= 2;
        wsmem = size_for(wth, hr);
        wide = wsmem <= limit;
    }
    if (!wide)
        while (hr > 0 && (size_t)maxima_smem_floats(boxsize, hr) * sizeof(float) > 220 * 1024) hr /= 2;
    const size_t smem = wide ? wsmem : (size_t)maxima_smem_floats(boxsize, hr) * sizeof(float);
    auto kern = idx64 ? (words ? maxima_kernel<true, true> : maxima_kernel<true, false>)
                      : (words ? maxima_kernel<false, true> : maxima_kernel<false, false>);
    const bool f256 = KX == 256 && KY == 256;
    /* the 256 x 256 builds write the bit mask; byte flags asked for take the
     * run-time build */
    auto wkern = boxsize == 7
                     ? (words ? (f256 ? maxima_wide_kernel<7, 256, true> : maxima_wide_kernel<7, 0, true>)
                              : maxima_wide_kernel<7, 0, false>)
                 : boxsize == 8
                     ? (words ? (f256 ? maxima_wide_kernel<8, 256, true> : maxima_wide_kernel<8, 0, true>)
                              : maxima_wide_kernel<8, 0, false>)
                     : (words ? maxima_wide_kernel<0, 0, true> : maxima_wide_kernel<0, 0, false>);
    if (smem > 48 * 1024 && cudaFuncSetAttribute(wide ? (const void *)wkern : (const void *)kern,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return cuda_fail();
    auto maxima = [&](int z0, int z1) {
        if (z1 <= z0) return BAMF_OK;
        if (wide) {
            dim3 grid((unsigned)((KX + WIDE_TW - 1) / WIDE_TW), (unsigned)((KY + wth - 1) / wth),
                      (unsigned)std::min(z1 - z0, 65535));
            wkern<<<grid, 32 * WIDE_WARPS, smem, s>>>(A, flags, KX, KY, zsize, z0, z1, boxsize, minval, eps_hi,
                                                      boxsize + hr, wlv, wth);
        } else {
            dim3 grid((unsigned)((KX + MAX_TW - 1) / MAX_TW), (unsigned)((KY + MAX_TH - 1) / MAX_TH),
                      (unsigned)std::min(z1 - z0, 65535));
            kern<<<grid, 32 * MAX_WARPS, smem, s>>>(A, flags, KX, KY, zsize, z0, z1, boxsize, minval, eps_hi, hr);
        }
        return launch_err();
    };
    /* frames in host memory: the maxima of a chunk's frames start once the
     * chunk is filtered, while later chunks are still being copied, except
     * the frames whose windows may reach into frames not filtered yet (the
     * float-rounded bounds reach at most k + hr_bound stack pixels past a
     * frame) */
    const int reach = 1 + (int)((int64_t)(boxsize + hr_bound) / ((int64_t)KX * KY));
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int32_t *cnt = (int32_t *)ws->chunks.p;
    int64_t *total = (int64_t *)ws->total.p;
    const unsigned crop_blocks = (unsigned)((std::min<int64_t>(std::max<int64_t>(capacity, 1), (int64_t)sms * 64) + 7) / 8);
    if (fit) {
        const int step = std::max(1, chunk_frames);
        if (!ws->ranges.ensure((size_t)2 * ((zsize + step - 1) / step + 2) * sizeof(int64_t))) return BAMF_ERR_CUDA;
    }
    /* compaction of flag chunks [cdone, c1), their maxima after those of the
     * chunks before; with `fit`, the crops and fits of those maxima */
    int64_t cdone = 0;
    int seg = 0;
    auto compact = [&](int64_t c1) -> bamf_status {
        if (c1 <= cdone) return BAMF_OK;
        const unsigned nb = (unsigned)(c1 - cdone);
        int64_t *range = fit ? (int64_t *)ws->ranges.p + 2 * seg : nullptr;
        if (words)
            count_kernel<true><<<nb, 256, 0, s>>>(flags, n, cnt, cdone);
        else
            count_kernel<false><<<nb, 256, 0, s>>>(flags, n, cnt, cdone);
        scan_kernel<<<1, 1024, 0, s>>>(cnt + cdone, c1 - cdone, total, cdone > 0, range);
        (words ? emit_kernel<true> : emit_kernel<false>)<<<nb, 256, 0, s>>>(
            flags, n, cnt, cdone, ysize, xsize, boxsize, capacity, coords, corners);
        if (fit) {
            crop_kernel<<<crop_blocks, 256, 0, s>>>(frames, ysize, xsize, coords, corners, total, range, boxsize,
                                                    roi_stack, capacity);
            const bamf_status r = launch_gauss_mle_range(roi_stack, boxsize, fit->psf_sigma, fit->iterations,
                                                         fit->params, fit->crlb, fit->loglik, capacity, range,
                                                         capacity, sms * 8, s);
            if (r) return r;
        }
        cdone = c1;
        ++seg;
        return launch_err();
    };
    int done = 0;
    const std::function<bamf_status(int)> after = [&](int filtered) {
        const int upto = filtered >= zsize ? zsize : filtered - reach;
        bamf_status r = maxima(done, upto);
        if (upto > done) done = upto;
        /* the flag chunks wholly inside frames [0, upto) */
        if (!r && fit) r = compact(upto >= zsize ? nchunks : (int64_t)upto * KX * KY / CHUNK);
        return r;
    };
    bamf_status st = run_filter(ws, host_frames, chunk_frames, frames, KX, KY, zsize, sigma1, sigma2, A, s,
                                host_frames ? &after : nullptr);
    if (st) return st;
    if ((st = maxima(done, zsize))) return st;
    if ((st = compact(nchunks))) return st;
    if (cudaMemcpyAsync(count, total, sizeof(int64_t), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return cuda_fail();
    if (!fit && roi_stack && capacity > 0)
        crop_kernel<<<crop_blocks, 256, 0, s>>>(frames, ysize, xsize, coords, corners, total, nullptr, boxsize,
                                                roi_stack, capacity);
    return launch_err();
}

/* Every float q run through div_fast and __fdiv_rn by one b0: differing
 * results with |q| in [lo, hi] (the range the filter sends through
 * div_fast) and in all (NaN results compare equal). */
__global__ void division_check_kernel(Coef c, unsigned long long *bad_in_range, unsigned long long *bad)
{
    unsigned long long n_in = 0, n_all = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (1ull << 32); i += stride) {
        const float q = __uint_as_float((unsigned)i);
        const float want = __fdiv_rn(q, c.b0), got = div_fast(q, c.b0, c.rb0);
        if (__float_as_uint(want) != __float_as_uint(got) && !(isnan(want) && isnan(got))) {
            ++n_all;
            if (fabsf(q) >= c.lo && fabsf(q) <= c.hi) ++n_in;
        }
    }
    if (n_all) atomicAdd(bad, n_all);
    if (n_in) atomicAdd(bad_in_range, n_in);
}

}  // namespace

extern "C" bamf_status bamf_find_roi_dog_device(bamf_findroi_ws *ws, const float *frames, int ysize, int xsize,
                                                int zsize, double sigma1, double sigma2, float *dog, void *stream)
{
    if (!ws || !frames || !dog || ysize < 1 || xsize < 1 || zsize < 1) return BAMF_ERR_INVALID_ARG;
    if (xsize > ysize * 64 || ysize > xsize * 64) return BAMF_ERR_INVALID_ARG;
    return run_filter(ws, nullptr, 0, frames, xsize, ysize, zsize, sigma1, sigma2, dog, (cudaStream_t)stream);
}

extern "C" bamf_status bamf_findroi_division_check(double sigma, int *host_exact,
                                                   unsigned long long *dev_mismatch_in_range,
                                                   unsigned long long *dev_mismatch)
{
    if (!host_exact) return BAMF_ERR_INVALID_ARG;
    const Coef c = iir_coef(sigma);
    *host_exact = c.lo <= c.hi;
    if (!dev_mismatch_in_range && !dev_mismatch) return BAMF_OK;
    if (!dev_mismatch_in_range || !dev_mismatch) return BAMF_ERR_INVALID_ARG;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof *d) != cudaSuccess) return cuda_fail();
    bamf_status st = BAMF_OK;
    unsigned long long h[2] = {0, 0};
    if (cudaMemset(d, 0, 2 * sizeof *d) != cudaSuccess) st = BAMF_ERR_CUDA;
    if (!st) {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        division_check_kernel<<<sms * 8, 256>>>(c, d, d + 1);
        if (cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) st = BAMF_ERR_CUDA;
    }
    if (st) cudaGetLastError();
    cudaFree(d);
    *dev_mismatch_in_range = h[0];
    *dev_mismatch = h[1];
    return st;
}

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

extern "C" bamf_status bamf_find_roi_fit_pinned(bamf_findroi_ws *ws, const float *host_frames, float *dev_frames,
                                                int chunk_frames, int ysize, int xsize, int zsize, double sigma1,
                                                double sigma2, int boxsize, float minval, int64_t capacity,
                                                float psf_sigma, int iterations, int32_t *coords,
                                                int32_t *corners, float *roi_stack, int64_t *count,
                                                float *params, float *crlb, float *loglik, void *stream)
{
    if (!host_frames || chunk_frames < 1 || !corners || !roi_stack || !params || !crlb || !loglik ||
        capacity < 1 || iterations < 0 || !(psf_sigma > 0.0f))
        return BAMF_ERR_INVALID_ARG;
    if (boxsize > GAUSS_MLE_MAX_SIZE) return BAMF_ERR_TOO_LARGE;
    const FitArgs fit{psf_sigma, iterations, params, crlb, loglik};
    return find_roi(ws, host_frames, chunk_frames, dev_frames, ysize, xsize, zsize, sigma1, sigma2, boxsize,
                    minval, capacity, coords, corners, roi_stack, count, nullptr, (cudaStream_t)stream, &fit);
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
