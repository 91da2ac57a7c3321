/*
 * api_noalloc.cu - the batched sampler without any memory allocation.
 *
 * bamf_rjmcmc_batch_device needs device scratch (work-queue counters, the
 * size-class ordering of the ROIs, the prior tables, one byte per chain step
 * per ROI for the MAP count) and takes it from a bamf_workspace that grows
 * with cudaMalloc.  Some callers cannot do that: hosts that hand all device
 * memory out through their own pool (MATLAB's gpuArray allocator, a
 * framework's caching allocator) and must not see the driver's free memory
 * change underneath them, and latency-sensitive loops that cannot afford the
 * device-wide synchronisation cudaMalloc and cudaFree imply.  bamf_rjmcmc_batch_device_noalloc serves them: its scratch
 * is the fixed array below, which the CUDA runtime reserves on every device
 * when the library's device code is loaded there and keeps until the process
 * exits.
 *
 * Scratch layout (byte offsets into the array, 256-aligned sections):
 *   [0, 256)     work-queue counter per size class (cleared every call)
 *   [256, 512)   begin/end of every size class in the ROI order
 *   tables       the three prior tables: per table x[L], pdf[L], ux[L], uc[L]
 *   order        n_rois int32
 *   entries      n_rois int32 (only when map_n is wanted and n_entries is not)
 *   trace        n_rois * (N_Burnin + N_Trials) bytes (only when map_n is wanted)
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "bamf.h"
#include "sampler_common.h"
#include "sampler_launch.h"

/* a failed CUDA runtime call: clear its error so that a later call on this
 * thread does not report it again */
static inline bamf_status clear_cuda_error()
{
    cudaGetLastError();
    return BAMF_ERR_CUDA;
}

/* defined in api_sampler.cu */
bamf_status check_proposal_and_traces(const bamf_roi_batch *rois, const bamf_mcmc_params *p, int arith,
                                      const bamf_batch_results *out);
bamf_status launch_batch_order(const bamf_roi_batch *rois, int n, void *order_scratch, int32_t *class_range,
                               cudaStream_t s);
__global__ void map_n_kernel(const uint8_t *__restrict__ trace, int trace_cap,
                             const int32_t *__restrict__ n_entries, int n_rois,
                             int32_t *__restrict__ map_n);

using namespace bamf;

/* The scratch every call of the entry point uses. */
static __device__ __align__(256) unsigned char g_noalloc_scratch[BAMF_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_addr[MAX_DEVICES] = {nullptr};

/* Once per device, with that device current: the device address of the
 * array (host code only holds a stand-in for it). */
bamf_status scratch_address(unsigned char **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return BAMF_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return BAMF_ERR_CUDA;
        }
        g_scratch_addr[dev] = (unsigned char *)p;
    }
    *out = g_scratch_addr[dev];
    return BAMF_OK;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

/* Checks a prior PDF the way the workspace path does and counts the nodes
 * of its unique CDF (the Stat construction, LibRJMCMC.cpp:176-217), in
 * O(1) host memory. */
bamf_status count_unique(const float *pdf, int L, float DX, int *nu)
{
    if (!pdf || L < 1) return BAMF_ERR_INVALID_ARG;
    if (!(DX > 0.0f)) return BAMF_ERR_BAD_PRIOR;
    for (int i = 0; i < L; ++i)
        if (!(pdf[i] >= 0.0f) || std::isinf(pdf[i])) return BAMF_ERR_BAD_PRIOR;
    float cdf = 0.0f, x = 0.0f;
    int n = 1;
    for (int i = 1; i < L; ++i) {
        float c = cdf + (pdf[i] + pdf[i - 1]) * DX / 2.0f;
        if (c > 1.0f) c = 1.0f;
        float xn = x + DX;
        if (!(xn > x)) return BAMF_ERR_BAD_PRIOR;
        if (c != cdf) n++;
        cdf = c;
        x = xn;
    }
    *nu = n;
    return BAMF_OK;
}

/* Builds x, ux, uc of one table in place next to its pdf (one thread per
 * table); the float operations are the host construction's. */
__global__ void build_tables_kernel(float *t0, float *t1, float *t2, int L0, int L1, int L2, float DX)
{
    float *t = blockIdx.x == 0 ? t0 : (blockIdx.x == 1 ? t1 : t2);
    int L = blockIdx.x == 0 ? L0 : (blockIdx.x == 1 ? L1 : L2);
    if (threadIdx.x != 0) return;
    float *x = t, *pdf = t + L, *ux = t + 2 * L, *uc = t + 3 * L;
    float cdf = 0.0f;
    x[0] = 0.0f;
    ux[0] = 0.0f;
    uc[0] = 0.0f;
    int n = 1;
    for (int i = 1; i < L; ++i) {
        float c = __fadd_rn(cdf, __fdiv_rn(__fmul_rn(__fadd_rn(pdf[i], pdf[i - 1]), DX), 2.0f));
        if (c > 1.0f) c = 1.0f;
        x[i] = __fadd_rn(x[i - 1], DX);
        if (c != cdf) {
            ux[n] = x[i];
            uc[n] = c;
            n++;
        }
        cdf = c;
    }
    if (uc[n - 1] != 1.0f) uc[n - 1] = 1.0f;
    if (uc[0] != 0.0f) uc[0] = 0.0f;
}

int sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace

extern "C" bamf_status bamf_rjmcmc_batch_device_noalloc(const bamf_roi_batch *rois,
                                                        const bamf_mcmc_params *p,
                                                        const bamf_priors *pri, uint32_t seed,
                                                        int arith, const bamf_batch_results *out,
                                                        void *stream)
{
    if (!rois || !p || !pri || !out) return BAMF_ERR_INVALID_ARG;
    if (arith != BAMF_ARITH_EXACT && arith != BAMF_ARITH_FAST) return BAMF_ERR_INVALID_ARG;
    if (rois->n_rois < 0 || p->N_Burnin < 0 || p->N_Trials < 0 || p->Grid_Zoom < 0) return BAMF_ERR_INVALID_ARG;
    if (rois->n_rois == 0) return BAMF_OK;
    if (!rois->data || !rois->offsets || !rois->xsize || !rois->ysize) return BAMF_ERR_INVALID_ARG;
    if ((rois->init_n != nullptr) != (rois->init_ixy != nullptr)) return BAMF_ERR_INVALID_ARG;
    int side_max = rois->side_max > 0 ? rois->side_max : BAMF_MAX_ROI_SIDE;
    if (side_max > BAMF_MAX_ROI_SIDE) return BAMF_ERR_TOO_LARGE;
    const int L[3] = {pri->offset_len, pri->signal_len, pri->back_len};
    const float *pdf[3] = {pri->offset_pdf, pri->signal_pdf, pri->back_pdf};
    int nu[3];
    for (int k = 0; k < 3; ++k) {
        bamf_status r = count_unique(pdf[k], L[k], p->DX, &nu[k]);
        if (r) return r;
    }
    bamf_status r0 = check_proposal_and_traces(rois, p, arith, out);
    if (r0) return r0;
    /* scratch plan; reject what does not fit */
    const int n = rois->n_rois;
    const int64_t steps = (int64_t)p->N_Burnin + p->N_Trials;
    const bool want_map = out->map_n != nullptr;
    const bool user_trace = out->n_trace != nullptr;
    size_t off_tables = 512, tab_off[3], used = off_tables;
    for (int k = 0; k < 3; ++k) {
        tab_off[k] = used;
        used = align256(used + (size_t)4 * L[k] * sizeof(float));
    }
    size_t off_order = used;
    used = align256(used + BAMF_ORDER_SCRATCH(n));
    size_t off_entries = used;
    bool own_entries = want_map && out->n_entries == nullptr;
    if (own_entries) used = align256(used + (size_t)n * sizeof(int32_t));
    size_t off_trace = used;
    if (want_map && !user_trace) {
        if (steps > INT32_MAX) return BAMF_ERR_TOO_LARGE;
        used += (size_t)n * (size_t)steps;
    }
    if (used > (size_t)BAMF_NOALLOC_SCRATCH_BYTES) return BAMF_ERR_TOO_LARGE;

    unsigned char *S = nullptr;
    bamf_status r = scratch_address(&S);
    if (r) return r;
    cudaStream_t s = (cudaStream_t)stream;
    /* what must start at zero: the work-queue counters */
    if (cudaMemsetAsync(S, 0, 256, s) != cudaSuccess) return clear_cuda_error();
    for (int k = 0; k < 3; ++k)
        if (cudaMemcpyAsync(S + tab_off[k] + (size_t)L[k] * sizeof(float), pdf[k], (size_t)L[k] * sizeof(float),
                            cudaMemcpyHostToDevice, s) != cudaSuccess)
            return clear_cuda_error();
    build_tables_kernel<<<3, 32, 0, s>>>((float *)(S + tab_off[0]), (float *)(S + tab_off[1]),
                                         (float *)(S + tab_off[2]), L[0], L[1], L[2], p->DX);

    SamplerConsts K;
    std::memset(&K, 0, sizeof K);
    K.p = *p;
    for (int ii = 0; ii < 8; ii++) {
        float tb = 0.0f, tt = 0.0f;
        for (int mm = 0; mm <= ii; mm++) {
            tb = tb + p->P_Burnin[mm];
            tt = tt + p->P_Trials[mm];
        }
        K.PVB[ii] = tb;
        K.PVT[ii] = tt;
    }
    DevStat *ds[3] = {&K.off, &K.sig, &K.back};
    for (int k = 0; k < 3; ++k) {
        float *t = (float *)(S + tab_off[k]);
        ds[k]->x = t;
        ds[k]->pdf = t + L[k];
        ds[k]->ux = t + 2 * L[k];
        ds[k]->uc = t + 3 * L[k];
        ds[k]->L = L[k];
        ds[k]->nu = nu[k];
        ds[k]->inv_dx = 1.0f / p->DX;
    }
    K.seed = seed;
    K.bg0 = rois->bg0;
    K.sync_moves = arith == BAMF_ARITH_FAST ? 1 : 0;
    K.proposal = rois->proposal;
    K.opt_model = rois->opt_model;

    SamplerBatch B;
    std::memset(&B, 0, sizeof B);
    B.n_rois = n;
    B.side_max = side_max;
    B.data = rois->data;
    B.offsets = rois->offsets;
    B.xsize = rois->xsize;
    B.ysize = rois->ysize;
    B.psf_sigma = rois->psf_sigma;
    B.scmos = rois->scmos;
    B.init_n = rois->init_n;
    B.init_bg = rois->init_bg;
    B.init_ixy = rois->init_ixy;
    B.final_n = out->final_n;
    B.final_state = out->final_state;
    B.counters = out->counters;
    B.status = out->status;
    B.overflow = out->overflow;
    B.llr_evals = out->llr_evals;
    B.model_drift = arith == BAMF_ARITH_FAST ? out->model_drift : nullptr;
    B.order = (int32_t *)(S + off_order);
    B.class_range = (int32_t *)(S + 256);
    if ((r = launch_batch_order(rois, n, S + off_order, (int32_t *)B.class_range, s))) return r;
    int32_t *entries = out->n_entries;
    if (own_entries) entries = (int32_t *)(S + off_entries);
    B.n_entries = entries;
    if (user_trace) {
        B.nsig_trace = out->n_trace;
        B.trace_cap = out->trace_len;
    } else if (want_map) {
        B.nsig_trace = S + off_trace;
        B.trace_cap = (int32_t)steps;
    }
    if (out->x_trace) {
        B.x_trace = out->x_trace;
        B.x_cap = out->trace_len;
    }
    B.sampled_psf = rois->opt_model == 1 ? rois->sampled_psf : nullptr;
    B.psf_slot = rois->opt_model == 1 ? rois->psf_slot : nullptr;
    B.n_psf = rois->n_psf > 1 ? rois->n_psf : 1;
    B.birth_cdf = rois->birth_cdf;
    B.birth_sub = rois->birth_sub;
    B.pgrid = out->pgrid;
    B.pback = out->pback;
    B.grid_stride = out->grid_stride;
    B.grid_ld = out->grid_ld;
    B.grid_slot = out->grid_slot;
    B.pos_trace = out->pos_trace;
    B.pos_len = out->pos_len;
    B.pos_thin = out->pos_thin;
    if (cudaGetLastError() != cudaSuccess) return BAMF_ERR_CUDA;

    const bool exact = arith == BAMF_ARITH_EXACT;
    const int sms = sm_count();
    for (int c = BAMF_N_CLASSES - 1; c >= 0; --c) {
        int lo = c == 0 ? 1 : class_side(c - 1) + 1;
        if (lo > side_max) continue;
        SamplerBatch Bc = B;
        Bc.queue = (int32_t *)S + c;
        Bc.cls = c;
        Bc.side_max = std::min(class_side(c), side_max);
        int wpb = 4, mc = 2;
        int per_sm = exact ? blocks_per_sm_exact(Bc.side_max, wpb, K.opt_model)
                           : best_fast_shape(Bc.side_max, K.opt_model, &wpb, &mc);
        if (per_sm < 1) return BAMF_ERR_TOO_LARGE;
        int blocks = std::min((n + wpb - 1) / wpb, per_sm * sms);
        cudaError_t e = exact ? launch_rjmcmc_exact(K, Bc, Bc.side_max, blocks, wpb, s)
                              : launch_rjmcmc_fast(K, Bc, Bc.side_max, blocks, wpb, mc, s);
        if (e != cudaSuccess) return clear_cuda_error();
    }
    if (want_map) {
        map_n_kernel<<<(n + 7) / 8, 256, 0, s>>>(B.nsig_trace, B.trace_cap, entries, n, out->map_n);
        if (cudaGetLastError() != cudaSuccess) return BAMF_ERR_CUDA;
    }
    return BAMF_OK;
}
