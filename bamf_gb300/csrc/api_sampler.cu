/*
 * api_sampler.cu - host side of the sampler C ABI (include/bamf.h): prior
 * tables, device buffers, launches, the MAP-count reduction.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bamf.h"
#include "sampler_common.h"
#include "sampler_launch.h"

using namespace bamf;

static thread_local std::string g_last_error;

static bamf_status cuda_fail(cudaError_t e, const char *where)
{
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    cudaGetLastError(); /* not reported again by a later call on this thread */
    return BAMF_ERR_CUDA;
}

#define CU(call)                                                     \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);          \
    } while (0)

extern "C" const char *bamf_version(void) { return "bamf_gb300 0.1.0 (sm_103a)"; }

extern "C" int bamf_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

extern "C" const char *bamf_last_error(void) { return g_last_error.c_str(); }

/* ------------------------------------------------------------ prior tables */
/* The reference's Stat construction (LibRJMCMC.cpp:176-217) in float, plus
 * the checks the device lookups rely on: the grid and the unique CDF must be
 * strictly increasing (binary search stands in for the linear scans). */
struct HostStat {
    std::vector<float> x, pdf, ux, uc;
};

static bamf_status build_stat(const float *in, int L, float DX, HostStat &s)
{
    if (!in || L < 1) return BAMF_ERR_INVALID_ARG;
    if (!(DX > 0.0f)) return BAMF_ERR_BAD_PRIOR;
    for (int i = 0; i < L; ++i)
        if (!(in[i] >= 0.0f) || std::isinf(in[i])) return BAMF_ERR_BAD_PRIOR;
    std::vector<float> cdf(L), xm(L);
    s.x.assign(L, 0.0f);
    s.pdf.assign(in, in + L);
    cdf[0] = 0.0f;
    xm[0] = 0.0f;
    for (int i = 1; i < L; ++i) {
        cdf[i] = cdf[i - 1] + (s.pdf[i] + s.pdf[i - 1]) * DX / 2.0f;
        if (cdf[i] > 1.0f) cdf[i] = 1.0f;
        xm[i] = cdf[i];
        s.x[i] = s.x[i - 1] + DX;
        if (!(s.x[i] > s.x[i - 1])) return BAMF_ERR_BAD_PRIOR;
    }
    for (int i = L - 2; i >= 0; --i)
        if (cdf[i] == cdf[i + 1]) xm[i + 1] = -1.0f;
    s.ux.clear();
    s.uc.clear();
    for (int i = 0; i < L; ++i)
        if (xm[i] != -1.0f) {
            s.ux.push_back(s.x[i]);
            s.uc.push_back(cdf[i]);
        }
    if (s.uc.back() != 1.0f) s.uc.back() = 1.0f;
    if (s.uc[0] != 0.0f) s.uc[0] = 0.0f;
    for (size_t i = 1; i < s.uc.size(); ++i)
        if (!(s.uc[i] > s.uc[i - 1])) return BAMF_ERR_BAD_PRIOR;
    return BAMF_OK;
}

static void cumulative(const float *P, float *PV)
{
    for (int ii = 0; ii < 8; ii++) {
        float t = 0.0f;
        for (int mm = 0; mm <= ii; mm++) t = t + P[mm];
        PV[ii] = t;
    }
}

/* ---------------------------------------------------------------- workspace */
struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
    bamf_status ensure(size_t bytes)
    {
        if (bytes <= n) return BAMF_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        size_t b = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        n = b;
        return BAMF_OK;
    }
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
};

struct bamf_workspace {
    /* streams the size-class launches fork onto, and their join events */
    cudaStream_t cls_stream[BAMF_N_CLASSES] = {};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[BAMF_N_CLASSES] = {};
    ~bamf_workspace()
    {
        for (int c = 0; c < BAMF_N_CLASSES; ++c) {
            if (cls_stream[c]) cudaStreamDestroy(cls_stream[c]);
            if (join_ev[c]) cudaEventDestroy(join_ev[c]);
        }
        if (fork_ev) cudaEventDestroy(fork_ev);
    }
    bool streams_ready()
    {
        if (fork_ev) return true;
        for (int c = 0; c < BAMF_N_CLASSES; ++c) {
            if (cudaStreamCreateWithFlags(&cls_stream[c], cudaStreamNonBlocking) != cudaSuccess) return false;
            if (cudaEventCreateWithFlags(&join_ev[c], cudaEventDisableTiming) != cudaSuccess) return false;
        }
        return cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming) == cudaSuccess;
    }
    /* CTA shape (chains per CTA, and for fast arithmetic the register
     * budget in CTAs per SM) per arithmetic and size class chosen by
     * bamf_autotune; 0 = not tuned (occupancy rule) */
    int tuned_wpb[2][BAMF_N_CLASSES] = {};
    int tuned_min_ctas[BAMF_N_CLASSES] = {};
    DevBuf tune_range; /* class ranges clipped to the tuning sample    */
    std::vector<float> tables_host; /* what `tables` holds, to skip re-uploads */
    DevStat tables_dev[3] = {};
    DevBuf tables;   /* the three prior tables                       */
    DevBuf queue;    /* work-queue counter                             */
    DevBuf trace;    /* per-ROI Signal==1 count per chain entry        */
    DevBuf entries;  /* per-ROI entry count when the caller wants none */
    DevBuf order;    /* ROI ids largest first                           */
    DevBuf hostin;   /* staging for the host entry point                */
};

extern "C" bamf_status bamf_workspace_create(bamf_workspace **ws)
{
    if (!ws) return BAMF_ERR_INVALID_ARG;
    *ws = new bamf_workspace();
    return BAMF_OK;
}

extern "C" void bamf_workspace_destroy(bamf_workspace *ws) { delete ws; }

/* Copies the three tables into one device buffer and fills the DevStats. */
static bamf_status upload_tables(bamf_workspace *ws, const HostStat st[3], DevStat out[3],
                                 cudaStream_t s)
{
    size_t total = 0;
    for (int k = 0; k < 3; ++k)
        total += st[k].x.size() * 2 + st[k].ux.size() * 2;
    std::vector<float> h;
    h.reserve(total + 12);
    size_t off[3][4];
    for (int k = 0; k < 3; ++k) {
        off[k][0] = h.size(); h.insert(h.end(), st[k].x.begin(), st[k].x.end());
        off[k][1] = h.size(); h.insert(h.end(), st[k].pdf.begin(), st[k].pdf.end());
        off[k][2] = h.size(); h.insert(h.end(), st[k].ux.begin(), st[k].ux.end());
        off[k][3] = h.size(); h.insert(h.end(), st[k].uc.begin(), st[k].uc.end());
    }
    /* the same tables as last time: nothing to upload (and no
     * synchronisation, so a batch can be captured into a graph) */
    for (int k = 0; k < 3; ++k) {
        h.push_back((float)st[k].x.size());
        h.push_back((float)st[k].ux.size());
    }
    if (ws->tables.p && h == ws->tables_host) {
        for (int k = 0; k < 3; ++k) out[k] = ws->tables_dev[k];
        return BAMF_OK;
    }
    bamf_status r = ws->tables.ensure(total * sizeof(float));
    if (r) return r;
    /* synchronous: h is a temporary */
    CU(cudaMemcpyAsync(ws->tables.p, h.data(), total * sizeof(float), cudaMemcpyHostToDevice, s));
    CU(cudaStreamSynchronize(s));
    float *base = (float *)ws->tables.p;
    for (int k = 0; k < 3; ++k) {
        out[k].x = base + off[k][0];
        out[k].pdf = base + off[k][1];
        out[k].ux = base + off[k][2];
        out[k].uc = base + off[k][3];
        out[k].L = (int)st[k].x.size();
        out[k].nu = (int)st[k].ux.size();
        out[k].inv_dx = st[k].x.size() > 1 ? 1.0f / (st[k].x[1] - st[k].x[0]) : 0.0f; /* x[1] - x[0] = DX */
        ws->tables_dev[k] = out[k];
    }
    ws->tables_host.swap(h);
    return BAMF_OK;
}

static bamf_status make_consts(bamf_workspace *ws, const bamf_mcmc_params *p,
                               const bamf_priors *pri, uint32_t seed, float bg0,
                               SamplerConsts &K, cudaStream_t s)
{
    if (!p || !pri) return BAMF_ERR_INVALID_ARG;
    if (p->N_Burnin < 0 || p->N_Trials < 0 || p->Grid_Zoom < 0) return BAMF_ERR_INVALID_ARG;
    HostStat st[3];
    bamf_status r;
    if ((r = build_stat(pri->offset_pdf, pri->offset_len, p->DX, st[0]))) return r;
    if ((r = build_stat(pri->signal_pdf, pri->signal_len, p->DX, st[1]))) return r;
    if ((r = build_stat(pri->back_pdf, pri->back_len, p->DX, st[2]))) return r;
    DevStat ds[3];
    if ((r = upload_tables(ws, st, ds, s))) return r;
    std::memset(&K, 0, sizeof K);
    K.p = *p;
    cumulative(p->P_Burnin, K.PVB);
    cumulative(p->P_Trials, K.PVT);
    K.off = ds[0];
    K.sig = ds[1];
    K.back = ds[2];
    K.seed = seed;
    K.bg0 = bg0;
    return BAMF_OK;
}

static int sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

/* Launch the chains of batch B as a persistent grid: as many CTAs as fit
 * on the GPU at once (or fewer for small batches); warps pull ROI ids from
 * the work queue until it runs dry. */
/* Warps per CTA for an exact launch: the choice among 4, 2, 1 that keeps
 * the most warps resident per SM (shared memory per warp grows with the ROI
 * side). */
static int pick_wpb_exact(int side_max, int opt_model, int *per_sm_out)
{
    int best_w = 0, best_wpb = 4, best_per = 0;
    const int cand[3] = {4, 2, 1};
    for (int i = 0; i < 3; ++i) {
        int per = blocks_per_sm_exact(side_max, cand[i], opt_model);
        if (per * cand[i] > best_w) {
            best_w = per * cand[i];
            best_wpb = cand[i];
            best_per = per;
        }
    }
    *per_sm_out = best_per;
    return best_wpb;
}

/* Launch the chains of batch B as persistent grids.  With size classes, one
 * launch per non-empty class, each on its own stream forked from s (largest
 * class first, so the small ones fill the SMs the large ones drain) and
 * joined back into s. */
static bamf_status launch_batch(bamf_workspace *ws, const SamplerConsts &K, SamplerBatch B,
                                int arith, cudaStream_t s)
{
    bamf_status r;
    bool exact = arith == BAMF_ARITH_EXACT;
    SamplerConsts Kl = K;
    /* fast arithmetic runs move-synchronous CTAs (rjmcmc_kernel_sync) */
    Kl.sync_moves = exact ? 0 : 1;
    int ncls = B.class_range ? BAMF_N_CLASSES : 1;
    if ((r = ws->queue.ensure(sizeof(int32_t) * BAMF_N_CLASSES))) return r;
    CU(cudaMemsetAsync(ws->queue.p, 0, sizeof(int32_t) * BAMF_N_CLASSES, s));
    bool fork = ncls > 1 && ws->streams_ready();
    if (fork) CU(cudaEventRecord(ws->fork_ev, s));
    int sms = sm_count();
    for (int c = ncls - 1; c >= 0; --c) {
        SamplerBatch Bc = B;
        Bc.queue = (int32_t *)ws->queue.p + c;
        Bc.cls = c;
        if (B.class_range) {
            int lo = c == 0 ? 1 : class_side(c - 1) + 1; /* smallest side of class c */
            if (lo > B.side_max) continue;                /* no ROI of the batch is that large */
            Bc.side_max = std::min(class_side(c), B.side_max);
        }
        int per_sm = 0, wpb = 0, mc = 2;
        if (exact) wpb = pick_wpb_exact(Bc.side_max, K.opt_model, &per_sm);
        else per_sm = best_fast_shape(Bc.side_max, K.opt_model, &wpb, &mc);
        if (per_sm < 1) return BAMF_ERR_TOO_LARGE;
        const int tw = ws->tuned_wpb[exact ? 0 : 1][c], tm = exact ? 0 : ws->tuned_min_ctas[c];
        if (tw > 0) {
            int pt = exact ? blocks_per_sm_exact(Bc.side_max, tw, K.opt_model)
                           : blocks_per_sm_fast(Bc.side_max, tw, tm, K.opt_model);
            if (pt > 0) {
                wpb = tw;
                mc = tm;
                per_sm = pt;
            }
        }
        int need = (B.n_rois + wpb - 1) / wpb;
        int blocks = std::min(need, per_sm * sms);
        if (blocks < 1) return BAMF_OK;
        cudaStream_t cs = s;
        if (fork) {
            cs = ws->cls_stream[c];
            CU(cudaStreamWaitEvent(cs, ws->fork_ev, 0));
        }
        cudaError_t e = exact ? launch_rjmcmc_exact(Kl, Bc, Bc.side_max, blocks, wpb, cs)
                              : launch_rjmcmc_fast(Kl, Bc, Bc.side_max, blocks, wpb, mc, cs);
        if (e != cudaSuccess) return cuda_fail(e, "rjmcmc kernel launch");
        if (fork) {
            CU(cudaEventRecord(ws->join_ev[c], cs));
            CU(cudaStreamWaitEvent(s, ws->join_ev[c], 0));
        }
    }
    return BAMF_OK;
}

/* MAP emitter count per ROI (findMap.m:29-45): the MEX output drops the
 * last chain entry (cRJMCMC.cpp:174), so Iter = entries - 1; the mode of the
 * Signal==1 count over entries round(Iter/2)..Iter (1-based), smallest on
 * ties.  One warp per ROI. */
__global__ void map_n_kernel(const uint8_t *__restrict__ trace, int trace_cap,
                             const int32_t *__restrict__ n_entries, int n_rois,
                             int32_t *__restrict__ map_n)
{
    __shared__ int hist[8][BAMF_NMAX + 1];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int roi = blockIdx.x * 8 + warp;
    for (int k = lane; k <= BAMF_NMAX; k += 32) hist[warp][k] = 0;
    __syncwarp();
    if (roi >= n_rois) return;
    int iter = min(n_entries[roi], trace_cap) - 1;
    if (iter < 1) {
        if (lane == 0) map_n[roi] = 0;
        return;
    }
    int start = (iter + 1) / 2;
    const uint8_t *t = trace + (int64_t)roi * trace_cap;
    for (int k = start + lane; k <= iter; k += 32) atomicAdd(&hist[warp][min((int)t[k - 1], BAMF_NMAX)], 1);
    __syncwarp();
    if (lane == 0) {
        int best = 0;
        for (int v = 1; v <= BAMF_NMAX; ++v)
            if (hist[warp][v] > hist[warp][best]) best = v;
        map_n[roi] = best;
    }
}

/* Photon estimate of each ROI, one warp per ROI: the pixels above a
 * background (the mean of the pixels below the ROI's mean), summed; its
 * bucket in half octaves (0..BAMF_N_BUCKETS-1) is the secondary key of the
 * batch order.  Warp sums in a fixed order: the same bucket on every call. */
constexpr int BAMF_N_BUCKETS = 32;

__global__ void photon_bucket_kernel(const float *__restrict__ data, const int64_t *__restrict__ offsets,
                                     const int32_t *__restrict__ xs, const int32_t *__restrict__ ys, int n,
                                     uint8_t *__restrict__ bucket)
{
    const int lane = threadIdx.x & 31;
    const int i = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (i >= n) return;
    const int npix = max(xs[i], 0) * max(ys[i], 0);
    const float *d = data + offsets[i];
    auto wsum = [](float v) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return v;
    };
    float s = 0.0f;
    for (int p = lane; p < npix; p += 32) s += d[p];
    const float mean = wsum(s) / (float)max(npix, 1);
    float sb = 0.0f, cb = 0.0f;
    for (int p = lane; p < npix; p += 32)
        if (d[p] < mean) {
            sb += d[p];
            cb += 1.0f;
        }
    sb = wsum(sb);
    cb = wsum(cb);
    const float bg = cb > 0.0f ? sb / cb : mean;
    float e = 0.0f;
    for (int p = lane; p < npix; p += 32) e += fmaxf(d[p] - bg, 0.0f);
    e = wsum(e);
    if (lane == 0) bucket[i] = (uint8_t)min(BAMF_N_BUCKETS - 1, max(0, (int)(2.0f * log2f(1.0f + e))));
}

/* One block: stable counting sort of the ids in[0..n) (0..n-1 when in is
 * null) by key(id) in [0, K), largest key first; out gets the ids and, when
 * range is given, range[2k], range[2k+1] the [begin, end) of key k.  Ranks
 * within a warp by ballot, warp offsets by a per-key scan over the warps, in
 * id order: the same order on every call. */
template <int K, class KeyF>
__device__ void block_count_sort(int n, const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                 int32_t *__restrict__ range, KeyF key)
{
    __shared__ int cnt[K], pos[K];
    __shared__ int wbase[32][K];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = threadIdx.x; k < K; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&cnt[key(in ? in[i] : i)], 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int c = K - 1; c >= 0; --c) {
            pos[c] = acc;
            if (range) range[2 * c] = acc;
            acc += cnt[c];
            if (range) range[2 * c + 1] = acc;
        }
    }
    __syncthreads();
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int id = i < n ? (in ? in[i] : i) : -1;
        const int c = i < n ? key(id) : -1;
        int rank = 0;
        for (int k = 0; k < K; ++k) {
            const unsigned m = __ballot_sync(0xffffffffu, c == k);
            if (c == k) rank = __popc(m & ((1u << lane) - 1u));
            if (lane == 0) wbase[wid][k] = __popc(m);
        }
        __syncthreads();
        for (int k = threadIdx.x; k < K; k += blockDim.x) {
            int acc = pos[k];
            for (int w = 0; w < nw; ++w) {
                const int t = wbase[w][k];
                wbase[w][k] = acc;
                acc += t;
            }
            pos[k] = acc;
        }
        __syncthreads();
        if (c >= 0) out[wbase[wid][c] + rank] = id;
        __syncthreads();
    }
}

/* The batch order: ROI ids by size class, largest class first, and within a
 * class by photon bucket, brightest first (two stable passes: bucket, then
 * class), plus the [begin, end) of every class.  The chains of a
 * move-synchronous CTA then carry similar emitter counts (they wait less
 * for each other at the per-jump barrier) and the costliest chains of a
 * class start first. */
__global__ void order_kernel(const int32_t *__restrict__ xs, const int32_t *__restrict__ ys,
                             const uint8_t *__restrict__ bucket, int n, int32_t *__restrict__ tmp,
                             int32_t *__restrict__ order, int32_t *__restrict__ class_range)
{
    block_count_sort<BAMF_N_BUCKETS>(n, nullptr, tmp, nullptr, [&](int id) { return (int)bucket[id]; });
    __syncthreads();
    block_count_sort<BAMF_N_CLASSES>(n, tmp, order, class_range, [&](int id) {
        return side_class(min(max(max(xs[id], ys[id]), 1), BAMF_MAX_ROI_SIDE));
    });
}

/* The autotuner's sample of a class: slots [lo, lo + m) of pick get m of
 * the class's ROIs [lo, hi) of order, evenly strided, so that the sample
 * spans the class's whole photon range (the order puts the brightest first)
 * and neighbouring slots stay neighbours in brightness. */
__global__ void strided_pick_kernel(const int32_t *__restrict__ order, int lo, int hi, int m,
                                    int32_t *__restrict__ pick)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) pick[lo + j] = order[lo + (int)((int64_t)j * (hi - lo) / m)];
}

/* Enqueues the batch order on s: `order_scratch` holds BAMF_ORDER_SCRATCH(n)
 * bytes (the order first, then the buckets and the first pass's ids). */
bamf_status launch_batch_order(const bamf_roi_batch *rois, int n, void *order_scratch, int32_t *class_range,
                               cudaStream_t s)
{
    int32_t *order = (int32_t *)order_scratch;
    int32_t *tmp = order + n;
    uint8_t *bucket = (uint8_t *)(tmp + n);
    photon_bucket_kernel<<<(unsigned)(((int64_t)n * 32 + 255) / 256), 256, 0, s>>>(rois->data, rois->offsets,
                                                                                   rois->xsize, rois->ysize, n,
                                                                                   bucket);
    order_kernel<<<1, 1024, 0, s>>>(rois->xsize, rois->ysize, bucket, n, tmp, order, class_range);
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}

/* Checks of the proposal fields of a batch and of the trace outputs, shared
 * with the allocation-free entry point. */
/* OptModel 1 needs a sampled PSF whose four extents are positive and whose
 * element count fits an int (NumModel indexes it with int, :81-84). */
static int64_t psf_elems(const bamf_mcmc_params *p)
{
    int64_t n = 1;
    for (int k = 0; k < 4; ++k) {
        if (p->PSFsize[k] < 1) return -1;
        n *= p->PSFsize[k];
        if (n > INT32_MAX) return -1;
    }
    return n;
}

static bamf_status check_model(int32_t opt_model, const float *psf, const bamf_mcmc_params *p)
{
    if (opt_model == 0) return BAMF_OK;
    if (opt_model != 1 || !psf || psf_elems(p) < 1) return BAMF_ERR_INVALID_ARG;
    return BAMF_OK;
}

bamf_status check_proposal_and_traces(const bamf_roi_batch *rois, const bamf_mcmc_params *p, int arith,
                                      const bamf_batch_results *out)
{
    if (check_model(rois->opt_model, rois->sampled_psf, p) || rois->n_psf < 0) return BAMF_ERR_INVALID_ARG;
    if (rois->opt_model == 1 && (int64_t)std::max(rois->n_psf, 1) * psf_elems(p) > ((int64_t)1 << 40))
        return BAMF_ERR_TOO_LARGE;
    if (rois->proposal < BAMF_PROPOSAL_REFERENCE || rois->proposal > BAMF_PROPOSAL_LEARNED)
        return BAMF_ERR_INVALID_ARG;
    if (rois->proposal != BAMF_PROPOSAL_REFERENCE && arith != BAMF_ARITH_FAST) return BAMF_ERR_INVALID_ARG;
    if (rois->proposal == BAMF_PROPOSAL_LEARNED && (!rois->birth_cdf || !rois->birth_sub))
        return BAMF_ERR_INVALID_ARG;
    if ((out->n_trace || out->x_trace) && out->trace_len < 1) return BAMF_ERR_INVALID_ARG;
    if ((out->pgrid || out->pback) && (out->grid_stride < 1 || out->grid_ld < 0 || p->Grid_Zoom < 1))
        return BAMF_ERR_INVALID_ARG;
    if (out->pos_trace && (out->pos_len < 1 || out->pos_thin < 1)) return BAMF_ERR_INVALID_ARG;
    if (out->n_trace && out->map_n && (int64_t)out->trace_len < (int64_t)p->N_Burnin + p->N_Trials)
        return BAMF_ERR_INVALID_ARG;
    return BAMF_OK;
}

extern "C" bamf_status bamf_rjmcmc_batch_device(bamf_workspace *ws, const bamf_roi_batch *rois,
                                                const bamf_mcmc_params *p,
                                                const bamf_priors *priors, uint32_t seed,
                                                int arith, const bamf_batch_results *out,
                                                void *stream)
{
    if (!ws || !rois || !p || !priors || !out) return BAMF_ERR_INVALID_ARG;
    if (arith != BAMF_ARITH_EXACT && arith != BAMF_ARITH_FAST) return BAMF_ERR_INVALID_ARG;
    if (rois->n_rois < 0) return BAMF_ERR_INVALID_ARG;
    if (rois->n_rois == 0) return BAMF_OK;
    if (!rois->data || !rois->offsets || !rois->xsize || !rois->ysize) return BAMF_ERR_INVALID_ARG;
    if ((rois->init_n != nullptr) != (rois->init_ixy != nullptr)) return BAMF_ERR_INVALID_ARG;
    int side_max = rois->side_max > 0 ? rois->side_max : BAMF_MAX_ROI_SIDE;
    if (side_max > BAMF_MAX_ROI_SIDE) return BAMF_ERR_TOO_LARGE;
    bamf_status r0 = check_proposal_and_traces(rois, p, arith, out);
    if (r0) return r0;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    cudaStream_t s = (cudaStream_t)stream;
    SamplerConsts K;
    bamf_status r = make_consts(ws, p, priors, seed, rois->bg0, K, s);
    if (r) return r;
    K.proposal = rois->proposal;
    K.opt_model = rois->opt_model;
    int n = rois->n_rois;
    int64_t steps = (int64_t)p->N_Burnin + p->N_Trials;
    int trace_cap = (int)std::min<int64_t>(steps, INT32_MAX);
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
    B.birth_cdf = rois->birth_cdf;
    B.birth_sub = rois->birth_sub;
    B.sampled_psf = rois->opt_model == 1 ? rois->sampled_psf : nullptr;
    B.psf_slot = rois->opt_model == 1 ? rois->psf_slot : nullptr;
    B.n_psf = std::max(rois->n_psf, 1);
    B.pgrid = out->pgrid;
    B.pback = out->pback;
    B.grid_stride = out->grid_stride;
    B.grid_ld = out->grid_ld;
    B.grid_slot = out->grid_slot;
    B.pos_trace = out->pos_trace;
    B.pos_len = out->pos_len;
    B.pos_thin = out->pos_thin;
    if (out->x_trace) {
        B.x_trace = out->x_trace;
        B.x_cap = out->trace_len;
    }
    if ((r = ws->order.ensure(BAMF_ORDER_SCRATCH(n) + 256))) return r;
    B.order = (int32_t *)((char *)ws->order.p + 256);
    int32_t *class_range = (int32_t *)ws->order.p; /* 2 * BAMF_N_CLASSES ints */
    if ((r = launch_batch_order(rois, n, (char *)ws->order.p + 256, class_range, s))) return r;
    B.class_range = class_range;
    if (out->n_trace) {
        B.nsig_trace = out->n_trace;
        B.trace_cap = out->trace_len;
    } else if (out->map_n) {
        if ((r = ws->trace.ensure((size_t)n * trace_cap))) return r;
        B.nsig_trace = (uint8_t *)ws->trace.p;
        B.trace_cap = trace_cap;
    }
    int32_t *entries = out->n_entries;
    if (!entries && out->map_n) {
        if ((r = ws->entries.ensure((size_t)n * sizeof(int32_t)))) return r;
        entries = (int32_t *)ws->entries.p;
    }
    B.n_entries = entries;
    if ((r = launch_batch(ws, K, B, arith, s))) return r;
    if (out->map_n) {
        map_n_kernel<<<(n + 7) / 8, 256, 0, s>>>(B.nsig_trace, B.trace_cap, entries, n, out->map_n);
        CU(cudaGetLastError());
    }
    return BAMF_OK;
}

/* ------------------------------------------------------------ graph capture */
struct bamf_batch_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t stream = nullptr;
};

extern "C" void bamf_rjmcmc_batch_graph_destroy(bamf_batch_graph *g)
{
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

/* One batch run on a private stream (prior tables uploaded, buffers sized,
 * kernels configured), then the same batch captured into a CUDA graph. */
extern "C" bamf_status bamf_rjmcmc_batch_graph_create(bamf_workspace *ws, const bamf_roi_batch *rois,
                                                      const bamf_mcmc_params *p, const bamf_priors *priors,
                                                      uint32_t seed, int arith, const bamf_batch_results *out,
                                                      bamf_batch_graph **graph)
{
    if (!graph) return BAMF_ERR_INVALID_ARG;
    *graph = nullptr;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    bamf_batch_graph *g = new bamf_batch_graph();
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        bamf_rjmcmc_batch_graph_destroy(g);
        return BAMF_ERR_CUDA;
    }
    bamf_status r = bamf_rjmcmc_batch_device(ws, rois, p, priors, seed, arith, out, g->stream);
    if (!r && cudaStreamSynchronize(g->stream) != cudaSuccess) r = cuda_fail(cudaGetLastError(), "warm-up batch");
    if (!r && cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess)
        r = cuda_fail(cudaGetLastError(), "cudaStreamBeginCapture");
    if (!r) {
        bamf_status rc = bamf_rjmcmc_batch_device(ws, rois, p, priors, seed, arith, out, g->stream);
        cudaError_t e = cudaStreamEndCapture(g->stream, &g->graph);
        if (rc) r = rc;
        else if (e != cudaSuccess) r = cuda_fail(e, "cudaStreamEndCapture");
    }
    if (!r && cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess)
        r = cuda_fail(cudaGetLastError(), "cudaGraphInstantiate");
    if (r) {
        cudaGetLastError();
        bamf_rjmcmc_batch_graph_destroy(g);
        return r;
    }
    *graph = g;
    return BAMF_OK;
}

extern "C" bamf_status bamf_rjmcmc_batch_graph_launch(bamf_batch_graph *g, void *stream)
{
    if (!g || !g->exec) return BAMF_ERR_INVALID_ARG;
    cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
    return e == cudaSuccess ? BAMF_OK : cuda_fail(e, "cudaGraphLaunch");
}

/* ---------------------------------------------------------------- autotuner */
/* Times every CTA shape (chains per CTA) on a sample of each size class of
 * the batch, with chains of `jumps` burn-in jumps, and keeps the fastest
 * per class in the workspace for later batches of that arithmetic.  In
 * fast arithmetic the chains' results do not depend on the shape (move
 * streams are keyed by slot groups), in exact arithmetic every chain is one
 * warp's, so tuning changes speed only. */
extern "C" bamf_status bamf_autotune(bamf_workspace *ws, const bamf_roi_batch *rois, const bamf_mcmc_params *p,
                                     const bamf_priors *priors, int arith, int jumps, int sample, void *stream)
{
    if (!ws || !rois || !p || !priors || jumps < 1 || sample < 1) return BAMF_ERR_INVALID_ARG;
    if (arith != BAMF_ARITH_EXACT && arith != BAMF_ARITH_FAST) return BAMF_ERR_INVALID_ARG;
    if (rois->n_rois < 1 || !rois->data || !rois->offsets || !rois->xsize || !rois->ysize) return BAMF_ERR_INVALID_ARG;
    int side_max = rois->side_max > 0 ? rois->side_max : BAMF_MAX_ROI_SIDE;
    if (side_max > BAMF_MAX_ROI_SIDE) return BAMF_ERR_TOO_LARGE;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    cudaStream_t s = (cudaStream_t)stream;
    bamf_mcmc_params pt = *p;
    pt.N_Burnin = jumps;
    pt.N_Trials = 0;
    SamplerConsts K;
    bamf_status r = make_consts(ws, &pt, priors, 1u, rois->bg0, K, s);
    if (r) return r;
    K.sync_moves = arith == BAMF_ARITH_FAST ? 1 : 0;
    if (check_model(rois->opt_model, rois->sampled_psf, p)) return BAMF_ERR_INVALID_ARG;
    K.opt_model = rois->opt_model;
    const bool exact = arith == BAMF_ARITH_EXACT;
    const int n = rois->n_rois;
    SamplerBatch B;
    std::memset(&B, 0, sizeof B);
    B.n_rois = n;
    B.data = rois->data;
    B.offsets = rois->offsets;
    B.xsize = rois->xsize;
    B.ysize = rois->ysize;
    B.psf_sigma = rois->psf_sigma;
    B.scmos = rois->scmos;
    B.sampled_psf = rois->opt_model == 1 ? rois->sampled_psf : nullptr;
    B.psf_slot = rois->opt_model == 1 ? rois->psf_slot : nullptr;
    B.n_psf = std::max(rois->n_psf, 1);
    if ((r = ws->order.ensure(BAMF_ORDER_SCRATCH(n) + 256))) return r;
    if ((r = ws->tune_range.ensure(sizeof(int32_t) * 2 * BAMF_N_CLASSES))) return r;
    if ((r = ws->queue.ensure(sizeof(int32_t) * BAMF_N_CLASSES))) return r;
    B.order = (int32_t *)((char *)ws->order.p + 256);
    int32_t *class_range = (int32_t *)ws->order.p;
    if ((r = launch_batch_order(rois, n, (char *)ws->order.p + 256, class_range, s))) return r;
    /* the order's first-pass ids (dead once the order is built) hold the
     * tuning samples */
    int32_t *tune_order = (int32_t *)B.order + n;
    int32_t cr[2 * BAMF_N_CLASSES];
    CU(cudaMemcpyAsync(cr, class_range, sizeof cr, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    const int sms = sm_count();
    /* (chains per CTA, register budget in CTAs per SM) */
    const int cand_f[9][2] = {{8, 2}, {4, 2}, {2, 2}, {1, 2}, {8, 3}, {4, 3}, {2, 3}, {1, 3}, {BAMF_SYNC_GROUP, 1}};
    const int cand_e[3][2] = {{4, 0}, {2, 0}, {1, 0}};
    const int(*cand)[2] = exact ? cand_e : cand_f;
    const int ncand = exact ? 3 : 9;
    bamf_status res = BAMF_OK;
    for (int c = 0; c < BAMF_N_CLASSES && !res; ++c) {
        int lo = cr[2 * c], hi = cr[2 * c + 1];
        if (hi <= lo) continue;
        SamplerBatch Bc = B;
        Bc.class_range = (const int32_t *)ws->tune_range.p;
        Bc.order = tune_order;
        Bc.cls = c;
        Bc.queue = (int32_t *)ws->queue.p + c;
        Bc.side_max = std::min(class_side(c), side_max);
        float best_ms = 0.0f;
        int best = 0, best_mc = 0;
        /* every shape runs the same ROIs: at least `sample`, and at least
         * three rounds of the largest shape's resident chains, so that the
         * wait for the last chains of a round weighs on every shape alike
         * (at most the class) */
        int max_resident = 0;
        for (int k = 0; k < ncand; ++k) {
            const int wpb = cand[k][0], mc = cand[k][1];
            const int per = exact ? blocks_per_sm_exact(Bc.side_max, wpb, K.opt_model)
                                  : blocks_per_sm_fast(Bc.side_max, wpb, mc, K.opt_model);
            max_resident = std::max(max_resident, per * sms * wpb);
        }
        const int m = std::min(hi - lo, std::max(sample, 3 * max_resident));
        for (int k = 0; k < ncand && !res; ++k) {
            const int wpb = cand[k][0], mc = cand[k][1];
            int per = exact ? blocks_per_sm_exact(Bc.side_max, wpb, K.opt_model)
                            : blocks_per_sm_fast(Bc.side_max, wpb, mc, K.opt_model);
            if (per < 1) continue;
            int32_t clip[2 * BAMF_N_CLASSES] = {};
            clip[2 * c] = lo;
            clip[2 * c + 1] = lo + m;
            if (cudaMemcpyAsync(ws->tune_range.p, clip, sizeof clip, cudaMemcpyHostToDevice, s) != cudaSuccess) {
                res = BAMF_ERR_CUDA;
                break;
            }
            strided_pick_kernel<<<(m + 255) / 256, 256, 0, s>>>(B.order, lo, hi, m, tune_order);
            int blocks = std::min((m + wpb - 1) / wpb, per * sms);
            for (int rep = 0; rep < 2 && !res; ++rep) { /* the first launch warms up */
                if (cudaMemsetAsync(Bc.queue, 0, sizeof(int32_t), s) != cudaSuccess ||
                    cudaEventRecord(e0, s) != cudaSuccess) {
                    res = BAMF_ERR_CUDA;
                    break;
                }
                cudaError_t e = exact ? launch_rjmcmc_exact(K, Bc, Bc.side_max, blocks, wpb, s)
                                      : launch_rjmcmc_fast(K, Bc, Bc.side_max, blocks, wpb, mc, s);
                float ms = 0.0f;
                if (e != cudaSuccess || cudaEventRecord(e1, s) != cudaSuccess ||
                    cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                    res = cuda_fail(e != cudaSuccess ? e : cudaGetLastError(), "autotune launch");
                    break;
                }
                ms /= (float)m;
                if (rep == 1 && (best == 0 || ms < best_ms)) {
                    best_ms = ms;
                    best = wpb;
                    best_mc = mc;
                }
            }
        }
        ws->tuned_wpb[exact ? 0 : 1][c] = best;
        if (!exact) ws->tuned_min_ctas[c] = best_mc;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return res;
}

extern "C" bamf_status bamf_autotune_shapes(const bamf_workspace *ws, int arith, int32_t *chains_per_cta,
                                            int32_t *ctas_per_sm_budget)
{
    bamf_status r = bamf_autotune_result(ws, arith, chains_per_cta);
    if (r || !ctas_per_sm_budget) return r ? r : BAMF_ERR_INVALID_ARG;
    for (int c = 0; c < BAMF_N_CLASSES; ++c)
        ctas_per_sm_budget[c] = arith == BAMF_ARITH_EXACT ? 4 * (ws->tuned_wpb[0][c] > 0) : ws->tuned_min_ctas[c];
    return BAMF_OK;
}

extern "C" bamf_status bamf_autotune_result(const bamf_workspace *ws, int arith, int32_t *chains_per_cta)
{
    if (!ws || !chains_per_cta || (arith != BAMF_ARITH_EXACT && arith != BAMF_ARITH_FAST))
        return BAMF_ERR_INVALID_ARG;
    for (int c = 0; c < BAMF_N_CLASSES; ++c) chains_per_cta[c] = ws->tuned_wpb[arith == BAMF_ARITH_EXACT ? 0 : 1][c];
    return BAMF_OK;
}

/* ------------------------------------------------------- host entry points */
template <typename T>
static bamf_status dalloc(std::vector<void *> &owned, T **p, size_t count)
{
    *p = nullptr;
    if (count == 0) return BAMF_OK;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    owned.push_back(*p);
    return BAMF_OK;
}

struct Owned {
    std::vector<void *> v;
    ~Owned()
    {
        for (void *p : v) cudaFree(p);
    }
};

template <typename T>
static bamf_status upload(Owned &o, T **dst, const T *src, size_t count)
{
    *dst = nullptr;
    if (!src || count == 0) return BAMF_OK;
    bamf_status r = dalloc(o.v, dst, count);
    if (r) return r;
    CU(cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice));
    return BAMF_OK;
}

template <typename T>
static bamf_status download(T *dst, const T *src, size_t count)
{
    if (!dst || !src || count == 0) return BAMF_OK;
    CU(cudaMemcpy(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost));
    return BAMF_OK;
}

extern "C" bamf_status bamf_rjmcmc_batch_host(bamf_workspace *ws, const bamf_roi_batch *rois,
                                              const bamf_mcmc_params *p,
                                              const bamf_priors *priors, uint32_t seed,
                                              int arith, const bamf_batch_results *out)
{
    if (!ws || !rois || !p || !priors || !out) return BAMF_ERR_INVALID_ARG;
    int n = rois->n_rois;
    if (n < 0) return BAMF_ERR_INVALID_ARG;
    if (n == 0) return BAMF_OK;
    if (!rois->data || !rois->offsets || !rois->xsize || !rois->ysize) return BAMF_ERR_INVALID_ARG;
    bamf_status r0 = check_proposal_and_traces(rois, p, arith, out);
    if (r0) return r0;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;
    int64_t npix = 0;
    int side_max = 0;
    for (int k = 0; k < n; ++k) {
        if (rois->xsize[k] < 1 || rois->ysize[k] < 1 || rois->offsets[k] < 0) return BAMF_ERR_INVALID_ARG;
        npix = std::max<int64_t>(npix, rois->offsets[k] + (int64_t)rois->xsize[k] * rois->ysize[k]);
        side_max = std::max(side_max, (int)std::max(rois->xsize[k], rois->ysize[k]));
    }
    if (side_max > BAMF_MAX_ROI_SIDE) return BAMF_ERR_TOO_LARGE;
    Owned o;
    bamf_roi_batch d = *rois;
    d.side_max = side_max;
    bamf_status r;
    if ((r = upload(o, (float **)&d.data, rois->data, (size_t)npix))) return r;
    if ((r = upload(o, (int64_t **)&d.offsets, rois->offsets, (size_t)n))) return r;
    if ((r = upload(o, (int32_t **)&d.xsize, rois->xsize, (size_t)n))) return r;
    if ((r = upload(o, (int32_t **)&d.ysize, rois->ysize, (size_t)n))) return r;
    if ((r = upload(o, (float **)&d.psf_sigma, rois->psf_sigma, (size_t)n))) return r;
    if ((r = upload(o, (float **)&d.scmos, rois->scmos, (size_t)npix))) return r;
    if ((r = upload(o, (int32_t **)&d.init_n, rois->init_n, (size_t)n))) return r;
    if ((r = upload(o, (float **)&d.init_bg, rois->init_bg, (size_t)n))) return r;
    if ((r = upload(o, (float **)&d.init_ixy, rois->init_ixy, (size_t)n * 3 * BAMF_NMAX))) return r;
    if (rois->opt_model == 1) {
        const size_t npsf = (size_t)std::max(rois->n_psf, 1);
        if ((r = upload(o, (float **)&d.sampled_psf, rois->sampled_psf, npsf * (size_t)psf_elems(p)))) return r;
        if ((r = upload(o, (int32_t **)&d.psf_slot, rois->psf_slot, (size_t)n))) return r;
    }
    if (rois->proposal == BAMF_PROPOSAL_LEARNED) {
        if ((r = upload(o, (float **)&d.birth_cdf, rois->birth_cdf, (size_t)npix))) return r;
        if ((r = upload(o, (float **)&d.birth_sub, rois->birth_sub, (size_t)npix * 16))) return r;
    }
    bamf_batch_results dout;
    std::memset(&dout, 0, sizeof dout);
    const size_t fs = 4 + 4 * BAMF_NMAX;
    if (out->map_n && (r = dalloc(o.v, &dout.map_n, n))) return r;
    if (out->final_n && (r = dalloc(o.v, &dout.final_n, n))) return r;
    if (out->final_state && (r = dalloc(o.v, &dout.final_state, n * fs))) return r;
    if (out->counters && (r = dalloc(o.v, &dout.counters, (size_t)n * 30))) return r;
    if (out->n_entries && (r = dalloc(o.v, &dout.n_entries, n))) return r;
    if (out->status && (r = dalloc(o.v, &dout.status, n))) return r;
    if (out->overflow && (r = dalloc(o.v, &dout.overflow, n))) return r;
    if (out->llr_evals && (r = dalloc(o.v, &dout.llr_evals, n))) return r;
    if (out->model_drift && (r = dalloc(o.v, &dout.model_drift, n))) return r;
    const size_t tl = out->trace_len > 0 ? (size_t)out->trace_len : 0;
    dout.trace_len = out->trace_len;
    if (out->n_trace && tl && (r = dalloc(o.v, &dout.n_trace, (size_t)n * tl))) return r;
    if (out->x_trace && tl && (r = dalloc(o.v, &dout.x_trace, (size_t)n * tl))) return r;
    if ((r = bamf_rjmcmc_batch_device(ws, &d, p, priors, seed, arith, &dout, nullptr))) return r;
    CU(cudaDeviceSynchronize());
    if ((r = download(out->map_n, dout.map_n, n))) return r;
    if ((r = download(out->final_n, dout.final_n, n))) return r;
    if ((r = download(out->final_state, dout.final_state, n * fs))) return r;
    if ((r = download(out->counters, dout.counters, (size_t)n * 30))) return r;
    if ((r = download(out->n_entries, dout.n_entries, n))) return r;
    if ((r = download(out->status, dout.status, n))) return r;
    if ((r = download(out->overflow, dout.overflow, n))) return r;
    if ((r = download(out->llr_evals, dout.llr_evals, n))) return r;
    if (arith == BAMF_ARITH_FAST && (r = download(out->model_drift, dout.model_drift, n))) return r;
    if (arith != BAMF_ARITH_FAST && out->model_drift) std::memset(out->model_drift, 0, sizeof(float) * (size_t)n);
    if ((r = download(out->n_trace, dout.n_trace, (size_t)n * tl))) return r;
    if ((r = download(out->x_trace, dout.x_trace, (size_t)n * tl))) return r;
    return BAMF_OK;
}

extern "C" bamf_status bamf_crjmcmc_host(const float *data, int xsize, int ysize,
                                         const bamf_emitters *e0, const bamf_mcmc_params *p,
                                         const float *off, int off_len, const float *sig,
                                         int sig_len, const float *back, int back_len,
                                         const float *scmos, const bamf_rng *rng, int arith,
                                         float *pgrid, float *pback, bamf_chain *chain,
                                         bamf_chain *chain_test, bamf_counters *counters)
{
    return bamf_crjmcmc_host_model(data, xsize, ysize, e0, p, off, off_len, sig, sig_len, back, back_len, scmos,
                                   nullptr, 0, rng, arith, pgrid, pback, chain, chain_test, counters);
}

extern "C" bamf_status bamf_crjmcmc_host_model(const float *data, int xsize, int ysize,
                                               const bamf_emitters *e0, const bamf_mcmc_params *p,
                                               const float *off, int off_len, const float *sig,
                                               int sig_len, const float *back, int back_len,
                                               const float *scmos, const float *sampled_psf, int opt_model,
                                               const bamf_rng *rng, int arith, float *pgrid, float *pback,
                                               bamf_chain *chain, bamf_chain *chain_test,
                                               bamf_counters *counters)
{
    if (!data || !e0 || !p || !off || !sig || !back || !rng) return BAMF_ERR_INVALID_ARG;
    if (check_model(opt_model, sampled_psf, p)) return BAMF_ERR_INVALID_ARG;
    if (xsize < 1 || ysize < 1 || off_len < 1 || sig_len < 1 || back_len < 1) return BAMF_ERR_INVALID_ARG;
    if (arith != BAMF_ARITH_EXACT && arith != BAMF_ARITH_FAST) return BAMF_ERR_INVALID_ARG;
    if ((pgrid == nullptr) != (pback == nullptr)) return BAMF_ERR_INVALID_ARG;
    if ((chain == nullptr) != (chain_test == nullptr)) return BAMF_ERR_INVALID_ARG;
    if (e0->N < 0 || (e0->N > 0 && (!e0->I || !e0->X || !e0->Y))) return BAMF_ERR_INVALID_ARG;
    if (xsize > BAMF_MAX_ROI_SIDE || ysize > BAMF_MAX_ROI_SIDE || e0->N > BAMF_NMAX) return BAMF_ERR_TOO_LARGE;
    if (p->N_Burnin < 0 || p->N_Trials < 0 || p->Grid_Zoom < 0) return BAMF_ERR_INVALID_ARG;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;

    bamf_workspace ws;
    bamf_priors pri = {off, off_len, sig, sig_len, back, back_len};
    SamplerConsts K;
    bamf_status r = make_consts(&ws, p, &pri, rng->seed, e0->BG, K, nullptr);
    if (r) return r;
    K.opt_model = opt_model;
    Owned o;
    int npix = xsize * ysize;
    SamplerBatch B;
    std::memset(&B, 0, sizeof B);
    B.n_rois = 1;
    B.side_max = std::max(xsize, ysize);
    int64_t zero = 0;
    int32_t xs = xsize, ys = ysize;
    if ((r = upload(o, (float **)&B.data, data, (size_t)npix))) return r;
    if ((r = upload(o, (int64_t **)&B.offsets, &zero, 1))) return r;
    if ((r = upload(o, (int32_t **)&B.xsize, &xs, 1))) return r;
    if ((r = upload(o, (int32_t **)&B.ysize, &ys, 1))) return r;
    if ((r = upload(o, (float **)&B.scmos, scmos, (size_t)npix))) return r;
    if (opt_model == 1 && (r = upload(o, (float **)&B.sampled_psf, sampled_psf, (size_t)psf_elems(p)))) return r;
    B.n_psf = 1;
    std::vector<float> ixy(3 * BAMF_NMAX, 0.0f);
    for (int k = 0; k < e0->N; ++k) {
        ixy[k] = e0->I[k];
        ixy[BAMF_NMAX + k] = e0->X[k];
        ixy[2 * BAMF_NMAX + k] = e0->Y[k];
    }
    int32_t n0 = e0->N;
    float bg = e0->BG;
    if ((r = upload(o, (int32_t **)&B.init_n, &n0, 1))) return r;
    if ((r = upload(o, (float **)&B.init_bg, &bg, 1))) return r;
    if ((r = upload(o, (float **)&B.init_ixy, ixy.data(), ixy.size()))) return r;
    uint32_t cid = rng->chain_id, roff = rng->offset;
    if ((r = upload(o, (uint32_t **)&B.chain_ids, &cid, 1))) return r;
    if ((r = upload(o, (uint32_t **)&B.rng_offset, &roff, 1))) return r;
    int32_t *d_counters = nullptr, *d_status = nullptr, *d_entries = nullptr;
    if ((r = dalloc(o.v, &d_counters, 30))) return r;
    if ((r = dalloc(o.v, &d_status, 1))) return r;
    if ((r = dalloc(o.v, &d_entries, 1))) return r;
    B.counters = d_counters;
    B.status = d_status;
    B.n_entries = d_entries;
    size_t gsz = (size_t)npix * p->Grid_Zoom * p->Grid_Zoom;
    if (pgrid) {
        if ((r = dalloc(o.v, &B.pgrid, gsz))) return r;
        if ((r = dalloc(o.v, &B.pback, gsz))) return r;
        CU(cudaMemset(B.pgrid, 0, gsz * sizeof(float)));
        CU(cudaMemset(B.pback, 0, gsz * sizeof(float)));
        B.grid_stride = (int64_t)gsz;
    }
    bamf_chain dch[2];
    bamf_chain *hch[2] = {chain, chain_test};
    if (chain) {
        for (int w = 0; w < 2; ++w) {
            bamf_chain &c = dch[w];
            std::memset(&c, 0, sizeof c);
            c.capacity_entries = hch[w]->capacity_entries;
            c.capacity_records = hch[w]->capacity_records;
            size_t ce = (size_t)std::max(c.capacity_entries, 1), cr = (size_t)std::max(c.capacity_records, 1);
            if ((r = dalloc(o.v, &c.N, ce)) || (r = dalloc(o.v, &c.LLR, ce)) || (r = dalloc(o.v, &c.PR, ce)) ||
                (r = dalloc(o.v, &c.JumpType, ce)) || (r = dalloc(o.v, &c.Accepted, ce)) ||
                (r = dalloc(o.v, &c.BG, ce)) || (r = dalloc(o.v, &c.ABG, ce)) || (r = dalloc(o.v, &c.BBG, ce)) ||
                (r = dalloc(o.v, &c.Index, cr)) || (r = dalloc(o.v, &c.Photons, cr)) || (r = dalloc(o.v, &c.X, cr)) ||
                (r = dalloc(o.v, &c.Y, cr)) || (r = dalloc(o.v, &c.Signal, cr)))
                return r;
        }
        bamf_chain *dchains = nullptr;
        if ((r = upload(o, &dchains, dch, 2))) return r;
        B.chains = dchains;
    }
    if ((r = launch_batch(&ws, K, B, arith, nullptr))) return r;
    CU(cudaDeviceSynchronize());
    int32_t st = 0, ne = 0;
    if ((r = download(&st, d_status, 1))) return r;
    if (st != BAMF_OK) return st;
    if ((r = download(&ne, d_entries, 1))) return r;
    if (counters) {
        if ((r = download((int32_t *)counters, d_counters, 30))) return r;
    }
    if (pgrid) {
        if ((r = download(pgrid, B.pgrid, gsz))) return r;
        if ((r = download(pback, B.pback, gsz))) return r;
    }
    if (chain) {
        bamf_chain got[2];
        CU(cudaMemcpy(got, B.chains, sizeof got, cudaMemcpyDeviceToHost));
        for (int w = 0; w < 2; ++w) {
            bamf_chain *h = hch[w];
            if (ne > h->capacity_entries || got[w].n_records > h->capacity_records) return BAMF_ERR_CAPACITY;
            size_t e = (size_t)ne, rc = (size_t)got[w].n_records;
            if ((r = download(h->N, dch[w].N, e)) || (r = download(h->LLR, dch[w].LLR, e)) ||
                (r = download(h->PR, dch[w].PR, e)) || (r = download(h->JumpType, dch[w].JumpType, e)) ||
                (r = download(h->Accepted, dch[w].Accepted, e)) || (r = download(h->BG, dch[w].BG, e)) ||
                (r = download(h->ABG, dch[w].ABG, e)) || (r = download(h->BBG, dch[w].BBG, e)) ||
                (r = download(h->Index, dch[w].Index, rc)) || (r = download(h->Photons, dch[w].Photons, rc)) ||
                (r = download(h->X, dch[w].X, rc)) || (r = download(h->Y, dch[w].Y, rc)) ||
                (r = download(h->Signal, dch[w].Signal, rc)))
                return r;
            h->n_entries = ne;
            h->n_records = got[w].n_records;
        }
    }
    return BAMF_OK;
}

/* Many cRJMCMC calls as one launch: the ROIs of the batch share the MCMC
 * struct and the priors, each keeps its own start state, uniform stream and
 * full MEX outputs.  One persistent launch over all ROIs (no size-class
 * split: the launch is sized for the largest side). */
extern "C" bamf_status bamf_crjmcmc_batch_host(int n_rois, const float *data, const int64_t *offsets,
                                               const int32_t *xsize, const int32_t *ysize,
                                               const bamf_emitters *e0, const bamf_mcmc_params *p,
                                               const bamf_priors *priors, const float *scmos, uint32_t seed,
                                               const uint32_t *chain_id, const uint32_t *rng_offset, int arith,
                                               float *pgrids, float *pbacks, bamf_chain *chains,
                                               bamf_counters *counters, uint32_t *uniforms_used,
                                               int32_t *status)
{
    if (n_rois < 0 || !p || !priors || !status) return BAMF_ERR_INVALID_ARG;
    if (n_rois == 0) return BAMF_OK;
    if (!data || !offsets || !xsize || !ysize || !e0) return BAMF_ERR_INVALID_ARG;
    if (arith != BAMF_ARITH_EXACT && arith != BAMF_ARITH_FAST) return BAMF_ERR_INVALID_ARG;
    if ((pgrids == nullptr) != (pbacks == nullptr)) return BAMF_ERR_INVALID_ARG;
    if (p->N_Burnin < 0 || p->N_Trials < 0 || p->Grid_Zoom < 0) return BAMF_ERR_INVALID_ARG;
    if (pgrids && p->Grid_Zoom < 1) return BAMF_ERR_INVALID_ARG;
    const int n = n_rois;
    int64_t npix = 0, gmax = 0;
    int side_max = 0;
    const int64_t zz = (int64_t)p->Grid_Zoom * p->Grid_Zoom;
    for (int k = 0; k < n; ++k) {
        if (xsize[k] < 1 || ysize[k] < 1 || offsets[k] < 0) return BAMF_ERR_INVALID_ARG;
        if (e0[k].N < 0 || (e0[k].N > 0 && (!e0[k].I || !e0[k].X || !e0[k].Y))) return BAMF_ERR_INVALID_ARG;
        if (e0[k].N > BAMF_NMAX) return BAMF_ERR_TOO_LARGE;
        if (chains && (chains[2 * k].capacity_entries < 0 || chains[2 * k].capacity_records < 0 ||
                       chains[2 * k + 1].capacity_entries < 0 || chains[2 * k + 1].capacity_records < 0))
            return BAMF_ERR_INVALID_ARG;
        npix = std::max<int64_t>(npix, offsets[k] + (int64_t)xsize[k] * ysize[k]);
        gmax = std::max<int64_t>(gmax, (int64_t)xsize[k] * ysize[k] * zz);
        side_max = std::max(side_max, (int)std::max(xsize[k], ysize[k]));
    }
    if (side_max > BAMF_MAX_ROI_SIDE) return BAMF_ERR_TOO_LARGE;
    if (bamf_device_count() < 1) return BAMF_ERR_NO_DEVICE;

    bamf_workspace ws;
    SamplerConsts K;
    bamf_status r = make_consts(&ws, p, priors, seed, 0.0f, K, nullptr);
    if (r) return r;
    Owned o;
    SamplerBatch B;
    std::memset(&B, 0, sizeof B);
    B.n_rois = n;
    B.side_max = side_max;
    B.n_psf = 1;
    if ((r = upload(o, (float **)&B.data, data, (size_t)npix))) return r;
    if ((r = upload(o, (int64_t **)&B.offsets, offsets, (size_t)n))) return r;
    if ((r = upload(o, (int32_t **)&B.xsize, xsize, (size_t)n))) return r;
    if ((r = upload(o, (int32_t **)&B.ysize, ysize, (size_t)n))) return r;
    if ((r = upload(o, (float **)&B.scmos, scmos, (size_t)npix))) return r;
    std::vector<int32_t> n0(n);
    std::vector<float> bg(n), ixy((size_t)n * 3 * BAMF_NMAX, 0.0f);
    std::vector<uint32_t> cid(n), roff(n);
    for (int k = 0; k < n; ++k) {
        n0[k] = e0[k].N;
        bg[k] = e0[k].BG;
        float *row = &ixy[(size_t)k * 3 * BAMF_NMAX];
        for (int j = 0; j < e0[k].N; ++j) {
            row[j] = e0[k].I[j];
            row[BAMF_NMAX + j] = e0[k].X[j];
            row[2 * BAMF_NMAX + j] = e0[k].Y[j];
        }
        cid[k] = chain_id ? chain_id[k] : (uint32_t)k;
        roff[k] = rng_offset ? rng_offset[k] : 0u;
    }
    if ((r = upload(o, (int32_t **)&B.init_n, n0.data(), (size_t)n))) return r;
    if ((r = upload(o, (float **)&B.init_bg, bg.data(), (size_t)n))) return r;
    if ((r = upload(o, (float **)&B.init_ixy, ixy.data(), ixy.size()))) return r;
    if ((r = upload(o, (uint32_t **)&B.chain_ids, cid.data(), (size_t)n))) return r;
    if ((r = upload(o, (uint32_t **)&B.rng_offset, roff.data(), (size_t)n))) return r;
    int32_t *d_counters = nullptr, *d_status = nullptr, *d_entries = nullptr;
    uint32_t *d_unif = nullptr;
    if ((r = dalloc(o.v, &d_counters, (size_t)n * 30))) return r;
    if ((r = dalloc(o.v, &d_status, (size_t)n))) return r;
    if ((r = dalloc(o.v, &d_entries, (size_t)n))) return r;
    if ((r = dalloc(o.v, &d_unif, (size_t)n))) return r;
    B.counters = d_counters;
    B.status = d_status;
    B.n_entries = d_entries;
    B.uniforms_used = d_unif;
    if (pgrids) {
        if ((r = dalloc(o.v, &B.pgrid, (size_t)(n * gmax)))) return r;
        if ((r = dalloc(o.v, &B.pback, (size_t)(n * gmax)))) return r;
        CU(cudaMemset(B.pgrid, 0, (size_t)(n * gmax) * sizeof(float)));
        CU(cudaMemset(B.pback, 0, (size_t)(n * gmax) * sizeof(float)));
        B.grid_stride = gmax;
    }
    /* every chain field of all ROIs in one device buffer per field, ROI k's
     * arrays at the running sum of the capacities before it */
    std::vector<bamf_chain> dch;
    std::vector<int64_t> ebase(2 * (size_t)n + 1, 0), rbase(2 * (size_t)n + 1, 0);
    bamf_chain all;
    std::memset(&all, 0, sizeof all);
    if (chains) {
        for (int i = 0; i < 2 * n; ++i) {
            ebase[i + 1] = ebase[i] + chains[i].capacity_entries;
            rbase[i + 1] = rbase[i] + chains[i].capacity_records;
        }
        const size_t ce = (size_t)std::max<int64_t>(ebase[2 * n], 1), cr = (size_t)std::max<int64_t>(rbase[2 * n], 1);
        if ((r = dalloc(o.v, &all.N, ce)) || (r = dalloc(o.v, &all.LLR, ce)) || (r = dalloc(o.v, &all.PR, ce)) ||
            (r = dalloc(o.v, &all.JumpType, ce)) || (r = dalloc(o.v, &all.Accepted, ce)) ||
            (r = dalloc(o.v, &all.BG, ce)) || (r = dalloc(o.v, &all.ABG, ce)) || (r = dalloc(o.v, &all.BBG, ce)) ||
            (r = dalloc(o.v, &all.Index, cr)) || (r = dalloc(o.v, &all.Photons, cr)) || (r = dalloc(o.v, &all.X, cr)) ||
            (r = dalloc(o.v, &all.Y, cr)) || (r = dalloc(o.v, &all.Signal, cr)))
            return r;
        dch.resize(2 * (size_t)n);
        for (int i = 0; i < 2 * n; ++i) {
            bamf_chain &c = dch[i];
            std::memset(&c, 0, sizeof c);
            c.capacity_entries = chains[i].capacity_entries;
            c.capacity_records = chains[i].capacity_records;
            const int64_t e = ebase[i], q = rbase[i];
            c.N = all.N + e; c.LLR = all.LLR + e; c.PR = all.PR + e; c.JumpType = all.JumpType + e;
            c.Accepted = all.Accepted + e; c.BG = all.BG + e; c.ABG = all.ABG + e; c.BBG = all.BBG + e;
            c.Index = all.Index + q; c.Photons = all.Photons + q; c.X = all.X + q; c.Y = all.Y + q;
            c.Signal = all.Signal + q;
        }
        bamf_chain *d = nullptr;
        if ((r = upload(o, &d, dch.data(), dch.size()))) return r;
        B.chains = d;
    }
    if ((r = launch_batch(&ws, K, B, arith, nullptr))) return r;
    CU(cudaDeviceSynchronize());
    if ((r = download(status, d_status, (size_t)n))) return r;
    std::vector<int32_t> ne(n);
    if ((r = download(ne.data(), d_entries, (size_t)n))) return r;
    if (counters && (r = download((int32_t *)counters, d_counters, (size_t)n * 30))) return r;
    if (uniforms_used && (r = download(uniforms_used, d_unif, (size_t)n))) return r;
    if (pgrids) {
        std::vector<float> g((size_t)(n * gmax));
        for (int w = 0; w < 2; ++w) {
            if ((r = download(g.data(), w ? B.pback : B.pgrid, g.size()))) return r;
            float *dst = w ? pbacks : pgrids;
            for (int k = 0; k < n; ++k)
                std::memcpy(dst + offsets[k] * zz, g.data() + k * gmax,
                            sizeof(float) * (size_t)((int64_t)xsize[k] * ysize[k] * zz));
        }
    }
    if (chains) {
        std::vector<bamf_chain> got(2 * (size_t)n);
        CU(cudaMemcpy(got.data(), B.chains, got.size() * sizeof(bamf_chain), cudaMemcpyDeviceToHost));
        const size_t ce = (size_t)ebase[2 * n], cr = (size_t)rbase[2 * n];
        std::vector<int32_t> hi(std::max(ce, cr));
        std::vector<float> hf(std::max(ce, cr));
        /* one download per field, then each ROI's part into its own arrays */
        auto scatter_i = [&](int32_t *bamf_chain::*f, const std::vector<int64_t> &base, bool rec) -> bamf_status {
            bamf_status rr = download(hi.data(), all.*f, rec ? cr : ce);
            if (rr) return rr;
            for (int i = 0; i < 2 * n; ++i) {
                if (status[i / 2] != BAMF_OK) continue;
                const int32_t cnt = rec ? got[i].n_records : std::min(ne[i / 2], chains[i].capacity_entries);
                if (cnt > 0) std::memcpy(chains[i].*f, hi.data() + base[i], sizeof(int32_t) * (size_t)cnt);
            }
            return BAMF_OK;
        };
        auto scatter_f = [&](float *bamf_chain::*f, const std::vector<int64_t> &base, bool rec) -> bamf_status {
            bamf_status rr = download(hf.data(), all.*f, rec ? cr : ce);
            if (rr) return rr;
            for (int i = 0; i < 2 * n; ++i) {
                if (status[i / 2] != BAMF_OK) continue;
                const int32_t cnt = rec ? got[i].n_records : std::min(ne[i / 2], chains[i].capacity_entries);
                if (cnt > 0) std::memcpy(chains[i].*f, hf.data() + base[i], sizeof(float) * (size_t)cnt);
            }
            return BAMF_OK;
        };
        for (int i = 0; i < 2 * n; ++i) {
            if (status[i / 2] != BAMF_OK) continue;
            if (ne[i / 2] > chains[i].capacity_entries || got[i].n_records > chains[i].capacity_records)
                status[i / 2] = BAMF_ERR_CAPACITY;
        }
        if ((r = scatter_i(&bamf_chain::N, ebase, false)) || (r = scatter_f(&bamf_chain::LLR, ebase, false)) ||
            (r = scatter_f(&bamf_chain::PR, ebase, false)) || (r = scatter_i(&bamf_chain::JumpType, ebase, false)) ||
            (r = scatter_i(&bamf_chain::Accepted, ebase, false)) || (r = scatter_f(&bamf_chain::BG, ebase, false)) ||
            (r = scatter_f(&bamf_chain::ABG, ebase, false)) || (r = scatter_f(&bamf_chain::BBG, ebase, false)) ||
            (r = scatter_i(&bamf_chain::Index, rbase, true)) || (r = scatter_f(&bamf_chain::Photons, rbase, true)) ||
            (r = scatter_f(&bamf_chain::X, rbase, true)) || (r = scatter_f(&bamf_chain::Y, rbase, true)) ||
            (r = scatter_i(&bamf_chain::Signal, rbase, true)))
            return r;
        for (int i = 0; i < 2 * n; ++i) {
            if (status[i / 2] != BAMF_OK) continue;
            chains[i].n_entries = ne[i / 2];
            chains[i].n_records = got[i].n_records;
        }
    }
    return BAMF_OK;
}
