/*
 * tiles.cu - the sub-region tiling around the sampler (@RJ/makeSubRegions.m,
 * @RJ/removeOverlapping.m, @RJ/stitchROIs.m) on the device.
 *
 * Frames are Y x X x Z floats, y fastest.  A frame is cut into Xsub x Ysub
 * sub-regions of BoxSize pixels plus Overlap on every inner side
 * (makeSubRegions.m:42-107); sub-region n (0-based) of the stack is frame
 * n / (Xsub Ysub), ix = (n mod Xsub Ysub) / Ysub, iy = n mod Ysub (the
 * reference's Ind = Xsub*Ysub*(frame-1) + Ysub*(ix-1) + iy).  Every value is
 * a copy, so the kernels are bit-exact restatements; the stitch gathers each
 * output pixel's contributions in increasing ROI order, the order of the
 * reference's sequential accumulation (stitchROIs.m:46-65).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "bamf.h"
#include "bamf_tiles.h"

/* a failed CUDA runtime call: clear its error so that a later call on this
 * thread does not report it again */
static inline bamf_status clear_cuda_error()
{
    cudaGetLastError();
    return BAMF_ERR_CUDA;
}

namespace {

struct Geom {
    int B, O, Y, X, Z, Xsub, Ysub;
};

/* makeSubRegions.m:53-84 with 1-based ix, iy: the source rows sy..ey and
 * columns sx..ex (1-based, inclusive) and the ROI size. */
__host__ __device__ inline void extent(const Geom &g, int ix, int iy, int *sy, int *ey, int *sx, int *ex,
                                       int *ny, int *nx)
{
    int ROIex = g.B + 2 * g.O, ROIey = g.B + 2 * g.O;
    int a = g.B * (iy - 1) - (g.O - 1), b = g.B * iy + g.O;
    int c = g.B * (ix - 1) - (g.O - 1), d = g.B * ix + g.O;
    if (iy == 1) {
        ROIey = g.B + g.O;
        a = 1;
        b = g.B + g.O;
    }
    if (ix == 1) {
        ROIex = g.B + g.O;
        c = 1;
        d = g.B + g.O;
    }
    if (iy == g.Ysub) {
        b = g.Y;
        ROIey = g.Y - g.B * (g.Ysub - 1) + g.O;
    }
    if (ix == g.Xsub) {
        d = g.X;
        ROIex = g.X - g.B * (g.Xsub - 1) + g.O;
    }
    if (g.Xsub == 1) ROIex = g.X;
    if (g.Ysub == 1) ROIey = g.Y;
    *sy = a;
    *ey = b;
    *sx = c;
    *ex = d;
    *ny = ROIey;
    *nx = ROIex;
}

/* one thread per element of the (B+2O)^2 tile of every sub-region */
__global__ void subregions_kernel(const float *__restrict__ frames, const float *__restrict__ var, Geom g,
                                  int64_t n_sub, int packed, float *__restrict__ out, float *__restrict__ out_var,
                                  int32_t *__restrict__ xsize, int32_t *__restrict__ ysize,
                                  int32_t *__restrict__ frame_num, int32_t *__restrict__ roi_ind)
{
    const int T = g.B + 2 * g.O;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_sub * T * T) return;
    int64_t n = i / (T * T);
    int e = (int)(i - n * T * T);
    int xx = e / T, yy = e - (e / T) * T;
    int per = g.Xsub * g.Ysub;
    int frame = (int)(n / per), r = (int)(n - (int64_t)frame * per);
    int ix = r / g.Ysub + 1, iy = r - (r / g.Ysub) * g.Ysub + 1;
    int sy, ey, sx, ex, ny, nx;
    extent(g, ix, iy, &sy, &ey, &sx, &ex, &ny, &nx);
    bool in = yy < ny && xx < nx;
    float v = 0.0f, w = 0.0f;
    if (in) {
        int64_t src = (int64_t)(sy - 1 + yy) + (int64_t)g.Y * (sx - 1 + xx);
        v = frames[src + (int64_t)g.Y * g.X * frame];
        if (var) w = var[src];
    }
    int64_t dst = packed ? (in ? n * T * T + yy + (int64_t)ny * xx : -1) : n * T * T + e;
    if (dst >= 0) {
        out[dst] = v;
        if (out_var) out_var[dst] = w;
    }
    if (e == 0) {
        xsize[n] = nx;
        ysize[n] = ny;
        frame_num[n] = frame + 1;
        roi_ind[n] = g.Ysub * (ix - 1) + iy;
    }
}

/* removeOverlapping.m:28-53 on grids of tile side Tz = Zoom (B + 2O) */
__global__ void remove_overlap_kernel(float *__restrict__ grids, int n, int Tz, const int32_t *__restrict__ xsize,
                                      const int32_t *__restrict__ ysize, const int32_t *__restrict__ roi_ind,
                                      int Xsub, int Ysub, int overlap, int zoom)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n * Tz * Tz) return;
    int64_t nn = i / ((int64_t)Tz * Tz);
    int e = (int)(i - nn * Tz * Tz);
    int col = e / Tz, row = e - (e / Tz) * Tz; /* 0-based, row fastest */
    int Ind = roi_ind[nn];
    int ix = (Ind - 1) / Ysub + 1, iy = Ind - (ix - 1) * Ysub;
    int Xs = xsize[nn] * zoom, Ys = ysize[nn] * zoom, zo = zoom * overlap;
    bool zero = false;
    if (ix != Xsub && col >= Xs - zo && col < Xs) zero = true;
    if (iy != Ysub && row >= Ys - zo && row < Ys) zero = true;
    if (ix != 1 && col < zo) zero = true;
    if (iy != 1 && row < zo) zero = true;
    if (zero) grids[i] = 0.0f;
}

/* slot table: the ROI holding each (frame, sub-region); *bad is set when a
 * pair appears twice or lies outside the output */
__global__ void stitch_slots_kernel(const int32_t *__restrict__ frame_num, const int32_t *__restrict__ roi_ind,
                                    int n, int per, int Z, int *__restrict__ slot, int *__restrict__ bad)
{
    int nn = blockIdx.x * blockDim.x + threadIdx.x;
    if (nn >= n) return;
    int f = frame_num[nn] - 1, r = roi_ind[nn] - 1;
    if (f < 0 || f >= Z || r < 0 || r >= per) {
        atomicExch(bad, 1);
        return;
    }
    if (atomicCAS(&slot[(int64_t)f * per + r], -1, nn) != -1) atomicExch(bad, 1);
}

/* stitchROIs.m:27-66: output pixel (Yo, Xo) of frame f (zoomed, 0-based)
 * is the sum of the covering ROIs' grid values, added in increasing ROI
 * order starting from 0 (the reference accumulates ROI by ROI). */
__global__ void stitch_kernel(const float *__restrict__ grids, int Tz, const int32_t *__restrict__ xsize,
                              const int32_t *__restrict__ ysize, const int *__restrict__ slot, Geom g, int zoom,
                              int Zout, float *__restrict__ out)
{
    const int64_t YZ = (int64_t)g.Y * zoom, XZ = (int64_t)g.X * zoom;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= YZ * XZ * Zout) return;
    int f = (int)(i / (YZ * XZ));
    int64_t e = i - (int64_t)f * YZ * XZ;
    int Xo = (int)(e / YZ), Yo = (int)(e - (e / YZ) * YZ);
    int py = Yo / zoom + 1, px = Xo / zoom + 1; /* 1-based source pixel */
    const int per = g.Xsub * g.Ysub;
    int cn[9];
    int64_t co[9];
    int nc = 0;
    int ix0 = min(max((px - 1) / g.B + 1, 1), g.Xsub), iy0 = min(max((py - 1) / g.B + 1, 1), g.Ysub);
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy) {
            int ix = ix0 + dx, iy = iy0 + dy;
            if (ix < 1 || ix > g.Xsub || iy < 1 || iy > g.Ysub) continue;
            int sy, ey, sx, ex, ny, nx;
            extent(g, ix, iy, &sy, &ey, &sx, &ex, &ny, &nx);
            if (py < sy || py > ey || px < sx || px > ex) continue;
            int nn = slot[(int64_t)f * per + g.Ysub * (ix - 1) + (iy - 1)];
            if (nn < 0) continue;
            int ry = Yo - zoom * (sy - 1), rx = Xo - zoom * (sx - 1);
            if (ry >= ysize[nn] * zoom || rx >= xsize[nn] * zoom || ry >= Tz || rx >= Tz) continue;
            cn[nc] = nn;
            co[nc] = (int64_t)nn * Tz * Tz + ry + (int64_t)Tz * rx;
            ++nc;
        }
    for (int a = 1; a < nc; ++a)
        for (int b = a; b > 0 && cn[b - 1] > cn[b]; --b) {
            int t = cn[b];
            cn[b] = cn[b - 1];
            cn[b - 1] = t;
            int64_t u = co[b];
            co[b] = co[b - 1];
            co[b - 1] = u;
        }
    float acc = 0.0f;
    for (int k = 0; k < nc; ++k) acc = __fadd_rn(acc, grids[co[k]]);
    out[i] = acc;
}

/* geometry of a frame size and box; false when a sub-region would leave
 * the frame (the reference indexes out of range there) */
bool make_geom(int Y, int X, int Z, int B, int O, Geom *g)
{
    if (Y < 1 || X < 1 || Z < 1 || B < 1 || O < 0) return false;
    g->B = B;
    g->O = O;
    g->Y = Y;
    g->X = X;
    g->Z = Z;
    g->Xsub = (X + B - 1) / B;
    g->Ysub = (Y + B - 1) / B;
    for (int ix = 1; ix <= g->Xsub; ++ix)
        for (int iy = 1; iy <= g->Ysub; ++iy) {
            int sy, ey, sx, ex, ny, nx;
            extent(*g, ix, iy, &sy, &ey, &sx, &ex, &ny, &nx);
            if (sy < 1 || sx < 1 || ey > Y || ex > X || ey - sy + 1 != ny || ex - sx + 1 != nx) return false;
            if (ny > B + 2 * O || nx > B + 2 * O) return false;
        }
    return true;
}

unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

extern "C" int64_t bamf_subregion_count(int ysize, int xsize, int zsize, int box)
{
    if (ysize < 1 || xsize < 1 || zsize < 0 || box < 1) return -1;
    return (int64_t)((xsize + box - 1) / box) * ((ysize + box - 1) / box) * zsize;
}

extern "C" bamf_status bamf_make_subregions_device(const float *frames, int ysize, int xsize, int zsize, int box,
                                                   int overlap, const float *var, int packed, float *out,
                                                   float *out_var, int32_t *roi_xsize, int32_t *roi_ysize,
                                                   int32_t *frame_num, int32_t *roi_ind, void *stream)
{
    Geom g;
    if (!make_geom(ysize, xsize, zsize, box, overlap, &g)) return BAMF_ERR_INVALID_ARG;
    if (!frames || !out || !roi_xsize || !roi_ysize || !frame_num || !roi_ind) return BAMF_ERR_INVALID_ARG;
    if (out_var && !var) return BAMF_ERR_INVALID_ARG;
    const int T = box + 2 * overlap;
    int64_t n_sub = (int64_t)g.Xsub * g.Ysub * zsize;
    if (packed == 0) {
        /* the padding of every tile is zero, as in the reference's zeros() */
        if (cudaMemsetAsync(out, 0, (size_t)n_sub * T * T * sizeof(float), (cudaStream_t)stream) != cudaSuccess)
            return clear_cuda_error();
        if (out_var &&
            cudaMemsetAsync(out_var, 0, (size_t)n_sub * T * T * sizeof(float), (cudaStream_t)stream) != cudaSuccess)
            return clear_cuda_error();
    }
    int64_t work = n_sub * T * T;
    subregions_kernel<<<blocks_for(work, 256), 256, 0, (cudaStream_t)stream>>>(
        frames, var, g, n_sub, packed, out, out_var, roi_xsize, roi_ysize, frame_num, roi_ind);
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}

extern "C" bamf_status bamf_remove_overlapping_device(float *grids, int n, int tile, const int32_t *roi_xsize,
                                                      const int32_t *roi_ysize, const int32_t *roi_ind, int xsub,
                                                      int ysub, int overlap, int zoom, void *stream)
{
    if (n < 0 || tile < 1 || xsub < 1 || ysub < 1 || overlap < 0 || zoom < 1) return BAMF_ERR_INVALID_ARG;
    if (n == 0) return BAMF_OK;
    if (!grids || !roi_xsize || !roi_ysize || !roi_ind) return BAMF_ERR_INVALID_ARG;
    remove_overlap_kernel<<<blocks_for((int64_t)n * tile * tile, 256), 256, 0, (cudaStream_t)stream>>>(
        grids, n, tile, roi_xsize, roi_ysize, roi_ind, xsub, ysub, overlap, zoom);
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}

extern "C" bamf_status bamf_stitch_rois_device(const float *grids, int n, int tile, const int32_t *roi_xsize,
                                               const int32_t *roi_ysize, const int32_t *frame_num,
                                               const int32_t *roi_ind, int im_y, int im_x, int im_z, int box,
                                               int overlap, int zoom, int32_t *scratch, float *out, void *stream)
{
    Geom g;
    if (!make_geom(im_y, im_x, std::max(im_z, 1), box, overlap, &g) || zoom < 1 || tile < 1 || n < 0)
        return BAMF_ERR_INVALID_ARG;
    if (!out || !scratch || (n > 0 && (!grids || !roi_xsize || !roi_ysize || !frame_num || !roi_ind)))
        return BAMF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const int per = g.Xsub * g.Ysub;
    const int64_t nslot = (int64_t)im_z * per;
    if (cudaMemsetAsync(scratch, 0xff, (size_t)nslot * sizeof(int32_t), s) != cudaSuccess) return clear_cuda_error();
    if (cudaMemsetAsync(scratch + nslot, 0, sizeof(int32_t), s) != cudaSuccess) return clear_cuda_error();
    if (n > 0)
        stitch_slots_kernel<<<blocks_for(n, 256), 256, 0, s>>>(frame_num, roi_ind, n, per, im_z, scratch,
                                                               scratch + nslot);
    int64_t work = (int64_t)im_y * zoom * im_x * zoom * im_z;
    if (work > 0)
        stitch_kernel<<<blocks_for(work, 256), 256, 0, s>>>(grids, tile, roi_xsize, roi_ysize, scratch, g, zoom,
                                                            im_z, out);
    return cudaGetLastError() == cudaSuccess ? BAMF_OK : BAMF_ERR_CUDA;
}
