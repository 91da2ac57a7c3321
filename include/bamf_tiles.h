/*
 * bamf_tiles.h - the sub-region tiling that wraps the sampler in the
 * reference's analysis (@RJ/RJ.m:192-256): cut frames into overlapping
 * sub-regions (makeSubRegions.m), zero the overlap of their posterior grids
 * (removeOverlapping.m) and add the grids into the super-resolved image
 * (stitchROIs.m).  Device pointers, enqueued on `stream`; every value is a
 * copy or a sum in the reference's order, so results are bit-identical to
 * the reference's.
 *
 * Layouts (MATLAB's, y fastest): frames Y x X x Z; a sub-region stack holds
 * n tiles of side T = box + 2 overlap (tile k at k T^2, column stride T);
 * a grid stack holds n tiles of side Tz = zoom T.  Sub-region k of a stack
 * from bamf_make_subregions_device is frame k / (Xsub Ysub), then
 * ix = (k mod Xsub Ysub) / Ysub, iy = k mod Ysub, with Xsub = ceil(X/box),
 * Ysub = ceil(Y/box) (makeSubRegions.m:78: Ind = Xsub Ysub (frame-1) +
 * Ysub (ix-1) + iy).
 */
#ifndef BAMF_TILES_H
#define BAMF_TILES_H

#include <stdint.h>

#include "bamf.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Xsub * Ysub * zsize, or -1 for a bad size. */
int64_t bamf_subregion_count(int ysize, int xsize, int zsize, int box);

/* makeSubRegions(Data, BoxSize, Overlap, Camera_Var) (makeSubRegions.m:42-107).
 *   var        Y x X variance image cropped like the data, or NULL
 *   packed     0: out is the reference's ROI_Data, tiles of T x T with the
 *              sub-region in its top-left corner and zeros elsewhere;
 *              1: each sub-region packed with column stride equal to its own
 *              height at offset k T^2 (the layout bamf_roi_batch reads; the
 *              rest of each tile is left untouched)
 *   out, out_var   [n][T*T] (out_var may be NULL)
 *   roi_xsize, roi_ysize, frame_num (1-based), roi_ind (1-based)   [n]
 * BAMF_ERR_INVALID_ARG when a sub-region would leave the frame (the
 * reference would index outside its data there). */
bamf_status bamf_make_subregions_device(const float *frames, int ysize, int xsize, int zsize, int box, int overlap,
                                        const float *var, int packed, float *out, float *out_var,
                                        int32_t *roi_xsize, int32_t *roi_ysize, int32_t *frame_num,
                                        int32_t *roi_ind, void *stream);

/* removeOverlapping(ROI_Struct, Overlap, Zoom, ROI_Stack) in place on n
 * grids of side `tile` (removeOverlapping.m:28-53). */
bamf_status bamf_remove_overlapping_device(float *grids, int n, int tile, const int32_t *roi_xsize,
                                           const int32_t *roi_ysize, const int32_t *roi_ind, int xsub, int ysub,
                                           int overlap, int zoom, void *stream);

/* stitchROIs(ROIs, ROI_Struct, Overlap, [im_y im_x im_z], BoxSize, Zoom)
 * (stitchROIs.m:27-66) into out [im_z][zoom im_x][zoom im_y].  scratch:
 * im_z Xsub Ysub + 1 int32 of device memory; its last element is set to 1
 * when a (frame, sub-region) pair occurs twice in the list (only the first
 * is stitched then) or lies outside the output. */
bamf_status bamf_stitch_rois_device(const float *grids, int n, int tile, const int32_t *roi_xsize,
                                    const int32_t *roi_ysize, const int32_t *frame_num, const int32_t *roi_ind,
                                    int im_y, int im_x, int im_z, int box, int overlap, int zoom, int32_t *scratch,
                                    float *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif
