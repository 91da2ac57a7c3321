"""TEST INFRASTRUCTURE: plain-Python restatements of the reference's
sub-region tiling (@RJ/makeSubRegions.m:42-107, @RJ/removeOverlapping.m:28-53,
@RJ/stitchROIs.m:27-66), loop for loop with the reference's 1-based indices,
on numpy arrays in MATLAB orientation (Data[y, x, frame])."""
from __future__ import annotations

import numpy as np


def make_sub_regions(Data, BoxSize, Overlap, Camera_Var=None):
    """makeSubRegions.m:42-107."""
    YPix, XPix, ZPix = Data.shape
    Xsub = -(-XPix // BoxSize)
    Ysub = -(-YPix // BoxSize)
    T = BoxSize + 2 * Overlap
    ROI_Data = np.zeros((T, T, Xsub * Ysub * ZPix), np.float32)
    ROI_Var = np.zeros_like(ROI_Data)
    S = {k: np.zeros(Xsub * Ysub * ZPix, np.int64) for k in ("Xsize", "Ysize", "FrameNum", "ROI_Ind")}
    for frame in range(1, ZPix + 1):
        for ix in range(1, Xsub + 1):
            for iy in range(1, Ysub + 1):
                ROIex = BoxSize + 2 * Overlap
                ROIey = BoxSize + 2 * Overlap
                sy = BoxSize * (iy - 1) - (Overlap - 1)
                ey = BoxSize * iy + Overlap
                sx = BoxSize * (ix - 1) - (Overlap - 1)
                ex = BoxSize * ix + Overlap
                if iy == 1:
                    ROIey = BoxSize + Overlap
                    sy = 1
                    ey = BoxSize + Overlap
                if ix == 1:
                    ROIex = BoxSize + Overlap
                    sx = 1
                    ex = BoxSize + Overlap
                if iy == Ysub:
                    ey = YPix
                    ROIey = YPix - BoxSize * (Ysub - 1) + Overlap
                if ix == Xsub:
                    ex = XPix
                    ROIex = XPix - BoxSize * (Xsub - 1) + Overlap
                if Xsub == 1:
                    ROIex = XPix
                if Ysub == 1:
                    ROIey = YPix
                Ind = Xsub * Ysub * (frame - 1) + Ysub * (ix - 1) + iy
                S["Xsize"][Ind - 1] = ROIex
                S["Ysize"][Ind - 1] = ROIey
                S["FrameNum"][Ind - 1] = frame
                S["ROI_Ind"][Ind - 1] = Ysub * (ix - 1) + iy
                ROI_Data[:ROIey, :ROIex, Ind - 1] = Data[sy - 1:ey, sx - 1:ex, frame - 1]
                if Camera_Var is not None:
                    ROI_Var[:ROIey, :ROIex, Ind - 1] = Camera_Var[sy - 1:ey, sx - 1:ex]
    S.update(SizeData=[YPix, XPix, ZPix], Xsub=Xsub, Ysub=Ysub, Overlap=Overlap)
    return ROI_Data, S, ROI_Var


def remove_overlapping(S, Overlap, Zoom, ROI_Stack):
    """removeOverlapping.m:28-53."""
    ModGrid = ROI_Stack.copy()
    Xsub, Ysub = S["Xsub"], S["Ysub"]
    Xsize = S["Xsize"] * Zoom
    Ysize = S["Ysize"] * Zoom
    for nn in range(1, ROI_Stack.shape[2] + 1):
        Ind = S["ROI_Ind"][nn - 1]
        ix = (Ind - 1) // Ysub + 1
        iy = Ind - (ix - 1) * Ysub
        if ix != Xsub:
            ModGrid[:, Xsize[nn - 1] - (Zoom * Overlap - 1) - 1:Xsize[nn - 1], nn - 1] = 0
        if iy != Ysub:
            ModGrid[Ysize[nn - 1] - (Zoom * Overlap - 1) - 1:Ysize[nn - 1], :, nn - 1] = 0
        if ix != 1:
            ModGrid[:, :Zoom * Overlap, nn - 1] = 0
        if iy != 1:
            ModGrid[:Zoom * Overlap, :, nn - 1] = 0
    return ModGrid


def stitch_rois(ROIs, S, Overlap, ImSize, BoxSize, Zoom):
    """stitchROIs.m:27-66."""
    FinalIm = np.zeros((Zoom * ImSize[0], Zoom * ImSize[1], ImSize[2]), np.float32)
    Xsub, Ysub = S["Xsub"], S["Ysub"]
    Xsize = S["Xsize"] * Zoom
    Ysize = S["Ysize"] * Zoom
    for nn in range(1, ROIs.shape[2] + 1):
        frame = S["FrameNum"][nn - 1]
        Ind = S["ROI_Ind"][nn - 1]
        ix = (Ind - 1) // Ysub + 1
        iy = Ind - (ix - 1) * Ysub
        sy = BoxSize * (iy - 1) - (Overlap - 1)
        ey = BoxSize * iy + Overlap
        sx = BoxSize * (ix - 1) - (Overlap - 1)
        ex = BoxSize * ix + Overlap
        if iy == 1:
            sy = 1
            ey = BoxSize + Overlap
        if ix == 1:
            sx = 1
            ex = BoxSize + Overlap
        if iy == Ysub:
            ey = ImSize[0]
        if ix == Xsub:
            ex = ImSize[1]
        blk = FinalIm[Zoom * sy - (Zoom - 1) - 1:Zoom * ey, Zoom * sx - (Zoom - 1) - 1:Zoom * ex, frame - 1]
        FinalIm[Zoom * sy - (Zoom - 1) - 1:Zoom * ey, Zoom * sx - (Zoom - 1) - 1:Zoom * ex, frame - 1] = \
            (blk + ROIs[:Ysize[nn - 1], :Xsize[nn - 1], nn - 1]).astype(np.float32)
    return FinalIm
