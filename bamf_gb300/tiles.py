"""Python mirror of the reference's sub-region tiling over libbamf_gb300.so
(include/bamf_tiles.h): makeSubRegions, removeOverlapping, stitchROIs with
the reference's names, arguments and outputs (@RJ/makeSubRegions.m,
@RJ/removeOverlapping.m, @RJ/stitchROIs.m), computed on the GPU, plus the
device-tensor versions the batched pipeline uses."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


def _lib():
    L = abi.lib()
    if getattr(L, "_tiles_declared", False):
        return L
    vp, i32 = C.c_void_p, C.c_int
    L.bamf_subregion_count.restype = C.c_int64
    L.bamf_subregion_count.argtypes = [i32, i32, i32, i32]
    L.bamf_make_subregions_device.restype = C.c_int
    L.bamf_make_subregions_device.argtypes = [vp, i32, i32, i32, i32, i32, vp, i32, vp, vp, vp, vp, vp, vp, vp]
    L.bamf_remove_overlapping_device.restype = C.c_int
    L.bamf_remove_overlapping_device.argtypes = [vp, i32, i32, vp, vp, vp, i32, i32, i32, i32, vp]
    L.bamf_stitch_rois_device.restype = C.c_int
    L.bamf_stitch_rois_device.argtypes = [vp, i32, i32, vp, vp, vp, vp, i32, i32, i32, i32, i32, i32, vp, vp, vp]
    L._tiles_declared = True
    return L


def _p(t):
    return t.data_ptr() if t is not None else None


def make_subregions_device(frames, ysize: int, xsize: int, zsize: int, box: int, overlap: int, var=None,
                           packed: bool = True, stream=None) -> dict:
    """frames: CUDA float32 tensor of Y*X*Z values (y fastest).  Returns CUDA
    tensors: data [n*T*T] (tiles, packed or MATLAB layout), var (or None),
    xsize, ysize, frame_num, roi_ind [n], offsets [n] (k T^2), and the
    geometry (Xsub, Ysub, T)."""
    import torch
    L = _lib()
    n = int(L.bamf_subregion_count(ysize, xsize, zsize, box))
    if n < 0:
        raise abi.BamfError(abi.BAMF_ERR_INVALID_ARG, "bamf_subregion_count")
    T = box + 2 * overlap
    dev = frames.device
    out = {"data": (torch.zeros if packed else torch.empty)(n * T * T, dtype=torch.float32, device=dev),
           "var": torch.zeros(n * T * T, dtype=torch.float32, device=dev) if var is not None else None}
    for k in ("xsize", "ysize", "frame_num", "roi_ind"):
        out[k] = torch.empty(n, dtype=torch.int32, device=dev)
    st = L.bamf_make_subregions_device(_p(frames), ysize, xsize, zsize, box, overlap, _p(var), int(bool(packed)),
                                       _p(out["data"]), _p(out["var"]), _p(out["xsize"]), _p(out["ysize"]),
                                       _p(out["frame_num"]), _p(out["roi_ind"]),
                                       C.c_void_p(stream) if stream else None)
    abi.check(st, "bamf_make_subregions_device")
    out["offsets"] = torch.arange(n, dtype=torch.int64, device=dev) * (T * T)
    out.update(Xsub=-(-xsize // box), Ysub=-(-ysize // box), T=T, n=n)
    return out


def remove_overlapping_device(grids, n, tile, xsize, ysize, roi_ind, xsub, ysub, overlap, zoom, stream=None):
    abi.check(_lib().bamf_remove_overlapping_device(_p(grids), int(n), int(tile), _p(xsize), _p(ysize), _p(roi_ind),
                                                    int(xsub), int(ysub), int(overlap), int(zoom),
                                                    C.c_void_p(stream) if stream else None),
              "bamf_remove_overlapping_device")


def stitch_rois_device(grids, n, tile, xsize, ysize, frame_num, roi_ind, im_size, box, overlap, zoom,
                       stream=None):
    """Returns (image [Z][zoom X][zoom Y] CUDA tensor, duplicate flag tensor)."""
    import torch
    Y, X, Z = im_size
    xsub, ysub = -(-X // box), -(-Y // box)
    dev = grids.device
    scratch = torch.empty(Z * xsub * ysub + 1, dtype=torch.int32, device=dev)
    out = torch.empty(Z * zoom * X * zoom * Y, dtype=torch.float32, device=dev)
    abi.check(_lib().bamf_stitch_rois_device(_p(grids), int(n), int(tile), _p(xsize), _p(ysize), _p(frame_num),
                                             _p(roi_ind), Y, X, Z, box, overlap, zoom, _p(scratch), _p(out),
                                             C.c_void_p(stream) if stream else None), "bamf_stitch_rois_device")
    return out, scratch[-1:]


# ----------------------------------------------------- reference-named API
def _to_dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float32).ravel(order="F"))).cuda()


def makeSubRegions(Data, BoxSize, Overlap, Camera_Var=None):
    """[ROI_Data, ROI_Struct, ROI_Var] of makeSubRegions.m (MATLAB
    orientation: Data[y, x, frame])."""
    Data = np.asarray(Data, np.float32)
    if Data.ndim == 2:
        Data = Data[:, :, None]
    Y, X, Z = Data.shape
    var = None
    if Camera_Var is not None and np.ndim(Camera_Var) == 2:
        var = _to_dev(Camera_Var)
    r = make_subregions_device(_to_dev(Data), Y, X, Z, BoxSize, Overlap, var=var, packed=False)
    T, n = r["T"], r["n"]
    ROI_Data = r["data"].cpu().numpy().reshape(n, T, T).transpose(2, 1, 0)
    ROI_Var = (r["var"].cpu().numpy().reshape(n, T, T).transpose(2, 1, 0) if var is not None
               else np.zeros_like(ROI_Data))
    S = {"Xsize": r["xsize"].cpu().numpy().astype(np.float64), "Ysize": r["ysize"].cpu().numpy().astype(np.float64),
         "FrameNum": r["frame_num"].cpu().numpy().astype(np.float64),
         "ROI_Ind": r["roi_ind"].cpu().numpy().astype(np.float64),
         "SizeData": [Y, X, Z], "Xsub": r["Xsub"], "Ysub": r["Ysub"], "Overlap": Overlap}
    return np.ascontiguousarray(ROI_Data), S, np.ascontiguousarray(ROI_Var)


def _stack_to_dev(stack):
    stack = np.asarray(stack, np.float32)
    if stack.ndim == 2:
        stack = stack[:, :, None]
    t, t2, n = stack.shape
    if t != t2:
        raise ValueError("grid tiles must be square")
    return _to_dev(stack), t, n


def _ints(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a), np.int32)).cuda()


def removeOverlapping(ROI_Struct, Overlap, Zoom, ROI_Stack):
    """ModGrid of removeOverlapping.m."""
    g, t, n = _stack_to_dev(ROI_Stack)
    remove_overlapping_device(g, n, t, _ints(ROI_Struct["Xsize"]), _ints(ROI_Struct["Ysize"]),
                              _ints(ROI_Struct["ROI_Ind"]), ROI_Struct["Xsub"], ROI_Struct["Ysub"], Overlap, Zoom)
    return g.cpu().numpy().reshape(n, t, t).transpose(2, 1, 0).copy()


def stitchROIs(ROIs, ROI_Struct, Overlap, ImSize, BoxSize, Zoom):
    """FinalIm of stitchROIs.m: (Zoom Y) x (Zoom X) x Z."""
    Y, X, Z = (list(ImSize) + [1])[:3]
    if ROIs is None or np.size(ROIs) == 0:
        return np.zeros((Zoom * Y, Zoom * X, Z), np.float32)
    g, t, n = _stack_to_dev(ROIs)
    out, bad = stitch_rois_device(g, n, t, _ints(ROI_Struct["Xsize"][:n]), _ints(ROI_Struct["Ysize"][:n]),
                                  _ints(ROI_Struct["FrameNum"][:n]), _ints(ROI_Struct["ROI_Ind"][:n]),
                                  (Y, X, Z), BoxSize, Overlap, Zoom)
    if int(bad.item()):
        raise ValueError("a (frame, sub-region) pair occurs twice or lies outside the image")
    return out.cpu().numpy().reshape(Z, Zoom * X, Zoom * Y).transpose(2, 1, 0).copy()
