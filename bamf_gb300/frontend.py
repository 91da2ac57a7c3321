"""Python mirror of the reference front end, over libbamf_gb300.so.

  findROI(Image, Sigma1, Sigma2, Boxsize, Minval)  @RJ/findROI.m:1-224
  gaussMLE(Data, FitType, CameraType, Sigma, ...)   @RJ/gaussMLE.m:64-211 (all fit and camera types)

Images are (Ysize, Xsize[, Zsize]) arrays in MATLAB orientation.  Every call
runs the CUDA kernels; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import abi


def _declare():
    L = abi.lib()
    if getattr(L, "_frontend_declared", False):
        return L
    pf = C.POINTER(C.c_float)
    pi = C.POINTER(C.c_int32)
    L.bamf_find_roi_host.restype = C.c_int
    L.bamf_find_roi_host.argtypes = [pf, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                     C.c_float, C.c_int64, pi, pi, pf, C.POINTER(C.c_int64)]
    L.bamf_findroi_workspace_create.restype = C.c_int
    L.bamf_findroi_workspace_create.argtypes = [C.POINTER(C.c_void_p)]
    L.bamf_findroi_workspace_destroy.argtypes = [C.c_void_p]
    L.bamf_find_roi_device.restype = C.c_int
    L.bamf_find_roi_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                       C.c_double, C.c_int, C.c_float, C.c_int64, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.bamf_find_roi_dog_device.restype = C.c_int
    L.bamf_find_roi_dog_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                           C.c_double, C.c_void_p, C.c_void_p]
    L.bamf_findroi_division_check.restype = C.c_int
    L.bamf_findroi_division_check.argtypes = [C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_ulonglong),
                                              C.POINTER(C.c_ulonglong)]
    L.bamf_find_roi_pinned.restype = C.c_int
    L.bamf_find_roi_pinned.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_double, C.c_double, C.c_int, C.c_float, C.c_int64, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.bamf_find_roi_fit_pinned.restype = C.c_int
    L.bamf_find_roi_fit_pinned.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.c_double, C.c_double, C.c_int, C.c_float, C.c_int64, C.c_float,
                                           C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p]
    L.bamf_gauss_mle_device.restype = C.c_int
    L.bamf_gauss_mle_device.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_int, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p]
    L.bamf_gauss_mle_host.restype = C.c_int
    L.bamf_gauss_mle_host.argtypes = [pf, C.c_int, C.c_int, C.c_float, C.c_int, pf, pf, pf]
    L.bamf_gauss_mle_nparams.restype = C.c_int
    L.bamf_gauss_mle_nparams.argtypes = [C.c_int]
    L.bamf_gauss_mle_fit_host.restype = C.c_int
    L.bamf_gauss_mle_fit_host.argtypes = [pf, C.c_int, C.c_int, C.c_int, C.c_float, C.c_void_p, pf, pf, C.c_int,
                                          C.c_int, pf, pf, pf]
    L._frontend_declared = True
    return L


def default_minval(sigma: float = 1.3) -> float:
    """findROI.m:74: (1/4)*2000*(1/(2*pi*2*1.3^2))."""
    return (1 / 4) * 2000 * (1 / (2 * math.pi * 2 * 1.3 ** 2))


def findROI(Image, Sigma1: float = 1.3, Sigma2: float = 2 * 1.3, Boxsize: int = 7,
            Minval: float | None = None, capacity: int | None = None):
    """Returns (SMD, ROIStack, coords): SMD has XBoxCorner, YBoxCorner,
    FrameNum (1-based, findROI.m:161-163); ROIStack is (Boxsize, Boxsize, N)
    float32; coords (N, 3) are the 1-based (row, col, frame) of the maxima in
    MATLAB find order."""
    L = _declare()
    img = np.asarray(Image, np.float32)
    if img.ndim == 2:
        img = img[:, :, None]
    ys, xs, zs = img.shape
    flat = np.ascontiguousarray(img.ravel(order="F"))
    if Minval is None:
        Minval = default_minval()
    cap = capacity if capacity is not None else max(1024, flat.size // 16)
    while True:
        coords = np.zeros((cap, 3), np.int32)
        corners = np.zeros((cap, 2), np.int32)
        stack = np.zeros((cap, Boxsize, Boxsize), np.float32)
        count = C.c_int64()
        st = L.bamf_find_roi_host(abi.fptr(flat), ys, xs, zs, float(Sigma1), float(Sigma2), int(Boxsize),
                                  float(np.float32(Minval)), cap,
                                  coords.ctypes.data_as(C.POINTER(C.c_int32)),
                                  corners.ctypes.data_as(C.POINTER(C.c_int32)), abi.fptr(stack),
                                  C.byref(count))
        abi.check(st, "bamf_find_roi_host")
        n = int(count.value)
        if n <= cap:
            break
        cap = n
    coords, corners, stack = coords[:n], corners[:n], stack[:n]
    SMD = {"XBoxCorner": corners[:, 1].copy(), "YBoxCorner": corners[:, 0].copy(),
           "FrameNum": coords[:, 2].copy()}
    # stack[k] holds ROI k column-major (y fastest): as MATLAB (B, B, N)
    roistack = np.ascontiguousarray(np.transpose(stack, (2, 1, 0)))
    return SMD, roistack, coords


FIT_TYPES = {"Basic": 0, "Sigma": 1, "Z": 2, "SigmaYX": 3}
FIT_EXTRA = {"Basic": [], "Sigma": ["Sigma"], "Z": ["Z"], "SigmaYX": ["SigmaY", "SigmaX"]}


class ZFit(C.Structure):
    _fields_ = [(k, C.c_float) for k in ("sigma_x", "sigma_y", "Ax", "Ay", "Bx", "By", "gamma", "d")]


def gaussMLE(Data, FitType: str = "Basic", CameraType: str = "CCD", Sigma=1.3, *args, Iterations: int = 20):
    """Results of gaussMLE.m:64-205: gaussMLE(Data, FitType, CameraType,
    Sigma[, ZStruct]) for 'CCD' and gaussMLE(Data, FitType, 'SCMOS', Sigma,
    VarianceImage, BoxCorners[, ZStruct]).  Data: (sz, sz, N); Sigma a
    scalar, or [sigma_x0, sigma_y0] for 'Z'; ZStruct a dict with Ax, Ay, Bx,
    By, Gamma, D; BoxCorners (N, 2) per fit (the pair the kernel reads at
    2 k, 2 k + 1); VarianceImage square.  Iterations defaults to
    gaussMLE.m:98's 20."""
    if FitType not in FIT_TYPES or CameraType not in ("CCD", "SCMOS"):
        raise abi.BamfError(abi.BAMF_ERR_UNSUPPORTED, f"gaussMLE({FitType}, {CameraType})")
    L = _declare()
    d = np.asarray(Data, np.float32)
    if d.ndim == 2:
        d = d[:, :, None]
    sz, _, n = d.shape
    flat = np.ascontiguousarray(d.ravel(order="F"))
    sig = np.atleast_1d(np.asarray(Sigma, np.float64))
    zf = None
    var = corners = None
    rest = list(args)
    if CameraType == "SCMOS":
        if len(rest) < 2:
            raise abi.BamfError(abi.BAMF_ERR_INVALID_ARG, "SCMOS needs VarianceImage and BoxCorners")
        var = np.ascontiguousarray(np.asarray(rest[0], np.float32))
        if var.ndim != 2 or var.shape[0] != var.shape[1]:
            raise abi.BamfError(abi.BAMF_ERR_INVALID_ARG, "gaussMLE: SCMOS fitting needs a square variance image")
        var = np.ascontiguousarray(var.ravel(order="F"))
        corners = np.ascontiguousarray(np.asarray(rest[1], np.float32).reshape(n, 2))
        rest = rest[2:]
    if FitType == "Z":
        z = rest[0]
        zf = ZFit(float(sig[0]), float(sig[1] if len(sig) > 1 else sig[0]), z["Ax"], z["Ay"], z["Bx"], z["By"],
                  z["Gamma"], z["D"])
    npar = L.bamf_gauss_mle_nparams(FIT_TYPES[FitType])
    P = np.zeros(npar * n, np.float32)
    CR = np.zeros(npar * n, np.float32)
    LL = np.zeros(n, np.float32)
    msz = int(np.sqrt(var.size)) if var is not None else 0
    abi.check(L.bamf_gauss_mle_fit_host(abi.fptr(flat), sz, n, FIT_TYPES[FitType], float(np.mean(sig)),
                                        C.byref(zf) if zf is not None else None,
                                        abi.fptr(corners) if corners is not None else None,
                                        abi.fptr(var) if var is not None else None, msz, int(Iterations),
                                        abi.fptr(P), abi.fptr(CR), abi.fptr(LL)), "bamf_gauss_mle_fit_host")
    P = P.reshape(npar, n).T
    CR = CR.reshape(npar, n).T
    # a negative CRLB diagonal (an ill-conditioned fit) gives NaN here where
    # MATLAB's sqrt returns a complex value
    with np.errstate(invalid="ignore"):
        SE = np.sqrt(CR)
    out = {"Y": P[:, 0], "X": P[:, 1], "Photons": P[:, 2], "BG": P[:, 3],
           "Y_SE": SE[:, 0], "X_SE": SE[:, 1], "Photons_SE": SE[:, 2], "BG_SE": SE[:, 3]}
    for k, name in enumerate(FIT_EXTRA[FitType]):
        out[name] = P[:, 4 + k]
        out[name + "_SE"] = SE[:, 4 + k]
    out["LogLikelihood"] = LL
    return out


def division_check(sigma: float, device: bool = False) -> dict:
    """The filters' fast division by the recurrence constant b0 of width
    `sigma` (bamf_findroi_division_check): host_exact, and with device=True
    the device counts of results differing from IEEE division over all 2^32
    floats (in the fast range / in all)."""
    L = _declare()
    ok = C.c_int()
    if not device:
        abi.check(L.bamf_findroi_division_check(float(sigma), C.byref(ok), None, None),
                  "bamf_findroi_division_check")
        return {"host_exact": bool(ok.value)}
    a, b = C.c_ulonglong(), C.c_ulonglong()
    abi.check(L.bamf_findroi_division_check(float(sigma), C.byref(ok), C.byref(a), C.byref(b)),
              "bamf_findroi_division_check")
    return {"host_exact": bool(ok.value), "dev_mismatch_in_range": int(a.value), "dev_mismatch": int(b.value)}


class FindRoiDevice:
    """findROI on device-resident stacks (torch CUDA tensors)."""

    def __init__(self):
        L = _declare()
        h = C.c_void_p()
        abi.check(L.bamf_findroi_workspace_create(C.byref(h)), "bamf_findroi_workspace_create")
        self._ws, self._L = h, L

    def close(self):
        if self._ws:
            self._L.bamf_findroi_workspace_destroy(self._ws)
            self._ws = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, frames, ysize, xsize, zsize, sigma1=1.3, sigma2=2.6, boxsize=7, minval=None,
            capacity=None, stream=None, want_flags=False, want_stack=True):
        """Returns dict of CUDA tensors: coords (cap, 3), corners (cap, 2),
        stack (cap, box*box), count (1,), flags (n,) uint8 when asked.
        Enqueued on `stream`; read count after synchronising."""
        import torch
        if minval is None:
            minval = default_minval()
        n = ysize * xsize * zsize
        cap = capacity if capacity is not None else max(1024, n // 64)
        out = {"coords": torch.empty((cap, 3), dtype=torch.int32, device="cuda"),
               "corners": torch.empty((cap, 2), dtype=torch.int32, device="cuda"),
               "count": torch.zeros(1, dtype=torch.int64, device="cuda")}
        if want_stack:
            out["stack"] = torch.empty((cap, boxsize * boxsize), dtype=torch.float32, device="cuda")
        if want_flags:
            out["flags"] = torch.empty(n, dtype=torch.uint8, device="cuda")
        st = self._L.bamf_find_roi_device(
            self._ws, frames.data_ptr(), ysize, xsize, zsize, float(sigma1), float(sigma2), int(boxsize),
            float(np.float32(minval)), cap, out["coords"].data_ptr(), out["corners"].data_ptr(),
            out["stack"].data_ptr() if want_stack else None, out["count"].data_ptr(),
            out["flags"].data_ptr() if want_flags else None, C.c_void_p(stream) if stream else None)
        abi.check(st, "bamf_find_roi_device")
        return out

    def dog(self, frames, ysize, xsize, zsize, sigma1=1.3, sigma2=2.6, stream=None):
        """The difference-of-Gaussians image the maxima run on, a CUDA
        tensor of ysize*xsize*zsize floats in the frames' layout.  Enqueued
        on `stream`."""
        import torch
        out = torch.empty(ysize * xsize * zsize, dtype=torch.float32, device="cuda")
        abi.check(self._L.bamf_find_roi_dog_device(self._ws, frames.data_ptr(), ysize, xsize, zsize, float(sigma1),
                                                   float(sigma2), out.data_ptr(),
                                                   C.c_void_p(stream) if stream else None),
                  "bamf_find_roi_dog_device")
        return out

    def run_pinned(self, host_frames, ysize, xsize, zsize, sigma1=1.3, sigma2=2.6, boxsize=7, minval=None,
                   capacity=None, stream=None, chunk_frames=250, dev_frames=None):
        """`run` on frames in (pinned) host memory: a torch CPU tensor of
        ysize*xsize*zsize floats, y fastest.  The frames are copied in chunks
        whose filters start as each chunk lands; the dict adds `frames` (the
        device copy) and `host_frames` (the host tensor the copies read,
        kept referenced).  Enqueued on `stream`."""
        import torch
        if minval is None:
            minval = default_minval()
        n = ysize * xsize * zsize
        if host_frames.device.type != "cpu" or host_frames.dtype != torch.float32 or host_frames.numel() != n:
            raise ValueError("host_frames: a CPU float32 tensor of ysize*xsize*zsize values")
        host_frames = host_frames.contiguous()
        cap = capacity if capacity is not None else max(1024, n // 64)
        if dev_frames is None:
            dev_frames = torch.empty(n, dtype=torch.float32, device="cuda")
        out = {"coords": torch.empty((cap, 3), dtype=torch.int32, device="cuda"),
               "corners": torch.empty((cap, 2), dtype=torch.int32, device="cuda"),
               "count": torch.zeros(1, dtype=torch.int64, device="cuda"),
               "stack": torch.empty((cap, boxsize * boxsize), dtype=torch.float32, device="cuda"),
               "frames": dev_frames,
               "host_frames": host_frames}  # the copies read it until the stream gets there
        st = self._L.bamf_find_roi_pinned(
            self._ws, host_frames.data_ptr(), dev_frames.data_ptr(), int(chunk_frames), ysize, xsize, zsize,
            float(sigma1), float(sigma2), int(boxsize), float(np.float32(minval)), cap, out["coords"].data_ptr(),
            out["corners"].data_ptr(), out["stack"].data_ptr(), out["count"].data_ptr(), None,
            C.c_void_p(stream) if stream else None)
        abi.check(st, "bamf_find_roi_pinned")
        return out

    def run_fit_pinned(self, host_frames, ysize, xsize, zsize, sigma1=1.3, sigma2=2.6, boxsize=7, minval=None,
                       psf_sigma=1.3, iterations=10, capacity=None, stream=None, chunk_frames=250,
                       dev_frames=None):
        """`run_pinned` followed by gaussMLE (XYNB, CCD) of the ROIs found,
        chunk by chunk (bamf_find_roi_fit_pinned): the dict of run_pinned
        plus P and CR ([4, capacity], parameter-major, the first count
        columns written) and LL ([capacity]).  Enqueued on `stream`."""
        import torch
        if minval is None:
            minval = default_minval()
        n = ysize * xsize * zsize
        if host_frames.device.type != "cpu" or host_frames.dtype != torch.float32 or host_frames.numel() != n:
            raise ValueError("host_frames: a CPU float32 tensor of ysize*xsize*zsize values")
        host_frames = host_frames.contiguous()
        cap = capacity if capacity is not None else max(1024, n // 64)
        if dev_frames is None:
            dev_frames = torch.empty(n, dtype=torch.float32, device="cuda")
        out = {"coords": torch.empty((cap, 3), dtype=torch.int32, device="cuda"),
               "corners": torch.empty((cap, 2), dtype=torch.int32, device="cuda"),
               "count": torch.zeros(1, dtype=torch.int64, device="cuda"),
               "stack": torch.empty((cap, boxsize * boxsize), dtype=torch.float32, device="cuda"),
               "P": torch.empty((4, cap), dtype=torch.float32, device="cuda"),
               "CR": torch.empty((4, cap), dtype=torch.float32, device="cuda"),
               "LL": torch.empty(cap, dtype=torch.float32, device="cuda"),
               "frames": dev_frames,
               "host_frames": host_frames}  # the copies read it until the stream gets there
        st = self._L.bamf_find_roi_fit_pinned(
            self._ws, host_frames.data_ptr(), dev_frames.data_ptr(), int(chunk_frames), ysize, xsize, zsize,
            float(sigma1), float(sigma2), int(boxsize), float(np.float32(minval)), cap, float(psf_sigma),
            int(iterations), out["coords"].data_ptr(), out["corners"].data_ptr(), out["stack"].data_ptr(),
            out["count"].data_ptr(), out["P"].data_ptr(), out["CR"].data_ptr(), out["LL"].data_ptr(),
            C.c_void_p(stream) if stream else None)
        abi.check(st, "bamf_find_roi_fit_pinned")
        return out


def gauss_mle_device(rois, sz: int, nfits: int, sigma: float, iterations: int, stream=None):
    """kernel on device-resident ROIs (CUDA tensor, nfits*sz*sz); returns
    (P, CRLB, LL) CUDA tensors, param-major."""
    import torch
    L = _declare()
    P = torch.empty(4 * nfits, dtype=torch.float32, device="cuda")
    CR = torch.empty(4 * nfits, dtype=torch.float32, device="cuda")
    LL = torch.empty(nfits, dtype=torch.float32, device="cuda")
    abi.check(L.bamf_gauss_mle_device(rois.data_ptr(), sz, nfits, float(sigma), int(iterations),
                                      P.data_ptr(), CR.data_ptr(), LL.data_ptr(),
                                      C.c_void_p(stream) if stream else None), "bamf_gauss_mle_device")
    return P, CR, LL
