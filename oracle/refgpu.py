"""TEST INFRASTRUCTURE: the reference's own CUDA front-end kernels as a GPU
oracle.

oracle/Makefile (`make -C oracle ref-cubin`) compiles
source/cuda/cuda_FindROI/cuda_FindROI.cu and
source/cuda/cuda_gaussMLEv2/cuda_gaussMLEv2.cu unmodified into sm_103a cubins
under oracle/_ref/.  This module loads them with the CUDA driver API (in
torch's primary context) and launches them with the reference's launch
geometry:

  findROI.m:185-221  gaussX <<<Z, Ysize>>>, gaussY <<<Z, Xsize>>> per sigma,
                     subtract <<<(Ysize, Z), Xsize>>>, maxX <<<(Ysize, Z), Xsize>>>,
                     maxY <<<(Xsize, Z), Ysize>>>, with MATLAB's value
                     semantics (every feval output is a fresh array)
  gaussMLE.m:129-154 kernel_MLEFit_XYNB_ <<<ceil(N/128), 128>>>

kernel_maxX can read one element past the end of its input for the last
row of a deep stack (its window bounds are rounded in float); the input
buffer here is padded with NaN there, which fmaxf ignores.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBINS = {
    "findroi": os.path.join(HERE, "_ref", "cuda_FindROI.sm_103a.cubin"),
    "gaussmle": os.path.join(HERE, "_ref", "cuda_gaussMLEv2.sm_103a.cubin"),
}
NAMES = {
    "gaussX": "_Z13kernel_gaussXPfifffff",
    "gaussY": "_Z13kernel_gaussYPfifffff",
    "subtract": "_Z15kernel_subtractPfS_",
    "maxX": "_Z11kernel_maxXPfS_if",
    "maxY": "_Z11kernel_maxYPfS_if",
    "mle_xynb": "_Z19kernel_MLEFit_XYNB_PKffiiPfS1_S1_i",
    # the other fit types (cuda_gaussMLEv2.cu:144-1125), names from their
    # source signatures
    "mle_xynbs": "_Z20kernel_MLEFit_XYNBS_PKffiiPfS1_S1_i",
    "mle_xynbsxsy": "_Z23kernel_MLEFit_XYNBSXSY_PKffiiPfS1_S1_i",
    "mle_xynbz": "_Z20kernel_MLEFit_XYNBZ_PKfffffffffiiPfS1_S1_i",
    "mle_scmos_xynb": "_Z24kernel_MLEFit_SCMOSXYNB_PKfS0_S0_fiiiPfS1_S1_i",
    "mle_scmos_xynbs": "_Z25kernel_MLEFit_SCMOSXYNBS_PKfS0_S0_fiiiPfS1_S1_i",
    "mle_scmos_xynbsxsy": "_Z28kernel_MLEFit_SCMOSXYNBSXSY_PKfS0_S0_fiiiPfS1_S1_i",
    "mle_scmos_xynbz": "_Z25kernel_MLEFit_SCMOSXYNBZ_PKfS0_S0_S0_ffffffffiiiPfS1_S1_i",
}
NPARAM = {"Basic": 4, "Sigma": 5, "Z": 5, "SigmaYX": 6}
KNAME = {"Basic": "xynb", "Sigma": "xynbs", "Z": "xynbz", "SigmaYX": "xynbsxsy"}


def available(which: str) -> bool:
    return os.path.exists(CUBINS[which])


class _Driver:
    def __init__(self):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # makes the primary context current
        self.cu = C.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        self.mods = {}
        self.fns = {}

    @staticmethod
    def _check(r, what):
        if r != 0:
            raise RuntimeError(f"{what} failed with CUresult {r}")

    def fn(self, which, name):
        key = (which, name)
        if key not in self.fns:
            if which not in self.mods:
                m = C.c_void_p()
                self._check(self.cu.cuModuleLoad(C.byref(m), CUBINS[which].encode()), "cuModuleLoad")
                self.mods[which] = m
            f = C.c_void_p()
            self._check(self.cu.cuModuleGetFunction(C.byref(f), self.mods[which], NAMES[name].encode()),
                        "cuModuleGetFunction")
            self.fns[key] = f
        return self.fns[key]

    def launch(self, which, name, grid, block, args, stream=0):
        vals = []
        for a in args:
            if isinstance(a, C._SimpleCData):
                vals.append(a)
            else:
                raise TypeError(a)
        ptrs = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
        g = list(grid) + [1] * (3 - len(grid))
        b = list(block) + [1] * (3 - len(block))
        self._check(self.cu.cuLaunchKernel(self.fn(which, name), C.c_uint(g[0]), C.c_uint(g[1]),
                                           C.c_uint(g[2]), C.c_uint(b[0]), C.c_uint(b[1]), C.c_uint(b[2]),
                                           C.c_uint(0), C.c_void_p(stream), ptrs, None), "cuLaunchKernel")


_drv = None


def driver() -> _Driver:
    global _drv
    if _drv is None:
        _drv = _Driver()
    return _drv


def _coeffs(sigma: float):
    """findROI.m:169-182 (double), handed to the kernel as single."""
    if sigma > 2.5:
        Q = 0.98711 * sigma - 0.96330
    else:
        Q = 3.97156 - 4.14554 * math.sqrt(1 - 0.26891 * sigma)
    Qq = Q * Q
    Qqq = Qq * Q
    B0 = 1.57825 + 2.44413 * Q + 1.4281 * Qq + 0.422205 * Qqq
    B1 = 2.44413 * Q + 2.85619 * Qq + 1.26661 * Qqq
    B2 = -1.4281 * Qq - 1.26661 * Qqq
    B3 = 0.422205 * Qqq
    B = 1 - (B1 + B2 + B3) / B0
    return [C.c_float(v) for v in (B0, B1, B2, B3, B)]


def findroi_flags(frames_dev, ysize: int, xsize: int, zsize: int, sigma1: float, sigma2: float,
                  boxsize: int, minval: float):
    """Res of findROI.m:114-121 (one chunk) from the reference kernels, as a
    float32 CUDA tensor in memory order.  frames_dev: float32 CUDA tensor of
    ysize*xsize*zsize values, y fastest."""
    import torch
    d = driver()
    n = ysize * xsize * zsize
    ptr = lambda t: C.c_uint64(t.data_ptr())  # noqa: E731

    def gauss(sigma):
        im = frames_dev.clone()
        cf = _coeffs(sigma)
        d.launch("findroi", "gaussX", (zsize,), (ysize,), [ptr(im), C.c_int(xsize)] + cf)
        im0 = im.clone()
        d.launch("findroi", "gaussY", (zsize,), (xsize,), [ptr(im0), C.c_int(ysize)] + cf)
        return im0

    A = gauss(sigma1)
    B = gauss(sigma2)
    sub = torch.full((n + 1024,), float("nan"), dtype=torch.float32, device="cuda")
    sub[:n] = A
    d.launch("findroi", "subtract", (ysize, zsize), (xsize,), [ptr(sub), ptr(B)])
    im1 = A.clone()
    d.launch("findroi", "maxX", (ysize, zsize), (xsize,), [ptr(sub), ptr(im1), C.c_int(boxsize),
                                                            C.c_float(minval)])
    res = sub[:n].clone()
    d.launch("findroi", "maxY", (xsize, zsize), (ysize,), [ptr(res), ptr(im1), C.c_int(boxsize),
                                                            C.c_float(minval)])
    torch.cuda.synchronize()
    return res


def gaussmle_xynb(rois_dev, sz: int, nfits: int, sigma: float, iterations: int):
    """(P, CRLB, LL) CUDA tensors from kernel_MLEFit_XYNB_, param-major."""
    import torch
    d = driver()
    P = torch.zeros(4 * nfits, dtype=torch.float32, device="cuda")
    CR = torch.zeros(4 * nfits, dtype=torch.float32, device="cuda")
    LL = torch.zeros(nfits, dtype=torch.float32, device="cuda")
    ptr = lambda t: C.c_uint64(t.data_ptr())  # noqa: E731
    d.launch("gaussmle", "mle_xynb", ((nfits + 127) // 128,), (128,),
             [ptr(rois_dev), C.c_float(sigma), C.c_int(sz), C.c_int(iterations), ptr(P), ptr(CR), ptr(LL),
              C.c_int(nfits)])
    torch.cuda.synchronize()
    return P, CR, LL


def gaussmle_fit(rois_dev, sz: int, nfits: int, fit_type: str, sigma, iterations: int, zstruct=None,
                 var_map_dev=None, corners_dev=None, map_size: int = 0):
    """(P, CRLB, LL) CUDA tensors from the reference kernel of `fit_type`
    ('Basic', 'Sigma', 'Z', 'SigmaYX'; sCMOS when var_map_dev is given),
    with the arguments gaussMLE.m:150-168 passes."""
    import torch
    d = driver()
    np_ = NPARAM[fit_type]
    P = torch.zeros(np_ * nfits, dtype=torch.float32, device="cuda")
    CR = torch.zeros(np_ * nfits, dtype=torch.float32, device="cuda")
    LL = torch.zeros(nfits, dtype=torch.float32, device="cuda")
    ptr = lambda t: C.c_uint64(t.data_ptr())  # noqa: E731
    scmos = var_map_dev is not None
    name = ("mle_scmos_" if scmos else "mle_") + KNAME[fit_type]
    tail = [C.c_int(sz)] + ([C.c_int(map_size)] if scmos else []) + [C.c_int(iterations), ptr(P), ptr(CR), ptr(LL),
                                                                    C.c_int(nfits)]
    if fit_type == "Z":
        z = zstruct
        zargs = [C.c_float(sigma[0]), C.c_float(z["Ax"]), C.c_float(z["Ay"]), C.c_float(z["Bx"]),
                 C.c_float(z["By"]), C.c_float(z["Gamma"]), C.c_float(z["D"]), C.c_float(sigma[1])]
        if scmos:
            z0 = torch.zeros(nfits, dtype=torch.float32, device="cuda")
            args = [ptr(rois_dev), ptr(corners_dev), ptr(var_map_dev), ptr(z0)] + zargs + tail
        else:
            args = [ptr(rois_dev)] + zargs + tail
    else:
        s_ = C.c_float(float(np.mean(sigma)))
        args = ([ptr(rois_dev), ptr(corners_dev), ptr(var_map_dev), s_] if scmos else [ptr(rois_dev), s_]) + tail
    d.launch("gaussmle", name, ((nfits + 127) // 128,), (128,), args)
    torch.cuda.synchronize()
    return P, CR, LL