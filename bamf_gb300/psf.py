"""Sampled PSF arrays for the sampler's OptModel 1 (NumModel,
LibRJMCMC.cpp:67-170).

Layout (MATLAB order, first index fastest, as rjmcmc.m:86 hands it to the
MEX): shape (P0, P1, P2, P3) = (y pixels, x pixels, y sub-positions, x
sub-positions), P2 = P3 = the oversampling.  NumModel puts an emitter at
(x, y) on PSF pixel c0 = P0 // 2, so that ROI pixel xx reads PSF x pixel
ceil(c0 - x) + xx of sub-position plane floor(P3 * frac(x)), blended with
the next plane.
"""
from __future__ import annotations

import numpy as np


def _pixel_integrals(n: int, c0: int, os: int, sigma: float) -> np.ndarray:
    """g[i, s] = integral of a unit normal of std sigma over PSF pixel i for an
    emitter at c0 + s / os: pixel i covers [i - c0 - s/os, i - c0 - s/os + 1)
    relative to the emitter."""
    from scipy.special import erf
    i = np.arange(n, dtype=np.float64)[:, None]
    s = np.arange(os, dtype=np.float64)[None, :] / os
    lo = (i - c0 - s) / (np.sqrt(2.0) * sigma)
    hi = (i - c0 - s + 1.0) / (np.sqrt(2.0) * sigma)
    return 0.5 * (erf(hi) - erf(lo))


def gaussian_sampled_psf(sigma: float, pixels: int = 64, oversampling: int = 4) -> np.ndarray:
    """The pixel-integrated Gaussian PSF of std `sigma` (pixels) sampled at
    oversampling x oversampling sub-pixel positions: a (pixels, pixels, os,
    os) float32 array in the layout above.  With it NumModel reproduces the
    Gaussian model (Model, LibRJMCMC.cpp:15-59) exactly at the sampled
    sub-positions and by bilinear blending between them."""
    c0 = pixels // 2
    g = _pixel_integrals(pixels, c0, oversampling, sigma)      # [pixel][sub]
    psf = g[:, None, :, None] * g[None, :, None, :]            # [y][x][sy][sx]
    return psf.astype(np.float32)


def psf_size(psf: np.ndarray) -> tuple:
    """bamf_mcmc_params.PSFsize of a sampled PSF (its four extents)."""
    if np.ndim(psf) != 4:
        raise ValueError("a sampled PSF is a 4-D array (y, x, y-sub, x-sub)")
    return tuple(int(v) for v in np.shape(psf))
