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


# --------------------------------------------------------------- findPSF
OVERSAMPLING = 4     # findPSF.m:52
FIT_BOX = 16         # findPSF.m:53


def _round_half_away(v: float) -> int:
    """MATLAB round (halves away from zero)."""
    return int(np.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1)


def find_psf(roi_stack: np.ndarray, gain: float, offset: float, psf_sigma: float, box_size: int) -> np.ndarray:
    """findPSF.m:30-119: the sampled PSF from a stack of isolated emitters.

    roi_stack (box, box, N), MATLAB orientation.  Steps as there:
      * photo-electrons (R - offset) / gain, gaussMLE 'Sigma' positions;
      * the centred 2-D spectra of the first min(N, 1000) spots (R / 10),
        each multiplied by the phase ramp that moves its fitted position to
        the box centre, summed;
      * zero-padded by 12 on every side, inverse transform, modulus: the
        average spot at 4x sampling; minus the mean of its four edge lines,
        negatives to 0, peak 1;
      * zero-padded by 112 on every side to 256 x 256 and cut into the
        4 x 4 sub-grids of every 4th pixel (phase (-m) mod 4 along each
        axis); in planes with a nonzero sub-position the rows (or columns)
        21..43 (0-based) take the values of rows 20..42; each plane
        normalised to sum 1.
    The 256 = 4 * 16 * 4 geometry holds for box 8 only (the reference's
    reshape to 64 x 64 fails otherwise), so other boxes raise ValueError.
    With gaussMLE's coordinates (pixel edges at integers) the array puts
    the emitter half a pixel past the centre pixel NumModel assumes, in x
    and in y, so positions sampled with it sit about half a pixel lower in
    both (measured: plane (0, 0) centroid at 32.5 in pixel-centre units,
    NumModel's centre 32.0); this is the reference's construction, kept.
    Returns float32 (64, 64, 4, 4) = (y, x, y-sub, x-sub)."""
    from . import frontend
    B = int(box_size)
    OS = OVERSAMPLING
    if B + 24 + 224 != OS * FIT_BOX * OS:
        raise ValueError("findPSF's geometry needs an 8-pixel box")
    R = ((np.asarray(roi_stack, np.float32) - np.float32(offset)) / np.float32(gain)).astype(np.float32)
    if R.ndim == 2:
        R = R[:, :, None]
    res = frontend.gaussMLE(R, "Sigma", "CCD", float(psf_sigma))
    X, Y = res["X"].astype(np.float64), res["Y"].astype(np.float64)
    v = np.arange(-int(np.ceil((B - 1) / 2)), int(np.floor((B - 1) / 2)) + 1, dtype=np.float64)
    XG, YG = np.meshgrid(v, v)
    F = np.zeros((B, B), np.complex128)
    for n in range(min(R.shape[2], 1000)):
        f = np.fft.fftshift(np.fft.fft2(np.fft.fftshift(R[:, :, n] / np.float32(10.0))))
        f = f * np.exp(2j * np.pi * XG * (X[n] - B / 2 - 0.5) / B) * np.exp(2j * np.pi * YG * (Y[n] - B / 2 - 0.5) / B)
        F += f
    Fp = np.pad(F.astype(np.complex64), 12)
    S = np.abs(np.fft.fftshift(np.fft.ifft2(Fp))).astype(np.float64)
    edge = np.mean([S[0, :].mean(), S[-1, :].mean(), S[:, -1].mean(), S[:, 0].mean()])
    S = S - edge
    S[S < 0] = 0
    S = S / S.max()
    S = np.pad(S.astype(np.float32), 112)
    n = S.shape[0]
    g = np.arange(-int(np.ceil(n / 2)), int(np.floor((n - 1) / 2)) + 1, dtype=np.float64)
    Xg, Yg = np.meshgrid(g, g)
    XGm = OS - Xg / OS
    XGm = (XGm - np.floor(XGm)) * OS
    YGm = OS - Yg / OS
    YGm = (YGm - np.floor(YGm)) * OS
    side = OS * FIT_BOX
    out = np.zeros((side, side, OS, OS), np.float32)
    lo, hi = _round_half_away(side / 3), _round_half_away(2 * side / 3)
    for ii in range(OS):
        for jj in range(OS):
            mask = (XGm == ii) & (YGm == jj)
            vals = S.T[mask.T]                       # MATLAB column-major gather
            T = vals.reshape(side, side, order="F").astype(np.float32)
            if jj > 0:
                T[lo:hi + 1, :] = T[lo - 1:hi, :].copy()
            if ii > 0:
                T[:, lo:hi + 1] = T[:, lo - 1:hi].copy()
            out[:, :, jj, ii] = T / T.sum(dtype=np.float32)
    return out


def find_psf_sma(tile_stacks, psf_sigma: float, mean_photons: float, box_size: int = 8) -> list:
    """findPSF_SMA.m:26-75: one sampled PSF per sub-region position.

    tile_stacks: per position a (Ysize, Xsize, frames) stack (MATLAB
    orientation).  For each: findROI (sigmas psf_sigma and 2 psf_sigma, box
    box_size, minimum MeanPhotons / (4 pi sigma^2) / 4), and with more than
    30 spots a gaussMLE 'Sigma' fit; spots are kept that are compact
    (Sigma < (box - 4)/2, Sigma_SE < 1), bright but not too bright
    (MeanPhotons/2 < Photons < 5 MeanPhotons, |Photons_SE| < MeanPhotons/5),
    well fitted (LogLikelihood above the threshold there, then at least the
    mean of the kept ones) and central (box/4 < X, Y < 3 box/4); with fewer
    than 30 such spots the PSF comes from 50 copies of a Gaussian spot of
    sigma psf_sigma, else from the first 250 kept spots brighter than half
    their mean, with their mean Sigma; then find_psf(spots, 1, 0, sigma,
    box)."""
    from . import frontend
    B = int(box_size)
    min_int = mean_photons / (4 * np.pi * psf_sigma ** 2) / 4
    out = []
    for data in tile_stacks:
        data = np.asarray(data, np.float32)
        if data.ndim == 2:
            data = data[:, :, None]
        _, stack, _ = frontend.findROI(data, psf_sigma, 2 * psf_sigma, B, min_int)
        stack = np.asarray(stack, np.float32)
        keep = None
        if stack.ndim == 3 and stack.shape[2] > 30:
            r = frontend.gaussMLE(stack, "Sigma", "CCD", psf_sigma)
            good_se = r["Photons_SE"] < mean_photons / 5
            m = abs(np.mean(r["Photons"][good_se]) - 1000) if good_se.any() else np.nan
            ll_min = -(12 - 10 / np.exp(m / 8000)) * B ** 2
            ind1 = ((r["Sigma"] < (B - 4) / 2) & (r["Photons"] < 5 * mean_photons)
                    & (r["Photons"] > mean_photons / 2) & (np.abs(r["Photons_SE"]) < mean_photons / 5)
                    & (r["LogLikelihood"] > ll_min) & (r["Sigma_SE"] < 1)
                    & (r["X"] > B / 4) & (r["X"] < B - B / 4) & (r["Y"] > B / 4) & (r["Y"] < B - B / 4))
            if ind1.any():
                keep = ind1 & (r["LogLikelihood"] >= r["LogLikelihood"][ind1].mean())
            else:
                keep = ind1
        if keep is None or keep.sum() < 30:
            g = np.arange(0.5, B, 1.0)
            xg, yg = np.meshgrid(g, g)
            spot = mean_photons * _normpdf(xg, B / 2, psf_sigma) * _normpdf(yg, B / 2, psf_sigma)
            spots = np.repeat(spot[:, :, None], 50, axis=2)
            sigma = psf_sigma
        else:
            keep = keep & (r["Photons"] > r["Photons"][keep].mean() / 2)
            sigma = float(np.mean(r["Sigma"][keep]))
            spots = stack[:, :, keep][:, :, :250]
        out.append(find_psf(spots, 1.0, 0.0, sigma, B))
    return out


def _normpdf(x, mu, s):
    return np.exp(-0.5 * ((x - mu) / s) ** 2) / (np.sqrt(2 * np.pi) * s)


def tile_stacks(ROI_Data: np.ndarray, ROI_Struct: dict) -> list:
    """Per sub-region position the stack of its tiles over all frames, as
    findPSF_SMA.m:34 cuts it from makeSubRegions' output:
    ROI_Data[:Ysize(nn), :Xsize(nn), nn::Xsub*Ysub]."""
    per = int(ROI_Struct["Xsub"]) * int(ROI_Struct["Ysub"])
    xs = np.asarray(ROI_Struct["Xsize"]).astype(int)
    ys = np.asarray(ROI_Struct["Ysize"]).astype(int)
    return [np.ascontiguousarray(ROI_Data[:ys[nn], :xs[nn], nn::per]) for nn in range(per)]
