"""Seeded synthetic SMLM data drawn from BAMF's own forward model.

The generator is the reference's Gaussian-PSF model (Stencil/Model,
source/c/LibRJMCMC.cpp:15-59): pixel (y, x) spans [x, x+1] x [y, y+1] and
collects I * 1/2[erf((x-X+1)/(sqrt2 s)) - erf((x-X)/(sqrt2 s))] * (same in y)
from every emitter, on top of a flat background; Poisson noise is added.
Evaluated in float64 with numpy/scipy; images are returned as float32 arrays
of shape (Ysize, Xsize) in MATLAB orientation (rows = y).

Workloads (the sizes the benchmark and the tests use):
  * roi_batch_c0   - 200 ROIs 16x16, N ~ Poisson(3) clipped to [0, 8],
                     positions U[0,16)^2, sigma 1.3, I ~ LogN(ln 1000, 0.3),
                     background 10.
  * roi_batch_uneven - ROIs with sides uniform over {8,12,16,20,24},
                     N ~ Poisson(lam), lam ~ U[0,12], sigma ~ U[1.1,1.5],
                     I ~ LogN(ln 1000, 0.4), background ~ U[5,50].
  * frames         - 256x256 frames, N ~ Poisson(50) per frame uniform over
                     the frame, sigma 1.3, I ~ LogN(ln 1500, 0.3), bg 20.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
from scipy.special import erf


def _pixel_profile(side: int, centers: np.ndarray, sigma) -> np.ndarray:
    """(n, side) integrated 1-D Gaussian profile of each emitter."""
    s = np.asarray(sigma, dtype=np.float64).reshape(-1, 1)
    c = 1.0 / (s * np.sqrt(2.0))
    px = np.arange(side, dtype=np.float64)[None, :]
    mu = np.asarray(centers, dtype=np.float64)[:, None]
    return 0.5 * (erf((px - mu + 1.0) * c) - erf((px - mu) * c))


def model_image(ysize: int, xsize: int, X, Y, I, bg: float, sigma) -> np.ndarray:
    """Expected counts, shape (ysize, xsize), float64."""
    img = np.full((ysize, xsize), float(bg), dtype=np.float64)
    if len(X):
        px = _pixel_profile(xsize, X, sigma) * np.asarray(I, dtype=np.float64)[:, None]
        py = _pixel_profile(ysize, Y, sigma)
        img += py.T @ px
    return img


@dataclass
class RoiBatch:
    """ROIs of possibly different sizes packed back to back.

    data     float32, all ROIs concatenated; ROI k occupies
             data[offsets[k] : offsets[k] + ysize[k]*xsize[k]] in column-major
             (y fastest) order, the layout cRJMCMC receives from MATLAB.
    """
    data: np.ndarray
    offsets: np.ndarray
    xsize: np.ndarray
    ysize: np.ndarray
    sigma: np.ndarray
    bg: np.ndarray
    true_n: np.ndarray
    true_x: list
    true_y: list
    true_i: list

    @property
    def n(self) -> int:
        return int(self.offsets.shape[0])

    def roi(self, k: int) -> np.ndarray:
        """ROI k as a (ysize, xsize) array (MATLAB orientation)."""
        o, ys, xs = int(self.offsets[k]), int(self.ysize[k]), int(self.xsize[k])
        return self.data[o:o + ys * xs].reshape(xs, ys).T


def _pack(rois, sig, bgs, tn, tx, ty, ti) -> RoiBatch:
    sizes = np.array([r.size for r in rois], dtype=np.int64)
    offsets = np.zeros(len(rois), dtype=np.int64)
    if len(rois):
        offsets[1:] = np.cumsum(sizes)[:-1]
    data = np.concatenate([r.ravel(order="F") for r in rois]).astype(np.float32) if rois else \
        np.zeros(0, np.float32)
    return RoiBatch(
        data=data, offsets=offsets,
        xsize=np.array([r.shape[1] for r in rois], dtype=np.int32),
        ysize=np.array([r.shape[0] for r in rois], dtype=np.int32),
        sigma=np.asarray(sig, dtype=np.float32), bg=np.asarray(bgs, dtype=np.float32),
        true_n=np.asarray(tn, dtype=np.int32), true_x=tx, true_y=ty, true_i=ti)


def roi_batch_c0(n_rois: int = 200, side: int = 16, seed: int = 0) -> RoiBatch:
    rng = np.random.default_rng(seed)
    rois, sig, bgs, tn, tx, ty, ti = [], [], [], [], [], [], []
    for _ in range(n_rois):
        n = int(np.clip(rng.poisson(3.0), 0, 8))
        X = rng.uniform(0, side, n)
        Y = rng.uniform(0, side, n)
        I = rng.lognormal(np.log(1000.0), 0.3, n)
        lam = model_image(side, side, X, Y, I, 10.0, 1.3)
        rois.append(rng.poisson(lam).astype(np.float32))
        sig.append(1.3); bgs.append(10.0); tn.append(n); tx.append(X); ty.append(Y); ti.append(I)
    return _pack(rois, sig, bgs, tn, tx, ty, ti)


def roi_batch_uneven(n_rois: int = 100_000, seed: int = 2,
                     sides=(8, 12, 16, 20, 24)) -> RoiBatch:
    rng = np.random.default_rng(seed)
    rois, sig, bgs, tn, tx, ty, ti = [], [], [], [], [], [], []
    for _ in range(n_rois):
        side = int(rng.choice(sides))
        lam_n = rng.uniform(0, 12)
        n = int(min(rng.poisson(lam_n), 24))
        s = rng.uniform(1.1, 1.5)
        X = rng.uniform(0, side, n)
        Y = rng.uniform(0, side, n)
        I = rng.lognormal(np.log(1000.0), 0.4, n)
        b = rng.uniform(5, 50)
        lam = model_image(side, side, X, Y, I, b, s)
        rois.append(rng.poisson(lam).astype(np.float32))
        sig.append(s); bgs.append(b); tn.append(n); tx.append(X); ty.append(Y); ti.append(I)
    return _pack(rois, sig, bgs, tn, tx, ty, ti)


def frames(n_frames: int = 2000, size: int = 256, seed: int = 1, density: float = 50.0,
           sigma: float = 1.3, median_i: float = 1500.0, log_sd: float = 0.3,
           bg: float = 20.0):
    """Frames stack (size, size, n_frames) float32 in MATLAB orientation
    (frame k = stack[:, :, k]) and the ground truth per frame."""
    rng = np.random.default_rng(seed)
    stack = np.empty((size, size, n_frames), dtype=np.float32, order="F")
    truth = []
    for k in range(n_frames):
        n = rng.poisson(density)
        X = rng.uniform(0, size, n)
        Y = rng.uniform(0, size, n)
        I = rng.lognormal(np.log(median_i), log_sd, n)
        lam = model_image(size, size, X, Y, I, bg, sigma)
        stack[:, :, k] = rng.poisson(lam)
        truth.append((X, Y, I))
    return stack, truth


def frames_dense(n_frames: int = 10_000, size: int = 256, seed: int = 5, px_nm: float = 100.0,
                 density=(1.0, 10.0), sigma: float = 1.3, median_i: float = 800.0, log_sd: float = 0.5,
                 bg=(50.0, 200.0)):
    """The dense end-to-end stress frames: per frame an emitter density
    uniform on `density` per um^2 (pixel size px_nm), Poisson count over the
    frame, positions uniform, LogN(ln median_i, log_sd) intensities, a
    uniform background drawn per frame from `bg`, Poisson noise.  Returns
    (stack (size, size, n) float32 MATLAB orientation, truth per frame as
    (X, Y, I) arrays, backgrounds)."""
    rng = np.random.default_rng(seed)
    area_um2 = (size * px_nm / 1000.0) ** 2
    stack = np.empty((size, size, n_frames), dtype=np.float32, order="F")
    truth, bgs = [], []
    for k in range(n_frames):
        rho = rng.uniform(*density)
        n = rng.poisson(rho * area_um2)
        X = rng.uniform(0, size, n)
        Y = rng.uniform(0, size, n)
        I = rng.lognormal(np.log(median_i), log_sd, n)
        b = rng.uniform(*bg)
        lam = model_image(size, size, X, Y, I, b, sigma)
        stack[:, :, k] = rng.poisson(lam)
        truth.append((X, Y, I))
        bgs.append(b)
    return stack, truth, np.array(bgs)


def lognormal_pdf(x: np.ndarray, median: float, log_sd: float) -> np.ndarray:
    x = np.asarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    pos = x > 0
    out[pos] = np.exp(-0.5 * ((np.log(x[pos]) - np.log(median)) / log_sd) ** 2) / (
        x[pos] * log_sd * np.sqrt(2 * np.pi))
    return out


def gamma_pdf(x: np.ndarray, shape: float, scale: float) -> np.ndarray:
    from scipy.stats import gamma
    return gamma.pdf(np.asarray(x, dtype=np.float64), shape, scale=scale)
