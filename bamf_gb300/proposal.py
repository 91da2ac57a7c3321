"""Birth-proposal tables of the batched sampler (BAMF_PROPOSAL_LEARNED).

A birth density over an X x Y ROI is given on a grid of 4X x 4Y sub-pixel
cells (cell (cx, cy) covers [cx/4, (cx+1)/4) x [cy/4, (cy+1)/4) in ROI
coordinates, where pixel (x, y) spans [x, x+1) x [y, y+1)).  The sampler
reads it as two arrays laid out like the ROI pixels (column-major, y
fastest):

  cdf  [pixel]      running sum of the pixel probabilities
  sub  [pixel][16]  probabilities of the pixel's sub-cells, sub-cell
                    s = sy + 4*sx, summing to 1 per pixel

The sampler draws a birth position from this density half of the time and
uniformly on the extended box otherwise, and enters the exact mixture
density into the birth and death ratios, so the posterior it samples does
not depend on the density.
"""
from __future__ import annotations

import numpy as np


def tables_from_cells(cells: np.ndarray, floor: float = 0.0):
    """cells: [4X, 4Y] non-negative weights (x-major: cells[cx, cy]) ->
    (cdf [X*Y], sub [X*Y*16]) float32 for one ROI."""
    cells = np.asarray(cells, np.float64)
    X4, Y4 = cells.shape
    if X4 % 4 or Y4 % 4:
        raise ValueError("cell grid must be 4X x 4Y")
    X, Y = X4 // 4, Y4 // 4
    w = cells + floor
    if not (w >= 0).all() or not w.sum() > 0:
        raise ValueError("cell weights must be non-negative with a positive sum")
    # [x, sx, y, sy] -> pixel (x, y) with y fastest, sub-cell sy + 4*sx
    b = w.reshape(X, 4, Y, 4).transpose(0, 2, 1, 3)          # [x, y, sx, sy]
    pix = b.sum(axis=(2, 3))                                   # [x, y]
    cdf = np.cumsum((pix / pix.sum()).ravel())                 # pixel index y + x*Y
    sub = np.where(pix[..., None, None] > 0, b / np.maximum(pix[..., None, None], 1e-300), 1.0 / 16)
    sub = sub.reshape(X * Y, 16)                               # s = sy + 4*sx
    return cdf.astype(np.float32), sub.reshape(-1).astype(np.float32)


def batch_tables(cell_maps, xsize, ysize, floor: float = 0.0):
    """Concatenated (cdf, sub) of a batch in ROI order (ROI k at pixel
    offset sum of the previous ROIs' X*Y, the layout synth.RoiBatch uses)."""
    cdfs, subs = [], []
    for c, X, Y in zip(cell_maps, xsize, ysize):
        c = np.asarray(c)
        if c.shape != (4 * X, 4 * Y):
            raise ValueError(f"cell map {c.shape} does not match ROI {X}x{Y}")
        a, b = tables_from_cells(c, floor)
        cdfs.append(a)
        subs.append(b)
    return np.concatenate(cdfs), np.concatenate(subs)


def density(cdf: np.ndarray, sub: np.ndarray, X: int, Y: int, x: float, y: float) -> float:
    """The learned density (per unit area) at (x, y) that the tables encode."""
    if not (0 <= x < X and 0 <= y < Y):
        return 0.0
    px, py = min(int(x), X - 1), min(int(y), Y - 1)
    pix = py + px * Y
    sc = min(int((y - py) * 4), 3) + 4 * min(int((x - px) * 4), 3)
    pp = (cdf[pix] - (cdf[pix - 1] if pix > 0 else 0.0)) / cdf[-1]
    s = sub[16 * pix:16 * pix + 16]
    return float(pp * s[sc] / s.sum() * 16.0)
