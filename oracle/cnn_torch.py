"""TEST INFRASTRUCTURE: the gradient oracle of the learned birth proposal.

A PyTorch (CPU) statement of the network and loss that include/bamf_cnn.h
defines, from the same FP32 parameter vector.  With `bf16=True` it rounds
the 32 -> 32 convolution weights and the activations a1..a4 to BF16 at the
points where the CUDA kernels store BF16 (straight-through in the backward
pass), so forward values match the GPU up to FP32 summation order and
gradients up to the BF16 rounding of the GPU's backward intermediates.
Also a generator-free reference of the birth tables the inference writes.
"""
from __future__ import annotations

import numpy as np
import torch

SIDE, NPX, CH, NSUB, NC = 16, 256, 32, 16, 11
OFF = dict(W1=(0, (32, 1, 3, 3)), b1=(288, (32,)), W2=(320, (32, 32, 3, 3)), b2=(9536, (32,)),
           W3=(9568, (32, 32, 3, 3)), b3=(18784, (32,)), W4=(18816, (32, 32, 3, 3)), b4=(28032, (32,)),
           Wl=(28064, (16, 32)), bl=(28576, (16,)), Wc=(28592, (11, 32)), bc=(28944, (11,)))
NPARAM = 28955


def unpack(theta: torch.Tensor) -> dict:
    out = {}
    for k, (o, shp) in OFF.items():
        n = int(np.prod(shp))
        out[k] = theta[o:o + n].reshape(shp)
    return out


def _q(t: torch.Tensor, bf16: bool) -> torch.Tensor:
    if not bf16:
        return t
    return t + (t.to(torch.bfloat16).to(t.dtype) - t).detach()


def forward(theta: torch.Tensor, data: torch.Tensor, bf16: bool = True):
    """data [n][256] (p = y + 16 x) -> (loc logits [n][256][16], count logits
    [n][11], a4 [n][32][16][16])."""
    P = unpack(theta)
    n = data.shape[0]
    v = torch.sqrt(torch.clamp(data, min=0) + 0.375)
    x0 = ((v - v.mean(dim=1, keepdim=True)) * 0.25).reshape(n, 1, SIDE, SIDE)  # [n][1][x][y]
    a = _q(torch.relu(torch.nn.functional.conv2d(x0, P["W1"], P["b1"], padding=1)), bf16)
    for l in (2, 3, 4):
        W = _q(P[f"W{l}"], bf16)
        a = _q(torch.relu(torch.nn.functional.conv2d(a, W, P[f"b{l}"], padding=1)), bf16)
    loc = torch.einsum("ncxy,sc->nxys", a, P["Wl"]) + P["bl"]
    loc = loc.reshape(n, NPX, NSUB)
    g = a.mean(dim=(2, 3))
    cnt = g @ P["Wc"].T + P["bc"]
    return loc, cnt, a


def loss(theta: torch.Tensor, data: torch.Tensor, n_em: np.ndarray, xyi: np.ndarray, bf16: bool = True):
    """Batch-mean loss of include/bamf_cnn.h."""
    loc, cnt, _ = forward(theta, data, bf16)
    n = data.shape[0]
    logp = torch.log_softmax(loc.reshape(n, -1), dim=1)
    logc = torch.log_softmax(cnt, dim=1)
    total = torch.zeros((), dtype=theta.dtype)
    for r in range(n):
        cells = []
        for e in range(int(n_em[r])):
            X, Y = float(xyi[r, e, 0]), float(xyi[r, e, 1])
            if not (0 <= X < SIDE and 0 <= Y < SIDE):
                continue
            cx, cy = min(int(X), SIDE - 1), min(int(Y), SIDE - 1)
            s = min(int((Y - cy) * 4), 3) + 4 * min(int((X - cx) * 4), 3)
            cells.append((cx * SIDE + cy) * NSUB + s)
        if cells:
            total = total - logp[r, cells].sum() / len(cells)
        total = total - logc[r, min(int(n_em[r]), NC - 1)]
    return total / n


def birth_tables(theta: torch.Tensor, data: torch.Tensor, bf16: bool = True):
    """(cdf [n*256], sub [n*256*16]) the inference kernel writes."""
    loc, _, _ = forward(theta, data, bf16)
    n = data.shape[0]
    p = torch.softmax(loc.reshape(n, -1), dim=1).reshape(n, NPX, NSUB)
    pix = p.sum(dim=2)
    cdf = torch.cumsum(pix, dim=1)
    sub = p / pix[..., None]
    return cdf.reshape(-1), sub.reshape(-1)
