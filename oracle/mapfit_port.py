"""TEST INFRASTRUCTURE: numpy restatement of the chain summaries of
@RJ/findMap.m:29-111 (MAP count, k-means, per-cluster mean/std) and
@RJ/mcmc.m:142-169 (per-emitter mean/std) on the thinned state records the
batched sampler writes, with the device kernels' k-means start (the first
qualifying state's emitters) and float32 distances."""
from __future__ import annotations

import numpy as np

S = 32


def _half(n_entries):
    it = int(n_entries) - 1
    return (it + 1) // 2 - 1, it - 1


def _std(v):
    v = np.asarray(v, np.float64)
    if len(v) == 0:
        return np.nan
    if len(v) == 1:
        return 0.0
    return float(np.std(v, ddof=1))


def map_kmeans(recs, thin, n_entries, K, max_iter=100):
    lo, hi = _half(n_entries)
    nw = min(len(recs), -(-int(n_entries) // thin))
    K = min(max(int(K), 0), S)
    q = [r for r in range(nw) if recs[r, 1] == K and lo <= r * thin <= hi]
    bg = np.array([recs[r, 2] for r in q], np.float64)
    out = {"N": K, "records": len(q), "Bg": bg.mean() if len(q) else np.nan, "Bg_SE": _std(bg),
           "ABg": np.mean([recs[r, 3] for r in q]) if q else np.nan,
           "BBg": np.mean([recs[r, 4] for r in q]) if q else np.nan,
           "X": np.full(S, np.nan), "Y": np.full(S, np.nan), "I": np.full(S, np.nan),
           "X_SE": np.full(S, np.nan), "Y_SE": np.full(S, np.nan), "I_SE": np.full(S, np.nan)}
    if K == 0 or not q:
        return out
    P = np.array([[recs[r, 5 + s], recs[r, 5 + S + s], recs[r, 5 + 2 * S + s]] for r in q for s in range(K)],
                 np.float32)
    c = P[:K, :2].copy()
    asg = np.full(len(P), -1)
    for _ in range(max_iter):
        d = ((P[:, None, 0] - c[None, :, 0]) ** 2 + (P[:, None, 1] - c[None, :, 1]) ** 2).astype(np.float32)
        new = np.argmin(d, axis=1)
        if (new == asg).all():
            break
        asg = new
        for k in range(K):
            m = asg == k
            if m.any():
                c[k] = P[m, :2].astype(np.float64).mean(axis=0).astype(np.float32)
    for k in range(K):
        m = asg == k
        for j, name in enumerate(("X", "Y", "I")):
            v = P[m, j].astype(np.float64)
            out[name][k] = v.mean() if len(v) else np.nan
            out[name + "_SE"][k] = _std(v)
    return out


def refine_stats(recs, thin, n_entries):
    lo, hi = _half(n_entries)
    nw = min(len(recs), -(-int(n_entries) // thin))
    q = [r for r in range(nw) if lo <= r * thin <= hi]
    K = min(int(recs[q[0], 1]), S) if q else 0
    out = {"N": K, "records": len(q)}
    for j, name in enumerate(("X", "Y", "I")):
        out[name] = np.full(S, np.nan)
        out[name + "_SE"] = np.full(S, np.nan)
        for s in range(K):
            v = np.array([recs[r, 5 + j * S + s] for r in q], np.float64)
            out[name][s] = v.mean()
            out[name + "_SE"][s] = _std(v)
    return out
