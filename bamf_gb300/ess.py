"""Effective sample size of sampler traces.

ESS of a scalar chain by Geyer's initial monotone sequence estimator
(C. J. Geyer, "Practical Markov chain Monte Carlo", Statistical Science 7(4),
1992, section 3.3): with the lag-k autocovariances g_k (biased, divided by
n) and the pair sums G_m = g_{2m} + g_{2m+1}, keep the initial run of
positive G_m, make it non-increasing, and take the asymptotic variance
s^2 = -g_0 + 2 * sum G_m; ESS = n * g_0 / s^2.

The sampler records one trace entry per chain entry (bamf_batch_results
n_trace / x_trace).  `batch_ess` takes the trial-phase part of every ROI's
trace and returns the per-ROI ESS of the emitter count and of the mean-X
position functional.
"""
from __future__ import annotations

import numpy as np


def autocov(x: np.ndarray) -> np.ndarray:
    """Biased autocovariances g_0..g_{n-1} of a 1-D series (FFT)."""
    x = np.asarray(x, np.float64)
    n = x.size
    d = x - x.mean()
    m = 1 << int(np.ceil(np.log2(2 * n)))
    f = np.fft.rfft(d, m)
    return np.fft.irfft(f * np.conj(f), m)[:n] / n


def ess_geyer(x) -> float:
    """ESS of one chain; NaN when the chain is constant or shorter than 4."""
    x = np.asarray(x, np.float64)
    n = x.size
    if n < 4:
        return float("nan")
    g = autocov(x)
    if not g[0] > 0:
        return float("nan")
    npair = n // 2
    G = g[0:2 * npair:2] + g[1:2 * npair:2]
    pos = np.nonzero(G <= 0)[0]
    G = G[:pos[0]] if pos.size else G
    if G.size == 0:
        return float(n)
    G = np.minimum.accumulate(G)
    s2 = -g[0] + 2.0 * G.sum()
    if not s2 > 0:
        return float(n)
    return float(min(n * g[0] / s2, n * np.log10(n)))


def _fill_nan(t: np.ndarray) -> np.ndarray:
    """NaN entries (no emitter) take the chain's mean over the others."""
    ok = np.isfinite(t)
    if ok.all():
        return t
    out = t.copy()
    out[~ok] = t[ok].mean() if ok.any() else 0.0
    return out


def batch_ess(n_trace: np.ndarray, x_trace: np.ndarray | None, n_entries: np.ndarray,
              n_burnin_entries: np.ndarray | int) -> dict:
    """Per-ROI ESS over the entries after burn-in.

    n_trace [k][T] uint8, x_trace [k][T] float or None, n_entries [k] (chain
    entries recorded), n_burnin_entries: entries recorded during burn-in
    (scalar or [k]); entries past T are not in the trace and are ignored.
    """
    k, T = n_trace.shape
    b = np.broadcast_to(np.asarray(n_burnin_entries), (k,))
    ess_n = np.full(k, np.nan)
    ess_x = np.full(k, np.nan)
    length = np.zeros(k, np.int64)
    for i in range(k):
        e = min(int(n_entries[i]), T)
        s = min(int(b[i]), e)
        length[i] = e - s
        if e - s < 4:
            continue
        ess_n[i] = ess_geyer(n_trace[i, s:e].astype(np.float64))
        if x_trace is not None:
            xt = x_trace[i, s:e].astype(np.float64)
            if np.isfinite(xt).sum() >= 4:
                ess_x[i] = ess_geyer(_fill_nan(xt))
    return {"ess_n": ess_n, "ess_x": ess_x, "length": length}


def summarize(ess: dict, seconds: float) -> dict:
    """Totals over ROIs (constant chains count as zero effective samples)
    and per-second rates."""
    en = np.nan_to_num(ess["ess_n"], nan=0.0)
    ex = np.nan_to_num(ess["ess_x"], nan=0.0)
    return {"ess_n_total": float(en.sum()), "ess_x_total": float(ex.sum()),
            "ess_n_per_s": float(en.sum() / seconds), "ess_x_per_s": float(ex.sum() / seconds),
            "ess_n_median": float(np.nanmedian(ess["ess_n"])) if np.isfinite(ess["ess_n"]).any() else 0.0,
            "ess_x_median": float(np.nanmedian(ess["ess_x"])) if np.isfinite(ess["ess_x"]).any() else 0.0,
            "entries_median": float(np.median(ess["length"]))}
