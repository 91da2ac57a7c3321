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

Several chains of one ROI (`rhat`, `ess_bulk`, `multi_chain_ess`): the
rank-normalised split-R-hat and bulk ESS of A. Vehtari, A. Gelman, D.
Simpson, B. Carpenter and P.-C. Buerkner, "Rank-normalization, folding, and
localization: an improved R-hat for assessing convergence of MCMC",
Bayesian Analysis 16(2), 2021: every chain is split in half, the pooled
draws are replaced by the normal scores of their (average) ranks, R-hat is
the square root of the pooled-variance estimate over the mean within-chain
variance (the larger of the bulk and the folded |x - median| version), and
the multi-chain autocorrelation rho_t = 1 - (W - mean_m s_m^2 rho_{t,m}) /
var+ is summed by Geyer's initial monotone sequence; ESS = M N / tau.
Chains that have not mixed (different modes) get R-hat well above 1 and an
ESS near the number of chains, where one chain's own ESS would not show it.
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


def _split(chains: np.ndarray) -> np.ndarray:
    """[M][N] -> [2M][N//2]: the first and second half of every chain."""
    c = np.asarray(chains, np.float64)
    h = c.shape[1] // 2
    return np.concatenate([c[:, :h], c[:, c.shape[1] - h:]], 0)


def _rank_normal(c: np.ndarray) -> np.ndarray:
    """Normal scores of the pooled average ranks: Phi^-1((r - 3/8) / (S + 1/4))."""
    from scipy.special import ndtri
    from scipy.stats import rankdata
    S = c.size
    r = rankdata(c.ravel(), method="average").reshape(c.shape)
    return ndtri((r - 0.375) / (S + 0.25))


def _rhat_raw(c: np.ndarray) -> float:
    M, N = c.shape
    w = c.var(axis=1, ddof=1).mean()
    if not w > 0:
        return float("nan")
    b = N * c.mean(axis=1).var(ddof=1)
    var_plus = (N - 1) / N * w + b / N
    return float(np.sqrt(var_plus / w))


def rhat(chains) -> float:
    """Rank-normalised split-R-hat: the larger of the bulk and the folded
    values.  NaN when every draw is the same."""
    c = _split(chains)
    if c.shape[1] < 2 or np.ptp(c) == 0:
        return float("nan")
    bulk = _rhat_raw(_rank_normal(c))
    fold = _rhat_raw(_rank_normal(np.abs(c - np.median(c))))
    return float(np.nanmax([bulk, fold]))


def _ess_chains(c: np.ndarray) -> float:
    M, N = c.shape
    acov = np.stack([autocov(c[m]) for m in range(M)])  # biased (divided by N)
    w = (acov[:, 0] * N / (N - 1)).mean()               # mean within-chain variance
    if not w > 0:
        return float("nan")
    var_plus = (N - 1) / N * w + (c.mean(axis=1).var(ddof=1) if M > 1 else 0.0)
    # rho_t = 1 - (W - mean_m s_m^2 rho_{t,m}) / var+, with s_m^2 rho_{t,m} the chain's lag-t autocovariance
    rho = 1.0 - (w - acov.mean(axis=0)) / var_plus
    rho[0] = 1.0
    npair = N // 2
    P = rho[0:2 * npair:2] + rho[1:2 * npair:2]
    neg = np.nonzero(P <= 0)[0]
    P = P[:neg[0]] if neg.size else P
    if P.size == 0:
        return float(M * N)
    P = np.minimum.accumulate(P)
    tau = -1.0 + 2.0 * P.sum()
    tau = max(tau, 1.0 / np.log10(M * N))
    return float(M * N / tau)


def ess_bulk(chains) -> float:
    """Bulk ESS of several chains of one quantity ([M][N]): split chains,
    rank-normalised draws, multi-chain autocorrelation, Geyer's initial
    monotone sequence.  NaN when every draw is the same."""
    c = _split(chains)
    if c.shape[1] < 4 or np.ptp(c) == 0:
        return float("nan")
    return _ess_chains(_rank_normal(c))


def multi_chain_ess(n_trace: np.ndarray, x_trace: np.ndarray | None, n_entries: np.ndarray, groups: np.ndarray,
                    start_frac: float = 0.5) -> dict:
    """Per ROI: bulk ESS and R-hat of the emitter count and of the mean-X
    functional over its chains.  groups [G][M] names the trace rows of
    each ROI's M chains; every chain contributes its entries from
    start_frac of its length on (the trial phase), cut to the shortest
    chain of the group.  A chain entry with no emitter has no mean X: it
    takes the mean of the group's other entries."""
    G = len(groups)
    out = {k: np.full(G, np.nan) for k in ("ess_n", "rhat_n", "ess_x", "rhat_x")}
    for g, rows in enumerate(groups):
        ends = [min(int(n_entries[r]), n_trace.shape[1]) for r in rows]
        starts = [int(e * start_frac) for e in ends]
        L = min(e - s for e, s in zip(ends, starts))
        if L < 8:
            continue
        cn = np.stack([n_trace[r, s:s + L].astype(np.float64) for r, s in zip(rows, starts)])
        out["ess_n"][g] = ess_bulk(cn)
        out["rhat_n"][g] = rhat(cn)
        if x_trace is not None:
            cx = np.stack([x_trace[r, s:s + L].astype(np.float64) for r, s in zip(rows, starts)])
            ok = np.isfinite(cx)
            if ok.sum() >= 8:
                cx[~ok] = cx[ok].mean()
                out["ess_x"][g] = ess_bulk(cx)
                out["rhat_x"][g] = rhat(cx)
    return out
