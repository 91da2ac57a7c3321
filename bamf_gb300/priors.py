"""Prior construction from the front end (@RJ/findPriors.m:35-111 with
@RJ/threhsSMA.m:1-29): signal-intensity, offset-background and
background-emitter priors of the sampler, on the grid 0:P_dP:max+1000 P_dP.

FindROI and gaussMLE run on the GPU (bamf_gb300.frontend); the statistics
that follow are host code, as in the reference:
  * threhsSMA: keep fits with X_SE, Y_SE < MaxXY_SE, chi-square p-value of
    -2 LL (k = Boxsize^2 - 4 degrees of freedom) above MinPValue, Photons
    above MinPhotons, 0 < X, Y < Boxsize, BG > 0;
  * signal prior: kernel density estimate with a normal kernel of bandwidth
    75 photons (MATLAB fitdist 'Kernel', 'BandWidth', 75) of the kept
    intensities below their 98% quantile (when more than 200), refitted
    without the intensities beyond the first trough after the main peak
    when the density has further extrema there;
  * offset prior: gamma pdf with the maximum-likelihood shape and scale of
    the kept backgrounds (MATLAB fitdist 'Gamma');
  * background-emitter prior: exponential pdf of mean mean(I)/BgPriorRange
    (Y_N_BgPrior = 'Yes'), else zeros.
MATLAB's Statistics Toolbox is not available to pin these against; the
tests compare them with scipy's implementations of the same definitions.
"""
from __future__ import annotations

import numpy as np

from . import frontend


def p_value(fit_type: str, box: int, LL: np.ndarray) -> np.ndarray:
    """threhsSMA.m pValue: 1 - chi-square CDF of -2 LL."""
    from scipy.special import gammainc
    k = {"Basic": box * box - 4, "Sigma": box * box - 5, "Astig": box * box - 5,
         "SampledZ": box * box - 5}[fit_type]
    X2 = -2.0 * np.asarray(LL, np.float64)
    return 1.0 - gammainc(k / 2.0, X2 / 2.0)


def threhsSMA(SMD: dict, SMAStruct: dict, BoxSize: int) -> dict:
    """threhsSMA.m:1-16."""
    max_se = SMAStruct.get("MaxXY_SE", 0.2)
    pv = p_value("Basic", BoxSize, SMD["LogLikelihood"])
    X, Y = np.asarray(SMD["X"]), np.asarray(SMD["Y"])
    ind = ((SMD["X_SE"] < max_se) & (SMD["Y_SE"] < max_se) & (pv > SMAStruct["MinPValue"])
           & (SMD["Photons"] > SMAStruct["MinPhotons"]) & np.isfinite(X) & np.isfinite(Y)
           & (X > 0) & (Y > 0) & (X < BoxSize) & (Y < BoxSize) & (SMD["BG"] > 0))
    return {"Photons": np.asarray(SMD["Photons"])[ind], "Bg": np.asarray(SMD["BG"])[ind]}


def kernel_pdf(samples: np.ndarray, bandwidth: float, x: np.ndarray, chunk: int = 4096) -> np.ndarray:
    """Normal-kernel density of `samples` with bandwidth h at x (double):
    (1 / (n h)) sum_i phi((x - s_i) / h)."""
    s = np.asarray(samples, np.float64)
    x = np.asarray(x, np.float64)
    out = np.zeros(x.shape, np.float64)
    c = 1.0 / (len(s) * bandwidth * np.sqrt(2 * np.pi))
    for a in range(0, len(s), chunk):
        d = (x[:, None] - s[None, a:a + chunk]) / bandwidth
        out += np.exp(-0.5 * d * d).sum(axis=1)
    return out * c


def gamma_fit(x: np.ndarray, iters: int = 50) -> tuple:
    """Maximum-likelihood (shape a, scale b) of a gamma sample: Newton on
    log a - digamma(a) = log(mean) - mean(log x), started from Minka's
    closed-form approximation (T. Minka, "Estimating a Gamma
    distribution", 2002)."""
    from scipy.special import digamma, polygamma
    x = np.asarray(x, np.float64)
    x = x[x > 0]
    m = x.mean()
    s = np.log(m) - np.log(x).mean()
    a = (3.0 - s + np.sqrt((s - 3.0) ** 2 + 24.0 * s)) / (12.0 * s)
    for _ in range(iters):
        f = np.log(a) - digamma(a) - s
        fp = 1.0 / a - polygamma(1, a)
        step = f / fp
        a_new = a - step
        if a_new <= 0:
            a_new = a / 2
        if abs(a_new - a) < 1e-12 * a:
            a = a_new
            break
        a = a_new
    return float(a), float(m / a)


def gamma_pdf(x: np.ndarray, a: float, b: float) -> np.ndarray:
    from scipy.special import gammaln
    x = np.asarray(x, np.float64)
    out = np.zeros_like(x)
    pos = x > 0
    out[pos] = np.exp((a - 1) * np.log(x[pos]) - x[pos] / b - gammaln(a) - a * np.log(b))
    if a == 1:
        out[x == 0] = 1.0 / b
    return out


def signal_prior(photons: np.ndarray, dP: float, bandwidth: float = 75.0):
    """findPriors.m:49-67: (SignalPDF, Xarray, photons kept)."""
    photon = np.asarray(photons, np.float64)
    if len(photon) > 200:
        q = np.quantile(photon, 0.98)
        photon = photon[~(photon > q)]
    xarray = np.arange(0.0, photon.max() + 1000 * dP + dP / 2, dP)
    pdf = kernel_pdf(photon, bandwidth, xarray)
    gr = np.gradient(pdf)
    sg = np.sign(gr)
    ind = np.nonzero(np.concatenate([[0.0], np.diff(sg)]))[0] + 1      # 1-based
    if ind.size:
        ind_max = np.nonzero(pdf == pdf[ind - 1].max())[0] + 1
        remove = np.nonzero(ind > ind_max[0])[0]
        if remove.size >= 2:
            photon = photon[~(photon > ind[remove[0]] * dP)]
            xarray = np.arange(0.0, photon.max() + 1000 * dP + dP / 2, dP)
            pdf = kernel_pdf(photon, bandwidth, xarray)
    return pdf, xarray, photon


def findPriors(Data, RJStruct, SMAStruct: dict, Y_N_BgPrior: str = "No", BgPriorRange: float | None = None):
    """findPriors.m:35-111 on frames Data (Y, X, Z), MATLAB orientation.
    Returns (SignalPDF, OffsetPDF, BgPDF, info) as float32 arrays on the
    grid 0:P_dP:..., and sets RJStruct.P_EmPhotons / P_BgEmPhotons /
    P_Offset like the reference."""
    box = 8
    s1 = float(RJStruct.PSF_Sigma)
    minval = SMAStruct["MeanPhotons"] / (4 * np.pi * s1 ** 2) / 4
    _, roistack, _ = frontend.findROI(Data, s1, 2 * s1, box, minval)
    SMD = frontend.gaussMLE(roistack, "Basic", "CCD", s1)
    SMR = threhsSMA(SMD, SMAStruct, box)
    dP = float(RJStruct.P_dP)
    signal, xarray, photon = signal_prior(SMR["Photons"], dP)
    a, b = gamma_fit(SMR["Bg"])
    offset = gamma_pdf(xarray, a, b)
    if Y_N_BgPrior == "Yes":
        rng = BgPriorRange if BgPriorRange is not None else getattr(RJStruct, "BgPriorRange")
        mean_bg = photon.mean() / rng
        back = np.exp(-xarray / mean_bg) / mean_bg
    else:
        back = np.zeros_like(xarray)
    RJStruct.P_EmPhotons = signal.astype(np.float32)
    RJStruct.P_BgEmPhotons = back.astype(np.float32)
    RJStruct.P_Offset = offset.astype(np.float32)
    info = {"n_fits": int(len(SMD["X"])), "n_kept": int(len(SMR["Photons"])), "gamma_shape": a,
            "gamma_scale": b, "photons_used": int(len(photon))}
    return RJStruct.P_EmPhotons, RJStruct.P_Offset, RJStruct.P_BgEmPhotons, info
