"""The other gaussMLE fit types ('Sigma', 'Z', 'SigmaYX', and sCMOS for all
four) against the reference's own kernels (cuda_gaussMLEv2.cu:144-1125,
compiled unmodified for sm_103a) on the same ROIs, with the arguments
gaussMLE.m passes."""
import numpy as np
import pytest

from oracle import refgpu

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refgpu.available("gaussmle"), reason="reference gaussMLE cubin not built")]

Z = {"Ax": 0.05, "Ay": -0.05, "Bx": 0.02, "By": 0.03, "Gamma": 0.35, "D": 0.6}


def _profile(side, c, s):
    from scipy.special import erf
    i = np.arange(side)[None, :]
    return 0.5 * (erf((i - c[:, None] + 1) / (np.sqrt(2) * s[:, None])) - erf((i - c[:, None]) / (np.sqrt(2) * s[:, None])))


def _rois(fit, n=3000, sz=7, seed=0):
    """n ROIs (sz, sz, n), one emitter each: axis 0 (rows) uses sigma_0, axis 1 sigma_1."""
    rng = np.random.default_rng(seed)
    y = rng.uniform(2.5, 4.5, n)     # along axis 0 (contiguous)
    x = rng.uniform(2.5, 4.5, n)
    I = rng.lognormal(np.log(1500), 0.3, n)
    bg = rng.uniform(5, 30, n)
    if fit == "Sigma":
        s0 = s1 = rng.uniform(1.0, 1.6, n)
    elif fit == "SigmaYX":
        s0, s1 = rng.uniform(1.0, 1.6, n), rng.uniform(1.0, 1.6, n)
    elif fit == "Z":
        z = rng.uniform(-0.4, 0.4, n)
        t0, t1 = (z - Z["Gamma"]) / Z["D"], (z + Z["Gamma"]) / Z["D"]
        s0 = 1.2 * np.sqrt(1 + t0 ** 2 + Z["Ax"] * t0 ** 3 + Z["Bx"] * t0 ** 4)
        s1 = 1.3 * np.sqrt(1 + t1 ** 2 + Z["Ay"] * t1 ** 3 + Z["By"] * t1 ** 4)
    else:
        s0 = s1 = np.full(n, 1.3)
    py, px = _profile(sz, y, s0), _profile(sz, x, s1)         # [n][sz]
    lam = bg[:, None, None] + I[:, None, None] * py[:, :, None] * px[:, None, :]   # [n][row][col]
    d = rng.poisson(lam).astype(np.float32)
    return np.ascontiguousarray(np.transpose(d, (1, 2, 0)))   # (sz, sz, n)


@pytest.mark.parametrize("camera", ["CCD", "SCMOS"])
@pytest.mark.parametrize("fit", ["Basic", "Sigma", "Z", "SigmaYX"])
def test_fit_types_match_reference_kernels(cuda_lib, fit, camera):
    pytest.importorskip("scipy")
    import torch
    from bamf_gb300 import frontend
    sz, n = 7, 3000
    rois = _rois(fit, n, sz, seed=3)
    sigma = [1.2, 1.3] if fit == "Z" else 1.3
    args = []
    var_dev = corners_dev = None
    msz = 0
    if camera == "SCMOS":
        rng = np.random.default_rng(9)
        msz = 64
        var = rng.uniform(1.0, 20.0, (msz, msz)).astype(np.float32)
        corners = rng.integers(0, msz - sz, size=(n, 2)).astype(np.float32)
        args = [var, corners]
        var_dev = torch.from_numpy(np.ascontiguousarray(var.ravel(order="F"))).cuda()
        corners_dev = torch.from_numpy(np.ascontiguousarray(corners.ravel())).cuda()
    if fit == "Z":
        args.append(Z)
    res = frontend.gaussMLE(rois, fit, camera, sigma, *args, Iterations=20)
    flat = torch.from_numpy(np.ascontiguousarray(rois.ravel(order="F"))).cuda()
    P, CR, LL = refgpu.gaussmle_fit(flat, sz, n, fit, sigma, 20, zstruct=Z if fit == "Z" else None,
                                    var_map_dev=var_dev, corners_dev=corners_dev, map_size=msz)
    npar = refgpu.NPARAM[fit]
    Pr = P.cpu().numpy().reshape(npar, n)
    names = ["Y", "X", "Photons", "BG"] + frontend.FIT_EXTRA[fit]
    Pg = np.stack([res[k] for k in names])
    rel = np.abs(Pg - Pr) / np.maximum(np.abs(Pr), 1e-3)
    q99 = np.quantile(rel, 0.99, axis=1)
    print(fit, camera, "max rel", rel.max(axis=1), "99%", q99)
    assert (q99 < 1e-4).all() and (np.median(rel, axis=1) < 1e-5).all()
    LLr = LL.cpu().numpy()
    assert np.quantile(np.abs(res["LogLikelihood"] - LLr) / np.maximum(np.abs(LLr), 1.0), 0.99) < 1e-3
    # the fits recover the generator on average
    assert abs(np.median(res["Photons"]) / 1500.0 - 1) < 0.1
